"""Training of the a-priori MLP gate on the GPU with the library's own kernels.

Pipeline (the reference's script_auto.sh:8-21 in spirit, GPU-native):
  1. harvest: plain GP-MOOD runs of seeded initial conditions; at every step
     the library appends the stage-1 samples of every non-constant interior
     cell (36 features, label = the plain MOOD loop lowered the cell's order),
     keeping negatives with a small probability to balance the classes
     (mod_append_NN_dataset.f90:42-49 balances by rejection too);
  2. train: mini-batch Adam on the weighted binary cross-entropy, forward and
     backward in BF16 on the tensor cores (gpmood_nn_loss_grad, gpmood_nn_adam);
  3. export: the FP32 parameter vector in PyTorch flatten order, the format of
     the reference's save_NN_for_fortran.py (one value per line).

PyTorch is used only to hold device buffers; every FLOP runs in libgpmood.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import ic
from .gpmood import NN_NPARAMS, GpmoodError, Solver, load_library

NIN, NH = 36, 64


def init_params(seed: int = 0) -> np.ndarray:
    """nn.Linear's default init: U(-1/sqrt(fan_in), 1/sqrt(fan_in)) for weights and biases."""
    rng = np.random.default_rng(seed)
    parts = []
    for fan_in, fan_out in ((NIN, NH), (NH, NH), (NH, 1)):
        b = 1.0 / math.sqrt(fan_in)
        parts.append(rng.uniform(-b, b, size=fan_out * fan_in))
        parts.append(rng.uniform(-b, b, size=fan_out))
    p = np.concatenate(parts).astype(np.float32)
    assert p.size == NN_NPARAMS
    return p


def _lib():
    L = load_library()
    return L


def _check(rc: int, what: str) -> None:
    if rc != 0:
        buf = C.create_string_buffer(512)
        _lib().gpmood_last_error(None, buf, 512)
        raise GpmoodError(rc, f"{what}: {buf.value.decode(errors='replace')}")


def loss_grad(params_d, x_d, y_d, n, grad_d, loss_d, pos_weight=1.0, stream=None):
    """One fused BF16 forward+backward over n samples (device pointers)."""
    _check(_lib().gpmood_nn_loss_grad(C.c_void_p(params_d), C.c_void_p(x_d), C.c_void_p(y_d), int(n),
                                      float(pos_weight), C.c_void_p(grad_d), C.c_void_p(loss_d),
                                      C.c_void_p(stream)), "gpmood_nn_loss_grad")


def forward(params_d, x_d, n, logits_d, stream=None):
    _check(_lib().gpmood_nn_forward(C.c_void_p(params_d), C.c_void_p(x_d), int(n), C.c_void_p(logits_d),
                                    C.c_void_p(stream)), "gpmood_nn_forward")


def adam(params_d, grad_d, m_d, v_d, step, lr, beta1=0.9, beta2=0.999, eps=1e-8, stream=None):
    _check(_lib().gpmood_nn_adam(C.c_void_p(params_d), C.c_void_p(grad_d), C.c_void_p(m_d), C.c_void_p(v_d),
                                 int(step), float(lr), float(beta1), float(beta2), float(eps),
                                 C.c_void_p(stream)), "gpmood_nn_adam")


@dataclass
class Dataset:
    x: "object"   # torch float32 [n, 36] on the GPU
    y: "object"   # torch float32 [n]
    positives: int

    @property
    def n(self) -> int:
        return int(self.y.shape[0])


def harvest(runs, capacity: int, keep_negative: float, steps_per_run: int, seed: int = 0, fp_mode: int = 1):
    """Run plain GP-MOOD on each (ic_array, knobs) of ``runs`` and collect stage-1 samples."""
    import torch
    x = torch.empty((capacity, NIN), dtype=torch.float32, device="cuda")
    y = torch.empty((capacity,), dtype=torch.float32, device="cuda")
    count = torch.zeros((1,), dtype=torch.int32, device="cuda")
    for k, (U0, knobs) in enumerate(runs):
        with Solver(fp_mode=fp_mode, **knobs) as s:
            s.Boundary_C(U0, 0.0)
            s.set_state(U0, 0.0)
            s.nn_harvest(x.data_ptr(), y.data_ptr(), capacity, keep_negative, seed * 7919 + k, count.data_ptr())
            s.advance(steps_per_run)
            s.nn_harvest(0, 0, 0, 0.0, 0, 0)
        if int(count.item()) >= capacity:
            break
    n = min(int(count.item()), capacity)
    pos = int(y[:n].sum().item())
    return Dataset(x[:n], y[:n], pos)


def training_runs(seed: int = 0, sedov_n: int = 2048, rp_n: int = 256):
    """The seeded training runs: the 2DRP3 IC at 256^2 and the Sedov IC with
    rho, p and E0 perturbed by up to +-20 %."""
    rng = np.random.default_rng(seed)
    runs = [(ic.rp2d3(rp_n, rp_n), dict(lf=rp_n, nf=rp_n, bc_type=17, tmax=0.8))]
    for _ in range(4):
        f = rng.uniform(0.8, 1.2, size=3)
        U = ic.sedov(sedov_n, sedov_n, e0=float(f[0]), rho0=float(f[1]), p0=float(1e-5 * f[2]))
        runs.append((U, dict(lf=sedov_n, nf=sedov_n, bc_type=20, tmax=0.05)))
    return runs


def train(ds: Dataset, params0: np.ndarray, epochs: int = 3, batch: int = 4096, lr: float = 3e-3,
          pos_weight: float = 1.0, seed: int = 0, log=None):
    """Mini-batch Adam; returns the trained FP32 parameters and the loss history."""
    import torch
    dev = "cuda"
    p = torch.from_numpy(params0.astype(np.float32)).to(dev)
    g = torch.zeros_like(p)
    m = torch.zeros_like(p)
    v = torch.zeros_like(p)
    loss = torch.zeros((1,), dtype=torch.float32, device=dev)
    gen = torch.Generator(device="cpu").manual_seed(seed)
    step = 0
    hist = []
    n = ds.n
    for ep in range(epochs):
        perm = torch.randperm(n, generator=gen).to(dev)
        xs = ds.x[perm].contiguous()
        ys = ds.y[perm].contiguous()
        tot, nb = 0.0, 0
        for i in range(0, n - batch + 1, batch):
            step += 1
            loss_grad(p.data_ptr(), xs[i:].data_ptr(), ys[i:].data_ptr(), batch, g.data_ptr(), loss.data_ptr(),
                      pos_weight)
            adam(p.data_ptr(), g.data_ptr(), m.data_ptr(), v.data_ptr(), step, lr)
            if nb % 50 == 0:
                tot += float(loss.item())
                hist.append((step, float(loss.item())))
            nb += 1
        if log:
            log(f"epoch {ep}: {nb} batches, loss {hist[-1][1] if hist else float('nan'):.4f}")
    torch.cuda.synchronize()
    return p.cpu().numpy(), hist


def evaluate(ds: Dataset, params: np.ndarray, threshold: float = 0.0):
    """Accuracy, recall of troubled cells and false-positive rate on a dataset."""
    import torch
    p = torch.from_numpy(params.astype(np.float32)).cuda()
    z = torch.empty((ds.n,), dtype=torch.float32, device="cuda")
    forward(p.data_ptr(), ds.x.data_ptr(), ds.n, z.data_ptr())
    pred = z > threshold
    yb = ds.y > 0.5
    tp = int((pred & yb).sum().item())
    fp = int((pred & ~yb).sum().item())
    fn = int((~pred & yb).sum().item())
    tn = int((~pred & ~yb).sum().item())
    return {"accuracy": (tp + tn) / max(ds.n, 1), "recall": tp / max(tp + fn, 1),
            "false_positive_rate": fp / max(fp + tn, 1), "tp": tp, "fp": fp, "fn": fn, "tn": tn}


def save_text(params: np.ndarray, path: str) -> None:
    """One value per line, PyTorch flatten order (save_NN_for_fortran.py:13-23)."""
    np.savetxt(path, np.asarray(params, dtype=np.float32).ravel(), fmt="%.9e")


def load_text(path: str) -> np.ndarray:
    p = np.loadtxt(path, dtype=np.float32).ravel()
    if p.size != NN_NPARAMS:
        raise ValueError(f"{path}: expected {NN_NPARAMS} values, got {p.size}")
    return p
