#!/usr/bin/env python
"""Train the a-priori MLP gate on the GPU and write its parameter file.

  python gp-mood_gb300/train_gate.py [--out gp-mood_gb300/gates/gate_sedov_rp2d3.txt] [--seed 0]

Labels come from plain GP-MOOD runs (the 2DRP3 problem at 256^2 and the Sedov
blast with rho, p and E0 perturbed by up to +-20 % at 1024^2 and 2048^2): a
cell is positive when stage 1's MOOD loop lowered its order.  Training is
mini-batch Adam on the weighted cross-entropy with the library's BF16
tensor-core forward/backward kernels; the output is one FP32 value per line in
PyTorch flatten order (the reference's save_NN_for_fortran.py format).
"""
from __future__ import annotations

import argparse
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))

import numpy as np  # noqa: E402


def runs(seed: int):
    from gpmood_gb300 import ic
    rng = np.random.default_rng(seed)
    out = [(ic.rp2d3(256, 256), dict(lf=256, nf=256, bc_type=17, tmax=0.8), 400)]
    for n, steps in ((1024, 400), (1024, 400), (2048, 80), (2048, 80)):
        f = rng.uniform(0.8, 1.2, size=3)
        U = ic.sedov(n, n, e0=float(f[0]), rho0=float(f[1]), p0=float(1e-5 * f[2]))
        out.append((U, dict(lf=n, nf=n, bc_type=20, tmax=0.05), steps))
    return out


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(HERE / "gates" / "gate_sedov_rp2d3.txt"))
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--max-fpr", type=float, default=1e-3)
    args = ap.parse_args()

    import __graft_entry__ as ge
    ge.import_package()
    from gpmood_gb300 import nn_train as T

    import torch
    xs, ys, pos = [], [], 0
    for k, (U, knobs, steps) in enumerate(runs(args.seed)):
        ds = T.harvest([(U, knobs)], capacity=1_500_000, keep_negative=0.03, steps_per_run=steps,
                       seed=args.seed * 31 + k)
        xs.append(ds.x)
        ys.append(ds.y)
        pos += ds.positives
        print(f"run {k}: {knobs['lf']}^2, {steps} steps -> {ds.n} samples, {ds.positives} positive", flush=True)
    ds = T.Dataset(torch.cat(xs), torch.cat(ys), pos)
    p, hist = T.train(ds, T.init_params(args.seed), epochs=args.epochs, batch=4096, lr=3e-3, seed=args.seed,
                      log=print)
    # Operating point: the logit threshold at which at most a fraction
    # --max-fpr of the harvested negatives fires (extra flags change the
    # solution, missed ones only cost a MOOD pass).
    z = torch.empty((ds.n,), dtype=torch.float32, device="cuda")
    pt = torch.from_numpy(p).cuda()
    T.forward(pt.data_ptr(), ds.x.data_ptr(), ds.n, z.data_ptr())
    neg = torch.sort(z[ds.y < 0.5]).values
    k = min(neg.numel() - 1, int(np.ceil((1.0 - args.max_fpr) * neg.numel())))
    thr = max(0.0, float(neg[k].item())) if neg.numel() else 0.0
    m0 = T.evaluate(ds, p)
    m = T.evaluate(ds, p, threshold=thr)
    out = Path(args.out)
    out.parent.mkdir(parents=True, exist_ok=True)
    T.save_text(p, str(out))
    meta = {"samples": ds.n, "positives": pos, "loss_first": hist[0][1], "loss_last": hist[-1][1],
            "threshold": thr, "max_fpr": args.max_fpr, "at_threshold": m, "at_zero": m0, "seed": args.seed,
            "epochs": args.epochs, "keep_negative": 0.03}
    out.with_suffix(".json").write_text(json.dumps(meta, indent=1) + "\n")
    print(json.dumps(meta), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
