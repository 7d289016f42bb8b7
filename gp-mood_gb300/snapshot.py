"""Snapshots, restarts and training datasets in the reference's field layout.

The reference writes HDF5 files (gp-mood-code/output.f90:77-192 for
snapshots, :302-400 for NN datasets) and restarts from a snapshot
(gp-mood-code/reader.f90:12-120).  No HDF5 library exists on these machines,
so the same datasets, with the same names, shapes and types, go into a NumPy
``.npz`` archive instead:

snapshot  rho, ux, uy, p   float64 (nf, lf)  primitive variables of the interior
                                            (C order (nf, lf) is Fortran's (lf, nf))
          ordr, ordr_priori int32  (nf, lf)  CellGPO after the last stage, a-priori orders
          CFL, problem, method, NN_filename  strings
          lf, nf, niter, time
dataset   labels           float32 (2, size) one-hot: (1, 0) = the MOOD loop lowered
                                             the cell, (0, 1) = it kept the top order
                                             (mod_append_NN_dataset.f90:55-60)
          inputs           float32 (L, size) the gate's features
          CFL, problem, method, NN_filename  strings
"""
from __future__ import annotations

import numpy as np

GAMMA = 1.4
NGC = 4


def conservative_to_primitive(U: np.ndarray) -> np.ndarray:
    """physics.f90 conservative_to_primitive on (..., 4) arrays: rho, u, v, p."""
    r = U[..., 0]
    u = U[..., 1] / r
    v = U[..., 2] / r
    p = (GAMMA - 1.) * (U[..., 3] - 0.5 * r * (u * u + v * v))
    return np.stack([r, u, v, p], axis=-1)


def primitive_to_conservative(W: np.ndarray) -> np.ndarray:
    """physics.f90:146-160 on (..., 4) arrays."""
    r, u, v, p = W[..., 0], W[..., 1], W[..., 2], W[..., 3]
    return np.stack([r, r * u, r * v, p / (GAMMA - 1.) + 0.5 * r * (u * u + v * v)], axis=-1)


def save_snapshot(path, U: np.ndarray, t: float, niter: int, orders: np.ndarray, orders_priori=None,
                  cfl: float = 0.8, problem: str = "", method: str = "", nn_filename: str = "") -> None:
    """U is the padded conservative state (nf+8, lf+8, 4); orders CellGPO (nf, lf)."""
    W = conservative_to_primitive(U[NGC:-NGC, NGC:-NGC])
    nf, lf = W.shape[:2]
    op = np.full((nf, lf), -1, np.int32) if orders_priori is None else np.asarray(orders_priori, np.int32)
    np.savez(path, rho=W[..., 0], ux=W[..., 1], uy=W[..., 2], p=W[..., 3],
             ordr=np.asarray(orders, np.int32), ordr_priori=op, CFL=np.str_(repr(float(cfl))),
             problem=np.str_(problem), method=np.str_(method), NN_filename=np.str_(nn_filename),
             lf=np.int32(lf), nf=np.int32(nf), niter=np.int32(niter), time=np.float64(t))


def load_snapshot(path) -> dict:
    with np.load(path) as z:
        return {k: (z[k].item() if z[k].ndim == 0 else z[k]) for k in z.files}


def state_from_snapshot(snap: dict) -> np.ndarray:
    """The padded conservative state of a snapshot (reader.f90:12-120); the
    ghost cells are left zero for Boundary_C to fill."""
    lf, nf = int(snap["lf"]), int(snap["nf"])
    U = np.zeros((nf + 2 * NGC, lf + 2 * NGC, 4))
    W = np.stack([snap["rho"], snap["ux"], snap["uy"], snap["p"]], axis=-1)
    U[NGC:-NGC, NGC:-NGC] = primitive_to_conservative(W)
    return U


def save_dataset(path, x: np.ndarray, y: np.ndarray, cfl: float = 0.8, problem: str = "", method: str = "",
                 nn_filename: str = "") -> None:
    """Training samples: x (size, L) features, y (size,) 1 where the MOOD loop lowered the cell."""
    x = np.asarray(x, np.float32)
    y = np.asarray(y, np.float32).ravel()
    labels = np.stack([y, 1.0 - y]).astype(np.float32)
    np.savez(path, labels=labels, inputs=np.ascontiguousarray(x.T), CFL=np.str_(repr(float(cfl))),
             problem=np.str_(problem), method=np.str_(method), NN_filename=np.str_(nn_filename))


def load_dataset(path):
    """(x (size, L), y (size,)) of a dataset file."""
    with np.load(path) as z:
        return np.ascontiguousarray(z["inputs"].T), z["labels"][0].copy()
