"""ctypes binding of the CPU oracle (oracle/gpmood_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA path.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline / reference arm load it.
Pinned to the reference's own recorded runs (bit for bit on the deprecated
code line's 2DRP3 outputs; gpmood_oracle.h lists the pins).
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "gpmood_oracle.c"
LIB = HERE / "_build" / "liboracle.so"

NGC = 4
# constants.f90:17-34
GP_MOOD, GP_SE = 2, 202
NEUMANN, PERIODIC, REFLECTIVE, DMR = 17, 18, 20, 35
FE, SSP_RK2, SSP_RK3, SSP_RK4 = 8, 9, 10, 12
HLLC, LLF, HLL, UNSPLIT = 100, 101, 102, 103


class OrcParams(C.Structure):
    _fields_ = [("cfl", C.c_double), ("ell_o_dx", C.c_double), ("lx", C.c_double), ("ly", C.c_double),
                ("tmax", C.c_double), ("mord", C.c_int), ("ngp", C.c_int), ("method", C.c_int),
                ("dmp", C.c_int), ("u2", C.c_int), ("u2_tol", C.c_int), ("lf", C.c_int), ("nf", C.c_int),
                ("bc_type", C.c_int), ("integrator", C.c_int), ("num_flux", C.c_int), ("setdt_kind", C.c_int),
                ("lf0", C.c_int), ("nf0", C.c_int), ("slow_start", C.c_double), ("csd_kind", C.c_int)]


class OrcGp(C.Structure):
    _fields_ = [("zt", C.c_double * (3 * 4 * 5 * 13)), ("d2x", C.c_double * 5), ("d2y", C.c_double * 5),
                ("gauss_w", C.c_double * 5), ("inv_err", C.c_double * 3), ("ixiy", C.c_int * 26)]


def build(force: bool = False) -> Path:
    """Compile the oracle with the reference's rounding: no FP contraction."""
    if LIB.exists() and not force and LIB.stat().st_mtime >= max(SRC.stat().st_mtime,
                                                                  (HERE / "gpmood_oracle.h").stat().st_mtime):
        return LIB
    LIB.parent.mkdir(exist_ok=True)
    cc = shutil.which("gcc") or "cc"
    tmp = LIB.with_suffix(".tmp.so")
    cmd = [cc, "-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-fopenmp",
           str(SRC), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P = C.POINTER
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        L.orc_gp_presim.argtypes = [P(OrcParams), P(OrcGp)]
        L.orc_hllc.argtypes = [dp, dp, C.c_int, dp]
        L.orc_pressure.argtypes = [dp]
        L.orc_pressure.restype = C.c_double
        L.orc_boundary.argtypes = [P(OrcParams), dp, C.c_double]
        L.orc_setdt.argtypes = [P(OrcParams), dp, C.c_double]
        L.orc_setdt.restype = C.c_double
        L.orc_create.argtypes = [P(OrcParams)]
        L.orc_create.restype = C.c_void_p
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_set_cc.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.orc_weights.argtypes = [C.c_void_p]
        L.orc_weights.restype = C.c_void_p
        L.orc_time_stepping.argtypes = [C.c_void_p, dp, dp, C.c_double, C.c_double, C.c_void_p, C.c_void_p,
                                        P(C.c_longlong)]
        L.orc_shock_detector.argtypes = [P(OrcParams), dp, C.c_int, C.c_int]
        for f in ("orc_ic_rp2d3", "orc_ic_sedov", "orc_ic_dmr", "orc_ic_vortex"):
            getattr(L, f).argtypes = [P(OrcParams), dp]
        L.orc_run.argtypes = [C.c_void_p, dp, P(C.c_double), C.c_int, P(C.c_longlong)]
        L.orc_num_threads.restype = C.c_int
        L.orc_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def make_params(lf, nf, *, lx=1.0, ly=1.0, tmax=0.8, mord=5, ngp=3, method=GP_MOOD, bc=NEUMANN, cfl=0.8,
                ell_o_dx=12.0, dmp=1, u2=1, u2_tol=1, integrator=SSP_RK3, num_flux=HLLC, setdt_kind=0, lf0=0,
                nf0=0, slow_start=0.0, csd_kind=0) -> OrcParams:
    """The knobs of parameters.f90; setdt_kind, lf0/nf0, slow_start and csd_kind
    select the deprecated code line's time step and shock detector (see
    gpmood_oracle.h)."""
    return OrcParams(cfl, ell_o_dx, lx, ly, tmax, mord, ngp, method, dmp, u2, u2_tol, lf, nf, bc, integrator,
                     num_flux, setdt_kind, lf0, nf0, slow_start, csd_kind)


def padded(lf: int, nf: int) -> np.ndarray:
    """U(4, lb:le, nb:ne) as a C array of shape (nf+8, lf+8, 4)."""
    return np.zeros((nf + 2 * NGC, lf + 2 * NGC, 4), dtype=np.float64)


def gp_weights(p: OrcParams) -> OrcGp:
    g = OrcGp()
    rc = lib().orc_gp_presim(C.byref(p), C.byref(g))
    if rc != 0:
        raise ValueError("oracle GP precompute rejected the knobs")
    return g


def initial_condition(p: OrcParams, name: str) -> np.ndarray:
    U = padded(p.lf, p.nf)
    getattr(lib(), {"rp2d3": "orc_ic_rp2d3", "sedov": "orc_ic_sedov", "dmr": "orc_ic_dmr",
                    "vortex": "orc_ic_vortex"}[name])(C.byref(p), U)
    return U


def setdt(p: OrcParams, U: np.ndarray, dtfinal: float) -> float:
    return lib().orc_setdt(C.byref(p), U, dtfinal)


def boundary(p: OrcParams, U: np.ndarray, t_rk: float = 0.0) -> None:
    lib().orc_boundary(C.byref(p), U, t_rk)


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


class Stepper:
    """The reference's time_stepping with its module-global work arrays."""

    def __init__(self, p: OrcParams):
        self.p = p
        self._h = lib().orc_create(C.byref(p))
        if not self._h:
            raise ValueError("oracle context creation failed")
        self.counters = (C.c_longlong * 3)()

    def close(self):
        if self._h:
            lib().orc_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def weights(self) -> OrcGp:
        """The weights the context steps with (GP, or pol_presim's for POL_MOOD / Unlim_POL)."""
        return OrcGp.from_address(lib().orc_weights(self._h))

    def set_cc(self, col: int, w=None):
        """NN_GP_MOOD_CC_ blend of column `col` with row pairs w[nf+2, 2] (None: off)."""
        if w is None:
            lib().orc_set_cc(self._h, -1, None)
            return
        a = np.ascontiguousarray(w, dtype=np.float32).reshape(self.p.nf + 2, 2)
        lib().orc_set_cc(self._h, int(col), a.ctypes.data)

    def time_stepping(self, Uin: np.ndarray, Uout: np.ndarray, t: float, dt: float,
                      init_orders=None, want_orders: bool = False):
        """One SSP-RK3 step.  Returns the three per-stage CellGPO masks if asked."""
        lf, nf = self.p.lf, self.p.nf
        init_ptr = None
        keep = []
        if init_orders is not None:
            arrs = [np.ascontiguousarray(o, dtype=np.int8).reshape(nf, lf) for o in init_orders]
            keep += arrs
            ptrs = (C.c_void_p * 3)(*[a.ctypes.data for a in arrs])
            keep.append(ptrs)
            init_ptr = C.cast(ptrs, C.c_void_p)
        out_ptr = None
        masks = None
        if want_orders:
            masks = [np.zeros((nf, lf), dtype=np.int8) for _ in range(3)]
            optrs = (C.c_void_p * 3)(*[m.ctypes.data for m in masks])
            keep.append(optrs)
            out_ptr = C.cast(optrs, C.c_void_p)
        rc = lib().orc_time_stepping(self._h, Uin, Uout, t, dt, init_ptr, out_ptr, self.counters)
        if rc != 0:
            raise RuntimeError(f"oracle time_stepping failed ({rc})")
        return masks

    def run(self, U: np.ndarray, t: float, nsteps: int) -> tuple[float, int]:
        tt = C.c_double(t)
        n = lib().orc_run(self._h, U, C.byref(tt), nsteps, self.counters)
        if n < 0:
            raise RuntimeError(f"oracle run failed ({n})")
        return tt.value, n
