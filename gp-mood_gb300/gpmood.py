"""Python host side of the GB300 GP-MOOD step: a ctypes binding of libgpmood.so.

Mirrors the reference's Fortran interface for the per-step path under the
same names: ``time_stepping`` (gp-mood-code/time_stepper.f90:12),
``Setdt`` (gp-mood-code/physics.f90:78), ``Boundary_C`` (gp-mood-code/BC.f90:10)
and the knobs of ``parameters.f90``.  State arrays use the reference layout
U(4, lb:le, nb:ne), i.e. a C array of shape (nf+8, lf+8, 4).

There is no CPU fallback: importing this module without the built CUDA library
raises, and creating a Solver without a GPU raises.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libgpmood.so"

NGC = 4
# gp-mood-code/constants.f90:17-34
GP_MOOD, GP_SE, NN_GP_MOOD, NN_GP_MOOD_CC = 2, 202, 203, 204
POL_MOOD, UNLIM_POL = 200, 201  # mod_pol_MOOD.f90, mod_Unlim_Pol.f90: Mord 3, ngp 2
FOG = 1  # mod_FOG.f90: first-order Godunov, ngp 1
FE, SSP_RK2, SSP_RK3, SSP_RK4 = 8, 9, 10, 12
HLLC, LLF, HLL, UNSPLIT = 100, 101, 102, 103
NEUMANN, PERIODIC, REFLECTIVE, DMR = 17, 18, 20, 35
DIRICHLET, MACH800, DOUBLE_MACH800, RMI, RT, KH = 19, 201, 301, 401, 402, 403  # BC.f90, constants.f90:24-25
FP_EXACT, FP_FAST = 0, 1

E_ARG, E_CUDA, E_MOOD_CAP, E_DT, E_STATE = -1, -2, -3, -4, -5
NN_NPARAMS = 64 * 36 + 64 + 64 * 64 + 64 + 64 + 1


class GpmoodError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gpmood error {code}: {msg}")
        self.code = code


class Params(C.Structure):
    """gpmood_params of include/gpmood.h (parameters.f90 knobs)."""
    _fields_ = [("cfl", C.c_double), ("ell_o_dx", C.c_double), ("lx", C.c_double), ("ly", C.c_double),
                ("tmax", C.c_double), ("integrator", C.c_int), ("method", C.c_int), ("mord", C.c_int),
                ("ngp", C.c_int), ("dmp", C.c_int), ("u2", C.c_int), ("u2_tol", C.c_int), ("num_flux", C.c_int),
                ("lf", C.c_int), ("nf", C.c_int), ("bc_type", C.c_int), ("nmax", C.c_int), ("fp_mode", C.c_int),
                ("max_mood_iters", C.c_int), ("nsteps_with_no_nn", C.c_int), ("nn_reference", C.c_int)]


class Counters(C.Structure):
    _fields_ = [("detected_last_step", C.c_longlong), ("detected_total", C.c_longlong),
                ("a_priori_last_step", C.c_longlong), ("mood_passes_last_step", C.c_longlong),
                ("max_passes_stage", C.c_longlong), ("steps", C.c_longlong), ("status_flags", C.c_longlong),
                ("kernel_launches", C.c_longlong)]


class Timing(C.Structure):
    _fields_ = [("flux_ms", C.c_double), ("flux_launches", C.c_longlong), ("flux_faces", C.c_longlong),
                ("update_ms", C.c_double), ("update_launches", C.c_longlong), ("mood_ms", C.c_double),
                ("mood_passes", C.c_longlong)]


# Every entry point of include/gpmood.h with its ctypes signature.
_DP = C.POINTER(C.c_double)
SIGNATURES = {
    "gpmood_default_params": ([C.POINTER(Params)], C.c_int),
    "gpmood_create": ([C.POINTER(Params), C.POINTER(C.c_void_p)], C.c_int),
    "gpmood_destroy": ([C.c_void_p], None),
    "gpmood_last_error": ([C.c_void_p, C.c_char_p, C.c_int], C.c_int),
    "gpmood_get_weights": ([C.c_void_p, _DP, _DP, _DP], C.c_int),
    "gpmood_gp_weights": ([C.POINTER(Params), _DP, _DP, _DP], C.c_int),
    "gpmood_boundary_c": ([C.c_void_p, _DP, C.c_double], C.c_int),
    "gpmood_setdt": ([C.c_void_p, _DP, C.c_double, _DP], C.c_int),
    "gpmood_time_stepping": ([C.c_void_p, _DP, _DP, C.c_double, C.c_double], C.c_int),
    "gpmood_setdt_time_stepping": ([C.c_void_p, _DP, _DP, C.c_double, C.c_double, C.POINTER(C.c_double)], C.c_int),
    "gpmood_set_state": ([C.c_void_p, _DP, C.c_double], C.c_int),
    "gpmood_get_state": ([C.c_void_p, _DP, _DP, C.POINTER(C.c_int)], C.c_int),
    "gpmood_get_orders": ([C.c_void_p, C.POINTER(C.c_byte)], C.c_int),
    "gpmood_advance": ([C.c_void_p, C.c_int, C.POINTER(C.c_int)], C.c_int),
    "gpmood_get_counters": ([C.c_void_p, C.POINTER(Counters)], C.c_int),
    "gpmood_time_stepping_dev": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double], C.c_int),
    "gpmood_set_nn": ([C.c_void_p, C.POINTER(C.c_float), C.c_int], C.c_int),
    "gpmood_set_nn_threshold": ([C.c_void_p, C.c_float], C.c_int),
    "gpmood_set_wait_limit": ([C.c_void_p, C.c_int], C.c_int),
    "gpmood_set_nn_repair": ([C.c_void_p, C.c_int], C.c_int),
    "gpmood_nn_ref_logits": ([C.c_void_p, C.c_void_p], C.c_int),
    "gpmood_nn_gate_logits": ([C.c_void_p, C.c_void_p], C.c_int),
    "gpmood_nn_predict": ([C.c_void_p, C.POINTER(C.c_byte), C.POINTER(C.c_longlong)], C.c_int),
    "gpmood_get_stage_orders": ([C.c_void_p, C.c_int, C.POINTER(C.c_byte)], C.c_int),
    "gpmood_nn_features": ([C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "gpmood_nn_harvest": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_float, C.c_uint, C.c_void_p], C.c_int),
    "gpmood_nn_forward": ([C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p], C.c_int),
    "gpmood_nn_loss_grad": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_float, C.c_void_p, C.c_void_p,
                             C.c_void_p], C.c_int),
    "gpmood_nn_adam": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_float, C.c_float, C.c_float,
                        C.c_float, C.c_void_p], C.c_int),
    "gpmood_get_stream": ([C.c_void_p], C.c_void_p),
    "gpmood_set_timing": ([C.c_void_p, C.c_int], C.c_int),
    "gpmood_get_timing": ([C.c_void_p, C.POINTER(Timing)], C.c_int),
    "gpmood_probe_fp64": ([_DP], C.c_int),
    "gpmood_probe_fp64_pipes": ([_DP], C.c_int),
    "gpmood_fast_rcp": ([C.c_void_p, C.c_void_p, C.c_int], C.c_int),
    "gpmood_fast_sqrt": ([C.c_void_p, C.c_void_p, C.c_int], C.c_int),
    "gpmood_time_stepping_noalloc": ([C.POINTER(Params), C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                                      C.c_void_p, C.POINTER(C.c_int)], C.c_int),
    "gpmood_batch_create": ([C.POINTER(Params), C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                             C.POINTER(C.c_void_p)], C.c_int),
    "gpmood_batch_destroy": ([C.c_void_p], None),
    "gpmood_batch_set_state": ([C.c_void_p, C.c_int, _DP, C.c_double], C.c_int),
    "gpmood_batch_get_state": ([C.c_void_p, C.c_int, _DP, _DP], C.c_int),
    "gpmood_batch_advance": ([C.c_void_p, C.c_int], C.c_int),
    "gpmood_batch_autotune": ([C.c_void_p, C.POINTER(C.c_int), _DP], C.c_int),
    "gpmood_batch_stats": ([C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                            C.POINTER(C.c_longlong), C.POINTER(C.c_int)], C.c_int),
    "gpmood_set_state_dev": ([C.c_void_p, C.c_void_p, C.c_double], C.c_int),
    "gpmood_get_state_dev": ([C.c_void_p, C.c_void_p], C.c_int),
    "gpmood_adj_record": ([C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_void_p)], C.c_int),
    "gpmood_adj_destroy": ([C.c_void_p], None),
    "gpmood_adj_info": ([C.c_void_p, C.POINTER(C.c_int), _DP, _DP], C.c_int),
    "gpmood_adj_orders": ([C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_byte)], C.c_int),
    "gpmood_adj_replay": ([C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "gpmood_adj_backward": ([C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
}

_lib: C.CDLL | None = None


def load_library() -> C.CDLL:
    """Load libgpmood.so; raise if it has not been built (no fallback)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
        L = C.CDLL(str(LIB_PATH))
        for name, (args, res) in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_DP)


def padded(lf: int, nf: int) -> np.ndarray:
    """A zero state U(4, lb:le, nb:ne) as a C array of shape (nf+8, lf+8, 4)."""
    return np.zeros((nf + 2 * NGC, lf + 2 * NGC, 4), dtype=np.float64)


def default_params(**kw) -> Params:
    p = Params()
    load_library().gpmood_default_params(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise TypeError(f"unknown knob {k}")
        setattr(p, k, v)
    return p


def gp_weights(params: Params):
    """GP_presim_sphere on the host (no GPU): zt[3][4][ngp][13], d2[2][5], inv_err[3]."""
    zt = np.zeros((3, 4, params.ngp, 13))
    d2 = np.zeros((2, 5))
    inv = np.zeros(3)
    L = load_library()
    rc = L.gpmood_gp_weights(C.byref(params), _dp(zt), _dp(d2), _dp(inv))
    if rc != 0:
        buf = C.create_string_buffer(512)
        L.gpmood_last_error(None, buf, 512)
        raise GpmoodError(rc, buf.value.decode(errors="replace"))
    return zt, d2, inv


def probe_fp64() -> float:
    """FP64 FMA throughput of the current GPU in GFLOP/s (2 flops per FMA)."""
    g = C.c_double()
    L = load_library()
    rc = L.gpmood_probe_fp64(C.byref(g))
    if rc != 0:
        buf = C.create_string_buffer(512)
        L.gpmood_last_error(None, buf, 512)
        raise GpmoodError(rc, buf.value.decode(errors="replace"))
    return g.value


def probe_fp64_pipes() -> dict:
    """GFLOP/s of FP64 FMA chains alone, FP64 m8n8k4 MMAs alone, and both at
    once (half the warps each): whether the tensor-core path adds FP64 rate."""
    g = (C.c_double * 3)()
    L = load_library()
    rc = L.gpmood_probe_fp64_pipes(g)
    if rc != 0:
        buf = C.create_string_buffer(512)
        L.gpmood_last_error(None, buf, 512)
        raise GpmoodError(rc, buf.value.decode(errors="replace"))
    return {"dfma": g[0], "dmma": g[1], "mixed": g[2]}


@dataclass
class StepInfo:
    detected: int
    passes: int


class Solver:
    """One GP-MOOD context on the current GPU (gpmood_create .. gpmood_destroy)."""

    def __init__(self, params: Params | None = None, **kw):
        self.lib = load_library()
        self.p = params if params is not None else default_params(**kw)
        if params is not None:
            for k, v in kw.items():
                setattr(self.p, k, v)
        h = C.c_void_p()
        rc = self.lib.gpmood_create(C.byref(self.p), C.byref(h))
        if rc != 0:
            raise GpmoodError(rc, self._err(None))
        self._h = h
        self.lf, self.nf = self.p.lf, self.p.nf

    def _err(self, h) -> str:
        buf = C.create_string_buffer(512)
        self.lib.gpmood_last_error(h, buf, 512)
        return buf.value.decode(errors="replace")

    def _check(self, rc: int) -> None:
        if rc != 0:
            raise GpmoodError(rc, self._err(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self.lib.gpmood_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- shapes -----------------------------------------------------------
    @property
    def shape(self) -> tuple[int, int, int]:
        return (self.nf + 2 * NGC, self.lf + 2 * NGC, 4)

    def _state(self, U: np.ndarray, name: str) -> np.ndarray:
        if U.shape != self.shape or U.dtype != np.float64 or not U.flags.c_contiguous:
            raise ValueError(f"{name} must be a C-contiguous float64 array of shape {self.shape}")
        return U

    # -- reference-facing calls ----------------------------------------
    def weights(self):
        zt = np.zeros((3, 4, self.p.ngp, 13))
        d2 = np.zeros((2, 5))
        inv = np.zeros(3)
        self._check(self.lib.gpmood_get_weights(self._h, _dp(zt), _dp(d2), _dp(inv)))
        return zt, d2, inv

    def Boundary_C(self, U: np.ndarray, t_rk: float = 0.0) -> None:
        self._check(self.lib.gpmood_boundary_c(self._h, _dp(self._state(U, "U")), t_rk))

    def Setdt(self, U: np.ndarray, dtfinal: float) -> float:
        dt = C.c_double()
        self._check(self.lib.gpmood_setdt(self._h, _dp(self._state(U, "U")), dtfinal, C.byref(dt)))
        return dt.value

    def time_stepping(self, Uin: np.ndarray, Uout: np.ndarray, t: float, dt: float) -> StepInfo:
        self._check(self.lib.gpmood_time_stepping(self._h, _dp(self._state(Uin, "Uin")),
                                                  _dp(self._state(Uout, "Uout")), t, dt))
        c = self.counters()
        return StepInfo(c.detected_last_step, c.mood_passes_last_step)

    def time_stepping_ptr(self, uin_ptr: int, uout_ptr: int, t: float, dt: float) -> None:
        """One step on host pointers (e.g. pinned torch tensors), same layout."""
        self._check(self.lib.gpmood_time_stepping(self._h, C.cast(C.c_void_p(uin_ptr), _DP),
                                                  C.cast(C.c_void_p(uout_ptr), _DP), t, dt))

    def setdt_ptr(self, u_ptr: int, dtfinal: float) -> float:
        dt = C.c_double()
        self._check(self.lib.gpmood_setdt(self._h, C.cast(C.c_void_p(u_ptr), _DP), dtfinal, C.byref(dt)))
        return dt.value

    def setdt_time_stepping_ptr(self, uin_ptr: int, uout_ptr: int, t: float, dtfinal: float) -> float:
        """Setdt + time_stepping in one call on host pointers (one upload, one
        download); returns the dt taken."""
        dt = C.c_double()
        self._check(self.lib.gpmood_setdt_time_stepping(self._h, C.cast(C.c_void_p(uin_ptr), _DP),
                                                        C.cast(C.c_void_p(uout_ptr), _DP), t, dtfinal,
                                                        C.byref(dt)))
        return dt.value

    def time_stepping_dev(self, d_uin: int, d_uout: int, t: float, dt: float) -> None:
        self._check(self.lib.gpmood_time_stepping_dev(self._h, C.c_void_p(d_uin), C.c_void_p(d_uout), t, dt))

    # -- device-resident run ------------------------------------------------
    def set_state(self, U: np.ndarray, t: float = 0.0) -> None:
        self._check(self.lib.gpmood_set_state(self._h, _dp(self._state(U, "U")), t))

    def get_state(self):
        U = np.empty(self.shape)
        t = C.c_double()
        n = C.c_int()
        self._check(self.lib.gpmood_get_state(self._h, _dp(U), C.byref(t), C.byref(n)))
        return U, t.value, n.value

    def advance(self, nsteps: int) -> int:
        done = C.c_int()
        self._check(self.lib.gpmood_advance(self._h, int(nsteps), C.byref(done)))
        return done.value

    def orders(self) -> np.ndarray:
        o = np.zeros((self.nf, self.lf), dtype=np.int8)
        self._check(self.lib.gpmood_get_orders(self._h, o.ctypes.data_as(C.POINTER(C.c_byte))))
        return o

    def counters(self) -> Counters:
        c = Counters()
        self._check(self.lib.gpmood_get_counters(self._h, C.byref(c)))
        return c

    # -- measurement --------------------------------------------------------
    @property
    def stream(self) -> int:
        """The context's cudaStream_t as an integer handle."""
        return int(self.lib.gpmood_get_stream(self._h) or 0)

    def set_timing(self, on: bool) -> None:
        self._check(self.lib.gpmood_set_timing(self._h, 1 if on else 0))

    def timing(self) -> Timing:
        t = Timing()
        self._check(self.lib.gpmood_get_timing(self._h, C.byref(t)))
        return t

    def set_nn(self, params: np.ndarray) -> None:
        a = np.ascontiguousarray(params, dtype=np.float32).ravel()
        self._check(self.lib.gpmood_set_nn(self._h, a.ctypes.data_as(C.POINTER(C.c_float)), a.size))

    def nn_ref_logits(self, d_logits: int) -> None:
        """r(1), r(2) of the reference's network for every interior cell (device array)."""
        self._check(self.lib.gpmood_nn_ref_logits(self._h, C.c_void_p(d_logits)))

    def nn_gate_logits(self, d_logits: int) -> None:
        """The gate's logit of every interior cell (device float array of lf*nf)."""
        self._check(self.lib.gpmood_nn_gate_logits(self._h, C.c_void_p(d_logits)))

    def set_nn_repair(self, on: bool) -> None:
        """The gate's extras repair: gated cells that pass DETECTION at Mord get Mord back."""
        self._check(self.lib.gpmood_set_nn_repair(self._h, int(bool(on))))

    def set_wait_limit(self, polls: int) -> None:
        """Test hook: bound the kernels' spin-waits to `polls` polls (0: ~1 s)."""
        self._check(self.lib.gpmood_set_wait_limit(self._h, int(polls)))

    def set_nn_threshold(self, logit_threshold: float) -> None:
        self._check(self.lib.gpmood_set_nn_threshold(self._h, float(logit_threshold)))

    def nn_predict(self):
        """Gate decision on the device-resident state: (mask [nf, lf] int8, count)."""
        m = np.zeros((self.nf, self.lf), dtype=np.int8)
        n = C.c_longlong()
        self._check(self.lib.gpmood_nn_predict(self._h, m.ctypes.data_as(C.POINTER(C.c_byte)), C.byref(n)))
        return m, n.value

    def stage_orders(self, stage: int) -> np.ndarray:
        o = np.zeros((self.nf, self.lf), dtype=np.int8)
        self._check(self.lib.gpmood_get_stage_orders(self._h, int(stage), o.ctypes.data_as(C.POINTER(C.c_byte))))
        return o

    def nn_features(self, d_x: int, d_const: int = 0) -> None:
        self._check(self.lib.gpmood_nn_features(self._h, C.c_void_p(d_x), C.c_void_p(d_const or None)))

    def save_snapshot(self, path, problem: str = "", nn_filename: str = "") -> None:
        """The device-resident state as a snapshot file (snapshot.py; the
        datasets of the reference's output.f90:77-192)."""
        from . import snapshot
        U, t, n = self.get_state()
        method = {GP_MOOD: "GP_MOOD", GP_SE: "GP_SE", NN_GP_MOOD: "NN_GP_MOOD", NN_GP_MOOD_CC: "NN_GP_MOOD_CC",
                  POL_MOOD: "POL_MOOD", UNLIM_POL: "Unlim_POL", FOG: "FOG"}.get(self.p.method, str(self.p.method))
        snapshot.save_snapshot(path, U, t, n, self.orders(), cfl=self.p.cfl, problem=problem, method=method,
                               nn_filename=nn_filename)

    def restore(self, path) -> dict:
        """Restart from a snapshot file (reader.f90:12-120): primitive fields ->
        conservative state, Boundary_C at the snapshot's time, set_state."""
        from . import snapshot
        snap = snapshot.load_snapshot(path)
        if (int(snap["lf"]), int(snap["nf"])) != (self.lf, self.nf):
            raise ValueError(f"snapshot is {snap['lf']}x{snap['nf']}, the solver {self.lf}x{self.nf}")
        U = snapshot.state_from_snapshot(snap)
        self.Boundary_C(U, float(snap["time"]))
        self.set_state(U, float(snap["time"]))
        return snap

    def set_state_dev(self, d_u: int, t: float = 0.0) -> None:
        self._check(self.lib.gpmood_set_state_dev(self._h, C.c_void_p(d_u), float(t)))

    def get_state_dev(self, d_u: int) -> None:
        self._check(self.lib.gpmood_get_state_dev(self._h, C.c_void_p(d_u)))

    def adj_record(self, nsteps: int, every: int = 10) -> "Adjoint":
        """Advance nsteps steps recording dt and the frozen order masks, with a
        state checkpoint every ``every`` steps (gpmood_adj_record)."""
        h = C.c_void_p()
        self._check(self.lib.gpmood_adj_record(self._h, int(nsteps), int(every), C.byref(h)))
        return Adjoint(self, h)

    def nn_harvest(self, d_x: int, d_y: int, capacity: int, keep_negative: float, seed: int, d_count: int) -> None:
        """Attach (d_x != 0) or detach (d_x == 0) training-sample buffers."""
        self._check(self.lib.gpmood_nn_harvest(self._h, C.c_void_p(d_x or None), C.c_void_p(d_y or None),
                                               int(capacity), float(keep_negative), int(seed) & 0xFFFFFFFF,
                                               C.c_void_p(d_count or None)))


class Adjoint:
    """A recording of steps with frozen MOOD order masks (gpmood_adj_*): frozen
    replay and the vector-Jacobian product along the recorded trajectory.
    Device arrays are passed as integer pointers to padded-layout float64 data."""

    def __init__(self, solver: Solver, handle):
        self.solver = solver
        self.lib = solver.lib
        self._h = handle
        n = C.c_int()
        self.lib.gpmood_adj_info(self._h, C.byref(n), None, None)
        self.nsteps = n.value

    def _check(self, rc: int) -> None:
        if rc != 0:
            raise GpmoodError(rc, self.solver._err(self.solver._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self.lib.gpmood_adj_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def info(self):
        """(t, dt) of every recorded step."""
        t = np.zeros(self.nsteps)
        dt = np.zeros(self.nsteps)
        self._check(self.lib.gpmood_adj_info(self._h, None, _dp(t), _dp(dt)))
        return t, dt

    def orders(self, step: int, stage: int) -> np.ndarray:
        """Padded CellGPO (nf+8, lf+8) of RK stage ``stage`` of step ``step``."""
        o = np.zeros(self.solver.shape[:2], dtype=np.int8)
        self._check(self.lib.gpmood_adj_orders(self._h, int(step), int(stage), o.ctypes.data_as(C.POINTER(C.c_byte))))
        return o

    def replay(self, d_u0: int, d_uN: int) -> None:
        self._check(self.lib.gpmood_adj_replay(self._h, C.c_void_p(d_u0), C.c_void_p(d_uN)))

    def backward(self, d_lamN: int, d_lam0: int) -> None:
        self._check(self.lib.gpmood_adj_backward(self._h, C.c_void_p(d_lamN), C.c_void_p(d_lam0)))


class Batch:
    """Many independent problems of uneven size stepped together (gpmood_batch_*)."""

    def __init__(self, sizes, params: Params | None = None, **kw):
        self.lib = load_library()
        self.p = params if params is not None else default_params(**kw)
        self.sizes = [(int(a), int(b)) for a, b in sizes]
        n = len(self.sizes)
        lf = (C.c_int * n)(*[a for a, _ in self.sizes])
        nf = (C.c_int * n)(*[b for _, b in self.sizes])
        h = C.c_void_p()
        rc = self.lib.gpmood_batch_create(C.byref(self.p), n, lf, nf, C.byref(h))
        if rc != 0:
            raise GpmoodError(rc, self._err())
        self._h = h

    def _err(self) -> str:
        buf = C.create_string_buffer(512)
        self.lib.gpmood_last_error(None, buf, 512)
        return buf.value.decode(errors="replace")

    def _check(self, rc: int) -> None:
        if rc != 0:
            raise GpmoodError(rc, self._err())

    def close(self) -> None:
        if getattr(self, "_h", None):
            self.lib.gpmood_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_state(self, i: int, U: np.ndarray, t: float = 0.0) -> None:
        lf, nf = self.sizes[i]
        if U.shape != (nf + 2 * NGC, lf + 2 * NGC, 4) or U.dtype != np.float64 or not U.flags.c_contiguous:
            raise ValueError("state has the wrong shape or dtype")
        self._check(self.lib.gpmood_batch_set_state(self._h, i, _dp(U), t))

    def get_state(self, i: int):
        lf, nf = self.sizes[i]
        U = np.empty((nf + 2 * NGC, lf + 2 * NGC, 4))
        t = C.c_double()
        self._check(self.lib.gpmood_batch_get_state(self._h, i, _dp(U), C.byref(t)))
        return U, t.value

    def advance(self, nsteps: int) -> None:
        self._check(self.lib.gpmood_batch_advance(self._h, int(nsteps)))

    def autotune(self):
        k = C.c_int()
        ms = np.zeros(5)  # one time per tile shape (gpmood_batch_autotune)
        self._check(self.lib.gpmood_batch_autotune(self._h, C.byref(k), _dp(ms)))
        return k.value, ms

    def stats(self) -> dict:
        vals = [C.c_longlong() for _ in range(4)]
        g = C.c_int()
        self._check(self.lib.gpmood_batch_stats(self._h, *[C.byref(v) for v in vals], C.byref(g)))
        return {"interior_cells": vals[0].value, "steps": vals[1].value, "detected": vals[2].value,
                "status": vals[3].value, "graphed": g.value}
