#!/usr/bin/env python
"""Benchmark: FP64 cell-updates/s of the GP-MOOD step on the 2048x2048 Sedov
point blast (plain GP-MOOD, R2 -> R1 -> first order, HLLC, SSP-RK3, CFL 0.8,
reflecting BCs) on one GB300 per rank.

A step is one pass of the hot path over the grid: Setdt + time_stepping
(three RK stages with their MOOD loops) + t += dt.  Cell-updates/s counts
lf*nf per step, the reference's own definition (gp-mood-code/main.f90:214-215).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One JSON line is printed by rank 0.  --impl reference times the reference
algorithm on the host cores instead (the CPU oracle, since the Fortran
reference cannot be compiled on these machines).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_DEFAULT = 2048
TMAX = 0.05
# Algorithmic FP64 flops per face of the first-pass face kernel at ngp = 3,
# counting +,-,*,/,sqrt as one flop each: two 13-point GP reconstructions of 4
# variables at 3 Gauss points (2*3*4*25 = 600), 3 HLLC solves (3*103 = 309)
# and the quadrature (4*5 = 20).
FLOPS_PER_FACE = 929
# Algorithmic HBM bytes per cell-update of one full SSP-RK3 step: each stage
# reads its input (32 B) and writes its output (32 B); stages 2-3 also read U^n.
BYTES_PER_CELL_UPDATE = 256
FLOPS_PER_CELL_UPDATE = 5900


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--fp-mode", choices=("fast", "exact"), default="fast")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--nn", type=int, default=1, help="also time the NN-gated variant (0: skip)")
    ap.add_argument("--batch-problems", type=int, default=1024)
    ap.add_argument("--batch-steps", type=int, default=10, help="timed steps of the batched form (0: skip)")
    ap.add_argument("--adjoint", type=int, default=1, help="also time the adjoint form (0: skip)")
    ap.add_argument("--skip-plain", type=int, default=0, help="with --final: leave out the plain run")
    ap.add_argument("--repair", type=int, default=0,
                    help="with --final: also the NN-gated run with the gate's extras repair (gpmood_set_nn_repair)")
    ap.add_argument("--l1-ref", type=int, default=0,
                    help="with --final: also the plain run on the twice finer grid, and both runs' L1 errors against it")
    ap.add_argument("--dmr", type=int, default=1,
                    help="also time whole DMR runs, plain against NN-gated, with their L1 errors (0: skip)")
    ap.add_argument("--final", action="store_true",
                    help="run plain (and NN-gated unless --nn 0) GP-MOOD from t=0 to t_final and compare them")
    ap.add_argument("--case", choices=tuple(FINAL_CASES), default="sedov",
                    help="problem of --final: Sedov n^2 (t_final 0.05), 2DRP3 256^2 (0.8), DMR 4096x1024 (0.2)")
    return ap.parse_args()


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if (args.impl == "ours" and torch.cuda.is_available()) else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return ws, rank, local


def dist_barrier(ws: int) -> None:
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def dist_max(x: float, ws: int) -> float:
    """Max of a host scalar over the ranks (NCCL: through a device tensor)."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(cells_per_rank: int, steps: int, elapsed_ms: float, ws: int) -> float:
    """Whole-job throughput of ws independent replicas: the cell-updates of all
    ranks over the slowest rank's time."""
    return ws * cells_per_rank * steps / (dist_max(elapsed_ms, ws) * 1e-3)


def workload_name(n):
    return (f"2D Sedov point blast {n}x{n} on [0,1]^2, E0=1 within 3.5dx, rho=1, p=1e-5, reflecting BCs; "
            f"plain GP-MOOD Mord=5 (R2->R1->1), ngp=3, ell=12dx, HLLC, SSP-RK3, CFL 0.8")


class ClockSampler:
    """nvidia-smi SM clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        return None


# DRAM bytes per face of one launch of the fast two-direction face kernel
# (k_flux_xy_tma) on the 2048^2 Sedov first pass, from one ncu capture of this
# workload: dram__bytes_read.sum + dram__bytes_write.sum = 136.13 MB + 208.49 MB
# over 8,392,704 faces.  A constant of that capture, not a live measurement.
DRAM_BYTES_PER_FACE_NCU = 41.06


def cpu_oracle_rate(n, steps, threads):
    """Reference algorithm (the CPU oracle) on the same Sedov workload."""
    import __graft_entry__ as ge
    O = ge.import_oracle()
    O.build()
    O.set_threads(threads)
    p = O.make_params(n, n, bc=O.REFLECTIVE, tmax=TMAX)
    U = O.initial_condition(p, "sedov")
    st = O.Stepper(p)
    t0 = time.perf_counter()
    _, k = st.run(U, 0.0, steps)
    el = time.perf_counter() - t0
    return n * n * k / el, k, el


GATE = ROOT / "gp-mood_gb300" / "gates" / "gate_sedov_rp2d3.txt"


def _rel_l1(a, b):
    import numpy as np
    I = (slice(4, -4), slice(4, -4))
    return [float(np.abs(a[I + (k,)] - b[I + (k,)]).sum() / np.abs(b[I + (k,)]).sum()) for k in range(4)]


def measure_nn_gated(pkg, n, K, W, fp, U0, plain_final, plain_ms, diag_steps=5):
    """The same K timed steps with the MLP gate (method NN_GP_MOOD), the gate's
    flags against plain MOOD's stage-1 decisions, and the state difference."""
    import numpy as np
    import torch
    from gpmood_gb300 import nn_train as T
    if not GATE.exists():
        return {"unavailable": f"no trained gate parameters ({GATE.name})"}
    params = T.load_text(str(GATE))
    meta_f = GATE.with_suffix(".json")
    thr = float(json.loads(meta_f.read_text()).get("threshold", 0.0)) if meta_f.exists() else 0.0
    with pkg.Solver(lf=n, nf=n, bc_type=pkg.REFLECTIVE, tmax=TMAX, fp_mode=fp, method=pkg.NN_GP_MOOD) as s:
        s.set_nn(params)
        s.set_nn_threshold(thr)
        s.set_state(U0, 0.0)
        s.advance(W)
        det0 = s.counters().detected_total
        stream = torch.cuda.ExternalStream(s.stream)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        done = s.advance(K)
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
        det = s.counters().detected_total - det0
        Ug, tg, _ = s.get_state()
    Up, tp = plain_final
    # gate decisions against plain MOOD on the plain trajectory (untimed)
    missed = extra = hits = 0
    with pkg.Solver(lf=n, nf=n, bc_type=pkg.REFLECTIVE, tmax=TMAX, fp_mode=fp) as s:
        s.set_nn(params)
        s.set_nn_threshold(thr)
        s.set_state(Up, tp)
        for _ in range(diag_steps):
            gated, _ = s.nn_predict()
            s.advance(1)
            low = s.stage_orders(0) < 5
            g = gated.astype(bool)
            hits += int((g & low).sum())
            missed += int((~g & low).sum())
            extra += int((g & ~low).sum())
    return {"value": n * n * done / (ms * 1e-3), "unit": "cell-updates/s", "ms_per_step": ms / max(done, 1),
            "speedup_vs_plain": plain_ms / (ms / max(done, 1)), "steps": done,
            "rel_l1_vs_plain_after_steps": _rel_l1(Ug, Up), "t_gated": tg, "t_plain": tp,
            "a_posteriori_detections_timed_steps": det, "logit_threshold": thr,
            "gate_vs_plain_stage1": {"steps": diag_steps, "hits": hits, "missed": missed, "extra": extra},
            "gate": GATE.name}


def measure_batched(pkg, nprob, steps, fp):
    """The batched form: nprob seeded four-quadrant Riemann problems of sizes
    {64,96,128,192,256}^2 stepped together (persistent kernels, CUDA graphs)."""
    import numpy as np
    import torch
    from gpmood_gb300 import ic
    sizes, states = [], []
    for i in range(nprob):
        U, m = ic.random_riemann(i)
        # Boundary_C with BC_type 17 (Neumann): ghosts copy the edge cells
        states.append(np.ascontiguousarray(np.pad(U[4:-4, 4:-4], ((4, 4), (4, 4), (0, 0)), mode="edge")))
        sizes.append((m, m))
    with pkg.Batch(sizes, lf=64, nf=64, bc_type=pkg.NEUMANN, tmax=1e30, fp_mode=fp) as b:
        for i, U in enumerate(states):
            b.set_state(i, U, 0.0)
        tile, tile_ms = b.autotune()
        b.advance(3)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.advance(steps)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        st = b.stats()
    cells = st["interior_cells"]
    return {"workload": f"{nprob} seeded 4-quadrant Riemann problems (PCG64 seed = index; rho~U[0.1,2], "
                        f"p~U[0.02,2], u,v~U[-1.5,1.5], split~U[0.3,0.8]^2, size~U{{64,96,128,192,256}}^2), "
                        f"Neumann BCs, per-problem dt",
            "value": cells * steps / el, "unit": "cell-updates/s", "ms_per_step": 1e3 * el / steps,
            "timed_steps": steps, "warmup": 3, "interior_cells": cells, "graphed": st["graphed"],
            "tile": int(tile), "tile_flux_ms": [float(x) for x in tile_ms], "status": st["status"],
            "timing": "host clock around gpmood_batch_advance (synchronous) with device sync on both sides"}


def measure_adjoint(pkg):
    """The adjoint form: 50 recorded steps of the 128^2 periodic vortex and
    the checkpointed backward (every 10 steps)."""
    import torch
    from gpmood_gb300 import ic
    n, nsteps, every = 128, 50, 10
    with pkg.Solver(lf=n, nf=n, lx=10.0, ly=10.0, bc_type=pkg.PERIODIC, tmax=1e30, fp_mode=pkg.FP_EXACT) as s:
        U = ic.isentropic_vortex(n, n, 10.0, 10.0, beta=5.0)
        s.Boundary_C(U, 0.0)
        s.set_state(U, 0.0)
        t0 = time.perf_counter()
        rec = s.adj_record(nsteps, every)
        t_rec = time.perf_counter() - t0
        lam = torch.zeros(s.shape, dtype=torch.float64, device="cuda")
        lam[4:-4, 4:-4, 0] = 1.0
        out = torch.empty_like(lam)
        rec.backward(lam.data_ptr(), out.data_ptr())  # warm-up
        t0 = time.perf_counter()
        rec.backward(lam.data_ptr(), out.data_ptr())
        t_bwd = time.perf_counter() - t0
        rec.close()
    return {"workload": "isentropic vortex beta=5, 128^2 periodic on [0,10]^2, 50 SSP-RK3 steps, J=sum rho^2 dxdy, "
                        "checkpoints every 10 steps",
            "forward_ms_per_step": 1e3 * t_rec / nsteps, "backward_ms_per_step": 1e3 * t_bwd / nsteps,
            "backward_over_forward": t_bwd / t_rec,
            "timing": "host clock around synchronous C-ABI calls (record = gpmood_advance with mask capture; "
                      "backward includes the segment recomputation)"}


# Whole runs of the benchmark problems (t = 0 to t_final): name -> (IC builder
# name, lf, nf, Lx, Ly, BC, t_final).
FINAL_CASES = {
    "sedov": ("sedov", None, None, 1.0, 1.0, 20, TMAX),
    "rp2d3": ("rp2d3", 256, 256, 1.0, 1.0, 17, 0.8),
    "dmr": ("dmr", 4096, 1024, 4.0, 1.0, 35, 0.2),
    "dmr_1024x256": ("dmr", 1024, 256, 4.0, 1.0, 35, 0.2),
    "dmr_256x64": ("dmr", 256, 64, 4.0, 1.0, 35, 0.2),
}


def whole_run(pkg, icname, lf, nf, lx, ly, bc, tfinal, fp, method, params=None, thr=0.0, repair=False):
    """One run from t = 0 to t_final, timed with CUDA events on the context's
    stream; returns (figures, final state)."""
    import torch
    from gpmood_gb300 import ic
    U0 = getattr(ic, icname)(lf, nf) if icname != "dmr" else ic.dmr(lf, nf, lx, ly)
    with pkg.Solver(lf=lf, nf=nf, lx=lx, ly=ly, bc_type=bc, tmax=tfinal, fp_mode=fp, method=method) as s:
        s.Boundary_C(U0, 0.0)
        if method == pkg.NN_GP_MOOD:
            s.set_nn(params)
            s.set_nn_threshold(thr)
            s.set_nn_repair(repair)
        s.set_state(U0, 0.0)
        s.set_timing(True)
        stream = torch.cuda.ExternalStream(s.stream)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        steps = s.advance(1 << 30)
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
        U, t, _ = s.get_state()
        c = s.counters()
        tm = s.timing()
    return ({"steps": steps, "t": t, "seconds": ms / 1e3, "value": lf * nf * steps / (ms * 1e-3),
             "unit": "cell-updates/s", "detected_total": c.detected_total,
             "max_passes_stage": c.max_passes_stage, "status_flags": c.status_flags,
             "flux_share": tm.flux_ms / ms if ms else None, "mood_share": tm.mood_ms / ms if ms else None,
             "mood_passes": tm.mood_passes,
             "us_per_mood_pass": tm.mood_ms * 1e3 / tm.mood_passes if tm.mood_passes else None,
             "final_state": {"sum_rho": float(U[4:-4, 4:-4, 0].sum()), "sum_E": float(U[4:-4, 4:-4, 3].sum())}},
            U)


def load_gate():
    from gpmood_gb300 import nn_train as T
    params = T.load_text(str(GATE))
    meta_f = GATE.with_suffix(".json")
    thr = float(json.loads(meta_f.read_text()).get("threshold", 0.0)) if meta_f.exists() else 0.0
    return params, thr


def run_final(args):
    """Plain (and, unless --nn 0, NN-gated) GP-MOOD from t = 0 to t_final on one
    of the benchmark problems: time to solution, steps, and the relative L1
    difference of the final states."""
    import __graft_entry__ as ge
    pkg = ge.import_package()
    icname, lf, nf, lx, ly, bc, tfinal = FINAL_CASES[args.case]
    lf = lf or args.n
    nf = nf or args.n
    fp = pkg.FP_FAST if args.fp_mode == "fast" else pkg.FP_EXACT
    params, thr = load_gate()
    out = {}
    finals = {}
    variants = [("plain", pkg.GP_MOOD, False)] + ([("nn_gated", pkg.NN_GP_MOOD, False)] if args.nn else [])
    if args.nn and args.repair:
        variants.append(("nn_gated_repaired", pkg.NN_GP_MOOD, True))
    if args.skip_plain:  # e.g. a long run whose plain half is on record already
        variants = [v for v in variants if v[0] != "plain"]
    for name, method, repair in variants:
        out[name], finals[name] = whole_run(pkg, icname, lf, nf, lx, ly, bc, tfinal, fp, method, params, thr, repair)
        # each variant on stderr as soon as it ends, so that a long run that is cut off still reports
        print(json.dumps({"partial": name, "case": args.case, **out[name]}), file=sys.stderr, flush=True)
    if args.nn and "plain" in out:
        out["nn_gated"]["speedup_vs_plain"] = out["plain"]["seconds"] / out["nn_gated"]["seconds"]
        out["rel_l1_final"] = _rel_l1(finals["nn_gated"], finals["plain"])
    if "nn_gated_repaired" in out and "plain" in out:
        out["nn_gated_repaired"]["speedup_vs_plain"] = out["plain"]["seconds"] / out["nn_gated_repaired"]["seconds"]
        out["nn_gated_repaired"]["rel_l1_vs_plain"] = _rel_l1(finals["nn_gated_repaired"], finals["plain"])
    if args.l1_ref:
        # L1 density errors against the plain run on the twice finer grid
        ref, Uref = whole_run(pkg, icname, 2 * lf, 2 * nf, lx, ly, bc, tfinal, fp, pkg.GP_MOOD, params, thr)
        out["l1_reference"] = {"grid": f"{2 * lf}x{2 * nf}", "seconds": ref["seconds"], "steps": ref["steps"]}
        for name in finals:
            out[name]["l1_rho_vs_2x_plain"] = l1_density_error(finals[name], Uref, lx, ly)
    line = {"metric": "time to t_final", "case": args.case,
            "workload": f"{icname} {lf}x{nf} on [0,{lx:g}]x[0,{ly:g}], BC {bc}, t_final={tfinal}, plain GP-MOOD "
                        f"Mord=5 (R2->R1->1), ngp=3, ell=12dx, HLLC, SSP-RK3, CFL 0.8",
            "fp_mode": args.fp_mode, "gate": GATE.name, "logit_threshold": thr, **out}
    print(json.dumps(line), flush=True)
    return 0


def l1_density_error(U, Uref, lx, ly):
    """sum |rho - R(rho_ref)| dx dy over the interior, R = the average of each
    2x2 block of the twice finer reference run (the L1 error against a
    converged solution, as the deprecated code's error() measures it)."""
    import numpy as np
    r = U[4:-4, 4:-4, 0]
    f = Uref[4:-4, 4:-4, 0]
    nf, lf = r.shape
    R = f.reshape(nf, 2, lf, 2).mean(axis=(1, 3))
    return float(np.abs(r - R).sum() * (lx / lf) * (ly / nf))


def measure_dmr_whole_runs(pkg, fp):
    """The oblique-shock (double Mach reflection) problem from t = 0 to 0.2, where
    plain MOOD's cascade crawls for hundreds of passes per stage: plain and
    NN-gated at 1024x256 (speed, final-state difference), and at 512x128 both
    runs' L1 density error against the plain 1024x256 run (the error at which
    the two speeds are compared)."""
    if not GATE.exists():
        return {"unavailable": f"no trained gate parameters ({GATE.name})"}
    params, thr = load_gate()
    lx, ly, bc, tf = 4.0, 1.0, 35, 0.2
    out = {"workload": "double Mach reflection (Mach-10 oblique shock) on [0,4]x[0,1], t_final=0.2, plain GP-MOOD "
                       "Mord=5 (R2->R1->1), ngp=3, ell=12dx, HLLC, SSP-RK3, CFL 0.8; the same with the BF16 gate",
           "gate": GATE.name, "logit_threshold": thr}
    fine = {}
    for name, method in (("plain", pkg.GP_MOOD), ("nn_gated", pkg.NN_GP_MOOD)):
        out[f"{name}_1024x256"], fine[name] = whole_run(pkg, "dmr", 1024, 256, lx, ly, bc, tf, fp, method, params, thr)
    out["speedup_1024x256"] = out["plain_1024x256"]["seconds"] / out["nn_gated_1024x256"]["seconds"]
    out["rel_l1_gated_vs_plain_1024x256"] = _rel_l1(fine["nn_gated"], fine["plain"])
    errs = {}
    for name, method in (("plain", pkg.GP_MOOD), ("nn_gated", pkg.NN_GP_MOOD)):
        fig, U = whole_run(pkg, "dmr", 512, 128, lx, ly, bc, tf, fp, method, params, thr)
        errs[name] = l1_density_error(U, fine["plain"], lx, ly)
        out[f"{name}_512x128"] = {"seconds": fig["seconds"], "steps": fig["steps"], "value": fig["value"],
                                  "l1_rho_vs_plain_1024x256": errs[name]}
    out["speedup_512x128"] = out["plain_512x128"]["seconds"] / out["nn_gated_512x128"]["seconds"]
    out["l1_ratio_gated_over_plain_512x128"] = errs["nn_gated"] / errs["plain"]
    out["timing"] = "CUDA events on the context's stream around gpmood_advance to t_final"
    return out


def run_final_reference(args):
    """The CPU oracle (all host cores) on the same whole run as run_final."""
    import numpy as np
    import __graft_entry__ as ge
    O = ge.import_oracle()
    O.build()
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    icname, lf, nf, lx, ly, bc, tfinal = FINAL_CASES[args.case]
    lf = lf or args.n
    nf = nf or args.n
    p = O.make_params(lf, nf, lx=lx, ly=ly, bc=bc, tmax=tfinal)
    U = O.initial_condition(p, icname)
    st = O.Stepper(p)
    t0 = time.perf_counter()
    t, k = st.run(U, 0.0, 1 << 30)
    el = time.perf_counter() - t0
    print(json.dumps({"impl": "reference", "metric": "time to t_final", "case": args.case,
                      "workload": f"{icname} {lf}x{nf}, BC {bc}, t_final={tfinal} (CPU oracle, OpenMP)",
                      "steps": k, "t": t, "seconds": el, "value": lf * nf * k / el, "unit": "cell-updates/s",
                      "cores": threads, "final_state": {"sum_rho": float(U[4:-4, 4:-4, 0].sum()),
                                                        "sum_E": float(U[4:-4, 4:-4, 3].sum())}}), flush=True)
    return 0


def run_reference(args, ws, rank):
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    n = args.n
    # Warm-up steps and timed steps of the oracle, each a full SSP-RK3 step of
    # the same grid (bounded: the oracle takes ~1 s per 2048^2 step on 16 cores).
    rate_w, _, _ = cpu_oracle_rate(n, max(1, min(args.warmup, 1)), threads)
    rate, k, el = cpu_oracle_rate(n, args.steps, threads)
    line = {
        "impl": "reference", "metric": "FP64 cell-updates/s", "value": rate, "unit": "cell-updates/s",
        "n_gpus": ws, "steps": k, "warmup": args.warmup, "ms_per_step": 1e3 * el / max(k, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(n), "implementation": "CPU restatement of the reference Fortran "
                   "(oracle/gpmood_oracle.c, OpenMP); the Fortran itself has no compiler on this host"},
        "cpu_baseline": {"value": rate, "unit": "cell-updates/s", "cores": threads, "kind": "port",
                         "sample": f"{k} SSP-RK3 steps of the {n}x{n} Sedov IC from t=0"},
        "e2e": {"value": rate, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args, ws, rank, local):
    import numpy as np
    import torch
    import __graft_entry__ as ge

    pkg = ge.import_package()
    from gpmood_gb300 import ic
    from gpmood_gb300.gpmood import probe_fp64, probe_fp64_pipes

    torch.cuda.set_device(local)
    n, K, W = args.n, args.steps, max(args.warmup, 3)
    fp = pkg.FP_FAST if args.fp_mode == "fast" else pkg.FP_EXACT
    U0 = ic.sedov(n, n)
    solver = pkg.Solver(lf=n, nf=n, bc_type=pkg.REFLECTIVE, tmax=TMAX, fp_mode=fp)
    solver.Boundary_C(U0, 0.0)
    state_bytes = U0.nbytes
    peak_fp64_gflops = probe_fp64()
    fp64_pipes = probe_fp64_pipes()

    def barrier():
        dist_barrier(ws)

    def max_over_ranks(x: float) -> float:
        return dist_max(x, ws)

    # ---- device-resident throughput (inputs in HBM) ----
    solver.set_state(U0, 0.0)
    solver.advance(W)
    stream = torch.cuda.ExternalStream(solver.stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = solver.counters().kernel_launches
    solver.set_timing(True)
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    ev0.record(stream)
    done = solver.advance(K)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    # the FP64 rate right after the timed region too: the denominator is the
    # higher of the two readings, so a change of the part's rate during the run
    # can only lower the reported fraction
    peak_after_gflops = probe_fp64()
    el_local = ev0.elapsed_time(ev1)
    value = replica_value(n * n, done, el_local, ws)
    el_ms = max_over_ranks(el_local)
    tm = solver.timing()
    ctr = solver.counters()
    Uend, t_end, _ = solver.get_state()
    checksum = {"t": t_end, "sum_rho": float(Uend[4:-4, 4:-4, 0].sum()),
                "sum_E": float(Uend[4:-4, 4:-4, 3].sum())}
    launches = ctr.kernel_launches - launches0

    # ---- end to end through the reference-facing C ABI with host buffers ----
    Uh = torch.empty(U0.shape, dtype=torch.float64).pin_memory()
    Urh = torch.empty(U0.shape, dtype=torch.float64).pin_memory()
    Uh.numpy()[...] = U0
    t = 0.0
    ke = max(1, args.e2e_steps)
    for _ in range(2):  # warm-up
        dt = solver.setdt_ptr(Uh.data_ptr(), TMAX - t)
        solver.time_stepping_ptr(Uh.data_ptr(), Urh.data_ptr(), t, dt)
        t += dt
        Uh, Urh = Urh, Uh
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(ke):
        dt = solver.setdt_ptr(Uh.data_ptr(), TMAX - t)
        solver.time_stepping_ptr(Uh.data_ptr(), Urh.data_ptr(), t, dt)
        t += dt
        Uh, Urh = Urh, Uh
    torch.cuda.synchronize()
    barrier()
    two_s = max_over_ranks(time.perf_counter() - t0)
    # the same steps through the one-call form (one upload of U per step)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(ke):
        dt = solver.setdt_time_stepping_ptr(Uh.data_ptr(), Urh.data_ptr(), t, TMAX - t)
        t += dt
        Uh, Urh = Urh, Uh
    torch.cuda.synchronize()
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e = {"value": ws * n * n * ke / e2e_s, "unit": "cell-updates/s",
           "h2d_bytes_per_step": state_bytes, "d2h_bytes_per_step": state_bytes,
           "path": "gpmood_setdt_time_stepping (Setdt + time_stepping in one call) on pinned host arrays "
                   "(Fortran layout), host clock",
           "two_calls": {"value": ws * n * n * ke / two_s, "h2d_bytes_per_step": 2 * state_bytes,
                         "d2h_bytes_per_step": state_bytes,
                         "path": "gpmood_setdt + gpmood_time_stepping, the reference's two calls"}}
    solver.close()

    # ---- roofline of the dominant kernel (first-pass face kernel) ----
    # one "launch" of the roofline = the first pass of one RK stage: every face
    # of the grid (fast mode: k_flux_xy_tma + k_flux_edge; exact: the x and y kernels)
    launch_ms = tm.flux_ms / max(tm.flux_launches, 1)
    faces_per_launch = tm.flux_faces / max(tm.flux_launches, 1)
    achieved_tflops = FLOPS_PER_FACE * faces_per_launch / (launch_ms * 1e-3) / 1e12
    peak_tflops = max(peak_fp64_gflops, peak_after_gflops) / 1e3
    tpf = DRAM_BYTES_PER_FACE_NCU if fp == pkg.FP_FAST else None  # the capture is of the fast kernel
    kname = ("first pass of one RK stage: k_flux_xy_tma (interior, both directions, TMA-staged halo tiles) + "
             "k_flux_edge (faces of ghost cells); GP recon + HLLC + quadrature" if fp == pkg.FP_FAST
             else "first pass of one RK stage: k_flux_tile x and y (GP recon + HLLC + quadrature)")
    roofline = {"bound": "fp64", "kernel": kname,
                "achieved": achieved_tflops, "peak": peak_tflops, "unit": "TFLOP/s",
                "frac": achieved_tflops / peak_tflops,
                "traffic": (tpf * faces_per_launch) if tpf else None,
                "peak_source": "FP64 FMA microbenchmark (gpmood_probe_fp64) run live on this GPU just before and "
                               "just after the timed region, the higher reading; MEASURED_PEAKS.json has no FP64 "
                               "figure",
                "peak_before_after": [peak_fp64_gflops / 1e3, peak_after_gflops / 1e3],
                "flops_per_face": FLOPS_PER_FACE, "faces_per_launch": faces_per_launch,
                "launch_ms": launch_ms, "share_of_step": tm.flux_ms / el_ms if el_ms else None}
    peaks = measured_peaks()
    hbm_peak = peaks.get("hbm_gbs") if peaks else 6800.0
    step_gbs = BYTES_PER_CELL_UPDATE * value / ws / 1e9
    roofline_hbm = {"bound": "hbm", "achieved": step_gbs, "peak": hbm_peak, "unit": "GB/s",
                    "frac": step_gbs / hbm_peak, "traffic": None,
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback 6.8 TB/s",
                    "note": "whole step, 256 algorithmic bytes per cell-update; the path is FP64-pipe bound"}

    forms = {}
    if args.nn:
        forms["nn_gated"] = measure_nn_gated(pkg, n, K, W, fp, U0, (Uend, t_end), el_ms / max(done, 1))
    if args.batch_steps > 0:
        forms["batched"] = measure_batched(pkg, args.batch_problems, args.batch_steps, fp)
    if args.adjoint:
        forms["adjoint"] = measure_adjoint(pkg)
    if args.dmr and args.nn:
        forms["dmr_whole_runs"] = measure_dmr_whole_runs(pkg, fp)

    cpu = None
    if rank == 0 and ws == 1 and args.cpu_steps > 0:
        threads = os.cpu_count() or 1
        rate, k, el = cpu_oracle_rate(n, args.cpu_steps, threads)
        cpu = {"value": rate, "unit": "cell-updates/s", "cores": threads, "kind": "port",
               "sample": f"{k} SSP-RK3 steps of the {n}x{n} Sedov IC from t=0 (CPU oracle, OpenMP)"}
        # the serial reference's stand-in: the same oracle on one thread, one step
        rate1, k1, _ = cpu_oracle_rate(n, 1, 1)
        cpu["serial"] = {"value": rate1, "cores": 1, "sample": f"{k1} SSP-RK3 step of the same IC, 1 thread"}

    line = {
        "metric": "FP64 cell-updates/s", "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": done,
        "warmup": W, "ms_per_step": el_ms / max(done, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(n), "variant": "plain GP-MOOD", "fp_mode": args.fp_mode,
                   "l2": "inputs larger than L2 (each state array is %.0f MB)" % (state_bytes / 1e6),
                   "parallelism": "replicas" if ws > 1 else "1 GPU",
                   "mood_passes_last_step": ctr.mood_passes_last_step,
                   "detected_last_step": ctr.detected_last_step, "final_state": checksum},
        "roofline": roofline, "roofline_hbm": roofline_hbm, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": launches, "clocks": clk,
        "fp64_peak_gflops": peak_fp64_gflops,
        "fp64_pipes_gflops": fp64_pipes,
        "flops_per_cell_update": FLOPS_PER_CELL_UPDATE,
        "achieved_step_tflops": FLOPS_PER_CELL_UPDATE * value / ws / 1e12,
        "mood_share_of_step": tm.mood_ms / el_ms if el_ms else None,
        "forms": forms,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    ws, rank, local = dist_setup(args)
    if args.final:
        if rank != 0:
            rc = 0
        else:
            rc = run_final_reference(args) if args.impl == "reference" else run_final(args)
    elif args.impl == "reference":
        rc = run_reference(args, ws, rank)
    else:
        rc = run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
