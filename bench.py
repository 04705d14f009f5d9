#!/usr/bin/env python
"""Benchmark: time to solution of the 2048x1024 steady transport problem,
with the 1024x256 Euler configuration and the reduced Navier-Stokes cavity in
the same JSON line.

Workload: 2D advection-diffusion on the unit square, 2048x1024 cells split
into 4,194,304 linear triangles (2,100,225 nodes), interior nodes perturbed by
a seeded uniform offset of +-0.2h (seed 1234), k = 1e-4, beta = (cos30, sin30),
f = 0, SUPG + CAU shock capturing, CSR storage in the SYMRCM numbering (the
reference's reverse Cuthill-McKee option; --reorder NOT for the mesh's own
numbering).

A step is one nonlinear (Picard) iteration: element build and assembly,
ILU(0) factorisation, and the linear solve to a relative residual of 1e-8 on
the unpreconditioned FP64 residual ||F - A u|| / ||F||, checked on the true
residual (right-preconditioned flexible GMRES(80); the reference's
left-preconditioned stopping rule is not used because it accepts residuals of
0.5 on this mesh).  Default preconditioner: block ILU(0) over 32 contiguous
row blocks of the SYMRCM numbering cut at equal spans of the factor's
dependency levels, each factorised by its own thread-block cluster and swept
by its own thread block (--ilu-blocks 0: ILU(0) of the whole matrix).  The
sweeps solve rows chained along the SYMRCM fronts 32 at a time by a warp scan
in double-single arithmetic (48-bit significands on the FP32 pipes, the
residual and Arnoldi in FP64), forward and backward in one launch.  Each
FGMRES step starts the next direction's sweeps on a second stream as soon as
the operator product is done and runs the Gram-Schmidt on the other SMs
meanwhile (the look-ahead step; FEMGPU_LOOKAHEAD=0 for the plain step).
Steps continue the Picard sequence from the warm-up steps.

The same line carries an "euler" object (REFLETIDO on 1024x256 cells, a step
being one implicit time step: predictor + 2 correctors) and an "ns" object
(lid-driven cavity at Re 1000 on 256x256 cells, a step being one damped-Newton
iteration); --no-euler / --no-ns leave them out, --workload euler|ns runs
only that leg as the line.

Arms: --impl ours (default): the GPU library through its device API (value)
and through the host-buffer C ABI (e2e).  --impl reference: the reference's
CPU algorithm (the oracle's restatement built -Ofast as the reference ships,
one core -- the reference is serial) on the same workload, run to the same
1e-8 true residual by host-checked refinement with its own left-preconditioned
pgmres; the reference's own stopping point is reported beside it.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time-to-solution at 1e-8 residual, learned vs ILU/AMG precond; matvec HBM GB/s"
L2_BYTES = 129 * 1024 * 1024


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nx", type=int, default=2048)
    ap.add_argument("--ny", type=int, default=1024)
    ap.add_argument("--precision", default="FP64", choices=["FP64", "MIXED", "MIXED_IR"])
    ap.add_argument("--precond", default="ILU0")
    ap.add_argument("--reorder", default="SYMRCM", choices=["NOT", "SYMRCM"])
    ap.add_argument("--kmax", type=int, default=80)
    ap.add_argument("--ilu-blocks", type=int, default=32,
                    help="0: ILU(0) of the whole matrix; P > 1: block ILU(0) over P row blocks")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-amg", action="store_true", help="skip the AMG-preconditioned leg")
    ap.add_argument("--workload", default="transport", choices=["transport", "euler", "ns"])
    ap.add_argument("--ns-n", type=int, default=256,
                    help="Navier-Stokes cavity cells per side (the 1024 of the full configuration takes ~70 s "
                         "per Newton iteration)")
    ap.add_argument("--euler-nx", type=int, default=1024)
    ap.add_argument("--euler-ny", type=int, default=256)
    ap.add_argument("--euler-precision", default="MIXED_IR", choices=["FP64", "MIXED_IR"],
                    help="MIXED_IR: FP32 element matrices and preconditioner inside FGMRES, FP64 residuals")
    ap.add_argument("--euler-solver", default="GMRES", choices=["GMRES", "FGMRES"])
    ap.add_argument("--euler-ilu-blocks", type=int, default=-1,
                    help="the Euler line's CSR + ILU(0) GMRES(50) leg: global ILU(0) (0), block ILU(0) over "
                         "that many blocks, or -1 to leave the leg out")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-euler", action="store_true", help="leave the Euler leg out of the transport line")
    ap.add_argument("--no-ns", action="store_true", help="leave the Navier-Stokes leg out of the transport line")
    ap.add_argument("--cpu-budget-s", type=float, default=150.0,
                    help="reference arm: wall-clock budget of the timed to-1e-8 steps (at least one runs)")
    return ap.parse_args(argv)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def workload(nx, ny):
    from fem_codes_gb300.mesh import skew_problem, structured_mesh
    m = structured_mesh(nx, ny, perturb=0.2, seed=1234)
    return m, skew_problem(m)


def config(a):
    return {"workload": f"steady transport SUPG+CAU {a.nx}x{a.ny} cells ({2 * a.nx * a.ny} triangles), "
                        f"perturbed +-0.2h, CSR ({a.reorder} numbering), "
                        + (f"block ILU(0) x{a.ilu_blocks}" if a.ilu_blocks > 1 else "ILU(0)")
                        + f"-FGMRES({a.kmax}) {a.precision}, rel tol 1e-8 (true residual)",
            "nx": a.nx, "ny": a.ny, "reorder": a.reorder, "precision": a.precision, "precond": a.precond,
            "kmax": a.kmax,
            "ilu_blocks": a.ilu_blocks,
            "step": "build + ILU(0) factor + solve to 1e-8", "l2": "inputs larger than L2 (matrix+factors > 129 MB)"}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.seek(0)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            c = [x.strip() for x in line.split(",")]
            if len(c) < 9 or c[0] != "0":
                continue
            try:
                sm.append(float(c[1]))
                mx = max(mx, float(c[2]))
            except ValueError:
                continue
            for nm, v in zip(names, c[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(x, dist=None):
    """The job's time per step with N replicas: the slowest rank's (an
    all-reduce MAX on the process group; CUDA tensor for NCCL, CPU for gloo)."""
    if dist is None or not dist.is_initialized():
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# --------------------------------------------------------------------- CPU
def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo) and its core count."""
    name = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                name = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if not name:
        try:
            for line in open("/proc/cpuinfo"):
                if line.lower().startswith("model name"):
                    name = line.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    import platform
    return f"{name or platform.processor() or 'unknown'} ({platform.machine()}, {os.cpu_count()} cores on the host)"


CPU_BUILD = "oracle restatement of the reference's C path, built -Ofast as its Makefiles ship (liboracle_fast.so)"


def cpu_run(m, p, npicard, kmax, reorder, refine_from=None, budget_s=0.0):
    """The reference's algorithm (oracle restatement, -Ofast, one core):
    set-up, then up to npicard Picard steps with its ILU(0) and left-
    preconditioned pgmres.  From step refine_from on (None: never) every solve
    is refined with the same pgmres until the host-checked true residual is
    <= 1e-8, and the loop ends once budget_s seconds went into such steps.
    Returns (phase times [s], per-step times [s], GMRES iterations, true
    residual of every step, refinement rounds of every step)."""
    from oracle import pyoracle
    out = pyoracle.run_transport(m.x, m.y, p.node_type, m.vert, p.k, p.gamma, p.beta, p.fsrc, p.upresc,
                                 scheme="CSR", reord=reorder, precond="ILU0", kmax=kmax, lmax=1000,
                                 tol=1e-8, npicard=npicard, fast=True, refine_to=1e-8, refine_tol=1e-10,
                                 refine_from=npicard if refine_from is None else refine_from,
                                 refine_budget_s=budget_s)
    nrun = int(out["npicard_run"])
    times, steps = pyoracle.last_times(nrun, fast=True)
    ref = out["refine"]
    return times, steps, out["iters"][:nrun], ref["true_rel_residual"], ref["rounds"]


def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    m, p = workload(a.nx, a.ny)
    # one Picard run: the warm-up steps stop where the reference stops, the
    # timed ones are solved to a true residual of 1e-8, as many as fit the budget
    times, steps, iters, res, rounds = cpu_run(m, p, a.warmup + a.steps, a.kmax, a.reorder,
                                               refine_from=a.warmup, budget_s=a.cpu_budget_s)
    w = a.warmup
    ntimed = len(steps) - w
    ms = 1e3 * float(np.mean(steps[w:]))
    shipped_ms = 1e3 * float(np.mean(steps[:w])) if w else None
    sample = (f"{ntimed} of the {a.steps} requested Picard steps of the full workload timed (~{ms / 1e3:.0f} s "
              f"each; the arm is bounded to ~{a.cpu_budget_s:.0f} s of timed work), after {w} warm-up steps "
              f"solved with the reference's own stop; reference algorithm (ILU(0) + left-preconditioned "
              f"pgmres({a.kmax})) refined with the same pgmres until the host-checked true residual is <= 1e-8: "
              f"true residuals {['%.1e' % r for r in res[w:]]}, GMRES iterations "
              f"{[int(i) for i in iters[w:]]}, refinement rounds {[int(r) for r in rounds[w:]]}.  "
              + (f"The reference's own stop (||M^-1 r|| <= 1e-8 ||M^-1 b||) took {shipped_ms:.0f} ms per step "
                 f"({[int(i) for i in iters[:w]]} iterations) at true residuals {['%.1e' % r for r in res[:w]]}.  "
                 if w else "")
              + f"Set-up (pattern, SYMRCM) {times[0]:.1f} s excluded.")
    line = {"impl": "reference", "metric": METRIC, "value": ms, "unit": "ms", "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config(a),
            "cpu_baseline": {"value": ms, "unit": "ms", "cores": 1, "kind": "port", "build": CPU_BUILD,
                             "cpu": cpu_model(), "steps_timed": ntimed,
                             "true_rel_residual": [float(r) for r in res[w:]],
                             "as_shipped": {"ms_per_step": shipped_ms,
                                            "true_rel_residual": [float(r) for r in res[:w]]},
                             "sample": sample},
            "e2e": {"value": ms, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)


def cpu_baseline_sample(m, p, a):
    """The GPU arm's bounded CPU sample (rank 0, N = 1): two Picard steps of the
    full workload on one core, the first with the reference's own stop, the
    second solved to a true residual of 1e-8 (the value)."""
    times, steps, iters, res, rounds = cpu_run(m, p, 2, a.kmax, a.reorder, refine_from=1)
    return {"value": 1e3 * float(steps[1]), "unit": "ms", "cores": 1, "kind": "port", "build": CPU_BUILD,
            "cpu": cpu_model(),
            "sample": f"Picard step 2 of the full workload on one core, reference algorithm (ILU(0) + "
                      f"left-preconditioned pgmres) refined with the same pgmres to a host-checked true "
                      f"residual of {res[1]:.1e} ({int(iters[1])} GMRES iterations, {int(rounds[1])} refinement "
                      f"rounds); step 1 with the reference's own stop took {1e3 * float(steps[0]):.0f} ms "
                      f"({int(iters[0])} iterations) at a true residual of {res[0]:.2e}; set-up "
                      f"{times[0]:.1f} s excluded"}


# --------------------------------------------------------------------- GPU
def run_ours(a):
    import torch
    import fem_codes_gb300 as fg

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    cpu = None
    m, p = workload(a.nx, a.ny)
    if rank == 0 and not a.no_cpu_baseline:
        cpu = cpu_baseline_sample(m, p, a)

    T = fg.SSTransport.from_problem(m, p, scheme="CSR", reorder=a.reorder, precond=a.precond, kmax=a.kmax,
                                    lmax=200, tol=1e-8, solver="FGMRES", precision=a.precision,
                                    inner_tol=1e-4, ir_max=40, ilu_blocks=a.ilu_blocks)
    L = T._L
    s = torch.cuda.Stream()
    T.set_stream(s.cuda_stream)
    n1 = T.neq + 1
    launches_per_step = None

    def step():
        T.build_dev()
        T.precond_setup_dev(2)
        return T.solve_dev()

    for _ in range(a.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = Clocks()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    iters, rels = [], []
    torch.cuda.synchronize()
    e0.record(s)
    t_wall = time.perf_counter()
    for _ in range(a.steps):
        iters.append(step())
    e1.record(s)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall
    clocks = clk.stop()
    ms = e0.elapsed_time(e1) / a.steps
    rel = T.true_residual()
    ms = max_over_ranks(ms, dist)

    # ---- end to end through the host-buffer C ABI (pinned host memory) ----
    u_h = torch.zeros(n1, dtype=torch.float64, pin_memory=True)
    F_h = torch.zeros(n1, dtype=torch.float64, pin_memory=True)
    X_h = torch.zeros(n1, dtype=torch.float64, pin_memory=True)
    vp = ctypes.c_void_p
    it_c = ctypes.c_int(0)
    # start from the current iterate
    L.femgpu_transport_solve(T.handle, vp(u_h.data_ptr()), ctypes.byref(it_c))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        rc = L.femgpu_transport_build(T.handle, vp(u_h.data_ptr()), vp(F_h.data_ptr()), None)
        rc |= L.femgpu_transport_precond_setup(T.handle, 2, None)
        rc2 = L.femgpu_transport_solve(T.handle, vp(X_h.data_ptr()), ctypes.byref(it_c))
        if rc or rc2:
            raise fg.FemGpuError(rc or rc2, "e2e step")
        u_h, X_h = X_h, u_h            # the solution is the next step's iterate (no host copy)
    torch.cuda.synchronize()
    e2e_ms = 1e3 * (time.perf_counter() - t0) / a.steps

    # ---- per-kernel rooflines (CUDA events on the context's stream) ----
    peak, peak_kind = peaks()
    chain_lv = np.zeros(2, np.int32)
    chain = T._L.femgpu_transport_ilu_chain(T.handle, chain_lv.ctypes.data_as(ctypes.c_void_p)) == 1
    kern = kernel_times(T, s, a)
    nnz, neq = T.nnzero, T.neq
    # dominant kernel of a step: the preconditioner sweeps (two per iteration)
    mean_it = float(np.mean(iters))
    sweep_key = "ilu0_apply_f32" if a.precision != "FP64" else "ilu0_apply_f64"
    shares = {
        "ilu_apply": mean_it * kern[sweep_key],
        "spmv": mean_it * kern["spmv_f64_fused"],
    }
    dom = max(shares, key=shares.get)
    if dom == "ilu_apply":
        vs = 4 if a.precision != "FP64" else 8
        # algorithmic bytes: L and U values + 4-byte indices once, pivots, in/out vectors
        alg = nnz * (vs + 4) + neq * vs + 4 * neq * vs
        t_k = kern[sweep_key]
        if chain:
            ds = a.precision == "FP64" and os.environ.get("FEMGPU_SWEEP_DS", "1") != "0"
            fb = ds and os.environ.get("FEMGPU_SWEEP_FB", "1") != "0"
            name = (("k_sweep_cs_fb (ILU(0) forward and backward sweeps in one launch" if fb else
                     "k_sweep_cs (ILU(0) forward+backward")
                    + ", chain-scan: rows chained along the SYMRCM fronts solved "
                    "32 at a time by a warp scan" + (" in double-single arithmetic" if ds else "")
                    + ", row records, dataflow between warps")
        elif os.environ.get("FEMGPU_SWEEP_LAYOUT") == "ell":
            name = "k_sweep (ILU(0) forward+backward, ELL layout, a barrier per level"
        elif os.environ.get("FEMGPU_SWEEP_SYNC") == "barrier":
            name = "k_sweep_rec (ILU(0) forward+backward, row records, a barrier per level"
        else:
            name = "k_sweep_df (ILU(0) forward+backward, row records, dataflow between warps"
        name += f", TMA-staged, one CTA per matrix block, {max(a.ilu_blocks, 1)} blocks)"
    else:
        alg = nnz * 12 + (neq + 1) * 4 + 2 * neq * 8
        t_k = kern["spmv_f64_fused"]
        name = "k_sellmv<double, fused> (FP64 CSR product over the SELL-32 copy, fused multiply-adds)"
    achieved = alg / (t_k * 1e-3) / 1e9
    traffic = read_traffic(dom)
    spmv_bytes = nnz * 12 + (neq + 1) * 4 + 2 * neq * 8
    spmv_gbs = spmv_bytes / (kern["spmv_f64"] * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": ms, "unit": "ms", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64/f32 mixed" if a.precision != "FP64" else "f64", "data": "synthetic",
        "config": config(a),
        "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": n1 * 8, "d2h_bytes_per_step": 2 * n1 * 8},
        "roofline": {"kernel": name, "bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                     else "fallback 6.8 TB/s"},
        "matvec": {"kernel": "k_sellmv<double, fused> (FP64 CSR over the SELL-32 copy, the FGMRES operator: fused "
                             "multiply-adds)",
                   "GB/s": spmv_bytes / (kern["spmv_f64_fused"] * 1e-3) / 1e9,
                   "frac": spmv_bytes / (kern["spmv_f64_fused"] * 1e-3) / 1e9 / peak,
                   "us": kern["spmv_f64_fused"] * 1e3, "bytes": spmv_bytes,
                   "exact_kernel": "k_sellmv<double> (csrmv.c's rounding, bit-identical; FP64-pipe bound)",
                   "exact_us": kern["spmv_f64"] * 1e3, "exact_GB/s": spmv_gbs, "exact_frac": spmv_gbs / peak,
                   "f32_us": kern["spmv_f32"] * 1e3,
                   "f32_GB/s": (nnz * 8 + (neq + 1) * 4 + 2 * neq * 4) / (kern["spmv_f32"] * 1e-3) / 1e9},
        "breakdown_ms": {k: round(v, 4) for k, v in kern.items()},
        "gmres_iters": [int(i) for i in iters], "true_rel_residual": rel,
        "neq": neq, "nnz": nnz, "ilu_levels": [T.ilu_levels_L, T.ilu_levels_U],
        "ilu_chain_levels": [int(v) for v in chain_lv] if chain else None,
        "wall_ms_per_step": 1e3 * wall / a.steps,
        "gpu_launches": launches_estimate(a, iters),
    }
    if cpu:
        line["cpu_baseline"] = cpu
    if clocks:
        line["clocks"] = clocks
    T.close()
    if not a.no_learned:
        line["learned"] = learned_leg(m, p, a, s)
    if not a.no_amg:
        line["amg"] = amg_leg(m, p, a, s)
    if rank == 0:
        line["matvec_compare"] = matvec_compare(m, p, s, peak)
    if not a.no_euler:
        line["euler"] = euler_leg(a, max(a.steps, 5), max(a.warmup, 3), cpu=rank == 0 and not a.no_cpu_baseline)
    if not a.no_ns:
        line["ns"] = ns_leg(a.ns_n, 6)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


WEIGHTS = os.path.join(ROOT, "fem_codes_gb300", "weights", "gnn_transport.npy")


def learned_leg(m, p, a, s, steps=1):
    """Time to solution of the same Picard step with the learned
    preconditioner (FGMRES(kmax), FP64 Arnoldi, bf16 network activations,
    fallback to the step's ILU(0) on a stalled cycle); None without trained
    weights."""
    import torch
    import fem_codes_gb300 as fg
    from fem_codes_gb300.learned import MeshGNN
    if not os.path.exists(WEIGHTS):
        return None
    net = MeshGNN(np.load(WEIGHTS))
    T = fg.SSTransport.from_problem(m, p, scheme="CSR", reorder=a.reorder, precond="LEARNED", kmax=a.kmax,
                                    lmax=400, tol=1e-8, solver="FGMRES", precision="FP64", stall_ratio=0.9,
                                    ilu_blocks=a.ilu_blocks)
    T.set_stream(s.cuda_stream)
    T.set_learned(net)
    out = {}
    try:
        def step():
            T.build_dev()
            T.precond_setup_dev(2)
            return T.solve_dev(raise_on_nonconvergence=False)
        step()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(s)
        its = [step() for _ in range(steps)]
        e1.record(s)
        torch.cuda.synchronize()
        out = {"ms_per_step": e0.elapsed_time(e1) / steps, "gmres_iters": its, "fell_back_to_ilu0": T.fell_back(),
               "true_rel_residual": T.true_residual(),
               "network": "3 message-passing layers, width 32, fp32 weights, bf16 activations",
               "weights": "fem_codes_gb300/weights/gnn_transport.npy (python -m fem_codes_gb300.train_learned)"}
    finally:
        T.close()
        net.close()
    return out


def amg_leg(m, p, a, s, steps=1):
    """Time to solution of the same Picard step with the DPA AMG preconditioner
    (amg_dpa.c: pairwise aggregation with 3 coarsening sweeps per level, beta -1,
    SOR omega 1.0, 2 sweeps per side; the hierarchy is rebuilt on the host from
    each step's matrix, as AMG_precond_setup does), FGMRES(kmax) in FP64 with at
    most 25 restart cycles."""
    import torch
    import fem_codes_gb300 as fg
    T = fg.SSTransport.from_problem(m, p, scheme="CSR", reorder=a.reorder, precond="AMG", kmax=a.kmax,
                                    lmax=25, tol=1e-8, solver="FGMRES", precision="FP64")
    T.set_stream(s.cuda_stream)
    amg = fg.AMG(ncl=3, beta=-1.0, omega=1.0, nr=2)
    out = {}
    try:
        T.set_amg(amg)

        def step():
            T.build_dev()
            T.precond_setup_dev(2)
            return T.solve_dev(raise_on_nonconvergence=False)
        step()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        its, setup_s = [], 0.0
        e0.record(s)
        for _ in range(steps):
            T.build_dev()
            t0 = time.perf_counter()
            T.precond_setup_dev(2)                      # host hierarchy (synchronises the stream)
            setup_s += time.perf_counter() - t0
            its.append(T.solve_dev(raise_on_nonconvergence=False))
        e1.record(s)
        torch.cuda.synchronize()
        out = {"ms_per_step": e0.elapsed_time(e1) / steps, "setup_ms_per_step": 1e3 * setup_s / steps,
               "gmres_iters": its, "true_rel_residual": T.true_residual(), "levels": amg.levels(),
               "amg": "DPA pairwise aggregation, ncl 3, beta -1, SOR omega 1.0 x 2, one V-cycle per application"}
    finally:
        T.close()
        amg.close()
    return out


def matvec_compare(m, p, s, peak, reps=10):
    """The C2 comparison of the three storage schemes' products (csrmv.c,
    ebemv.c, edemv.c, each bit-identical to the reference): one EBE and one
    EDE context on the same mesh, one Build, then Q = A P timed with CUDA
    events on stream s, L2 flushed between launches.  Algorithmic bytes:
    CSR nnz*12 + (n+1)*4 + 2n*8; EBE Ne*(9*8 + 3*4) + incidence lists
    n + 3*Ne codes + 2n*8; EDE (nedge+1)*32 + nedge*8 + incidence + 2n*8."""
    import torch
    import fem_codes_gb300 as fg
    out = {}
    vp = ctypes.c_void_p
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    for scheme in ("EBE", "EDE"):
        T = fg.SSTransport.from_problem(m, p, scheme=scheme, precond="NOT", kmax=8, lmax=1, solver="FGMRES")
        T.set_stream(s.cuda_stream)
        T.build_dev()
        x = torch.randn(T.neq + 1, dtype=torch.float64, device="cuda")
        y = torch.zeros_like(x)
        torch.cuda.synchronize()
        for _ in range(2):
            T._L.femgpu_transport_matvec_dev(T.handle, vp(x.data_ptr()), vp(y.data_ptr()))
        tot = 0.0
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(s):
                flush.zero_()
                e0.record(s)
                T._L.femgpu_transport_matvec_dev(T.handle, vp(x.data_ptr()), vp(y.data_ptr()))
                e1.record(s)
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        ms = tot / reps
        n, ne = T.neq, m.nel
        if scheme == "EBE":
            alg = ne * (9 * 8 + 3 * 4) + (n + 1) * 4 + 3 * ne * 4 + 2 * n * 8
            kern = "k_ebemv (3x3 FP64 element matrices, row gather)"
        else:
            alg = (T.nedge + 1) * 32 + T.nedge * 8 + (n + 1) * 4 + 2 * T.nedge * 4 + 2 * n * 8
            kern = "k_edemv (4 FP64 values per edge, row gather)"
        out[scheme] = {"kernel": kern, "us": 1e3 * ms, "GB/s": alg / (ms * 1e-3) / 1e9,
                       "frac": alg / (ms * 1e-3) / 1e9 / peak, "bytes": alg}
        T.close()
    return out


def kernel_times(T, s, a, reps=10):
    """Average duration (ms) of single launches, CUDA events on stream s."""
    import torch
    L = T._L
    vp = ctypes.c_void_p
    n1 = T.neq + 1
    x = torch.randn(n1, dtype=torch.float64, device="cuda")
    y = torch.zeros_like(x)
    z32 = torch.zeros(n1, dtype=torch.float32, device="cuda")
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    out = {}

    def timeit(fn):
        for _ in range(2):
            fn()
        tot = 0.0
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(s):
                flush.zero_()  # evict L2 between launches (same stream)
                e0.record(s)
                fn()
                e1.record(s)
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        return tot / reps

    torch.cuda.synchronize()
    s.wait_stream(torch.cuda.current_stream())
    out["spmv_f64"] = timeit(lambda: L.femgpu_transport_matvec_dev(T.handle, vp(x.data_ptr()), vp(y.data_ptr())))
    # the FGMRES operator: the same product with fused multiply-adds
    out["spmv_f64_fused"] = timeit(lambda: L.femgpu_transport_operator_dev(T.handle, vp(x.data_ptr()),
                                                                           vp(y.data_ptr())))
    out["ilu0_apply_f64"] = timeit(lambda: L.femgpu_transport_precond_dev(T.handle, vp(x.data_ptr()),
                                                                          vp(y.data_ptr())))
    out["ilu0_apply_f32"] = timeit(lambda: L.femgpu_transport_precond32_dev(T.handle, vp(x.data_ptr()),
                                                                            vp(z32.data_ptr())))
    out["build"] = timeit(lambda: L.femgpu_transport_build_dev(T.handle))
    out["precond_setup"] = timeit(lambda: L.femgpu_transport_precond_setup_dev(T.handle, 2))
    # FP32 CSR product on the same pattern (stateless entry point)
    out["spmv_f32"] = spmv32_time(T, s, timeit)
    return out


def spmv32_time(T, s, timeit):
    import torch
    L = T._L
    vp = ctypes.c_void_p
    pat = T.pattern()
    IA = torch.from_numpy(pat["IA"]).cuda()
    JA = torch.from_numpy(pat["JA"]).cuda()
    AA = torch.randn(T.nnzero, dtype=torch.float32, device="cuda")
    P = torch.randn(T.neq + 1, dtype=torch.float32, device="cuda")
    Q = torch.zeros_like(P)
    return timeit(lambda: L.femgpu_csrmv_f32(T.neq, vp(IA.data_ptr()), vp(JA.data_ptr()), vp(AA.data_ptr()),
                                             vp(P.data_ptr()), vp(Q.data_ptr()), vp(s.cuda_stream)))


def read_traffic(kind):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/), or None if not captured."""
    path = os.path.join(ROOT, "profiles", "traffic_per_launch.txt")
    try:
        lines = open(path).read().splitlines()
    except OSError:
        return None
    for line in lines:
        if line.startswith("#") or ":" not in line:
            continue
        k, v = line.split(":", 1)
        if k.strip() == kind:
            try:
                return float(v.split()[0])
            except (ValueError, IndexError):
                return None
    return None


def launches_estimate(a, iters):
    """Kernel launches of the timed steps (a FGMRES cycle enqueues all kmax
    steps; those past convergence are predicated off but launched): build 2
    (element build, CSR assembly with the RHS) + factor 5 (cluster elimination,
    double-single program refresh and scan multipliers of both sweeps) + per
    cycle 5 (product, residual start, scaling; back-substitution and update)
    and in the look-ahead step 3 more for the first direction's preconditioner
    (gather, both sweeps in one launch, conversion) + per step (look-ahead step: product with the
    gather 1, flag copy 1, sweeps 1, classical Gram-Schmidt 3 per pass (one
    pass in the first cycle, two in restarted ones), Z h 1, scaling 1, Givens
    1, next direction 1; the last step of a cycle has no next direction; plain
    step (FEMGPU_LOOKAHEAD=0): preconditioner 3, product 1, Gram-Schmidt,
    scaling, Givens) + the true-residual check 2."""
    kmax = a.kmax
    la = os.environ.get("FEMGPU_LOOKAHEAD", "1") != "0" and a.precision == "FP64"
    tot = 0
    for it in iters:
        cyc = max(1, (int(it) + kmax - 1) // kmax)
        for c in range(cyc):
            gs = 3 * (1 if c == 0 else 2)
            if la:
                tot += 8 + (kmax - 1) * (7 + gs) + (3 + gs)
            else:
                tot += 5 + kmax * (3 + 1 + gs + 2)
        tot += 2 + 5 + 2
    return tot


# ------------------------------------------------------------------ Euler
EULER_METRIC = "time per implicit time step (predictor + 2 correctors, GMRES to 1e-8)"


def euler_setup(nx, ny):
    from fem_codes_gb300.mesh import euler_cfl_dt, refletido_problem, structured_mesh
    m = structured_mesh(nx, ny, lx=4.0, ly=1.0)
    return m, refletido_problem(m), euler_cfl_dt(m, 5.0)


def euler_config(a):
    return {"workload": f"2D Euler REFLETIDO (oblique shock reflection, Mach 2.9 inflow, gamma 1.4) on a 4x1 "
                        f"domain, {a.euler_nx}x{a.euler_ny} cells ({2 * a.euler_nx * a.euler_ny} triangles), "
                        "SUPG+CAU, Predictor_Old alpha 0.5, 2 correctors, dt from CFL 5, "
                        + ("EBE 12x12 FP64, BlockDiag-preconditioned " + euler_solver(a) if a.euler_precision == "FP64"
                           else "EBE 12x12 FP32 element matrices and FP32 BlockDiag inside FGMRES, FP64 Arnoldi and "
                                "residuals,") + "(50) to 1e-8",
            "nx": a.euler_nx, "ny": a.euler_ny, "kmax": 50, "precision": a.euler_precision,
            "solver": euler_solver(a),
            "step": "one time step: predictor + 2 x (build + block-diagonal setup + GMRES + update)",
            "l2": "inputs larger than L2 (element matrices 603 MB)"}


def euler_solver(a):
    return "FGMRES" if a.euler_precision != "FP64" else a.euler_solver


def euler_cpu(nx, ny, steps=1, warm=1):
    """The oracle's predictor (reference algorithm: BlockDiag-preconditioned
    pgmres(50), -Ofast, one core) on the full REFLETIDO mesh: seconds per time
    step over `steps` steps after `warm` untimed ones (the first step starts
    from the uniform inflow state and is the cheapest)."""
    from oracle import pyoracle
    m, pb, dt = euler_setup(nx, ny)
    u0 = pb.u0
    if warm:
        uh, _ = pyoracle.euler_predictor(m.x, m.y, m.vert, pb.node_id, pb.neq, pb.upresc, u0, warm, 2, dt=dt,
                                         kmax=50, lmax=100, tol=1e-8, fast=True)
        u0 = uh[-1]
    t0 = time.perf_counter()
    _, its = pyoracle.euler_predictor(m.x, m.y, m.vert, pb.node_id, pb.neq, pb.upresc, u0, steps, 2, dt=dt,
                                      kmax=50, lmax=100, tol=1e-8, fast=True)
    return (time.perf_counter() - t0) / steps, m.nel, its


def euler_cpu_line(a, sec, nel, its):
    ms = 1e3 * sec
    return {"value": ms, "unit": "ms", "cores": 1, "kind": "port", "build": CPU_BUILD, "cpu": cpu_model(),
            "sample": f"time step 2 of the full {a.euler_nx}x{a.euler_ny} mesh ({nel} triangles) on one core, "
                      f"reference algorithm (Predictor_Old, 2 correctors, BlockDiag-preconditioned "
                      f"pgmres(50) to 1e-8 on the left-preconditioned residual; GMRES iterations "
                      f"{its.reshape(-1).tolist()})"}


def run_euler(a):
    rank = int(os.environ.get("RANK", "0"))
    if a.impl == "reference":
        if rank != 0:
            return
        sec, nel, its = euler_cpu(a.euler_nx, a.euler_ny)
        cpu = euler_cpu_line(a, sec, nel, its)
        ms = cpu["value"]
        print(json.dumps({"impl": "reference", "metric": EULER_METRIC, "value": ms, "unit": "ms",
                          "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms,
                          "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                          "data": "synthetic", "config": euler_config(a), "cpu_baseline": cpu,
                          "e2e": {"value": ms, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
              flush=True)
        return
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    line = euler_leg(a, a.steps, a.warmup, cpu=rank == 0 and not a.no_cpu_baseline)
    if rank == 0:
        print(json.dumps(line), flush=True)


def euler_leg(a, steps, warmup, cpu=True):
    """The C3 Euler configuration on the GPU: `warmup` untimed and `steps`
    timed implicit time steps through the device API (CUDA events), the same
    through the host-buffer entry point (e2e), the error of the mixed mode
    against FP64 runs, kernel rooflines and the CPU baseline at full size."""
    import torch
    import fem_codes_gb300 as fg
    cpu_line = None
    if cpu:
        sec, nel, its_cpu = euler_cpu(a.euler_nx, a.euler_ny)
        cpu_line = euler_cpu_line(a, sec, nel, its_cpu)
    m, pb, dt = euler_setup(a.euler_nx, a.euler_ny)
    E = fg.Euler.from_problem(m, pb, alpha=0.5, dt=dt, stab_tol=1e-6, kmax=50, lmax=100, tol=1e-8, ncorr=2,
                              solver=euler_solver(a), precision=a.euler_precision)
    s = torch.cuda.Stream()
    E.set_stream(s.cuda_stream)
    n1 = pb.neq + 1
    L = E._L
    u_h = torch.from_numpy(pb.u0.copy()).pin_memory()
    # warm-up from the initial state through the host-buffer entry point; the
    # device keeps the state for the timed steps, u_h the same state
    rc = L.femgpu_euler_predictor(E.handle, ctypes.c_void_p(u_h.data_ptr()), warmup, None, None)
    if rc:
        raise fg.FemGpuError(rc, "warm-up")
    torch.cuda.synchronize()
    clk = Clocks()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s)
    its = E.predictor_dev(steps)
    e1.record(s)
    torch.cuda.synchronize()
    clocks = clk.stop()
    ms = e0.elapsed_time(e1) / steps
    phase = E.last_times()
    # end to end: host state in, one step, host state out, per step
    t0 = time.perf_counter()
    for _ in range(steps):
        rc = L.femgpu_euler_predictor(E.handle, ctypes.c_void_p(u_h.data_ptr()), 1, None, None)
        if rc:
            raise fg.FemGpuError(rc, "e2e step")
    e2e_ms = 1e3 * (time.perf_counter() - t0) / steps
    err = None
    if a.euler_precision != "FP64":
        # u_h holds the state after the warm-up and the end-to-end steps (each
        # of which restarts from u_h with a = 0): the same calls in FP64 FGMRES
        # at this tolerance and at 1e-11, and the relative max-norm differences
        def fp64_run(tol):
            E64 = fg.Euler.from_problem(m, pb, alpha=0.5, dt=dt, stab_tol=1e-6, kmax=50, lmax=400, tol=tol, ncorr=2,
                                        solver="FGMRES", precision="FP64")
            E64.set_stream(s.cuda_stream)
            u64 = torch.from_numpy(pb.u0.copy()).pin_memory()
            for nst in [warmup] + [1] * steps:
                rc = L.femgpu_euler_predictor(E64.handle, ctypes.c_void_p(u64.data_ptr()), nst, None, None)
                if rc:
                    raise fg.FemGpuError(rc, "FP64 comparison run")
            torch.cuda.synchronize()
            E64.close()
            return u64[:pb.neq].clone()

        def rel(x, y):
            return (x - y).abs().max().item() / max(y.abs().max().item(), 1e-300)

        u8, u11 = fp64_run(1e-8), fp64_run(1e-11)
        um = u_h[:pb.neq]
        err = {"mixed_vs_fp64": rel(um, u8), "mixed_vs_fp64_tight": rel(um, u11), "fp64_vs_fp64_tight": rel(u8, u11)}
    peak, peak_kind = peaks()
    mixed = a.euler_precision != "FP64"
    kt = euler_kernel_times(E, s, pb.neq, m.nel, mixed=mixed)
    if mixed:   # the solve's operator: FP32 element matrices, FP32 vector in, FP64 out
        mv_bytes = m.nel * (144 * 4 + 48) + pb.neq * (4 + 8)
        mv_gbs = mv_bytes / (kt["ebemv32"] * 1e-3) / 1e9
        mv_name, mv_note, mv_traffic = ("k_ebemv_blk32<4> (12x12 FP32 EBE matvec, row gather)",
                                        "FP32 fused multiply-adds, FP64 row totals", read_traffic("euler_ebemv32"))
    else:
        mv_bytes = m.nel * (144 * 8 + 48) + 2 * pb.neq * 8
        mv_gbs = mv_bytes / (kt["ebemv"] * 1e-3) / 1e9
        mv_name, mv_note, mv_traffic = ("k_ebemv_blk<4> (12x12 FP64 EBE matvec, row gather)",
                                        "FP64 issue-bound on GB300 (288 FP64 ops per element, no FMA contraction)",
                                        read_traffic("euler_ebemv"))
    build_gbs = m.nel * (144 * 8 + 12 * 8 + 12) / (kt["build"] * 1e-3) / 1e9
    line = {"metric": EULER_METRIC, "value": ms, "unit": "ms", "n_gpus": 1, "steps": steps, "warmup": warmup,
            "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if a.euler_precision == "FP64" else "f64/f32 mixed",
            "data": "synthetic", "config": euler_config(a),
            "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": n1 * 8, "d2h_bytes_per_step": n1 * 8},
            "roofline": {"kernel": mv_name, "bound": "hbm",
                         "achieved": mv_gbs, "peak": peak, "unit": "GB/s", "frac": mv_gbs / peak,
                         "traffic": mv_traffic, "note": mv_note},
            "kernel_ms": {k: round(v, 4) for k, v in kt.items()},
            "build": {"kernel": "k_euler_element", "ms": kt["build"],
                      "elements_per_s": m.nel / (kt["build"] * 1e-3), "GB/s": build_gbs},
            "phase_ms_per_step": {k: round(1e3 * v / steps, 3) for k, v in
                                  zip(["build", "precond_setup", "solve"], phase)},
            "gmres_iters": its.reshape(-1).tolist(), "neq": pb.neq, "nel": m.nel, "dt": dt}
    if err is not None:
        err["what"] = (f"max |u - u_ref| / max |u_ref| after {warmup + steps} time steps; fp64: FP64 FGMRES at "
                       "1e-8 (agrees with the oracle to 1e-8 on the tested meshes), fp64_tight: FP64 FGMRES at 1e-11")
        line["err_vs_fp64"] = err
    if cpu_line:
        line["cpu_baseline"] = cpu_line
    if clocks:
        line["clocks"] = clocks
    E.close()
    if a.euler_ilu_blocks >= 0:
        line["csr_ilu0"] = euler_csr_ilu0_leg(a, m, pb, dt, s, steps, warmup)
    return line


def euler_csr_ilu0_leg(a, m, pb, dt, s, steps, warmup):
    """The configuration's own preconditioner on the 4-dof system: the
    reference's Euler CSR storage (csr_Initialization.c, csr_assembly.c) with
    ILU(0) (setPreconditioner.c:118-128), (block) ILU(0)-FGMRES(50) in FP64,
    the same steps as the main leg, timed on the device."""
    import torch
    import fem_codes_gb300 as fg
    E = fg.Euler.from_problem(m, pb, alpha=0.5, dt=dt, stab_tol=1e-6, kmax=50, lmax=100, tol=1e-8, ncorr=2,
                              solver="FGMRES", precision="FP64", scheme="CSR", precond="ILU0",
                              ilu_blocks=a.euler_ilu_blocks)
    E.set_stream(s.cuda_stream)
    u_h = torch.from_numpy(pb.u0.copy()).pin_memory()
    rc = E._L.femgpu_euler_predictor(E.handle, ctypes.c_void_p(u_h.data_ptr()), warmup, None, None)
    if rc:
        raise fg.FemGpuError(rc, "warm-up (CSR ILU(0))")
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s)
    its = E.predictor_dev(steps)
    e1.record(s)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    phase = E.last_times()
    out = {"ms_per_step": ms,
           "config": ("CSR storage (4x4 nodal blocks), " + (f"block ILU(0) x{a.euler_ilu_blocks}"
                      if a.euler_ilu_blocks > 1 else "ILU(0)") + "-FGMRES(50) in FP64, rel tol 1e-8"),
           "phase_ms_per_step": {k: round(1e3 * v / steps, 3) for k, v in
                                 zip(["build", "precond_setup", "solve"], phase)},
           "gmres_iters": its.reshape(-1).tolist()}
    E.close()
    return out


def euler_kernel_times(E, s, neq, nel, reps=10, mixed=False):
    import torch
    L = E._L
    vp = ctypes.c_void_p
    ebe = L.femgpu_euler_ebe(E.handle)
    L.femgpu_ebe_matvec_dev.argtypes = [vp, vp, vp]
    L.femgpu_ebe_matvec_dev.restype = ctypes.c_int
    x = torch.randn(neq + 1, dtype=torch.float64, device="cuda")
    y = torch.zeros_like(x)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")

    def timeit(fn):
        for _ in range(2):
            fn()
        tot = 0.0
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(s):
                flush.zero_()
                e0.record(s)
                fn()
                e1.record(s)
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        return tot / reps

    torch.cuda.synchronize()
    s.wait_stream(torch.cuda.current_stream())
    out = {"ebemv": timeit(lambda: L.femgpu_ebe_matvec_dev(ebe, vp(x.data_ptr()), vp(y.data_ptr())))}
    if mixed:
        L.femgpu_ebe_matvec32_dev.argtypes = [vp, vp, vp]
        L.femgpu_ebe_matvec32_dev.restype = ctypes.c_int
        x32 = x.float()
        out["ebemv32"] = timeit(lambda: L.femgpu_ebe_matvec32_dev(ebe, vp(x32.data_ptr()), vp(y.data_ptr())))
    out["build"] = timeit(lambda: L.femgpu_euler_build_dev(E.handle))
    return out


NS_METRIC = "time per damped-Newton iteration (VMS build + ILU(0) set-up + FGMRES(50) to the forcing term)"


def ns_config(n, nit):
    return {"workload": f"steady Navier-Stokes VMS, lid-driven cavity Re 1000, {n}x{n} cells "
                        f"({2 * n * n} triangles), CSR + ILU(0), FGMRES(50), forcing terms eta_newton case 2",
            "n": n, "newton": nit}


def run_ns(a):
    """Steady Navier-Stokes lid-driven cavity, Re 1000, CSR storage with
    ILU(0), FGMRES(50), the reference's forcing terms (eta_newton case 2,
    eta0 0.1); a step is one damped-Newton iteration.  --impl reference: the
    oracle's restatement is EBE/BlockDiag only, so the arm prints its
    unavailable line."""
    rank = int(os.environ.get("RANK", "0"))
    if a.impl == "reference":
        if rank == 0:
            print(json.dumps({"impl": "reference", "metric": NS_METRIC, "config": ns_config(a.ns_n, a.warmup + a.steps),
                              "unavailable": "no CPU restatement of the CSR/ILU(0) Navier-Stokes path to time"}))
        return
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    line = ns_leg(a.ns_n, a.warmup + a.steps)
    if rank == 0:
        print(json.dumps(line), flush=True)


def ns_leg(n, n_it):
    """n_it damped-Newton iterations of the cavity on n x n cells through the
    host-buffer entry point (the Newton loop runs behind one call)."""
    import torch
    import fem_codes_gb300 as fg
    from fem_codes_gb300.mesh import cavity_problem, structured_mesh
    m = structured_mesh(n, n)
    pb = cavity_problem(m, 1000.0)
    ns = fg.NavierStokes.from_problem(m, pb, solver="FGMRES", kmax=50, lmax=40, eta0=0.1, eta_case=2, tol_nl=1e-8,
                                      scheme="CSR", precond="ILU0")
    clk = Clocks()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    u, uh, nF, w, its = ns.Process(n_it)          # host-buffer entry point: u and the history come back
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clocks = clk.stop()
    ns.close()
    ms = 1e3 * wall / max(len(nF), 1)
    line = {"metric": NS_METRIC, "value": ms, "unit": "ms", "n_gpus": 1, "steps": len(nF), "warmup": 0,
            "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": ns_config(n, n_it),
            "e2e": {"value": ms, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 8 * (pb.neq + 1),
                    "note": "the Newton loop runs behind one host-buffer call; the timing covers it whole"},
            "newton": {"normF": [float(v) for v in nF], "damping": [float(v) for v in w],
                       "gmres_iters": [int(v) for v in its]},
            "neq": pb.neq, "nel": m.nel,
            "full_size_note": "the 1024x1024 configuration (3.1M unknowns) takes ~70 s per Newton iteration with "
                              "ILU(0)-FGMRES(50), its linear solves at the 2000-iteration cap; --ns-n 1024 runs it"}
    if clocks:
        line["clocks"] = clocks
    return line


def main():
    a = parse()
    if a.workload == "euler":
        run_euler(a)
    elif a.workload == "ns":
        run_ns(a)
    elif a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
