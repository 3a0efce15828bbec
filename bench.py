#!/usr/bin/env python3
"""Benchmark: one implicit step of the Vanadis DR transport model on the
large synthetic mesh, solved on one GB300 by libvdr.so.

Workload (one "step"): rotation + shear flow on a 256x256x128-element
jittered HEX8 mesh (8,388,608 elements, 8,520,321 nodes), lognormal
per-element diffusivity, two Gaussian sources, zero Dirichlet on inflow
faces, VF DR variant; the reference's theta-scheme system
A = 2H + (3/dt)M, b = 3f - (H - (3/dt)M) T_old with T_old = 0, at Courant
number |u|max dt/h = 10 (the reference's recorded run has |v| dt/h = 10
along its flow); FP64 Jacobi-BiCGStab from x = 0 to ||r||/||b|| <= 1e-8.
A step does what one pass of the reference's przest3d does on the GPU:
element matrices + Jacobi diagonal (DR recompute), right-hand side, solve.

  value     seconds per step with mesh and fields resident in HBM (CUDA
            events on the library's stream)
  e2e       the same step through the C ABI with host arrays: fields
            uploaded, right-hand side downloaded, solution downloaded
  roofline  the dominant kernel, the stored-matrix EBE apply, timed alone
  --impl reference   the reference's CPU algorithm (the C oracle port of
            vanadis_full_DR_OpenMP_timing.for) on this host's cores
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("solve time to rel. residual 1e-8: learned+FP32 vs plain FP64; "
          "matvec HBM GB/s")
COURANT = 10.0
TOL = 1e-8


def args_parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--nex", type=int, default=256)
    ap.add_argument("--ney", type=int, default=256)
    ap.add_argument("--nez", type=int, default=128)
    ap.add_argument("--scatter", default="atomic", choices=["atomic", "color"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the many-right-hand-side section")
    ap.add_argument("--no-meshes", action="store_true",
                    help="skip the many-mesh section")
    ap.add_argument("--no-dropin", action="store_true",
                    help="skip the kernel_dbcg_simple_ section")
    ap.add_argument("--no-time-loop", action="store_true",
                    help="skip the device time-loop section")
    ap.add_argument("--no-text", action="store_true",
                    help="skip the text-output section")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the learned-preconditioner section")
    ap.add_argument("--learn-steps", type=int, default=LEARN_STEPS)
    ap.add_argument("--learn-epochs", type=int, default=1)
    ap.add_argument("--case", default=None,
                    choices=["build", "apply", "block_apply", "block_apply_tc", "bicg", "mixed",
                             "unet_train", "unet_forward"],
                    help="run one small fixed workload for a profiler "
                         "capture instead of the benchmark")
    ap.add_argument("--inner-tol", type=float, default=1e-5,
                    help="inner tolerance of --case mixed (the bench's mixed step: 1e-3)")
    ap.add_argument("--build-mode", default="auto", choices=["auto", "recompute"],
                    help="element geometry of --case build: the mesh's "
                         "geometric factors or the Jacobians at every build")
    ap.add_argument("--cpu-iters", type=int, default=4,
                    help="BiCGStab iterations timed in the CPU sample")
    return ap.parse_args(argv)


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def reduce_max_over_ranks(value, device):
    """The largest of one float per rank (every rank gets it): the step time
    of a replica run is the slowest rank's.  NCCL on the GPUs, gloo in the
    CPU tests."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload_config(a, prob):
    return {
        "workload": "rotation_shear %dx%dx%d, theta-step at Courant %g, FP64 "
                    "Jacobi-BiCGStab to 1e-8 (VF DR variant)"
                    % (a.nex, a.ney, a.nez, COURANT),
        "elements": prob.mesh.nelem, "nodes": prob.mesh.nnode,
        "dirichlet_nodes": int(prob.bc.sum()),
        "apply": "stored element matrices, double-float pairs (built on GPU "
                 "each step from the fields and the mesh's geometric factors, "
                 "which the handle forms once)",
        "scatter": a.scatter, "solver": "bicgstab", "precision": "fp64",
        "l2": "inputs larger than L2 (element matrices 4.3 GB per apply)",
    }


def make_problem(a):
    import __graft_entry__
    P = __graft_entry__.package().problems
    prob = P.rotation_shear(a.nex, a.ney, a.nez, seed=1002)
    h = 1.0 / max(a.nex, a.ney, a.nez)
    dt = COURANT * h  # max |u| = 1
    return prob, dt


# --------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device),
                 "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sms, maxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sms.append(float(f[1]))
                maxs.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sms:
            return None
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": max(maxs),
                "samples": len(sms), "reasons": sorted(reasons)}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_value(name, key):
    """A 'key: <number>' line of a committed ncu summary under profiles/."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            if line.startswith(key + ":"):
                return float(line.split(":", 1)[1])
    except (OSError, ValueError):
        pass
    return None


# The element build is bound by instruction issue (FP32 pipe for the
# double-float rows, FP64 for the DR scalars): its roofline is the SMs'
# issue rate, 4 warp instructions per SM per clock, against the warp
# instructions per element that ncu counted for the kernel.
BUILD_PROFILE = "elem_build_geo_rotation_shear_128x128x64.md"
ISSUE_PER_SM_CLOCK = 4.0


def profile_traffic():
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary: a 1M-element capture's traffic scaled to the bench size by the
    units processed (traffic grows in proportion to E and N)."""
    return profile_value("stored_apply_df_rotation_shear.md",
                         "traffic_bytes_per_launch")


# --------------------------------------------------------------- CPU legs
def cpu_solve_sample(prob, dt, iters, full=False):
    """The oracle port on the host cores: OpenMP assembly of the whole
    system + `iters` BiCGStab iterations with the OpenMP colour-parallel
    apply (or a full solve).  Returns timings."""
    import numpy as np
    import oracle as O
    threads = os.cpu_count() or 1
    m = prob.mesh
    t0 = time.perf_counter()
    bb, b, d = O.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss, prob.vel,
                          prob.lam, prob.pdec, prob.q, kod=m.kod,
                          robin_alpha=prob.robin_alpha, aH=2.0, aM=3.0 / dt,
                          cf=3.0, rM=3.0 / dt, nthreads=threads)
    b[prob.bc == 1] = 0.0
    d[prob.bc == 1] = 1.0
    t_asm = time.perf_counter() - t0
    c, nc = O.greedy_colors(m.iss, m.nnode)
    ce, co = O.color_lists(c, nc)
    t0 = time.perf_counter()
    x, it, err, st = O.bicgstab(b, np.zeros(m.nnode), bb, m.iss, d, prob.bc,
                                TOL, 100000 if full else iters,
                                colors=(ce, co), nthreads=threads)
    t_sol = time.perf_counter() - t0
    return {"t_asm": t_asm, "t_solve": t_sol, "iters": it, "err": err,
            "status": st, "threads": threads}


def run_reference(a):
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    prob, dt = make_problem(a)
    # the oracle's own iteration count, from one full CPU solve
    full = cpu_solve_sample(prob, dt, 0, full=True)
    n_it = full["iters"]
    vals = []
    for k in range(a.warmup + a.steps):
        s = cpu_solve_sample(prob, dt, a.cpu_iters)
        proj = s["t_asm"] + n_it * s["t_solve"] / max(1, s["iters"])
        if k >= a.warmup:
            vals.append(proj)
    v = statistics.mean(vals)
    sample = ("per step: full-system OpenMP assembly + %d BiCGStab iterations "
              "(OpenMP colour-parallel apply) on %d threads, projected to the "
              "%d iterations of one full CPU solve (that solve: %.1f s)"
              % (a.cpu_iters, full["threads"], n_it,
                 full["t_asm"] + full["t_solve"]))
    line = {"metric": METRIC, "value": v, "unit": "s", "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": v * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": workload_config(a, prob),
            "cpu_baseline": {"value": v, "unit": "s",
                             "cores": full["threads"], "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "reference_iterations": n_it}
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------- GPU arm
def timed_steps(s, stream, b, x, aH, aM, cf, rM, solve, reps=3):
    """One theta step on handle `s`, timed on its stream: the operator
    invalidated, element matrices + Jacobi diagonal + right-hand side in one
    element pass, then `solve()` from x = 0.  Returns the medians over
    `reps` (after one untimed step) of (build + RHS, solve alone, whole
    step) in seconds, and the last solve's return value."""
    import torch
    builds, solves, steps = [], [], []
    out = None
    for k in range(reps + 1):
        with torch.cuda.stream(stream):
            x.zero_()
        s.set_operator(aH, aM)
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        s.assemble_rhs_device(b, cf, rM, None)
        e1.record(stream)
        out = solve()
        e2.record(stream)
        torch.cuda.synchronize()
        if k:
            builds.append(e0.elapsed_time(e1) / 1e3)
            solves.append(e1.elapsed_time(e2) / 1e3)
            steps.append(e0.elapsed_time(e2) / 1e3)
    return (statistics.median(builds), statistics.median(solves),
            statistics.median(steps), out)


def _r(v, n=4):
    """v to n significant digits (short summary keys)."""
    if v is None or not isinstance(v, (int, float)) or v != v:
        return v
    return float("%.*g" % (n, v))


BATCH_MESH = (128, 128, 64)
BATCH_K = 64


BLOCK_TILE_KERNEL = ("block_apply_tile<split> (8x2x2-element boxes, node rows "
                     "staged in shared memory by cp.async, mma.sync m16n8k8 TF32 "
                     "x3, one float4 atomic per node and 4 columns)")
BLOCK_TC_KERNEL = ("block_apply_tc_kernel<split> (4x4x4-element boxes: element "
                   "matrices and node rows by 4-D TMA, box operator assembled "
                   "in TMEM, node rows split and transposed in shared memory, "
                   "tcgen05.mma kind::tf32 x3 M=128 N=128+64 K=128, Y by two "
                   "TMA tensor reduces per box)")


def batched_rhs_section(vdr, device):
    """Many right-hand sides with one operator: the 128x128x64 rotation +
    shear mesh (same theta-step operator at Courant 10), K = 64 seeded
    Gaussian sources, every column to FP64 relative residual 1e-8 by the
    block solve (FP64 refinement around K simultaneous FP32 BiCGStab solves
    with the split-TF32 tensor-core block apply), against the same 64
    columns solved one at a time by the FP64 path."""
    import torch
    P = vdr.problems
    nx, ny, nz = BATCH_MESH
    prob = P.rotation_shear(nx, ny, nz, seed=1004)
    dt = COURANT / max(nx, ny, nz)
    aH, aM = 2.0, 3.0 / dt
    N, E = prob.mesh.nnode, prob.mesh.nelem
    K = BATCH_K
    s = vdr.Solver(prob, vdr.Options(apply_mode="stored", device=device),
                   aH=aH, aM=aM)
    st = torch.cuda.ExternalStream(s.stream())
    Qd = torch.as_tensor(P.random_gaussian_sources(prob.mesh, K),
                         device="cuda")
    B = torch.empty((N, K), dtype=torch.float64, device="cuda")
    s.assemble_rhs_block_device(Qd, B, 3.0)
    X = torch.zeros_like(B)
    times = []
    for rep in range(3):
        with torch.cuda.stream(st):
            X.zero_()
        e0, e1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
        e0.record(st)
        no, ni, errs, bst = s.solve_block_device(B, X, tol=TOL, inner_tol=1e-4,
                                                 precision="tf32x3")
        e1.record(st)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    t_block = statistics.median(times[1:])
    # the same columns one at a time, FP64 Jacobi-BiCGStab
    xs = torch.zeros(N, dtype=torch.float64, device="cuda")
    bs = torch.empty_like(xs)
    its = []
    s.solve_device(B[:, 0].contiguous(), xs, tol=TOL, itmax=20000)  # warm
    e0, e1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
    torch.cuda.synchronize()
    e0.record(st)
    worst_single = 0.0
    for k in range(K):
        with torch.cuda.stream(st):
            bs.copy_(B[:, k])
            xs.zero_()
        it, err, sst = s.solve_device(bs, xs, tol=TOL, itmax=20000)
        its.append(it)
        worst_single = max(worst_single, err)
    e1.record(st)
    torch.cuda.synchronize()
    t_single = e0.elapsed_time(e1) / 1e3
    # block apply roofline (split TF32, K columns): the accumulating call,
    # so that only the apply kernel runs between the events
    Xf = torch.randn((N, K), dtype=torch.float32, device="cuda")
    Yf = torch.zeros_like(Xf)
    for _ in range(3):
        s.apply_block_accumulate_device(Xf, Yf, "tf32x3")
    def time_apply(reps=20):
        r0, r1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
        torch.cuda.synchronize()
        r0.record(st)
        for _ in range(reps):
            s.apply_block_accumulate_device(Xf, Yf, "tf32x3")
        r1.record(st)
        torch.cuda.synchronize()
        return r0.elapsed_time(r1) / reps
    t_apply = time_apply()
    tuning = {k: v for k, v in s.apply_tuning().items() if k.startswith("block")}
    # both K = 64 forms on their own (the solve above used the measured choice)
    form_ms = {}
    for form in ("tile", "tcgen05"):
        s.set_block_apply(form)
        for _ in range(3):
            s.apply_block_accumulate_device(Xf, Yf, "tf32x3")
        form_ms[form] = time_apply()
    s.set_block_apply("auto")
    # FP32 element matrix (256 B) per element (the node-tile kernel forms
    # node numbers from the structured numbering: no connectivity read); X
    # read once and Y read + written once (4 B per column per node)
    alg = 256.0 * E + 12.0 * K * N
    peak, peak_kind = measured_peak()
    ach = alg / (t_apply * 1e-3) / 1e9
    out = {"workload": "rotation_shear %dx%dx%d, theta-step at Courant %g, "
                       "K=%d seeded Gaussian sources, every column to FP64 "
                       "relative residual %g" % (nx, ny, nz, COURANT, K, TOL),
           "elements": E, "nodes": N, "K": K,
           "block_solve_s": t_block, "per_rhs_s": t_block / K,
           "outer_corrections": no, "inner_iterations": ni,
           "worst_fp64_rel_residual": float(errs.max()), "status": bst,
           "sequential_fp64_s": t_single,
           "sequential_fp64_iterations_max": max(its),
           "sequential_worst_rel_residual": worst_single,
           "speedup_vs_sequential_fp64": t_single / t_block,
           "block_apply": {"kernel": BLOCK_TC_KERNEL if tuning["block_tcgen05"]
                                     else BLOCK_TILE_KERNEL,
                           "ms": t_apply, "achieved_gbs": ach,
                           "algorithmic_bytes": alg, "peak": peak,
                           "frac": ach / peak, "peak_kind": peak_kind,
                           "form_ms": form_ms,
                           "form_frac": {f: alg / (ms * 1e-3) / 1e9 / peak
                                         for f, ms in form_ms.items()}}}
    out["block_apply"]["tuning"] = tuning
    s.close()
    return out


MESHES = 256
MESH_DT = COURANT / 32.0   # one time step for every mesh: Courant 2.5..15


def batched_meshes_section(vdr, device):
    """256 independent meshes of uneven size (cube edges drawn from 8..48
    elements, seeds 2001+m), each with a random-axis rotation field,
    lognormal diffusivity and a Gaussian source, theta-step operator with
    dt = 10/32 for all: every mesh to FP64 relative residual 1e-8 in one
    segmented solve (per-mesh BiCGStab scalars, all meshes in one CUDA
    graph, autotuned tile shape), against the same meshes solved one at a
    time on their own handles."""
    import numpy as np
    import torch
    P = vdr.problems
    t0 = time.perf_counter()
    probs = P.cube_batch(MESHES, seed=2001, nmin=8, nmax=48)
    union = P.concat(probs)
    t_gen = time.perf_counter() - t0
    aH, aM = 2.0, 3.0 / MESH_DT
    s = vdr.Solver(union, vdr.Options(apply_mode="stored", device=device),
                   aH=aH, aM=aM)
    s.set_segments(union.mesh.node_off)
    st_ = torch.cuda.ExternalStream(s.stream())
    N = union.mesh.nnode
    b = torch.empty(N, dtype=torch.float64, device="cuda")
    x = torch.zeros_like(b)
    torch.cuda.synchronize()
    s.assemble_rhs_device(b, 3.0, 0.0, None)
    times = []
    for rep in range(3):
        with torch.cuda.stream(st_):
            x.zero_()
        e0, e1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
        e0.record(st_)
        its, errs, sts, st = s.solve_segmented_device(b, x, tol=TOL, itmax=5000)
        e1.record(st_)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    t_batch = statistics.median(times[1:])
    tile, threads = s.segment_tuning()
    # element build + right-hand side of all meshes in one pass
    e0, e1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
    e0.record(st_)
    s.set_operator(aH, aM)
    s.assemble_rhs_device(b, 3.0, 0.0, None)
    e1.record(st_)
    torch.cuda.synchronize()
    t_build = e0.elapsed_time(e1) / 1e3
    bh = b.cpu().numpy()
    s.close()
    # the same meshes one at a time (each on its own handle; setup untimed)
    off = union.mesh.node_off
    t_seq = 0.0
    seq_its = []
    worst = 0.0
    for m, p in enumerate(probs):
        sm = vdr.Solver(p, vdr.Options(apply_mode="stored", device=device),
                        aH=aH, aM=aM)
        bm = torch.as_tensor(bh[off[m]:off[m + 1]], device="cuda")
        xm = torch.zeros_like(bm)
        torch.cuda.synchronize()
        sm.solve_device(bm, xm, tol=TOL, itmax=5000)      # warm (graph)
        xm.zero_()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        it, err, stm = sm.solve_device(bm, xm, tol=TOL, itmax=5000)
        torch.cuda.synchronize()
        t_seq += time.perf_counter() - t1
        seq_its.append(it)
        worst = max(worst, err)
        sm.close()
    return {"workload": "%d rotation cubes, edges 8..48 elements (seeds "
                        "2001+m), theta-step dt=10/32, each mesh to FP64 "
                        "relative residual %g" % (MESHES, TOL),
            "meshes": MESHES, "elements": int(union.mesh.nelem),
            "nodes": int(N),
            "segmented_solve_s": t_batch,
            "build_and_rhs_s": t_build,
            "iterations_max": int(its.max()),
            "iterations_mean": float(its.mean()),
            "all_converged": bool(np.all(sts == 0)),
            "worst_rel_residual": float(errs.max()),
            "autotuned_tile": {"nodes": tile, "threads": threads},
            "one_at_a_time_s": t_seq,
            "one_at_a_time_iterations_max": int(max(seq_its)),
            "one_at_a_time_worst_rel_residual": worst,
            "speedup_vs_one_at_a_time": t_seq / t_batch,
            "generation_s": t_gen}


LEARN_MESH = (128, 128, 64)
LEARN_STEPS = 200
LEARN_TRAIN_STEPS = 40
LEARN_PAIRS = 50           # per training step: 2000 pairs
LEARN_DAGGER_PAIRS = 25    # per training step, from the learned solver
LEARN_TILT = 0.5


def dropin_section(vdr, s, prob, cf, rM):
    """The reference's own solve entry on the 256x256x128 step:
    kernel_dbcg_simple_ called with host arrays as VANADIS.FOR:809 calls it -- B, X, BB (64E doubles, 4.3 GB),
    ISS, DIAG and bc uploaded and X downloaded on every call -- on the
    GPU-built theta-step operator, exported once in the reference's BB layout
    (vdr_get_element_matrices); Jacobi-preconditioned BiCG, the reference's
    method, to 1e-8 from X = 0."""
    import ctypes
    import numpy as np
    import torch
    m = prob.mesh
    N, E = m.nnode, m.nelem
    keep = []

    def pinned(n, dtype):
        t = torch.empty(n, dtype=dtype, pin_memory=True)
        keep.append(t)
        return t.numpy()

    bb = pinned(64 * E, torch.float64)
    s.element_matrices(out=bb)
    diag = pinned(N, torch.float64)
    diag[:] = s.diag()
    b = pinned(N, torch.float64)
    s.assemble_rhs(cf, rM, None, out=b)
    iss = pinned(8 * E, torch.int32)
    iss[:] = np.ascontiguousarray(m.iss, dtype=np.int32).ravel()
    bc = pinned(N, torch.int32)
    bc[:] = np.asarray(prob.bc, dtype=np.int32)
    x = pinned(N, torch.float64)
    lib = vdr.load_library()
    n_, tol_, itmax_ = ctypes.c_int(N), ctypes.c_double(TOL), ctypes.c_int(20000)
    it_, err_ = ctypes.c_int(0), ctypes.c_double(0.0)
    nax, nay, naz = (ctypes.c_int(int(v)) for v in (m.nax, m.nay, m.naz))
    pd = lambda arr: arr.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    pi = lambda arr: arr.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    times = []
    for k in range(6):
        x[:] = 0.0
        t0 = time.perf_counter()
        lib.kernel_dbcg_simple_(ctypes.byref(n_), pd(b), pd(x), ctypes.byref(tol_),
                                ctypes.byref(itmax_), ctypes.byref(it_),
                                ctypes.byref(err_), pd(bb), pi(iss), pd(diag),
                                ctypes.byref(nax), ctypes.byref(nay),
                                ctypes.byref(naz), pi(bc))
        times.append(time.perf_counter() - t0)
    h2d = 8 * (64 * E + 3 * N) + 4 * (8 * E + N)
    # the same BB upload alone (pinned host -> device), for the split
    dbb = torch.empty(64 * E, dtype=torch.float64, device="cuda")
    hbb = torch.from_numpy(bb)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dbb.copy_(hbb, non_blocking=True)
    torch.cuda.synchronize()
    t_bb = time.perf_counter() - t0
    del dbb
    return {"workload": "rotation_shear 256x256x128 theta-step system, BB from "
                        "the GPU build; Jacobi BiCG to 1e-8 from X = 0",
            "call_s": statistics.median(times[1:]), "call_s_min": min(times[1:]),
            "call_s_each": times[1:], "bb_upload_alone_s": t_bb,
            "note": "host-to-device bandwidth on the shared box varies between "
                    "runs (the 4.3 GB BB upload alone took 0.02-0.15 s)",
            "iterations": it_.value,
            "err": err_.value, "h2d_bytes_per_call": h2d,
            "d2h_bytes_per_call": 8 * N,
            "what": "kernel_dbcg_simple_ with host arrays: uploads, BB to the "
                    "double-float store, graph-captured BiCG with the fused "
                    "A p / A^T p~ apply, X download"}


def text_output_section(vdr, prob, x):
    """The step's text output at the bench size: the T_sssss.TXT text of the
    solution (x, y, z, T * 1e6 per node in Fortran e12.5 fields, 55 bytes a
    line) formatted by the library's host threads into memory, then the
    file written to a scratch directory (the disk's speed, for context)."""
    import tempfile
    import numpy as np
    m = prob.mesh
    t = x.cpu().numpy()
    text = np.empty(55 * m.nnode, dtype=np.uint8)
    fmt = []
    for _ in range(2):
        t0 = time.perf_counter()
        vdr.format_result_txt(m.xx, m.yy, m.zz, t, 1e6, out=text)
        fmt.append(time.perf_counter() - t0)
    with tempfile.TemporaryDirectory() as d:
        t0 = time.perf_counter()
        vdr.write_result_txt(d, 1, m.xx, m.yy, m.zz, t, 1e6)
        t_write = time.perf_counter() - t0
    t_fmt = min(fmt)
    return {"nodes": int(m.nnode), "bytes": int(text.size), "format_s": t_fmt,
            "format_mb_s": text.size / t_fmt / 1e6,
            "format_lines_per_s": m.nnode / t_fmt,
            "write_file_s": t_write, "host_threads": os.cpu_count(),
            "what": "vdr_format_result_txt / vdr_write_result_txt: the "
                    "reference's T_sssss.TXT (format 122) of one step"}


def time_loop_section(vdr, s, prob, aH, aM, cf, rM):
    """The device time loop (vdr_time_steps) on the 256x256x128 rotation +
    shear theta step: per step the right-hand side from T, the solve to 1e-8
    and the mass integral, T kept on the device.  The first step of a call
    builds the element matrices (keeping M and F = sum f_e); every later step
    forms its right-hand side from the stored A and M.  Calls of 1 and 6
    steps from T = 0; a later step costs (t6 - t1) / 5."""
    import torch
    N = prob.mesh.nnode
    runs = {}
    for n in (1, 6, 1, 6):
        t = torch.zeros(N, dtype=torch.float64, device="cuda")
        s.set_operator(aH, aM)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        masses, its, errs, st, done = s.time_steps_device(t, n, cf, rM, tol=TOL,
                                                          itmax=20000)
        torch.cuda.synchronize()
        runs[n] = (time.perf_counter() - t0, [int(v) for v in its], int(st),
                   float(max(errs)))
    t1, t6 = runs[1][0], runs[6][0]
    out = {"steps_1_s": t1, "steps_6_s": t6, "later_step_s": (t6 - t1) / 5,
           "iterations": runs[6][1], "status": runs[6][2],
           "worst_rel_residual": runs[6][3],
           "what": "vdr_time_steps from T = 0: first step = element build "
                   "(A, M, F) + solve, later steps = RHS from two applies + "
                   "solve; mass integral every step"}
    # the same loop with Options(precision="mixed"): FP64 refinement around
    # FP32-operator inner solves, same FP64 tolerance, on its own handle
    sm = vdr.Solver(prob, vdr.Options(apply_mode="stored", precision="mixed"),
                    aH=aH, aM=aM)
    mruns = {}
    for n in (1, 6, 1, 6):
        t = torch.zeros(N, dtype=torch.float64, device="cuda")
        sm.set_operator(aH, aM)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        masses, its, errs, st, done = sm.time_steps_device(t, n, cf, rM, tol=TOL,
                                                           itmax=20000)
        torch.cuda.synchronize()
        mruns[n] = (time.perf_counter() - t0, [int(v) for v in its], int(st),
                    float(max(errs)))
    sm.close()
    out["mixed"] = {"steps_1_s": mruns[1][0], "steps_6_s": mruns[6][0],
                    "later_step_s": (mruns[6][0] - mruns[1][0]) / 5,
                    "inner_iterations": mruns[6][1], "status": mruns[6][2],
                    "worst_fp64_rel_residual": mruns[6][3]}
    return out


# FLOPs of one forward pass of the network (3x3x3 convolutions, 2 per
# multiply-add) per level-0 voxel: sum over layers of 27 cin cout x (voxels
# of the layer's level / voxels of level 0), with levels 1 and 2 holding
# ~1/8 and ~1/64 of the voxels (computed exactly from the grid below).
def network_flops(dims):
    layers = [(16, 16, 0), (16, 16, 0), (16, 32, 1), (32, 32, 1), (32, 64, 2),
              (64, 64, 2), (96, 32, 1), (32, 32, 1), (48, 16, 0), (16, 16, 0)]
    return sum(2.0 * 27 * ci * co * dims[l] for ci, co, l in layers)


def network_forward_times(vdr, net, run, reps=10):
    """One forward pass of the network on the workload's grid, per
    convolution path, timed with CUDA events on the library's stream; the
    rate counts the convolutions' FLOPs (the pools, upsampled copies and
    head are in the time, not in the count)."""
    import torch
    m = run.prob.mesh
    n0 = (m.nax, m.nay, m.naz)
    n1 = tuple((v + 1) // 2 for v in n0)
    n2 = tuple((v + 1) // 2 for v in n1)
    vox = [n0[0] * n0[1] * n0[2], n1[0] * n1[1] * n1[2], n2[0] * n2[1] * n2[2]]
    flops = network_flops(vox)
    net.update_features(None)
    st = torch.cuda.ExternalStream(run.s.stream())
    rh = torch.randn(m.nnode, dtype=torch.float32, device="cuda")
    out = torch.empty_like(rh)
    torch.cuda.synchronize()
    res = {"gflop": flops / 1e9}
    for mode in ("tcgen05", "mma"):
        net.set_conv(mode)
        for _ in range(3):
            net.forward(rh, out)
        e0, e1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
        torch.cuda.synchronize()
        e0.record(st)
        for _ in range(reps):
            net.forward(rh, out)
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        res[mode] = {"ms": ms, "tflops": flops / (ms * 1e-3) / 1e12}
    net.set_conv("tcgen05")
    res["speedup"] = res["mma"]["ms"] / res["tcgen05"]["ms"]
    return res


def learned_section(vdr, device, a):
    """The learned preconditioner on the tilting-axis transient problem
    (128x128x64, theta-step at Courant 10, rotation axis tilting 0.5 degrees
    per step, every step to FP64 relative residual 1e-8).  Steps 0-39 give
    2000 (residual, error) pairs from the Jacobi-BiCGStab solves' iterates;
    the network is trained on the GPU (residual loss), then once more on
    pairs from its own GCR solves of the same steps; steps 40-199 are solved
    by Jacobi-BiCGStab and by two learned GCR steps followed by
    Jacobi-BiCGStab, from the same T_old each step; pure learned GCR is
    measured on the first 8 of them."""
    import numpy as np
    import torch
    L = vdr.learned
    nx, ny, nz = LEARN_MESH
    t_all = time.perf_counter()
    run = L.TiltingRun(nx, ny, nz, seed=1005, courant=COURANT, tol=TOL,
                       tilt_deg=LEARN_TILT, device=device)
    net = vdr.LearnedNet(run.s, seed=5)
    net.set_smoothing(0)
    fwd = network_forward_times(vdr, net, run)
    steps_train = list(range(LEARN_TRAIN_STEPS))
    total = a.learn_steps
    t0 = time.perf_counter()
    T0 = run.T.clone()
    data = L.collect_pairs(run, net, steps_train, pairs_per_step=LEARN_PAIRS)
    T_after = run.T.clone()
    t_collect = time.perf_counter() - t0
    t0 = time.perf_counter()
    curve0 = L.train(net, data, epochs=a.learn_epochs, lr=1e-3, loss="residual",
                     run=run)
    t_train0 = time.perf_counter() - t0
    t0 = time.perf_counter()
    with torch.cuda.stream(run.stream):
        run.T.copy_(T0)
    more = L.collect_pairs_learned(run, net, steps_train,
                                   pairs_per_step=LEARN_DAGGER_PAIRS,
                                   max_iters=40)
    curve1 = L.train(net, more, epochs=1, lr=5e-4, loss="residual", run=run,
                     seed=1)
    t_train1 = time.perf_counter() - t0
    with torch.cuda.stream(run.stream):
        run.T.copy_(T_after)
    torch.cuda.synchronize()
    # every remaining step: Jacobi-BiCGStab vs 2 learned GCR steps then
    # Jacobi-BiCGStab
    res = L.evaluate(run, net, range(LEARN_TRAIN_STEPS, total), method="hybrid",
                     restart=2)
    # pure learned GCR(20) on the first 8 of them (capped at 300 iterations,
    # Jacobi-BiCGStab after a 20-iteration stall)
    with torch.cuda.stream(run.stream):
        run.T.copy_(T_after)
    torch.cuda.synchronize()
    pure = L.evaluate(run, net, range(LEARN_TRAIN_STEPS, LEARN_TRAIN_STEPS + 8),
                      method="gcr", restart=20, stall_window=20, itmax=300)

    def summary(rows, key):
        its = [r[key + "_iters"] for r in rows]
        return {"solve_s_total": sum(r[key + "_s"] for r in rows),
                "mean_iterations": float(np.mean(its)),
                "max_iterations": int(max(its))}

    jt = sum(r["jacobi_s"] for r in res)
    lt = sum(r["learned_s"] for r in res)
    out = {
        "workload": "tilting-axis rotation_shear %dx%dx%d, %d theta-steps at "
                    "Courant %g (axis tilts %g deg/step), each to FP64 "
                    "relative residual %g" % (nx, ny, nz, total, COURANT,
                                              LEARN_TILT, TOL),
        "network": "3-level 3D U-Net 16/32/64 channels, 3^3 kernels, BF16 "
                   "weights/activations, FP32 accumulate; forward convolutions "
                   "on tcgen05 (TMA halo slabs, TMEM accumulators), backward "
                   "passes on mma.sync m16n8k16",
        "network_forward": fwd,
        "training": {"pairs": int(data["rhat"].shape[0]),
                     "pairs_from_learned_solves": int(more["rhat"].shape[0]),
                     "epochs": a.learn_epochs, "loss": "residual",
                     "loss_curve": curve0 + curve1,
                     "collect_s": t_collect, "train_s": t_train0,
                     "second_round_s": t_train1},
        "eval_steps": len(res),
        "jacobi_bicgstab": summary(res, "jacobi"),
        "learned_then_jacobi": dict(
            summary(res, "learned"),
            what="2 GCR steps with the network, then Jacobi-BiCGStab",
            worst_true_residual=float(max(r["learned_true_residual"]
                                          for r in res)),
            all_converged=all(r["learned_status"] == 0 for r in res),
            worst_rel_diff_vs_fp64=float(max(r["rel_diff"] for r in res))),
        "learned_vs_plain_time": lt / jt if jt > 0 else None,
        "pure_learned_gcr_first_8_steps": dict(
            summary(pure, "learned"),
            jacobi_bicgstab=summary(pure, "jacobi"),
            fell_back=int(sum(r["fell_back"] for r in pure)),
            all_converged=all(r["learned_status"] == 0 for r in pure)),
        "section_s": time.perf_counter() - t_all,
    }
    net.close()
    run.close()
    return out


def run_native(a):
    import numpy as np
    import torch
    import __graft_entry__

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    vdr = __graft_entry__.package()
    vdr.load_library()
    prob, dt = make_problem(a)
    N, E = prob.mesh.nnode, prob.mesh.nelem
    aH, aM, cf, rM = 2.0, 3.0 / dt, 3.0, 3.0 / dt
    opts = vdr.Options(apply_mode="stored", scatter=a.scatter,
                       solver="bicgstab", device=local)
    s = vdr.Solver(prob, opts, aH=aH, aM=aM)
    stream = torch.cuda.ExternalStream(s.stream())
    b = torch.zeros(N, dtype=torch.float64, device="cuda")
    x = torch.zeros_like(b)
    torch.cuda.synchronize()

    def step():
        with torch.cuda.stream(stream):
            x.zero_()
        s.set_operator(aH, aM)          # element matrices rebuilt this step
        s.assemble_rhs_device(b, cf, rM, None)
        it, err, st = s.solve_device(b, x, tol=TOL, itmax=20000)
        return it, err, st

    for _ in range(a.warmup):
        it, err, st = step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = vdr.kernel_launch_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    iters = []
    for _ in range(a.steps):
        it, err, st = step()
        iters.append(it)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / a.steps
    launches = vdr.kernel_launch_count() - launches0
    clk = clocks.stop()
    if world > 1:
        ms = reduce_max_over_ranks(ms, "cuda")
    rel_true = s.true_residual_device(b, x)
    stats = s.stats()

    # ---- step = element matrices + RHS, then the solve alone ----
    t_build_s, t_krylov_s, step_s, fp64_out = timed_steps(
        s, stream, b, x, aH, aM, cf, rM,
        lambda: s.solve_device(b, x, tol=TOL, itmax=20000))
    t_build, t_krylov = t_build_s * 1e3, t_krylov_s * 1e3
    y = torch.zeros_like(b)

    # ---- roofline of the dominant kernel: stored EBE apply ----
    xr = torch.randn(N, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    reps = 20
    for _ in range(3):
        s.apply_accumulate_device(xr, y)
    r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    r0.record(stream)
    for _ in range(reps):
        s.apply_accumulate_device(xr, y)
    r1.record(stream)
    torch.cuda.synchronize()
    t_apply_ms = r0.elapsed_time(r1) / reps
    alg_bytes = 544.0 * E + 24.0 * N
    peak, peak_kind = measured_peak()
    achieved = alg_bytes / (t_apply_ms * 1e-3) / 1e9
    traffic = profile_traffic()

    # ---- element build: roofline against the SMs' instruction issue rate ----
    inst_per_elem = profile_value(BUILD_PROFILE, "warp_instructions_per_element")
    n_sm = torch.cuda.get_device_properties(local).multi_processor_count
    sm_mhz = (clk or {}).get("sm_mhz") or 2070.0
    issue_peak = n_sm * ISSUE_PER_SM_CLOCK * sm_mhz * 1e6 / 1e9   # G/s
    build_issue = (inst_per_elem * E / (t_build * 1e-3) / 1e9
                   if inst_per_elem else None)

    # ---- the build that evaluates the Jacobians from the coordinates at
    # every step (no geometric factors), and the one-time cost of forming
    # the factors (the first build after they were dropped) ----
    geo_state, geo_bytes = s.geometry_status()
    s.set_build_mode("recompute")
    t_build_rc_s, _, _, _ = timed_steps(s, stream, b, x, aH, aM, cf, rM, lambda: None)
    s.set_build_mode("auto")   # the factors were freed: the next build forms them
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.set_operator(aH, aM)
    g0.record(stream)
    s.assemble_rhs_device(b, cf, rM, None)
    g1.record(stream)
    torch.cuda.synchronize()
    build_modes = {
        "geometric_factors_ms": t_build, "recompute_ms": t_build_rc_s * 1e3,
        "first_build_with_factor_setup_ms": g0.elapsed_time(g1),
        "geometry_bytes": geo_bytes, "geometry_state": geo_state,
        "what": "element build + diag + RHS per step: from the mesh's "
                "geometric factors (J^-1, detJ per Gauss point and the "
                "unit-diffusivity stiffness, formed once per handle; the "
                "headline step) vs evaluating the Jacobians from the "
                "coordinates at every step"}

    # ---- the same step with the pure FP64 element-matrix store ----
    s64 = vdr.Solver(prob, vdr.Options(apply_mode="stored",
                                       matrix_storage="fp64",
                                       solver="bicgstab", device=local),
                     aH=aH, aM=aM)
    st64 = torch.cuda.ExternalStream(s64.stream())
    x64 = torch.zeros_like(b)
    b64 = torch.zeros_like(b)
    _, f64_solve, f64_step, f64_out = timed_steps(
        s64, st64, b64, x64, aH, aM, cf, rM,
        lambda: s64.solve_device(b64, x64, tol=TOL, itmax=20000))
    fp64_store = {"step_s": f64_step, "solve_s": f64_solve,
                  "iterations": f64_out[0], "rel_residual": f64_out[1],
                  "status": f64_out[2],
                  "rel_l2_vs_double_float_solution":
                      float(torch.linalg.norm(x64 - x) / torch.linalg.norm(x)),
                  "what": "element matrices kept as FP64 (512 B/element), "
                          "contracted on the FP64 pipe"}
    s64.close()
    del x64, b64

    # ---- mixed precision (FP32 operator inside FP64 refinement) ----
    xm = torch.zeros_like(b)
    with torch.cuda.stream(stream):
        x.zero_()
    s.set_operator(aH, aM)
    s.assemble_rhs_device(b, cf, rM, None)
    s.solve_device(b, x, tol=TOL, itmax=20000)        # FP64 reference solution
    torch.cuda.synchronize()

    def mixed_step(op, inner_tol=1e-5):
        s.set_mixed_operator(op)
        _, t_solve, t_step, out = timed_steps(
            s, stream, b, xm, aH, aM, cf, rM,
            lambda: s.solve_mixed_device(b, xm, tol=TOL, inner_tol=inner_tol))
        mo, mi, merr, mst = out
        return {"value": t_step, "unit": "s", "solve_s": t_solve,
                "outer_corrections": mo, "inner_iterations": mi,
                "fp64_rel_residual": merr, "status": mst,
                "true_rel_residual": s.true_residual_device(b, xm),
                "rel_l2_vs_fp64_solution": float(torch.linalg.norm(xm - x) /
                                                 torch.linalg.norm(x))}

    recompute = mixed_step("recompute")
    rounded = mixed_step("rounded")
    mixed = mixed_step("half", inner_tol=1e-3)
    s.set_mixed_operator("rounded")
    mixed["what"] = ("Jacobi-scaled projected operator P A P D^-1 in binary16 "
                     "(one power-of-two scale per element, 128 B/element, "
                     "built from the FP64 element matrices inside the solve) "
                     "in FP32-vector BiCGStab inside FP64 refinement; each "
                     "correction solved to max(1e-3, 0.5 tol/outer residual); "
                     "the step includes the element build")
    mixed["speedup_vs_fp64_step"] = (ms / 1e3) / mixed["value"]
    mixed["speedup_vs_fp64_solve"] = t_krylov_s / mixed["solve_s"]
    rounded["what"] = ("FP64 element matrices rounded to FP32 (the hi parts of "
                       "the double-float store, 256 B/element), Jacobi "
                       "vectors, corrections to max(1e-5, 0.5 tol/outer "
                       "residual)")
    recompute["what"] = ("element Jacobians and DR terms recomputed in FP32, "
                         "FP32 element matrices, same refinement as rounded")
    mixed["fp32_rounded_variant"] = rounded
    mixed["fp32_recompute_variant"] = recompute

    # ---- the other scatter forms of the same step: colour by colour (no
    # atomics) and warp-aggregated atomics ----
    scatter_variants = {
        "atomic": {"step_s": ms / 1e3, "solve_s": t_krylov_s,
                   "apply_ms": t_apply_ms, "apply_gbs": achieved,
                   "iterations": fp64_out[0]}}
    for form in ("color", "warp"):
        sc = vdr.Solver(prob, vdr.Options(apply_mode="stored", scatter=form,
                                          solver="bicgstab", device=local),
                        aH=aH, aM=aM)
        cstream = torch.cuda.ExternalStream(sc.stream())
        xc = torch.zeros_like(b)
        bcv = torch.zeros_like(b)
        _, c_solve, c_step, c_out = timed_steps(
            sc, cstream, bcv, xc, aH, aM, cf, rM,
            lambda: sc.solve_device(bcv, xc, tol=TOL, itmax=20000))
        yc = torch.zeros_like(b)
        for _ in range(3):
            sc.apply_accumulate_device(xr, yc)
        c2e, c3e = (torch.cuda.Event(enable_timing=True) for _ in range(2))
        c2e.record(cstream)
        for _ in range(reps):
            sc.apply_accumulate_device(xr, yc)
        c3e.record(cstream)
        torch.cuda.synchronize()
        a_ms = c2e.elapsed_time(c3e) / reps
        scatter_variants[form] = {
            "step_s": c_step, "solve_s": c_solve, "apply_ms": a_ms,
            "apply_gbs": alg_bytes / (a_ms * 1e-3) / 1e9,
            "iterations": c_out[0], "status": c_out[2],
            "rel_l2_vs_atomic_solution":
                float(torch.linalg.norm(xc - x) / torch.linalg.norm(x))}
        sc.close()
        del xc, bcv, yc
    scatter_variants["warp"]["what"] = (
        "FP64 atomics after neighbouring lanes add their shared x-face nodes "
        "by shuffles (4 instead of 8 atomics per element)")
    scatter_variants["color"]["what"] = "8 launches per apply, no atomics"

    # ---- the launch shapes the handle chose by measurement (the binary16
    # apply's after the mixed steps above) ----
    tuning = s.apply_tuning()

    def section(skip, fn, *args):
        """An optional section; a failure is reported in its key (and on
        stderr) instead of ending the run without the headline line."""
        if skip:
            return None
        try:
            return fn(*args)
        except Exception as exc:  # noqa: BLE001 -- reported, not hidden
            import traceback
            traceback.print_exc()
            return {"error": "%s: %s" % (type(exc).__name__, exc)}

    batched = section(a.no_batched, batched_rhs_section, vdr, local)
    meshes = section(a.no_meshes, batched_meshes_section, vdr, local)
    learned = section(a.no_learned, learned_section, vdr, local, a)
    dropin = section(a.no_dropin, dropin_section, vdr, s, prob, cf, rM)
    tloop = section(a.no_time_loop, time_loop_section, vdr, s, prob, aH, aM, cf, rM)
    text_out = section(a.no_text, text_output_section, vdr, prob, x)

    # ---- e2e through the C ABI with host buffers ----
    # The step's inputs (per-element fields) and outputs (right-hand side,
    # solution) live in pinned host memory; every step uploads the fields,
    # assembles and downloads b, uploads b and x and downloads x.
    keep = []

    def pinned(arr):
        t = torch.empty(arr.shape, dtype=torch.float64, pin_memory=True)
        keep.append(t)
        view = t.numpy()
        view[:] = arr
        return view

    vel, lam, pdec, q = (pinned(v) for v in (prob.vel, prob.lam, prob.pdec,
                                             prob.q))
    bh = pinned(np.zeros(N))
    xh = pinned(np.zeros(N))
    h2d = 8 * (vel.size + lam.size + pdec.size + q.size) + 8 * N + 8 * N
    d2h = 8 * N + 8 * N
    e2e_times = []
    for k in range(2 + a.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.set_fields(vel, lam, pdec, q, prob.robin_alpha)   # H2D fields
        s.set_operator(aH, aM)
        s.assemble_rhs(cf, rM, None, out=bh)                 # D2H b
        xh[:] = 0.0
        s.solve(bh, tol=TOL, itmax=20000, out=xh)            # H2D b,x; D2H x
        e2e_times.append(time.perf_counter() - t0)
    e2e = statistics.mean(e2e_times[2:])

    # ---- CPU baseline (oracle port on the host cores, bounded sample) ----
    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        smp = cpu_solve_sample(prob, dt, a.cpu_iters)
        proj = smp["t_asm"] + iters[-1] * smp["t_solve"] / max(1, smp["iters"])
        cpu = {"value": proj, "unit": "s", "cores": smp["threads"],
               "kind": "port",
               "sample": "full-system OpenMP assembly (%.2f s) + %d BiCGStab "
                         "iterations (%.3f s each, OpenMP colour-parallel "
                         "apply) projected to the GPU run's %d iterations"
                         % (smp["t_asm"], smp["iters"],
                            smp["t_solve"] / max(1, smp["iters"]), iters[-1])}

    if rank == 0:
        line = {
            "metric": METRIC, "value": ms / 1e3, "unit": "s", "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms,
            "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(a, prob),
            "iterations": iters[-1], "final_err": err,
            "true_rel_residual": rel_true, "status": st,
            "breakdown_ms": {"element_matrices_and_rhs": t_build,
                             "krylov": t_krylov,
                             "per_iteration": t_krylov / max(1, fp64_out[0]),
                             "step": step_s * 1e3},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic,
                         "traffic_kind": "ncu DRAM bytes of a 1,048,576-"
                                         "element capture scaled to this "
                                         "size by elements and nodes "
                                         "(profiles/stored_apply_df_"
                                         "rotation_shear.md)",
                         "kernel": "stored_apply_df (EBE apply, double-float "
                                   "element matrices, atomic scatter)",
                         "algorithmic_bytes_per_launch": alg_bytes,
                         "launch_ms": t_apply_ms, "peak_kind": peak_kind},
            "roofline_build": {"bound": "issue", "achieved": build_issue,
                               "peak": issue_peak,
                               "unit": "G warp instructions/s",
                               "frac": (build_issue / issue_peak
                                        if build_issue else None),
                               "kernel": "elem_build_geo_kernel (element "
                                         "matrices + diag + RHS from the "
                                         "mesh's geometric factors; rows in "
                                         "double-float on the FP32 pipe)",
                               "warp_instructions_per_element": inst_per_elem,
                               "peak_kind": "%d SMs x 4 warp instructions "
                                            "per clock at the median SM "
                                            "clock of the timed region" % n_sm,
                               "instructions_from": "profiles/" + BUILD_PROFILE},
            "build_modes": build_modes,
            "fp64_store": fp64_store,
            "apply_tuning": tuning,
            "scatter_variants": scatter_variants,
            "mixed_precision": mixed,
            "batched_rhs": batched,
            "batched_meshes": meshes,
            "learned_preconditioner": learned,
            "dropin_bicg": dropin,
            "time_loop": tloop,
            "text_output": text_out,
            "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "solve_stats": stats,
            "clocks": clk,
            "cpu_baseline": cpu,
        }
        line["summary"] = summary_keys(line, ms / 1e3, t_krylov_s)
        print(json.dumps(line), flush=True)
    s.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def summary_keys(line, step_s, solve_s):
    """The numbers of every section in a few short keys, placed last in the
    JSON line: seconds per step and per solve (device-resident, to FP64
    relative residual 1e-8) for each precision form, the speed-ups of the
    batched and learned forms, and the apply's HBM fraction."""
    def g(d, *ks):
        for k in ks:
            if not isinstance(d, dict):
                return None
            d = d.get(k)
        return d

    mp, f64 = line.get("mixed_precision") or {}, line.get("fp64_store") or {}
    lp = line.get("learned_preconditioner") or {}
    sv = line.get("scatter_variants") or {}
    out = {
        "fp64_step_s": _r(step_s), "fp64_solve_s": _r(solve_s),
        "fp64_iters": line.get("iterations"),
        "fp64store_step_s": _r(f64.get("step_s")),
        "fp64store_solve_s": _r(f64.get("solve_s")),
        "color_step_s": _r(g(sv, "color", "step_s")),
        "warp_step_s": _r(g(sv, "warp", "step_s")),
        "apply_ms": _r(g(sv, "atomic", "apply_ms")),
        "color_apply_ms": _r(g(sv, "color", "apply_ms")),
        "warp_apply_ms": _r(g(sv, "warp", "apply_ms")),
        "mixed_step_s": _r(mp.get("value")), "mixed_solve_s": _r(mp.get("solve_s")),
        "mixed_inner_iters": mp.get("inner_iterations"),
        "mixed_outer": mp.get("outer_corrections"),
        "mixed32_solve_s": _r(g(mp, "fp32_rounded_variant", "solve_s")),
        "mixed_true_res": _r(mp.get("true_rel_residual"), 3),
        "mixed_err_vs_fp64": _r(mp.get("rel_l2_vs_fp64_solution"), 3),
        "mixed_solve_speedup": _r(solve_s / mp["solve_s"]) if mp.get("solve_s") else None,
        "mixed_step_speedup": _r(step_s / mp["value"]) if mp.get("value") else None,
        "c5_jacobi_s": _r(g(lp, "jacobi_bicgstab", "solve_s_total")),
        "c5_learned_s": _r(g(lp, "learned_then_jacobi", "solve_s_total")),
        "c5_learned_vs_jacobi_time": _r(lp.get("learned_vs_plain_time")),
        "net_fwd_tc_ms": _r(g(lp, "network_forward", "tcgen05", "ms")),
        "net_fwd_mma_ms": _r(g(lp, "network_forward", "mma", "ms")),
        "c4a_block_s": _r(g(line, "batched_rhs", "block_solve_s")),
        "c4a_speedup": _r(g(line, "batched_rhs", "speedup_vs_sequential_fp64")),
        "c4a_apply_frac": _r(g(line, "batched_rhs", "block_apply", "frac"), 3),
        "c4a_tile_ms": _r(g(line, "batched_rhs", "block_apply", "form_ms", "tile"), 4),
        "c4a_tcgen05_ms": _r(g(line, "batched_rhs", "block_apply", "form_ms", "tcgen05"), 4),
        "c4b_s": _r(g(line, "batched_meshes", "segmented_solve_s")),
        "c4b_speedup": _r(g(line, "batched_meshes", "speedup_vs_one_at_a_time")),
        "apply_frac": _r(g(line, "roofline", "frac"), 3),
        "apply_per_sm": g(line, "apply_tuning", "apply_blocks_per_sm"),
        "half_per_sm": g(line, "apply_tuning", "half_blocks_per_sm"),
        "build_ms": _r(g(line, "breakdown_ms", "element_matrices_and_rhs")),
        "build_recompute_ms": _r(g(line, "build_modes", "recompute_ms")),
        "build_first_ms": _r(g(line, "build_modes", "first_build_with_factor_setup_ms")),
        "time_loop_later_s": _r(g(line, "time_loop", "later_step_s")),
        "time_loop_mixed_later_s": _r(g(line, "time_loop", "mixed", "later_step_s")),
    }
    return {k: v for k, v in out.items() if v is not None}


def run_case(a):
    """Small fixed workloads for profiler captures (not benchmarks): the
    stored double-float apply (--case apply), the K=64 block solve
    (--case block_apply), four K=64 block applies on the tcgen05 box form
    (--case block_apply_tc), a BiCG solve (--case bicg, fused A/A^T apply), a
    mixed-precision solve (--case mixed, FP32-vector inner apply) and
    learned-network training steps (--case unet_train), each on the
    --nex x --ney x --nez mesh."""
    import torch
    import __graft_entry__
    vdr = __graft_entry__.package()
    vdr.load_library()
    P = vdr.problems
    prob = P.rotation_shear(a.nex, a.ney, a.nez, seed=1002)
    dt = COURANT / max(a.nex, a.ney, a.nez)
    if a.case == "build":
        # element build + diag + RHS, as in the theta step (three builds)
        s = vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=2.0, aM=3.0 / dt)
        s.set_build_mode(a.build_mode)
        b = torch.zeros(prob.mesh.nnode, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        for _ in range(3):
            s.set_operator(2.0, 3.0 / dt)
            s.assemble_rhs_device(b, 3.0, 3.0 / dt, None)
    elif a.case == "apply":
        s = vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=2.0, aM=3.0 / dt)
        x = torch.randn(prob.mesh.nnode, dtype=torch.float64, device="cuda")
        y = torch.zeros_like(x)
        torch.cuda.synchronize()
        for _ in range(3):
            s.apply_accumulate_device(x, y)
    elif a.case == "block_apply":
        s = vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=2.0, aM=3.0 / dt)
        K = BATCH_K
        Q = torch.as_tensor(P.random_gaussian_sources(prob.mesh, K), device="cuda")
        B = torch.empty((prob.mesh.nnode, K), dtype=torch.float64, device="cuda")
        s.assemble_rhs_block_device(Q, B, 3.0)
        X = torch.zeros_like(B)
        s.solve_block_device(B, X, tol=TOL, inner_tol=1e-3, precision="tf32x3")
    elif a.case == "block_apply_tc":
        # four 64-column accumulating block applies on the tcgen05 form
        s = vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=2.0, aM=3.0 / dt)
        s.set_block_apply("tcgen05")
        X = torch.randn((prob.mesh.nnode, BATCH_K), dtype=torch.float32, device="cuda")
        Y = torch.zeros_like(X)
        torch.cuda.synchronize()
        for _ in range(4):
            s.apply_block_accumulate_device(X, Y, "tf32x3")
    elif a.case == "bicg":
        # BiCG: the fused A p / A^T p~ apply over the double-float store
        s = vdr.Solver(prob, vdr.Options(apply_mode="stored", solver="bicg"),
                       aH=2.0, aM=3.0 / dt)
        b = torch.empty(prob.mesh.nnode, dtype=torch.float64, device="cuda")
        s.assemble_rhs_device(b, 3.0, 0.0, None)
        x = torch.zeros_like(b)
        s.solve_device(b, x, tol=TOL, itmax=20000)
    elif a.case == "mixed":
        # FP64 refinement around FP32-vector inner BiCGStab (FP32 apply)
        s = vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=2.0, aM=3.0 / dt)
        b = torch.empty(prob.mesh.nnode, dtype=torch.float64, device="cuda")
        s.assemble_rhs_device(b, 3.0, 0.0, None)
        x = torch.zeros_like(b)
        for _ in range(2):  # the second solve is the one to read in a launch list
            x.zero_()
            s.solve_mixed_device(b, x, tol=TOL, inner_tol=a.inner_tol)
    elif a.case == "unet_forward":
        # three forward passes of the network per convolution path
        run = vdr.learned.TiltingRun(a.nex, a.ney, a.nez, seed=1005, courant=COURANT,
                                     tol=TOL, tilt_deg=LEARN_TILT)
        net = vdr.LearnedNet(run.s, seed=11)
        net.update_features(None)
        rh = torch.randn(prob.mesh.nnode, dtype=torch.float32, device="cuda")
        out = torch.empty_like(rh)
        torch.cuda.synchronize()
        for mode in ("tcgen05", "mma"):
            net.set_conv(mode)
            for _ in range(3):
                net.forward(rh, out)
        torch.cuda.synchronize()
    elif a.case == "unet_train":
        L = vdr.learned
        run = L.TiltingRun(a.nex, a.ney, a.nez, seed=1005, courant=COURANT,
                           tol=TOL, tilt_deg=LEARN_TILT)
        net = vdr.LearnedNet(run.s, seed=11)
        data = L.collect_pairs(run, net, range(0, 1), pairs_per_step=4)
        run.set_step(0)
        net.set_features(data["feats"][0], float(data["dbars"][0]))
        for i in range(3):
            net.train_step_residual(data["rhat"][i], 1e-4)
    torch.cuda.synchronize()
    print(json.dumps({"case": a.case, "elements": prob.mesh.nelem}))
    return 0


def main():
    a = args_parse()
    if a.case:
        return run_case(a)
    if a.impl == "reference":
        return run_reference(a)
    return run_native(a)


if __name__ == "__main__":
    sys.exit(main())
