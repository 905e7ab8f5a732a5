#!/usr/bin/env python
"""Design iterations/s of the SIMP compliance loop with its multigrid-CG state
solve at 256x128x128 elements (-l 4), mixed precision (FP32 V-cycle; FP64 CG
vectors with a double-single matvec and coarse factor) against the plain FP64
form, plus the fine-grid matvec's HBM roofline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one design iteration of the loop at stencil_optimization.c:148-189
(state solve, compliance, filter adjoint, OC update, filter) on the
cantilever of the reference. W untimed design iterations precede the K timed
ones. Rank 0 prints one JSON line. Under torchrun each rank runs an
independent replica (the path does not shard across GPUs).

Passes on the GPU (one rank):
  A  mixed form, fields resident in HBM, per-kernel CUDA-event profiling on
     -> value (design iters/s), the roofline of the fine-grid operator
  B  mixed form through the C ABI with host buffers: each step uploads x and
     xPhys from pinned host memory and reads xPhys and the compliance back
     -> e2e
  C  plain FP64 form, same iterations -> fp64 design iters/s and the
     compliance error of the mixed form against it
Then a bounded CPU sample of the same workload on the host cores (the oracle
restatement of the reference's CPU path).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "topopt-in-openmp-gpu_gb300")
sys.path.insert(0, PKG)

METRIC = "design iters/s @256x128x128, mixed vs FP64 (rel err<=1e-6); matvec HBM GB/s"
UNIT = "design_iters/s"


def args_parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=17)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--shape", default="256x128x128")
    ap.add_argument("--nl", type=int, default=4)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison pass")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the default level-0 launch shapes (short runs under a profiler)")
    ap.add_argument("--passes", default="APBCD",
                    help="GPU passes to run (A resident, P the same with per-kernel timing, B e2e, C FP64, "
                         "D batched multi-load)")
    ap.add_argument("--batched-shape", default="384x192x192")
    ap.add_argument("--batched-cases", type=int, default=8)
    ap.add_argument("--cpu-budget", type=float, default=150.0, help="seconds of CPU work for the reference arm")
    ap.add_argument("--cpu-sample", default=None, help=argparse.SUPPRESS)  # internal: child process mode
    return ap.parse_args()


# ---------------------------------------------------------------------------
def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_from_profiles(klass):
    """Per-launch DRAM bytes of a kernel class from a committed ncu summary
    (line: 'traffic_bytes_per_launch <class> <bytes>'), scaled by the summary's
    own 'units' line when it was captured on a smaller grid."""
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return None
    for f in sorted(os.listdir(d)):
        if not f.endswith((".txt", ".md")):
            continue
        for line in open(os.path.join(d, f)):
            parts = line.split()
            if len(parts) >= 3 and parts[0] == "traffic_bytes_per_launch" and parts[1] == klass:
                try:
                    return float(parts[2])
                except ValueError:
                    pass
    return None


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    Q = ("index,uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid):
        self.uuid = uuid
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = []
        for line in open(self.f.name):
            c = [x.strip() for x in line.split(",")]
            if len(c) < 10:
                continue
            if self.uuid and c[1] != self.uuid:
                continue
            rows.append(c)
        os.unlink(self.f.name)
        if not rows:
            return None
        sm = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        smax = [float(r[3]) for r in rows if r[3].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[6 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------
def cpu_sample(shape, nl, iters, threads):
    """Runs the oracle design loop in a fresh interpreter (its OpenMP pool is
    sized there) and returns per-iteration seconds and CG counts."""
    env = dict(os.environ)
    env["OMP_NUM_THREADS"] = str(threads)
    env["OMP_PROC_BIND"] = "close"
    cmd = [sys.executable, os.path.abspath(__file__), "--cpu-sample",
           "%dx%dx%d:%d:%d" % (shape[0], shape[1], shape[2], nl, iters)]
    r = subprocess.run(cmd, env=env, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("CPU sample failed: " + r.stderr[-400:])
    return json.loads(r.stdout.strip().splitlines()[-1])


def cpu_sample_child(spec):
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle
    dims, nl, iters = spec.split(":")
    nx, ny, nz = (int(v) for v in dims.split("x"))
    loops, h, _, _ = Oracle.run(nx, ny, nz, float(np.float32(0.2)), 1.5, int(nl), float(np.float32(1e-5)),
                                int(iters))
    print(json.dumps({"seconds": [float(s) for s in h["seconds"]], "cgiters": [int(c) for c in h["cgiters"]],
                      "c": [float(c) for c in h["c"]]}))


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ---------------------------------------------------------------------------
def dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def whole_job(times, K, world, device="cuda"):
    """Replicas: every rank runs the same K design iterations on its own GPU,
    with no data exchange. The job's time is the slowest rank's (max over
    ranks, one all-reduce) and its throughput counts every rank's
    iterations: world * K / max time."""
    if world > 1:
        import torch
        import torch.distributed as td
        t = torch.tensor(times, device=device, dtype=torch.float64)
        td.all_reduce(t, op=td.ReduceOp.MAX)
        times = [float(v) for v in t]
    return times, [world * K / v for v in times]


def run_reference(a):
    world, rank, _ = dist()
    if rank != 0:
        return
    shape = tuple(int(v) for v in a.shape.split("x"))
    cores = cpu_cores()
    # per-iteration cost grows with the CG count; the loop is run from its
    # start and the timed steps are the iterations after the warm-up ones,
    # as many as fit in the CPU budget (at least one)
    w = min(a.warmup, 1)
    budget_iters = max(1, min(a.steps, 2))
    s = cpu_sample(shape, a.nl, w + budget_iters, cores)
    secs = s["seconds"][w:]
    cg = s["cgiters"][w:]
    v = len(secs) / sum(secs)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus,
        "steps": len(secs), "warmup": w, "ms_per_step": 1000.0 * sum(secs) / len(secs),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "SIMP cantilever %s -l %d, FP64, host OpenMP" % (a.shape, a.nl),
                   "elements": shape[0] * shape[1] * shape[2], "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "design iterations %d..%d of the %s loop (CG iterations %s) on %d host threads; "
                                   "oracle restatement of the reference's CPU path (the reference tree is not "
                                   "on the GPU box)" % (w + 1, w + len(secs), a.shape, cg, cores)},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def fine_bytes(shape):
    nx, ny, nz = shape
    nn = (nx + 1) * (ny + 1) * (nz + 1)
    ne = nx * ny * nz
    return {
        # algorithmic bytes per launch: every vector read/written once, E once
        "fine_apply_f64": 48 * nn + 8 * ne,
        "fine_jacobi_f64": 96 * nn + 8 * ne,
        "fine_resid_f64": 72 * nn + 8 * ne,
        "fine_apply_f32": 24 * nn + 4 * ne,
        "fine_jacobi_f32": 48 * nn + 4 * ne,
        "fine_resid_f32": 36 * nn + 4 * ne,
    }, 1152.0 * ne


def design_pass(tp, torch, shape, nl, precision, W, K, profile=False, e2e=False, barrier=None):
    ctx = tp.TopOpt(shape[0], shape[1], shape[2], nl, precision=precision)
    if TUNE:
        ctx.autotune()  # level-0 launch shapes for this grid (set-up, untimed)
    ctx.init_design()
    hist = []
    for _ in range(W):
        hist.append(ctx.design_iteration())
    ne = ctx.nelem()
    host_x = host_xp = None
    if e2e:
        host_x = torch.empty(ne, dtype=torch.float64).pin_memory()
        host_xp = torch.empty(ne, dtype=torch.float64).pin_memory()
        ctx._check(ctx.L.tp_download(ctx.ctx, tp.FIELDS["x"], host_x.data_ptr(), ne))
        ctx._check(ctx.L.tp_download(ctx.ctx, tp.FIELDS["xphys"], host_xp.data_ptr(), ne))
    if profile:
        ctx.L.tp_profile_enable(ctx.ctx, 1)
        ctx.L.tp_profile_reset(ctx.ctx)
    if barrier:
        barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    t0 = time.perf_counter()
    timed = []
    for _ in range(K):
        if e2e:
            ctx._check(ctx.L.tp_upload(ctx.ctx, tp.FIELDS["x"], host_x.data_ptr(), ne))
            ctx._check(ctx.L.tp_upload(ctx.ctx, tp.FIELDS["xphys"], host_xp.data_ptr(), ne))
        info = ctx.design_iteration()
        if e2e:
            ctx._check(ctx.L.tp_download(ctx.ctx, tp.FIELDS["xphys"], host_xp.data_ptr(), ne))
            ctx._check(ctx.L.tp_download(ctx.ctx, tp.FIELDS["x"], host_x.data_ptr(), ne))
        timed.append(info)
    ev1.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if barrier:
        barrier()
    ms_events = ev0.elapsed_time(ev1)
    prof = {}
    if profile:
        import ctypes
        nm = ctypes.c_char_p()
        la = ctypes.c_long()
        ms = ctypes.c_double()
        ctx.L.tp_profile_get.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                                         ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_double)]
        for i in range(ctx.L.tp_profile_classes()):
            ctx.L.tp_profile_get(ctx.ctx, i, ctypes.byref(nm), ctypes.byref(la), ctypes.byref(ms))
            prof[nm.value.decode()] = (la.value, ms.value)
        ctx.L.tp_profile_enable(ctx.ctx, 0)
    ctx.close()
    return hist + timed, timed, ms_events, wall, prof


def batched_pass(tp, torch, shape, nl, nrhs, nload, W, K, hbm):
    """Several load cases sharing one operator: nrhs seeded multi-load cases
    (nload unit nodal forces each on the end face), mixed precision, summed
    compliance; every state solve is one multi-column PCG whose CG loop is a
    single CUDA graph launch."""
    import ctypes
    ctx = tp.TopOpt(shape[0], shape[1], shape[2], nl, precision=tp.TP_MIXED, nrhs=nrhs)
    if TUNE:
        ctx.autotune()
    F = tp.multiload(shape[0], shape[1], shape[2], nrhs, nload, seed=0)
    ctx.upload("F", F.ravel())
    del F
    ctx.init_design()
    for _ in range(W):
        ctx.design_iteration()
    ctx.L.tp_profile_enable(ctx.ctx, 1)
    ctx.L.tp_profile_reset(ctx.ctx)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    timed = [ctx.design_iteration() for _ in range(K)]
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    ctx.L.tp_profile_enable(ctx.ctx, 0)
    # per-kernel times: one more design iteration with the CG loop driven from
    # the host (kernels inside a graph launch are not timed one by one)
    ctx.set_graph_solve(2)
    ctx.L.tp_profile_enable(ctx.ctx, 1)
    ctx.L.tp_profile_reset(ctx.ctx)
    ctx.design_iteration()
    nm, la, pms = ctypes.c_char_p(), ctypes.c_long(), ctypes.c_double()
    ctx.L.tp_profile_get.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                                     ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_double)]
    prof = {}
    for i in range(ctx.L.tp_profile_classes()):
        ctx.L.tp_profile_get(ctx.ctx, i, ctypes.byref(nm), ctypes.byref(la), ctypes.byref(pms))
        prof[nm.value.decode()] = (la.value, pms.value)
    ctx.L.tp_profile_enable(ctx.ctx, 0)
    mem = ctx.L.tp_device_bytes(ctx.ctx)
    ctx.close()
    nn = (shape[0] + 1) * (shape[1] + 1) * (shape[2] + 1)
    ne = shape[0] * shape[1] * shape[2]
    out = {"workload": "%d load cases x %dx%dx%d -l %d, %d unit nodal loads per case on the end face (seed 0), "
                       "mixed precision, summed compliance, CG loop as one CUDA graph launch" %
                       ((nrhs,) + tuple(shape) + (nl, nload)),
           "value": K / (ms / 1000.0), "unit": UNIT, "ms_per_step": ms / K, "steps": K, "warmup": W,
           "dofs_per_case": 3 * nn, "device_bytes": mem,
           "cg_iters": [h.cgiters for h in timed], "compliance": [h.c for h in timed]}
    total = sum(v[1] for v in prof.values()) or 1.0
    out["kernels"] = {k: {"launches": v[0], "ms": round(v[1], 3), "share": round(v[1] / total, 4)}
                      for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1]) if v[0]}
    for k, b in (("fine_apply_f64", nrhs * 48 * nn + 8 * ne), ("fine_jacobi_f32", nrhs * 48 * nn + 4 * ne)):
        if k in prof and prof[k][0]:
            avg = prof[k][1] / prof[k][0] / 1000.0
            out["kernels"][k].update({"columns": nrhs, "algorithmic_bytes": b, "gbs": round(b / avg / 1e9, 1),
                                      "hbm_frac": round(b / avg / 1e9 / hbm, 4)})
    return out


TUNE = True


def main():
    global TUNE
    a = args_parse()
    TUNE = not a.no_tune
    if a.cpu_sample:
        cpu_sample_child(a.cpu_sample)
        return
    if a.impl == "reference":
        run_reference(a)
        return
    import numpy as np
    import torch
    import topopt_gb300 as tp

    world, rank, local = dist()
    torch.cuda.set_device(local)
    barrier = None
    if world > 1:
        import torch.distributed as td
        td.init_process_group("nccl")
        barrier = td.barrier
    tp.load()
    shape = tuple(int(v) for v in a.shape.split("x"))
    W, K = a.warmup, a.steps
    dev = torch.cuda.current_device()
    uuid = None
    try:
        uuid = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        uuid = None

    clocks = Clocks(uuid)
    clocks.start()
    # the headline: the loop with the per-kernel timing off
    all_a, timed_a, ms_a, wall_a, _ = design_pass(tp, torch, shape, a.nl, tp.TP_MIXED, W, K, barrier=barrier)
    clk = clocks.stop()
    # the same iterations again with CUDA events around every kernel class (a
    # few percent slower): the kernel breakdown and the roofline's launch times
    prof = {}
    if "P" in a.passes:
        _, _, _, _, prof = design_pass(tp, torch, shape, a.nl, tp.TP_MIXED, W, K, profile=True, barrier=barrier)
    wall_b = ms_a / 1000.0
    if "B" in a.passes:
        _, timed_b, ms_b, wall_b, _ = design_pass(tp, torch, shape, a.nl, tp.TP_MIXED, W, K, e2e=True,
                                                  barrier=barrier)
    fp64 = None
    if not a.no_fp64 and "C" in a.passes:
        all_c, timed_c, ms_c, wall_c, _ = design_pass(tp, torch, shape, a.nl, tp.TP_FP64, W, K, barrier=barrier)
        cm = np.array([h.c for h in all_a])
        cd = np.array([h.c for h in all_c])
        n = min(len(cm), len(cd))
        fp64 = {"value": K / (ms_c / 1000.0), "ms_per_step": ms_c / K,
                "compliance_rel_err_max": float(np.max(np.abs(cm[:n] - cd[:n]) / np.abs(cd[:n]))),
                "cg_iters_fp64": [h.cgiters for h in timed_c], "cg_iters_mixed": [h.cgiters for h in timed_a]}

    # whole-job numbers: max time over ranks, units summed over ranks
    (t_a, t_b), (value, e2e_value) = whole_job([ms_a / 1000.0, wall_b], K, world)

    nbytes, flops = fine_bytes(shape)
    hbm, peak_kind = peaks()
    total_ms = sum(v[1] for v in prof.values()) or 1.0
    kernels = {}
    for k, (la, ms) in sorted(prof.items(), key=lambda kv: -kv[1][1]):
        if la == 0:
            continue
        ent = {"launches": la, "ms": round(ms, 3), "share": round(ms / total_ms, 4)}
        if k in nbytes:
            avg = ms / la / 1000.0
            ent["gbs"] = round(nbytes[k] / avg / 1e9, 1)
            ent["hbm_frac"] = round(nbytes[k] / avg / 1e9 / hbm, 4)
            ent["tflops"] = round(flops / avg / 1e12, 3)
        kernels[k] = ent
    # The HBM roofline is reported for the level-0 FP32 Jacobi sweep: the
    # bandwidth-bound matvec kernel of the mixed V-cycle (the most launched
    # fine-grid kernel). The larger shares -- the coarse band Cholesky and the
    # CG matvec on FP64 vectors -- are compute kernels: in the mixed form both
    # run in double-single arithmetic (FP32 issue and dependent latency bound;
    # the factor's chain of 32-column steps), in the FP64 form on the FP64 pipe
    # (about 600 GFMA/s on this part). Their FP64-equivalent operation rates
    # are in "compute_bound".
    dom = "fine_jacobi_f32" if "fine_jacobi_f32" in kernels else None
    roofline = None
    if dom:
        la, ms = prof[dom]
        avg_s = ms / la / 1000.0
        ach = nbytes[dom] / avg_s / 1e9
        tr = traffic_from_profiles(dom)
        roofline = {"bound": "hbm", "kernel": dom, "achieved": round(ach, 1), "peak": hbm, "unit": "GB/s",
                    "frac": round(ach / hbm, 4), "traffic": tr, "algorithmic_bytes": nbytes[dom],
                    "avg_launch_us": round(avg_s * 1e6, 2), "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % peak_kind
                    if peak_kind == "measured" else "fallback 6.8 TB/s"}
    compute_bound = {}
    nn = (shape[0] + 1) * (shape[1] + 1) * (shape[2] + 1)
    if "fine_apply_f64" in prof and prof["fine_apply_f64"][0]:
        la, ms = prof["fine_apply_f64"]
        # operations of the element-centric matvec: about 171 per element
        # (butterflies, the 45-term product, accumulation) and the recomputed
        # halo rows and layers (x 1.25), each one double-single operation here
        compute_bound["fine_apply_f64"] = {"share": kernels["fine_apply_f64"]["share"], "arith": "double-single",
                                           "fp64_equiv_gops": round(171 * 1.25 * nn / (ms / la / 1000.0) / 1e9, 1)}
    if "coarse_factor" in prof and prof["coarse_factor"][0]:
        q = 2 ** (a.nl - 1)
        nzc, nyc = shape[2] // q + 1, shape[1] // q + 1
        ncoarse = 3 * (shape[0] // q + 1) * nyc * nzc
        bw = 3 * (nzc * nyc + nyc + 1) + 2
        la, ms = prof["coarse_factor"]  # two timed scopes per factorisation: band assembly, factor
        compute_bound["coarse_factor"] = {"share": kernels["coarse_factor"]["share"], "arith": "double-single",
                                          "gfma": round(ncoarse * bw * bw / 2 / 1e9, 2),
                                          "gfma_per_s": round(ncoarse * bw * bw / 2 / (2 * ms / la / 1000.0) / 1e9, 1)}
    launches = sum(v[0] for k, v in prof.items())

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms_a / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 V-cycle; f64 CG vectors, dots and coarse sweeps; double-single (2 x f32) CG matvec and "
                 "coarse factor", "data": "synthetic",
        "config": {"workload": "SIMP cantilever %s -l %d, volfrac 0.2, rmin 1.5, mixed (FP32 V-cycle; FP64 CG "
                               "vectors; double-single CG matvec and coarse factor)" % (a.shape, a.nl),
                   "elements": shape[0] * shape[1] * shape[2], "dofs": 3 * (shape[0] + 1) * (shape[1] + 1) * (shape[2] + 1),
                   "design_iterations": "%d..%d" % (W + 1, W + K), "parallelism": "replicas" if world > 1 else "single",
                   "l2": "inputs larger than L2 (129 MB): fine vectors are %d MB each" %
                         (24 * (shape[0] + 1) * (shape[1] + 1) * (shape[2] + 1) // 2 ** 20)},
        "fp64": fp64,
        "speedup_vs_fp64": (value / fp64["value"]) if fp64 else None,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 2 * 8 * shape[0] * shape[1] * shape[2],
                "d2h_bytes_per_step": 2 * 8 * shape[0] * shape[1] * shape[2] + 8 * 6},
        "roofline": roofline,
        "compute_bound": compute_bound,
        "kernels": kernels,
        "gpu_launches": launches,
        "clocks": clk,
        "cg_iters": [h.cgiters for h in timed_a],
    }
    if "D" in a.passes:
        bshape = tuple(int(v) for v in a.batched_shape.split("x"))
        line["batched"] = batched_pass(tp, torch, bshape, a.nl, a.batched_cases, 8, 1, 2, hbm)
    if rank == 0 and world == 1 and not a.no_cpu:
        cores = cpu_cores()
        s = cpu_sample(shape, a.nl, 1, cores)
        v = 1.0 / s["seconds"][0]
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": "design iteration 1 of the %s loop (%d CG iterations), oracle restatement "
                                          "of the reference's CPU path, %d host threads" %
                                          (a.shape, s["cgiters"][0], cores)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as td
        td.destroy_process_group()


if __name__ == "__main__":
    main()
