#!/usr/bin/env python
"""Design iterations/s of the SIMP compliance loop with its multigrid-CG state
solve at 256x128x128 elements (-l 4), mixed precision (FP32 V-cycle; FP64 CG
vectors with a double-single matvec and coarse factor) against the plain FP64
form, plus the fine-grid matvec's HBM roofline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one design iteration of the loop at stencil_optimization.c:148-189
(state solve, volume, compliance, filter adjoint, OC update, change, filter)
on the reference's cantilever. Each GPU pass creates its context, tunes the
level-0 launch shapes, runs W untimed design iterations, resets the design to
its start (x = xPhys = volfrac, U = 0) and times design iterations 1..K. Rank
0 prints one JSON line. Under torchrun each rank runs an independent replica
(the path does not shard across GPUs).

GPU passes (letters of --passes):
  A  mixed form, fields resident in HBM -> value (design iters/s)
  P  the same iterations with CUDA events around every kernel class
     -> kernel breakdown, the roofline of the fine-grid FP32 sweep
  C  plain FP64 form -> its rate, parity against the reference's own history
  M  the mixed form with an FP64 CG matvec and FP64 coarse factor
  B  mixed form through the reference's own C entry points (drop-in library,
     host arrays in the reference's padded layout, copies every call) -> e2e
  H  mixed form through the handle API with x and xPhys copied from and to
     pinned host memory every step -> e2e_handle
  D  8 load cases at 384x192x192 sharing one operator (batched)
Then, on rank 0, a bounded sample of the reference's own CPU code on the
host cores (cpu_baseline).

The reference arm (--impl reference) times the reference's own C
(oracle/_ref/libref64.so, built from the patched copies of its sources) on
all host cores, on the same configuration and steps; see run_reference().
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
VOLFRAC_F32 = 0.20000000298023224  # float(np.float32(0.2)): main() holds volfrac as float
CGTOL_F32 = 9.999999747378752e-06  # float(np.float32(1e-5))


def args_parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--shape", default="256x128x128")
    ap.add_argument("--nl", type=int, default=4)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the default level-0 launch shapes (short runs under a profiler)")
    ap.add_argument("--passes", default="APCMBHD", help="GPU passes to run (see the module docstring)")
    ap.add_argument("--host-loop", action="store_true",
                    help="drive every design iteration from the host (no graph launches): for profilers that "
                         "skip kernels inside conditional graphs")
    ap.add_argument("--batched-shape", default="384x192x192")
    ap.add_argument("--batched-cases", type=int, default=8)
    ap.add_argument("--batched-steps", type=int, default=4)
    ap.add_argument("--cpu-sample", default=None, help=argparse.SUPPRESS)  # internal: child process mode
    return ap.parse_args()


def config_of(a):
    """The workload, the same dict in both arms."""
    shape = tuple(int(v) for v in a.shape.split("x"))
    nn = (shape[0] + 1) * (shape[1] + 1) * (shape[2] + 1)
    return {"workload": "SIMP cantilever %s -l %d, volfrac 0.2, rmin 1.5, cgtol 1e-5, design iterations 1..%d"
                        % (a.shape, a.nl, a.steps),
            "elements": shape[0] * shape[1] * shape[2], "dofs": 3 * nn,
            "parallelism": "replicas" if a.gpus > 1 else "single",
            "l2": "inputs larger than L2 (129 MB): fine vectors are %d MB each" % (24 * nn // 2 ** 20)}


# ---------------------------------------------------------------------------
def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_from_profiles(klass):
    """Per-launch DRAM bytes of a kernel class from a committed ncu summary
    (line: 'traffic_bytes_per_launch <class> <bytes>')."""
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


def reference_history(shape, nl):
    """The reference's own 20-iteration history on this grid, recorded by
    tests/golden/make_golden.py from its C, or None."""
    p = os.path.join(ROOT, "tests", "golden", "history_%dx%dx%d_l%d.npz" % (shape + (nl,)))
    if not os.path.exists(p):
        return None
    import numpy as np
    h = np.load(p)
    return {"c": [float(v) for v in h["c"]], "cgiters": [int(v) for v in h["cgiters"]]}


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
# CPU side: the reference's own C (oracle/_ref/libref64.so), run in a child
# interpreter so that its OpenMP pool is sized there.
def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def ensure_reference_build():
    """oracle/_ref/libref64.so, compiled from the patched copies of the
    reference's sources if it is not there yet (the GPU machine builds it);
    returns its path or None."""
    so = os.path.join(ROOT, "oracle", "_ref", "libref64.so")
    if not os.path.exists(so):
        subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh")], stdout=subprocess.DEVNULL,
                       stderr=subprocess.DEVNULL)
    return so if os.path.exists(so) else None


def cpu_child(spec, threads):
    env = dict(os.environ)
    env["OMP_NUM_THREADS"] = str(threads)
    env["OMP_PROC_BIND"] = "close"
    env["OMP_TARGET_OFFLOAD"] = "DISABLED"
    r = subprocess.run([sys.executable, os.path.abspath(__file__), "--cpu-sample", spec], env=env,
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("CPU sample failed: " + r.stderr[-600:])
    return json.loads(r.stdout.strip().splitlines()[-1])


def cpu_sample_child(spec):
    """Child process. spec = json: {"kind": "ref"|"port", "shape", "nl",
    "warm_cg", "cg", "kernels"} -> one JSON line of seconds."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    s = json.loads(spec)
    shape, nl = tuple(s["shape"]), s["nl"]
    if s["kind"] == "ref":
        from oracle import ReferenceBench
        b = ReferenceBench(*shape, nl, VOLFRAC_F32, 1.5)
        t0 = time.perf_counter()
        fixed = b.fixed()
        design, c = b.design()
        warm = [b.cg() for _ in range(s["warm_cg"])]
        t1 = time.perf_counter()
        steps = []
        for _ in range(s["cg"]):
            ts = time.perf_counter()
            b.cg()
            steps.append(time.perf_counter() - ts)
        t2 = time.perf_counter()
        kern = b.kernels_ms() if s.get("kernels") else None
        b.close()
        print(json.dumps({"fixed": fixed, "design": design, "warm": warm, "cg": steps, "warm_wall": t1 - t0,
                          "timed_wall": t2 - t1, "kernels_ms": kern, "so": "oracle/_ref/libref64.so"}))
    else:
        from oracle import Oracle
        loops, h, _, _ = Oracle.run(*shape, VOLFRAC_F32, 1.5, nl, CGTOL_F32, 1)
        print(json.dumps({"seconds": [float(v) for v in h["seconds"]], "cgiters": [int(v) for v in h["cgiters"]],
                          "so": "oracle/liboracle.so"}))


def reference_estimate(sample, hist, K):
    """Design iterations/s of the reference's own C over iterations 1..K from
    a timing sample: iteration k costs fixed + (n_k - 1) * cg + design with
    n_k the CG iterations the reference itself takes there (its recorded
    history: index of the last iteration + 1)."""
    cg = statistics.mean(sample["cg"])
    n = [hist["cgiters"][min(k, len(hist["cgiters"]) - 1)] + 1 for k in range(K)]
    per = [sample["fixed"] + (nk - 1) * cg + sample["design"] for nk in n]
    return K / sum(per), per, n, cg


def run_reference(a):
    """The reference arm: the reference's own CPU code on all host cores.

    A design iteration of the reference at 256x128x128 takes minutes on the
    host cores, so each step is a bounded sample of it: the warm-up measures
    the iteration's fixed part (assembly, diagonals, coarse factor, initial
    residual and one CG iteration, through solveStateMG_halo with its loop cut
    to one iteration) and its design update once, and W-1 CG iterations; each
    timed step is one more CG iteration of the reference's loop (V-cycle and
    matvec on its own functions). The value is design iterations/s over
    iterations 1..K with the reference's own CG count for each (its recorded
    history on this grid): K / sum_k (fixed + (n_k - 1) * cg + design).
    ms_per_step is the measured sample per step."""
    world, rank, _ = (int(os.environ.get(k, d)) for k, d in (("WORLD_SIZE", "1"), ("RANK", "0"),
                                                             ("LOCAL_RANK", "0")))
    if rank != 0:
        return
    shape = tuple(int(v) for v in a.shape.split("x"))
    cores = cpu_cores()
    cfg = config_of(a)
    hist = reference_history(shape, a.nl)
    so = ensure_reference_build()
    line = {"impl": "reference", "metric": METRIC, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
            "warmup": a.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": cfg}
    if so and hist:
        s = cpu_child(json.dumps({"kind": "ref", "shape": shape, "nl": a.nl, "warm_cg": max(0, a.warmup - 1),
                                  "cg": a.steps, "kernels": False}), cores)
        v, per, n, cg = reference_estimate(s, hist, a.steps)
        sample = ("reference's own C (oracle/_ref/libref64.so, FP64 typedefs, CHOLMOD replaced by a band "
                  "Cholesky), %d host threads; warm-up: the iteration's fixed part %.2f s and design update %.2f s "
                  "once, %d CG iterations; each timed step one CG iteration (mean %.2f s); value = K / sum over "
                  "iterations 1..%d of fixed + (n_k - 1) cg + design, n_k the reference's own CG counts %s"
                  % (cores, s["fixed"], s["design"], max(0, a.warmup - 1), cg, a.steps, n))
        line.update({"value": v, "ms_per_step": 1000.0 * statistics.mean(s["cg"]),
                     "design_iteration_ms_estimated": 1000.0 * statistics.mean(per),
                     "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "reference",
                                      "sample": sample},
                     "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
    else:
        # no reference build or no recorded history for this grid: the oracle
        # restatement's full design iteration 1
        s = cpu_child(json.dumps({"kind": "port", "shape": shape, "nl": a.nl}), cores)
        v = 1.0 / s["seconds"][0]
        line.update({"value": v, "ms_per_step": 1000.0 * s["seconds"][0],
                     "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                      "sample": "design iteration 1 of the oracle restatement (%d CG iterations), "
                                                "%d host threads" % (s["cgiters"][0] + 1, cores)},
                     "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
    print(json.dumps(line), flush=True)


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


def get_profile(ctx):
    import ctypes
    nm, la, ms = ctypes.c_char_p(), ctypes.c_long(), ctypes.c_double()
    ctx.L.tp_profile_get.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                                     ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_double)]
    prof = {}
    for i in range(ctx.L.tp_profile_classes()):
        ctx.L.tp_profile_get(ctx.ctx, i, ctypes.byref(nm), ctypes.byref(la), ctypes.byref(ms))
        prof[nm.value.decode()] = (la.value, ms.value)
    return prof


def timed_iterations(tp, torch, ctx, K, barrier=None, e2e=False):
    """Design iterations 1..K of ctx from the start design, timed with CUDA
    events on the context's work (the context's stream is synchronised by
    every design iteration); e2e copies x and xPhys from and to pinned host
    memory around each step."""
    ctx.init_design()
    ne = ctx.nelem()
    host_x = host_xp = None
    if e2e:
        host_x = torch.empty(ne, dtype=torch.float64).pin_memory()
        host_xp = torch.empty(ne, dtype=torch.float64).pin_memory()
        ctx._check(ctx.L.tp_download(ctx.ctx, tp.FIELDS["x"], host_x.data_ptr(), ne))
        ctx._check(ctx.L.tp_download(ctx.ctx, tp.FIELDS["xphys"], host_xp.data_ptr(), ne))
    if barrier:
        barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    t0 = time.perf_counter()
    hist = []
    for _ in range(K):
        if e2e:
            ctx._check(ctx.L.tp_upload(ctx.ctx, tp.FIELDS["x"], host_x.data_ptr(), ne))
            ctx._check(ctx.L.tp_upload(ctx.ctx, tp.FIELDS["xphys"], host_xp.data_ptr(), ne))
        hist.append(ctx.design_iteration())
        if e2e:
            ctx._check(ctx.L.tp_download(ctx.ctx, tp.FIELDS["xphys"], host_xp.data_ptr(), ne))
            ctx._check(ctx.L.tp_download(ctx.ctx, tp.FIELDS["x"], host_x.data_ptr(), ne))
    ev1.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if barrier:
        barrier()
    return hist, ev0.elapsed_time(ev1), wall


def make_ctx(tp, shape, nl, precision, W, fine_arith=None, coarse_arith=None):
    """A context tuned and warmed up (W design iterations, then the design is
    reset by the timed run)."""
    ctx = tp.TopOpt(shape[0], shape[1], shape[2], nl, precision=precision)
    if HOST_LOOP:
        ctx.set_device_loop(0)
    if fine_arith is not None:
        ctx.set_fine_arith(fine_arith)
    if coarse_arith is not None:
        ctx.set_coarse_arith(coarse_arith)
    if TUNE:
        ctx.autotune()
    ctx.init_design()
    for _ in range(W):
        ctx.design_iteration()
    return ctx


def rel_err_max(a, b):
    n = min(len(a), len(b))
    return max(abs(a[i] - b[i]) / abs(b[i]) for i in range(n)) if n else None


def dropin_pass(tp, torch, shape, nl, W, K):
    """e2e through the reference's own entry points (libtopopt_ref64.so) with
    host arrays in its padded layout: the loop body of
    stencil_optimization.c:148-189, each call copying its host arrays to the
    device and back, mixed form (TOPOPT_PRECISION=mixed)."""
    os.environ["TOPOPT_PRECISION"] = "mixed"
    loop = tp.RefLoop(shape[0], shape[1], shape[2], nl, VOLFRAC_F32, 1.5, CGTOL_F32)
    for _ in range(W):
        loop.iteration()
    loop.reset()
    loop.transfer_bytes(reset=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = [loop.iteration() for _ in range(K)]
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    h2d, d2h = loop.transfer_bytes(reset=True)
    loop.close()
    return hist, wall, h2d // K, d2h // K


def batched_pass(tp, torch, shape, nl, nrhs, nload, W, K, hbm):
    """Several load cases sharing one operator: nrhs seeded multi-load cases
    (nload unit nodal forces each on the end face), mixed precision, summed
    compliance; every state solve is one multi-column PCG whose CG loop is a
    single CUDA graph launch. Parity at this size: after the timed
    iterations, load case 0 solved alone on the same design matches its
    column of the multi-column solve."""
    import numpy as np
    ctx = tp.TopOpt(shape[0], shape[1], shape[2], nl, precision=tp.TP_MIXED, nrhs=nrhs)
    if TUNE:
        ctx.autotune()
    F = tp.multiload(shape[0], shape[1], shape[2], nrhs, nload, seed=0)
    ctx.upload("F", F.ravel())
    ctx.init_design()
    for _ in range(W):
        ctx.design_iteration()
    ctx.init_design()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    timed = [ctx.design_iteration() for _ in range(K)]
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    # per-kernel times: one more design iteration with the CG loop driven from
    # the host (kernels inside a graph launch are not timed one by one)
    ctx.set_graph_solve(2)
    ctx.L.tp_profile_enable(ctx.ctx, 1)
    ctx.L.tp_profile_reset(ctx.ctx)
    ctx.design_iteration()
    prof = get_profile(ctx)
    ctx.L.tp_profile_enable(ctx.ctx, 0)
    ctx.set_graph_solve(0)
    mem = ctx.L.tp_device_bytes(ctx.ctx)
    # parity at full size: one more multi-column solve on the current design,
    # then case 0 alone from the same warm start; each column follows the
    # single-load recurrence, so the two agree to rounding
    n0 = F.shape[1]
    U0 = ctx.download("U")[:n0].copy()
    ctx.solve()
    it_cols, _ = ctx.solve_columns()
    U = ctx.download("U")[:n0].copy()
    xphys = ctx.download("xphys")
    ctx.close()
    one = tp.TopOpt(shape[0], shape[1], shape[2], nl, precision=tp.TP_MIXED)
    one.upload("F", F[0])
    one.upload("xphys", xphys)
    one.upload("U", U0)
    it1, _, _ = one.solve()
    U1 = one.download("U")
    one.close()
    col_err = float(np.max(np.abs(U - U1)) / np.max(np.abs(U1)))
    nn = (shape[0] + 1) * (shape[1] + 1) * (shape[2] + 1)
    ne = shape[0] * shape[1] * shape[2]
    out = {"workload": "%d load cases x %dx%dx%d -l %d, %d unit nodal loads per case on the end face (seed 0), "
                       "mixed, summed compliance, CG loop as one CUDA graph launch, iterations 1..%d" %
                       ((nrhs,) + tuple(shape) + (nl, nload, K)),
           "value": K / (ms / 1000.0), "unit": UNIT, "ms_per_step": round(ms / K, 1), "steps": K, "warmup": W,
           "dofs_per_case": 3 * nn, "device_bytes": mem, "cg_iters": [h.cgiters for h in timed],
           "case0_alone_vs_column_rel_err": col_err, "case0_cg_iters_alone_vs_column": [it1, int(it_cols[0])]}
    total = sum(v[1] for v in prof.values()) or 1.0
    kern = {k: [v[0], round(v[1], 2), round(v[1] / total, 3)]
            for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1]) if v[0]}
    for k, b in (("fine_apply_f64", nrhs * 48 * nn + 8 * ne), ("fine_jacobi_f32", nrhs * 48 * nn + 4 * ne)):
        if k in prof and prof[k][0]:
            avg = prof[k][1] / prof[k][0] / 1000.0
            kern[k].append(round(b / avg / 1e9 / hbm, 3))
    out["kernels_n_ms_share_hbmfrac"] = kern
    return out


TUNE = True
HOST_LOOP = False


def main():
    global TUNE, HOST_LOOP
    a = args_parse()
    TUNE = not a.no_tune
    HOST_LOOP = a.host_loop
    if a.cpu_sample:
        cpu_sample_child(a.cpu_sample)
        return
    if a.impl == "reference":
        run_reference(a)
        return
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
    try:
        uuid = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
    except Exception:
        uuid = None
    hbm, peak_kind = peaks()
    ref_hist = reference_history(shape, a.nl)

    # A: the headline, mixed form, per-kernel timing off
    ctx = make_ctx(tp, shape, a.nl, tp.TP_MIXED, W)
    clocks = Clocks(uuid)
    clocks.start()
    hist_a, ms_a, _ = timed_iterations(tp, torch, ctx, K, barrier=barrier)
    clk = clocks.stop()
    # P: the same iterations with CUDA events around every kernel class (a few
    # percent slower; iterations then run host-driven)
    prof = {}
    if "P" in a.passes:
        ctx.L.tp_profile_enable(ctx.ctx, 1)
        ctx.L.tp_profile_reset(ctx.ctx)
        timed_iterations(tp, torch, ctx, K, barrier=barrier)
        prof = get_profile(ctx)
        ctx.L.tp_profile_enable(ctx.ctx, 0)
    ctx.close()

    fp64 = parity = ns = None
    hist_c = []
    if "C" in a.passes:
        ctx = make_ctx(tp, shape, a.nl, tp.TP_FP64, W)
        hist_c, ms_c, _ = timed_iterations(tp, torch, ctx, K, barrier=barrier)
        ctx.close()
        (t_c,), (v_c,) = whole_job([ms_c / 1000.0], K, world)
        cm, cd = [h.c for h in hist_a], [h.c for h in hist_c]
        gm, gd = [h.cgiters for h in hist_a], [h.cgiters for h in hist_c]
        fp64 = {"value": v_c, "ms_per_step": round(ms_c / K, 2), "cg_iters": gd,
                "mixed_c_rel_err_max": rel_err_max(cm, cd),
                "mixed_cg_iters_equal": "%d/%d" % (sum(1 for x, y in zip(gm, gd) if x == y), len(gd))}
        if ref_hist:
            n = min(len(hist_c), len(ref_hist["c"]))
            parity = {"vs": "the reference's own C, FP64, this grid, iterations 1..%d (tests/golden)" % n,
                      "fp64_c_rel_err_iter1": abs(cd[0] - ref_hist["c"][0]) / abs(ref_hist["c"][0]),
                      "fp64_c_rel_err_max": rel_err_max(cd[:n], ref_hist["c"][:n]),
                      "fp64_cg_iters_equal": gd[:n] == ref_hist["cgiters"][:n],
                      "mixed_c_rel_err_max": rel_err_max(cm[:n], ref_hist["c"][:n])}
    if "M" in a.passes:
        ctx = make_ctx(tp, shape, a.nl, tp.TP_MIXED, W, fine_arith=0, coarse_arith=0)
        hist_m, ms_m, _ = timed_iterations(tp, torch, ctx, K, barrier=barrier)
        ctx.close()
        (t_m,), (v_m,) = whole_job([ms_m / 1000.0], K, world)
        ns = {"form": "FP32 V-cycle; FP64 CG (matvec, dots, updates) and FP64 coarse factor", "value": v_m,
              "ms_per_step": round(ms_m / K, 2)}
        if hist_c:
            ns["speedup_vs_fp64"] = v_m / fp64["value"]
            ns["c_rel_err_max_vs_fp64"] = rel_err_max([h.c for h in hist_m], [h.c for h in hist_c])
    e2e = e2e_handle = None
    if "B" in a.passes:
        hist_b, wall_b, h2d, d2h = dropin_pass(tp, torch, shape, a.nl, min(W, 1), K)
        (t_b,), (v_b,) = whole_job([wall_b], K, world)
        e2e = {"value": v_b, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "route": "the reference's entry points (libtopopt_ref64.so: solveStateMG_halo, compute_volume, "
                        "getComplianceAndSensetivity_halo, applyDensityFilterGradient, update_solution, "
                        "compute_change, applyDensityFilter) on host arrays in its padded layout, mixed form",
               "c_rel_err_max_vs_value_pass": rel_err_max([h["c"] for h in hist_b], [h.c for h in hist_a])}
    if "H" in a.passes:
        ctx = make_ctx(tp, shape, a.nl, tp.TP_MIXED, W)
        _, _, wall_h = timed_iterations(tp, torch, ctx, K, barrier=barrier, e2e=True)
        ctx.close()
        (t_h,), (v_h,) = whole_job([wall_h], K, world)
        ne = shape[0] * shape[1] * shape[2]
        e2e_handle = {"value": v_h, "unit": UNIT, "h2d_bytes_per_step": 16 * ne, "d2h_bytes_per_step": 16 * ne,
                      "route": "handle API, x and xPhys from and to pinned host memory each step"}
    if e2e is None:
        e2e = e2e_handle

    (t_a,), (value,) = whole_job([ms_a / 1000.0], K, world)
    nbytes, flops = fine_bytes(shape)
    total_ms = sum(v[1] for v in prof.values()) or 1.0
    kernels = {}
    for k, (la, ms) in sorted(prof.items(), key=lambda kv: -kv[1][1]):
        if la == 0:
            continue
        ent = [la, round(ms, 1), round(ms / total_ms, 3)]
        if k in nbytes:
            ent.append(round(nbytes[k] / (ms / la / 1000.0) / 1e9 / hbm, 3))
        kernels[k] = ent
    # The HBM roofline is reported for the level-0 FP32 Jacobi sweep: the
    # bandwidth-bound matvec of the mixed V-cycle (the most launched fine-grid
    # kernel). The larger shares -- the coarse band Cholesky and the CG matvec
    # on FP64 vectors -- are compute kernels (double-single arithmetic in the
    # mixed form, FP32 issue and dependent latency bound).
    dom = "fine_jacobi_f32" if "fine_jacobi_f32" in prof and prof["fine_jacobi_f32"][0] else None
    roofline = None
    if dom:
        la, ms = prof[dom]
        avg_s = ms / la / 1000.0
        ach = nbytes[dom] / avg_s / 1e9
        roofline = {"bound": "hbm", "kernel": dom, "achieved": round(ach, 1), "peak": hbm, "unit": "GB/s",
                    "frac": round(ach / hbm, 4), "traffic": traffic_from_profiles(dom),
                    "algorithmic_bytes": nbytes[dom], "avg_launch_us": round(avg_s * 1e6, 2),
                    "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                    else "fallback 6.8 TB/s"}
    launches = sum(v[0] for v in prof.values())

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms_a / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 V-cycle; f64 CG vectors, dots and coarse sweeps; double-single (2 x f32) CG matvec and "
                 "coarse factor", "data": "synthetic",
        "config": config_of(a),
        "gpu_launches": launches,
        "clocks": clk,
        "roofline": roofline,
        "e2e": e2e,
        "e2e_handle": e2e_handle,
        "cg_iters": [h.cgiters for h in hist_a],
        "kernels_n_ms_share_hbmfrac": kernels,
    }
    if "D" in a.passes:
        bshape = tuple(int(v) for v in a.batched_shape.split("x"))
        line["batched"] = batched_pass(tp, torch, bshape, a.nl, a.batched_cases, 8, 1, a.batched_steps, hbm)
    if rank == 0 and world == 1 and not a.no_cpu:
        so = ensure_reference_build()
        cores = cpu_cores()
        if so and ref_hist:
            s = cpu_child(json.dumps({"kind": "ref", "shape": shape, "nl": a.nl, "warm_cg": 0, "cg": 2,
                                      "kernels": True}), cores)
            v, per, n, cg = reference_estimate(s, ref_hist, K)
            line["cpu_baseline"] = {
                "value": v, "unit": UNIT, "cores": cores, "kind": "reference",
                "sample": "reference's own C (oracle/_ref/libref64.so) on %d host threads: design iteration 1's "
                          "fixed part %.2f s and design update %.2f s, 2 CG iterations (mean %.2f s); value over "
                          "iterations 1..%d with the reference's own CG counts" % (cores, s["fixed"], s["design"],
                                                                                  cg, K),
                "kernels_ms": {k: round(t, 1) for k, t in s["kernels_ms"].items()},
                "gpu_ms_per_launch": {k: round(prof[k][1] / prof[k][0], 3) for k in
                                      ("fine_apply_f64", "fine_jacobi_f32", "stencil", "transfer", "design")
                                      if k in prof and prof[k][0]}}
        else:
            s = cpu_child(json.dumps({"kind": "port", "shape": shape, "nl": a.nl}), cores)
            v = 1.0 / s["seconds"][0]
            line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                    "sample": "design iteration 1 of the oracle restatement, %d host threads" % cores}
    # the headline claim last, where a truncated record keeps it
    line["mixed_fp64_cg"] = ns
    line["fp64"] = fp64
    line["speedup_vs_fp64"] = (value / fp64["value"]) if fp64 else None
    line["parity"] = parity
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as td
        td.destroy_process_group()


if __name__ == "__main__":
    main()
