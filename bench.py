"""Benchmark of the girih star-stencil hot path on GB300.

Workload (default): the 7-point constant-coefficient leapfrog stencil (operator
8: u = 2v - u + roc2*(c0 v + c1 sum6 v)), nx=ny=nz=512, nt=500, seeded U(0,1)
fields, roc2 U(0.5,1.5), c = (-0.75, 0.125), the inputs drawn in FP64 (the FP32
forms round them when they are stored).  One benchmark "step" is one call of the
hot path: the whole nt=500 time loop over the 512^3 grid.

Forms measured on the same grid, each from device-resident inputs:
  plain64    FP64, one sweep per kernel launch (the drop-in form)
  fused64    FP64, time-fused passes, FP64 arithmetic (bound by GB300's FP64 pipe)
  fused64df  FP64 fields, time-fused passes, double-float arithmetic (FP32 pairs);
             the FP64-accurate time-fused form and the headline `value`
  plainmixed FP32 fields, one sweep per launch (x quads)
  mixed      FP32 fields, compensated leapfrog, time-fused passes
Every form's max-norm and L2 error is measured against the FP64 CPU oracle run
on the same FP64 inputs; the FP32 forms' arithmetic error alone (inputs rounded
to FP32 first) is measured against the FP64 plain GPU run from those inputs.
`e2e` is the headline form through the C ABI from pinned FP64 HOST arrays
(upload + run + download of U1 inside the timed region).  A `secondary` block
covers the other configurations (25-point leapfrog at 480^3, the
variable-coefficient operators at 384^3, the 64-grid batch) with their errors
against the CPU oracle.

The CPU baseline (`cpu_baseline`, and `--impl reference`) is the reference's
own OpenMP build (oracle/_ref/mwd_kernel, compiled from the reference sources
by `make -C oracle ref`) with its MWD time stepper on the host cores; the
reference has no 7-point leapfrog, so the default workload's baseline is the
reference's 7-point constant-coefficient operator (kernel 1: two arrays per
update instead of three, which favours the reference).  Where that binary is
absent the oracle restatement stands in (kind "port").
Multi-GPU (torchrun): every rank advances its own replica of the grid
("replicas only": the path has no exchange on one grid per GPU).
"""
import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GLUP/s at 512^3: time-fused & mixed vs plain FP64 on GB300; % HBM roofline; err"

WORKLOADS = {
    # name: op, n, nt, seed, field range, roc2 range, constant coefficients, reference kernel of the CPU baseline
    "star7_leapfrog_512": dict(op=8, n=512, nt=500, seed=1, f=(0.0, 1.0), roc2=(0.5, 1.5), coefs=[-0.75, 0.125],
                               ref_kernel=1),
    # Jacobi smoother c0 + 6 c1 = 1: the reference's default pair (-0.28472, 0.16) amplifies the
    # checkerboard mode by |c0 - 6 c1| = 1.24 per step (1e46 after 500 steps, past the FP32 range)
    "star7_jacobi_512": dict(op=1, n=512, nt=500, seed=1, f=(0.0, 1.0), roc2=(0.0, 0.0), coefs=[0.25, 0.125],
                             ref_kernel=1),
    "star25_leapfrog_480": dict(op=0, n=480, nt=200, seed=2, f=(-1.0, 1.0), roc2=(0.05, 0.15),
                                coefs=[-8.541667, 1.6, -0.2, 0.025396826, -0.0017857143], error_nts=[50, 100],
                                ref_kernel=0),
    # variable coefficients, coefficient arrays U(0.01, 0.1/radius)
    "var7_384": dict(op=5, n=384, nt=200, seed=3, f=(0.0, 1.0), roc2=(0.0, 0.0), c=(0.01, 0.1), coefs=None,
                     ref_kernel=5),
    "var25_384": dict(op=4, n=384, nt=200, seed=3, f=(0.0, 1.0), roc2=(0.0, 0.0), c=(0.01, 0.025), coefs=None,
                      ref_kernel=4),
}

# The reference's time stepper and its parameters per kernel for the CPU
# baseline (src/kernels/diamond_ts.c:871-976, options parsed at
# src/utils.c:1219-1356): MWD with one thread per diamond (thread groups of one,
# the fastest setting that passes the reference's own --verify 1 in a sweep on
# the GPU machine's 16 host cores; the thread layout inside a group is given
# explicitly, as the defaults of --thx/--thy give wrong results with larger
# groups), and the sample's time steps (MWD raises nt to 2 + a multiple of
# 2 (t_dim + 1), src/kernels/diamond_utils.c:1042-1056).  Relaxed
# synchronisation (--mwd-type 2) is refused for radius 4 (diamond_utils.c:859).
_ONE = ["--thread-group-size", "1", "--thz", "1", "--thy", "1", "--thx", "1", "--num-wavefronts", "1"]
REFERENCE_STEPPER = {
    1: dict(args=["--target-ts", "2", "--mwd-type", "2", "--t-dim", "7"] + _ONE, nt=66),
    0: dict(args=["--target-ts", "2", "--mwd-type", "1", "--t-dim", "1"] + _ONE, nt=18),
    5: dict(args=["--target-ts", "2", "--mwd-type", "2", "--t-dim", "7"] + _ONE, nt=34),
    4: dict(args=["--target-ts", "2", "--mwd-type", "0", "--t-dim", "1"] + _ONE, nt=18),
}
REFERENCE_BINARY = os.path.join(ROOT, "oracle", "_ref", "mwd_kernel")


def rank_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(x, device=None):
    """Max of a float over all ranks (the slowest rank sets the job time); the
    identity without torch.distributed."""
    import torch
    import torch.distributed as tdist
    if not (tdist.is_available() and tdist.is_initialized()) or tdist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic(kernel_key):
    """DRAM bytes per launch of a kernel from the committed ncu summary, or None."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            return json.load(f).get(kernel_key)
    except Exception:
        return None


def pass_bytes(op_info, tsz, schedule, precision):
    """Compulsory HBM bytes per grid point of one kernel launch.
    plain: read v (+u, roc2), write u.  fused: read cur (+prev, roc2), write two states."""
    r, to, nc, var = op_info
    cb = nc * (2 if precision == "mixed" else tsz) if var else 0  # coefficient arrays, read once per launch
    if schedule == "plain":
        return 2 * tsz + (2 * tsz if to == 2 else 0) + cb
    return ((3 * tsz + 2 * tsz) if to == 2 else (tsz + tsz)) + cb


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


# ---------------------------------------------------------------- CPU side

def oracle_reference_run(wl, marks, f32_exact=False):
    """The FP64 CPU oracle on the workload's seeded inputs, advanced to each
    checkpoint in `marks` (cumulative steps); yields (mark, grid)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    n, op = wl["n"], wl["op"]
    threads = host_threads()
    g = oracle.Grid(op, n, n, n)
    g.fill_seeded(wl["seed"], wl["f"], wl["roc2"], wl.get("c", (0.0, 0.0)), coefs=wl["coefs"],
                  f32_exact=f32_exact, nthreads=threads)
    done = 0
    for m in marks:
        g.run(m - done, nthreads=threads)
        done = m
        yield m, g


def reference_binary_ok():
    """The reference's own build is present and runs on this machine."""
    if not (os.path.isfile(REFERENCE_BINARY) and os.access(REFERENCE_BINARY, os.X_OK)):
        return False
    try:
        r = subprocess.run([REFERENCE_BINARY, "--list"], capture_output=True, text=True, timeout=60)
        return r.returncode == 0 and "Diamond" in r.stdout
    except Exception:
        return False


def fit_thread_groups(args, threads):
    """The reference requires the thread count to be a multiple of the MWD
    thread-group size (src/kernels/diamond_utils.c): on a host with fewer or
    differently divisible cores, shrink the group (and its z threads) to the
    largest divisor of the thread count."""
    a = list(args)
    if "--thread-group-size" not in a:
        return a
    i = a.index("--thread-group-size") + 1
    tgs = int(a[i])
    if threads % tgs == 0:
        return a
    fit = max(d for d in range(1, min(tgs, threads) + 1) if threads % d == 0)
    a[i] = str(fit)
    if "--thz" in a:
        j = a.index("--thz") + 1
        a[j] = str(min(int(a[j]), fit))
    return a


def run_reference_binary(kernel, n, tests, nt=None, threads=None, stepper=None):
    """Run the reference's mwd_kernel (performance mode, --n-tests tests) and
    return (per-test seconds, effective nt, threads, command)."""
    cfg = REFERENCE_STEPPER[kernel]
    threads = threads or host_threads()
    args = fit_thread_groups(list(stepper if stepper is not None else cfg["args"]), threads)
    nt = nt or cfg["nt"]
    cmd = [REFERENCE_BINARY, "--nx", str(n), "--ny", str(n), "--nz", str(n), "--nt", str(nt),
           "--target-kernel", str(kernel), "--n-tests", str(tests), "--verbose", "1"] + args
    env = dict(os.environ, OMP_NUM_THREADS=str(threads), OMP_PROC_BIND="true", OMP_PLACES="cores")
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=1200, cwd="/tmp")
    if r.returncode != 0:
        raise RuntimeError(f"reference run failed ({r.returncode}): {r.stdout[-500:]} {r.stderr[-500:]}")
    nt_eff = nt
    m = re.search(r"Number of time steps:\s*(\d+)", r.stdout)
    if m:
        nt_eff = int(m.group(1))
    # tests are printed in order (src/performance.c:88-97)
    times = [float(x) for x in re.findall(r"Rank 0 TEST#\d+ time:\s*([0-9.eE+-]+)", r.stdout)]
    if len(times) != tests:
        raise RuntimeError(f"reference run printed {len(times)} test times, expected {tests}")
    return times, nt_eff, threads, " ".join(os.path.basename(c) if i == 0 else c for i, c in enumerate(cmd))


def stepper_name(args):
    a = dict(zip(args[::2], args[1::2]))
    if a.get("--target-ts") == "2":
        return (f"MWD (--mwd-type {a.get('--mwd-type')}, t_dim {a.get('--t-dim')}, thread groups of "
                f"{a.get('--thread-group-size')}, {a.get('--num-wavefronts')} wavefronts)")
    return "spatial blocking"


def cpu_baseline(wl, seconds, tests=3):
    """The reference's own OpenMP build on the host cores (kind "reference"),
    else the oracle restatement (kind "port"), on a bounded sample of the
    workload: the full grid, a few time steps per test."""
    n = wl["n"]
    kernel = wl.get("ref_kernel", wl["op"])
    if reference_binary_ok() and kernel in REFERENCE_STEPPER:
        try:
            times, nt_eff, threads, cmd = run_reference_binary(kernel, n, tests)
        except Exception as e:
            cb = cpu_baseline_port(wl, seconds)
            cb["reference_failed"] = str(e)[:200]
            return cb
        rates = [float(n) ** 3 * nt_eff / t / 1e9 for t in times]
        note = "" if kernel == wl["op"] else (
            f"; the reference has no operator {wl['op']}: its kernel {kernel} (the same stencil shape, fewer "
            f"arrays per update) stands in")
        return {"value": statistics.median(rates), "unit": "GLUP/s", "cores": threads, "kind": "reference",
                "sample": f"{n}^3 grid, kernel {kernel}, {tests} tests of {nt_eff} time steps "
                          f"({sum(times):.1f} s), {stepper_name(REFERENCE_STEPPER[kernel]['args'])}{note}",
                "command": cmd}
    return cpu_baseline_port(wl, seconds)


def cpu_baseline_port(wl, seconds, steps=None):
    """The oracle restatement (OpenMP over all host threads) on a bounded sample
    of the workload: the full grid, a few sweeps."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    n, op = wl["n"], wl["op"]
    threads = host_threads()
    g = oracle.Grid(op, n, n, n)
    g.fill_seeded(wl["seed"], wl["f"], wl["roc2"], wl.get("c", (0.0, 0.0)), coefs=wl["coefs"], nthreads=threads)
    t0 = time.perf_counter()
    g.run(2, nthreads=threads)
    per_pair = time.perf_counter() - t0
    pairs = steps if steps else max(1, int(seconds / max(per_pair, 1e-3)))
    t0 = time.perf_counter()
    g.run(2 * pairs, nthreads=threads)
    dt = time.perf_counter() - t0
    glups = float(n) ** 3 * 2 * pairs / dt / 1e9
    return {"value": glups, "unit": "GLUP/s", "cores": threads, "kind": "port",
            "sample": f"{n}^3 grid, {2 * pairs} sweeps of operator {op} ({dt:.1f} s)"}


# ---------------------------------------------------------------- GPU side

def forms_of(op):
    from girih_gb300 import gpu
    if gpu.OP_INFO[op][3]:  # variable coefficients: the mixed form streams them in the x-quad plain sweep
        return {
            "plain64": dict(precision="fp64", schedule="plain"),
            "mixed": dict(precision="mixed", schedule="plain"),
            "fused32": dict(precision="fp32", schedule="fused"),
            "mixedfused": dict(precision="mixed", schedule="fused"),
        }
    return {
        "plain64": dict(precision="fp64", schedule="plain"),
        "fused64": dict(precision="fp64", schedule="fused"),
        "fused64df": dict(precision="fp64df", schedule="fused"),
        "plainmixed": dict(precision="mixed", schedule="plain"),  # one step per pass, x quads
        "mixed": dict(precision="mixed", schedule="fused"),
    }


def seed_ctx(ctx, wl, f32_exact=False):
    ctx.fill_seeded(wl["seed"], wl["f"], wl["roc2"], wl.get("c", (0.0, 0.0)), coefs=wl["coefs"], f32_exact=f32_exact)


def time_forms(wl, forms, steps, warmup, local, world=1, depth=0, block="", headline=None, sync=None):
    """Autotune and time each form; returns ({name: result}, {name: context})."""
    from girih_gb300 import gpu
    n, nt, op = wl["n"], wl["nt"], wl["op"]
    lups = float(n) ** 3 * (2 * ((nt + 1) // 2))
    results, ctxs = {}, {}
    for name, kw in forms.items():
        blk = tuple(int(x) for x in block.split(",")) if block and kw["schedule"] == "fused" else (0, 0)
        ctx = gpu.Context(op, n, n, n, device=local, fusion_depth=depth if kw["schedule"] == "fused" else 0,
                          block=blk, **kw)
        seed_ctx(ctx, wl)
        if kw["schedule"] != "plain" and not depth and not block:
            ctx.autotune()  # picks tile and fusion depth on this grid; the grid state is restored
        k = steps if (headline is None or name == headline) else min(steps, 5)
        for _ in range(warmup):
            ctx.run(nt)
        if sync:
            sync()
        ms = []
        t0 = time.perf_counter()
        for _ in range(k):
            ms.append(ctx.run(nt))
        if sync:
            sync()
        wall = time.perf_counter() - t0
        dev_s = max_over_ranks(sum(ms) / 1e3, "cuda")
        info = ctx.info()
        results[name] = dict(glups=world * k * lups / dev_s / 1e9, ms_per_step=1e3 * dev_s / k, steps=k,
                             wall_s=wall, launches_per_step=info["launches_last_run"],
                             depth=info["fusion_depth"], tile=[info["block_x"], info["block_y"]],
                             kernel=info["kernel_name"], tsz=8 if kw["precision"] in ("fp64", "fp64df") else 4,
                             schedule=info_schedule(info), precision=kw["precision"],
                             bytes_per_lup=info["bytes_per_lup"])
        ctxs[name] = ctx
    return results, ctxs


def info_schedule(info):
    return {0: "plain", 1: "fused", 2: "auto"}.get(info["schedule"], "plain")


def form_errors(wl, forms, local, depth=0):
    """Each form's max-norm / L2 error against the FP64 CPU oracle on the same
    FP64 inputs, at every checkpoint of the workload; plus the FP32 forms'
    arithmetic error alone against the FP64 plain GPU run when both start from
    FP32-representable inputs."""
    from girih_gb300 import gpu
    n, nt, op = wl["n"], wl["nt"], wl["op"]
    marks = [m for m in wl.get("error_nts", []) if 0 < m < nt] + [nt]
    errors = {name: {"nt": nt, "against": "FP64 CPU oracle, same FP64 inputs"} for name in forms}
    ctxs = {}
    for name, kw in forms.items():
        c = gpu.Context(op, n, n, n, device=local, fusion_depth=depth if kw["schedule"] == "fused" else 0, **kw)
        seed_ctx(c, wl)  # creation picked up the autotuned choice cached for this operator and size
        ctxs[name] = c
    done = 0
    for m, g in oracle_reference_run(wl, marks):
        for name, c in ctxs.items():
            c.run(m - done)
            mr, l2 = gpu.rel_errors(c.error_norms(g.U1))
            errors[name]["max_rel"], errors[name]["l2_rel"] = mr, l2
            if len(marks) > 1:
                errors[name].setdefault("by_nt", {})[str(m)] = {"max_rel": mr, "l2_rel": l2}
        done = m
    for c in ctxs.values():
        c.close()
    # arithmetic only: FP32-representable inputs, against the FP64 plain GPU run (parity-checked)
    f32 = [k for k, kw in forms.items() if kw["precision"] in ("mixed", "fp32")]
    if f32:
        ref = gpu.Context(op, n, n, n, device=local, precision="fp64", schedule="plain")
        seed_ctx(ref, wl, f32_exact=True)
        ref.run(nt)
        for name in f32:
            kw = forms[name]
            with gpu.Context(op, n, n, n, device=local, fusion_depth=depth if kw["schedule"] == "fused" else 0,
                             **kw) as c:
                seed_ctx(c, wl, f32_exact=True)
                c.run(nt)
                mr, l2 = gpu.rel_errors(c.compare(ref))
            errors[name]["arithmetic_only"] = {"max_rel": mr, "l2_rel": l2,
                                               "against": "FP64 plain GPU run, FP32-representable inputs"}
        ref.close()
    return errors


def roofline_of(h, op_info, n, peak, peak_kind, workload, form):
    """Roofline of a form's dominant kernel: algorithmic bytes per launch (the
    one-pass bytes per lattice point x the n^3 points one launch updates) over
    the average launch time from CUDA events."""
    per_pt = pass_bytes(op_info, h["tsz"], h["schedule"], h["precision"])
    launch_ms = h["ms_per_step"] / max(1, h["launches_per_step"])
    achieved = per_pt * float(n) ** 3 / (launch_ms / 1e3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": committed_traffic(f"{h['kernel']}:{workload}:{form}"), "peak_source": peak_kind,
            "kernel": h["kernel"], "algorithmic_bytes_per_point_per_launch": per_pt,
            "points_per_launch": float(n) ** 3, "launch_ms": launch_ms,
            "effective_bandwidth_gbs": h["glups"] * (per_pt if h["schedule"] == "plain" else
                                                     pass_bytes(op_info, h["tsz"], "plain", h["precision"]))}


def run_e2e(wl, form_kw, steps, warmup, local, world, sync, depth=0):
    """The form end to end through the C ABI from pinned FP64 host arrays:
    upload (+ conversion), the nt-step loop, download of U1, every step."""
    import numpy as np
    import torch
    from girih_gb300 import gpu
    n, nt, op = wl["n"], wl["nt"], wl["op"]
    op_info = gpu.OP_INFO[op]
    lups = float(n) ** 3 * (2 * ((nt + 1) // 2))
    crange = wl.get("c", (0.0, 0.0))
    init = gpu.Context(op, n, n, n, device=local, precision="fp64", schedule="plain")
    seed_ctx(init, wl)
    shape = init.shape
    host = [torch.empty(shape, dtype=torch.float64, pin_memory=True) for _ in range(3)]
    init.download(host[0].data_ptr(), host[1].data_ptr())
    if op_info[1] == 2:
        init.download_roc2(host[2].data_ptr())
    init.close()
    if op_info[3]:
        rng = np.random.default_rng(wl["seed"])
        coefs = torch.empty((op_info[2],) + tuple(shape), dtype=torch.float64, pin_memory=True)
        coefs.numpy()[...] = rng.uniform(*crange, size=coefs.shape)
        cptr = coefs.data_ptr()
    else:
        coefs = np.array(wl["coefs"] + [0.0] * (11 - len(wl["coefs"])))
        cptr = coefs
    ectx = gpu.Context(op, n, n, n, device=local, fusion_depth=depth if form_kw["schedule"] == "fused" else 0,
                       **form_kw)
    u3 = host[2].data_ptr() if op_info[1] == 2 else None
    for _ in range(max(1, warmup)):
        ectx.upload(host[0].data_ptr(), host[1].data_ptr(), u3, cptr)
        ectx.run(nt)
        ectx.download(host[0].data_ptr(), None)
    sync()
    # each call returns after its stream work completed, so host clocks
    # between the calls split the step into its phases
    ph = {"upload": 0.0, "run": 0.0, "download": 0.0}
    t0 = time.perf_counter()
    for _ in range(steps):
        a = time.perf_counter()
        ectx.upload(host[0].data_ptr(), host[1].data_ptr(), u3, cptr)
        b = time.perf_counter()
        ectx.run(nt)
        c = time.perf_counter()
        ectx.download(host[0].data_ptr(), None)
        d = time.perf_counter()
        ph["upload"] += b - a
        ph["run"] += c - b
        ph["download"] += d - c
    sync()
    wall = max_over_ranks(time.perf_counter() - t0, "cuda")
    nbytes = host[0].numel() * 8
    ectx.close()
    return {"value": world * steps * lups / wall / 1e9, "unit": "GLUP/s",
            "h2d_bytes_per_step": nbytes * (3 if u3 else 2) + (nbytes * op_info[2] if op_info[3] else 0),
            "d2h_bytes_per_step": nbytes,
            "host_arrays": "pinned FP64 (reference real_t=double layout)",
            "phases_ms_per_step": {k: 1e3 * v / steps for k, v in ph.items()}}


def run_ours(args, wl, rank, world, local):
    import torch
    from girih_gb300 import gpu

    torch.cuda.set_device(local)
    n, nt, op = wl["n"], wl["nt"], wl["op"]
    forms = forms_of(op)
    if args.forms:
        forms = {k: v for k, v in forms.items() if k in args.forms.split(",")}
    dist = world > 1
    if dist:
        import torch.distributed as tdist

    def barrier_sync():
        torch.cuda.synchronize()
        if dist:
            tdist.barrier()

    head = args.headline if args.headline in forms else list(forms)[0]
    sampler = ClockSampler(local)
    with sampler:
        results, ctxs = time_forms(wl, forms, args.steps, args.warmup, local, world, args.depth, args.block,
                                   headline=head, sync=barrier_sync)
    clocks = sampler.summary()
    for c in ctxs.values():
        c.close()

    errors = {} if args.no_error else form_errors(wl, forms, local, args.depth)

    h = results[head]
    peak, peak_kind = measured_peak_hbm()
    op_info = gpu.OP_INFO[op]
    roofline = roofline_of(h, op_info, n, peak, peak_kind, WORKLOAD_NAME, head)
    forms_out = {}
    for k, v in results.items():
        forms_out[k] = {kk: v[kk] for kk in ("glups", "ms_per_step", "steps", "launches_per_step", "depth", "tile",
                                             "schedule", "kernel")}
        if k != head:
            rf = roofline_of(v, op_info, n, peak, peak_kind, WORKLOAD_NAME, k)
            forms_out[k]["roofline"] = {kk: rf[kk] for kk in ("achieved", "frac", "traffic", "kernel")}

    e2e = None if args.no_e2e else run_e2e(wl, forms[head], args.steps, args.warmup, local, world, barrier_sync,
                                           args.depth)

    line = {
        "metric": METRIC,
        "value": h["glups"], "unit": "GLUP/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": h["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp64": "f64", "fp64df": "df64 (FP32 pairs, FP64 fields)"}.get(h["precision"], "f32"),
        "data": "synthetic (seeded SplitMix64, FP64 inputs)",
        "config": workload_config(wl, world),
        "form": {"name": head, "precision": h["precision"], "schedule": h["schedule"], "fusion_depth": h["depth"],
                 "tile": h["tile"], "kernel": h["kernel"]},
        "forms": forms_out,
        "errors": errors,
        "roofline": roofline,
        "e2e": e2e,
        "gpu_launches": args.steps * h["launches_per_step"],
        "clocks": clocks,
    }
    if "plain64" in results:
        line["speedup_vs_plain64"] = {k: v["glups"] / results["plain64"]["glups"] for k, v in results.items()}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(wl, args.cpu_seconds)
    if rank == 0 and args.secondary:
        line["secondary"] = run_secondary(args, local)
    return line


def workload_config(wl, world):
    """The workload description shared by both arms' lines."""
    return {"workload": WORKLOAD_NAME, "operator": wl["op"], "grid": [wl["n"]] * 3, "nt": wl["nt"],
            "seed": wl["seed"], "parallelism": f"replicas{world}", "l2": "inputs larger than L2 (no flush needed)"}


# ---------------------------------------------------------------- secondary configurations

SECONDARY_FORMS = {
    # 25-point leapfrog: FP64 plain and time-fused (double-float), FP32 storage/accumulation, mixed
    "star25_leapfrog_480": {"plain64": dict(precision="fp64", schedule="plain"),
                            "fused64df": dict(precision="fp64df", schedule="fused"),
                            "fp32": dict(precision="fp32", schedule="auto"),
                            "mixed": dict(precision="mixed", schedule="auto")},
    # variable coefficients: FP64 plain, mixed (BF16 coefficients, FP32 fields), plain and fused
    "var7_384": {"plain64": dict(precision="fp64", schedule="plain"),
                 "mixed": dict(precision="mixed", schedule="plain"),
                 "mixedfused": dict(precision="mixed", schedule="fused")},
    "var25_384": {"plain64": dict(precision="fp64", schedule="plain"),
                  "mixed": dict(precision="mixed", schedule="plain"),
                  "mixedfused": dict(precision="mixed", schedule="fused")},
}


def run_secondary(args, local):
    """The other configurations in compact form: a few timed runs per form,
    errors against the FP64 CPU oracle, the reference's CPU rate on a short
    sample, and the batched workload."""
    from girih_gb300 import gpu
    import torch
    out = {}
    peak, peak_kind = measured_peak_hbm()
    for name, forms in SECONDARY_FORMS.items():
        wl = dict(WORKLOADS[name])
        t0 = time.perf_counter()
        res, ctxs = time_forms(wl, forms, 2, 1, local, sync=torch.cuda.synchronize)
        for c in ctxs.values():
            c.close()
        errs = form_errors(wl, forms, local)
        op_info = gpu.OP_INFO[wl["op"]]
        o = {"operator": wl["op"], "grid": [wl["n"]] * 3, "nt": wl["nt"], "seed": wl["seed"], "forms": {}}
        for k, v in res.items():
            # one step per pass (plain, or fused at depth 1): the one-step bytes per update are the
            # pass's algorithmic bytes; deeper passes move fewer and report none here
            algo = v["bytes_per_lup"] * v["glups"] if (v["schedule"] == "plain" or v["depth"] == 1) else None
            o["forms"][k] = {"glups": v["glups"], "ms_per_step": v["ms_per_step"], "schedule": v["schedule"],
                             "kernel": v["kernel"], "depth": v["depth"], "tile": v["tile"],
                             "bytes_per_lup": v["bytes_per_lup"],
                             "hbm_gbs_algorithmic": algo,
                             "hbm_frac_of_peak": (algo / peak) if algo else None,
                             "errors": errs.get(k)}
        try:
            o["cpu_reference"] = cpu_baseline(wl, 5.0, tests=2)
        except Exception as e:  # the CPU baseline is reported, not required
            o["cpu_reference"] = {"unavailable": str(e)[:200]}
        o["wall_s"] = time.perf_counter() - t0
        out[name] = o
    t0 = time.perf_counter()
    b = run_batched_core(local, nt=100, steps=2, warmup=1)
    b["wall_s"] = time.perf_counter() - t0
    out["batched64"] = b
    out["peak_source"] = peak_kind
    return out


def batched_grids(seed=4, n=64):
    """64 grids: edges from {32,48,64,96,128,160,192}, cubes and 2:1:1 boxes,
    half the 7-point leapfrog (operator 8), half the 25-point leapfrog (operator 0)."""
    import numpy as np
    rng = np.random.Generator(np.random.PCG64(seed))
    edges = [32, 48, 64, 96, 128, 160, 192]
    grids = []
    for k in range(n):
        e = int(rng.choice(edges))
        op = 8 if k < n // 2 else 0
        if k % 2 == 0:
            grids.append((op, e, e, e))
        else:
            grids.append((op, e, max(8, e // 2), max(8, e // 2)))
    return grids


BATCH_INPUTS = {8: dict(f=(0.0, 1.0), roc2=(0.5, 1.5), coefs=[-0.75, 0.125]),
                0: dict(f=(-1.0, 1.0), roc2=(0.05, 0.15),
                        coefs=[-8.541667, 1.6, -0.2, 0.025396826, -0.0017857143])}


def run_batched_core(local, nt=100, steps=5, warmup=3, precision="mixed"):
    """64 uneven grids, FP32 fields, nt steps: one persistent launch per fused
    pass vs looping the single-grid kernels; every grid against the FP64 CPU
    oracle from the same FP64 inputs."""
    import torch
    from girih_gb300 import gpu
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    torch.cuda.set_device(local)
    grids = batched_grids()
    lups = sum(float(nx) * ny * nz for _, nx, ny, nz in grids) * 2 * ((nt + 1) // 2)
    threads = host_threads()
    with gpu.Batch(grids, precision=precision, device=local) as b:
        def seed_all():
            for k, (op, nx, ny, nz) in enumerate(grids):
                w = BATCH_INPUTS[op]
                b.grid(k).fill_seeded(4000 + k, w["f"], w["roc2"], coefs=w["coefs"])
        seed_all()
        b.autotune()
        res = {}
        sampler = ClockSampler(local)
        with sampler:
            for name, fn in (("batched", b.run), ("looped", b.run_looped)):
                for _ in range(warmup):
                    fn(nt)
                torch.cuda.synchronize()
                ms = [fn(nt) for _ in range(steps)]
                info = b.info()
                res[name] = dict(glups=steps * lups / (sum(ms) / 1e3) / 1e9, ms_per_step=sum(ms) / steps,
                                 launches_per_step=info["launches_last_run"], items_per_step=info["items_last_run"])
        depths = b.info()["depths"]
        seed_all()
        b.run(nt)
        worst = {"max_rel": 0.0, "l2_rel": 0.0, "grid": None}
        t0 = time.perf_counter()
        for k, (op, nx, ny, nz) in enumerate(grids):
            w = BATCH_INPUTS[op]
            g = oracle.Grid(op, nx, ny, nz)
            g.fill_seeded(4000 + k, w["f"], w["roc2"], coefs=w["coefs"], nthreads=threads)
            g.run(nt, nthreads=threads)
            mr, l2 = gpu.rel_errors(b.grid(k).error_norms(g.U1))
            if mr > worst["max_rel"]:
                worst["max_rel"], worst["grid"] = mr, [op, nx, ny, nz]
            worst["l2_rel"] = max(worst["l2_rel"], l2)
        oracle_s = time.perf_counter() - t0
    return {"grids": len(grids), "nt": nt, "precision": precision,
            "points": sum(nx * ny * nz for _, nx, ny, nz in grids), "depths": depths,
            "forms": res, "speedup_vs_looped": res["batched"]["glups"] / res["looped"]["glups"],
            "errors": {"worst_grid": worst, "against": "FP64 CPU oracle of each grid, same FP64 inputs",
                       "oracle_s": oracle_s},
            "clocks": sampler.summary(), "gpu_launches": steps * res["batched"]["launches_per_step"]}


def run_batched(args, rank, world, local):
    """Batched workload line (64 independent grids of uneven sizes, the batched configuration)."""
    nt = args.nt or 100
    b = run_batched_core(local, nt=nt, steps=args.steps, warmup=args.warmup)
    return {"metric": "GLUP/s, 64 batched grids (7-pt and 25-pt leapfrog, FP32 fields), nt=100",
            "value": b["forms"]["batched"]["glups"], "unit": "GLUP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": b["forms"]["batched"]["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, FP64 inputs)",
            "config": {"workload": "batched64", "grids": b["grids"], "nt": nt, "points": b["points"],
                       "depths": b["depths"]},
            "forms": b["forms"], "speedup_vs_looped": b["speedup_vs_looped"], "errors": b["errors"],
            "clocks": b["clocks"], "gpu_launches": b["gpu_launches"]}


# ---------------------------------------------------------------- reference arm

def run_reference(args, wl, rank, world):
    """The reference's own CPU implementation on the host cores: one reference
    performance test (a bounded sample of the workload's time loop on the full
    grid) per step, W warm-up tests untimed."""
    if rank != 0:
        return None
    base = {"impl": "reference", "metric": METRIC, "unit": "GLUP/s", "n_gpus": world, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": workload_config(wl, world)}
    n = wl["n"]
    kernel = wl.get("ref_kernel", wl["op"])
    ran, why = None, None
    if reference_binary_ok() and kernel in REFERENCE_STEPPER:
        try:
            ran = run_reference_binary(kernel, n, args.warmup + args.steps)
        except Exception as e:
            why = str(e)[:200]
    if ran:
        times, nt_eff, threads, cmd = ran
        timed = times[args.warmup:]
        rates = [float(n) ** 3 * nt_eff / t / 1e9 for t in timed]
        v = statistics.median(rates)
        note = "" if kernel == wl["op"] else (
            f"; the reference has no operator {wl['op']} (7-point leapfrog): its 7-point constant-coefficient "
            f"kernel {kernel}, two arrays per update instead of three, stands in")
        cb = {"value": v, "unit": "GLUP/s", "cores": threads, "kind": "reference",
              "sample": f"{n}^3 grid, kernel {kernel}, each step one reference performance test of {nt_eff} "
                        f"time steps ({statistics.median(timed):.2f} s), "
                        f"{stepper_name(REFERENCE_STEPPER[kernel]['args'])}{note}",
              "command": cmd}
        line = dict(base, value=v, steps=args.steps, ms_per_step=1e3 * statistics.median(timed),
                    sampled={"time_steps_per_step": nt_eff, "of": wl["nt"]}, reference_kernel=kernel)
    else:
        vals = []
        per_step_s = max(1.0, args.cpu_seconds / max(1, args.steps))
        cb = None
        for _ in range(args.steps):
            cb = cpu_baseline_port(wl, per_step_s)
            vals.append(cb["value"])
        v = statistics.median(vals)
        cb["value"] = v
        if why:
            cb["reference_failed"] = why
        line = dict(base, value=v, steps=args.steps, sampled={"seconds_per_step": per_step_s})
    line["cpu_baseline"] = cb
    line["e2e"] = {"value": v, "unit": "GLUP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    return line


WORKLOAD_NAME = "star7_leapfrog_512"


def main():
    global WORKLOAD_NAME
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="star7_leapfrog_512", choices=sorted(WORKLOADS) + ["batched64"])
    ap.add_argument("--forms", default="")
    ap.add_argument("--headline", default="fused64df")
    ap.add_argument("--depth", type=int, default=0)
    ap.add_argument("--block", default="", help="fused output tile BX,BY (selects the tile variant)")
    ap.add_argument("--grid", "--n", dest="n", type=int, default=0,
                    help="override the grid edge (small profiling cases)")
    ap.add_argument("--nt", type=int, default=0, help="override the number of time steps")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-error", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--secondary", dest="secondary", action="store_true", default=None,
                    help="run the secondary configurations (default: on for the default workload)")
    ap.add_argument("--no-secondary", dest="secondary", action="store_false")
    args = ap.parse_args()
    WORKLOAD_NAME = args.workload
    if args.secondary is None:
        args.secondary = args.workload == "star7_leapfrog_512" and not (args.n or args.nt or args.forms)
    rank, world, local = rank_env()
    if args.workload == "batched64":
        if args.impl == "reference":
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference advances one grid per "
                                  "process; it has no batched counterpart"}), flush=True)
            return
        line = run_batched(args, rank, world, local)
        if rank == 0:
            print(json.dumps(line), flush=True)
        return
    wl = dict(WORKLOADS[args.workload])
    if args.n:
        wl["n"] = args.n
    if args.nt:
        wl["nt"] = args.nt
        wl["error_nts"] = [m for m in wl.get("error_nts", []) if m < args.nt]
    if world > 1 and args.impl == "ours":
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(local)
        tdist.init_process_group("nccl")
    if args.impl == "reference":
        line = run_reference(args, wl, rank, world)
    else:
        line = run_ours(args, wl, rank, world, local)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if world > 1 and args.impl == "ours":
        import torch.distributed as tdist
        tdist.destroy_process_group()


if __name__ == "__main__":
    main()
