"""Benchmark of the girih star-stencil hot path on GB300.

Workload (default): the 7-point constant-coefficient leapfrog stencil (operator
8: u = 2v - u + roc2*(c0 v + c1 sum6 v)), nx=ny=nz=512, nt=500, seeded U(0,1)
fields, roc2 U(0.5,1.5), c = (-0.75, 0.125); inputs FP32-representable so that
FP32 and FP64 runs see identical data.  One benchmark "step" is one call of the
hot path: the whole nt=500 time loop over the 512^3 grid.

Forms measured on the same grid, each from device-resident inputs:
  plain64  FP64, one sweep per kernel launch (the drop-in form)
  fused64  FP64, time-fused passes, FP64 arithmetic (bound by GB300's FP64 pipe)
  fused64df FP64 fields, time-fused passes, double-float arithmetic (FP32 pairs)
  mixed    FP32 fields, compensated leapfrog, time-fused passes
`value` is the headline form's GLUP/s (--headline, default mixed); `e2e` is the
same form through the C ABI from pinned HOST arrays (upload + run + download).

--impl reference times the CPU restatement of the reference operator (the
oracle, OpenMP over all host cores) on a bounded sample of the same workload.
Multi-GPU (torchrun): every rank advances its own replica of the grid
("replicas only": the path has no exchange on one grid per GPU).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: op, n, nt, seed, field range, roc2 range, constant coefficients
    "star7_leapfrog_512": dict(op=8, n=512, nt=500, seed=1, f=(0.0, 1.0), roc2=(0.5, 1.5), coefs=[-0.75, 0.125]),
    # Jacobi smoother c0 + 6 c1 = 1: the reference's default pair (-0.28472, 0.16) amplifies the
    # checkerboard mode by |c0 - 6 c1| = 1.24 per step (1e46 after 500 steps, past the FP32 range)
    "star7_jacobi_512": dict(op=1, n=512, nt=500, seed=1, f=(0.0, 1.0), roc2=(0.0, 0.0), coefs=[0.25, 0.125]),
    "star25_leapfrog_480": dict(op=0, n=480, nt=200, seed=2, f=(-1.0, 1.0), roc2=(0.05, 0.15),
                                coefs=[-8.541667, 1.6, -0.2, 0.025396826, -0.0017857143], error_nts=[50, 100]),
    # variable coefficients, coefficient arrays U(0.01, 0.1/radius)
    "var7_384": dict(op=5, n=384, nt=200, seed=3, f=(0.0, 1.0), roc2=(0.0, 0.0), c=(0.01, 0.1), coefs=None),
    "var25_384": dict(op=4, n=384, nt=200, seed=3, f=(0.0, 1.0), roc2=(0.0, 0.0), c=(0.01, 0.025), coefs=None),
}


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


def run_ours(args, wl, rank, world, local):
    import numpy as np
    import torch
    from girih_gb300 import gpu

    torch.cuda.set_device(local)
    n, nt, op = wl["n"], wl["nt"], wl["op"]
    lups = float(n) ** 3 * (2 * ((nt + 1) // 2))
    if gpu.OP_INFO[op][3]:  # variable coefficients: the mixed form streams them in the x-quad plain sweep
        forms = {
            "plain64": dict(precision="fp64", schedule="plain"),
            "mixed": dict(precision="mixed", schedule="plain"),
            "fused32": dict(precision="fp32", schedule="fused"),
            "mixedfused": dict(precision="mixed", schedule="fused"),
        }
    else:
        forms = {
            "plain64": dict(precision="fp64", schedule="plain"),
            "fused64": dict(precision="fp64", schedule="fused"),
            "fused64df": dict(precision="fp64df", schedule="fused"),
            "plainmixed": dict(precision="mixed", schedule="plain"),  # one step per pass, x quads
            "mixed": dict(precision="mixed", schedule="fused"),
        }
    crange = wl.get("c", (0.0, 0.0))
    if args.forms:
        forms = {k: v for k, v in forms.items() if k in args.forms.split(",")}
    dist = world > 1
    if dist:
        import torch.distributed as tdist

    def barrier_sync():
        torch.cuda.synchronize()
        if dist:
            tdist.barrier()

    results, ctxs = {}, {}
    sampler = ClockSampler(local)
    with sampler:
        for name, kw in forms.items():
            blk = tuple(int(x) for x in args.block.split(",")) if args.block and kw["schedule"] == "fused" else (0, 0)
            ctx = gpu.Context(op, n, n, n, device=local, fusion_depth=args.depth if kw["schedule"] == "fused" else 0,
                              block=blk, **kw)
            ctx.fill_seeded(wl["seed"], wl["f"], wl["roc2"], crange, coefs=wl["coefs"], f32_exact=True)
            if kw["schedule"] != "plain" and not args.depth and not args.block:
                ctx.autotune()  # picks tile and fusion depth on this grid; the grid state is restored
            for _ in range(args.warmup):
                ctx.run(nt)
            barrier_sync()
            ms = []
            t0 = time.perf_counter()
            for _ in range(args.steps):
                ms.append(ctx.run(nt))
            barrier_sync()
            wall = time.perf_counter() - t0
            dev_s = max_over_ranks(sum(ms) / 1e3, "cuda")
            info = ctx.info()
            results[name] = dict(glups=world * args.steps * lups / dev_s / 1e9, ms_per_step=1e3 * dev_s / args.steps,
                                 wall_s=wall, launches_per_step=info["launches_last_run"],
                                 depth=info["fusion_depth"], tile=[info["block_x"], info["block_y"]],
                                 kernel=info["kernel_name"], tsz=8 if kw["precision"] in ("fp64", "fp64df") else 4,
                                 schedule=kw["schedule"], precision=kw["precision"])
            ctxs[name] = ctx
    clocks = sampler.summary()

    # errors: fresh nt-step runs from the same init against the FP64 plain form
    errors = {}
    if "plain64" in forms and not args.no_error:
        # checkpoints (cumulative steps; the last is nt): runs continue from the state
        marks = [m for m in wl.get("error_nts", []) if 0 < m < nt] + [nt]
        ref = gpu.Context(op, n, n, n, device=local, precision="fp64", schedule="plain")
        ref.fill_seeded(wl["seed"], wl["f"], wl["roc2"], crange, coefs=wl["coefs"], f32_exact=True)
        others = {}
        for name, kw in forms.items():
            if name == "plain64":
                continue
            c = gpu.Context(op, n, n, n, device=local, fusion_depth=args.depth if kw["schedule"] == "fused" else 0, **kw)
            # creation picks up the autotuned choice cached above for this operator and size
            c.fill_seeded(wl["seed"], wl["f"], wl["roc2"], crange, coefs=wl["coefs"], f32_exact=True)
            others[name] = c
            errors[name] = {"nt": nt, "against": "plain64 (FP64, parity-checked vs the oracle)"}
        done = 0
        for m in marks:
            ref.run(m - done)
            for name, c in others.items():
                c.run(m - done)
                mr, l2 = gpu.rel_errors(c.compare(ref))
                errors[name]["max_rel"], errors[name]["l2_rel"] = mr, l2
                if len(marks) > 1:
                    errors[name].setdefault("by_nt", {})[str(m)] = {"max_rel": mr, "l2_rel": l2}
            done = m
        for c in others.values():
            c.close()
        ref.close()

    head = args.headline if args.headline in results else list(results)[0]
    h = results[head]
    # roofline of the headline form's kernel (one launch = one pass over the grid)
    peak, peak_kind = measured_peak_hbm()
    op_info = gpu.OP_INFO[op]
    per_pt = pass_bytes(op_info, h["tsz"], h["schedule"], h["precision"])
    launch_ms = h["ms_per_step"] / max(1, h["launches_per_step"])
    achieved = per_pt * float(n) ** 3 / (launch_ms / 1e3) / 1e9
    kernel_key = f"{h['kernel']}:{WORKLOAD_NAME}:{head}"
    traffic = committed_traffic(kernel_key)

    # end to end through the C ABI from pinned host arrays
    e2e = None
    if not args.no_e2e:
        ctx = ctxs[head]
        shape = ctx.shape
        host = [torch.empty(shape, dtype=torch.float64, pin_memory=True) for _ in range(3)]
        # fill the host arrays with the seeded inputs: download the initial state
        init = gpu.Context(op, n, n, n, device=local, precision="fp64", schedule="plain")
        init.fill_seeded(wl["seed"], wl["f"], wl["roc2"], crange, coefs=wl["coefs"], f32_exact=True)
        init.download(host[0].data_ptr(), host[1].data_ptr())
        init.download_roc2(host[2].data_ptr()) if op_info[1] == 2 else None
        init.close()
        if op_info[3]:
            # coefficient arrays: seeded host values in the workload's range (uploaded every step)
            rng = np.random.default_rng(wl["seed"])
            coefs = torch.empty((op_info[2],) + tuple(shape), dtype=torch.float64, pin_memory=True)
            coefs.numpy()[...] = rng.uniform(*crange, size=coefs.shape)
        else:
            coefs = np.array(wl["coefs"] + [0.0] * (11 - len(wl["coefs"])))
        ctx.close()
        ectx = gpu.Context(op, n, n, n, device=local, fusion_depth=args.depth if forms[head]["schedule"] == "fused" else 0,
                           **forms[head])
        u3 = host[2].data_ptr() if op_info[1] == 2 else None
        for _ in range(max(1, args.warmup)):
            ectx.upload(host[0].data_ptr(), host[1].data_ptr(), u3, coefs if not op_info[3] else coefs.data_ptr())
            ectx.run(nt)
            ectx.download(host[0].data_ptr(), None)
        barrier_sync()
        # each call returns after its stream work completed, so host clocks
        # between the calls split the step into its phases
        ph = {"upload": 0.0, "run": 0.0, "download": 0.0}
        t0 = time.perf_counter()
        for _ in range(args.steps):
            a = time.perf_counter()
            ectx.upload(host[0].data_ptr(), host[1].data_ptr(), u3, coefs if not op_info[3] else coefs.data_ptr())
            b = time.perf_counter()
            ectx.run(nt)
            c = time.perf_counter()
            ectx.download(host[0].data_ptr(), None)
            d = time.perf_counter()
            ph["upload"] += b - a
            ph["run"] += c - b
            ph["download"] += d - c
        barrier_sync()
        wall = max_over_ranks(time.perf_counter() - t0, "cuda")
        nbytes = host[0].numel() * 8
        e2e = {"value": world * args.steps * lups / wall / 1e9, "unit": "GLUP/s",
               "h2d_bytes_per_step": nbytes * (3 if u3 else 2) + (nbytes * op_info[2] if op_info[3] else 0),
               "d2h_bytes_per_step": nbytes,
               "host_arrays": "pinned FP64 (reference real_t=double layout)",
               "phases_ms_per_step": {k: 1e3 * v / args.steps for k, v in ph.items()}}
        ectx.close()
    for c in ctxs.values():
        c.close()

    line = {
        "metric": "GLUP/s at 512^3: time-fused & mixed vs plain FP64 on GB300; % HBM roofline; err",
        "value": h["glups"], "unit": "GLUP/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": h["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp64": "f64", "fp64df": "df64 (FP32 pairs)"}.get(h["precision"], "f32"),
        "data": "synthetic (seeded SplitMix64, FP32-representable)",
        "config": {"workload": WORKLOAD_NAME, "operator": op, "grid": [n, n, n], "nt": nt, "headline_form": head,
                   "fusion_depth": h["depth"], "tile": h["tile"],
                   "parallelism": f"replicas{world}", "l2": "inputs larger than L2 (no flush needed)"},
        "forms": {k: {kk: v[kk] for kk in ("glups", "ms_per_step", "launches_per_step", "depth", "tile")}
                  for k, v in results.items()},
        "errors": errors,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_source": peak_kind, "kernel": h["kernel"],
                     "algorithmic_bytes_per_point_per_launch": per_pt,
                     "effective_bandwidth_gbs": h["glups"] * (per_pt if h["schedule"] == "plain" else
                                                              pass_bytes(op_info, h["tsz"], "plain", h["precision"]))},
        "e2e": e2e,
        "gpu_launches": args.steps * h["launches_per_step"],
        "clocks": clocks,
    }
    if "plain64" in results:
        line["speedup_vs_plain64"] = {k: v["glups"] / results["plain64"]["glups"] for k, v in results.items()}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(wl, args.cpu_seconds)
    return line


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


def run_batched(args, rank, world, local):
    """Batched workload: 64 uneven grids, FP32 fields (mixed), nt=100, one
    persistent launch per fused pass vs looping the single-grid kernels."""
    import torch
    from girih_gb300 import gpu
    torch.cuda.set_device(local)
    nt = args.nt or 100
    grids = batched_grids()
    lups = sum(float(nx) * ny * nz for _, nx, ny, nz in grids) * 2 * ((nt + 1) // 2)
    with gpu.Batch(grids, precision="mixed", device=local) as b:
        for k, (op, nx, ny, nz) in enumerate(grids):
            w = BATCH_INPUTS[op]
            b.grid(k).fill_seeded(4000 + k, w["f"], w["roc2"], coefs=w["coefs"], f32_exact=True)
        b.autotune()
        res = {}
        sampler = ClockSampler(local)
        with sampler:
            for name, fn in (("batched", b.run), ("looped", b.run_looped)):
                for _ in range(args.warmup):
                    fn(nt)
                torch.cuda.synchronize()
                ms = [fn(nt) for _ in range(args.steps)]
                info = b.info()
                res[name] = dict(glups=args.steps * lups / (sum(ms) / 1e3) / 1e9, ms_per_step=sum(ms) / args.steps,
                                 launches_per_step=info["launches_last_run"], items_per_step=info["items_last_run"])
        depths = b.info()["depths"]
        # every grid against an FP64 plain run of its own, from the same inputs:
        # re-seed the whole batch, one batched run of nt steps, then compare
        for k, (op, nx, ny, nz) in enumerate(grids):
            w = BATCH_INPUTS[op]
            b.grid(k).fill_seeded(4000 + k, w["f"], w["roc2"], coefs=w["coefs"], f32_exact=True)
        b.run(nt)
        worst = {"max_rel": 0.0, "l2_rel": 0.0}
        for k, (op, nx, ny, nz) in enumerate(grids):
            w = BATCH_INPUTS[op]
            with gpu.Context(op, nx, ny, nz, precision="fp64", schedule="plain", device=local) as ref:
                ref.fill_seeded(4000 + k, w["f"], w["roc2"], coefs=w["coefs"], f32_exact=True)
                ref.run(nt)
                mr, l2 = gpu.rel_errors(b.grid(k).compare(ref))
            worst["max_rel"] = max(worst["max_rel"], mr)
            worst["l2_rel"] = max(worst["l2_rel"], l2)
    return {"metric": "GLUP/s, 64 batched grids (7-pt and 25-pt leapfrog, FP32 fields), nt=100",
            "value": res["batched"]["glups"], "unit": "GLUP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": res["batched"]["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, FP32-representable)",
            "config": {"workload": "batched64", "grids": len(grids), "nt": nt,
                       "points": sum(nx * ny * nz for _, nx, ny, nz in grids), "depths": depths},
            "forms": res, "speedup_vs_looped": res["batched"]["glups"] / res["looped"]["glups"],
            "errors": {"worst_grid": worst, "against": "FP64 plain run of each grid (single-grid path)"},
            "clocks": sampler.summary(), "gpu_launches": args.steps * res["batched"]["launches_per_step"]}


def cpu_baseline(wl, seconds, steps=None):
    """The oracle restatement (OpenMP over all host threads) on a bounded sample of
    the workload: the full grid, a few sweeps.  Returns the cpu_baseline object."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    n, op = wl["n"], wl["op"]
    threads = os.cpu_count() or 1
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


def run_reference(args, wl, rank, world):
    if rank != 0:
        return None
    vals = []
    # no warm-up runs: each step's sample times its own sweeps after one untimed pair
    # (cpu_baseline), which is the only state the CPU restatement warms
    threads = os.cpu_count() or 1
    per_step_s = max(1.0, args.cpu_seconds / max(1, args.steps))
    cb = None
    for _ in range(args.steps):
        cb = cpu_baseline(wl, per_step_s)
        vals.append(cb["value"])
    v = statistics.median(vals)
    cb["value"] = v
    return {"impl": "reference", "metric": "GLUP/s at 512^3: time-fused & mixed vs plain FP64 on GB300; % HBM roofline; err",
            "value": v, "unit": "GLUP/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD_NAME, "operator": wl["op"], "grid": [wl["n"]] * 3, "nt": wl["nt"],
                       "threads": threads},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": "GLUP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


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
    ap.add_argument("--headline", default="mixed")
    ap.add_argument("--depth", type=int, default=0)
    ap.add_argument("--block", default="", help="fused output tile BX,BY (selects the tile variant)")
    ap.add_argument("--grid", "--n", dest="n", type=int, default=0,
                    help="override the grid edge (small profiling cases)")
    ap.add_argument("--nt", type=int, default=0, help="override the number of time steps")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-error", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    WORKLOAD_NAME = args.workload
    if args.workload == "batched64":
        rank, world, local = rank_env()
        line = run_batched(args, rank, world, local)
        if rank == 0:
            print(json.dumps(line), flush=True)
        return
    wl = dict(WORKLOADS[args.workload])
    if args.n:
        wl["n"] = args.n
    if args.nt:
        wl["nt"] = args.nt
    rank, world, local = rank_env()
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
