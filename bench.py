#!/usr/bin/env python
"""Throughput of the GB300 Siddon projector + backprojector.

Workload (the differentiable-reconstruction configuration): float32 cube of
256^3 voxels spanning [-1.5, 1.5] solar radii, 360 conic views of 512 x 512
pixels over 0-360 deg at d = 215 solar radii, obstacle = "sun", seeded
shell + blob phantom.  One step = one projection of the cube into the
(zeroed) data stack + one backprojection of that stack into a (zeroed) cube,
i.e. the operator work of one CG / gradient iteration, over all
512 * 512 * 360 = 94,371,840 rays.

metric "proj+backproj rays/s": rays per second through a projection +
backprojection pair (value = N_gpus * rays / step time).  Multi-GPU runs are
independent replicas (the path's only cross-view exchange is the sum of cube
partials, which this single-GPU deployment does not need): scaling "weak".

Lines printed (one JSON line from rank 0):
  default          our kernels (CUDA events on the launching stream; L2 flushed
                   between steps by a 256 MiB write), plus the e2e figure through
                   the public operator API with pinned host buffers, the
                   roofline of the dominant kernel and a CPU baseline;
  --impl reference the reference algorithm's CPU implementation (the oracle's C
                   restatement, float32, all host threads) on a bounded sample
                   of the same workload.
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
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "proj+backproj rays/s"
UNIT = "rays/s"
WORKLOAD = "recon256"
WORKLOAD_DESC = ("differentiable-reconstruction geometry: 256^3 f32 cube on [-1.5,1.5] Rsun, 360 views of "
                 "512x512 over 0-360 deg at d=215 Rsun, obstacle=sun; step = projection + backprojection")
L2_FLUSH_BYTES = 256 << 20
CPU_SAMPLE_VIEWS = 16


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-other", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the uneven multi-job batch measurement")
    ap.add_argument("--no-served", action="store_true", help="skip the serving-stream measurement")
    ap.add_argument("--no-4d", action="store_true", help="skip the time-dependent (4-D) measurement")
    ap.add_argument("--no-lbfgs", action="store_true", help="skip the differentiable-reconstruction measurement")
    ap.add_argument("--served-jobs", type=int, default=2000,
                    help="requests of the serving stream (Poisson, 20 jobs/s)")
    ap.add_argument("--profile-packed", action="store_true",
                    help="one packed projection + backprojection of the 32-job uneven batch (the case of the "
                         "packed-kernel ncu summary in profiles/)")
    ap.add_argument("--profile-case", action="store_true",
                    help="one projection + one backprojection on the workload's geometry restricted to every "
                         "10th view (36 views): the case the ncu summaries in profiles/ are captured on")
    return ap.parse_args()


def slowest_rank_ms(ms, world, device):
    """Step time of the job: the maximum over ranks (all ranks get it)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank, ms, world):
    """Whole-job rate of `world` independent replicas that each process
    `units_per_rank` units per step in `ms` (the slowest rank's time)."""
    return world * units_per_rank / (ms / 1000.0)


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


# ---------------------------------------------------------------------------
# clocks during the timed region

class Clocks:
    FIELDS = ("uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid=None):
        self.uuid = uuid
        self.path = os.path.join(tempfile.gettempdir(), "tomograpy_gb300_clocks_%d.csv" % os.getpid())
        self.proc = None

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            if self.uuid and self.uuid not in p[0] and p[0] not in self.uuid:
                continue
            rows.append(p)
        if not rows:
            return None
        try:
            sm = [float(r[1]) for r in rows]
            smax = max(float(r[2]) for r in rows)
            power = [float(r[3]) for r in rows]
        except ValueError:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        pmax = max(power)
        loaded = [s for s, pw in zip(sm, power) if pw >= 0.5 * pmax] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": smax, "reasons": reasons,
                "samples": len(rows), "power_w_max": pmax}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(kernel):
    """DRAM bytes (read + write) per launch of ``kernel`` on the full workload,
    from the committed ncu summary profiles/siddon_f32_dram_256cube_360x512.md."""
    path = os.path.join(ROOT, "profiles", "siddon_f32_dram_256cube_360x512.md")
    try:
        for line in open(path):
            if line.startswith(kernel + " dram_bytes_per_launch:"):
                return float(line.split(":")[1].split()[0])
    except Exception:
        pass
    return None


ISSUE_PROFILE = "siddon_f32_ncu_full_256cube_36x512.md"


def ncu_issue(kernel):
    """Issue-roof figures of ``kernel`` from the committed ncu summary of the
    36-view case (profiles/siddon_f32_ncu_full_256cube_36x512.md): issue-active
    share, warp instructions, segments, active lanes per instruction."""
    path = os.path.join(ROOT, "profiles", ISSUE_PROFILE)
    try:
        for line in open(path):
            if line.startswith(kernel + " issue:"):
                kv = dict(tok.split("=") for tok in line.split(":", 1)[1].split())
                return {k: float(v) for k, v in kv.items()}
    except Exception:
        pass
    return None


def issue_roofline(kernel, segments, ms, sm_mhz, n_sms=152, schedulers=4):
    """The roof the kernel is actually under: instruction issue.  Warp
    instructions per segment (from the ncu capture of the 36-view case)
    times this launch's segments, over the issue rate of all schedulers
    (one warp-instruction per cycle each) at the sampled SM clock."""
    prof = ncu_issue(kernel)
    if not prof:
        return None
    per_seg = prof["warp_inst"] / prof["segments"]
    inst = per_seg * segments
    roof_ms = 1000.0 * inst / (n_sms * schedulers * sm_mhz * 1e6)
    return {"issue_active_pct": prof["issue_active_pct"], "warp_inst_per_segment": per_seg,
            "lanes_per_inst": prof["lanes_per_inst"], "lane_inst_per_segment": per_seg * prof["lanes_per_inst"],
            "warp_inst_per_launch": inst, "issue_roof_ms": roof_ms, "frac": roof_ms / ms,
            "sm_mhz": sm_mhz, "source": "profiles/" + ISSUE_PROFILE + " (36-view case, scaled by segments)"}


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (C restatement of the reference's OpenMP kernel).
# One method everywhere: after an untimed warm-up run, a timing is the best of
# several runs of one projection + one backprojection of the sample on all
# host threads, float32 (the benchmark's precision) unless stated; float64
# (the reference's precision of record) is timed beside it.  The bench line's
# cpu_baseline is the reference arm itself, run in a fresh process.

CPU_REPEATS = 3
_CPU_CACHE = {}


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_model():
    """Host CPU model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def _cpu_geometry(name):
    import numpy as np

    from tomograpy_gb300 import synthetic
    if name not in _CPU_CACHE:
        ch, vh = synthetic.make_geometry(name)
        if name == "frames128":
            cfg = synthetic.CONFIGS[name]
            x = synthetic.phantom4d(ch, cfg["n_frames"], seed=0)
        else:
            x = synthetic.phantom(ch, seed=0)
        _CPU_CACHE[name] = (ch, vh, np.ascontiguousarray(x))
    return _CPU_CACHE[name]


def _cpu_pair(ch, vh, x, dtype, threads):
    """Seconds of one oracle projection + backprojection of views vh."""
    import numpy as np

    import oracle
    from tomograpy_gb300.infoarray import InfoArray
    N1, N2 = int(vh[0]["NAXIS1"]), int(vh[0]["NAXIS2"])
    data = InfoArray(shape=(N1, N2, len(vh)), header=[dict(h) for h in vh], dtype=dtype)
    cube = InfoArray(data=x.astype(dtype), header=dict(ch))
    bcube = InfoArray(shape=x.shape, header=dict(ch), dtype=dtype)
    t0 = time.perf_counter()
    oracle.projector(data, cube, obstacle="sun", nthread=threads)
    oracle.backprojector(data, bcube, obstacle="sun", nthread=threads)
    return time.perf_counter() - t0


def cpu_time(name, dtype="float32", n_views=None, threads=None, repeats=CPU_REPEATS):
    """(best seconds, rays) of the pj + bpj pair of workload ``name`` on the
    oracle: every view, or ``n_views`` of them spread over the orbit.  The
    time-dependent workload runs frame by frame (each frame's views against
    its own 3-D cube: the same rays and voxels as the 4-D call)."""
    import numpy as np
    threads = threads or host_threads()
    ch, vh, x = _cpu_geometry(name)
    if n_views is not None:
        idx = np.linspace(0, len(vh) - 1, n_views).round().astype(int)
        vh = [vh[i] for i in idx]
    rays = int(vh[0]["NAXIS1"]) * int(vh[0]["NAXIS2"]) * len(vh)
    best = None
    for _ in range(repeats):
        if x.ndim == 4:
            F = x.shape[3]
            per = len(vh) // F
            ch3 = dict(ch, NAXIS=3)
            dt = sum(_cpu_pair(ch3, vh[f * per:(f + 1) * per], x[..., f], dtype, threads) for f in range(F))
        else:
            dt = _cpu_pair(ch, vh, x, dtype, threads)
        best = dt if best is None else min(best, dt)
    return best, rays


def cpu_other(threads):
    """CPU timings beside the headline baseline: the float64 sample of the
    headline workload and the full-size plain (64^3 x 60 x 128^2) and
    time-dependent (128^3 x 28 frames, 784 x 256^2) workloads, float32 and
    float64 (one untimed warm-up run each, then the best of the repeats)."""
    other = {}
    cpu_time(WORKLOAD, "float64", CPU_SAMPLE_VIEWS, threads, repeats=1)
    dt64, rays = cpu_time(WORKLOAD, "float64", CPU_SAMPLE_VIEWS, threads)
    other["recon256_sample_f64"] = {"value": rays / dt64, "unit": UNIT, "seconds": dt64, "rays": rays,
                                    "repeats": CPU_REPEATS}
    for name, reps in (("plain64", CPU_REPEATS), ("frames128", 1)):
        for dtype in ("float32", "float64"):
            cpu_time(name, dtype, None, threads, repeats=1)
            t, r = cpu_time(name, dtype, None, threads, repeats=reps)
            other["%s_full_%s" % (name, "f32" if dtype == "float32" else "f64")] = {
                "value": r / t, "unit": UNIT, "seconds": t, "rays": r, "repeats": reps}
    return other


def _bench_subprocess(extra):
    """Run this script in a fresh process (no CUDA context, nothing else on
    the host threads) and return its last JSON line."""
    out = subprocess.run([sys.executable, os.path.abspath(__file__)] + extra, capture_output=True, text=True,
                         env=dict(os.environ, RANK="0", WORLD_SIZE="1"), timeout=1800)
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    if out.returncode != 0 or not lines:
        raise RuntimeError("CPU baseline subprocess failed: %s" % out.stderr[-500:])
    return json.loads(lines[-1])


def cpu_baseline(args):
    """The bench line's CPU baseline: exactly the reference arm
    (``--impl reference`` with the same --steps / --warmup, in a fresh
    process), so the two agree by construction, plus cpu_other()."""
    ref = _bench_subprocess(["--impl", "reference", "--steps", str(args.steps), "--warmup", str(args.warmup)])
    entry = dict(ref["cpu_baseline"])
    entry["ms_per_step"] = ref["ms_per_step"]
    entry["other"] = _bench_subprocess(["--cpu-other"])
    return entry


def run_reference(args):
    """The reference algorithm's CPU path (the oracle port, float32, all host
    threads): each step is one projection + backprojection of the fixed
    16-view sample of the headline workload; the value is the best step,
    the same method as the bench line's cpu_baseline."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = host_threads()
    for _ in range(max(1, args.warmup)):
        cpu_time(WORKLOAD, "float32", CPU_SAMPLE_VIEWS, threads, repeats=1)
    times = []
    rays = None
    for _ in range(args.steps):
        dt, rays = cpu_time(WORKLOAD, "float32", CPU_SAMPLE_VIEWS, threads, repeats=1)
        times.append(dt)
    best = min(times)
    value = rays / best
    sample = ("oracle float32 (C/OpenMP restatement of tomograpy/C_siddon.c.template), %d of 360 views "
              "(%d rays) per step, projection + backprojection, best of %d steps, %d threads of %s"
              % (CPU_SAMPLE_VIEWS, rays, args.steps, threads, cpu_model()))
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * best,
        "ms_per_step_mean": 1000.0 * statistics.mean(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "description": WORKLOAD_DESC, "sample_views": CPU_SAMPLE_VIEWS,
                   "parallelism": "host threads (OpenMP over views)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                         "cpu_model": cpu_model()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


# ---------------------------------------------------------------------------
# our path

def run_ours(args):
    import numpy as np
    import torch
    import torch.distributed as dist

    from tomograpy_gb300 import lo_wrapper, siddon, synthetic

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    # CPU baseline first (host threads only; no GPU context yet)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = guarded(cpu_baseline, args)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    cfg = synthetic.CONFIGS[WORKLOAD]
    n, T, N = cfg["n"], cfg["T"], cfg["N"]
    ch, vh = synthetic.make_geometry(WORKLOAD)
    x = torch.from_numpy(synthetic.phantom(ch, seed=0)).to(dev)
    views = siddon.upload_views(vh, None, dev)
    mh = siddon.pack_map_header(ch)
    y = torch.zeros((T, N, N), device=dev).permute(1, 2, 0)  # view-major storage, (N1, N2, T) view
    c = torch.zeros((n, n, n), device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, device=dev)
    rays = N * N * T

    # exact intersection count (outside the timed region)
    counts = siddon.segment_counts(views, mh, (n, n, n), N, N, T, obstacle="sun")
    inter = float(counts.sum(dtype=torch.float64))
    hit = float((counts > 0).sum())
    del counts

    def step():
        y.zero_()
        e[0].record()
        siddon.run_device("pj", y, x, views, mh, T, obstacle="sun")
        e[1].record()
        c.zero_()
        e[2].record()
        siddon.run_device("bpj", y, c, views, mh, T, obstacle="sun")
        e[3].record()

    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    for _ in range(args.warmup):
        flush.fill_(1.0)
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    props = torch.cuda.get_device_properties(dev)
    clocks = Clocks(str(getattr(props, "uuid", "")) or None)
    clocks.start()
    time.sleep(0.3)
    pj_ms, bpj_ms, step_ms = [], [], []
    s0 = torch.cuda.Event(enable_timing=True)
    s1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    for _ in range(args.steps):
        flush.fill_(1.0)  # L2 flush between steps (not timed)
        s0.record()
        step()
        s1.record()
        torch.cuda.synchronize()
        pj_ms.append(e[0].elapsed_time(e[1]))
        bpj_ms.append(e[2].elapsed_time(e[3]))
        step_ms.append(s0.elapsed_time(s1))
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    ms = slowest_rank_ms(statistics.mean(step_ms), world, dev)
    value = replica_throughput(rays, ms, world)

    # roofline of the dominant kernel (algorithmic bytes per launch / its mean duration)
    peak, peak_kind = measured_peak()
    kern = {
        "siddon_pj_f32": {"ms": statistics.mean(pj_ms), "bytes": 4.0 * inter + 4.0 * hit},
        "siddon_bpj_f32": {"ms": statistics.mean(bpj_ms), "bytes": 8.0 * inter + 4.0 * hit},
    }
    for k in kern.values():
        k["gbs"] = k["bytes"] / (k["ms"] / 1000.0) / 1e9
        k["frac"] = k["gbs"] / peak
    det_ms = deterministic_bpj_ms(y, c, views, mh, T, n, flush, e)
    dom = max(kern, key=lambda k: kern[k]["ms"])
    traffic = ncu_traffic(dom)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": kern[dom]["gbs"], "peak": peak, "unit": "GB/s",
                "frac": kern[dom]["frac"], "traffic": traffic, "peak_kind": peak_kind + " hbm_gbs",
                "algorithmic_bytes_per_launch": kern[dom]["bytes"],
                "note": "the 64 MiB cube is L2-resident, so DRAM moves ~2% of the algorithmic bytes (traffic); "
                        "the binding roof is instruction issue (issue)",
                "issue": issue_roofline(dom, inter, kern[dom]["ms"], (clk or {}).get("sm_mhz") or 2070.0)}
    kern_issue = {k: issue_roofline(k, inter, v["ms"], (clk or {}).get("sm_mhz") or 2070.0) for k, v in kern.items()}

    # end to end through the public operator API with pinned host buffers
    e2e = None
    if not args.no_e2e:
        op = lo_wrapper.siddon_lo(vh, ch, obstacle="sun", dtype=np.float32, device=dev)
        xh = x.cpu().pin_memory()
        # view-major pinned stack (the layout of the device path): the kernels
        # write / read it in place over the host link
        yh = torch.empty((T, N, N), dtype=torch.float32).pin_memory().permute(1, 2, 0)
        chost = torch.empty((n, n, n), dtype=torch.float32).pin_memory()
        for _ in range(max(1, args.warmup)):
            op.project(xh, out=yh)
            op.backproject(yh, out=chost)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            op.project(xh, out=yh)
            op.backproject(yh, out=chost)
        torch.cuda.synchronize()
        e2e_ms = 1000.0 * (time.perf_counter() - t0) / args.steps
        vol = n * n * n * 4
        img = N * N * T * 4
        e2e = {"value": world * rays / (e2e_ms / 1000.0), "unit": UNIT, "ms_per_step": e2e_ms,
               "h2d_bytes_per_step": vol + img, "d2h_bytes_per_step": img + vol,
               "path": "lo_wrapper.siddon_lo project/backproject, pinned host tensors: the cube copied in and out, "
                       "the view-major data stack written and read by the kernels in place over the host link"}
        e2e["drop_in_numpy"] = guarded(drop_in_numpy_rate, ch, vh, x.cpu().numpy(), rays, reps=2)

    batched = served = four_d = lbfgs = None
    if rank == 0 and not args.no_lbfgs:
        lbfgs = guarded(measure_lbfgs, dev)
    if rank == 0 and not args.no_4d:
        four_d = guarded(measure_4d, dev)
    full_rate = inter / (ms / 1000.0)   # segments per second through a pj + bpj pair, fully loaded
    if rank == 0 and not args.no_batched:
        batched = guarded(measure_batched, dev, full_rate=full_rate)
        if "error" not in batched:
            batched["small_jobs"] = guarded(measure_batched, dev, n_jobs=256, mix=SMALL_MIX, full_rate=full_rate)
    if rank == 0 and not args.no_served:
        served = guarded(measure_served, dev, args.served_jobs, full_rate=full_rate)
        if "error" not in served:
            served["small_jobs"] = guarded(measure_served, dev, 500, rate=4000.0, mix=SMALL_MIX, large=0.0,
                                           pool=500, full_rate=full_rate)

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "description": WORKLOAD_DESC, "rays_per_step": rays,
                       "intersections_per_step": inter, "hit_rays_per_step": hit,
                       "l2": "flushed between steps (256 MiB write, untimed)", "parallelism": "replicas"},
            "intersections_per_s": world * inter * 2 / (ms / 1000.0),
            "kernels": dict({k: {"ms": v["ms"], "GB_s": v["gbs"], "frac": v["frac"],
                                 "issue_frac": (kern_issue[k] or {}).get("frac")} for k, v in kern.items()},
                            siddon_bpj_f32_deterministic={"ms": det_ms}),
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": 2 * args.steps,
            "clocks": clk,
            "lbfgs": lbfgs,
            "four_d": four_d,
            "batched": batched,
            "served": served,
        }
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


def guarded(fn, *a, **kw):
    """Run a secondary measurement; a failure is reported in its entry (the
    headline line is printed whatever happens to the secondary ones)."""
    try:
        return fn(*a, **kw)
    except Exception as e:  # noqa: BLE001 - reported, not hidden
        print("bench: %s failed: %r" % (fn.__name__, e), file=sys.stderr)
        return {"error": "%s: %s" % (type(e).__name__, e)}


def drop_in_numpy_rate(ch, vh, x, rays, reps=2):
    """The reference's own call pattern: tomograpy.projector(data, cube) then
    tomograpy.backprojector(data, cube) on NumPy arrays with headers (each
    call stages its arrays through the GPU and writes back in place)."""
    import numpy as np

    import tomograpy_gb300 as tgp
    from tomograpy_gb300.infoarray import InfoArray
    N, T = int(vh[0]["NAXIS1"]), len(vh)
    data = InfoArray(shape=(N, N, T), header=[dict(h) for h in vh], dtype=np.float32)
    cube = InfoArray(data=x, header=dict(ch))
    back = InfoArray(shape=x.shape, header=dict(ch), dtype=np.float32)
    tgp.projector(data, cube, obstacle="sun")
    tgp.backprojector(data, back, obstacle="sun")
    t0 = time.perf_counter()
    for _ in range(reps):
        data[...] = 0
        back[...] = 0
        tgp.projector(data, cube, obstacle="sun")
        tgp.backprojector(data, back, obstacle="sun")
    ms = 1000.0 * (time.perf_counter() - t0) / reps
    return {"value": rays / (ms / 1000.0), "unit": UNIT, "ms_per_step": ms,
            "path": "tomograpy_gb300.projector / backprojector on NumPy arrays (pageable host memory)"}


def deterministic_bpj_ms(y, c, views, mh, T, n, flush, e, reps=3):
    """Mean time of the deterministic (int64 fixed-point) backprojection of the
    workload's data stack (outside the headline step)."""
    import torch

    from tomograpy_gb300 import _lib, siddon
    need = _lib.load().tg_deterministic_workspace_bytes(_lib.i64([n, n, n, 1]))
    ws = torch.empty(need, dtype=torch.uint8, device=c.device)
    ts = []
    for r in range(reps + 1):
        flush.fill_(1.0)
        c.zero_()
        e[0].record()
        siddon.run_device("bpj", y, c, views, mh, T, obstacle="sun", deterministic=True, workspace=ws)
        e[1].record()
        torch.cuda.synchronize()
        if r:
            ts.append(e[0].elapsed_time(e[1]))
    return statistics.mean(ts)


def measure_lbfgs(dev, iters=50):
    """Differentiable reconstruction on the benchmark geometry: L-BFGS on
    0.5 |P x - y|^2 / |y|^2 + 1e-3 TV_eps(x) with x = s softplus(z), the
    projector as a torch.autograd.Function whose backward is the
    backprojector; y = P(phantom) with Poisson noise at 1e4 counts peak."""
    import numpy as np
    import torch

    from tomograpy_gb300 import autograd, lo_wrapper, synthetic
    ch, vh = synthetic.make_geometry(WORKLOAD)
    op = lo_wrapper.siddon_lo(vh, ch, obstacle="sun", dtype=np.float32, device=dev)
    x = torch.from_numpy(synthetic.phantom(ch, seed=0) / np.float32(1e8)).to(dev)
    y = op.project(x)
    y = torch.from_numpy(synthetic.poisson_noise(y.cpu().numpy())).to(dev)
    autograd.reconstruct_lbfgs(op, y, iters=1)          # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    xr, losses = autograd.reconstruct_lbfgs(op, y, iters=iters)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    return {"workload": "256^3 x 360 x 512^2, sun, L-BFGS (strong Wolfe) with TV 1e-3 and softplus positivity",
            "iterations": iters, "loss_evaluations": len(losses), "seconds": dt,
            "s_per_evaluation": dt / max(1, len(losses)), "loss_first": losses[0], "loss_last": losses[-1]}


def measure_4d(dev, reps=5, cg_iters=30):
    """Time-dependent workload: 128^3 x 28-frame cube (frame-major), 784 views
    of 256^2 over 0-360 deg, view v -> frame v // 28, sun; projection +
    backprojection rays/s (L2 flushed between steps), and 30 CG iterations on
    (P^T P + 1e-2 I + 1e-2 D_t^T D_t) x = P^T y through the 4-D operator."""
    import numpy as np
    import torch

    from tomograpy_gb300 import cg, lo_wrapper, siddon, synthetic
    cfg = synthetic.CONFIGS["frames128"]
    n, T, N, F = cfg["n"], cfg["T"], cfg["N"], cfg["n_frames"]
    ch, vh = synthetic.make_geometry("frames128")
    frames = np.arange(T) // (T // F)
    views = siddon.upload_views(vh, frames, dev)
    mh = siddon.pack_map_header(ch)
    x4 = synthetic.phantom4d(ch, F, seed=0)                       # (n, n, n, F)
    x = torch.empty((F, n, n, n), device=dev).permute(1, 2, 3, 0)  # frame-major storage
    x.copy_(torch.from_numpy(x4))
    c = torch.zeros_like(x)
    y = torch.zeros((T, N, N), device=dev).permute(1, 2, 0)
    flush = torch.empty(L2_FLUSH_BYTES // 4, device=dev)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    pj, bpj = [], []
    for r in range(reps + 2):
        flush.fill_(1.0)
        y.zero_()
        c.zero_()
        e[0].record()
        siddon.run_device("pjt", y, x, views, mh, T, obstacle="sun")
        e[1].record()
        flush.fill_(1.0)
        e[2].record()
        siddon.run_device("bpjt", y, c, views, mh, T, obstacle="sun")
        e[3].record()
        torch.cuda.synchronize()
        if r >= 2:
            pj.append(e[0].elapsed_time(e[1]))
            bpj.append(e[2].elapsed_time(e[3]))
    rays = N * N * T
    P = lo_wrapper.siddon4d_lo(vh, ch, ng=T // F, obstacle="sun", dtype=np.float32, device=dev)
    b = P.backproject(y.contiguous())
    A = cg.NormalOperator(P, lam=1e-2, temporal=1e-2)
    cg.cg(A, b, maxiter=2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = cg.cg(A, b, maxiter=cg_iters)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    return {"workload": "128^3 x 28 frames (frame-major), 784 views of 256^2 over 0-360 deg, view -> frame v // 28, sun",
            "rays_per_step": rays, "pjt_ms": statistics.mean(pj), "bpjt_ms": statistics.mean(bpj),
            "rays_per_s": rays / ((statistics.mean(pj) + statistics.mean(bpj)) / 1000.0),
            "cg": {"iterations": cg_iters, "it_per_s": cg_iters / dt, "seconds": dt,
                   "terms": "P^T P + 1e-2 I + 1e-2 D_t^T D_t (4-D operator, frame-major cube)",
                   "relative_residual": res.residuals[-1]}}


SERVE_BUDGET = 48 << 30   # device memory the serving measurement may keep resident
SMALL_MIX = dict(edges=(16, 24, 32, 48), sides=(32, 48, 64), views=(8, 32))


def job_segments(job, dev):
    """Voxel segments one projection of a job traces (the exact count)."""
    import torch

    from tomograpy_gb300 import siddon
    n1, n2, T = job.data_shape
    views = siddon.upload_views(job.view_headers, job.frames, dev)
    c = siddon.segment_counts(views, siddon.pack_map_header(job.cube_header), job.cube_shape[:3], n1, n2, T,
                              obstacle="sun")
    return float(c.sum(dtype=torch.float64))


def measure_batched(dev, n_jobs=32, iters=20, seed=0, mix=None, full_rate=None):
    """Uneven multi-job batch: 32 seeded reconstructions (cube edge in
    {32..192}, 16-256 views of 64-512 px, d in [150, 230]; or the sizes of
    `mix`), 20 CG iterations on (P^T P + 1e-2 I) x = P^T y each, solved (a)
    together with one packed launch per direction per iteration, CUDA-graph
    captured, tile shape autotuned, and (b) one after another with the
    single-job operator.  Also: the same with fixed-point backprojections
    (every job's iterate then bitwise the plain loop's), and the ceiling of
    any batching: plain time / the time of the batch's voxel segments at the
    fully loaded rate of the headline workload (``full_rate``, segments per
    second through a projection + backprojection pair)."""
    import torch

    from tomograpy_gb300 import batch, synthetic
    specs = synthetic.uneven_specs(n_jobs, seed=seed, **(mix or {}))
    jobs = [synthetic.make_job(s, seed=k) for k, s in enumerate(specs)]
    pack = batch.PackedJobs(jobs, obstacle="sun", device=dev)
    x = pack.new_cube()
    for k, j in enumerate(jobs):
        pack.cube_view(x, k).copy_(torch.from_numpy(j.phantom))
    pack.project(x)
    b = pack.backproject(pack.new_cube())
    rhs = [pack.cube_view(b, k).clone() for k in range(n_jobs)]
    batch.batched_cg(pack, b, iters=2)          # warm-up (graph capture path)
    batch.sequential_cg(jobs[:2], rhs[:2], iters=2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    xb, _ = batch.batched_cg(pack, b, iters=iters)
    torch.cuda.synchronize()
    tb = time.perf_counter() - t0
    t0 = time.perf_counter()
    xs = batch.sequential_cg(jobs, rhs, iters=iters)
    torch.cuda.synchronize()
    ts = time.perf_counter() - t0
    diff = max(float((pack.cube_view(xb, k) - xs[k]).abs().max() / xs[k].abs().max().clamp_min(1e-30))
               for k in range(n_jobs))
    # deterministic mode: bitwise isolation at the full iteration count
    batch.batched_cg(pack, b, iters=2, deterministic=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    xd, _ = batch.batched_cg(pack, b, iters=iters, deterministic=True)
    torch.cuda.synchronize()
    tbd = time.perf_counter() - t0
    t0 = time.perf_counter()
    xsd = batch.sequential_cg(jobs, rhs, iters=iters, deterministic=True)
    torch.cuda.synchronize()
    tsd = time.perf_counter() - t0
    bitwise = all(torch.equal(pack.cube_view(xd, k), xsd[k]) for k in range(n_jobs))
    rays = sum(int(j.data_shape[0] * j.data_shape[1] * j.data_shape[2]) for j in jobs)
    table = pack.tune_table or {}
    default = batch.DEFAULT_SCHEDULE
    out = {"rays_per_iteration": rays, "rows_per_warp": pack.rows_per_warp,
           "schedule": {"rows_per_warp": pack.schedule[0], "lane_axis": "lambda" if pack.schedule[1] else "gamma",
                        "batch_steps": pack.schedule[2] or "default",
                        "autotune_s_per_pj_bpj": {"%d/%s/%s" % (k[0], "lambda" if k[1] else "gamma", k[2] or "default"):
                                                  v for k, v in table.items()},
                        "gain_over_default": (table[default] / table[pack.schedule]
                                              if default in table and pack.schedule in table else None)},
           "batched_cg_it_per_s": n_jobs * iters / tb, "plain_cg_it_per_s": n_jobs * iters / ts,
           "speedup": ts / tb, "batched_s": tb, "plain_s": ts, "max_rel_diff_vs_plain": diff,
           "deterministic": {"batched_cg_it_per_s": n_jobs * iters / tbd, "plain_cg_it_per_s": n_jobs * iters / tsd,
                             "speedup": tsd / tbd, "bitwise_equal_to_plain": bitwise},
           "plain": "one job after another: single-job operator + the same CG kernels (no graph)"}
    if full_rate:
        segs = sum(job_segments(j, dev) for j in jobs)
        t_lb = iters * segs / full_rate
        out["ceiling"] = {"segments_per_iteration": segs, "lower_bound_s": t_lb, "speedup_ceiling": ts / t_lb,
                          "how": "plain time / (iterations x segments / fully loaded segment rate of the "
                                 "headline projection + backprojection pair)"}
    sizes = ("edges %s, %d-%d views, %s px" % (mix["edges"], mix["views"][0], mix["views"][1], mix["sides"])
             if mix else "edges 32-192, 16-256 views, 64-512 px")
    out["workload"] = "uneven batch: %d seeded jobs (%s), %d CG iterations, sun" % (n_jobs, sizes, iters)
    return out


def serving_payloads(dev, seed, mix, large, pool):
    """The stream's distinct request payloads (geometry + pinned host data
    stack P(phantom)): ``pool`` seeded draws of the uneven-batch sizes (or
    ``mix``), plus one 256^3 x 360 x 512^2 job when ``large`` > 0."""
    from tomograpy_gb300 import serve, synthetic
    specs = synthetic.uneven_specs(pool, seed=seed + 1, **(mix or {}))
    small = serve.poisson_requests(specs, rate=1.0, seed=seed, max_iters=20, tol=1e-4, device=dev)
    big = None
    if large > 0:
        big = serve.poisson_requests([dict(synthetic.CONFIGS["recon256"])], rate=1.0, seed=seed, max_iters=20,
                                     tol=1e-4, device=dev)[0]
    return small, big


def serving_requests(dev, n_jobs, rate, seed, mix, large, pool, payloads=None):
    """Poisson arrivals of ``n_jobs`` requests at ``rate`` jobs/s (seeded).
    Sizes: a fraction ``large`` of 256^3 x 360 x 512^2 jobs, the others drawn
    from ``pool`` seeded draws of the uneven-batch distribution (or ``mix``);
    requests that draw the same entry share its geometry and host data stack,
    which keeps the stream's host memory bounded."""
    import numpy as np

    from tomograpy_gb300 import serve
    small, big = payloads or serving_payloads(dev, seed, mix, large, pool)
    rng = np.random.default_rng(seed + 99)
    t = 0.0
    reqs = []
    for k in range(n_jobs):
        t += rng.exponential(1.0 / rate)
        src = big if (big is not None and rng.random() < large) else small[int(rng.integers(pool))]
        reqs.append(serve.Request(k, src.job, src.data, t, max_iters=20, tol=1e-4))
    return reqs, (small, big)


def measure_served(dev, n_jobs=2000, rate=20.0, seed=0, mix=None, large=0.1, pool=64, full_rate=None):
    """Serving stream: Poisson arrivals (20 jobs/s, seeded) of requests sized
    as the uneven batch (or `mix`) plus a fraction `large` of 256^3 x 360 x
    512^2 jobs, 20 CG iterations or relative residual 1e-4 each; continuous
    batching vs a FIFO plain loop on the same requests."""
    import numpy as np

    from tomograpy_gb300 import serve
    # warm-up (untimed): the first launches of every kernel variant and the
    # first pinned allocations of a process would otherwise land in the stream
    warm, _ = serving_requests(dev, 8, 1e6, seed, mix, 0.0, min(pool, 8))
    for r in warm:
        r.max_iters = 3
    serve.Server(budget_bytes=8 << 30, device=dev).run(warm)
    warm, _ = serving_requests(dev, 8, 1e6, seed, mix, 0.0, min(pool, 8))
    for r in warm:
        r.max_iters = 3
    serve.fifo_plain(warm, device=dev)
    # results are delivered to the host for every request; every 20th is kept
    # for the comparison of the two arms (bounded host memory)
    keep = set(range(0, n_jobs, 20))

    def done(r):
        if r.id not in keep:
            r.result = None
    reqs, payloads = serving_requests(dev, n_jobs, rate, seed, mix, large, pool)
    srv = serve.Server(budget_bytes=SERVE_BUDGET, device=dev, on_done=done)
    s = srv.run(reqs)
    reqs2, _ = serving_requests(dev, n_jobs, rate, seed, mix, large, pool, payloads)
    f = serve.fifo_plain(reqs2, device=dev, on_done=done)
    diff = max(float((reqs[k].result - reqs2[k].result).abs().max() /
                     reqs2[k].result.abs().max().clamp_min(1e-30)) for k in sorted(keep))
    out = {"served": s, "fifo_plain": f, "cg_it_per_s_ratio": s["cg_it_per_s"] / f["cg_it_per_s"],
           "p99_ratio": s["p99_s"] / f["p99_s"], "max_inflight": srv.max_inflight, "max_rel_diff_vs_plain": diff,
           "budget_bytes": SERVE_BUDGET, "server_host_s": srv.host_s, "server_rebuilds": srv.rebuilds,
           "large_requests": int(sum(r.job is payloads[1].job for r in reqs)) if large > 0 else 0}
    if full_rate:
        segs = {id(p.job): job_segments(p.job, dev) for p in payloads[0] + ([payloads[1]] if payloads[1] else [])}
        t_lb = sum(r.iters * segs[id(r.job)] for r in reqs2) / full_rate
        out["ceiling"] = {"lower_bound_s": t_lb, "cg_it_per_s_ceiling": f["wall_s"] / t_lb,
                          "how": "FIFO wall time / (the FIFO jobs' iterations x segments at the fully loaded "
                                 "segment rate of the headline pair); meaningful when arrivals outpace the GPU"}
    sizes = ("small uneven sizes (edges %s, %d-%d views, %s px)" % (mix["edges"], mix["views"][0], mix["views"][1],
                                                                      mix["sides"]) if mix else "uneven sizes")
    out["workload"] = ("serving stream: %d Poisson requests at %.0f jobs/s, %s from %d seeded draws + %d%% "
                       "256^3 x 360 x 512^2, 20 CG iterations or residual 1e-4" % (n_jobs, rate, sizes, pool,
                                                                                  round(100 * large)))
    return out


def run_profile_case():
    import torch

    from tomograpy_gb300 import siddon, synthetic
    cfg = synthetic.CONFIGS[WORKLOAD]
    ch, vh = synthetic.make_geometry(WORKLOAD)
    vh = vh[::10]
    T, N, n = len(vh), cfg["N"], cfg["n"]
    dev = torch.device("cuda")
    x = torch.from_numpy(synthetic.phantom(ch, seed=0)).to(dev)
    views = siddon.upload_views(vh, None, dev)
    mh = siddon.pack_map_header(ch)
    y = torch.zeros((T, N, N), device=dev).permute(1, 2, 0)
    c = torch.zeros((n, n, n), device=dev)
    siddon.run_device("pj", y, x, views, mh, T, obstacle="sun")
    siddon.run_device("bpj", y, c, views, mh, T, obstacle="sun")
    torch.cuda.synchronize()
    segments = float(siddon.segment_counts(views, mh, (n, n, n), N, N, T, obstacle="sun").sum(dtype=torch.float64))
    print(json.dumps({"profile_case": WORKLOAD, "views": T, "segments": segments, "y_sum": float(y.sum()),
                      "c_sum": float(c.sum())}))


def run_profile_packed():
    import torch

    from tomograpy_gb300 import batch, synthetic
    jobs = [synthetic.make_job(sp, seed=k) for k, sp in enumerate(synthetic.uneven_specs(32, seed=0))]
    pack = batch.PackedJobs(jobs, obstacle="sun", rows_per_warp=4)
    x = pack.new_cube()
    for k, j in enumerate(jobs):
        pack.cube_view(x, k).copy_(torch.from_numpy(j.phantom))
    pack.project(x)
    z = pack.backproject(pack.new_cube())
    torch.cuda.synchronize()
    print(json.dumps({"profile_packed": 32, "rays": int(pack.data.numel()), "y_sum": float(pack.data.sum()),
                      "c_sum": float(z.sum())}))


def main():
    args = parse()
    if args.profile_case:
        run_profile_case()
        return
    if args.profile_packed:
        run_profile_packed()
        return
    if args.cpu_other:
        print(json.dumps(cpu_other(host_threads())))
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
