"""Benchmark: the plain full-quality single frame (1920x1080 output at supersample 2, so a
3840x2160 bin grid; 1000 points per bin, 8,294,400,000 points per frame; synthetic genome seed 1
with 8 xforms plus a final xform; adaptive DE radius 9, min 0, curve 0.4; log-density tonemap).

A step is one frame: warmup (20 discarded passes), the chaos game over all walkers until the
frame's points are drawn, density estimation, tonemap.  A point is one post-fuse walker-step;
`binned_gpoints_s` counts the points that land in the frame.  Walkers that leave the plane
(NaN / beyond 1e10) restart, as the reference's commented-out reset at flame.glsl:68 would do
(--no-badval-reset keeps the reference's default, where they stay lost and over the frame's
3,331 passes most of them stop drawing).  `value` is points per second with the genome and all
buffers resident in HBM; `e2e` is the same frame through the C ABI's rf_render from a host
genome to a pinned host RGBA8 image (upload and read-back inside the timed region).

Genomes come from tests/golden/genomes/ (written once by tests/golden/make_genomes.py from the
library's seeded synthesiser), so the reference arm reads the same genome without the library.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl native|reference]

With N > 1 (torchrun) every rank renders an independent replica (its own seed); value is the
points of all ranks over the slowest rank's time.  --impl reference times the reference's path
as restated on the CPU (the reference has no CPU path of its own; the oracle port of
flame.glsl's iteration, all host threads) on a bounded sample of the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Workloads.  The default (`frame1080`) is the headline: the full-quality 1080p frame.  The
# others are the small CPU-runnable genome and the two atomic-contention / histogram-size stress
# genomes, measured the same way (chaos game only where no image is asked for).
WORKLOADS = {
    "frame1080": dict(name="plain 1080p frame, supersample 2 (3840x2160 bins), 1000 points/bin, DE r9 c0.4",
                      genome=dict(kind=1, seed=1, n_xforms=8, final_xform=True, force_parametric=True),
                      genome_file="frame1080.flam3",
                      out=(1920, 1080), ss=2, points=1000 * 3840 * 2160, de=(9, 0, 0.4), image=True),
    "small": dict(name="small genome (seed 0, 3 xforms), 512x512 bins, 65,536 walkers x 256 passes",
                  genome=dict(kind=0, seed=0, n_xforms=0, final_xform=False, force_parametric=False),
                  genome_file="small.flam3",
                  out=(512, 512), ss=1, points=65536 * 256, de=None, image=True, walkers=65536,
                  cta_slots=2048),  # 65,536 walkers fill only 16 CTAs of 4096 slots
    "contract": dict(name="contracting genome (seed 4, 6 xforms), 1920x1080 bins, 2^34 points",
                     genome=dict(kind=2, seed=4, n_xforms=0, final_xform=False, force_parametric=False),
                     genome_file="contract.flam3",
                     out=(1920, 1080), ss=1, points=2 ** 34, de=None, image=False),
    # (AUTO splat: the library fits a shared-memory tile over the attractor's hottest bins)
    "spacefill": dict(name="space-filling genome (seed 5, 16 xforms), 8192x8192 bins, 2^34 points",
                      genome=dict(kind=3, seed=5, n_xforms=0, final_xform=False, force_parametric=False),
                      genome_file="spacefill.flam3",
                      out=(4096, 4096), ss=2, points=2 ** 34, de=None, image=False),
    "batch": dict(name="batched animation: 120 frames interpolated seed 2 (4 xforms) -> seed 3 (10 xforms) at "
                       "1024x768 + 64 random genomes (2-16 xforms) at 512x512 / 1024x768 / 1920x1080, 200 spp, "
                       "one persistent graph-captured launch",
                  genome=None, genome_file="batch_frame0.flam3",
                  out=(1024, 768), ss=1, points=None, de=(9, 0, 0.4), image=True),
    "gemm": dict(name="tcgen05 BF16 GEMM of the learned density estimator: 8192^3 (FP32 accumulation) and the "
                      "U-Net's largest convolution (1,048,576 x 32 x 720) as a GEMM and as an implicit GEMM",
                 genome=None, out=(512, 512), ss=1, points=None, de=None, image=False),
    "learned": dict(name="learned density estimation: U-Net (32-48-64-96, BF16 on tcgen05) trained on 2000 genomes "
                         "(seeds 1000-2999, 2-12 xforms) at 512x512, 16 spp -> 1000-spp adaptive-DE target; 200 "
                         "held-out genomes; 1080p frame time, learned vs plain",
                    genome=None, out=(1920, 1080), ss=1, points=None, de=(9, 0, 0.4), image=True),
}
FUSE = 20
GENOME_DIR = os.path.join(ROOT, "tests", "golden", "genomes")
BATCH_SIZES = [(512, 512), (1024, 768), (1920, 1080)]
BATCH_POINTS = 120 * 200 * 1024 * 768 + sum(200 * BATCH_SIZES[k % 3][0] * BATCH_SIZES[k % 3][1] for k in range(64))
WL = WORKLOADS["frame1080"]
W_OUT, H_OUT = WL["out"]
SS = WL["ss"]
W, H = W_OUT * SS, H_OUT * SS
POINTS = WL["points"]
DE = WL["de"]
GENOME = WL["genome"]
CONFIG_NAME = WL["name"]


def select_workload(key):
    global WL, W_OUT, H_OUT, SS, W, H, POINTS, DE, GENOME, CONFIG_NAME
    WL = WORKLOADS[key]
    W_OUT, H_OUT = WL["out"]
    SS = WL["ss"]
    W, H = W_OUT * SS, H_OUT * SS
    POINTS = WL["points"]
    DE = WL["de"]
    GENOME = WL["genome"]
    CONFIG_NAME = WL["name"]


def genome_xml():
    """The workload's genome (flam3 XML) as committed under tests/golden/genomes/."""
    with open(os.path.join(GENOME_DIR, WL["genome_file"])) as f:
        return f.read()


def workload_config(reset):
    """The workload's definition — identical in the native and the reference arm's line (what
    each run chose at run time goes to the line's `launch`)."""
    if WL["genome"] is None:  # the batched animation
        return {"workload": CONFIG_NAME, "images": 184, "requested_points": BATCH_POINTS,
                "genome_file": WL["genome_file"], "density_estimation": list(DE), "fuse_passes": FUSE,
                "bad_value_reset": bool(reset),
                "l2": "%.1f GB of bins per batch (L2 129 MB)" %
                      ((120 * 1024 * 768 + sum(BATCH_SIZES[k % 3][0] * BATCH_SIZES[k % 3][1] for k in range(64)))
                       * 20 / 1e9)}
    return {"workload": CONFIG_NAME, "genome": GENOME, "genome_file": WL["genome_file"], "points_per_frame": POINTS,
            "bins": [W, H], "output": [W_OUT, H_OUT], "fuse_passes": FUSE,
            "density_estimation": list(DE) if DE else None, "bad_value_reset": bool(reset),
            "l2": "bins %dx%d x 20 B = %.0f MB (L2 129 MB)%s" % (
                W, H, W * H * 20 / 1e6, "; exceed L2" if W * H * 20 > 129e6 else "; an L2 flush separates frames")}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

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
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def slowest_rank_ms(ms):
    """Max of a per-rank duration over all ranks (identity without torch.distributed)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(ms)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(ms)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(points_per_rank, ms_per_step):
    """Whole-job Gpoints/s of independent replicas: every rank's points over the slowest rank's time."""
    import torch.distributed as dist
    ws = dist.get_world_size() if (dist.is_available() and dist.is_initialized()) else 1
    return points_per_rank * ws / (slowest_rank_ms(ms_per_step) * 1e-3) / 1e9


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _profile_figure(workload, key, summary="chaos_kernel_%s.md"):
    """A figure ("<key>: <number>") from the committed ncu summary of this workload (or None)."""
    import re
    try:
        with open(os.path.join(ROOT, "profiles", summary % workload)) as f:
            m = re.search(r"^%s: ([0-9.]+)" % re.escape(key), f.read(), re.M)
        return float(m.group(1)) if m else None
    except OSError:
        return None


def kernel_build_id(flame, variant=""):
    """Identifies the chaos kernel a run launches: a hash of the genome-specialised kernel's
    generated source, the device headers it is compiled from and the launch's compile-time
    choices (`variant`: splat strategy, walker reset, exchange).  The committed ncu summary
    records the id of the build it captured; bench.py uses its figures only when they match."""
    import hashlib
    sys.path.insert(0, os.path.join(ROOT, "refrakt_gb300"))
    from nvbuild import RTC_HEADERS
    h = hashlib.sha256(flame.kernel_source().encode() + variant.encode())
    for name in RTC_HEADERS + ["chaos_body.cuh"]:
        with open(os.path.join(ROOT, "refrakt_gb300", "csrc", name), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def _profile_build(workload):
    """The kernel build id recorded in the committed ncu summary of this workload (or None)."""
    import re
    try:
        with open(os.path.join(ROOT, "profiles", "chaos_kernel_%s.md" % workload)) as f:
            m = re.search(r"^kernel build: ([0-9a-f]+)", f.read(), re.M)
        return m.group(1) if m else None
    except OSError:
        return None


# FP32 operation counts of one evaluation of each variation, from its formula in variations.yaml
# (tests/golden/reference_vectors.json: `libm_calls` = sin, cos, pow, exp, log, atan, sqrt ...
# calls incl. the precalcs it uses; `arith_ops` = +, -, *, / and fused forms in its text).
def _variation_costs():
    try:
        with open(os.path.join(ROOT, "tests", "golden", "reference_vectors.json")) as f:
            g = json.load(f)
        return g.get("libm_calls", {}), g.get("arith_ops", {})
    except OSError:
        return {}, {}


def algorithmic_ops_per_point(xml):
    """Expected FP32 arithmetic operations and library (transcendental) calls per point of a
    genome: each xform's affine (4 FMA), its variations' formulas (weighted by the xform's
    selection probability), colour blend (3), the final xform when present, and the screen
    affine (4 FMA).  Counted from the formulas, not from any implementation."""
    import xml.etree.ElementTree as ET
    libm, arith = _variation_costs()
    root = ET.fromstring(xml)
    if root.tag != "flame":
        root = root.find("flame")
    xfs = root.findall("xform")
    fin = root.find("finalxform")
    tw = sum(float(x.get("weight", "0")) for x in xfs) or 1.0

    def cost(x):
        ops, calls = 4.0 + 3.0, 0.0
        for name, val in x.attrib.items():
            if name in libm and float(val) != 0.0:
                calls += libm[name]
                ops += arith.get(name, 0) + 2  # weight multiply and accumulate
        if x.get("post"):
            ops += 4
        return ops, calls

    ops = calls = 0.0
    for x in xfs:
        o, c = cost(x)
        p = float(x.get("weight", "0")) / tw
        ops += p * o
        calls += p * c
    if fin is not None:
        o, c = cost(fin)
        ops += o
        calls += c
    return ops + 4.0, calls


def splat_tile_capacity(slots):
    """Bins of a shared-memory splat tile that fit beside `slots` walker slots (a 16 KB genome)."""
    used = 3 * slots * 16 + 256 * 16 + 16384 + 2 * (slots // 256) * 4 + 256 * 4 + 16
    return max(0, (232448 - used) // 20)


def fit_splat_tile(hits, capacity):
    """(x0, y0, w, h): the bounding box of the bins a probe histogram hit, or, when that holds more
    than `capacity` bins, the square of that many bins around the most-hit bin."""
    import numpy as np
    ys, xs = np.nonzero(hits)
    if len(xs) == 0 or capacity == 0:
        return (0, 0, 0, 0)
    x0, x1, y0, y1 = int(xs.min()), int(xs.max()), int(ys.min()), int(ys.max())
    if (x1 - x0 + 1) * (y1 - y0 + 1) <= capacity:
        return (x0, y0, x1 - x0 + 1, y1 - y0 + 1)
    side = int(capacity ** 0.5)
    cy, cx = np.unravel_index(int(np.argmax(hits)), hits.shape)
    H, W = hits.shape
    w, h = min(side, W), min(side, H)
    x0 = min(max(0, int(cx) - w // 2), W - w)
    y0 = min(max(0, int(cy) - h // 2), H - h)
    return (x0, y0, w, h)


def _traffic(workload):
    """DRAM bytes per chaos launch from the committed ncu summary of this workload (or None)."""
    v = _profile_figure(workload, "dram bytes per launch")
    return int(v) if v is not None else None


def cpu_baseline(genome_xml, seconds=12.0, threads=None, reset=True):
    """The oracle's FP32 transcription of flame.glsl's draw pass on the host cores, on a bounded
    sample of this workload (same genome, same bin grid, same walker reset): returns (Gpoints/s,
    threads, sample description, seconds timed, binned Gpoints/s)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    g = O.Genome(genome_xml)
    threads = threads or os.cpu_count() or 1
    walkers = 256 * 64 * threads
    t0 = time.perf_counter()
    n, _, _ = g.cpu_baseline(walkers, 2, W, H, threads, badval_reset=reset)
    rate = n / max(time.perf_counter() - t0, 1e-6)
    passes = max(2, int(seconds * rate / walkers))
    t0 = time.perf_counter()
    n, _, _, nb = g.cpu_baseline(walkers, passes, W, H, threads, badval_reset=reset, binned=True)
    dt = time.perf_counter() - t0
    points = POINTS or BATCH_POINTS
    sample = "%d walkers x %d passes = %.3g points of the workload's %.3g, %dx%d bins" % (
        walkers, passes, n, points, W, H)
    return n / dt / 1e9, threads, sample, dt, nb / dt / 1e9


def run_reference(args):
    """The reference's path on the host cores (the oracle's FP32 port of flame.glsl's iteration;
    the reference has no CPU path of its own), on the same genome file and bin grid as the native
    arm.  Each step times one bounded sample of the workload; ms_per_step is that sample's time."""
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    xml = genome_xml()
    reset = not args.no_badval_reset
    vals, binned, dts = [], [], []
    last = None
    for i in range(args.warmup + args.steps):
        v, thr, sample, dt, vb = cpu_baseline(xml, seconds=max(3.0, 30.0 / (args.warmup + args.steps)), reset=reset)
        if i >= args.warmup:
            vals.append(v)
            binned.append(vb)
            dts.append(dt)
        last = (thr, sample)
    v = statistics.median(vals)
    points = POINTS or BATCH_POINTS
    line = {"metric": "Gpoints/s histogrammed", "value": v, "unit": "Gpoints/s", "impl": "reference",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.median(dts) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic genome (%s); no dataset" % WL["genome_file"],
            "config": workload_config(reset),
            "binned_gpoints_s": statistics.median(binned),
            "step": "one bounded sample of the workload per step (%s); the whole workload would take %.1f s "
                    "at this rate" % (last[1], points / (v * 1e9)),
            "cpu_baseline": {"value": v, "unit": "Gpoints/s", "cores": last[0], "kind": "port", "sample": last[1]},
            "e2e": {"value": v, "unit": "Gpoints/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_native(args):
    import numpy as np
    import torch
    import refrakt_gb300 as R

    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    R.build()
    comp = R.FlameCompiler()
    xml = genome_xml()
    flame = R.Flame.from_xml(xml, comp)
    info = flame.info()
    reset = not args.no_badval_reset
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    cta = args.cta_slots or WL.get("cta_slots", 4096)
    walkers = WL.get("walkers") or sms * args.ctas_per_sm * cta
    sim = R.Sim(walkers, cta_slots=cta, cta_threads=args.cta_threads, steps_per_launch=args.steps_per_launch,
                seed=1000 + rank, device=local, specialize={"auto": 0, "on": 1, "off": -1, "all": 0}[args.specialize])
    passes = (POINTS + walkers - 1) // walkers
    launches = (passes + args.steps_per_launch - 1) // args.steps_per_launch
    bins = torch.zeros(H, W, 4, device="cuda")
    hits = torch.zeros(H, W, dtype=torch.int32, device="cuda")
    img = torch.zeros(H_OUT, W_OUT, 4, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    sim.set_stream(stream)
    sim.set_splat({"auto": R.SPLAT_AUTO, "global": R.SPLAT_GLOBAL, "warp": R.SPLAT_WARP,
                   "tile": R.SPLAT_TILE}[args.splat])
    sim.set_bad_value_reset(reset)
    sim.set_exchange({"auto": R.EXCHANGE_AUTO, "pipelined": R.EXCHANGE_PIPELINED,
                      "barrier": R.EXCHANGE_BARRIER}[args.exchange])
    tile = None
    if args.splat == "tile":  # the shared-memory tile: the attractor's bounding box from a short probe
        sim.warmup(flame, FUSE - 1)
        sim.set_splat_tile(0, 0, 0, 0)
        probe = torch.zeros(H, W, dtype=torch.int32, device="cuda")
        sim.draw_to_bins(flame, bins, probe, W, H, 4)
        tile = fit_splat_tile(probe.cpu().numpy(), splat_tile_capacity(cta))
        sim.set_splat_tile(*tile)
        bins.zero_()

    # bins smaller than the 129 MB L2: write a 256 MB buffer before every frame
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda") if W * H * 20 <= 129e6 else None

    def frame(ev=None):
        if flush is not None:
            flush.zero_()
        sim.warmup(flame, FUSE - 1)
        bins.zero_()
        hits.zero_()
        if ev:
            ev[0].record(stream)
        sim.draw_to_bins(flame, bins, hits, W, H, passes, sync=False)
        if ev:
            ev[1].record(stream)
        if not WL["image"]:
            return
        if DE:  # main.cpp:490-535 in one call: the estimator's tiles are tonemapped on chip
            R.density_tonemap(bins, W, H, DE[0], DE[1], DE[2], SS, info["gamma"], info["brightness"],
                              info["vibrancy"], 0.0, None, img, stream=stream)
        else:
            R.tonemap(bins, W, H, SS, info["gamma"], info["brightness"], info["vibrancy"], 0.0, None, img,
                      stream=stream)
        if ev:
            ev[2].record(stream)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    t_first = time.perf_counter()
    sim.warmup(flame, FUSE - 1)  # the first warm-up of this genome structure compiles its kernel
    torch.cuda.synchronize()
    first_warmup_s = time.perf_counter() - t_first
    for _ in range(args.warmup):
        frame()
    barrier()
    evs = [tuple(torch.cuda.Event(enable_timing=True) for _ in range(3)) for _ in range(args.steps)]
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        t0.record(stream)
        for i in range(args.steps):
            frame(evs[i])
        t1.record(stream)
        barrier()
    ms = t0.elapsed_time(t1)
    cnt = sim.counters()  # the last frame's draw call: points binned (in frame, opacity > 0)
    binned_fraction = cnt["drawn"] / float(passes * walkers)
    draw_ms = sum(e[0].elapsed_time(e[1]) for e in evs) / args.steps
    image_passes = None
    if WL["image"]:
        tail_ms = sum(e[1].elapsed_time(e[2]) for e in evs) / args.steps
        # algorithmic bytes of the image tail: the bins read once (16 B per bin) and the RGBA8
        # image written (4 B per output pixel); with DE the passes read the bins twice (the radius
        # pass, then the tiles) plus a radius byte per bin, and never write the estimator's output
        tail_bytes = W * H * 16 + W_OUT * H_OUT * 4
        peak_, _ = _peaks()
        image_passes = {"kernels": "de_radius_sum_kernel + de_tile_kernel<9, tonemap>" if DE else
                                   "stats_kernel + tonemap_kernel",
                        "ms": tail_ms, "algorithmic_bytes": tail_bytes,
                        "gbs": tail_bytes / (tail_ms * 1e-3) / 1e9 if tail_ms > 0 else None, "peak_gbs": peak_}
    ms_step = slowest_rank_ms(ms / args.steps)
    value = replica_throughput(POINTS, ms / args.steps)

    # end to end through the C ABI: host genome in, pinned host image out
    out = torch.empty(H_OUT, W_OUT, 4, dtype=torch.uint8, pin_memory=True)
    out_np = out.numpy()
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        barrier()
        t_a = time.perf_counter()
        f2 = R.Flame.from_xml(xml, comp)
        _, st = sim.render(f2, W_OUT, H_OUT, POINTS, supersample=SS, fuse_passes=FUSE, out=out_np,
                           density_estimation=DE is not None)
        barrier()
        if i >= args.warmup:
            e2e_ms.append((time.perf_counter() - t_a) * 1e3)
    e2e_step = slowest_rank_ms(statistics.median(e2e_ms))
    e2e_value = replica_throughput(POINTS, statistics.median(e2e_ms))
    prog_bytes = info["total_params"] * 4  # order of the uploaded genome
    h2d = prog_bytes + 256 * 16
    d2h = W_OUT * H_OUT * 4

    # roofline of the chaos kernel (per launch of steps_per_launch passes)
    peak, peak_kind = _peaks()
    clk_sum = clk.summary()
    clk_mhz = clk_sum.get("sm_mhz") or 2070.0
    per_launch_ms = draw_ms / launches
    pts_per_launch = walkers * args.steps_per_launch
    pts_s = pts_per_launch / (per_launch_ms * 1e-3)
    prof_key = {"frame1080": "1080p"}.get(args.workload, args.workload)
    exchange = "pipelined" if sim.exchange() == R.EXCHANGE_PIPELINED else "barrier"
    splat_used = "tile" if sim.splat_tile() else args.splat  # AUTO may have fitted a tile
    build = kernel_build_id(flame, "%s/%d/%s" % (splat_used, int(reset), exchange)) if sim.specialized() else None
    same_build = build is not None and build == _profile_build(prof_key)
    inst = _profile_figure(prof_key, "warp instructions per point") if same_build else None
    l2_busy = _profile_figure(prof_key, "l2 atomic unit busy") if same_build else None
    traffic = _traffic(prof_key) if same_build else None
    issue_bound = sms * 4 * clk_mhz * 1e6 / inst if inst else None  # points/s at one warp-inst per SMSP-cycle
    payload = 20.0 * binned_fraction  # float4 RGBA + u32 count reduced per binned point
    ops, calls = algorithmic_ops_per_point(xml)
    fp32_rate = sms * 128 * clk_mhz * 1e6  # FP32 lane operations per second (FMA = one)
    xu_rate = sms * 16 * clk_mhz * 1e6     # transcendental (XU) operations per second
    alg_bound = min(fp32_rate / ops, xu_rate / calls if calls else float("inf"))
    roofline = {
        "bound": "issue", "kernel": "rfk_chaos_spec" if sim.specialized() else "chaos_kernel",
        "achieved": pts_s / 1e9, "peak": issue_bound / 1e9 if issue_bound else None, "unit": "Gpoints/s",
        "frac": pts_s / issue_bound if issue_bound else None, "traffic": traffic,
        "peak_source": "152 SMs x 4 schedulers x %.0f MHz / %s warp instructions per point (ncu, same kernel "
                       "build %s)" % (clk_mhz, inst, build) if inst else
                       "no ncu summary of this kernel build (%s)" % build,
        "points_per_launch": pts_per_launch, "launch_ms": per_launch_ms,
        "l2_reduction": {"bytes_per_point": payload, "gbs": payload * pts_s / 1e9,
                         "atomic_unit_busy": l2_busy / 100.0 if l2_busy is not None else None,
                         "note": "20 B (float4 RGBA + u32 count) per binned point; atomic_unit_busy = the L2 "
                                 "atomic units' active fraction (ncu, same kernel build): the splat's roofline"},
        "hbm": {"achieved": (traffic / (per_launch_ms * 1e-3) / 1e9) if traffic else None, "peak": peak,
                "unit": "GB/s", "peak_source": peak_kind},
        "algorithmic": {"fp32_ops_per_point": ops, "library_calls_per_point": calls,
                        "bound_gpoints_s": alg_bound / 1e9, "frac": pts_s / alg_bound,
                        "note": "operations of the genome's formulas (variations.yaml) against %d FP32 lanes and "
                                "16 XU lanes per SM; a library call counted as one XU operation" % 128},
    }
    line = {
        "metric": "Gpoints/s histogrammed", "value": value, "unit": "Gpoints/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic genome (%s); no dataset" % WL["genome_file"],
        "config": workload_config(reset),
        "launch": {"walkers": walkers, "cta_slots": cta, "steps_per_launch": args.steps_per_launch,
                   "passes_per_frame": passes, "splat": args.splat, "splat_tile": tile or sim.splat_tile(),
                   "exchange": exchange, "exchange_mode": args.exchange,
                   "specialized_kernel": sim.specialized(),
                   "kernel_build": build, "first_warmup_s": first_warmup_s,
                   "parallelism": "replicas" if ws > 1 else "single"},
        "s_per_frame": ms_step / 1e3,
        "draw_ms_per_frame": draw_ms,
        "binned_fraction": binned_fraction,
        "binned_gpoints_s": value * binned_fraction,
        "image_passes": image_passes,
        # per frame: the drawing launches, the warmup launch, animate_kernel, and the image tail
        # (radius/sum + tile-tonemap with DE, statistics + tonemap without)
        "gpu_launches": (launches + (FUSE + args.steps_per_launch - 1) // args.steps_per_launch + 3) * args.steps,
        "e2e": {"value": e2e_value, "unit": "Gpoints/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "s_per_frame": e2e_step / 1e3, "binned_gpoints_s": st["binned"] / (statistics.median(e2e_ms) * 1e-3) / 1e9},
        "roofline": roofline,
        "clocks": clk_sum,
    }
    if rank == 0:
        if ws == 1 and not args.no_cpu_baseline and args.workload == "frame1080":
            v, thr, sample, _, vb = cpu_baseline(xml, reset=reset)
            line["cpu_baseline"] = {"value": v, "unit": "Gpoints/s", "cores": thr, "kind": "port", "sample": sample,
                                    "binned_gpoints_s": vb}
        print(json.dumps(line))
    sim.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def batch_items(R, comp):
    """The batched-animation workload: (flame, width, height, points, seed) tuples."""
    a = R.Flame.synthesize(comp, R.SYNTH_RANDOM, 2, 1024, 768, n_xforms=4)
    b = R.Flame.synthesize(comp, R.SYNTH_RANDOM, 3, 1024, 768, n_xforms=10)
    items = []
    for k in range(120):
        f = a.interpolate(b, k / 119.0)
        items.append((f, 1024, 768, 200 * 1024 * 768, 7))  # one seed: coherent frames
    sizes = [(512, 512), (1024, 768), (1920, 1080)]
    for k in range(64):
        w, h = sizes[k % 3]
        f = R.Flame.synthesize(comp, R.SYNTH_RANDOM, 100 + k, w, h, n_xforms=2 + k % 15)
        items.append((f, w, h, 200 * w * h, 100 + k))
    return items


def run_batch(args):
    import torch
    import refrakt_gb300 as R

    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    R.build()
    comp = R.FlameCompiler()
    items = batch_items(R, comp)
    for f, *_ in items:
        f.set_estimator(*DE)
    points = sum(it[3] for it in items)
    n_img = len(items)
    reset = not args.no_badval_reset
    # the bench renders this batch again and again: every structure gets a specialised kernel
    # (compiled once, in the first warm-up step; the cache keeps them)
    bspec = {"auto": 2, "on": 0, "off": -1, "all": 2}[args.specialize]
    b = R.Batch(items, fuse_passes=FUSE, density_estimation=True, device=local, bad_value_reset=reset,
                specialize=bspec)
    info = b.info()
    spec_groups = len({items[i][0].kernel_source() for i, sp in enumerate(info["specialized"]) if sp})

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        b.run()
        b.sync()
    barrier()
    dev_ms = []
    with ClockSampler(local) as clk:
        barrier()
        t_a = time.perf_counter()
        for _ in range(args.steps):
            b.run()
            dev_ms.append(b.sync()["ms"])  # events around the graph launch on the batch's stream
        barrier()
        wall = (time.perf_counter() - t_a) * 1e3
    st = b.sync()
    ms = sum(dev_ms) / args.steps
    ms_step = slowest_rank_ms(ms)
    value = replica_throughput(st["points"], ms)

    # end to end through the public API: genomes from host XML, create (compile, upload, autotune,
    # capture), run, every image back to pinned host memory, destroy
    xmls = [(it[0].to_xml(),) + tuple(it[1:]) for it in items]
    outs = [torch.empty(h, w, 4, dtype=torch.uint8, pin_memory=True).numpy() for _, w, h, *_ in xmls]
    e2e_ms = []
    for i in range(max(1, args.warmup // 3) + args.steps):
        barrier()
        t_a = time.perf_counter()
        fl = [(R.Flame.from_xml(x, comp), w, h, p, s) for x, w, h, p, s in xmls]
        bb = R.Batch(fl, fuse_passes=FUSE, density_estimation=True, device=local, bad_value_reset=reset,
                     specialize=bspec)
        bb.run()
        for k in range(n_img):
            bb.image(k, outs[k])
        bb.close()
        barrier()
        if i >= max(1, args.warmup // 3):
            e2e_ms.append((time.perf_counter() - t_a) * 1e3)
    e2e_step = slowest_rank_ms(statistics.median(e2e_ms))
    d2h = sum(w * h * 4 for _, w, h, *_ in xmls)
    h2d = sum(it[0].info()["total_params"] * 4 + 256 * 16 for it in items)
    line = {
        "metric": "Gpoints/s histogrammed", "value": value, "unit": "Gpoints/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic genomes (seeds 2, 3, 100-163); no dataset",
        "config": workload_config(reset),
        "launch": {"images": n_img, "points_per_batch": st["points"], "requested_points": points,
                   "autotuned": info, "exchange": "barrier", "parallelism": "replicas" if ws > 1 else "single"},
        "frames_per_s": n_img / (ms_step * 1e-3),
        "binned_fraction": st["binned"] / st["points"],
        "binned_gpoints_s": value * st["binned"] / st["points"],
        "wall_ms_per_step": wall / args.steps,
        # per batch: the persistent chaos launches (one per specialised structure group + the
        # interpreted one) and per image the DE radius/sum pass + the tile-tonemap pass
        "gpu_launches": (spec_groups + (1 if 0 in info["specialized"] else 0) + 2 * n_img) * args.steps,
        "e2e": {"value": replica_throughput(st["points"], statistics.median(e2e_ms)), "unit": "Gpoints/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "frames_per_s": n_img / (e2e_step * 1e-3),
                "includes": "genome parse + compile + upload + autotune + graph capture + run + image readback"},
        "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line))
    b.close()
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_gemm(args):
    """Tensor-core GEMM throughput against the measured cuBLAS bf16 peak."""
    import torch
    import refrakt_gb300 as R
    ws, rank, local = _dist()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    R.build()
    g = torch.Generator(device="cuda").manual_seed(0)
    res = {}

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        t = []
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()  # launches on the current stream and synchronises it
            e1.record()
            torch.cuda.synchronize()
            t.append(e0.elapsed_time(e1))
        return statistics.median(t)

    for name, (M, N, K) in (("square_8192", (8192, 8192, 8192)), ("unet_conv", (1048576, 32, 720)),
                            ("unet_dw", (32, 720, 1048576))):
        a = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
        b = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
        c = torch.zeros(M, N, device="cuda")
        splits = 64 if K > 65536 else 1
        mode = R.GEMM_ATOMIC_F32 if splits > 1 else R.GEMM_STORE_F32
        ms = timed(lambda: R.gemm_bf16(a, b, c, mode=mode, splits=splits))
        res[name] = {"M": M, "N": N, "K": K, "ms": ms, "tflops": 2.0 * M * N * K / (ms * 1e-3) / 1e12}
        del a, b, c
    # the same U-Net level-0 decoder convolution as an implicit GEMM: 48 channels upsampled from
    # 512 x 512 and 32 skip channels at 1024 x 1024, 32 outputs, BF16 + bias + ReLU as in the network
    xa = torch.randn(1, 512, 512, 48, device="cuda", generator=g).to(torch.bfloat16)
    xb = torch.randn(1, 1024, 1024, 32, device="cuda", generator=g).to(torch.bfloat16)
    wt = torch.randn(32, 720, device="cuda", generator=g).to(torch.bfloat16)
    bias = torch.zeros(32, device="cuda")
    c = torch.zeros(1048576, 32, device="cuda", dtype=torch.bfloat16)
    ms = timed(lambda: R.conv3x3_bf16(xa, wt, c, xb=xb, up=True, mode=R.GEMM_STORE_BF16, bias=bias, relu=True))
    hbm = (xa.numel() + xb.numel() + wt.numel() + c.numel()) * 2
    res["unet_conv_implicit"] = {"M": 1048576, "N": 32, "K": 720, "ms": ms,
                                 "tflops": 2.0 * 1048576 * 32 * 720 / (ms * 1e-3) / 1e12,
                                 "hbm_bytes": hbm, "gbs": hbm / (ms * 1e-3) / 1e9}
    del xa, xb, wt, c
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak, src = float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        peak, src = 1900.0, "fallback"
    v = res["square_8192"]["tflops"]
    print(json.dumps({
        "metric": "TFLOP/s bf16 (tcgen05 GEMM)", "value": v, "unit": "TFLOP/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": res["square_8192"]["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16", "data": "random normal operands",
        "config": {"workload": CONFIG_NAME}, "shapes": res,
        "roofline": {"bound": "tensor", "achieved": v, "peak": peak, "unit": "TFLOP/s", "frac": v / peak,
                     "traffic": _profile_figure("tcgen05", "dram bytes per launch", "gemm_%s.md"), "peak_source": src,
                     "kernel": "umma_gemm_tma_kernel<256>", "shape": "8192^3"},
        "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
    return 0


def run_learned(args):
    import numpy as np
    import torch
    import refrakt_gb300 as R
    from refrakt_gb300 import learned as LD

    ws, rank, local = _dist()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    R.build()
    comp = R.FlameCompiler()
    log = lambda m: print(m, file=sys.stderr, flush=True)
    S = 512
    n_train, n_test = args.learned_train, args.learned_test
    # training seeds 1000-2999, then from 4000 on: never the held-out 3000-3199
    tr_seeds = list(range(1000, 1000 + min(n_train, 2000))) + list(range(4000, 4000 + max(0, n_train - 2000)))
    te_seeds = list(range(3000, 3000 + n_test))
    t0 = time.perf_counter()
    tr = [LD.genome(R, comp, s, S, S) for s in tr_seeds]
    te = [LD.genome(R, comp, s, S, S) for s in te_seeds]
    levels = [int(x) for x in args.learned_spp.split(",")]
    # one network over all input levels, or (separate) one network per level
    groups = [[l] for l in levels] if args.learned_separate else [levels]
    nets, losses, t_train = {}, {}, 0.0
    losses_val = {}
    loads = args.learned_load.split(",") if args.learned_load else []
    if loads:  # evaluate trained weights (one file per group) instead of training
        for grp, path in zip(groups, loads):
            net = R.Denoiser(4 * S * S, seed=0)
            net.set_params(np.load(path))
            for spp in grp:
                nets[spp], losses[spp] = net, None
        groups = []
    else:
        targets = torch.empty(n_train, S, S, 3, device="cuda")
        LD.render_images(tr, S, S, args.learned_target_spp, [s * 7 + 2 for s in tr_seeds], targets)
    t_data = time.perf_counter() - t0
    for gi, grp in enumerate(groups):
        t0 = time.perf_counter()
        feats = [torch.empty(n_train, S, S, 8, dtype=torch.bfloat16, device="cuda") for _ in grp]
        for k, spp in enumerate(grp):
            LD.render_features(tr, S, S, spp, [s * 7 + 1 + 100 * levels.index(spp) for s in tr_seeds], feats[k])
        torch.cuda.synchronize()
        t_data += time.perf_counter() - t0
        log("training data: %d genomes x input levels %s" % (n_train, grp))
        net = R.Denoiser(4 * S * S, seed=7 + gi)
        t0 = time.perf_counter()
        val = None
        if args.learned_val:  # the last genomes of the training range, kept out of its minibatches
            nv = args.learned_val
            vf = torch.empty(nv, S, S, 8, dtype=torch.bfloat16, device="cuda")
            LD.render_features(tr[-nv:], S, S, grp[0], [s * 7 + 1 + 100 * levels.index(grp[0]) for s in tr_seeds[-nv:]],
                               vf)
            val = (vf, targets[-nv:])
            feats = [f[:-nv] for f in feats]
        ls = LD.train(net, feats, targets[:feats[0].shape[0]], args.learned_steps, batch=args.learned_batch, lr=1e-3,
                      log=log, crop=args.learned_crop, val=val)
        if val is not None:
            ls, val_history = ls
            losses_val[tuple(grp)] = val_history
        torch.cuda.synchronize()
        t_train += time.perf_counter() - t0
        for spp in grp:
            nets[spp], losses[spp] = net, (ls[0], ls[-1])
        if args.learned_save:  # right after training, so a later failure keeps the weights
            np.save(args.learned_save.replace(".npy", "") + "_%s.npy" % "-".join(map(str, grp)), net.params())
        del feats
    if not loads:
        del targets

    # held-out evaluation against a converged adaptive-DE reference (args.learned_ref_spp)
    ref = torch.empty(n_test, S, S, 3, device="cuda")
    LD.render_images(te, S, S, args.learned_ref_spp, [s * 7 + 3 for s in te_seeds], ref)
    spps = [16, 32, 64, 125, 250, 500, 1000]
    img = torch.empty(n_test, S, S, 3, device="cuda")
    plain = {}
    for k, spp in enumerate(spps):
        LD.render_images(te, S, S, spp, [s * 7 + 10 + k for s in te_seeds], img)
        plain[spp] = float(LD.l1(img, ref).mean())
    f16 = torch.empty(n_test, S, S, 8, dtype=torch.bfloat16, device="cuda")
    learned = {}
    for spp in levels:
        LD.render_features(te, S, S, spp, [s * 7 + 20 + spp for s in te_seeds], f16)
        LD.infer_all(nets[spp], f16, img)
        learned[spp] = float(LD.l1(img, ref).mean())
    equiv = {spp: LD.plain_equivalent_spp(spps, [plain[x] for x in spps], learned[spp]) for spp in learned}
    meets = [spp for spp in levels if learned[spp] <= plain[1000]]
    spp_fast = min(meets) if meets else min(levels)
    net = nets[spp_fast]
    # 1080p frame, seconds per frame: plain (1000 spp + adaptive DE + tonemap) vs learned (16 spp + U-Net)
    W1, H1 = 1920, 1080
    f1 = LD.genome(R, comp, 1, W1, H1)
    inf = R.Denoiser(W1 * H1, seed=0)
    inf.set_params(net.params())
    out1 = torch.empty(1, H1, W1, 3, device="cuda")
    fe1 = torch.empty(1, H1, W1, 8, dtype=torch.bfloat16, device="cuda")

    def learned_frame():
        LD.render_features([f1], W1, H1, spp_fast, [5], fe1)
        inf.infer(fe1, out1)
        torch.cuda.synchronize()

    def plain_frame():
        LD.render_images([f1], W1, H1, 1000, [5], out1)
        torch.cuda.synchronize()

    times = {}
    with ClockSampler(local) as clk:
        for name, fn in (("learned", learned_frame), ("plain", plain_frame)):
            for _ in range(args.warmup):
                fn()
            ts = []
            for _ in range(args.steps):
                t = time.perf_counter()
                fn()
                ts.append(time.perf_counter() - t)
            times[name] = statistics.median(ts)
    # the fallback policy on held-out frames: split estimates from two short runs, calibrated
    # (scale = sum of true errors / sum of estimates) on the first half, applied to the second
    # with the plain path's 1000-spp error as the bound
    n_cal = min(32, n_test // 2)
    lr_ = LD.LearnedRenderer(net, spp=spp_fast, bound=args.learned_bound)
    est_err = []
    for k in range(n_cal):
        out, est, pest = lr_.estimate(te[k], S, S, seed=te_seeds[k] * 7 + 40)
        est_err.append((est, pest, float((out - ref[k]).abs().mean())))
    true_e = np.array([x[2] for x in est_err])
    est_corr = {"learned_split": float(np.corrcoef([x[0] for x in est_err], true_e)[0, 1]),
                "plain_split": float(np.corrcoef([x[1] for x in est_err], true_e)[0, 1])}
    scale = float(true_e.sum() / max(1e-12, sum(x[0] for x in est_err)))
    policy = LD.LearnedRenderer(net, spp=spp_fast, bound=plain[1000], scale=scale)
    fallbacks, errs = 0, []
    for k in range(n_cal, 2 * n_cal):
        out, e, fb = policy.render(te[k], S, S, seed=te_seeds[k] * 7 + 50)
        fallbacks += int(fb)
        errs.append(float((out - ref[k]).abs().mean()))
    line = {
        "metric": "s per 1080p frame at fixed L1 err, learned vs plain DE", "value": times["learned"],
        "unit": "s/frame", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": times["learned"] * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16", "data": "synthetic genomes rendered by the library (seeds 1000-2999 train, 3000-%d test)" %
                                  (3000 + n_test - 1),
        "config": {"workload": CONFIG_NAME, "train_genomes": n_train, "test_genomes": n_test,
                   "train_steps": args.learned_steps, "batch": args.learned_batch, "crop": args.learned_crop,
                   "resolution": [S, S],
                   "params": net.num_params(), "input_spp": levels, "target_spp": 1000, "reference_spp": args.learned_ref_spp,
                   "weights": "loaded" if loads else "trained in this run",
                   "train_target_spp": args.learned_target_spp, "validation_genomes": args.learned_val,
                   "frame_spp_learned": spp_fast},
        "plain_s_per_frame": times["plain"],
        "speedup_vs_plain": times["plain"] / times["learned"],
        "l1_plain_by_spp": plain, "l1_learned_by_input_spp": learned,
        "plain_spp_equivalent": equiv,
        "iteration_ratio_at_plain_1000spp_error": None,
        "train": {"data_s": t_data, "train_s": t_train, "separate_networks": bool(args.learned_separate),
                  "loss_first_last": {str(k): v for k, v in losses.items() if v is not None},
                  "validation_l1": {str(list(k)): v for k, v in losses_val.items()}},
        "fallback": {"calibration_frames": n_cal, "scale": scale, "bound": plain[1000],
                     "correlation_with_true_l1": est_corr, "estimate_vs_true_l1": est_err[:6],
                     "policy_frames": n_cal, "policy_fallbacks": fallbacks,
                     "policy_mean_l1": float(np.mean(errs)) if errs else None},
        "gpu_launches": None,
        "e2e": {"value": times["learned"], "unit": "s/frame", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "clocks": clk.summary(),
    }
    line["iteration_ratio_at_plain_1000spp_error"] = (1000.0 / spp_fast) if meets else None
    line["learned_reaches_plain_1000spp_error"] = bool(meets)
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--cta-slots", type=int, default=0, help="walker slots per CTA (0: the workload's default)")
    ap.add_argument("--cta-threads", type=int, default=0)
    ap.add_argument("--ctas-per-sm", type=int, default=4)
    ap.add_argument("--steps-per-launch", type=int, default=256,
                    help="passes per chaos launch (the library's default; at most 256)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-badval-reset", action="store_true",
                    help="keep walkers that leave the plane lost (the reference's default, flame.glsl:68)")
    ap.add_argument("--splat", default=None, choices=["auto", "global", "warp", "tile"],
                    help="splat strategy (default: the workload's, else auto); tile: a shared-memory histogram "
                         "tile over the attractor's bounding box")
    ap.add_argument("--exchange", default="auto", choices=["auto", "pipelined", "barrier"],
                    help="walker exchange of the specialised chaos kernel: the faster of the two timed on the first "
                         "drawing launches (default), mbarrier-pipelined, or one CTA barrier per pass")
    ap.add_argument("--specialize", default="auto", choices=["auto", "on", "off", "all"],
                    help="genome-specialised chaos kernels compiled at run time (the batch workload: auto and all = "
                         "every structure its own kernel, on = the large structures only, off = interpreted)")
    ap.add_argument("--learned-train", type=int, default=2000)
    ap.add_argument("--learned-test", type=int, default=200)
    ap.add_argument("--learned-steps", type=int, default=2000)
    ap.add_argument("--learned-bound", type=float, default=0.02)
    ap.add_argument("--learned-spp", default="16,32,64,128", help="input sample counts the denoiser trains on")
    ap.add_argument("--learned-save", default="", help="write the trained parameters (.npy) here")
    ap.add_argument("--learned-separate", action="store_true", help="one network per input level")
    ap.add_argument("--learned-batch", type=int, default=4)
    ap.add_argument("--learned-crop", type=int, default=0, help="random crops of this size (0: whole images)")
    ap.add_argument("--learned-load", default="", help="evaluate these trained parameter files (.npy, one per "
                                                       "network) instead of training")
    ap.add_argument("--learned-ref-spp", type=int, default=16000, help="samples per pixel of the reference images")
    ap.add_argument("--learned-target-spp", type=int, default=1000, help="samples per pixel of the training targets")
    ap.add_argument("--learned-val", type=int, default=0,
                    help="training genomes kept out for validation and early stopping (0: none)")
    ap.add_argument("--workload", default="frame1080", choices=sorted(WORKLOADS))
    args = ap.parse_args()
    select_workload(args.workload)
    if args.splat is None:
        args.splat = WL.get("splat", "auto")
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "learned":
        return run_learned(args)
    if args.workload == "gemm":
        return run_gemm(args)
    return run_native(args)


if __name__ == "__main__":
    sys.exit(main())
