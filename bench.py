"""Benchmark: plain GB300 delta tracker on the neural-radiance-cache scene.

Workload (one step = one progressive pass, 1 camera sample per pixel):
  1024x512x1024 fBm cloud (8 octaves), FP16 8^3 bricks with FP32 per-brick
  scale and majorant, sigma_t = 32 * density, 1920x1080, albedo 0.99,
  HG g = 0.857, <= 64 scatter events, ratio-tracking sun NEE, DDA majorant
  traversal, persistent warp-refilled wavefront kernel.
  The grid (1 GiB of FP16 texels) is larger than L2 (129 MB), so no L2
  flush is needed between timed passes.

value  : camera samples per second over the timed passes (Msamples/s),
         device-timed with CUDA events on the launching stream.
e2e    : the same metric through the C-ABI with host buffers: the grid is
         uploaded from pinned host memory once inside the timed region, and
         every pass reads its FP32 mean image back to the host.
roofline: the wavefront kernel's algorithmic bytes (8 texels x 2 B per
         density lookup) per launch / its launch time, against the measured
         HBM copy bandwidth.
time_to_1pct: the headline comparison on the same scene.  R is an FP64
         high-spp image of the plain tracker (two independent halves; their
         difference measures R's own noise, which is subtracted from every
         error below).  relRMSE = sqrt(mean_p sum_c (I - R)^2 / (R^2 + 1e-2)).
         Plain tracker: unbiased, so its error is sqrt(V / passes) with V
         the per-sample relative variance measured from R's halves (the
         measured curve is reported beside it); time = passes to 1 % x
         measured pass time.  Cached tracker (paths end in the radiance
         cache after 2 events, Adam lr 1e-3, moving-average weights for
         queries): a warm-up of 6,000 Adam steps on 16,384-record batches
         (9 training launches of 32 sets of ~65,536 records each; a
         training-only launch lasts as long as its longest path, so one
         launch of 32 sets costs about 3 of one set), then frames until its
         corrected error reaches 1 %: each frame renders and takes one Adam
         step on the next 65,536 records of a pool of 32 training sets,
         traced in one launch every 96 frames (training paths never read
         the weights, so the pool is as good as per-frame paths); time =
         warm-up + frames, device-timed.
--impl reference: the CPU restatement of the reference's tracker (the
         oracle) on all host cores, on a bounded sample of the same passes.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "cloudrendering-vulkan_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "time-to-1% relRMSE & Msamples/s: NN-cached vs plain tracker on 1 GB300"
UNIT = "Msamples/s"
BYTES_PER_LOOKUP = {0: 32, 1: 16, 2: 16}  # 8 texels x element size


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def replica_seed(rank: int) -> int:
    """Ranks render independent replicas of the pass: disjoint stream seeds."""
    return 1000 + rank


def max_over_ranks(x: float, device=None) -> float:
    """Max of a per-rank time over the default process group (x alone when
    there is none)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world: int, samples_per_step: int, steps: int, ms_max: float) -> float:
    """Msamples/s of all replicas: every rank renders samples_per_step per
    step; the job takes the slowest rank's time."""
    return world * samples_per_step * steps / (ms_max / 1e3) / 1e6


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling of the timed region.  The sampler starts before
    the region and the constructor waits (at most `ready_s`) for its first
    row, so that the tool's start-up does not eat a short region; `mark()`
    at the region's start drops the rows written before it, and `stop()`
    after the region keeps the rows since the mark (waiting up to 0.25 s for
    one, when the region was shorter than the sampling interval)."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int, interval_ms: int = 20, ready_s: float = 5.0):
        fd, self.path = tempfile.mkstemp(prefix="vcr_clocks_", suffix=".csv")
        os.close(fd)
        self.skip = 0
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={self.QUERY}",
                                       "--format=csv,noheader,nounits", "-lms", str(interval_ms)],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
            return
        t_end = time.time() + ready_s
        while self.p.poll() is None and time.time() < t_end and self._rows() == 0:
            time.sleep(0.005)

    def _rows(self) -> int:
        """Complete rows written so far."""
        with open(self.path) as r:
            return r.read().count("\n")

    def mark(self):
        if self.p:
            self.skip = self._rows()

    def stop(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        t_end = time.time() + 0.25
        while self.p.poll() is None and time.time() < t_end and self._rows() <= self.skip:
            time.sleep(0.005)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as r:
            rows = r.read().split("\n")[self.skip:]
        for line in rows:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        try:
            os.remove(self.path)
        except OSError:
            pass
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def traffic_per_lookup():
    """DRAM bytes per density lookup of the wavefront kernel from the
    committed ncu summary (profiles/pt_wavefront_c5.json), or None."""
    path = os.path.join(ROOT, "profiles", "pt_wavefront_c5.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f).get("dram_bytes_per_lookup")
    return None


def set_l2_fetch_granularity(nbytes: int) -> int:
    """cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity) for this process's
    context on the current device (a per-process limit; it ends with the
    process).  Returns the limit read back."""
    import ctypes

    import torch

    torch.zeros(1, device="cuda")  # the primary context exists
    rt = ctypes.CDLL(os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64", "libcudart.so"))
    limit_max_l2_fetch_granularity = 5
    if rt.cudaDeviceSetLimit(limit_max_l2_fetch_granularity, ctypes.c_size_t(nbytes)) != 0:
        raise RuntimeError("cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity) failed")
    got = ctypes.c_size_t(0)
    rt.cudaDeviceGetLimit(ctypes.byref(got), limit_max_l2_fetch_granularity)
    return got.value


def samples_per_step_of(sc) -> int:
    return sc.width * sc.height  # one sample per pixel a pass


def run_vcr(args):
    import torch
    import vcr
    from vcr import configs

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    sc = _divided(configs.C5_NRC, args.image_div, args.grid_div)  # a small case for profiler captures
    W, H = sc.width, sc.height
    prec = sc.precision
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    with vcr.Context(local) as ctx:
        configs.setup_context(ctx, sc, tracker=vcr.TRACKER_DDA)
        ctx.synchronize()
        tuning = ctx.autotune(seed=999, stream=sh)  # picks majorant level / DDA steps / CTA size
        seed = replica_seed(rank)
        # The timed steps are the K passes rendered by one persistent launch
        # (vcr_pt_passes): the same paths and streams as K single-pass
        # launches, without each launch's tail of long paths.
        for k in range(args.warmup):
            ctx.pt_pass(seed=seed, pass_index=k, stream=sh)
        ctx.pt_passes(seed=seed, first=0, count=args.warmup, stream=sh)
        barrier()
        clk = Clocks(local)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        clk.mark()
        ev0.record(stream)
        ctx.pt_passes(seed=seed, first=args.warmup, count=args.steps, stream=sh)
        ev1.record(stream)
        barrier()
        clocks = clk.stop()
        ms_total = max_over_ranks(ev0.elapsed_time(ev1), device="cuda")
        c = ctx.counters()
        launch = {"passes": args.steps, "lookups": c[1], "events": c[2], "paths": c[0], "ms": ms_total}
        # the same passes with one launch per pass, for comparison
        durs, looks, events, paths = [], [], [], []
        for k in range(min(args.steps, 5)):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ctx.pt_pass(seed=seed, pass_index=args.warmup + k, stream=sh)
            b.record(stream)
            b.synchronize()
            durs.append(a.elapsed_time(b))
            c = ctx.counters()
            paths.append(c[0]); looks.append(c[1]); events.append(c[2])
        img = ctx.image_mean()
        # the opt-in fast-math build of the same kernel (contracted FMAs,
        # hardware log / exp / sincos; not bit-exact): the same K passes in
        # one launch
        ctx.set_tuning(**dict(tuning, fast_math=1))
        ctx.pt_passes(seed=seed, first=0, count=args.warmup, stream=sh)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.pt_passes(seed=seed, first=args.warmup, count=args.steps, stream=sh)
        b.record(stream)
        b.synchronize()
        fast = {"ms_per_pass": round(a.elapsed_time(b) / args.steps, 4),
                "value": round(samples_per_step_of(sc) / (a.elapsed_time(b) / args.steps / 1e3) / 1e6, 3),
                "lookups_per_launch": ctx.counters()[1],
                "note": "opt-in (vcr_tuning.fast_math); path decisions can differ from the oracle's"}
        ctx.set_tuning(**tuning)
        conv = convergence(ctx, sc, stream, args) if rank == 0 and not args.no_convergence else None
    samples_per_step = samples_per_step_of(sc)
    value = whole_job_rate(ws, samples_per_step, args.steps, ms_total)
    peak, peak_kind = measured_peaks()
    bpl = BYTES_PER_LOOKUP[prec]
    # the dominant kernel's launch in the timed region: K passes, its lookups, its CUDA-event time
    lookups = float(launch["lookups"])
    dur_ms = float(launch["ms"])
    achieved = lookups * bpl / (dur_ms / 1e3) / 1e9
    single_ms = float(np.mean(durs))
    single_lookups = float(np.mean(looks))
    tpl = traffic_per_lookup()

    # e2e through the C-ABI with host buffers
    e2e = run_e2e(args, sc, local, sh, tuning) if rank == 0 else None

    if rank != 0:
        return
    cpu = cpu_baseline(sc, args) if ws == 1 and not args.no_cpu else None
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_total / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (fp16 texels, fp64 accumulation)",
        "data": "synthetic: seeded 8-octave Perlin fBm cloud generated on the device",
        "config": {"workload": sc.name, "scene_hash": sc.digest(), "grid": list(sc.size), "precision": "fp16-bricks",
                   "sigma_t_scale": 32,
                   "image": [W, H], "spp_per_step": 1, "max_events": sc.max_events, "tracker": "dda-wavefront",
                   "tuning": tuning,
                   "l2": f"inputs larger than L2 ({int(np.prod(sc.size)) * 2 / 2**30:.2f} GiB FP16 grid, 16x that in "
                         "corner blocks), no flush",
                   **({"l2_fetch_bytes": args.l2_fetch} if args.l2_fetch else {}),
                   "parallelism": f"replicas{ws}"},
        "gpu_launches": 1,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                     "traffic": (round(tpl * lookups) if tpl else None),
                     "kernel": "pt_wavefront_kernel", "bytes_per_lookup": bpl,
                     "passes_per_launch": args.steps,
                     "lookups_per_launch": int(lookups), "launch_ms": round(dur_ms, 4),
                     "lookups_per_s": round(lookups / (dur_ms / 1e3), 1)},
        "single_pass_launches": {"ms_per_pass": round(single_ms, 4),
                                 "value": round(samples_per_step / (single_ms / 1e3) / 1e6, 3),
                                 "lookups_per_pass": int(single_lookups),
                                 "frac": round(single_lookups * bpl / (single_ms / 1e3) / 1e9 / peak, 4),
                                 "note": "one vcr_pt_pass launch per pass (each ends in its own tail of long paths)"},
        "fast_math": fast,
        "clocks": clocks,
        "time_to_1pct": conv,
        "e2e": e2e,
        "cpu_baseline": cpu,
        "stats": {"events_per_path": round(float(np.sum(events)) / max(1, float(np.sum(paths))), 3),
                  "lookups_per_path": round(single_lookups / samples_per_step, 2), "image_mean": float(img.mean())},
    }
    print(json.dumps(line), flush=True)


PLAIN_PASSES_PER_LAUNCH = 25  # the plain tracker's error curve: one launch of 25 passes per point

CONV = {"ref_samples": 147456, "ref_spp": 16, "plain_max_passes": 30000, "warm_steps": 6000, "warm_sets": 32, "warm_more": 19, "warm_batch": 16384,
        "pool_sets": 32, "pool_every": 96, "max_frames": 8000, "chunk": 500, "spp": 2, "train_samples": 65536,
        "learning_rate": 1e-3, "ema_decay": 0.99, "nrc_events": 2, "repeats": 3, "position_levels": 16,
        "ablation_levels": [8, 0], "frame_group": 4,
        # the grid-encoding leg: its best setting of those tried (8 coarse
        # levels, Adam 3e-3; 16 levels at 1e-3 did not reach 1 % in 8,000 frames)
        "ablation_grid": {"position_levels": 8, "learning_rate": 3e-3}}


class Reference:
    """FP64 high-spp image R of the plain tracker from two independent
    halves (each `launches` passes of `spp` samples per pixel); their
    difference gives R's own relative MSE (noise2) and the per-sample
    relative variance V of the plain tracker."""

    def __init__(self, ctx, sc, stream, samples, spp):
        import torch
        import vcr

        sh = stream.cuda_stream
        px = sc.width * sc.height
        launches = max(1, samples // (2 * spp))

        def render(seed):
            ctx.reset()
            for k in range(0, launches, 8):  # 8 passes of spp samples a launch
                ctx.pt_passes(seed=seed, first=k, count=min(8, launches - k), spp=spp, stream=sh)
            ctx.synchronize()
            buf = torch.empty(px * 3, dtype=torch.float64, device="cuda")
            ctx.readback_to(vcr.BUF_IMAGE_SUM, buf.data_ptr(), px * 24)
            return buf / (launches * spp)

        t0 = time.perf_counter()
        ra, rb = render(100), render(200)
        self.render_s = time.perf_counter() - t0
        self.R = (ra + rb) / 2
        e_ab = torch.sqrt(torch.sum((ra - rb) ** 2 / (self.R ** 2 + 1e-2)) / px).item()
        self.noise2 = e_ab ** 2 / 4
        self.samples = 2 * launches * spp  # per pixel, both halves
        self.V = e_ab ** 2 * (launches * spp) / 2
        self.spp = spp

    def corrected(self, e):
        return float(np.sqrt(max(e * e - self.noise2, 0.0)))


def _error_curve(ctx, stream, ref, n, frame, errs, ms, first):
    """Runs n frames, each timed with CUDA events, and records the relRMSE
    against R after each (outside the timed events)."""
    import torch

    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
    for k in range(n):
        evs[k][0].record(stream)
        frame(first + k)
        evs[k][1].record(stream)
        ctx.image_rel_rmse(ref.R.data_ptr(), errs[first + k:].data_ptr(), stream=stream.cuda_stream)
    torch.cuda.synchronize()
    ms.extend(a.elapsed_time(b) for a, b in evs)


def plain_time_to_1pct(ctx, sc, stream, ref, max_passes, chunk=500):
    """The plain tracker's measured error curve, pass by pass, until its
    corrected relRMSE reaches 1 % (at most max_passes); time = the device
    time of the passes run.  The unbiased prediction sqrt(V / passes) is
    reported beside it."""
    import torch

    errs = torch.zeros(max_passes, dtype=torch.float64, device="cuda")
    ms = []
    ctx.reset()
    done, hit = 0, None
    group = PLAIN_PASSES_PER_LAUNCH

    def frame(k):  # a launch of `group` passes; its error is recorded at the last of them
        ctx.pt_passes(seed=300, first=k * group, count=group, stream=stream.cuda_stream)

    chunk_launches = max(1, chunk // group)
    max_launches = max_passes // group
    while done < max_launches and hit is None:
        n = min(chunk_launches, max_launches - done)
        _error_curve(ctx, stream, ref, n, frame, errs, ms, done)
        done += n
        e = errs[:done].cpu().numpy()
        for i in range(done - n, done):
            if ref.corrected(e[i]) <= 0.01:
                hit = i
                break
    e = errs[:done].cpu().numpy()
    cum = np.cumsum(ms)
    pass_ms = float(np.mean(ms)) / group
    need = ref.V / 1e-4
    marks = sorted({i for i in (0, 3, 39, 399, 799, 1599, done - 1) if i < done} | ({hit} if hit else set()))
    return {"time_s": round(cum[hit] / 1e3, 3) if hit is not None else None,
            "passes": (hit + 1) * group if hit is not None else None, "pass_ms": round(pass_ms, 4),
            "passes_per_launch": group,
            "basis": "measured: device time of the launches until the corrected relRMSE, checked after every "
                     f"launch of {group} passes, first reaches 1 %",
            "predicted": {"passes": int(np.ceil(need)), "time_s": round(need * pass_ms / 1e3, 3),
                          "basis": "unbiased: relRMSE = sqrt(V/passes), V from the reference halves"},
            "curve": {str((i + 1) * group): {"measured": round(ref.corrected(e[i]), 5),
                                             "predicted": round(float(np.sqrt(ref.V / ((i + 1) * group))), 5)}
                      for i in marks}}


def cached_time_to_1pct(ctx, sc, stream, ref, cfg, to_end=False):
    """Warm-up (training launches of cfg["warm_sets"] record sets, each set
    feeding 1 + cfg["warm_more"] Adam steps on batches of its records), then
    frames of cfg["spp"] samples per pixel until the corrected relRMSE
    reaches 1 %."""
    import torch
    import vcr

    sh = stream.cuda_stream
    px = sc.width * sc.height
    spp = cfg["spp"]
    prm = sc.params(vcr.TRACKER_DDA)
    prm.nrc_events = cfg["nrc_events"]
    ctx.set_params(prm)
    plain_tuning = ctx.get_tuning()
    group = cfg.get("frame_group", 1)  # frames rendered by one launch (vcr_pt_passes)
    if cfg.get("tune_cached"):  # the autotuner on the cached pass itself (untimed set-up, as for the plain one)
        ctx.nrc_setup(train_samples=cfg["train_samples"], query_capacity=px * spp, seed=1)
        ctx.autotune(seed=998, spp=spp, stream=sh)
    ctx.nrc_setup(train_samples=cfg["train_samples"], learning_rate=cfg.get("warm_lr", cfg["learning_rate"]),
                  query_capacity=px * spp * group,
                  seed=1, ema_decay=cfg["ema_decay"], tail_survival=cfg.get("tail_survival", 0.0),
                  position_levels=cfg.get("position_levels", 16), encoding=cfg.get("encoding", 0))
    sets = cfg.get("warm_sets", 1)
    per_launch = sets * (1 + cfg["warm_more"])  # Adam steps a training launch feeds
    batches = max(1, cfg["warm_steps"] // per_launch)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for k in range(batches):
        ctx.nrc_train_step(seed=400, pass_index=k, stream=sh, sets=sets)
        if per_launch > 1:
            ctx.nrc_train_more(per_launch - 1, max_records=cfg.get("warm_batch", 0), stream=sh)
    b.record(stream)
    b.synchronize()
    warm_ms = a.elapsed_time(b)
    ctx.nrc_set_learning_rate(cfg["learning_rate"])
    ctx.reset()
    nmax, chunk = cfg["max_frames"], cfg["chunk"]
    errs = torch.zeros(nmax, dtype=torch.float64, device="cuda")
    ms = []
    hit = None
    done = 0
    more = cfg.get("frame_more", 0)
    every = cfg.get("train_every", 1)  # frames between training frames (0: none after the warm-up)
    pool = cfg.get("pool_sets", 0)

    def frame_group(k):
        # frames k*group .. (k+1)*group - 1 in one launch (their cache
        # queries all see the weights of the launch's start), then their
        # `group` Adam steps; a frame at a multiple of pool_every re-traces
        # the pool with its step
        f0 = k * group
        ctx.pt_passes(seed=500 ^ 0x5bd1e995, first=batches + f0, count=group, spp=spp, stream=sh)
        re = [f for f in range(f0, f0 + group) if f % cfg["pool_every"] == 0]
        steps = group
        if re:
            ctx.nrc_train_step(seed=600, pass_index=re[0] // cfg["pool_every"], stream=sh, sets=pool)
            steps -= 1
        if steps:
            ctx.nrc_train_more(steps, max_records=cfg.get("frame_batch", cfg["train_samples"]), stream=sh)

    def frame(k):
        if group > 1:
            frame_group(k)
            return
        if pool:
            # render-only frames; their Adam steps walk a pool of pool_sets
            # training sets, traced in one launch every pool_every frames
            ctx.pt_pass(seed=500 ^ 0x5bd1e995, pass_index=batches + k, spp=spp, stream=sh)
            if k % cfg["pool_every"] == 0:
                ctx.nrc_train_step(seed=600, pass_index=k // cfg["pool_every"], stream=sh, sets=pool)
            else:
                ctx.nrc_train_more(1, max_records=cfg.get("frame_batch", cfg["train_samples"]), stream=sh)
            return
        if every and k % every == 0:
            ctx.nrc_frame(seed=500, pass_index=batches + k, spp=spp, stream=sh)
            if more:
                ctx.nrc_train_more(more, stream=sh)
        else:  # render only: paths still end in the (current) cache
            ctx.pt_pass(seed=500 ^ 0x5bd1e995, pass_index=batches + k, spp=spp, stream=sh)
            if cfg.get("reuse_steps", 0):  # and train on the last frame's records again
                ctx.nrc_train_more(cfg["reuse_steps"], stream=sh)

    assert group == 1 or pool, "several frames a launch need the pooled training schedule"
    nmax, chunk = nmax // group, max(1, chunk // group)  # counted in launches from here
    while done < nmax and (hit is None or to_end):
        n = min(chunk, nmax - done)
        _error_curve(ctx, stream, ref, n, frame, errs, ms, done)
        done += n
        e = errs[:done].cpu().numpy()
        for i in range(done - n, done):
            if hit is None and ref.corrected(e[i]) <= 0.01:
                hit = i
                break
    info = ctx.nrc_info()
    cached_tuning = ctx.get_tuning()
    ctx.set_params(sc.params(vcr.TRACKER_DDA))
    ctx.set_tuning(**plain_tuning)
    e = errs[:done].cpu().numpy()
    frames_ms = np.cumsum(ms)
    return {"frames": (hit + 1) * group if hit is not None else None, "spp_per_frame": spp,
            "frames_per_launch": group,
            "frame_ms": round(float(np.mean(ms)) / group, 4), "warm_steps": cfg["warm_steps"],
            "warm_training_launches": batches, "warm_s": round(warm_ms / 1e3, 3),
            "time_s": round((warm_ms + frames_ms[hit]) / 1e3, 3) if hit is not None else None,
            "relrmse_last": round(ref.corrected(e[-1]), 5), "frames_run": done * group,
            "floor": ({"frames": done * group, "relrmse": round(ref.corrected(e[-1]), 5),
                       "relrmse_min": round(min(ref.corrected(x) for x in e[done // 2:]), 5),
                       "basis": "the cache's error left after max_frames frames (bias plus the frames' noise)"}
                      if to_end else None),
            "curve": {str((i + 1) * group): round(ref.corrected(e[i]), 5)
                      for i in sorted({max(0, f // group - 1) for f in (1, 10, 100, 500, 1000, 2000, 4000)} | {done - 1})
                      if i < done},
            "train_records": info["train_records"], "loss": round(info["last_loss"], 4), "tuning": cached_tuning}


def convergence(ctx, sc, stream, args, overrides=None):
    """Time to 1 % relRMSE against an FP64 high-spp image: plain tracker
    and radiance-cached tracker on the bound scene (see the module text)."""
    cfg = dict(CONV, **(overrides or {}))
    ref = Reference(ctx, sc, stream, cfg["ref_samples"], cfg["ref_spp"])
    plain = plain_time_to_1pct(ctx, sc, stream, ref, cfg["plain_max_passes"])
    # the cache's training trajectory varies from run to run (the order of
    # its training records follows atomic appends): the median of a few
    # runs; the first run goes on to max_frames for the cache's error floor
    runs = [cached_time_to_1pct(ctx, sc, stream, ref, cfg, to_end=(i == 0)) for i in range(cfg["repeats"])]
    done = [r for r in runs if r["time_s"] is not None]
    nrc = sorted(done, key=lambda r: r["time_s"])[len(done) // 2] if done else runs[0]
    nrc = dict(nrc, runs_s=[r["time_s"] for r in runs], floor=runs[0]["floor"])
    nrc.pop("floor_run", None)
    # encoding ablation: the same cached run with only the coarsest L
    # frequency levels of the position encoding (L = 0: no position input)
    ablation = {}
    for lv in cfg.get("ablation_levels", ()):
        r = cached_time_to_1pct(ctx, sc, stream, ref, dict(cfg, position_levels=lv))
        ablation[str(lv)] = {k: r[k] for k in ("frames", "time_s", "relrmse_last", "frames_run", "loss")}
    # the multiresolution grid encoding in place of the frequency one
    grid = None
    if cfg.get("ablation_grid"):
        import vcr
        r = cached_time_to_1pct(ctx, sc, stream, ref, dict(cfg, encoding=vcr.NRC_ENCODING_GRID, **cfg["ablation_grid"]))
        grid = {k: r[k] for k in ("frames", "time_s", "frame_ms", "warm_s", "relrmse_last", "frames_run", "loss")}
        grid["settings"] = cfg["ablation_grid"]
    return {"plain": plain, "nrc": nrc, "position_levels_ablation": ablation, "grid_encoding": grid,
            "speedup": round(plain["time_s"] / nrc["time_s"], 2) if (nrc["time_s"] and plain["time_s"]) else None,
            "reference": {"samples_per_pixel": ref.samples, "spp_per_launch": ref.spp,
                          "own_relrmse": round(float(np.sqrt(ref.noise2)), 5), "render_s": round(ref.render_s, 2),
                          "per_sample_rel_variance": round(ref.V, 4)},
            "settings": cfg}


def run_batch(args):
    """The batched configuration: 512^3 cloud, 64 square views with sides
    uniform in [256, 1024], 8 sun elevations, 4 spp a pass, one persistent
    launch per pass replayed from a CUDA graph after the batch autotuner.
    Prints one JSON line: batched Msamples/s, the wavefront roofline, and the
    FP16 / BF16 grids' relRMSE against the FP32 grid (the precision oracle)
    rendered with the same streams and FP64 accumulation."""
    import torch
    import vcr
    from vcr import configs

    sc = configs.C4_BATCH
    views = configs.c4_views(64, seed=1)
    spp = sc.spp
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    with vcr.Context() as ctx:
        ctx.grid_generate(sc.grid_desc(), sc.fbm(), vcr.PREC_FP16)
        ctx.set_cloud(sc.cloud())
        ctx.set_params(sc.params(vcr.TRACKER_DDA))
        ctx.batch_setup(views)
        info = ctx.batch_info()
        tuning = ctx.batch_autotune(seed=999, spp=spp, stream=sh)
        ctx.batch_graph_record(seed=1, pass_index=0, spp=spp)
        ctx.batch_graph_replay(args.warmup, stream=sh)
        torch.cuda.synchronize()
        clk = Clocks(0)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        clk.mark()
        a.record(stream)
        ctx.batch_graph_replay(args.steps, stream=sh)
        b.record(stream)
        b.synchronize()
        clocks = clk.stop()
        ms = a.elapsed_time(b) / args.steps
        # one direct pass for the counters (lookups of one launch)
        ctx.batch_pass(seed=2, pass_index=0, spp=spp, stream=sh)
        ctx.synchronize()
        c = ctx.counters()
        prec = precision_vs_fp32(ctx, sc, views[0], sh)
    samples = info["pixels"] * spp
    peak, peak_kind = measured_peaks()
    achieved = c[1] * BYTES_PER_LOOKUP[vcr.PREC_FP16] / (ms / 1e3) / 1e9
    print(json.dumps({
        "metric": "batched views Msamples/s", "value": round(samples / (ms / 1e3) / 1e6, 3), "unit": "Msamples/s",
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4), "dtype": "f32 (fp16 texels)",
        "config": {"workload": sc.name, "views": len(views), "pixels": info["pixels"], "spp": spp, "suns": 8,
                   "tuning": tuning, "graph": True,
                   "l2": "inputs larger than L2 (256 MiB FP16 grid + 670 MB sums), no flush"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_source": peak_kind, "lookups_per_launch": c[1]},
        "precision_vs_fp32": prec, "clocks": clocks}), flush=True)


def precision_vs_fp32(ctx, sc, view, sh, side=160, launches=4000, spp=16):
    """Error of the FP16 and BF16 bricks against the FP32 grid (the
    precision oracle) on one view of the scene, two ways:
      agreement: one pass at the view's full size with the same streams on
        every grid; the fraction of paths whose decisions (scatter events,
        density lookups) are identical, and the relRMSE over those paths
        (quantisation moves the radiance of a path that decides the same);
      converged: FP64 images of each grid at side x side, launches x spp
        samples per pixel with the same streams on every grid (common random
        numbers: the paths that decide alike cancel), and the relRMSE
        between the FP16 (BF16) and the FP32 image.  It is an upper bound of
        the quantisation's bias (what remains is the bias plus the noise of
        the few paths that decide differently, which falls with the sample
        count); each image's own noise, from its two halves, is given beside
        it for scale.
    relRMSE = sqrt(mean_p sum_c (I - R)^2 / (R^2 + 1e-2))."""
    import torch
    import vcr

    cam, w, h, sun = view
    prm = sc.params(vcr.TRACKER_DDA)
    for a in range(3):
        prm.sun_dir[a] = sun[a]
    pos = tuple(cam.position)
    fwd = tuple(cam.forward)
    small = vcr.camera_look(pos, fwd, 60.0, 0.1, side, side)
    stats, passes, conv = {}, {}, {}
    t0 = time.perf_counter()
    for name, prec in (("fp32", vcr.PREC_FP32), ("fp16", vcr.PREC_FP16), ("bf16", vcr.PREC_BF16)):
        ctx.grid_generate(sc.grid_desc(), sc.fbm(), prec)
        ctx.set_cloud(sc.cloud())
        ctx.set_params(prm)
        ctx.set_camera(cam)
        ctx.set_frame(w, h)
        ctx.pt_pass(seed=3, pass_index=0, flags=vcr.PASS_RECORD_STATS, stream=sh)
        ctx.synchronize()
        stats[name], passes[name] = ctx.path_stats(), ctx.image_sum()
        ctx.set_camera(small)
        ctx.set_frame(side, side)
        halves = []
        for seed in (11, 12):
            ctx.reset()
            for k in range(launches // 2):
                ctx.pt_pass(seed=seed, pass_index=k, spp=spp, stream=sh)
            ctx.synchronize()
            halves.append(ctx.image_sum() / ((launches // 2) * spp))
        conv[name] = halves

    def rel2(a, b, R):
        return float(np.mean(np.sum((a - b) ** 2 / (R ** 2 + 1e-2), axis=-1)))

    out = {}
    R32 = (conv["fp32"][0] + conv["fp32"][1]) / 2
    noise32 = rel2(conv["fp32"][0], conv["fp32"][1], R32) / 4
    for name in ("fp16", "bf16"):
        agree = np.all(stats[name][..., :2] == stats["fp32"][..., :2], axis=-1)
        a, b = passes[name][agree], passes["fp32"][agree]
        I = (conv[name][0] + conv[name][1]) / 2
        noise = rel2(conv[name][0], conv[name][1], R32) / 4
        out[name] = {"paths_agreeing": round(float(agree.mean()), 5),
                     "relrmse_agreeing_paths": round(float(np.sqrt(np.mean(np.sum((a - b) ** 2 / (b ** 2 + 1e-2),
                                                                                    axis=-1)))), 7),
                     "converged_relrmse_common_streams": round(float(np.sqrt(rel2(I, R32, R32))), 6),
                     "own_noise_relrmse": round(float(np.sqrt(noise)), 5)}
    out["fp32_own_noise_relrmse"] = round(float(np.sqrt(noise32)), 5)
    out["setup"] = {"agreement_view": [w, h], "converged_view": [side, side],
                    "samples_per_pixel": launches * spp, "seconds": round(time.perf_counter() - t0, 1)}
    return out


def _gather_roofline(kernel, units, bytes_per_unit, ms, basis):
    peak, peak_kind = measured_peaks()
    achieved = units * bytes_per_unit / (ms / 1e3) / 1e9 if ms > 0 else 0.0
    return {"bound": "hbm", "kernel": kernel, "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_source": peak_kind, "units_per_launch": units,
            "bytes_per_unit": bytes_per_unit, "launch_ms": round(ms, 4), "basis": basis}


def _timed_passes(stream, fn, steps):
    import torch
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for k in range(steps):
        fn(k)
    b.record(stream)
    b.synchronize()
    return a.elapsed_time(b) / steps


def _divided(sc, div, grid_div=1):
    """The scene with its image sides divided by div and its grid sides by
    grid_div (the same cloud at a coarser resolution: the box stays the
    unit-longest-axis box): a small case of the same workload, for profiler
    captures that must hold a few GB at most."""
    import dataclasses

    if div > 1:
        sc = dataclasses.replace(sc, name=f"{sc.name}/{div}", width=max(1, sc.width // div),
                                 height=max(1, sc.height // div))
    if grid_div > 1:
        sc = dataclasses.replace(sc, name=f"{sc.name}/grid{grid_div}",
                                 size=tuple(max(8, n // grid_div) for n in sc.size))
    return sc


def run_sort(args):
    """The stable LSD radix sort of (u32 key, u32 value) pairs: the C3
    pass's 10.3 M segments with 30-bit Morton keys (4 digit passes of 8
    bits, the last of 6), and 64 M pairs with 32-bit keys; inputs larger
    than L2 except the ping-pong of the C3 case (82 MB each way).
    Algorithmic bytes: 8 B read + 8 B written per pair and digit pass (64 B
    a pair for 4 passes) plus the one histogram read of the keys (4 B a
    pair).  The reference sorts on 4-bit digits (8 passes, 128 B a pair);
    the rate that cost model gives is reported beside the roofline."""
    import torch
    import vcr

    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    peak, peak_kind = measured_peaks()
    cases = []
    with vcr.Context() as ctx:
        for n, bits in ((10301598, 30), (1 << 26, 32)):
            g = torch.Generator(device="cuda").manual_seed(n)
            hi = (1 << bits) - 1 if bits < 32 else (1 << 31) - 1
            keys = torch.randint(0 if bits < 32 else -(1 << 31), hi, (n,), dtype=torch.int32, device="cuda",
                                 generator=g)
            vals = torch.arange(n, dtype=torch.int32, device="cuda")
            ko, vo = torch.empty_like(keys), torch.empty_like(keys)
            for _ in range(args.warmup):
                ctx.radix_sort_pairs(keys.data_ptr(), vals.data_ptr(), ko.data_ptr(), vo.data_ptr(), n, 0, bits,
                                     stream=sh)
            ms = _timed_passes(stream, lambda k: ctx.radix_sort_pairs(keys.data_ptr(), vals.data_ptr(), ko.data_ptr(),
                                                                        vo.data_ptr(), n, 0, bits, stream=sh),
                               args.steps)
            ctx.synchronize()
            passes = (bits + 7) // 8
            alg = n * (16 * passes + 4)
            alg4 = n * (16 * ((bits + 3) // 4) + 4)  # the reference's 4-bit passes
            achieved = alg / (ms / 1e3) / 1e9
            cases.append({"pairs": n, "key_bits": bits, "digit_passes": passes, "ms": round(ms, 4),
                          "pairs_per_s": round(n / (ms / 1e3), 1),
                          "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                                       "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                                       "algorithmic_bytes": alg},
                          "reference_cost_model": {"digit_passes": (bits + 3) // 4, "algorithmic_bytes": alg4,
                                                   "achieved": round(alg4 / (ms / 1e3) / 1e9, 1), "unit": "GB/s"}})
    print(json.dumps({"metric": "radix sort pairs/s", "steps": args.steps, "warmup": args.warmup, "cases": cases}),
          flush=True)


def run_display(args):
    """The display image of the 1920x1080 frame (the swapchain blit's
    headless form): one thread per pixel reads 3 FP64 sums (24 B) and writes
    one 8-bit RGBA pixel (4 B); device output, CUDA events, roofline against
    the measured HBM copy peak."""
    import torch
    import vcr
    from vcr import configs

    sc = configs.C5_NRC
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    px = sc.width * sc.height
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc, tracker=vcr.TRACKER_DDA)
        for k in range(2):
            ctx.pt_pass(seed=1, pass_index=k, stream=sh)
        out = torch.empty(px * 4, dtype=torch.uint8, device="cuda")
        flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # larger than L2, written between launches
        for k in range(args.warmup):
            ctx.display_to(out.data_ptr(), stream=sh)
        ms = []
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xFF)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ctx.display_to(out.data_ptr(), stream=sh)
            b.record(stream)
            b.synchronize()
            ms.append(a.elapsed_time(b))
    t = float(np.median(ms))
    peak, kind = measured_peaks()
    algo = px * 28
    print(json.dumps({
        "metric": "display image", "workload": f"{sc.width}x{sc.height} FP64 sums -> RGBA8 sRGB", "ms": round(t, 4),
        "steps": args.steps, "l2": "a 256 MiB buffer written between launches",
        "roofline": {"bound": "hbm", "achieved": round(algo / (t / 1e3) / 1e9, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(algo / (t / 1e3) / 1e9 / peak, 4), "peak_source": kind,
                     "bytes_per_pixel": 28}}), flush=True)


def run_ppm(args):
    """C2: 256^3 FP32 cloud (sigma_t = 16 rho), 1,048,576 photons a pass, r0
    0.01, alpha 0.7, 960x540; one JSON line of pass time and rates."""
    import torch
    import vcr
    from vcr import configs

    sc = _divided(configs.C2_PPM, args.image_div)
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    ex = sc.extra
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc)
        ctx.synchronize()
        ctx.ppm_setup(ex["photons"], 8 * ex["photons"], ex["r0"], ex["alpha"])
        for k in range(args.warmup):
            ctx.ppm_pass(seed=1, pass_index=k, stream=sh)
        ms = _timed_passes(stream, lambda k: ctx.ppm_pass(seed=1, pass_index=args.warmup + k, stream=sh), args.steps)
        info = ctx.ppm_info()
        stats = ctx.ppm_read("stats")
        tested, gather_ms = ctx.gather_stats("ppm")  # the last pass's gather kernel
    print(json.dumps({
        "metric": "PPM pass", "workload": sc.name, "ms_per_pass": round(ms, 4), "steps": args.steps,
        "photons_emitted_per_s": round(ex["photons"] / (ms / 1e3), 1),
        "photons_stored": info["photons_stored"], "dropped": info["dropped"],
        "pixel_gathers_per_s": round(sc.width * sc.height / (ms / 1e3), 1),
        "mean_radius": float(stats[..., 1].mean()), "mean_photon_count": float(stats[..., 0].mean()),
        "roofline": _gather_roofline("ppm_gather_kernel", tested, 32, gather_ms,
                                     "leaf photons tested x 32 B (position + power, direction packed)")}),
          flush=True)


def run_ppb(args):
    """C3: 256^3 FP32 cloud, photons scaled so that a pass deposits about
    262,144 beams, r0 0.02, alpha 0.8, 1280x720; segments are 30-bit
    Morton-keyed, radix-sorted and put in an LBVH every pass."""
    import torch
    import vcr
    from vcr import configs

    sc = _divided(configs.C3_PPB, args.image_div)
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    want = sc.extra["beams"]
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc)
        ctx.synchronize()
        probe = 16384
        ctx.ppb_setup(probe, 1 << 24, 0.02, 0.8)
        ctx.ppb_pass(seed=1, pass_index=0, stream=sh)
        ctx.synchronize()
        per_photon = max(float(ctx.ppb_read("nbeams", probe).sum()) / probe, 1e-3)
        photons = int(want / per_photon)
        ctx.ppb_setup(photons, 1 << 24, 0.02, 0.8)
        ctx.reset()
        for k in range(args.warmup):
            ctx.ppb_pass(seed=1, pass_index=k, stream=sh)
        ms = _timed_passes(stream, lambda k: ctx.ppb_pass(seed=1, pass_index=args.warmup + k, stream=sh), args.steps)
        info = ctx.ppb_info()
        beams = int(ctx.ppb_read("nbeams", photons).sum())
        evaluated, gather_ms = ctx.gather_stats("ppb")  # the last pass's gather kernel
    print(json.dumps({
        "metric": "PPB pass", "workload": sc.name, "ms_per_pass": round(ms, 4), "steps": args.steps,
        "photons": photons, "beams": beams, "segments": info["segments"], "dropped": info["dropped"],
        "segments_per_s": round(info["segments"] / (ms / 1e3), 1),
        "pixel_gathers_per_s": round(sc.width * sc.height / (ms / 1e3), 1), "radius": info["radius"],
        "roofline": _gather_roofline("ppb_gather_kernel", evaluated, 32 + 112, gather_ms,
                                     "(pixel, segment) pairs evaluated x (32 B segment + 112 B beam slot)")}),
          flush=True)


def run_nrc_frames(args):
    """Radiance-cached frames alone: warm-up steps, then args.nrc_frames
    frames, each timed on the device; one JSON line with the means."""
    import torch
    import vcr
    from vcr import configs

    sc = configs.C5_NRC
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    with vcr.Context() as ctx:
        configs.setup_context(ctx, sc)
        ctx.set_tuning(majorant_level=1, dda_steps=8, stage_majorants=1, block_threads=256)
        prm = sc.params(vcr.TRACKER_DDA)
        prm.nrc_events = CONV["nrc_events"]
        ctx.set_params(prm)
        enc = vcr.NRC_ENCODING_GRID if args.nrc_encoding == "grid" else vcr.NRC_ENCODING_FREQUENCY
        ctx.nrc_setup(train_samples=CONV["train_samples"], learning_rate=CONV["learning_rate"],
                      query_capacity=sc.width * sc.height, seed=1, ema_decay=CONV["ema_decay"], encoding=enc)
        for k in range(args.warmup):
            ctx.nrc_train_step(seed=400, pass_index=k, stream=sh)
        ms = []
        for k in range(args.nrc_frames):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ctx.nrc_frame(seed=500, pass_index=args.warmup + k, stream=sh)
            b.record(stream)
            b.synchronize()
            ms.append(a.elapsed_time(b))
        info = ctx.nrc_info()
    print(json.dumps({"workload": sc.name + " radiance-cached frames", "encoding": args.nrc_encoding,
                      "frames": args.nrc_frames,
                      "frame_ms": round(float(np.mean(ms)), 4), "queries": info["queries"],
                      "train_records": info["train_records"]}), flush=True)


def run_e2e(args, sc, device, sh, tuning=None):
    """Grid upload from pinned host memory + per-pass mean-image read back,
    all through the C-ABI, wall-clock timed (the tracker's tuning is set
    before the timed region, as a caller sets it once)."""
    import torch
    import vcr

    dense = vcr.fbm_fill_host(sc.size, sc.fbm())  # the library's host generator (threaded)
    pinned = torch.from_numpy(dense).pin_memory()
    img_bytes = sc.width * sc.height * 3 * 4
    # the result, read back after every pass into alternating pinned buffers
    imgs = [torch.empty(sc.width * sc.height * 3, dtype=torch.float32).pin_memory() for _ in range(2)]
    with vcr.Context(device) as ctx:
        if tuning:
            ctx.set_tuning(**tuning)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        import ctypes as C
        check = vcr.check
        check(vcr.lib().vcr_grid_upload(ctx.h, C.byref(sc.grid_desc()), C.c_void_p(pinned.data_ptr()),
                                        sc.precision), ctx.h)
        ctx.set_cloud(sc.cloud())
        ctx.set_camera(sc.camera())
        ctx.set_params(sc.params(vcr.TRACKER_DDA))
        ctx.set_frame(sc.width, sc.height)
        ctx.synchronize()
        t_up = time.perf_counter()
        for k in range(args.steps):
            ctx.pt_pass(seed=5, pass_index=k, stream=sh)
            # stream-ordered: the copy of pass k overlaps pass k + 1
            ctx.readback_async(vcr.BUF_IMAGE_MEAN, imgs[k % 2].data_ptr(), img_bytes, stream=sh)
        ctx.readback_wait()
        t1 = time.perf_counter()
    grid_bytes = dense.nbytes
    return {"value": round(sc.width * sc.height * args.steps / (t1 - t0) / 1e6, 3), "unit": UNIT,
            "h2d_bytes_per_step": int(grid_bytes // args.steps), "d2h_bytes_per_step": img_bytes,
            "upload_s": round(t_up - t0, 4), "passes_s": round(t1 - t_up, 4),
            "note": "grid (FP32, pinned) uploaded once per run; one launch per pass and its mean image read back "
                    "into pinned memory after every pass (vcr_readback_async: the copy of pass k overlaps pass k+1)"}


class OracleScene:
    """The oracle (a CPU port of the reference's tracker) set up on the
    benchmark scene, generated by the oracle's own fBm on all host cores."""

    def __init__(self, sc, threads=None):
        from oracle import oracle as orc
        from vcr import _abi

        self.sc = sc
        self.threads = threads or os.cpu_count() or 1
        t0 = time.perf_counter()
        dense = orc.fbm_fill(sc.size, seed=sc.seed, octaves=sc.octaves, threads=self.threads)
        self.g = orc.Grid(dense, sc.precision)
        del dense
        self.setup_s = time.perf_counter() - t0
        # the scene's structs from the oracle's restatement of the reference's
        # set-up: this leg loads no product library
        _, self.cloud, self.cam, self.prm = orc.scene_structs(sc, _abi.TRACKER_DDA)
        self.cloud.max_extinction = max(self.g.max_density(), 0.01)

    def pass_rows(self, rows, pass_index):
        """One pass over `rows` full-width image rows in (up to) 8 bands
        spaced evenly over the frame, so the sample has the whole frame's mix
        of dense, thin and empty (sky) rows; returns (paths, seconds)."""
        W, H = self.sc.width, self.sc.height
        nb = max(1, min(8, rows))
        band = max(1, rows // nb)
        t0 = time.perf_counter()
        for i in range(nb):
            y0 = min(H - band, max(0, int((i + 0.5) * H / nb) - band // 2))
            self.g.pt_pass(self.cloud, self.cam, self.prm, W, H, seed=3, pass_index=pass_index,
                           crop=(0, y0, W, band), threads=self.threads)
        return W * band * nb, time.perf_counter() - t0

    def rows_for(self, seconds):
        paths, dt = self.pass_rows(2, 0)
        per_row = dt / 2
        return int(max(1, min(self.sc.height, seconds / max(per_row, 1e-6))))


def cpu_baseline(sc, args, budget_s=12.0):
    """Passes over rows spread over the frame until about budget_s seconds
    of work are done (at most 64 passes)."""
    os_ = OracleScene(sc)
    rows = os_.rows_for(budget_s / 4)
    done = t = 0.0
    k = 0
    while (t < budget_s and k < 64) or k < 2:
        p, dt = os_.pass_rows(rows, k + 1)
        done += p
        t += dt
        k += 1
    return {"value": round(done / t / 1e6, 4), "unit": UNIT, "cores": os_.threads, "kind": "port",
            "sample": f"{k} passes x {rows} full-width rows in 8 bands spread over the frame = {int(done)} camera paths, "
                      f"{t:.1f} s on {os_.threads} threads (grid setup {os_.setup_s:.1f} s not counted)"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from vcr import configs
    sc = configs.C5_NRC
    os_ = OracleScene(sc)
    # each step: one pass over a band of rows, sized so that all steps take
    # about a minute (at most 6 s, at least 0.5 s a step)
    rows = os_.rows_for(min(6.0, max(0.5, 60.0 / max(1, args.steps))))
    for k in range(args.warmup):
        os_.pass_rows(max(1, rows // 4), k + 1)
    done = t = 0.0
    for k in range(args.steps):
        p, dt = os_.pass_rows(rows, args.warmup + k + 1)
        done += p
        t += dt
    v = round(done / t / 1e6, 4)
    cpu = {"cores": os_.threads,
           "sample": f"{args.steps} passes x {rows} full-width rows in 8 bands spread over the frame = {int(done)} "
                     f"camera paths, {t:.1f} s"}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (fp16 texels decoded, fp64 accumulation)", "data": "synthetic",
            "config": {"workload": sc.name, "scene_hash": sc.digest(), "grid": list(sc.size),
                       "image": [sc.width, sc.height], "tracker": "dda (CPU port)"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cpu["cores"], "kind": "port",
                             "sample": cpu["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="vcr", choices=["vcr", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-convergence", action="store_true", help="skip the time-to-1 %% comparison")
    ap.add_argument("--nrc-frames", type=int, default=0,
                    help="only time this many radiance-cached frames on the scene (a profiling workload)")
    ap.add_argument("--nrc-encoding", default="frequency", choices=["frequency", "grid"],
                    help="the cache's position encoding for --nrc-frames")
    ap.add_argument("--batch", action="store_true",
                    help="only measure the batched 64-view configuration (CUDA graph, autotuned)")
    ap.add_argument("--ppm", action="store_true", help="only measure the photon-mapping configuration")
    ap.add_argument("--ppb", action="store_true", help="only measure the photon-beam configuration")
    ap.add_argument("--display", action="store_true", help="only measure the display-image kernel")
    ap.add_argument("--sort", action="store_true", help="only measure the radix sort")
    ap.add_argument("--image-div", type=int, default=1,
                    help="divide the image sides (a small case of the workload for profiler captures)")
    ap.add_argument("--grid-div", type=int, default=1,
                    help="divide the grid sides (the same cloud, coarser; with --image-div, a small case)")
    ap.add_argument("--l2-fetch", type=int, default=0,
                    help="set this process's maximum L2 fetch granularity in bytes (32/64/128) before the run: "
                         "how DRAM traffic per lookup depends on the L2's fetch size")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference" and not (args.ppm or args.ppb or args.batch or args.nrc_frames or args.display
                                         or args.sort):
        run_reference(args)
        return
    import contextlib

    import __graft_entry__ as ge
    with contextlib.redirect_stdout(sys.stderr):  # stdout carries only the JSON line
        ge.build()
    if args.l2_fetch:
        set_l2_fetch_granularity(args.l2_fetch)
    if args.sort:
        run_sort(args)
    elif args.display:
        run_display(args)
    elif args.ppm or args.ppb:
        run_ppm(args) if args.ppm else run_ppb(args)
    elif args.batch:
        run_batch(args)
    elif args.nrc_frames:
        run_nrc_frames(args)
    else:
        run_vcr(args)


if __name__ == "__main__":
    main()
