#!/usr/bin/env python
"""Benchmark of the game-frame path on GB300.

Workload (one step = one frame): 1920x1080 with 4x SSAA (8,294,400 camera rays), maximum
recursion depth 5, two-level BVH of 1024 instances drawn from 8 seeded procedural meshes
(~11.7M instanced / 377k unique triangles).  Every frame 10% of the instances move (TLAS rebuilt
from scratch), each BLAS is refit with probability 0.05 after per-vertex jitter, then trace +
shade, the roughness approximation, the postprocess composite and FXAA run into the RGBA32F
framebuffer.

metric = Mrays/s: every ray that traverses the BVH (camera, shadow, reflection, refraction) per
second of the whole frame (TLAS build + refits + trace + post).
  value: inputs already resident in HBM (per-frame instance arrays and jittered vertices are
         device buffers), timed with CUDA events on the library's stream, L2 flushed (256 MiB
         memset) between frames.
  e2e:   the same frames through the C ABI with host buffers: per frame the instance array and the
         refit vertices are copied from pinned host memory and the framebuffer is read back into
         pinned host memory (rg_download_async: frame f's copy overlaps frame f+1's render), timed
         by wall clock until the last frame's pixels are in host memory.

--impl reference runs the reference arm: the reference's own GPU path needs a Vulkan ray-tracing
driver (unavailable on this machine), so it times the CPU restatement of the same shaders (the oracle)
on all host cores, each step the same frame sequence sampled on rows spread over the frame.
"""
from __future__ import annotations

import argparse
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

from raygun_gb300 import scenes as S  # noqa: E402
from raygun_gb300.rays import first_bounce_secondary  # noqa: E402

WORKLOAD = "game-frame: {w}x{h}, 4x SSAA, depth 5, 1024 instances of 8 procedural meshes (~11.7M instanced tris), " \
           "TLAS rebuilt + BLAS refit per frame, trace + roughness + composite + FXAA"
BYTES_RAY = 32 + 20   # ray in (origin+tmin, dir+tmax) + hit out (t, u, v, prim, inst)
BYTES_NODE = 112      # 4-wide BVH record: four child boxes + four child refs
BYTES_TRI = 36        # three vertex positions
CPU_ROWS_PER_STEP = 27


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-rows", type=int, default=0, help="rows per render of the CPU-baseline sample (0: full frames)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--res", default="1920x1080", help="WxH; smaller sizes are for profiling captures only")
    ap.add_argument("--workload", default="game-frame", choices=["game-frame", "batch", "serve", "filter", "spheres", "dist-check"],
                    help="game-frame: the 1080p 4x SSAA frame loop; batch: 64 independent scenes per step; "
                         "serve: Poisson render requests through the render server; dist-check: the --gpus N "
                         "launcher and the cross-rank aggregation alone, on CPU (gloo), with synthetic counts")
    ap.add_argument("--serve-requests", type=int, default=2000)
    ap.add_argument("--serve-rate", type=float, default=400.0, help="mean arrivals per second")
    ap.add_argument("--serve-large", type=int, default=12, help="large terrain scenes in the catalog")
    ap.add_argument("--serve-budget-gb", type=float, default=160.0)
    ap.add_argument("--serve-graph", action="store_true", help="serve: CUDA-graph batches instead of the host loop")
    ap.add_argument("--serve-filter-fraction", type=float, default=0.25,
                    help="serve: share of requests that ask for the learned filter (committed trained weights)")
    ap.add_argument("--filter-scenes", type=int, default=200, help="filter: training scenes")
    ap.add_argument("--filter-crops", type=int, default=20000, help="filter: 128x128 training crops")
    ap.add_argument("--filter-epochs", type=int, default=30)
    ap.add_argument("--filter-eval", type=int, default=4, help="filter: held-out 1080p scenes")
    ap.add_argument("--filter-weights", default=None, help="filter: load these weights instead of training")
    ap.add_argument("--filter-save", default=None, help="filter: write the trained weights here")
    ap.add_argument("--no-tune", action="store_true", help="batch: skip the autotuner (default launch shape)")
    ap.add_argument("--batch-slots", type=int, default=0, help="batch: path slots of the round loop (0: the library default)")
    ap.add_argument("--batch-scenes", type=int, default=64, help="batch: scenes per batch (profiling captures only)")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def replica_throughput(rays_local: float, ms_local: float, world: int, device=None):
    """Whole-job rate of N independent replicas: rays summed over ranks / the slowest rank's time
    (Mrays/s).  Every rank gets the same value; world == 1 needs no process group."""
    if world == 1:
        return rays_local / (ms_local * 1e-3) / 1e6, ms_local
    import torch
    import torch.distributed as dist
    t = torch.tensor([rays_local], dtype=torch.float64, device=device)
    m = torch.tensor([ms_local], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    dist.all_reduce(m, op=dist.ReduceOp.MAX)
    return float(t.item()) / (float(m.item()) * 1e-3) / 1e6, float(m.item())


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def trace_traffic():
    """DRAM bytes of one trace-kernel launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "k_wf_trace_game_frame_1080p.json")
    try:
        d = json.load(open(p))
        return d.get("dram_bytes_per_launch"), d.get("source")
    except (OSError, ValueError):
        return None, None


def game_config(sc, world):
    """The game-frame workload's identity, the same for both arms."""
    return {"workload": WORKLOAD.format(w=sc.width, h=sc.height), "width": sc.width, "height": sc.height,
            "spp": int(sc.ubo["numSamples"][0]), "max_recursions": int(sc.ubo["maxRecursions"][0]),
            "instances": len(sc.instances), "instanced_tris": sc.instanced_tri_count, "unique_tris": sc.tri_count,
            "frames": "seeded animation (FrameAnimator seed 101): frames 0 .. warmup+steps-1",
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}


class FrameInputs:
    """Per-frame inputs of the animated scene, precomputed so timed frames only move data."""

    def __init__(self, scene, nframes, seed=101):
        anim = S.FrameAnimator(scene, seed=seed)
        self.instances = []
        self.refits = []  # per frame: list of (blas, vertex_offset, nverts, vertex array)
        for _ in range(nframes):
            r = anim.step()
            self.instances.append(scene.instances.copy())
            self.refits.append([(b, vo, nv, scene.vertices[vo:vo + nv].copy()) for b, vo, nv in r])


def run_ours(args):
    import torch
    from raygun_gb300 import build as rgbuild, rgcuda

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    rgbuild.build()
    w, h = (int(x) for x in args.res.split("x"))
    sc = S.instanced_scene(width=w, height=h)
    orc_scene = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle
        orc_scene = oracle.OracleScene(sc)  # pristine frame-0 state, before any animation
    rt = rgcuda.Raytracer(sc, device=local).prepare()
    ctx = rt.ctx
    K, W = args.steps, args.warmup
    total = W + K + 1
    pristine = sc.vertices.copy()  # frame 0's vertices (the animation below moves sc's)
    frames = FrameInputs(sc, total)
    dev = torch.device("cuda", local)
    ext = torch.cuda.ExternalStream(ctx.stream(), device=dev)
    ninst = len(sc.instances)
    blas_ids = np.asarray(rt.blas_ids, np.uint32)

    def inst_bytes(f):
        inst = frames.instances[f].copy()
        inst["blas"] = blas_ids[inst["blas"]]
        return inst

    # device-resident inputs for the `value` loop
    inst_dev = torch.from_numpy(np.stack([inst_bytes(f).view(np.uint8) for f in range(total)])).to(dev)
    vert_chunks, vert_offsets, off = [], {}, 0
    for f in range(total):
        for j, (b, vo, nv, arr) in enumerate(frames.refits[f]):
            vert_chunks.append(arr.view(np.uint8).reshape(-1))
            vert_offsets[(f, j)] = off
            off += arr.nbytes
    vert_dev = torch.from_numpy(np.concatenate(vert_chunks) if vert_chunks else np.zeros(16, np.uint8)).to(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    ubo = sc.ubo
    stride = ninst * S.INSTANCE.itemsize

    def step_device(f):
        for j, (b, vo, nv, _) in enumerate(frames.refits[f]):
            ctx.update_vertices_device(vo, vert_dev.data_ptr() + vert_offsets[(f, j)], nv)
            ctx.refit_blas(int(blas_ids[b]))
        ctx.build_tlas_device(inst_dev.data_ptr() + f * stride, ninst)
        ctx.render(ubo, True)
        with torch.cuda.stream(ext):
            flush.zero_()

    # pinned host inputs / outputs for the e2e loop
    inst_pin = torch.from_numpy(np.stack([inst_bytes(f).view(np.uint8) for f in range(total)])).pin_memory()
    inst_host = inst_pin.numpy()
    vert_pin = torch.from_numpy(np.concatenate(vert_chunks) if vert_chunks else np.zeros(16, np.uint8)).pin_memory()
    vert_host = vert_pin.numpy()
    # two pinned framebuffers: frame f's read-back overlaps frame f+1's render (rg_download_async)
    fb_pins = [torch.empty(sc.height * sc.width * 16, dtype=torch.uint8).pin_memory() for _ in range(2)]

    def step_host(f):
        h2d = 0
        for j, (b, vo, nv, _) in enumerate(frames.refits[f]):
            o = vert_offsets[(f, j)]
            ctx.update_vertices(vo, vert_host[o:o + nv * 32].view(S.VERTEX))
            ctx.refit_blas(int(blas_ids[b]))
            h2d += nv * 32
        ctx.build_tlas(inst_host[f].view(S.INSTANCE))
        ctx.render(ubo, True)
        ctx.download_async(fb_pins[f % 2].data_ptr())
        with torch.cuda.stream(ext):
            flush.zero_()
        return h2d + stride + S.UBO.itemsize

    def barrier():
        torch.cuda.synchronize(dev)
        ctx.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---------------- value: device-resident inputs ----------------
    ctx.set_flags(rgcuda.RG_FLAG_KERNEL_TIMING)  # events around every traversal launch
    f = 0
    for _ in range(W):
        step_device(f)
        f += 1
    barrier()
    ctx.timings()  # drop warm-up frames from the timing sums
    ctx.reset_total_stats()
    launches0 = rgcuda.launch_count()
    clocks = ClockSampler(local)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    e0.record(ext)
    for _ in range(K):
        step_device(f)
        f += 1
    e1.record(ext)
    barrier()
    clk = clocks.stop()
    launches = rgcuda.launch_count() - launches0
    tot = ctx.total_stats()
    rays = tot["primary"] + tot["shadow"] + tot["secondary"]
    tm = ctx.timings()
    value, ms = replica_throughput(rays, e0.elapsed_time(e1), world, dev)

    ctx.set_flags(0)

    # ---------------- e2e: host buffers through the C ABI ----------------
    # the same frames as the device-resident loop: back to frame 0's vertices (and BLAS boxes), then
    # frames 0 .. W + K - 1 again
    ctx.update_vertices(0, pristine)
    for b in np.unique(blas_ids):
        ctx.refit_blas(int(b))
    f = 0
    for _ in range(W):
        step_host(f)
        f += 1
    barrier()
    ctx.reset_total_stats()
    h2d = 0
    barrier()
    # wall clock from the first frame's inputs to the last frame's pixels in host memory (the final
    # barrier waits for the render stream and the read-back copies)
    t_e2e = time.perf_counter()
    for _ in range(K):
        h2d += step_host(f)
        f += 1
    barrier()
    wall_ms = (time.perf_counter() - t_e2e) * 1e3
    tot2 = ctx.total_stats()
    e2e_value, ms_e2e = replica_throughput(tot2["primary"] + tot2["shadow"] + tot2["secondary"], wall_ms, world, dev)
    e2e = {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": int(h2d // K),
           "d2h_bytes_per_step": sc.height * sc.width * 16, "ms_per_step": ms_e2e / K}

    # ---------------- roofline of the trace kernel ----------------
    ctx.set_flags(rgcuda.RG_FLAG_COUNT_VISITS)
    ctx.timings()
    step_device(f)
    barrier()
    cst = ctx.stats()
    ctx.set_flags(0)
    crays = cst["primary"] + cst["shadow"] + cst["secondary"]
    bytes_per_ray = (crays * BYTES_RAY + cst["nodes"] * BYTES_NODE + cst["tris"] * BYTES_TRI) / max(crays, 1)
    # k_wf_trace runs once per wavefront round; one frame's launches are taken together as the unit
    trace_ms = tm["traceKernelSum"] / max(tm["frames"], 1)
    bytes_launch = bytes_per_ray * rays / K
    achieved = bytes_launch / (trace_ms * 1e-3) / 1e9
    peak, peak_src = measured_peak_hbm()
    traffic, traffic_src = trace_traffic()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": "k_wf_trace + k_wf_tail (all traversal launches of one frame; the tail launch also shades)",
                "launches_per_frame": tm["traceLaunches"] / max(tm["frames"], 1), "peak_source": f"{peak_src} hbm_gbs",
                "algorithmic_bytes_per_launch": bytes_launch, "bytes_per_ray": bytes_per_ray,
                "node_visits_per_ray": cst["nodes"] / max(crays, 1), "tri_tests_per_ray": cst["tris"] / max(crays, 1),
                "trace_kernel_ms_per_frame": trace_ms, "trace_stage_ms_per_frame": tm["rtOnlySum"] / max(tm["frames"], 1),
                "traffic_source": traffic_src}

    # the L2 bound: the scene's records, triangles and vertices (~64 MB) stay in the 126 MB L2 through
    # a frame, so the traversal's roofline is the L2's copy bandwidth, measured here
    l2_read, l2_copy = rgcuda.measure_l2(local, 64 << 20, 64)
    roofline["l2"] = {"peak": l2_read, "frac": achieved / l2_read, "unit": "GB/s", "copy_gbs": l2_copy,
                      "source": "measured in this run by rg_measure_l2: 64 MiB working set (inside the 126 MB L2) read "
                                "with 16-byte loads, 64 passes per launch, best of 4 launches; the traversal's bytes are "
                                "reads of L2-resident records and triangles"}

    # ---------------- incoherent secondary closest-hit throughput ----------------
    # the frame's first-bounce reflection / refraction rays (closesthit.rchit:215,232,244), traced by one
    # launch of the frame loop's traversal kernel per step (rg_trace_rays_device), L2 flushed between
    sec = first_bounce_secondary(ctx, sc, frames.instances[f - 1], dev, 2 * sc.width, 2 * sc.height)
    nsec = len(sec)
    d_tuv = torch.empty(nsec, 3, device=dev)
    d_ids = torch.empty(nsec, 2, dtype=torch.int32, device=dev)
    barrier()
    for _ in range(3):
        ctx.trace_rays_device(sec.data_ptr(), nsec, d_tuv.data_ptr(), d_ids.data_ptr())
    sec_ms = []
    for _ in range(max(5, min(K, 20))):
        with torch.cuda.stream(ext):
            flush.zero_()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(ext)
        ctx.trace_rays_device(sec.data_ptr(), nsec, d_tuv.data_ptr(), d_ids.data_ptr())
        a1.record(ext)
        barrier()
        sec_ms.append(a0.elapsed_time(a1))
    sst = ctx.stats()
    sec_med = statistics.median(sec_ms)
    secondary = {"value": nsec / (sec_med * 1e-3) / 1e9, "unit": "Grays/s", "rays": nsec, "ms_median": sec_med,
                 "stack_overflows": sst["stack_overflows"],
                 "rays_def": "GENERIC reflection + refraction rays at the hits of 3840x2160 pixel-centre camera rays "
                             "(the 4-spp frame's primary-ray count), materials as uploaded",
                 "kernel": "rg_trace_rays_device: one k_wf_trace launch in its query form (rays read from the caller's "
                           "buffer, hits written into the caller's buffers), CUDA events on the library stream, L2 "
                           "flushed before each launch"}

    out = {
        "metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded procedural scene (no dataset)",
        "secondary_grays_per_s": secondary,
        "config": game_config(sc, world),
        "l2": "flushed between frames (256 MiB memset on the library stream)",
        "frames_per_s": K / (ms * 1e-3),
        "rays_per_frame": rays / K,
        "profiler_ranges_ms": {k: tm[k + "Sum"] / max(tm["frames"], 1) for k in
                               ("asBuild", "refit", "rtOnly", "rough", "postproc", "rtTotal")},
        "e2e": e2e, "roofline": roofline, "clocks": clk, "gpu_launches": int(launches),
    }
    if orc_scene is not None:
        out["cpu_baseline"] = cpu_baseline(orc_scene, sc, args.cpu_rows)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


BATCH_WORKLOAD = "batched rendering: {n} independent scenes (instanced tris log-uniform 1k-4M from the game-frame meshes), " \
                 "resolution uniform over 320x180/640x360/1280x720/1920x1080, 1-4 spp, depth 1-6; one CUDA-graph launch " \
                 "per batch (device-side round loop), per-scene roughness + composite + FXAA"


def run_batch(args):
    import torch
    from raygun_gb300 import build as rgbuild, rgcuda

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    rgbuild.build()
    scenes = S.batch_scenes(n=args.batch_scenes)
    br = rgcuda.BatchRenderer(scenes, device=local)
    ctx = br.ctx
    if args.batch_slots:
        ctx.set_batch_slots(args.batch_slots)
    jobs = br.jobs()
    K, W = args.steps, args.warmup
    dev = torch.device("cuda", local)
    ext = torch.cuda.ExternalStream(ctx.stream(), device=dev)
    pixels = [sc.width * sc.height for sc in scenes]

    def barrier():
        torch.cuda.synchronize(dev)
        ctx.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    tune, table = None, None
    t_tune = time.perf_counter()
    if not args.no_tune:
        tune, table = ctx.autotune_batch(jobs, reps=1)
    t_tune = time.perf_counter() - t_tune

    # ---------------- value: scenes and job table resident, one graph launch per batch ----------------
    for _ in range(W):
        ctx.render_batch(jobs)
    barrier()
    ctx.timings()
    ctx.reset_total_stats()
    launches0 = rgcuda.launch_count()
    clocks = ClockSampler(local)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    e0.record(ext)
    for _ in range(K):
        ctx.render_batch(jobs)
    e1.record(ext)
    barrier()
    clk = clocks.stop()
    launches = rgcuda.launch_count() - launches0
    tot = ctx.total_stats()
    rays = tot["primary"] + tot["shadow"] + tot["secondary"]
    value, ms = replica_throughput(rays, e0.elapsed_time(e1), world, dev)

    # ---------------- e2e: job table from host memory, every image read back to pinned host memory ----
    # two pinned buffers: batch b's images are read back (rg_batch_download_async, every image of the
    # batch in job order) while batch b + 1 renders
    fb_pins = [torch.empty(sum(pixels) * 16, dtype=torch.uint8).pin_memory() for _ in range(2)]
    nstep = [0]

    def step_host():
        ctx.render_batch(jobs)
        ctx.batch_download_async(fb_pins[nstep[0] % 2].data_ptr())
        nstep[0] += 1

    for _ in range(W):
        step_host()
    barrier()
    ctx.reset_total_stats()
    t0 = time.perf_counter()
    for _ in range(K):
        step_host()
    barrier()
    dt = (time.perf_counter() - t0) * 1e3
    tot2 = ctx.total_stats()
    e2e_value, ms_e2e = replica_throughput(tot2["primary"] + tot2["shadow"] + tot2["secondary"], dt, world, dev)
    e2e = {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": int(rgcuda.JOB.itemsize * len(jobs)),
           "d2h_bytes_per_step": int(sum(pixels) * 16), "ms_per_step": ms_e2e / K,
           "timing": "host wall clock around K batches; each batch's images are read back to pinned host memory "
                     "(rg_batch_download_async) while the next batch renders, and the clock stops once the last "
                     "batch's images are in host memory"}

    # ---------------- roofline of the traversal launches (host-polled loop with events) ----------------
    ctx.set_flags(rgcuda.RG_FLAG_COUNT_VISITS)
    ctx.render_batch(jobs)
    barrier()
    cst = ctx.stats()
    ctx.set_flags(rgcuda.RG_FLAG_KERNEL_TIMING)
    ctx.timings()
    ctx.render_batch(jobs)
    barrier()
    tm = ctx.timings()
    ctx.set_flags(0)
    crays = cst["primary"] + cst["shadow"] + cst["secondary"]
    bytes_batch = crays * BYTES_RAY + cst["nodes"] * BYTES_NODE + cst["tris"] * BYTES_TRI
    trace_ms = tm["traceKernelSum"] / max(tm["frames"], 1)
    achieved = bytes_batch / (trace_ms * 1e-3) / 1e9
    peak, peak_src = measured_peak_hbm()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": None, "kernel": "k_wf_trace (batch form) + k_wf_tail: every traversal launch of one batch",
                "launches_per_batch": tm["traceLaunches"] / max(tm["frames"], 1), "peak_source": f"{peak_src} hbm_gbs",
                "algorithmic_bytes_per_batch": bytes_batch, "bytes_per_ray": bytes_batch / max(crays, 1),
                "node_visits_per_ray": cst["nodes"] / max(crays, 1), "tri_tests_per_ray": cst["tris"] / max(crays, 1),
                "trace_kernel_ms_per_batch": trace_ms}

    out = {
        "metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded procedural scenes (no dataset)",
        "config": {"workload": BATCH_WORKLOAD.format(n=len(scenes)), "scenes": len(scenes),
                   "instanced_tris": int(sum(sc.instanced_tri_count for sc in scenes)),
                   "unique_tris": int(sum(sc.tri_count for sc in scenes)), "pixels": int(sum(pixels)),
                   "samples": int(sum(p * int(sc.ubo["numSamples"][0]) for p, sc in zip(pixels, scenes))),
                   "l2": "inputs larger than L2 (path state and scene BVHs of the batch are several GB)",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "batches_per_s": K / (ms * 1e-3), "rays_per_batch": rays / K,
        "autotune": None if tune is None else {
            "chosen": {"threads": tune["threads"], "stack_depth": tune["stack_depth"],
                       "sort_key": {v: k for k, v in rgcuda.SORT_KEYS.items()}[tune["sort_key"]]},
            "seconds": t_tune,
            "ms_per_batch": {f"{t}x{d}/{k}": (None if v is None else round(v, 3)) for (t, d, k), v in table.items()}},
        "e2e": e2e, "roofline": roofline, "clocks": clk, "gpu_launches": int(launches),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_batch(scenes)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


SERVE_WORKLOAD = "serving loop: Poisson arrivals at {rate:g} req/s, {n} requests; scenes of the batched-rendering " \
                 "distribution ({small} scenes) or, with probability 0.05, large terrain scenes ({large} scenes of " \
                 "10-60 tessellated 1M-triangle heightfields) at 320x180..3840x2160 and 1-8 spp; the learned roughness " \
                 "filter on a share of the requests; LRU scene residency under a {budget:g} GB HBM budget; waiting " \
                 "requests batched per step; every image read back"


def run_serve(args):
    import torch
    from raygun_gb300 import build as rgbuild, rgcuda, serving as V

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    rgbuild.build()
    small = S.batch_scenes(n=64, seed=4)
    catalog = {f"b{k:02d}": sc for k, sc in enumerate(small)}
    rng = S.Rng(44)
    large_keys = []
    for k in range(args.serve_large):
        fields = 10 + min(int(rng.uniform(1, 0, 51)[0]), 50)
        key = f"t{k:02d}"
        catalog[key] = S.terrain_scene(rng, key, fields, 1920, 1080, 1, 3)
        large_keys.append(key)
    budget = int(args.serve_budget_gb * 1e9)
    ctx = rgcuda.Context(device=local, hbm_budget_bytes=budget,
                         flags=0 if args.serve_graph else rgcuda.RG_FLAG_HOST_LOOP)
    flt = None
    if args.serve_filter_fraction > 0:
        from raygun_gb300 import filter_train
        flt = rgcuda.Filter(ctx, seed=0)
        filter_train.load_weights(flt)
    srv = V.RenderServer(ctx, catalog, budget, learned_filter=flt)
    reqs = V.poisson_requests(args.serve_requests, args.serve_rate, 4, [(k, catalog[k]) for k in catalog if k[0] == "b"],
                              [(k, catalog[k]) for k in large_keys], filter_fraction=args.serve_filter_fraction)
    # a server that has been running: the working buffers of a large batch exist and the catalog is
    # resident as far as the budget allows (catalog order)
    warm = V.poisson_requests(96, args.serve_rate, 40, [(k, catalog[k]) for k in catalog if k[0] == "b"],
                              [(k, catalog[k]) for k in large_keys], large_fraction=0.2,
                              filter_fraction=args.serve_filter_fraction)
    for r in warm:
        r.arrival = 0.0
    t0 = time.perf_counter()
    V.run_open_loop(srv, warm)
    reserve = max(srv._working_held(), 24 << 30)
    for key in catalog:
        if srv.res.resident_bytes() + srv.res.footprint(key) + reserve > budget:
            break
        srv.res.ensure(key)
    t_warm = time.perf_counter() - t0
    srv.rays, srv.batches, srv.batch_sizes = 0, 0, []
    ev0, up0 = srv.res.evictions, srv.res.uploads
    launches0 = rgcuda.launch_count()
    clocks = ClockSampler(local)
    clocks.start()
    results, wall = V.run_open_loop(srv, reqs)
    clk = clocks.stop()
    summary = V.summarize(results, wall, srv.rays)
    ok = [r for r in results if r.ok]
    byid = {r.id: r for r in reqs}
    d2h = sum(byid[r.id].width * byid[r.id].height * 16 for r in ok)
    out = {
        "metric": "Mrays/s", "value": summary["mrays_per_s"], "unit": "Mrays/s", "n_gpus": world,
        "steps": srv.batches, "warmup": 1, "ms_per_step": summary["seconds"] * 1e3 / max(srv.batches, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded procedural scenes and arrivals (no dataset)",
        "config": {"workload": SERVE_WORKLOAD.format(rate=args.serve_rate, n=args.serve_requests, small=len(small),
                                                     large=len(large_keys), budget=args.serve_budget_gb),
                   "catalog_scenes": len(catalog),
                   "catalog_instanced_tris": int(sum(sc.instanced_tri_count for sc in catalog.values())),
                   "catalog_unique_tris": int(sum(int(sc.meshes["triCount"].astype(np.int64).sum()) for sc in catalog.values())),
                   "batch_mode": "graph" if args.serve_graph else "host loop",
                   "filter_fraction": args.serve_filter_fraction,
                   "l2": "inputs larger than L2", "parallelism": "single GPU"},
        "serving": {**summary, "batches": srv.batches, "mean_batch": float(np.mean(srv.batch_sizes)) if srv.batch_sizes else 0.0,
                    "evictions": srv.res.evictions - ev0, "uploads": srv.res.uploads - up0,
                    "resident_scenes_at_start": len(srv.res.slots), "warmup_seconds": t_warm},
        "e2e": {"value": summary["mrays_per_s"], "unit": "Mrays/s",
                "h2d_bytes_per_step": int(rgcuda.JOB.itemsize * len(ok) / max(srv.batches, 1)),
                "d2h_bytes_per_step": int(d2h / max(srv.batches, 1)),
                "timing": "wall clock from the first arrival to the last completion; requests arrive in real time"},
        "roofline": None, "clocks": clk, "gpu_launches": int(rgcuda.launch_count() - launches0),
    }
    if rank == 0:
        print(json.dumps(out), flush=True)


FILTER_FLOPS_PER_PX = 2 * 9 * (12 * 32 + 32 * 64 + 64 * 64 + 64 * 32 + 32 * 3)  # 156,096 (all layers at full resolution)


def measured_peak_bf16():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["bf16_tflops"]), "measured"
    except (OSError, KeyError, ValueError):
        return 1900.0, "fallback"


def run_filter(args):
    import torch
    from raygun_gb300 import build as rgbuild, rgcuda, filter_train as FT

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    rgbuild.build()
    ctx = rgcuda.Context(device=local)
    flt = rgcuda.Filter(ctx, seed=1)
    log = lambda m: print(m, file=sys.stderr, flush=True)
    t0 = time.perf_counter()
    if args.filter_weights:
        FT.load_weights(flt, args.filter_weights)
        data, stats = None, {"loaded": args.filter_weights}
    else:
        X, T = FT.build_dataset(ctx, args.filter_scenes, 640, 360, log=log)
        data = {"scenes": args.filter_scenes, "frame": "640x360", "seconds": time.perf_counter() - t0}
        stats = FT.train(flt, X, T, args.filter_crops, args.filter_epochs, log=log)
        del X, T
        if args.filter_save:
            FT.save_weights(flt, args.filter_save)
    mean, rows = FT.evaluate(flt, args.filter_eval, log=log)
    times = FT.post_times(flt)
    px = 1920 * 1080
    filt_ms = times["learned"]["rough_ms"]
    achieved = FILTER_FLOPS_PER_PX * px / (filt_ms * 1e-3) / 1e12
    peak, src = measured_peak_bf16()
    out = {
        "metric": "rough-reflection PSNR (dB) of the learned filter against 256-spp glossy references",
        "value": mean["rough_psnr_learned"], "unit": "dB", "n_gpus": world, "steps": stats.get("steps", 0), "warmup": 0,
        "ms_per_step": filt_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (fp32 accumulate)",
        "data": "synthetic: training frames and 256-spp glossy targets rendered by the tracer from seeded scenes (no dataset)",
        "config": {"workload": "learned roughness filter: 5-layer 3x3 conv 12-32-64-64-32-3, ReLU, skip 1->5, BF16 / FP32 "
                               "accumulate on tcgen05; trained on 128x128 crops of 1-spp G-buffers vs 256-spp glossy renders; "
                               "evaluated on held-out 1080p frames", "training_scenes": args.filter_scenes,
                   "crops": args.filter_crops, "epochs": args.filter_epochs, "eval_scenes": args.filter_eval,
                   "parallelism": "single GPU"},
        "quality": mean, "quality_per_scene": rows, "training": stats, "dataset": data,
        "post_times_ms": times,
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak, "traffic": None,
                     "kernel": "filter stage of a 1080p frame (G-buffer pack, 5 convolutions, composite); FLOPs counted "
                               f"{FILTER_FLOPS_PER_PX} per pixel", "peak_source": f"{src} bf16_tflops"},
        "frame_time_ratio": times["learned"]["frame_ms"] / times["plain"]["frame_ms"],
    }
    print(json.dumps(out), flush=True)


def cpu_baseline_batch(scenes, min_seconds=10.0, max_passes=10):
    """The oracle on all host cores over the whole batch (every scene, every row), repeated until at
    least `min_seconds` of CPU work."""
    import oracle
    nthreads = os.cpu_count() or 1
    orcs = [oracle.OracleScene(sc) for sc in scenes]
    rays, dt, n = 0, 0.0, 0
    while n < max_passes and (n == 0 or dt < min_seconds):
        for o, sc in zip(orcs, scenes):
            t = time.perf_counter()
            _, _, _, st = o.render(rows=(0, sc.height), row_step=1, nthreads=nthreads)
            dt += time.perf_counter() - t
            rays += st["primary"] + st["shadow"] + st["secondary"]
        n += 1
    return {"value": rays / dt / 1e6, "unit": "Mrays/s", "cores": nthreads, "kind": "port",
            "sample": f"{n} passes over all {len(scenes)} scenes (every row): {rays} rays in {dt:.2f} s (trace + shade)"}


def cpu_baseline(orc_scene, sc, rows, min_seconds=10.0, max_renders=20):
    """The oracle on all host cores: full renders of frame 0 repeated until at least `min_seconds`
    of CPU work (the frame takes ~2 s on 16 cores).  `rows` > 0 renders only that many rows spread
    over the frame per render (a shorter sample, for quick runs)."""
    nthreads = os.cpu_count() or 1
    step = max(1, sc.height // rows) if rows > 0 else 1
    rays, dt, n = 0, 0.0, 0
    while n < max_renders and (n == 0 or dt < min_seconds):
        t = time.perf_counter()
        _, _, _, st = orc_scene.render(rows=(0, sc.height), row_step=step, nthreads=nthreads)
        dt += time.perf_counter() - t
        rays += st["primary"] + st["shadow"] + st["secondary"]
        n += 1
    nrows = (sc.height + step - 1) // step
    what = "full frame 0" if step == 1 else f"every {step}th row of frame 0 ({nrows} rows)"
    return {"value": rays / dt / 1e6, "unit": "Mrays/s", "cores": nthreads, "kind": "port",
            "sample": f"{n} renders of the {what} ({sc.width} px wide, {int(sc.ubo['numSamples'][0])} spp): "
                      f"{rays} rays in {dt:.2f} s (trace + shade)"}


def run_spheres(args):
    """The single-level sphere scene (640x360, 1 spp, depth 4, 61,442 triangles; the reference's
    CPU-runnable case): GPU frame time and Mrays/s with the scene resident, the same frames read back
    to pinned host memory (e2e), and the oracle on every host core rendering the same frame."""
    import torch
    from raygun_gb300 import build as rgbuild, rgcuda
    import oracle

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    rgbuild.build()
    sc = S.sphere_scene()
    rt = rgcuda.Raytracer(sc, device=local).prepare()
    ctx = rt.ctx
    K, W = max(args.steps, 10), max(args.warmup, 3)
    for _ in range(W):
        rt.do_raytracing()
    ctx.synchronize()
    ctx.timings()
    ctx.reset_total_stats()
    for _ in range(K):
        rt.do_raytracing()
    ctx.synchronize()
    t = ctx.timings()
    st = ctx.total_stats()
    rays = st["primary"] + st["shadow"] + st["secondary"]
    frame_ms = t["rtTotalSum"] / t["frames"]
    value = rays / (t["rtTotalSum"] * 1e-3) / 1e6
    # two pinned framebuffers: frame f's read-back overlaps frame f + 1 (rg_download_async)
    hosts = [torch.empty(sc.height * sc.width * 4, dtype=torch.float32).pin_memory() for _ in range(2)]
    t0 = time.perf_counter()
    for k in range(K):
        rt.do_raytracing()
        ctx.download_async(hosts[k % 2].data_ptr())
    ctx.synchronize()
    e2e_ms = (time.perf_counter() - t0) / K * 1e3
    o = oracle.OracleScene(sc)
    cores = os.cpu_count() or 1
    o.render(nthreads=cores)
    t0 = time.perf_counter()
    n_cpu = 0
    cpu_rays = 0
    while time.perf_counter() - t0 < 5.0 and n_cpu < 20:
        _, _, _, cs = o.render(nthreads=cores)
        cpu_rays += cs["primary"] + cs["shadow"] + cs["secondary"]
        n_cpu += 1
    cpu_dt = time.perf_counter() - t0
    out = {"metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": K, "warmup": W, "ms_per_step": frame_ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic: seeded procedural scene (no dataset)",
           "config": {"workload": "spheres: 640x360, 1 spp, depth 4, ground quad + 64 UV spheres (61,442 tris), single-level BVH",
                      "width": sc.width, "height": sc.height, "parallelism": "single GPU"},
           "rays_per_frame": rays / K, "frame_ms": frame_ms,
           "e2e": {"value": rays / K / (e2e_ms * 1e-3) / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": sc.height * sc.width * 16, "ms_per_step": e2e_ms},
           "cpu_baseline": {"value": cpu_rays / cpu_dt / 1e6, "unit": "Mrays/s", "cores": cores, "kind": "port",
                            "sample": f"{n_cpu} renders of the whole frame (trace + shade), {cpu_dt:.2f} s"}}
    print(json.dumps(out), flush=True)


def run_reference(args):
    """Reference arm: the reference's path on the host cores.  Raygun's own GPU path needs a Vulkan
    ray-tracing driver (unavailable on this machine), so each step is the frame on the CPU: the frame's
    BLAS refits and TLAS rebuild (the oracle's, standing in for the driver's), then the reference's
    own raygen / closest-hit / miss shaders over every pixel and its compute post passes (the
    reference-compiled checker, oracle/_ref: Raygun's GLSL compiled as C++), on all host threads.
    Where that checker is not built, the oracle's restatement of the same shaders runs instead
    (kind "port").  The frames are the GPU arm's frames (same animation, frames 0 .. W+K-1).  Whole
    frames are traced; only if K + W whole frames would take more than 4 minutes are rows sampled,
    with the refit, TLAS and post time scaled to the rows traced."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle
    oracle.build()
    from oracle import ref as oref
    kind, note = "port", "oracle restatement of the reference shaders (reference-compiled checker not built here)"
    if oref.reference_present() or oref.staged_present():
        try:
            oref.build()
            oref.lib()
            kind, note = "reference", "the reference's own shaders compiled as C++ (oracle/_ref)"
        except Exception as e:  # the port stands in
            note = f"oracle restatement (reference-compiled checker failed to build: {str(e)[:120]})"
    w, h = (int(x) for x in args.res.split("x"))
    sc = S.instanced_scene(width=w, height=h)
    o = oracle.OracleScene(sc)
    nthreads = os.cpu_count() or 1
    K, W = args.steps, args.warmup
    frames = FrameInputs(sc, W + K)

    def step(f, row_step):
        t0 = time.perf_counter()
        for b, vo, nv, arr in frames.refits[f]:
            o.refit(b, arr, vo)
        o.set_instances(frames.instances[f])
        t1 = time.perf_counter()
        r0 = f % row_step
        if kind == "reference":
            base, nrm, rough, rays = oref.render_scene(o, sc.ubo, w, h, nthreads=nthreads, rows=(r0, row_step))
        else:
            base, nrm, rough, st = o.render(rows=(r0, h), row_step=row_step, nthreads=nthreads)
            rays = st["primary"] + st["shadow"] + st["secondary"]
        t2 = time.perf_counter()
        if kind == "reference":
            oref.post(sc.ubo, base, nrm, rough, fxaa=True, nthreads=nthreads)
        else:
            oracle.post(sc.ubo, base, nrm, rough, fxaa=True, nthreads=nthreads)
        t3 = time.perf_counter()
        frac = len(range(r0, h, row_step)) / h
        return rays, ((t1 - t0) + (t3 - t2)) * frac + (t2 - t1)

    # the first warm-up frame (whole) sizes the sample
    _, t_frame = step(0, 1)
    budget = 240.0
    row_step = 1 if t_frame * (W + K) <= budget else int(np.ceil(t_frame * (W + K) / budget))
    for f in range(1, W):
        step(f, row_step)
    rays, dt = 0, 0.0
    for k in range(K):
        r, t = step(W + k, row_step)
        rays += r
        dt += t
    v = rays / dt / 1e6
    what = "whole frames" if row_step == 1 else f"every {row_step}th row (refit, TLAS and post time scaled to the rows traced)"
    out = {"metric": "Mrays/s", "value": v, "unit": "Mrays/s", "n_gpus": world, "steps": K, "warmup": W,
           "ms_per_step": dt / K * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic: seeded procedural scene (no dataset)", "impl": "reference",
           "config": game_config(sc, world),
           "cpu_baseline": {"value": v, "unit": "Mrays/s", "cores": nthreads, "kind": kind,
                            "sample": f"{K} frames, {what}: BLAS refits + TLAS rebuild, raygen / closest-hit / miss "
                                      f"over the frame, roughness + composite + FXAA passes; {note}; the reference's "
                                      f"Vulkan RT path needs a ray-tracing driver, unavailable on this box"},
           "e2e": {"value": v, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def launch_replicas(n):
    """--gpus N without a launcher around us: start N ranks of this same command line, one per GPU
    (RANK / LOCAL_RANK / WORLD_SIZE / MASTER_* in their environment, as torchrun sets them), and wait
    for them; rank 0 prints the JSON line.  Returns the worst exit code."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    procs = []
    for r in range(n):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(n), LOCAL_WORLD_SIZE=str(n),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, os.path.abspath(__file__), *sys.argv[1:]], env=env))
    return max(p.wait() for p in procs)


def run_dist_check(args):
    """The N > 1 plumbing without a GPU: each rank joins a gloo group and reports synthetic counts
    (rank r: (r + 1) * 1e6 rays in 10 + r ms); rank 0 prints the aggregate line."""
    import torch.distributed as dist
    rank, world, _ = dist_env()
    if world > 1:
        dist.init_process_group("gloo")
    value, ms = replica_throughput((rank + 1) * 1e6, 10.0 + rank, world, "cpu")
    if rank == 0:
        print(json.dumps({"metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": world, "ms_per_step": ms,
                          "workload": "dist-check"}), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def main():
    args = parse()
    if args.gpus > 1 and "RANK" not in os.environ:
        sys.exit(launch_replicas(args.gpus))
    if args.workload == "dist-check":
        run_dist_check(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload == "filter":
        run_filter(args)
    elif args.workload == "spheres":
        run_spheres(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
