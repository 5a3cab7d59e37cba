"""Benchmark: clustered light assignment at 1920x1080 with 16,384 point lights (ms per frame),
plus radix-sort throughput (Gkeys/s, % of HBM) and the primitive sweep, on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one frame through vren::cluster_and_shade's clustering half (construct_point_light_bvh,
find_unique_cluster_list, assign_lights) replayed as a CUDA graph, inputs resident in HBM, L2
flushed (a 256 MiB write) before every timed step, each step timed with CUDA events on its stream.
`e2e` runs the same frames through the public API from pinned host buffers: host->device copy of
the G-buffer and lights, the pipeline, and a device->host read of the cluster references and the
per-cluster light lists, all inside the timed region.

--impl reference times the reference's CPU implementation of the path (the restated CPU oracle of
oracle/, since loryruta/vren's own code needs Vulkan) with all host threads.
Multi-GPU: frames are independent, so N ranks run N frame streams with no collective (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "1080p/16k-light cluster assign ms; radix sort Gkeys/s, %HBM; batched vs plain"
W, H, L = 1920, 1080, 16384
SEED = 20240611
RADIX_N = 1 << 20
L2_FLUSH_BYTES = 256 << 20
BYTES_PER_PX = 20  # depth 4 + normal 12 (f32x3) + cluster reference 4
# DRAM bytes (read + write) of one find_unique_cluster_list call at 1920x1080 (its two kernels, f32x3
# normals): one ncu capture at 3840x2160 (`--profile find_unique`: tile kernel 133.8 MB read + 17.6 MB
# written, self-offset fix-up 34.3 MB read) scaled by the pixel count (1/4).  ncu flushed the caches
# before each kernel, so the fix-up's read of the references (L2-resident in a timed run) is counted
# here.
FUC_TRAFFIC_BYTES = int((133.848320 + 17.563392 + 34.263296 + 0.001024) * 1e6 / 4)
FUC_TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of the two kernels (tiles, self-offset "
                      "fix-up) at 3840x2160 (caches flushed before each), scaled by pixels to 1920x1080")


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples during the timed region: median SM clock under load and throttle reasons."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int = 0):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def wait_first(self, timeout: float = 5.0):
        """Returns once nvidia-smi has printed its first sample, i.e. is past its start-up."""
        t0 = time.perf_counter()
        while self.proc is not None and not self.lines and time.perf_counter() - t0 < timeout:
            time.sleep(0.01)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------------------------------------
# Inputs (identical for both arms)
# ------------------------------------------------------------------------------------------------
def make_inputs(rank: int = 0):
    """Depth, normals f32x3 (the benchmark's G-buffer) and the same normals rounded into the reference's
    own G-buffer format RGBA16F (a labelled extra measurement), light positions, point lights, radix keys."""
    import vren_gb300.scene as scene

    depth, normals = scene.depth_planes(SEED + rank, W, H, planes=64)
    normals_h = np.zeros((W * H, 4), np.float16)
    normals_h[:, :3] = normals.reshape(-1, 3).astype(np.float16)
    pos, lights = scene.lights(SEED + 1000 + rank, L, W, H)
    keys = scene.gen_u32(SEED + 7, 1, RADIX_N)
    return depth, normals, normals_h, pos, lights, keys


# ------------------------------------------------------------------------------------------------
# Our arm
# ------------------------------------------------------------------------------------------------
def job_ms_over_ranks(local_ms_sum: float, steps: int, world: int, device) -> float:
    """Effective ms per frame of the whole job: frames are independent replicas, so the job's time is
    the slowest rank's timed total over the frames all ranks processed (steps x world)."""
    if world <= 1:
        return local_ms_sum / steps
    import torch

    t = torch.tensor([local_ms_sum], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item()) / (steps * world)


def run_ours(args, rank: int, world: int):
    import torch

    import vren_gb300 as vg
    import vren_gb300.clustered_shading as cs
    from vren_gb300 import _build

    _build.build()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    hbm_peak, peak_kind = peaks()
    depth, normals, normals_h, pos, lights, radix_keys = make_inputs(rank)
    stream = torch.cuda.Stream(device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)
    # Written once here: the first write to the fresh 256 MiB buffer is slow and, measured, adds
    # ~40 us to the device time of the frame that follows it.
    flush.zero_()

    cam = cs.scene_camera(W, H)
    view = cs.view_from_camera(cam, "ref")
    ctx = cs.cluster_and_shade(W, H, 65536, 1 << 24)
    d_depth = torch.from_numpy(depth).to(dev)
    d_norm = torch.from_numpy(normals).to(dev)
    d_pos = torch.from_numpy(pos).to(dev)
    d_light = torch.from_numpy(lights).to(dev)
    torch.cuda.synchronize()

    def frame():
        ctx.cluster(stream, view, W, H, d_depth, d_norm, d_pos, d_light, L)

    # The clock sampler spans the warm-up and all GPU work below (the frame loop alone is ~10 ms).  It
    # is started, and past its start-up, before the warm-up: a stall of this thread inside the timed
    # loop lets the device drain its queue and idle between a step's start event and its frame.
    clocks = ClockSampler(dev.index).__enter__().wait_first()
    # warm-up (captures the graph on the first call)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            frame()
    stream.synchronize()
    out = ctx.outputs()
    U = int(cs.read_device(out.key_count, 1)[0])
    total = int(cs.read_device(out.total, 1)[0])

    # timed region
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t_wall0 = time.perf_counter()
    with torch.cuda.stream(stream):
        # A 1 ms spin ahead of the first step (outside every step's events), so the host queues the
        # steps ahead of the device and no step's device time can take in the host's launch latency.
        torch.cuda._sleep(2_000_000)
        for i in range(args.steps):
            flush.zero_()
            ev[i][0].record(stream)
            frame()
            ev[i][1].record(stream)
        stream.synchronize()
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    ms_frame = sum(step_ms) / len(step_ms)
    job_ms = job_ms_over_ranks(sum(step_ms), args.steps, world, dev)
    err = vg.device_error()

    # dominant HBM kernel of the frame: find_unique_cluster_list (20 B/px), timed alone
    frame_dev = torch.empty(0)
    fr = cs.frame_build(view, W, H)
    frame_dev = cs.frame_to_device(fr, dev)
    T = ((W + 31) // 32) * ((H + 31) // 32)
    keys = torch.zeros(T * 1024, dtype=torch.int32, device=dev)
    kc = torch.zeros(1, dtype=torch.int32, device=dev)
    refs = torch.zeros(W * H, dtype=torch.int32, device=dev)
    fuc = cs.find_unique_cluster_list()
    kt = []
    with torch.cuda.stream(stream):
        for i in range(args.warmup + args.steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fuc(stream, W, H, frame_dev, d_depth, d_norm, keys, kc, refs)
            b.record(stream)
            if i >= args.warmup:
                kt.append((a, b))
        stream.synchronize()
    fuc_ms = sum(a.elapsed_time(b) for a, b in kt) / len(kt)
    fuc_bytes = BYTES_PER_PX * W * H
    fuc_gbs = fuc_bytes / (fuc_ms * 1e-3) / 1e9

    # end to end through the public API from pinned host buffers: vren_cs_cluster_host uploads the
    # G-buffer in bands (each band's tiles start on arrival) and the lights (their BVH built during the
    # G-buffer upload), downloads the cluster references during the light assignment, and has the
    # device write the light lists ([U, total, keys, counts, offsets, indices]) into host memory.
    h_depth = torch.from_numpy(depth).pin_memory()
    h_norm = torch.from_numpy(normals).pin_memory()
    h_pos = torch.from_numpy(pos).pin_memory()
    h_light = torch.from_numpy(lights).pin_memory()
    h_refs = torch.empty(W * H, dtype=torch.int32).pin_memory()
    cap = T * 1024
    h_lists = torch.empty(2 + 3 * cap + (1 << 24), dtype=torch.int32).pin_memory()

    h2d_bytes = sum(t.numel() * t.element_size() for t in (h_depth, h_norm, h_pos, h_light))
    lists_host = h_lists.numpy()  # the result is read from page-locked host memory
    zc_knob = vg._lib.TUNE["host_zero_copy"]
    zc_default = vg.lib().vren_tuning_get(zc_knob)

    def run_e2e(zero_copy: int):
        vg.lib().vren_tuning_set(zc_knob, zero_copy)
        times, d2h = [], 0
        for i in range(args.warmup + args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            with torch.cuda.stream(stream):
                ctx.cluster_host(stream, view, W, H, h_depth, h_norm, h_pos, h_light, L, h_refs, h_lists)
                stream.synchronize()
            u, tot = int(lists_host[0]), int(lists_host[1])
            if i >= args.warmup:
                times.append((time.perf_counter() - t0) * 1e3)
                d2h = 8 + W * H * 4 + u * 12 + tot * 4
        ok = bool(np.array_equal(h_refs.numpy(), cs.read_device(out.cluster_refs, W * H).view(np.int32)))
        return sum(times) / len(times), d2h, ok

    # both host-input forms (the G-buffer copied up in bands / read over the link by the kernel); the
    # headline is the library's default form
    e2e_forms = {}
    for zc, name in ((0, "banded_copies"), (1, "zero_copy_kernel_reads")):
        ms_f, _, ok_f = run_e2e(zc)
        e2e_forms[name] = {"ms": round(ms_f, 4), "refs_match_device": ok_f}
    e2e, d2h_total, e2e_refs_ok = run_e2e(zc_default)
    vg.lib().vren_tuning_set(zc_knob, zc_default)
    link = link_bench(dev, stream, h2d_bytes, d2h_total, max(5, args.steps), e2e)

    # extra, labelled: the same frame with 16384 lights packed in front of the camera, so that the
    # light lists are long (the workload's lights, uniform over a frustum box 1000 deep, reach few of
    # the visible clusters)
    import vren_gb300.scene as scene

    dpos, dlights = scene.lights_near_camera(SEED + 77, L)
    d_dpos, d_dlights = torch.from_numpy(dpos).to(dev), torch.from_numpy(dlights).to(dev)
    dense_ms = time_events(stream, lambda: ctx.cluster(stream, view, W, H, d_depth, d_norm, d_dpos, d_dlights, L), 3,
                           args.steps, flush)
    od = ctx.outputs()
    dense = {"frame_ms": round(dense_ms, 5), "assignments": int(cs.read_device(od.total, 1)[0]),
             "unique_clusters": int(cs.read_device(od.key_count, 1)[0]),
             "lights": "16384 lights uniform in x [-8, 8], y [-5, 5], z [0.5, 25], radius lognormal(ln 2, 0.5)"}

    # extra, labelled: the same frame with 32 exponential depth slices (FIXED32) instead of the
    # reference's slicing
    view32 = cs.view_from_camera(cam, "fixed32")
    f32s_ms = time_events(stream, lambda: ctx.cluster(stream, view32, W, H, d_depth, d_norm, d_pos, d_light, L), 3,
                          args.steps, flush)
    o32 = ctx.outputs()
    fixed32 = {"frame_ms": round(f32s_ms, 5), "unique_clusters": int(cs.read_device(o32.key_count, 1)[0]),
               "assignments": int(cs.read_device(o32.total, 1)[0]),
               "slicing": "32 exponential slices: near * (far/near)^(k/32)"}

    # extra, labelled: the frame with each form of the unique-cluster stage (a fresh context each, the
    # form being read when the frame's graph is captured)
    lib = vg.lib()
    knob = vg._lib.TUNE["fuc_fused"]
    fuc_forms = {}
    for form, name in ((0, "tiles+self_offset_fixup"), (1, "tiles+scan+fixup"), (2, "one_kernel_lookback")):
        lib.vren_tuning_set(knob, form)
        ctx_f = cs.cluster_and_shade(W, H, 65536, 1 << 24)
        fuc_forms[name] = round(time_events(stream, lambda: ctx_f.cluster(stream, view, W, H, d_depth, d_norm, d_pos,
                                                                           d_light, L), 3, args.steps, flush), 5)
        del ctx_f
    lib.vren_tuning_set(knob, 0)

    # extra, labelled: cluster_and_shade::operator() in one call (clustering, then shading over the
    # context's own light lists, one graph): the workload's frame with a seeded G-buffer (its normals are
    # the depth planes' normals), reference falloff, colour output with ambient and gamma
    gn_, galb, grough, gmetal = scene.gbuffer(SEED + 11, W, H)
    d_alb, d_rough, d_metal = (torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (galb, grough, gmetal))
    gbuf = cs.gbuffer(d_depth, d_norm, d_alb, d_rough, d_metal)
    img = torch.empty(W * H * 3, dtype=torch.float32, device=dev)
    cas_ms = time_events(stream, lambda: ctx(stream, view, W, H, gbuf, d_pos, d_light, L, img), 3, args.steps, flush)
    ocs = ctx.outputs()
    cluster_and_shade = {"frame_ms": round(cas_ms, 5), "assignments": int(cs.read_device(ocs.total, 1)[0]),
                         "path": "vren_cs_cluster_and_shade: light BVH, unique clusters, light lists, then shade "
                                 "(f32x3 colour out), one graph replay"}

    # extra, labelled: the frame with its normals in the reference's own G-buffer format (RGBA16F,
    # 8 B/px instead of 12), on the device and end to end from host buffers
    d_norm16 = torch.from_numpy(normals_h).to(dev)
    f16_ms = time_events(stream, lambda: ctx.cluster(stream, view, W, H, d_depth, d_norm16, d_pos, d_light, L), 3,
                         args.steps, flush)
    h_norm16 = torch.from_numpy(normals_h).pin_memory()
    e2e16 = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with torch.cuda.stream(stream):
            ctx.cluster_host(stream, view, W, H, h_depth, h_norm16, h_pos, h_light, L, h_refs, h_lists)
            stream.synchronize()
        u16 = int(lists_host[0])
        if i >= args.warmup:
            e2e16.append((time.perf_counter() - t0) * 1e3)
    rgba16f = {"frame_ms": round(f16_ms, 5), "e2e_ms": round(sum(e2e16) / len(e2e16), 4),
               "h2d_bytes_per_step": h2d_bytes - h_norm.numel() * 4 + h_norm16.numel() * 2, "unique_clusters": u16,
               "note": "normals rounded to half and passed as the reference's RGBA16F G-buffer "
                       "(vren/pipeline/gbuffer.cpp:7-12); other inputs as the main line"}

    # radix sort: 2^20 key/value pairs (config 1), plus sizes beyond L2
    radix = radix_bench(args, dev, stream, flush, radix_keys, hbm_peak)
    sweep = None if args.quick else primitive_sweep(args, dev, stream, flush, hbm_peak)
    shade_host, shade = shade_bench(args, dev, stream, flush, ctx)
    batched = None if args.quick else batched_vs_plain(args, dev, stream, flush)
    lbvh = None if args.quick else lbvh_bench(args, dev, stream, flush, depth, normals, pos, lights, view)
    debug_views = None if args.quick else debug_views_bench(args, dev, stream, flush, ctx, hbm_peak)
    bouncer = None if args.quick else bouncer_bench(args, dev, stream, flush, hbm_peak)
    animated = None if args.quick else animated_bench(args, dev, stream, flush, ctx, depth, normals, pos, lights,
                                                      view)
    pyramid = None if args.quick else depth_pyramid_bench(args, dev, stream, flush, hbm_peak)
    kdtree = None if args.quick else kd_tree_bench(args, dev, stream, flush)

    clocks.__exit__(None, None, None)
    clk = clocks.summary()
    peak32 = fp32_peak_tflops(clk["sm_mhz"])
    shade["roofline"] = {"bound": "fp32", "peak": round(peak32, 2), "unit": "TFLOP/s",
                         "peak_kind": "nominal (152 SMs x 128 FP32 lanes x 2 at the sampled SM clock)",
                         "forward_frac": round(shade["forward_tflops"] / peak32, 4),
                         "backward_frac": round(shade["backward_tflops"] / peak32, 4)}
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(depth, normals, pos, lights, radix_keys, view, shade_host)

    # light BVH at 16384 lights: one kernel on a 16-CTA cluster (1); unique clusters: tiles, then a
    # fix-up that sums the preceding tile counts itself (2); assignment: count, scan, write (3)
    launches_per_frame = 6
    if rank == 0:
        res = {
            "metric": METRIC,
            "value": round(job_ms, 5),
            "unit": "ms",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": round(ms_frame, 5),
            "step_ms": {"median": round(float(np.median(step_ms)), 5), "min": round(min(step_ms), 5),
                        "max": round(max(step_ms), 5), "first": round(step_ms[0], 5)},
            "higher_is_better": False,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32+u32",
            "data": "synthetic (seeded PCG32 scene: 64 oriented planar discs, 16384 point lights)",
            "config": {
                "workload": "cluster assignment 1920x1080, 16384 lights, 32x32 tiles, REF slicing, 15-bit Morton, "
                            "a6+a7+a8 per frame (construct light BVH, unique clusters, assign lights)",
                "unique_clusters": U, "assignments": total,
                "l2": "flushed (256 MiB write) before every timed step",
                "graph": "one CUDA graph replay per frame",
                "normals": "f32x3 per pixel",
                "parallelism": f"replicas x{world} (frames are independent)",
            },
            "e2e": {"value": round(e2e, 4), "unit": "ms", "h2d_bytes_per_step": h2d_bytes,
                    "d2h_bytes_per_step": d2h_total,
                    "path": "vren_cs_cluster_host from pinned buffers, the library's default host-input form "
                            "(" + ("the unique-cluster kernel reading the G-buffer and writing the references over "
                                   "the link" if zc_default else "banded G-buffer upload overlapping the light BVH "
                                   "and the unique-cluster tiles, reference download overlapping the assignment")
                            + "; light lists written to host memory by the device); host wall clock",
                    "forms_ms": e2e_forms,
                    "refs_match_device": e2e_refs_ok},
            "link": link,
            "normals_rgba16f": rgba16f,
            "dense_lights": dense,
            "fixed32_slicing": fixed32,
            "unique_cluster_forms_frame_ms": fuc_forms,
            "cluster_and_shade": cluster_and_shade,
            "gpu_launches": launches_per_frame * args.steps,
            "roofline": {"bound": "hbm", "kernel": "find_unique_cluster_list (find_unique_kernel, "
                                                     "find_unique_fixup_self_kernel)",
                         "achieved": round(fuc_gbs, 1),
                         "peak": hbm_peak, "unit": "GB/s", "frac": round(fuc_gbs / hbm_peak, 4),
                         "peak_kind": peak_kind, "traffic": FUC_TRAFFIC_BYTES,
                         "traffic_source": FUC_TRAFFIC_SOURCE,
                         "algorithmic_bytes": fuc_bytes, "kernel_ms": round(fuc_ms, 5)},
            "radix_sort": radix,
            "batched_vs_plain": batched,
            "primitive_sweep": sweep,
            "shade": shade,
            "karras_lbvh": lbvh,
            "light_bouncer": bouncer,
            "animated_frames": animated,
            "depth_pyramid": pyramid,
            "cluster_debug_views": debug_views,
            "kd_tree": kdtree,
            "cpu_baseline": cpu,
            "clocks": clk,
            "device_error": err,
            "wall_s_timed": round(t_wall, 4),
        }
        # the three targets of the workload definition, last on the line (the record keeps its tail)
        r26 = (radix or {}).get("n=2^26", {})
        adj = (cpu or {}).get("adjoint_check") or {}
        res["targets"] = {
            "radix_hbm_frac_2^26_pairs": r26.get("hbm_frac"), "radix_target": 0.60,
            "radix_bit_exact_2^20": (radix or {}).get("n=2^20", {}).get("bit_exact_vs_stable_sort"),
            "batched_speedup": (batched or {}).get("speedup"),
            "batched_bit_exact_all_frames": (batched or {}).get("bit_exact_all_frames"),
            "adjoint_rel_err_vs_fp64": adj.get("rel_err_max_group"), "adjoint_target": 1e-4,
            "adjoint_lights_checked": adj.get("lights_checked"),
            "e2e_ms": round(e2e, 4), "e2e_link_floor_ms": link["e2e_floor_ms"],
            "frame_ms": round(ms_frame, 5),
            "bucket_sort_hbm_frac_2^24_10bit": ((sweep or {}).get("bucket_sort_2^24_10bit") or {}).get("hbm_frac"),
        }
        print(json.dumps(res), flush=True)


def link_bench(dev, stream, up_bytes: int, down_bytes: int, steps: int, e2e_ms: float):
    """The host <-> device link at the end-to-end frame's byte counts (page-locked buffers, CUDA events):
    the upload alone, the download alone, and both at once on two streams.  Moving a frame's bytes both
    ways at once is the floor of the end-to-end frame; `frac` = that floor / the measured e2e time."""
    import torch

    up_h = torch.empty(up_bytes // 4, dtype=torch.int32).pin_memory()
    up_d = torch.empty(up_h.numel(), dtype=torch.int32, device=dev)
    dn_d = torch.zeros(down_bytes // 4, dtype=torch.int32, device=dev)
    dn_h = torch.empty(dn_d.numel(), dtype=torch.int32).pin_memory()
    side = torch.cuda.Stream(device=dev)

    def up():
        up_d.copy_(up_h, non_blocking=True)

    def down():
        dn_h.copy_(dn_d, non_blocking=True)

    def both():
        fork = torch.cuda.Event()
        fork.record(stream)
        side.wait_event(fork)
        with torch.cuda.stream(side):
            down()
        up()
        join = torch.cuda.Event()
        join.record(side)
        stream.wait_event(join)

    ms_up = time_events(stream, up, 3, steps)
    ms_down = time_events(stream, down, 3, steps)
    ms_both = time_events(stream, both, 3, steps)
    return {"h2d_bytes": up_bytes, "d2h_bytes": down_bytes, "h2d_ms": round(ms_up, 4), "d2h_ms": round(ms_down, 4),
            "h2d_gbs": round(up_bytes / (ms_up * 1e6), 1), "d2h_gbs": round(down_bytes / (ms_down * 1e6), 1),
            "both_ms": round(ms_both, 4), "both_gbs": round((up_bytes + down_bytes) / (ms_both * 1e6), 1),
            "e2e_floor_ms": round(ms_both, 4), "e2e_frac_of_floor": round(ms_both / e2e_ms, 4),
            "note": "page-locked copies, upload and download at once on two streams: the link carries "
                    "the frame's bytes no faster; e2e_frac_of_floor = floor / e2e"}


def time_events(stream, fn, warmup, steps, flush=None):
    import torch

    evs = []
    with torch.cuda.stream(stream):
        for i in range(warmup + steps):
            if flush is not None:
                flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            if i >= warmup:
                evs.append((a, b))
        stream.synchronize()
    return sum(a.elapsed_time(b) for a, b in evs) / len(evs)


def lbvh_bench(args, dev, stream, flush, depth, normals, pos, lights, view):
    """Light assignment through the Karras tree (extension) against the 32-ary traversal, on the
    cluster-assignment frame (1920x1080, 16384 lights uniform in the frustum box) and on the same
    frame with 16384 lights packed near the camera (many lights per cluster)."""
    import torch

    import vren_gb300 as vg
    import vren_gb300.clustered_shading as cs
    import vren_gb300.scene as scene

    frame = cs.frame_to_device(cs.frame_build(view, W, H), dev)
    T = ((W + 31) // 32) * ((H + 31) // 32)
    keys = torch.zeros(T * 1024, dtype=torch.int32, device=dev)
    kc = torch.zeros(1, dtype=torch.int32, device=dev)
    refs = torch.zeros(W * H, dtype=torch.int32, device=dev)
    cs.find_unique_cluster_list()(stream, W, H, frame, torch.from_numpy(depth).to(dev),
                                  torch.from_numpy(normals).to(dev), keys, kc, refs)
    out = {}
    for name, (p, q) in (("uniform_frustum_lights", (pos, lights)), ("lights_near_camera", scene.lights_near_camera(SEED + 77, L))):
        P = vg.calc_bvh_padded_leaf_count(L)
        vp = torch.zeros(L * 4, dtype=torch.float32, device=dev)
        bvh = torch.zeros(vg.calc_bvh_buffer_length(P) * 8, dtype=torch.int32, device=dev)
        lidx = torch.zeros(L * 2, dtype=torch.int32, device=dev)
        sph = torch.zeros(P * 4, dtype=torch.float32, device=dev)
        cs.construct_point_light_bvh(15)(stream, torch.from_numpy(p).to(dev), torch.from_numpy(q).to(dev), L, frame,
                                         vp, bvh, lidx, sph)
        nodes = torch.zeros((L - 1) * 8, dtype=torch.int32, device=dev)
        boxes, shift = cs.build_lbvh.group_boxes(bvh, L)
        cap = keys.numel()
        res = []
        for kind in ("32ary", "lbvh"):
            counts = torch.zeros(cap, dtype=torch.int32, device=dev)
            offsets = torch.zeros(cap, dtype=torch.int32, device=dev)
            indices = torch.zeros(1 << 24, dtype=torch.int32, device=dev)
            total = torch.zeros(1, dtype=torch.int32, device=dev)
            a32, al, bl = cs.assign_lights(), cs.assign_lights_lbvh(), cs.build_lbvh()
            if kind == "32ary":
                fn = lambda: a32(stream, keys, kc, frame, bvh, L, lidx, vp, counts, offsets, indices, total, sph)
            else:
                fn = lambda: al(stream, keys, kc, frame, nodes, bvh, L, lidx, vp, counts, offsets, indices, total, sph)
                ms_build = time_events(stream, lambda: bl(stream, lidx, L, boxes, shift, nodes), 3, args.steps, flush)
            ms = time_events(stream, fn, 3, args.steps, flush)
            res.append((ms, counts, offsets, indices, total))
        torch.cuda.synchronize()
        tot = int(res[0][4].cpu()[0])
        same = (int(res[1][4].cpu()[0]) == tot and torch.equal(res[0][1], res[1][1]) and
                torch.equal(res[0][3][:tot], res[1][3][:tot]))
        out[name] = {"assignments": tot, "assign_32ary_ms": round(res[0][0], 5), "assign_lbvh_ms": round(res[1][0], 5),
                     "build_lbvh_ms": round(ms_build, 5), "lists_identical": bool(same)}
    return out


def bouncer_bench(args, dev, stream, flush, hbm_peak):
    """vren_demo's point-light bouncer: 2^24 lights (64 B per light: position and direction read and
    written) against the HBM roofline, and the frame's 16384 lights at 60 frames/s."""
    import torch

    import vren_gb300.clustered_shading as cs

    out = {}
    lo, hi = [-400.0, -250.0, 0.1], [400.0, 250.0, 1000.0]
    for n, dt in ((1 << 24, 1.0 / 60.0), (L, 1.0 / 60.0)):
        rng = np.random.default_rng(SEED + n)
        pos = np.zeros((n, 4), np.float32)
        pos[:, 0] = rng.uniform(lo[0], hi[0], n)
        pos[:, 1] = rng.uniform(lo[1], hi[1], n)
        pos[:, 2] = rng.uniform(lo[2], hi[2], n)
        d = np.zeros((n, 4), np.float32)
        d[:, :3] = rng.standard_normal((n, 3))
        p_t = torch.from_numpy(pos.reshape(-1)).to(dev)
        d_t = torch.from_numpy(d.reshape(-1)).to(dev)
        ms = time_events(stream, lambda: cs.bounce_point_lights(stream, p_t, d_t, n, lo, hi, 20.0, dt), 3,
                         args.steps, flush)
        gbs = 64.0 * n / (ms * 1e-3) / 1e9
        out[f"lights={n}"] = {"ms": round(ms, 5), "glights_s": round(n / (ms * 1e-3) / 1e9, 3),
                              "gbs_at_64B_per_light": round(gbs, 1), "hbm_frac": round(gbs / hbm_peak, 4)}
    return out


def depth_pyramid_bench(args, dev, stream, flush, hbm_peak):
    """vren's depth-buffer pyramid (copy + all max levels, one launch) at the frame's 1920x1080, at
    3840x2160 and at 8192x8192 (beyond L2); algorithmic bytes = 4 B read per level-0 texel + 4 B written
    per texel of every level."""
    import torch

    from vren_gb300.depth_pyramid import depth_buffer_pyramid, depth_buffer_reductor

    out = {}
    red = depth_buffer_reductor()
    for w, h in ((W, H), (3840, 2160), (8192, 8192)):
        g = torch.Generator(device=dev).manual_seed(SEED + w)
        depth = torch.rand(w * h, device=dev, generator=g)
        pyr = depth_buffer_pyramid(w, h, dev)
        texels = sum(max(w >> l, 1) * max(h >> l, 1) for l in range(pyr.get_level_count()))
        ms = time_events(stream, lambda: red.copy_and_reduce(stream, depth, pyr), 3, args.steps, flush)
        gbs = (4.0 * w * h + 4.0 * texels) / (ms * 1e-3) / 1e9
        out[f"{w}x{h}"] = {"ms": round(ms, 5), "levels": pyr.get_level_count(), "gbs": round(gbs, 1),
                           "hbm_frac": round(gbs / hbm_peak, 4)}
        del depth, pyr
    return out


def debug_views_bench(args, dev, stream, flush, ctx, hbm_peak):
    """vren_demo's cluster debug views on the context's last frame (the 1920x1080 shading scene with
    4096 lights near visible surfaces): show_clusters in every mode
    (20 B per pixel: reference read, colour write; the per-cluster colour table is L2-resident) and
    show_clusters_geometry (512 B written per cluster)."""
    import vren_gb300.cluster_debug as cd
    from vren_gb300.clustered_shading import read_device

    out = ctx.outputs()
    U = int(read_device(out.key_count, 1)[0])
    view = cd.show_clusters()
    rgba = None
    res = {"clusters": U}
    for name, mode in cd.MODES.items():
        rgba = view(stream, mode, W, H, out, rgba)
        ms = time_events(stream, lambda: view(stream, mode, W, H, out, rgba), 3, args.steps, flush)
        gbs = 20.0 * W * H / (ms * 1e-3) / 1e9
        res[f"show_clusters_{name}"] = {"ms": round(ms, 5), "gbs": round(gbs, 1), "hbm_frac": round(gbs / hbm_peak, 4)}
    verts = cd.show_clusters_geometry(stream, out, max_clusters=max(U, 1))
    ms = time_events(stream, lambda: cd.show_clusters_geometry(stream, out, verts, max_clusters=max(U, 1)), 3,
                     args.steps, flush)
    res["show_clusters_geometry"] = {"ms": round(ms, 5), "gbs": round(512.0 * U / (ms * 1e-3) / 1e9, 1)}
    return res


def kd_tree_bench(args, dev, stream, flush):
    """vren's k-d tree: host build of 1M uniform points (max 8 per leaf, the reference test's tree),
    then nearest-neighbour searches on the GPU: the reference test's 100 samples and 1M samples."""
    import torch

    from vren_gb300 import kd_tree as kd

    rng = np.random.default_rng(SEED + 31)
    pts = rng.uniform(0, 100, (1_000_000, 3)).astype(np.float32)
    t0 = time.perf_counter()
    nodes, _ = kd.kd_tree_build(pts)
    build_ms = (time.perf_counter() - t0) * 1e3
    depth = kd.kd_tree_depth(nodes)
    d_pts = torch.from_numpy(pts.reshape(-1)).to(dev)
    d_nodes = torch.from_numpy(nodes.view(np.int32).reshape(-1)).to(dev)
    out = {"points": 1_000_000, "nodes": int(len(nodes)), "depth": depth, "host_build_ms": round(build_ms, 2)}
    for q in (100, 1_000_000):
        smp = torch.from_numpy(rng.uniform(0, 100, (q, 3)).astype(np.float32).reshape(-1)).to(dev)
        bp = torch.empty(q, dtype=torch.int32, device=dev)
        bd = torch.empty(q, dtype=torch.float32, device=dev)
        ms = time_events(stream, lambda: kd.kd_tree_search_batch(stream, d_pts, d_nodes, smp, depth, best_points=bp,
                                                                 best_distances=bd), 3, args.steps, flush)
        out[f"gpu_search_{q}_samples"] = {"ms": round(ms, 4), "msearch_s": round(q / (ms * 1e-3) / 1e6, 2)}
    return out


def animated_bench(args, dev, stream, flush, ctx, depth, normals, pos, lights, view):
    """Animated frames as vren_demo runs them: the point-light bouncer moves the 16384 lights
    (speed 20, 60 frames/s, inside the frustum's bounding box), then the clustered assignment runs on
    the moved lights; one step = bounce + frame, L2 flushed before each."""
    import torch

    import vren_gb300.clustered_shading as cs

    rng = np.random.default_rng(SEED + 44)
    d_depth, d_norm = torch.from_numpy(depth).to(dev), torch.from_numpy(normals).to(dev)
    d_pos = torch.from_numpy(pos.copy()).to(dev)
    d_light = torch.from_numpy(lights).to(dev)
    dirs = np.zeros((L, 4), np.float32)
    dirs[:, :3] = rng.standard_normal((L, 3))
    d_dir = torch.from_numpy(dirs.reshape(-1)).to(dev)
    p = pos.reshape(-1, 4)
    lo, hi = p[:, :3].min(0).tolist(), p[:, :3].max(0).tolist()

    def step():
        cs.bounce_point_lights(stream, d_pos, d_dir, L, lo, hi, 20.0, 1.0 / 60.0)
        ctx.cluster(stream, view, W, H, d_depth, d_norm, d_pos, d_light, L)

    ms = time_events(stream, step, 3, args.steps, flush)
    return {"ms_per_animated_frame": round(ms, 5), "frames_per_s": round(1e3 / ms, 1),
            "step": "bounce 16384 lights + cluster assignment (8 launches)"}


def radix_bench(args, dev, stream, flush, keys_np, hbm_peak):
    import torch

    import vren_gb300 as vg
    import vren_gb300.scene as scene

    out = {}
    for n in ([RADIX_N] if args.quick else [RADIX_N, 1 << 24, 1 << 26]):
        kn = keys_np if n == RADIX_N else scene.gen_u32(SEED + 7, 1, n)
        src_k = torch.from_numpy(kn.view(np.int32)).to(dev)
        src_v = torch.arange(n, dtype=torch.int32, device=dev)
        k, v = torch.empty_like(src_k), torch.empty_like(src_v)
        tk, tv = torch.empty_like(k), torch.empty_like(v)
        rs = vg.radix_sort(8)
        s1 = rs.create_scratch_buffer_1(n, dev)

        def run():
            k.copy_(src_k)
            v.copy_(src_v)

        # copies are outside the events: time only the sort
        evs = []
        with torch.cuda.stream(stream):
            for i in range(args.warmup + args.steps):
                run()
                flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                rs.sort(stream, k, v, n, s1, tk, tv)
                b.record(stream)
                if i >= args.warmup:
                    evs.append((a, b))
            stream.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in evs) / len(evs)
        # correctness spot check against numpy's stable sort
        if n == RADIX_N:
            order = np.argsort(kn, kind="stable")
            ok = bool(np.array_equal(k.cpu().numpy().view(np.uint32), kn[order]) and
                      np.array_equal(v.cpu().numpy(), order.astype(np.int32)))
        else:
            ok = None
        gbs = 64.0 * n / (ms * 1e-3) / 1e9
        out[f"n=2^{n.bit_length() - 1}"] = {"ms": round(ms, 5), "gkeys_s": round(n / (ms * 1e-3) / 1e9, 3),
                                            "gbs_at_64B_per_pair": round(gbs, 1),
                                            "hbm_frac": round(gbs / hbm_peak, 4), "bit_exact_vs_stable_sort": ok,
                                            "l2": "flushed before each sort" if n * 16 < (129 << 20) else
                                            "inputs larger than L2 (also flushed)"}
        del src_k, src_v, k, v, tk, tv, s1
    if args.quick:
        return out
    # beyond the workload's sizes: 2^28 pairs, and keys only (the reference's radix_sort::operator(),
    # 32 B/key over four 8-bit passes) at 2^26 and 2^28; checked for order and, for pairs, that the
    # values are a permutation carrying their keys
    for n, pairs in ((1 << 28, True), (1 << 26, False), (1 << 28, False)):
        g = torch.Generator(device=dev)
        g.manual_seed(SEED + n + pairs)
        src_k = torch.randint(-(1 << 31), 1 << 31, (n,), dtype=torch.int32, device=dev, generator=g)
        k, tk = torch.empty_like(src_k), torch.empty_like(src_k)
        v = tv = src_v = None
        if pairs:
            src_v = torch.arange(n, dtype=torch.int32, device=dev)
            v, tv = torch.empty_like(src_v), torch.empty_like(src_v)
        rs = vg.radix_sort(8)
        s1 = rs.create_scratch_buffer_1(n, dev)
        evs = []
        with torch.cuda.stream(stream):
            for i in range(args.warmup + args.steps):
                k.copy_(src_k)
                if pairs:
                    v.copy_(src_v)
                flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                rs.sort(stream, k, v, n, s1, tk, tv)
                b.record(stream)
                if i >= args.warmup:
                    evs.append((a, b))
            stream.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in evs) / len(evs)
        flip = torch.tensor(-(1 << 31), dtype=torch.int32, device=dev)
        ku = k ^ flip  # unsigned order as signed order
        ok = bool((ku[1:] >= ku[:-1]).all().item())
        if pairs:
            ok = ok and bool(torch.equal(src_k[v.long()], k)) and \
                bool(torch.equal(torch.sort(v).values, src_v))
        per = 64.0 if pairs else 32.0
        gbs = per * n / (ms * 1e-3) / 1e9
        out[f"n=2^{n.bit_length() - 1}" + ("" if pairs else "_keys_only")] = {
            "ms": round(ms, 5), "gkeys_s": round(n / (ms * 1e-3) / 1e9, 3),
            "gbs_at_%dB_per_%s" % (per, "pair" if pairs else "key"): round(gbs, 1),
            "hbm_frac": round(gbs / hbm_peak, 4), "sorted_and_permutation": ok}
        del src_k, src_v, k, v, tk, tv, s1, ku
    return out


# Arithmetic operations per (pixel, assigned light) pair, counted once on the restated formulas
# (pbr_apply_point_light with the windowed inverse-square falloff; every +, -, *, /, sqrt, min and max of
# the GLSL expression is one operation): distance and falloff 26, half vector 12, GGX NDF 14, N.L 7,
# Smith G 9, H.V 6, Schlick power 5, specular 5, three colour channels 54.  The adjoint recomputes
# the forward (135 without the accumulation) and adds 150 for the reverse sweep.
SHADE_FWD_FLOPS_PER_PAIR = 138
SHADE_BWD_FLOPS_PER_PAIR = 285
SHADE_W, SHADE_H, SHADE_L = 1920, 1080, 4096


def fp32_peak_tflops(sm_mhz):
    """Nominal FP32 CUDA-core rate: 152 SMs x 128 lanes x 2 (fused multiply-add) at the sampled clock."""
    return 152 * 128 * 2 * (sm_mhz or 2070.0) * 1e6 / 1e12


def shade_profile_setup(dev, stream, ctx):
    """Inputs of the differentiable-shading workload (1920x1080 G-buffer, 4096 lights near visible
    surfaces, windowed inverse-square falloff, N(0,1) upstream gradient), light lists from the
    clustering pipeline, and forward / adjoint closures."""
    import torch

    import vren_gb300.clustered_shading as cs
    import vren_gb300.scene as scene

    W_, H_, L_ = SHADE_W, SHADE_H, SHADE_L
    depth, normals_planes = scene.depth_planes(SEED + 500, W_, H_, planes=64)
    gn, galb, grough, gmetal = scene.gbuffer(SEED + 501, W_, H_)
    pos, lights = scene.lights_near_surfaces(SEED + 502, L_, depth, W_, H_)
    grad = scene.normal01(SEED + 503, 9, W_ * H_ * 3)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_depth, d_np, d_pos, d_light = t(depth), t(normals_planes), t(pos), t(lights)
    d_n, d_alb, d_r, d_m, d_grad = t(gn), t(galb), t(grough), t(gmetal), t(grad)
    view = cs.view_from_camera(cs.scene_camera(W_, H_), "ref")
    with torch.cuda.stream(stream):
        ctx.cluster(stream, view, W_, H_, d_depth, d_np, d_pos, d_light, L_)
    stream.synchronize()
    out = ctx.outputs()
    U = int(cs.read_device(out.key_count, 1)[0])
    total = int(cs.read_device(out.total, 1)[0])
    refs = cs.read_device(out.cluster_refs, W_ * H_)
    counts = cs.read_device(out.counts, U)
    pairs = int(counts[refs].astype(np.int64).sum()) if U else 0
    gb = cs.gbuffer(d_depth, d_n, d_alb, d_r, d_m)
    ll = cs.light_lists(out.cluster_refs, out.counts, out.offsets, out.indices, out.index_capacity)
    img = torch.empty(W_ * H_ * 3, dtype=torch.float32, device=dev)
    fwd = cs.shade("windowed_inv_sq", "radiance")
    bwd = cs.shade_backward("windowed_inv_sq")
    gpos = torch.zeros(L_ * 3, dtype=torch.float32, device=dev)
    gcol = torch.zeros(L_ * 3, dtype=torch.float32, device=dev)
    grr = torch.zeros(L_, dtype=torch.float32, device=dev)
    keep = (d_depth, d_np, d_pos, d_light, d_n, d_alb, d_r, d_m, d_grad, img, gpos, gcol, grr)
    # host copies for the FP64 check of the adjoint (the CPU leg)
    host = {"view": view, "W": W_, "H": H_, "L": L_, "gb": (depth, gn, galb, grough, gmetal), "pos": pos,
            "lights": lights, "grad": grad,
            "lists": (refs, counts, cs.read_device(out.offsets, U), cs.read_device(out.indices, total))}
    return {
        "forward": lambda: fwd(stream, out.frame, W_, H_, gb, ll, d_pos, d_light, L_, img),
        "backward": lambda: bwd(stream, out.frame, W_, H_, gb, ll, total, d_pos, d_light, L_, d_grad, gpos, gcol, grr),
        "pairs": pairs, "unique_clusters": U, "assignments": total, "img": img, "gpos": gpos, "gcol": gcol,
        "grr": grr, "keep": keep, "host": host,
    }


def shade_bench(args, dev, stream, flush, ctx):
    """Differentiable shading at 1920x1080 with 4096 lights: forward radiance and the adjoint w.r.t.
    light position/colour/radius, each timed alone with CUDA events (L2 flushed between runs).  Returns
    (host copies of the inputs, lists and GPU gradient for the CPU leg's FP64 check, results)."""
    import torch

    sb = shade_profile_setup(dev, stream, ctx)
    steps = max(3, args.steps // 2)
    ms_f = time_events(stream, sb["forward"], 3, steps, flush)
    ms_b = time_events(stream, sb["backward"], 3, steps, flush)
    pairs = sb["pairs"]
    ok = bool(torch.isfinite(sb["img"]).all().item() and torch.isfinite(sb["gpos"]).all().item())
    L_ = sb["host"]["L"]
    torch.cuda.synchronize()
    sb["host"]["gpu_gradient"] = np.concatenate([sb["gpos"].cpu().numpy().reshape(L_, 3),
                                                 sb["gcol"].cpu().numpy().reshape(L_, 3),
                                                 sb["grr"].cpu().numpy().reshape(L_, 1)], 1).astype(np.float64)
    return sb["host"], {
        "workload": "1920x1080 G-buffer, 4096 lights near visible surfaces, windowed inverse-square falloff, "
                    "radiance output; adjoint for an N(0,1) upstream gradient",
        "pairs": pairs, "unique_clusters": sb["unique_clusters"], "assignments": sb["assignments"],
        "forward_ms": round(ms_f, 5), "backward_ms": round(ms_b, 5),
        "forward_tflops": round(SHADE_FWD_FLOPS_PER_PAIR * pairs / (ms_f * 1e-3) / 1e12, 3),
        "backward_tflops": round(SHADE_BWD_FLOPS_PER_PAIR * pairs / (ms_b * 1e-3) / 1e12, 3),
        "flops_per_pair": {"forward": SHADE_FWD_FLOPS_PER_PAIR, "backward": SHADE_BWD_FLOPS_PER_PAIR},
        "finite": ok,
    }


BATCH_FRAMES = 64
BATCH_RES = [(640, 360), (1280, 720), (1920, 1080), (2560, 1440)]


def batch_specs(seed: int = SEED + 4000):
    """64 frames: resolution uniform over BATCH_RES, light count log-uniform in [1024, 65536]."""
    rng = np.random.default_rng(seed)
    specs = []
    for k in range(BATCH_FRAMES):
        w, h = BATCH_RES[int(rng.integers(0, len(BATCH_RES)))]
        L = int(round(float(np.exp(rng.uniform(np.log(1024.0), np.log(65536.0))))))
        specs.append((w, h, L))
    return specs


def batched_vs_plain(args, dev, stream, flush):
    """Frames per second of the batched form (one graph for all 64 frames, autotuned) against the
    plain per-frame form (64 cluster_and_shade calls, each a replay of its own captured graph), on
    the same inputs; every frame's outputs are compared bit for bit."""
    import torch

    import vren_gb300.clustered_shading as cs
    import vren_gb300.scene as scene

    specs = batch_specs()
    frames, plain = [], []
    for k, (w, h, L) in enumerate(specs):
        view = cs.view_from_camera(cs.scene_camera(w, h), "ref")
        depth, normals = scene.depth_planes(SEED + 5000 + k, w, h, planes=64)
        pos, lights = scene.lights(SEED + 6000 + k, L, w, h)
        t = lambda a: torch.from_numpy(a).to(dev)
        frames.append((view, w, h, t(depth), t(normals), t(pos), t(lights), L))
        plain.append(cs.cluster_and_shade(w, h, L, 1 << 22))
    torch.cuda.synchronize()

    def run_plain():
        for ctx, (view, w, h, d, n, p, l, L) in zip(plain, frames):
            ctx.cluster(stream, view, w, h, d, n, p, l, L)

    batch = cs.cluster_batch()
    batch.reserve(frames, 1 << 26)
    with torch.cuda.stream(stream):
        chosen = batch.autotune(stream, frames, reps=2)
    steps = max(3, args.steps // 2)
    with torch.cuda.stream(stream):
        ms_plain = time_events(stream, run_plain, 3, steps, flush)
        ms_batch = time_events(stream, lambda: batch.run(stream, frames), 3, steps, flush)
    # bit-exactness of every frame (outputs of the last run of each arm)
    exact = True
    for f, (ctx, fr) in enumerate(zip(plain, frames)):
        a, b = ctx.outputs(), batch.frame_outputs(stream, f)
        ua, ub = int(cs.read_device(a.key_count, 1)[0]), int(cs.read_device(b.key_count, 1)[0])
        ta, tb = int(cs.read_device(a.total, 1)[0]), int(cs.read_device(b.total, 1)[0])
        same = ua == ub and ta == tb
        for name, cnt in (("cluster_keys", ua), ("cluster_refs", fr[1] * fr[2]), ("counts", ua), ("offsets", ua),
                          ("indices", ta)):
            if not same:
                break
            same = np.array_equal(cs.read_device(getattr(a, name), cnt), cs.read_device(getattr(b, name), cnt))
        exact = exact and same
    total_px = sum(w * h for w, h, _ in specs)
    total_l = sum(L for _, _, L in specs)
    return {
        "workload": f"{BATCH_FRAMES} frames, resolution uniform over {BATCH_RES}, lights log-uniform in [1024, 65536], "
                    "cluster assignment (light BVH + unique clusters + light lists) per frame",
        "total_pixels": total_px, "total_lights": total_l,
        "plain_ms": round(ms_plain, 4), "batched_ms": round(ms_batch, 4),
        "plain_frames_per_s": round(BATCH_FRAMES / (ms_plain * 1e-3), 1),
        "batched_frames_per_s": round(BATCH_FRAMES / (ms_batch * 1e-3), 1),
        "speedup": round(ms_plain / ms_batch, 3),
        "bit_exact_all_frames": bool(exact),
        "autotuned_options": chosen,
        "plain": "64 vren_cs_cluster calls, each replaying its own captured graph",
        "l2": "flushed before each timed step",
    }


def primitive_sweep(args, dev, stream, flush, hbm_peak):
    import torch

    import vren_gb300 as vg
    import vren_gb300.scene as scene

    res = {}
    steps = max(3, args.steps // 2)
    for e in (16, 20, 24, 26):
        n = 1 << e
        x = torch.from_numpy(scene.gen_u32(SEED + e, 2, n, mask=255).view(np.int32)).to(dev)
        y = torch.empty_like(x)
        o = torch.zeros(1, dtype=torch.int32, device=dev)
        sc = vg.primitives.alloc_scratch(vg.primitives.reduce_scratch_bytes(n), dev)
        ms_red = time_events(stream, lambda: vg.reduce_scalar(stream, "add", x, o, sc), 3, steps, flush)
        xf = x.float()
        of = torch.zeros(1, dtype=torch.float32, device=dev)
        ms_max = time_events(stream, lambda: vg.reduce_scalar(stream, "max", xf, of, sc), 3, steps, flush)
        scan = vg.blelloch_scan()

        def do_scan():
            scan(stream, y, n)

        y.copy_(x)
        ms_scan = time_events(stream, do_scan, 3, steps, flush)
        res[f"2^{e}"] = {
            "reduce_u32_add": {"ms": round(ms_red, 5), "gbs": round(4 * n / ms_red / 1e6, 1),
                               "hbm_frac": round(4 * n / ms_red / 1e6 / hbm_peak, 4)},
            "reduce_f32_max": {"ms": round(ms_max, 5), "gbs": round(4 * n / ms_max / 1e6, 1)},
            "exclusive_scan": {"ms": round(ms_scan, 5), "gbs": round(8 * n / ms_scan / 1e6, 1),
                               "hbm_frac": round(8 * n / ms_scan / 1e6 / hbm_peak, 4)},
        }
        del x, y, xf
    # bucket sort: 2^24 uvec2(key, index), 1024 buckets on the low 10 bits
    n = 1 << 24
    keys = scene.gen_u32(SEED + 99, 3, n)
    pairs = np.stack([keys, np.arange(n, dtype=np.uint32)], 1).reshape(-1)
    src = torch.from_numpy(pairs.view(np.int32)).to(dev)
    lib = vg.lib()
    knobs = (vg._lib.TUNE["bucket_form"], vg._lib.TUNE["radix_rank"])
    saved = [lib.vren_tuning_get(k) for k in knobs]
    # 10 bits: the one-scatter form (tile histograms, column scan, scatter) and the radix-pass form;
    # 16 bits: radix passes
    for kb, form, rank, label in ((10, 0, 0, ""), (10, 1, 0, "_radix_passes"), (16, 0, 0, "")):
        lib.vren_tuning_set(knobs[0], form)
        lib.vren_tuning_set(knobs[1], rank)
        bs = vg.bucket_sort(kb)
        outb = torch.empty(bs.get_required_output_buffer_size(n) // 4, dtype=torch.int32, device=dev)
        ms_b = time_events(stream, lambda: bs(stream, src, n, 0, outb, 0), 3, steps, flush)
        res[f"bucket_sort_2^24_{kb}bit{label}"] = {"ms": round(ms_b, 5), "gbs_at_24B": round(24 * n / ms_b / 1e6, 1),
                                                   "hbm_frac": round(24 * n / ms_b / 1e6 / hbm_peak, 4)}
    for k, v in zip(knobs, saved):
        lib.vren_tuning_set(k, v)
    return res


def adjoint_check(oracle, host, lights_checked: int = 64):
    """The GPU adjoint of the differentiable-shading workload (1920x1080, 4096 lights) against the FP64
    forward-mode gradient of the oracle on `lights_checked` seeded lights, evaluated over those lights'
    own (pixel, light) pairs with all host threads: relative error per parameter group (normwise over
    the lights) and per light."""
    refs, counts, offsets, indices = host["lists"]
    total = int(counts.sum(dtype=np.uint64))
    pix = np.bincount(refs, minlength=len(counts)).astype(np.int64)
    pairs = np.bincount(indices[:total], weights=np.repeat(pix, counts.astype(np.int64)), minlength=host["L"])
    rng = np.random.default_rng(SEED + 505)
    sel = np.sort(rng.choice(np.flatnonzero(pairs > 0), lights_checked, replace=False)).astype(np.uint32)
    t0 = time.perf_counter()
    ref, _, _ = oracle.cs_shade_grad_lights_f64(host["view"], host["W"], host["H"], host["gb"], host["lists"],
                                                host["pos"], host["lights"], host["L"], host["grad"], sel, h=0.0,
                                                falloff=1, threads=os.cpu_count())
    got = host["gpu_gradient"][sel]
    groups = {name: float(np.linalg.norm(got[:, sl] - ref[:, sl]) / np.linalg.norm(ref[:, sl]))
              for name, sl in (("position", slice(0, 3)), ("colour", slice(3, 6)), ("radius", slice(6, 7)))}
    nz = np.linalg.norm(ref, axis=1) > 0
    per_light = np.linalg.norm(got[nz] - ref[nz], axis=1) / np.linalg.norm(ref[nz], axis=1)
    return {"lights_checked": lights_checked, "pairs_checked": int(pairs[sel].sum()),
            "rel_err_by_group": {k: float(f"{v:.3g}") for k, v in groups.items()},
            "rel_err_max_group": float(f"{max(groups.values()):.3g}"),
            "rel_err_per_light_max": float(f"{per_light.max():.3g}"),
            "check_s": round(time.perf_counter() - t0, 2), "reference": "FP64 forward-mode gradient (dual numbers)"}


def cpu_baseline(depth, normals, pos, lights, radix_keys, view, shade_host=None, budget_s: float = 12.0,
                 threads: int = 1):
    """The CPU oracle (port of the reference's algorithms) on a bounded sample, single-threaded; the
    primitive sweep's CPU counterparts (the reference test's tree reduce, std::exclusive_scan, the
    stable sort by masked key); and, as the checker, the FP64 gradient the GPU adjoint is held to."""
    import oracle
    import vren_gb300.scene as scene

    t0 = time.perf_counter()
    frames = 0
    while True:
        vp, bvh, lidx = oracle.cs_light_bvh(pos, lights, L, view, 15)
        keys, refs = oracle.cs_find_unique_clusters(depth, normals, W, H, view, 0, threads=threads)
        oracle.cs_assign_lights(keys, W, H, view, bvh, L, lidx, vp, threads=threads)
        frames += 1
        if time.perf_counter() - t0 > budget_s / 2 or frames >= 50:
            break
    ms_frame = (time.perf_counter() - t0) * 1e3 / frames
    t1 = time.perf_counter()
    sorts = 0
    vals = np.arange(RADIX_N, dtype=np.uint32)
    while True:
        oracle.stable_sort_u32(radix_keys, vals)
        sorts += 1
        if time.perf_counter() - t1 > budget_s / 4 or sorts >= 50:
            break
    ms_sort = (time.perf_counter() - t1) * 1e3 / sorts
    rng = np.random.default_rng(SEED)
    bp = np.zeros((1 << 20, 4), np.float32)
    bp[:, :3] = rng.uniform(-100.0, 100.0, (1 << 20, 3))
    bd = np.zeros((1 << 20, 4), np.float32)
    bd[:, :3] = rng.standard_normal((1 << 20, 3))
    t2 = time.perf_counter()
    oracle.bounce_point_lights(bp, bd, 1 << 20, [-400.0, -250.0, 0.1], [400.0, 250.0, 1000.0], 20.0, 1.0 / 60.0)
    ms_bounce = (time.perf_counter() - t2) * 1e3
    t3 = time.perf_counter()
    oracle.depth_pyramid(depth, W, H)
    ms_pyramid = (time.perf_counter() - t3) * 1e3
    kp = np.random.default_rng(SEED + 31).uniform(0, 100, (1_000_000, 3)).astype(np.float32)
    knodes, _ = oracle.kd_tree_build(kp)
    ks = np.random.default_rng(SEED + 32).uniform(0, 100, (100_000, 3)).astype(np.float32)
    t4 = time.perf_counter()
    oracle.kd_tree_search(kp, knodes, ks)
    ms_kd = (time.perf_counter() - t4) * 1e3
    # the primitive sweep's CPU counterparts at n = 2^24 (u32 uniform in [0, 255]), one core
    n2 = 1 << 24
    xs = scene.gen_u32(SEED + 24, 2, n2, mask=255)
    sweep = {}
    for name, fn, nbytes in (("tree_reduce_u32_add", lambda: oracle.reduce_tree_u32("add", xs), 8 * n2),
                             ("reduce_f32_max", lambda: oracle.reduce_f32("max", xs.astype(np.float32)), 4 * n2),
                             ("exclusive_scan", lambda: oracle.exclusive_scan_u32(xs), 8 * n2)):
        t5 = time.perf_counter()
        fn()
        ms = (time.perf_counter() - t5) * 1e3
        sweep[name] = {"ms": round(ms, 3), "gbs": round(nbytes / (ms * 1e6), 2)}
    nb = 1 << 22
    bkeys = scene.gen_u32(SEED + 99, 3, nb)
    bpairs = np.stack([bkeys, np.arange(nb, dtype=np.uint32)], 1).reshape(-1)
    t6 = time.perf_counter()
    oracle.bucket_sort_u32x2(bpairs, 10)
    ms_b = (time.perf_counter() - t6) * 1e3
    sweep["bucket_sort_2^22_10bit"] = {"ms": round(ms_b, 3), "gbs_at_24B": round(24 * nb / (ms_b * 1e6), 2)}
    sweep["n"] = "2^24 (bucket sort 2^22), 1 core; bytes counted as for the GPU lines"
    adjoint = adjoint_check(oracle, shade_host) if shade_host is not None else None
    return {"value": round(ms_frame, 3), "unit": "ms", "cores": threads, "kind": "port",
            "primitive_sweep": sweep, "adjoint_check": adjoint,
            "sample": f"{frames} frames of the CPU oracle pipeline (a6+a7+a8) at 1920x1080/16384 lights",
            "radix_sort_2^20_pairs_ms": round(ms_sort, 3),
            "radix_sort_gkeys_s": round(RADIX_N / (ms_sort * 1e-3) / 1e9, 4),
            "light_bouncer_2^20_lights_ms": round(ms_bounce, 3),
            "depth_pyramid_1920x1080_ms": round(ms_pyramid, 3),
            "kd_tree_search_100k_samples_1m_points_ms": round(ms_kd, 3)}


# ------------------------------------------------------------------------------------------------
# Reference arm: the CPU implementation of the path (oracle port), all host threads
# ------------------------------------------------------------------------------------------------
def numpy_view(cs, near: float = 0.1, far: float = 1000.0, fov_deg: float = 45.0):
    """The bench camera (origin, yaw = pitch = 0) with vren/vren/camera.cpp:32-50's formulas, so the
    CPU arm does not load the CUDA library."""
    fov = float(np.float32(np.deg2rad(fov_deg)))
    t = np.tan(fov / 2.0)
    proj = np.zeros((4, 4))  # row-major
    proj[0, 0] = 1.0 / (t * (W / H))
    proj[1, 1] = 1.0 / t
    proj[2, 2] = far / (far - near)
    proj[2, 3] = -(far * near) / (far - near)
    proj[3, 2] = 1.0
    inv = np.linalg.inv(proj)
    v = cs.View()
    v.view[:] = np.eye(4, dtype=np.float32).T.reshape(-1).tolist()
    v.inv_view[:] = np.eye(4, dtype=np.float32).T.reshape(-1).tolist()
    v.inv_proj[:] = inv.T.astype(np.float32).reshape(-1).tolist()
    v.near_plane, v.far_plane, v.half_fov_y = near, far, np.float32(fov) / np.float32(2)
    v.slicing = 0
    return v


def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    import oracle
    import vren_gb300.clustered_shading as cs
    from vren_gb300 import _build

    _build.build_scene()
    depth, normals, _, pos, lights, radix_keys = make_inputs(0)
    cores = os.cpu_count() or 1
    view = numpy_view(cs)

    def frame():
        vp, bvh, lidx = oracle.cs_light_bvh(pos, lights, L, view, 15)
        keys, refs = oracle.cs_find_unique_clusters(depth, normals, W, H, view, 0, threads=cores)
        oracle.cs_assign_lights(keys, W, H, view, bvh, L, lidx, vp, threads=cores)

    for _ in range(args.warmup):
        frame()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        frame()
    ms = (time.perf_counter() - t0) * 1e3 / args.steps
    vals = np.arange(RADIX_N, dtype=np.uint32)
    t1 = time.perf_counter()
    reps = 5
    for _ in range(reps):
        oracle.stable_sort_u32(radix_keys, vals)
    ms_sort = (time.perf_counter() - t1) * 1e3 / reps
    res = {
        "impl": "reference", "metric": METRIC, "value": round(ms, 4), "unit": "ms", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+u32",
        "data": "synthetic (seeded PCG32 scene: 64 oriented planar discs, 16384 point lights)",
        "config": {"workload": "cluster assignment 1920x1080, 16384 lights, 32x32 tiles, REF slicing, 15-bit Morton, "
                               "a6+a7+a8 per frame (construct light BVH, unique clusters, assign lights)",
                   "implementation": "CPU restatement of loryruta/vren's algorithms (oracle/); the reference's own "
                                     "GPU path needs Vulkan, which this machine does not have"},
        "cpu_baseline": {"value": round(ms, 4), "unit": "ms", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} frames at 1920x1080/16384 lights, OpenMP over tiles and clusters",
                         "radix_sort_2^20_pairs_ms": round(ms_sort, 3)},
        "e2e": {"value": round(ms, 4), "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(res), flush=True)


def run_profile(args):
    """One kernel family on a case larger than L2, for ncu captures (--profile KIND)."""
    import torch

    import vren_gb300 as vg
    import vren_gb300.clustered_shading as cs
    import vren_gb300.scene as scene
    from vren_gb300 import _build

    _build.build()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    reps = args.warmup + args.steps
    if args.profile in ("batch", "batch_small"):
        # the batched form on the 64 mixed frames, or on the first 8 of them (small enough for a full
        # ncu capture); fixed options: 6-bit digits, 2 traversal warps
        specs = batch_specs() if args.profile == "batch" else batch_specs()[:8]
        frames = []
        for k, (w, h, nl) in enumerate(specs):
            v = cs.view_from_camera(cs.scene_camera(w, h), "ref")
            depth, normals = scene.depth_planes(SEED + 5000 + k, w, h, planes=64)
            pos, lights = scene.lights(SEED + 6000 + k, nl, w, h)
            t = lambda a: torch.from_numpy(a).to(dev)
            frames.append((v, w, h, t(depth), t(normals), t(pos), t(lights), nl))
        batch = cs.cluster_batch()
        batch.reserve(frames, 1 << 26)
        batch.set_options(sort_digit_bits=6, radix_items=0, scan_slices=8, assign_warps=2)
        fn = lambda: batch.run(stream, frames)
    elif args.profile == "frame":
        # the benchmark's frame: 1920x1080, 16384 lights, one CUDA graph replay per frame
        depth, normals, _, pos, lights, _ = make_inputs(0)
        view = cs.view_from_camera(cs.scene_camera(W, H), "ref")
        ctx = cs.cluster_and_shade(W, H, 65536, 1 << 24)
        bufs = [torch.from_numpy(x).to(dev) for x in (depth, normals, pos, lights)]
        fn = lambda: ctx.cluster(stream, view, W, H, *bufs, L)
    elif args.profile == "frame_dense":
        # the benchmark's frame with its 16384 lights packed in front of the camera (long light lists)
        import vren_gb300.scene as scene

        depth, normals, _, _, _, _ = make_inputs(0)
        dpos, dlights = scene.lights_near_camera(SEED + 77, L)
        view = cs.view_from_camera(cs.scene_camera(W, H), "ref")
        ctx = cs.cluster_and_shade(W, H, 65536, 1 << 24)
        bufs = [torch.from_numpy(x).to(dev) for x in (depth, normals, dpos, dlights)]
        fn = lambda: ctx.cluster(stream, view, W, H, *bufs, L)
    elif args.profile in ("find_unique", "find_unique_rgba16f"):
        w, h = 3840, 2160  # 20 B/px (f32x3 normals; 16 with RGBA16F) -> 166 (133) MB > L2
        depth, normals = scene.depth_planes(SEED, w, h)
        fmt = cs.NORMALS["f32x3"]
        if args.profile == "find_unique_rgba16f":
            n16 = np.zeros((w * h, 4), np.float16)
            n16[:, :3] = normals.reshape(-1, 3).astype(np.float16)
            normals, fmt = n16, cs.NORMALS["rgba16f"]
        view = cs.view_from_camera(cs.scene_camera(w, h), "ref")
        frame = cs.frame_to_device(cs.frame_build(view, w, h, "wrap", fmt), dev)
        T = ((w + 31) // 32) * ((h + 31) // 32)
        keys = torch.zeros(T * 1024, dtype=torch.int32, device=dev)
        kc = torch.zeros(1, dtype=torch.int32, device=dev)
        refs = torch.zeros(w * h, dtype=torch.int32, device=dev)
        d, n = torch.from_numpy(depth).to(dev), torch.from_numpy(normals).to(dev)
        fuc = cs.find_unique_cluster_list()
        fn = lambda: fuc(stream, w, h, frame, d, n, keys, kc, refs)
    elif args.profile == "radix":
        n = 1 << 25
        k = torch.from_numpy(scene.gen_u32(SEED + 7, 1, n).view(np.int32)).to(dev)
        v = torch.arange(n, dtype=torch.int32, device=dev)
        tk, tv = torch.empty_like(k), torch.empty_like(v)
        rs = vg.radix_sort(8)
        s1 = rs.create_scratch_buffer_1(n, dev)
        fn = lambda: rs.sort(stream, k, v, n, s1, tk, tv)
    elif args.profile == "scan":
        n = 1 << 26
        x = torch.from_numpy(scene.gen_u32(SEED, 2, n, mask=255).view(np.int32)).to(dev)
        scan = vg.blelloch_scan()
        fn = lambda: scan(stream, x, n)
    elif args.profile == "reduce":
        # scalar u32 sum over 2^26 values (256 MB) and the reference's tree reduce over 2^24 (64 MB)
        n = 1 << 26
        x = torch.from_numpy(scene.gen_u32(SEED, 2, n, mask=255).view(np.int32)).to(dev)
        from vren_gb300.primitives import alloc_scratch, reduce_scratch_bytes

        o = torch.zeros(4, dtype=torch.int32, device=dev)
        sc = alloc_scratch(reduce_scratch_bytes(n), dev)
        t = torch.from_numpy(scene.gen_u32(SEED + 1, 2, 1 << 24, mask=255).view(np.int32)).to(dev)
        tree = vg.reduce("uint", "add")
        fn = lambda: (vg.reduce_scalar(stream, "add", x, o, sc), tree(stream, t, 1 << 24, 0))
    elif args.profile == "bucket":
        # 2^24 uvec2(key, index) into 1024 buckets on the low 10 bits
        n = 1 << 24
        kv = torch.empty(2 * n, dtype=torch.int32, device=dev)
        kv[0::2] = torch.from_numpy(scene.gen_u32(SEED + 3, 1, n).view(np.int32)).to(dev)
        kv[1::2] = torch.arange(n, dtype=torch.int32, device=dev)
        bs = vg.bucket_sort(10)
        out_b = torch.empty(bs.get_required_output_buffer_size(n) // 4, dtype=torch.int32, device=dev)
        fn = lambda: bs(stream, kv, n, 0, out_b, 0)
    elif args.profile == "build_bvh":
        # BuildBVH over 2^20 leaves (32 MB of leaves, 33.8 MB of nodes)
        n = 1 << 20
        nodes = torch.zeros(vg.calc_bvh_buffer_length(n) * 8, dtype=torch.int32, device=dev)
        leaves = np.zeros((n, 8), np.float32)
        rng = np.random.default_rng(SEED)
        p0 = rng.uniform(0, 100, (n, 3)).astype(np.float32)
        leaves[:, 0:3], leaves[:, 4:7] = p0, p0 + 1.0
        lv = leaves.view(np.uint32)
        lv[:, 3] = 0xFFFFFFFF
        nodes[: n * 8] = torch.from_numpy(lv.reshape(-1).view(np.int32)).to(dev)
        bb = vg.build_bvh()
        fn = lambda: bb(stream, nodes, n)
    elif args.profile in ("assign", "karras"):
        # the light assignment of the bench frame (1920x1080, 16384 lights), through the 32-ary BVH or
        # through the Karras tree (build + assignment)
        depth, normals, _, pos, lights, _ = make_inputs(0)
        view = cs.view_from_camera(cs.scene_camera(W, H), "ref")
        ctx = cs.cluster_and_shade(W, H, 65536, 1 << 24)
        bufs = [torch.from_numpy(x).to(dev) for x in (depth, normals, pos, lights)]
        ctx.cluster(stream, view, W, H, *bufs, L)
        stream.synchronize()
        o = ctx.outputs()
        U = int(cs.read_device(o.key_count, 1)[0])
        keys = torch.from_numpy(cs.read_device(o.cluster_keys, U).view(np.int32)).to(dev)
        kc = torch.tensor([U], dtype=torch.int32, device=dev)
        frame_dev = cs.frame_to_device(cs.frame_build(view, W, H), dev)
        vp = torch.from_numpy(cs.read_device(o.view_positions, 4 * L, np.float32)).to(dev)
        bvh = torch.from_numpy(cs.read_device(o.bvh, vg.calc_bvh_buffer_length(L) * 8).view(np.int32)).to(dev)
        li = torch.from_numpy(cs.read_device(o.light_index, 2 * L).view(np.int32)).to(dev)
        sph = torch.from_numpy(cs.read_device(o.leaf_spheres, 4 * vg.calc_bvh_padded_leaf_count(L), np.float32)).to(dev)
        counts = torch.zeros(U, dtype=torch.int32, device=dev)
        offs = torch.zeros(U, dtype=torch.int32, device=dev)
        idx = torch.zeros(1 << 24, dtype=torch.int32, device=dev)
        tot = torch.zeros(1, dtype=torch.int32, device=dev)
        if args.profile == "assign":
            al = cs.assign_lights()
            fn = lambda: al(stream, keys, kc, frame_dev, bvh, L, li, vp, counts, offs, idx, tot, sph)
        else:
            nodes_k = torch.zeros(max(L - 1, 1) * 8, dtype=torch.int32, device=dev)
            boxes, shift = cs.build_lbvh.group_boxes(bvh, L)
            bl, al = cs.build_lbvh(), cs.assign_lights_lbvh()
            fn = lambda: (bl(stream, li, L, boxes, shift, nodes_k),
                          al(stream, keys, kc, frame_dev, nodes_k, bvh, L, li, vp, counts, offs, idx, tot, sph))
    elif args.profile == "light_bvh_multi":
        # construct_point_light_bvh for 65536 lights (above the single-cluster kernel's 32768): view
        # transform, Morton codes, sort, leaves and BVH levels as separate kernels
        nl = 65536
        pos_l, li_l = scene.lights(SEED + 1000, nl, W, H)
        view = cs.view_from_camera(cs.scene_camera(W, H), "ref")
        frame_dev = cs.frame_to_device(cs.frame_build(view, W, H), dev)
        d_p, d_l = torch.from_numpy(pos_l).to(dev), torch.from_numpy(li_l).to(dev)
        vp = torch.zeros(4 * nl, dtype=torch.float32, device=dev)
        bvh = torch.zeros(vg.calc_bvh_buffer_length(nl) * 8, dtype=torch.int32, device=dev)
        lidx = torch.zeros(2 * nl, dtype=torch.int32, device=dev)
        sph = torch.zeros(4 * vg.calc_bvh_padded_leaf_count(nl), dtype=torch.float32, device=dev)
        cb = cs.construct_point_light_bvh()
        fn = lambda: cb(stream, d_p, d_l, nl, frame_dev, vp, bvh, lidx, sph)
    elif args.profile == "bouncer":
        n = 1 << 24  # 1 GB of positions and directions
        rng = np.random.default_rng(SEED)
        p_t = torch.from_numpy(rng.uniform(-100, 100, (n, 4)).astype(np.float32).reshape(-1)).to(dev)
        d_t = torch.from_numpy(rng.standard_normal((n, 4)).astype(np.float32).reshape(-1)).to(dev)
        fn = lambda: cs.bounce_point_lights(stream, p_t, d_t, n, [-400, -250, 0.1], [400, 250, 1000], 20.0, 1 / 60)
    elif args.profile == "debug_views":
        # show_clusters (light-index mode) and the cluster geometry on the 1080p shading frame
        import vren_gb300.cluster_debug as cd

        ctx = cs.cluster_and_shade(SHADE_W, SHADE_H, 65536, 1 << 24)
        shade_profile_setup(dev, stream, ctx)
        o = ctx.outputs()
        view_dbg = cd.show_clusters()
        rgba = view_dbg(stream, "light_indices", SHADE_W, SHADE_H, o)
        U = int(cs.read_device(o.key_count, 1)[0])
        verts = cd.show_clusters_geometry(stream, o, max_clusters=U)
        fn = lambda: (view_dbg(stream, "light_indices", SHADE_W, SHADE_H, o, rgba),
                      cd.show_clusters_geometry(stream, o, verts, max_clusters=U))
    elif args.profile == "kd_tree":
        from vren_gb300 import kd_tree as kd

        rng = np.random.default_rng(SEED + 31)
        pts = rng.uniform(0, 100, (1_000_000, 3)).astype(np.float32)
        nodes_np, _ = kd.kd_tree_build(pts)
        depth_kd = kd.kd_tree_depth(nodes_np)
        d_pts = torch.from_numpy(pts.reshape(-1)).to(dev)
        d_nodes = torch.from_numpy(nodes_np.view(np.int32).reshape(-1)).to(dev)
        smp = torch.from_numpy(rng.uniform(0, 100, (1 << 20, 3)).astype(np.float32).reshape(-1)).to(dev)
        bp = torch.empty(1 << 20, dtype=torch.int32, device=dev)
        bd = torch.empty(1 << 20, dtype=torch.float32, device=dev)
        fn = lambda: kd.kd_tree_search_batch(stream, d_pts, d_nodes, smp, depth_kd, best_points=bp, best_distances=bd)
    elif args.profile in ("pyramid", "pyramid_4k"):
        # the depth pyramid at 8192x8192 (268 MB read > L2) or at 3840x2160
        from vren_gb300.depth_pyramid import depth_buffer_pyramid, depth_buffer_reductor

        w, h = (8192, 8192) if args.profile == "pyramid" else (3840, 2160)
        g = torch.Generator(device=dev).manual_seed(SEED)
        depth = torch.rand(w * h, device=dev, generator=g)
        pyr = depth_buffer_pyramid(w, h, dev)
        red = depth_buffer_reductor()
        fn = lambda: red.copy_and_reduce(stream, depth, pyr)
    elif args.profile in ("shade", "shade_backward"):
        ctx = cs.cluster_and_shade(SHADE_W, SHADE_H, 65536, 1 << 24)
        sb = shade_profile_setup(dev, stream, ctx)
        fn = sb["forward"] if args.profile == "shade" else sb["backward"]
    else:
        raise SystemExit(f"unknown profile kind {args.profile}")
    with torch.cuda.stream(stream):
        for _ in range(reps):
            fn()
    stream.synchronize()
    print(json.dumps({"profile": args.profile, "runs": reps, "device_error": vg.device_error()}))


VENDOR_RADIX_SRC = r"""
// cub::DeviceRadixSort::SortPairs (u32 keys, u32 values, all 32 bits) timed with CUDA events on its
// stream, a 256 MiB memset before each run (L2 flushed), 5 warm-up + 20 timed runs per size.
#include <cub/device/device_radix_sort.cuh>
#include <cstdint>
#include <cstdio>
#include <vector>
int main() {
  void* flush; cudaMalloc(&flush, 256u << 20);
  cudaStream_t s; cudaStreamCreate(&s);
  for (int lg : {20, 24, 26}) {
    size_t n = size_t(1) << lg;
    std::vector<uint32_t> hk(n); uint32_t r = 12345u;
    for (auto& k : hk) { r ^= r << 13; r ^= r >> 17; r ^= r << 5; k = r; }
    uint32_t *k0, *k1, *v0, *v1;
    cudaMalloc(&k0, n * 4); cudaMalloc(&k1, n * 4); cudaMalloc(&v0, n * 4); cudaMalloc(&v1, n * 4);
    cudaMemcpy(k0, hk.data(), n * 4, cudaMemcpyHostToDevice);
    size_t tb = 0; cub::DeviceRadixSort::SortPairs(nullptr, tb, k0, k1, v0, v1, (int)n, 0, 32, s);
    void* tmp; cudaMalloc(&tmp, tb);
    cudaEvent_t a, b; cudaEventCreate(&a); cudaEventCreate(&b);
    float tot = 0; int cnt = 0;
    for (int i = 0; i < 25; ++i) {
      cudaMemsetAsync(flush, i, 256u << 20, s);
      cudaEventRecord(a, s);
      cub::DeviceRadixSort::SortPairs(tmp, tb, k0, k1, v0, v1, (int)n, 0, 32, s);
      cudaEventRecord(b, s); cudaEventSynchronize(b);
      float ms; cudaEventElapsedTime(&ms, a, b); if (i >= 5) { tot += ms; ++cnt; }
    }
    printf("%d %.6f\n", lg, tot / cnt);
    cudaFree(k0); cudaFree(k1); cudaFree(v0); cudaFree(v1); cudaFree(tmp);
  }
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}
"""


def vendor_radix(args):
    """The vendor's radix sort on the same GPU for comparison: CUB's onesweep SortPairs (the library
    shipped with the CUDA toolkit), built from a short program at run time; one JSON line."""
    import tempfile

    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "cub_sort.cu"), os.path.join(d, "cub_sort")
        with open(src, "w") as f:
            f.write(VENDOR_RADIX_SRC)
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-o", exe, src],
                       check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    res = {}
    for line in out.split("\n"):
        if line.strip():
            lg, ms = line.split()
            n = 1 << int(lg)
            res[f"n=2^{lg}"] = {"ms": round(float(ms), 4), "gkeys_s": round(n / (float(ms) * 1e-3) / 1e9, 3),
                                "gbs_at_64B_per_pair": round(64.0 * n / (float(ms) * 1e-3) / 1e9, 1)}
    print(json.dumps({"vendor_radix": "cub::DeviceRadixSort::SortPairs u32/u32", "results": res}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--quick", action="store_true", help="skip the primitive sweep and the large sorts")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--profile", choices=["frame", "frame_dense", "batch", "find_unique", "find_unique_rgba16f", "radix", "scan",
                                          "shade", "shade_backward", "pyramid", "pyramid_4k", "reduce", "bucket",
                                          "build_bvh", "assign", "karras", "bouncer", "debug_views", "kd_tree",
                                          "light_bvh_multi", "batch_small"],
                    default=None,
                    help="run one kernel family on a case larger than L2 (for ncu) and exit")
    ap.add_argument("--vendor-radix", action="store_true",
                    help="time the CUDA toolkit's CUB radix sort (pairs) on this GPU for comparison and exit")
    args = ap.parse_args()
    if args.vendor_radix:
        return vendor_radix(args)
    if args.profile:
        return run_profile(args)
    args.warmup = max(args.warmup, 3)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch

        torch.distributed.init_process_group("nccl")
    try:
        if args.impl == "reference":
            run_reference(args, rank, world)
        else:
            run_ours(args, rank, world)
    finally:
        if world > 1 and args.impl == "ours":
            import torch

            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
