#!/usr/bin/env python3
"""Benchmark: Whitted ray tracing with a full LBVH rebuild per frame.

Workload (plain method, mid scale): a 1024x512-cell fBm heightfield plus 200
mirror UV spheres (1,240,576 triangles), heights animated per frame, the LBVH
rebuilt from scratch every frame, then a 1920x1080 Whitted render with 2 point
lights and reflection depth 4.  One step = one frame: vertex update (device
to device) + LBVH build + render.  Metric: Mrays/s with the reference's ray
count convention (primary + secondary rays, shadow rays not counted).

Device-timed ``value``: inputs resident in HBM, CUDA events on the launching
stream, L2 flushed (256 MiB write) between steps.  ``e2e``: the same frames
through the public host-buffer entry points with pinned host buffers (vertex
upload, build, render, RGBA8 download inside the timed region for every
frame): two frames in flight through rt_render_host_async /
rt_render_host_wait on two streams with one scene copy each (``value``), and
one frame at a time through rt_render_host (``sync_value``).

--impl reference: the oracle (CPU restatement of the reference's kernels,
point lights and several lights included) on all host cores, on a bounded
sample of the same frame.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "tesina-rt_gb300"))

METRIC = "Whitted Mrays/s (primary+secondary), full LBVH rebuild per frame"
UNIT = "Mrays/s"
B_BUILD_PER_TRI = 312 + 16 * 4      # algorithmic LBVH bytes per triangle, 4 radix passes
B_RAY_CLOSEST, B_RAY_SHADOW, B_SHADE = 40, 25, 48
# dram__bytes_read.sum + dram__bytes_write.sum of one launch of a render
# kernel on the mid-scale frame (ncu, --clock-control none), by kernel; the
# line's roofline carries it only when the autotuner installed that kernel.
RENDER_DRAM_BYTES = {
    "k_render_pool<128, 6>": (297.9 + 32.7) * 1e6,
    "k_render_pool<128, 8>": (320.0 + 37.3) * 1e6,
    "k_render_pool<256, 3>": (286.5 + 28.8) * 1e6,
    "k_render_pool<256, 4>": (318.8 + 37.1) * 1e6,
}
# the same for the stress workload (17.7 M triangles, 3840x2160, 3 lights,
# depth 6), the mean over its 8 poses
STRESS_RENDER_DRAM_BYTES = {
    "k_render_pool<128, 6>": (2041.6 + 177.7) * 1e6,
    "k_render_pool<128, 8>": (2149.0 + 209.5) * 1e6,
    "k_render_pool<256, 3>": (1931.3 + 147.6) * 1e6,
    "k_render_pool<256, 4>": (2148.2 + 209.5) * 1e6,
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = [r.split(", ") for r in self.lines if r.count(",") >= 8]
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(rows)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=20).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part")):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build as ob
    import pyoracle
    ob.build_oracle()
    return pyoracle, pyoracle.Oracle()


def _block_rows(w, h, every):
    """Sample ranges spread over the frame: every `every`-th row of the
    reference's 32 x 32 pixel blocks (rays are generated block by block, so
    one block row is one contiguous range of samples)."""
    per_row = (w // 32) * 1024
    rows = range(0, h // 32, every)
    return [(r * per_row, per_row) for r in rows]


def _oracle_sample(s, cam, w, h, nb, ranges, threads):
    t0 = time.perf_counter()
    rays = shadow = 0
    for off, cnt in ranges:
        _, st = s.render(cam, w, h, nb, offset=off, count=cnt, threads=threads)
        rays += st.primary_rays + st.secondary_rays
        shadow += st.shadow_rays
    return time.perf_counter() - t0, rays, shadow


def cpu_baseline(scene, cam, w, h, nb, every=8, one_thread=True):
    """The oracle (CPU restatement of the reference's kernels) on a bounded,
    spread sample of one frame: the full LBVH build (sequential, as the
    restatement builds) and every `every`-th row of 32 x 32 pixel blocks
    traced, shadowed, shaded and reflected to the frame's depth, on all host
    cores and on one.  The build is charged in proportion to the sampled
    fraction of the frame; Mrays/s counts primary + secondary rays."""
    pyoracle, orc = _oracle()
    s = orc.new_scene(scene)
    t0 = time.perf_counter()
    s.build(30, 1, 0)
    t_build = time.perf_counter() - t0
    ranges = _block_rows(w, h, every)
    n_smp = sum(c for _, c in ranges)
    frac = n_smp / float(w * h)
    threads = os.cpu_count() or 1
    t_n, rays, shadow = _oracle_sample(s, cam, w, h, nb, ranges, threads)
    out = {"value": rays / (t_build * frac + t_n) / 1e6, "unit": UNIT, "cores": threads,
           "kind": "port", "cpu_model": cpu_model(),
           "sample": "oracle: full LBVH build of %d triangles (%.3f s, one thread, charged x%.4f) "
                     "+ every %dth row of 32x32 pixel blocks of the %dx%d frame (%d samples, "
                     "%.1f %%; %d primary + secondary rays) traced to depth %d on %d threads "
                     "(%.3f s)" % (scene.n_tris, t_build, frac, every, w, h, n_smp, 100 * frac,
                                   rays, nb, threads, t_n),
           "lbvh_mtri_s": scene.n_tris / t_build / 1e6,
           "mrays_all_incl_shadow": (rays + shadow) / (t_build * frac + t_n) / 1e6}
    if one_thread:
        t_1, rays1, _ = _oracle_sample(s, cam, w, h, nb, ranges, 1)
        out["one_thread"] = {"value": rays1 / (t_build * frac + t_1) / 1e6, "cores": 1,
                             "render_s": t_1}
    return out, s


def cpu_c0_full():
    """The small workload (10k-triangle soup, 512 x 512, depth 3) run in full
    on the oracle: LBVH build + the whole frame, one thread and all."""
    from rtgb import scenes
    pyoracle, orc = _oracle()
    wl = scenes.workload_small()
    s = orc.new_scene(wl["scene"])
    t0 = time.perf_counter()
    s.build(30, 1, 0)
    t_build = time.perf_counter() - t0
    out = {"workload": wl["name"], "build_s": t_build,
           "lbvh_mtri_s": wl["scene"].n_tris / t_build / 1e6}
    for name, thr in (("one_thread", 1), ("all_threads", os.cpu_count() or 1)):
        t0 = time.perf_counter()
        _, st = s.render(wl["camera"], 512, 512, 3, threads=thr)
        t = time.perf_counter() - t0
        rays = st.primary_rays + st.secondary_rays
        out[name] = {"cores": thr, "render_s": t, "rays": rays,
                     "mrays_s": rays / (t_build + t) / 1e6}
    return out


def traversal_work(s, cam, w, h, sample_rays=65536):
    """Node and triangle records the oracle's traversal reads per primary ray
    and per shadow ray of those rays (interior nodes entered, 64 B each;
    triangles tested, 48 B), on the first `sample_rays` samples."""
    pyoracle, orc = _oracle()
    smp = pyoracle.gen_primary(orc, cam, w, h, count=sample_rays)
    tc = s.traversal_counts(smp, threads=os.cpu_count() or 1)
    n_sh = max(1, tc["shadow_rays"])
    return {"rays": sample_rays, "shadow_traced_frac": tc["shadow_traced"] / n_sh,
            "nodes_per_ray": tc["nodes"] / sample_rays,
            "tris_per_ray": tc["tris"] / sample_rays,
            "shadow_nodes_per_ray": tc["shadow_nodes"] / n_sh,
            "shadow_tris_per_ray": tc["shadow_tris"] / n_sh,
            "bytes_per_ray": (64 * tc["nodes"] + 48 * tc["tris"]) / sample_rays,
            "bytes_per_shadow_ray": (64 * tc["shadow_nodes"] + 48 * tc["shadow_tris"]) / n_sh}


def emit_levels_of(n):
    """Launches of the LBVH emit for n triangles (512 per level-0 block,
    then groups of 8 blocks up to the root)."""
    levels, nb = 1, (n + 511) // 512
    while nb > 1:
        nb, levels = (nb + 7) // 8, levels + 1
    return levels


def measure_batched(ctx, lib, torch, reps=5):
    """Batched workload: 64 scenes built in one launch and rendered in one
    launch (CUDA-graph replay) against the same 64 requests through the plain
    per-request path (build + render per scene, one stream).  Pixels of both
    are compared; throughput is Mrays/s (primary + secondary)."""
    from rtgb import capi, scenes
    wl = scenes.workload_batched()
    items = wl["items"]
    stream = torch.cuda.Stream()
    sh = C.c_void_p(stream.cuda_stream)
    gs = [capi.Scene(ctx, it["scene"]) for it in items]
    px = sum(it["width"] * it["height"] for it in items)
    tris = sum(it["scene"].n_tris for it in items)
    # plain per-request path
    rgba_plain = [ctx.alloc(4 * it["width"] * it["height"]) for it in items]
    stats = ctx.alloc(32)

    def plain_all():
        for g, it, out in zip(gs, items, rgba_plain):
            g.build(30, 1, stream=sh)
            g.render(it["camera"], it["width"], it["height"], it["max_bounces"], out, None,
                     stats, stream=sh)

    for _ in range(2):
        plain_all()
    torch.cuda.synchronize()
    stats.zero(sh)
    t_plain = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plain_all()
        e1.record(stream)
        stream.synchronize()
        t_plain.append(e0.elapsed_time(e1))
    rays = stats.read(np.uint64)
    rays_plain = int(rays[0] + rays[1]) // reps
    # batched: one build launch + one render launch, graph-replayed
    batch = capi.Batch(ctx)
    batch.set([(g, it["camera"], it["width"], it["height"], it["max_bounces"])
               for g, it in zip(gs, items)])
    rgba_b = ctx.alloc(4 * px)
    bstats = ctx.alloc(32)
    batch.capture(rgba_b, bstats)
    for _ in range(2):
        batch.replay(sh)
    torch.cuda.synchronize()
    t_b = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batch.replay(sh)
        e1.record(stream)
        stream.synchronize()
        t_b.append(e0.elapsed_time(e1))
    st = bstats.read(np.uint64)
    rays_b = int(st[0] + st[1])
    out = rgba_b.read(np.uint8)
    same = all(np.array_equal(out[4 * off:4 * (off + w * h)], rp.read(np.uint8))
               for (off, w, h), rp in zip(batch.offsets, rgba_plain))
    mp = rays_plain / (statistics.median(t_plain) * 1e-3) / 1e6
    mb = rays_b / (statistics.median(t_b) * 1e-3) / 1e6
    batch.close()
    return {"workload": wl["name"], "scenes": len(items), "triangles": tris, "pixels": px,
            "rays_per_batch": rays_b, "plain_ms": statistics.median(t_plain),
            "batched_ms": statistics.median(t_b), "plain_mrays_s": mp, "batched_mrays_s": mb,
            "speedup": mb / mp, "identical_pixels": bool(same and rays_b == rays_plain),
            # build: the cooperative launch + one emit launch per level of the
            # largest scene; render: the pooled kernel + the RGBA8 conversion
            "launches_per_batch": 1 + max(emit_levels_of(it["scene"].n_tris) for it in items) + 2,
            "launches_plain": sum(7 + emit_levels_of(it["scene"].n_tris) + 2 for it in items)}


def measure_stress(ctx, lib, torch, builds=5, cpu=True):
    """Plain method at stress scale: a 4096x2048-cell fBm field plus 1,000
    mirror spheres (17,737,216 triangles), one LBVH build timed `builds`
    times (median), then one 3840x2160 Whitted frame (3 point lights, depth
    6) from each of 8 camera poses on a radius-10 sphere.  Build Mtri/s is
    reported against the HBM roofline with the same 376 B/triangle model as
    the main workload; Mrays/s counts primary + secondary rays (and,
    separately, shadow rays too).  The leg has its own e2e (build and the
    first pose through rt_render_host from pinned host vertices to a host
    RGBA8 image), render roofline and CPU baseline (the oracle on a spread
    sample of the first pose)."""
    from rtgb import abi, capi, scenes
    wl = scenes.workload_stress()
    t = time.time()
    sc = wl["terrain"].scene(0)
    log("stress: %d triangles made in %.1f s" % (sc.n_tris, time.time() - t))
    stream = torch.cuda.Stream()
    sh = C.c_void_p(stream.cuda_stream)
    g = capi.Scene(ctx, sc)
    w, h, nb = wl["width"], wl["height"], wl["max_bounces"]
    rgba = ctx.alloc(4 * w * h)
    stats = ctx.alloc(32)
    ctx.sync()
    rv = ctx.render_config().variant
    vt, vm, _ = ctx.variants()[rv]
    kname = ("k_render_pool<%d, %d>" if ctx.variant_pooled(rv) else "k_render<%d, %d>") % (vt, vm)
    t_build = []
    for k in range(2 + builds):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.build(wl["depth"], wl["min_leaf"], stream=sh)
        e1.record(stream)
        stream.synchronize()
        if k >= 2:
            t_build.append(e0.elapsed_time(e1))
    g.render(wl["cameras"][0], w, h, nb, rgba, None, None, stream=sh)   # warm-up
    stats.zero(sh)
    stream.synchronize()
    t_render = []
    for cam in wl["cameras"]:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.render(cam, w, h, nb, rgba, None, stats, stream=sh)
        e1.record(stream)
        stream.synchronize()
        t_render.append(e0.elapsed_time(e1))
    st = stats.read(np.uint64)
    rays, shadow = int(st[0] + st[1]), int(st[2])
    hbm, kind = peaks()
    mb = statistics.median(t_build)
    ach = B_BUILD_PER_TRI * sc.n_tris / (mb * 1e-3) / 1e9
    tr = sum(t_render)
    render_bytes = rays * (B_RAY_CLOSEST + B_SHADE) + shadow * B_RAY_SHADOW
    render_gbs = render_bytes / (tr * 1e-3) / 1e9
    # e2e: upload + build + pose 0 + RGBA8 download per step
    V = sc.n_verts
    pin_pos = torch.from_numpy(np.ascontiguousarray(sc.pos4)).pin_memory()
    pin_nrm = torch.from_numpy(np.ascontiguousarray(sc.nrm4)).pin_memory()
    host_rgba = torch.empty((h * w, 4), dtype=torch.uint8).pin_memory()
    cfg = abi.BvhCfg(wl["depth"], wl["min_leaf"])
    hst = abi.RenderStats()
    e2e_ms, e2e_rays = [], 0
    for k in range(4):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        capi.check(lib, lib.rt_render_host(ctx.h, g.h, C.c_void_p(pin_pos.data_ptr()),
                                           C.c_void_p(pin_nrm.data_ptr()), V, C.byref(cfg),
                                           C.byref(wl["cameras"][0]), w, h, nb,
                                           C.c_void_p(host_rgba.data_ptr()), C.byref(hst), sh))
        e1.record(stream)
        stream.synchronize()
        if k:
            e2e_ms.append(e0.elapsed_time(e1))
            e2e_rays += int(hst.primary_rays + hst.secondary_rays)
    cpu_leg = None
    if cpu:
        try:
            cpu_leg, _ = cpu_baseline(sc, wl["cameras"][0], w, h, nb, every=16, one_thread=False)
        except Exception as e:
            cpu_leg = {"value": None, "sample": "failed: %s" % e}
    return {"workload": wl["name"], "triangles": sc.n_tris, "width": w, "height": h,
            "max_bounces": nb, "lights": 3, "poses": len(wl["cameras"]),
            "build_ms": mb, "lbvh_mtri_s": sc.n_tris / (mb * 1e-3) / 1e6,
            "build_roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                               "frac": ach / hbm, "bytes_per_tri": B_BUILD_PER_TRI,
                               "peak_kind": kind},
            "render_ms_per_pose": tr / len(t_render), "rays": rays, "shadow_rays": shadow,
            "mrays_s": rays / (tr * 1e-3) / 1e6,
            "mrays_all_incl_shadow": (rays + shadow) / (tr * 1e-3) / 1e6,
            "roofline": {"kernel": kname, "bound": "hbm",
                         "achieved": render_gbs, "peak": hbm, "unit": "GB/s",
                         "frac": render_gbs / hbm,
                         "traffic": STRESS_RENDER_DRAM_BYTES.get(kname), "peak_kind": kind,
                         "algorithmic_bytes_per_pose": render_bytes / len(t_render)},
            "e2e": {"value": e2e_rays / (sum(e2e_ms) * 1e-3) / 1e6, "unit": UNIT,
                    "h2d_bytes_per_step": 2 * 16 * V, "d2h_bytes_per_step": 4 * w * h + 32,
                    "ms_per_step": statistics.median(e2e_ms)},
            "cpu_baseline": cpu_leg,
            "device_status": ctx.device_status()}


SERVED_KEYS = ("p50_ms", "p99_ms", "mean_ms", "max_ms", "mrays_s", "req_s", "rays", "span_ms",
               "launches", "mean_batch_views", "failed", "upload_failed", "upload_p50_ms",
               "evicted", "resident_scenes")


def measure_refit(ctx, torch, frames=20, warmup=3):
    """Refit-only frames (the reference's bvh_refit_only mode,
    renderer.cpp:53-70) with device-side animation (mangle, mangler.cl:12-32,
    run before each frame as rt-wave.cpp:141-167 runs it, wave height 0.2):
    the mid-scale terrain built once, then per frame mangle + refit + the
    1920x1080 depth-4 render, L2 flushed between frames.  Per-phase CUDA
    events on the frame's stream; Mrays/s counts primary + secondary rays."""
    from rtgb import capi, scenes
    wl = scenes.workload_mid()
    sc = wl["terrain"].scene(0)
    stream = torch.cuda.Stream()
    sh = C.c_void_p(stream.cuda_stream)
    g = capi.Scene(ctx, sc)
    g.build(30, 1, stream=sh)
    w, h, nb = wl["width"], wl["height"], wl["max_bounces"]
    rgba = ctx.alloc(4 * w * h)
    stats = ctx.alloc(32)
    flush = ctx.alloc(256 << 20)
    t_m, t_r, t_d = [], [], []
    stats.zero(sh)
    for f in range(warmup + frames):
        arg = 1.0 + f
        flush.zero(sh)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        ev[0].record(stream)
        g.mangle(arg, arg - 1.0, 0.2, stream=sh)
        ev[1].record(stream)
        g.refit(stream=sh)
        ev[2].record(stream)
        g.render(wl["camera"], w, h, nb, rgba, None, stats if f >= warmup else None, stream=sh)
        ev[3].record(stream)
        stream.synchronize()
        if f >= warmup:
            t_m.append(ev[0].elapsed_time(ev[1]))
            t_r.append(ev[1].elapsed_time(ev[2]))
            t_d.append(ev[2].elapsed_time(ev[3]))
    st = stats.read(np.uint64)
    rays = int(st[0] + st[1])
    total = sum(t_m) + sum(t_r) + sum(t_d)
    mr = statistics.median(t_r)
    return {"workload": wl["name"] + "_mangle_refit", "triangles": sc.n_tris,
            "vertices": sc.n_verts, "frames": frames, "mangle_ms": statistics.median(t_m),
            "refit_ms": mr, "refit_mtri_s": sc.n_tris / (mr * 1e-3) / 1e6,
            "render_ms": statistics.median(t_d), "frame_ms": total / frames,
            "mrays_s": rays / (total * 1e-3) / 1e6, "device_status": ctx.device_status()}


def measure_refraction(ctx, torch, frames=5):
    """Refraction: the mid-scale terrain with its 200 spheres made of glass
    (refractive index 1.333, reflectiveness 0.9: every hit on a sphere sends
    a refracted and a reflected ray, weighted by Schlick's factor), built
    once and rendered at 1920x1080 depth 4 through rt_render (the ray-tree
    variant).  Mrays/s counts primary + secondary rays."""
    from rtgb import capi, scenes
    wl = scenes.workload_mid()
    sc = wl["terrain"].scene(0)
    mats = sc.mats.copy()
    mats["refractive_index"][1] = 1.333      # the spheres' material
    mats["reflectiveness"][1] = 0.9
    sc = scenes.Scene(sc.pos4, sc.nrm4, sc.idx, mats, sc.mat_map, sc.lights)
    stream = torch.cuda.Stream()
    sh = C.c_void_p(stream.cuda_stream)
    g = capi.Scene(ctx, sc)
    g.build(30, 1, stream=sh)
    w, h, nb = wl["width"], wl["height"], wl["max_bounces"]
    rgba = ctx.alloc(4 * w * h)
    stats = ctx.alloc(32)
    g.render(wl["camera"], w, h, nb, rgba, None, None, stream=sh)
    stats.zero(sh)
    ts = []
    for _ in range(frames):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.render(wl["camera"], w, h, nb, rgba, None, stats, stream=sh)
        e1.record(stream)
        stream.synchronize()
        ts.append(e0.elapsed_time(e1))
    st = stats.read(np.uint64)
    rays = int(st[0] + st[1])
    return {"workload": "terrain1M_glass_spheres_1920x1080_d4", "triangles": sc.n_tris,
            "render_ms": statistics.median(ts), "rays_per_frame": rays // frames,
            "secondary_per_frame": int(st[1]) // frames,
            "mrays_s": rays / (sum(ts) * 1e-3) / 1e6, "device_status": ctx.device_status()}


def measure_obj(ctx, torch, frames=5):
    """OBJ input: the mid-scale terrain written as an OBJ file (v, vn and
    v//vn faces; the reference's own models are not on every machine), read
    through rt_obj_load (the reader's host time), then uploaded, built and
    rendered at 1920x1080 depth 4 as one aggregate mesh with one material,
    as the reference's OBJ scenes are."""
    import tempfile
    from rtgb import capi, obj, scenes
    wl = scenes.workload_mid()
    ter = wl["terrain"].scene(0)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "terrain1M.obj")
        obj.write(path, ter.pos4, ter.nrm4, ter.idx)
        size = os.path.getsize(path)
        t0 = time.perf_counter()
        sc = obj.load(path, lights=ter.lights)
        t_read = time.perf_counter() - t0
    stream = torch.cuda.Stream()
    sh = C.c_void_p(stream.cuda_stream)
    t0 = time.perf_counter()
    g = capi.Scene(ctx, sc)
    g.build(30, 1, stream=sh)
    stream.synchronize()
    t_up = time.perf_counter() - t0
    w, h, nb = wl["width"], wl["height"], wl["max_bounces"]
    rgba = ctx.alloc(4 * w * h)
    stats = ctx.alloc(32)
    g.render(wl["camera"], w, h, nb, rgba, None, None, stream=sh)
    stats.zero(sh)
    ts = []
    for _ in range(frames):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.render(wl["camera"], w, h, nb, rgba, None, stats, stream=sh)
        e1.record(stream)
        stream.synchronize()
        ts.append(e0.elapsed_time(e1))
    st = stats.read(np.uint64)
    return {"workload": "terrain1M_as_obj_1920x1080_d4", "triangles": sc.n_tris,
            "vertices": sc.n_verts, "file_mb": size / 1e6, "read_s": t_read,
            "read_mtri_s": sc.n_tris / t_read / 1e6, "read_mb_s": size / t_read / 1e6,
            "upload_build_s": t_up, "render_ms": statistics.median(ts),
            "mrays_s": int(st[0] + st[1]) / (sum(ts) * 1e-3) / 1e6,
            "device_status": ctx.device_status()}


def measure_instances(ctx, torch, frames=5):
    """Multi-root: 16 instances of two meshes (rtgb.scenes.workload_instances)
    rendered at 1920x1080 depth 4 through rt_instances_render, each frame
    after new transforms for the 12 soups (rt_instances_set_transforms, the
    per-frame root update of animated objects).  Beside it, the same
    geometry flattened into one mesh (vertices moved on the host) and
    rendered through the single-root path, for the cost of instancing.
    Mrays/s counts primary + secondary rays."""
    from rtgb import capi, scenes
    wl = scenes.workload_instances()
    stream = torch.cuda.Stream()
    sh = C.c_void_p(stream.cuda_stream)
    gs = []
    for sc in wl["meshes"]:
        g = capi.Scene(ctx, sc)
        g.build(30, 1, stream=sh)
        gs.append(g)
    stream.synchronize()
    I = capi.Instances(ctx, gs, wl["inst"], wl["tr"], wl["tr_inv"], wl["lights"])
    w, h, nb = wl["width"], wl["height"], wl["max_bounces"]
    rgba = ctx.alloc(4 * w * h)
    stats = ctx.alloc(32)
    I.render(wl["camera"], w, h, nb, rgba, None, None, stream=sh)
    stats.zero(sh)
    trs = []
    for f in range(frames):          # turn the soups a little each frame
        T, Ti = wl["tr"].copy(), wl["tr_inv"].copy()
        for k in range(4, T.shape[0]):
            m, mi = scenes.transform(5.0 * (f + 1))
            T[k] = T[k] @ m
            Ti[k] = mi @ Ti[k]
        trs.append((T, Ti))
    ts = []
    for f in range(frames):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        stream.synchronize()
        e0.record(stream)
        I.set_transforms(*trs[f])        # ordered on the context stream before the render
        I.render(wl["camera"], w, h, nb, rgba, None, stats, stream=sh)
        e1.record(stream)
        stream.synchronize()
        ts.append(e0.elapsed_time(e1))
    st = stats.read(np.uint64)
    rays = int(st[0] + st[1])
    out = {"workload": wl["name"], "instances": int(len(wl["inst"])), "meshes": len(gs),
           "triangles_instanced": int(sum(wl["meshes"][i].n_tris for i in wl["inst"])),
           "render_ms": statistics.median(ts), "rays_per_frame": rays // frames,
           "mrays_s": rays / (sum(ts) * 1e-3) / 1e6}
    I.close()
    # the same geometry as one aggregate mesh, at the first frame's transforms
    T, _ = trs[0]
    pos, nrm, idx, mats, mmap, base = [], [], [], [], [], 0
    for k, si in enumerate(wl["inst"]):
        sc = wl["meshes"][si]
        p = sc.pos4.copy()
        p[:, 3] = 1.0
        p = (p @ T[k].T).astype(np.float32)
        p[:, 3] = 0.0
        n = sc.nrm4.copy()
        n[:, :3] = n[:, :3] @ T[k][:3, :3].T
        pos.append(p), nrm.append(n.astype(np.float32)), idx.append(sc.idx + base)
        mmap.append(sc.mat_map + sum(len(m) for m in mats))
        mats.append(sc.mats)
        base += sc.pos4.shape[0]
    flat = scenes.Scene(np.concatenate(pos), np.concatenate(nrm), np.concatenate(idx),
                        np.concatenate(mats), np.concatenate(mmap).astype(np.uint32),
                        wl["lights"])
    g = capi.Scene(ctx, flat)
    g.build(30, 1, stream=sh)
    g.render(wl["camera"], w, h, nb, rgba, None, None, stream=sh)
    stats.zero(sh)
    ts = []
    for _ in range(frames):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.render(wl["camera"], w, h, nb, rgba, None, stats, stream=sh)
        e1.record(stream)
        stream.synchronize()
        ts.append(e0.elapsed_time(e1))
    st = stats.read(np.uint64)
    out.update({"flattened_render_ms": statistics.median(ts),
                "flattened_mrays_s": int(st[0] + st[1]) / (sum(ts) * 1e-3) / 1e6,
                "device_status": ctx.device_status()})
    return out


def measure_sah(ctx, torch, frames=5):
    """LBVH against the reference's CPU SAH BVH (rt_bvh_build_sah) on a
    1M-triangle soup (the small workload's kind of scene; the mid-scale
    terrain's SAH tree is 36 levels deep, beyond the traversal's 32-entry
    stack, and is refused): the SAH build's wall time (device to host copy,
    the host build on all cores, the tree back on the device) and the same
    1920x1080 depth-4 frame rendered over either tree."""
    from rtgb import capi, scenes
    sc = scenes.soup(1_000_000, seed=1)
    cam = scenes.camera((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), fov_deg=60.0, aspect=1920 / 1080)
    wl = {"camera": cam, "width": 1920, "height": 1080, "max_bounces": 4}
    stream = torch.cuda.Stream()
    sh = C.c_void_p(stream.cuda_stream)
    w, h, nb = wl["width"], wl["height"], wl["max_bounces"]
    rgba = ctx.alloc(4 * w * h)
    stats = ctx.alloc(32)
    out = {"workload": "soup1M_1920x1080_d4", "triangles": sc.n_tris,
           "host_threads": os.cpu_count()}
    for kind in ("lbvh", "sah"):
        g = capi.Scene(ctx, sc)
        stream.synchronize()
        t0 = time.perf_counter()
        if kind == "sah":
            g.build_sah(stream=sh)
        else:
            g.build(30, 1, stream=sh)
        stream.synchronize()
        t_build = time.perf_counter() - t0
        g.render(wl["camera"], w, h, nb, rgba, None, None, stream=sh)
        stats.zero(sh)
        ts = []
        for _ in range(frames):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            g.render(wl["camera"], w, h, nb, rgba, None, stats, stream=sh)
            e1.record(stream)
            stream.synchronize()
            ts.append(e0.elapsed_time(e1))
        st = stats.read(np.uint64)
        out[kind] = {"build_wall_ms": t_build * 1e3, "render_ms": statistics.median(ts),
                     "mrays_s": int(st[0] + st[1]) / (sum(ts) * 1e-3) / 1e6,
                     "image_crc": int(np.bitwise_xor.reduce(rgba.read(np.uint32)))}
        g.close()
    out["device_status"] = ctx.device_status()
    return out


def measure_served(ctx, rates=(2000, 1000, 300, 50), n_req=400, seed=5):
    """Served workload: 32 resident scenes (soups and fBm fields alternating,
    10k-2M triangles log-uniform), a 120 GB admission budget and a scene cap
    of 32, so that each upload (5% of requests; copy + LBVH build) displaces
    the least recently used scene.  Requests: camera on a sphere of radius
    U[3,6] aimed at the origin, pixels log-uniform 128^2..1920x1080, depth
    U{1..5}.  One burst (all requests at t=0: capacity) and Poisson streams
    at several rates, each through the served configuration (continuous
    batching: up to 256 requests per launch, 3 launches in flight) and the
    plain per-request configuration (one rt_render launch per request, one at
    a time).  Latency = submit to image in pinned host memory, server clock;
    Mrays/s = primary+secondary rays / (last done - first submit).  Images
    of the two configurations are compared request by request (CRC32)."""
    from rtgb import scenes, served
    wl = scenes.workload_served(seed)
    cache = served.SceneCache(wl)
    t = time.time()
    for s in wl["pool"] + wl["uploads"]:
        cache.get(s)
    log("served: %d pool + %d upload scenes made in %.1f s" % (len(wl["pool"]), len(wl["uploads"]),
                                                             time.time() - t))
    cfgs = (("served", dict(max_views=256, max_inflight=3)), ("plain", dict(max_views=1)))
    # warm-up: module loads, pinned staging, first launches
    warm = scenes.served_requests(24, None, seed=seed + 99)
    for _, kw in cfgs:
        served.run_stream(ctx, cache, warm, hash_images=False, **kw)
    runs = []
    identical = True
    for rate in (None,) + tuple(rates):
        n = n_req if rate is None or rate >= 200 else max(100, int(rate * 4))
        reqs = scenes.served_requests(n, rate, seed=seed + 100 + (rate or 0))
        row = {"rate_req_s": rate if rate else "burst", "requests": n,
               "uploads": sum(r["kind"] == "upload" for r in reqs)}
        crcs = {}
        for name, kw in cfgs:
            r = served.run_stream(ctx, cache, reqs, **kw)
            crcs[name] = r["crc"]
            row[name] = {k: r[k] for k in SERVED_KEYS}
        row["identical_images"] = bool(crcs["served"] == crcs["plain"] and
                                       len(crcs["plain"]) == n - row["uploads"])
        row["served_p99_le_plain_p50"] = row["served"]["p99_ms"] <= row["plain"]["p50_ms"]
        row["mrays_ratio"] = row["served"]["mrays_s"] / max(row["plain"]["mrays_s"], 1e-9)
        identical &= row["identical_images"]
        log("served rate %s: served p50 %.2f p99 %.2f ms %.0f Mrays/s | plain p50 %.2f p99 %.2f ms "
            "%.0f Mrays/s | same %s" % (row["rate_req_s"], row["served"]["p50_ms"],
                                        row["served"]["p99_ms"], row["served"]["mrays_s"],
                                        row["plain"]["p50_ms"], row["plain"]["p99_ms"],
                                        row["plain"]["mrays_s"], row["identical_images"]))
        runs.append(row)
    burst = runs[0]
    return {"workload": wl["name"],
            "pool_scenes": len(wl["pool"]),
            "pool_triangles": int(sum(s[1] for s in wl["pool"])),
            "hbm_budget_gb": 120, "max_scenes": len(wl["pool"]), "upload_frac": 0.05,
            "served_cfg": dict(cfgs[0][1]), "plain_cfg": dict(cfgs[1][1]),
            "capacity_mrays_s": {"served": burst["served"]["mrays_s"],
                                 "plain": burst["plain"]["mrays_s"],
                                 "ratio": burst["mrays_ratio"]},
            "identical_images": identical, "runs": runs}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from rtgb import scenes
    wl = scenes.workload_mid()
    ter = wl["terrain"]
    vals = []
    for i in range(args.warmup + args.steps):
        pos, nrm = ter.frame_vertices(i % 60)
        sc = scenes.Scene(pos, nrm, ter.idx, ter.mats, ter.mat_map, ter.lights)
        r, _ = cpu_baseline(sc, wl["camera"], wl["width"], wl["height"], wl["max_bounces"],
                            one_thread=False)
        if i >= args.warmup:
            vals.append(r)
    v = statistics.median([r["value"] for r in vals])
    out = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": wl["name"], "triangles": wl["terrain"].n_tris,
                      "width": wl["width"], "height": wl["height"],
                      "max_bounces": wl["max_bounces"], "lights": 2, "lbvh_depth": 30},
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": vals[-1]["cores"],
                            "kind": "port", "sample": vals[-1]["sample"],
                            "cpu_model": vals[-1]["cpu_model"]},
           "lbvh_mtri_s": statistics.median([r["lbvh_mtri_s"] for r in vals]),
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    return 0


def run_gpu(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from rtgb import abi, capi, scenes
    from rtgb import build as rb
    if rank == 0:
        rb.build()
    if world > 1:
        torch.distributed.barrier()
    lib = capi.load()
    wl = scenes.workload_mid(seed=1 + rank)       # each replica renders its own scene
    ter = wl["terrain"]
    w, h, nb = wl["width"], wl["height"], wl["max_bounces"]
    ctx = capi.Context(local)
    stream = torch.cuda.Stream()
    sh = C.c_void_p(stream.cuda_stream)
    # the animation has 60 frames; steps cycle through them
    nframes = min(60, args.warmup + args.steps)
    frames = [ter.frame_vertices(i) for i in range(nframes)]
    scene = capi.Scene(ctx, ter.scene(0))
    V = frames[0][0].shape[0]
    # device-resident per-frame vertices
    dpos = [ctx.to_device(p) for p, _ in frames]
    dnrm = [ctx.to_device(n) for _, n in frames]
    rgba = ctx.alloc(4 * w * h)
    stats = ctx.alloc(32)
    flush = ctx.alloc(256 << 20)
    ctx.sync()

    def step(i, ev=None):
        check = capi.check
        check(lib, lib.rt_scene_update_vertices_device(ctx.h, scene.h, dpos[i].ptr, dnrm[i].ptr,
                                                       V, sh))
        if ev:
            ev[0].record(stream)
        scene.build(30, 1, stream=sh)
        if ev:
            ev[1].record(stream)
        scene.render(wl["camera"], w, h, nb, rgba, None, stats, stream=sh)
        if ev:
            ev[2].record(stream)

    for i in range(args.warmup):
        stats.zero(sh)
        step(i)
    torch.cuda.synchronize()
    # the project's autotuner picks block shape, resident blocks and packet
    # width on this scene (outside the timed region)
    if args.render_variant is None:
        tuned, tuned_ms = scene.autotune(wl["camera"], w, h, nb, trials=3)
        log("autotuned", tuned, "%.3f ms" % tuned_ms)
    else:   # a fixed configuration (profiling runs: serialised launches mislead the tuner)
        ctx.set_render_config(args.render_variant, args.render_blocks, args.render_chunk)
        tuned, tuned_ms = ctx.render_config(), None
        log("fixed render configuration", tuned)
    sampler = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler.start()
    time.sleep(0.3)
    t_steps, t_build, t_render = [], [], []
    rays = 0
    shadow = 0
    wall0 = time.perf_counter()
    for k in range(args.steps):
        i = (args.warmup + k) % nframes
        flush.zero(sh)                                 # L2 flush, outside the timed interval
        stats.zero(sh)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        ev[3].record(stream)
        step(i, ev)
        stream.synchronize()
        st = stats.read(np.uint64)
        rays += int(st[0] + st[1])
        shadow += int(st[2])
        t_steps.append(ev[3].elapsed_time(ev[2]))
        t_build.append(ev[0].elapsed_time(ev[1]))
        t_render.append(ev[1].elapsed_time(ev[2]))
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    dev_status = ctx.device_status()
    total_ms = sum(t_steps)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([total_ms, float(rays)], device="cuda")
        mx = t.clone()
        dist.all_reduce(mx[0:1], op=dist.ReduceOp.MAX)
        dist.all_reduce(t[1:2], op=dist.ReduceOp.SUM)
        total_ms, rays_all = float(mx[0]), float(t[1])
    else:
        rays_all = float(rays)
    value = rays_all / (total_ms * 1e-3) / 1e6

    # e2e through the public entry point with pinned host buffers
    pin_pos = [torch.from_numpy(p).pin_memory() for p, _ in frames]
    pin_nrm = [torch.from_numpy(n).pin_memory() for _, n in frames]
    host_rgba = [torch.empty((h * w, 4), dtype=torch.uint8).pin_memory() for _ in range(2)]
    cfg = abi.BvhCfg(30, 1)
    hst = [abi.RenderStats(), abi.RenderStats()]

    def e2e_step(i):
        capi.check(lib, lib.rt_render_host(ctx.h, scene.h, C.c_void_p(pin_pos[i].data_ptr()),
                                           C.c_void_p(pin_nrm[i].data_ptr()), V, C.byref(cfg),
                                           C.byref(wl["camera"]), w, h, nb,
                                           C.c_void_p(host_rgba[0].data_ptr()), C.byref(hst[0]),
                                           sh))
        return int(hst[0].primary_rays + hst[0].secondary_rays)

    # (1) one frame at a time: rt_render_host, L2 flushed between frames
    for i in range(min(args.warmup, nframes)):
        e2e_step(i)
    sync_ms, sync_rays = [], 0
    for k in range(args.steps):
        flush.zero(sh)
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sync_rays += e2e_step((args.warmup + k) % nframes)
        e1.record(stream)
        stream.synchronize()
        sync_ms.append(e0.elapsed_time(e1))
    # (2) two frames in flight: rt_render_host_async on two streams, each
    # with its own copy of the scene, frame k collected after frame k + 1 is
    # queued, so one frame's uploads and read-back overlap the other's build
    # and render.  Each frame still uploads its vertices and reads back its
    # image inside the timed region.  Consecutive frames use different scene
    # copies: a frame's buffers were last touched two frames before, with the
    # other copy's frame (a working set of about 250 MB, twice the L2) between.
    scene2 = capi.Scene(ctx, ter.scene(0))
    pair = [scene, scene2]
    stream2 = torch.cuda.Stream()
    shs = [sh, C.c_void_p(stream2.cuda_stream)]

    def e2e_issue(k, i):
        j = k % 2
        capi.check(lib, lib.rt_render_host_async(
            ctx.h, pair[j].h, C.c_void_p(pin_pos[i].data_ptr()), C.c_void_p(pin_nrm[i].data_ptr()),
            V, C.byref(cfg), C.byref(wl["camera"]), w, h, nb, C.c_void_p(host_rgba[j].data_ptr()),
            C.byref(hst[j]), shs[j]))

    def e2e_collect(k):
        j = k % 2
        ctx.render_host_wait(shs[j])
        return int(hst[j].primary_rays + hst[j].secondary_rays)

    def e2e_run(first, count):
        rays_run = 0
        for k in range(count):
            e2e_issue(k, (first + k) % nframes)
            if k:
                rays_run += e2e_collect(k - 1)
        return rays_run + e2e_collect(count - 1)

    e2e_run(0, min(max(args.warmup, 2), nframes))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    stream2.wait_event(e0)
    e2e_rays = e2e_run(args.warmup, args.steps)
    stream.wait_stream(stream2)
    e1.record(stream)
    stream.synchronize()
    e2e_total = e0.elapsed_time(e1)
    sync_total = sum(sync_ms)
    # (3) the device-resident frame (vertex update from HBM, build, render)
    # with the same two frames in flight and no host copies: the device-side
    # counterpart of (2)
    outs = [rgba, ctx.alloc(4 * w * h)]
    pstats = [ctx.alloc(32), ctx.alloc(32)]

    def dev_issue(k, i):
        j = k % 2
        capi.check(lib, lib.rt_scene_update_vertices_device(ctx.h, pair[j].h, dpos[i].ptr,
                                                            dnrm[i].ptr, V, shs[j]))
        pair[j].build(30, 1, stream=shs[j])
        pair[j].render(wl["camera"], w, h, nb, outs[j], None, pstats[j], stream=shs[j])

    for k in range(2):
        dev_issue(k, k % nframes)
    torch.cuda.synchronize()
    for j in range(2):
        pstats[j].zero(shs[j])
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    stream2.wait_event(e0)
    for k in range(args.steps):
        dev_issue(k, (args.warmup + k) % nframes)
    stream.wait_stream(stream2)
    e1.record(stream)
    stream.synchronize()
    pipe_total = e0.elapsed_time(e1)
    pipe_rays = 0
    for j in range(2):
        st2 = pstats[j].read(np.uint64)
        pipe_rays += int(st2[0] + st2[1])
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([e2e_total, float(e2e_rays), sync_total, float(sync_rays), pipe_total,
                          float(pipe_rays)], device="cuda")
        for a in range(0, 6, 2):
            dist.all_reduce(t[a:a + 1], op=dist.ReduceOp.MAX)
            dist.all_reduce(t[a + 1:a + 2], op=dist.ReduceOp.SUM)
        e2e_total, e2e_rays, sync_total, sync_rays, pipe_total, pipe_rays = (float(x) for x in t)
    e2e_value = e2e_rays / (e2e_total * 1e-3) / 1e6
    sync_value = sync_rays / (sync_total * 1e-3) / 1e6
    pipe_value = pipe_rays / (pipe_total * 1e-3) / 1e6

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return 0

    peak, peak_kind = peaks()
    n_tris = ter.n_tris
    med_build = statistics.median(t_build)
    med_render = statistics.median(t_render)
    rays_step = rays / args.steps
    shadow_step = shadow / args.steps
    render_bytes = rays_step * (B_RAY_CLOSEST + B_SHADE) + shadow_step * B_RAY_SHADOW
    render_gbs = render_bytes / (med_render * 1e-3) / 1e9
    build_bytes = n_tris * B_BUILD_PER_TRI
    build_gbs = build_bytes / (med_build * 1e-3) / 1e9
    pooled = ctx.variant_pooled(tuned.variant)
    vt, vm, _ = ctx.variants()[tuned.variant]
    kname = ("k_render_pool<%d, %d>" if pooled else "k_render<%d, %d>") % (vt, vm)
    roofline = {"kernel": kname + (" (pooled trace + shadow + shade + reflect)" if pooled
                                   else " (fused trace + shadow + shade + reflect)"),
                "bound": "hbm", "achieved": render_gbs, "peak": peak, "unit": "GB/s",
                "frac": render_gbs / peak,
                # dram__bytes_read.sum + dram__bytes_write.sum of one launch of
                # the installed kernel on this frame, when one was captured
                "traffic": RENDER_DRAM_BYTES.get(kname),
                "peak_kind": peak_kind,
                "algorithmic_bytes_per_launch": render_bytes,
                "note": "traversal is latency/L2-bound; algorithmic bytes = 88 B per traced "
                        "ray + 25 B per shadow ray"}
    # the emit's levels: 512 triangles per level-0 block, then 8 blocks per block
    emit_levels = emit_levels_of(n_tris)
    # k_bounds, k_morton_hist, 4 radix passes, the emit levels (the first
    # one also permutes), then the render (+ k_fb_copy when pooled)
    launches_per_frame = 6 + emit_levels + (2 if pooled else 1)
    build_roofline = {"kernels": "k_bounds + k_morton_hist + 4x k_onesweep + "
                                 "k_emit_level0_permute + %dx k_emit_level" % (emit_levels - 1),
                      "bound": "hbm",
                      "achieved": build_gbs,
                      "peak": peak, "unit": "GB/s", "frac": build_gbs / peak,
                      "bytes_per_tri": B_BUILD_PER_TRI, "peak_kind": peak_kind,
                      "ms": med_build, "lbvh_mtri_s": n_tris / (med_build * 1e-3) / 1e6}
    batched = None
    if world == 1 and not args.no_batched:
        try:
            batched = measure_batched(ctx, lib, torch)
        except Exception as e:
            batched = {"error": str(e)}
    stress = None
    if world == 1 and not args.no_stress:
        try:
            stress = measure_stress(ctx, lib, torch, cpu=not args.no_cpu_baseline)
        except Exception as e:
            stress = {"error": str(e)}
    refit_leg = None
    if world == 1 and not args.no_refit:
        try:
            refit_leg = measure_refit(ctx, torch)
        except Exception as e:
            refit_leg = {"error": str(e)}
    refraction_leg = None
    if world == 1 and not args.no_refraction:
        try:
            refraction_leg = measure_refraction(ctx, torch)
        except Exception as e:
            refraction_leg = {"error": str(e)}
    sah_leg = None
    if world == 1 and not args.no_sah:
        try:
            sah_leg = measure_sah(ctx, torch)
        except Exception as e:
            sah_leg = {"error": str(e)}
    instances_leg = None
    if world == 1 and not args.no_instances:
        try:
            instances_leg = measure_instances(ctx, torch)
        except Exception as e:
            instances_leg = {"error": str(e)}
    obj_leg = None
    if world == 1 and not args.no_obj:
        try:
            obj_leg = measure_obj(ctx, torch)
        except Exception as e:
            obj_leg = {"error": str(e)}
    served_leg = None
    if world == 1 and not args.no_served:
        try:
            served_leg = measure_served(ctx)
        except Exception as e:
            served_leg = {"error": str(e)}
    cpu, tv = None, None
    if world == 1 and not args.no_cpu_baseline:
        try:
            sc0 = scenes.Scene(frames[0][0], frames[0][1], ter.idx, ter.mats, ter.mat_map,
                               ter.lights)
            cpu, osc = cpu_baseline(sc0, wl["camera"], w, h, nb)
            cpu["c0_full"] = cpu_c0_full()
            tv = traversal_work(osc, wl["camera"], w, h)
        except Exception as e:   # the oracle must not break the GPU line
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                   "sample": "failed: %s" % e}
    if tv:
        tb = tv["bytes_per_ray"] * rays_step + tv["bytes_per_shadow_ray"] * shadow_step
        roofline["traversal"] = dict(tv, bytes_per_frame=tb,
                                     gbs=tb / (med_render * 1e-3) / 1e9,
                                     note="node and triangle records the traversal reads per frame "
                                          "(oracle-counted on the sample's primary rays and their "
                                          "shadow rays, applied to every traced ray), served "
                                          "mostly from L1 and L2")
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": wl["name"], "triangles": n_tris, "width": w, "height": h,
                      "max_bounces": nb, "lights": 2, "lbvh_depth": 30, "lbvh_min_leaf": 1,
                      "rebuild_per_frame": True, "l2": "flushed (256 MiB write) between steps",
                      "e2e_l2": "two scene copies alternate: a frame's buffers were last touched "
                                "two frames before, the other copy's frame (about 250 MB, twice "
                                "the L2) between",
                      "parallelism": "replicas" if world > 1 else "single GPU"},
           "mrays_all_incl_shadow": (rays_all + shadow * world) / (total_ms * 1e-3) / 1e6,
           "lbvh_mtri_s": n_tris / (med_build * 1e-3) / 1e6,
           "build_ms": med_build, "render_ms": med_render,
           "rays_per_frame": rays_step, "shadow_rays_per_frame": shadow_step,
           "roofline": roofline, "build_roofline": build_roofline,
           "cpu_baseline": cpu,
           "batched": batched,
           "served": served_leg,
           "stress": stress,
           "refit": refit_leg,
           "obj": obj_leg,
           "refraction": refraction_leg,
           "instances": instances_leg,
           "sah": sah_leg,
           "e2e": {"value": e2e_value, "unit": UNIT,
                   "h2d_bytes_per_step": 2 * 16 * V,
                   "d2h_bytes_per_step": 4 * w * h + 32 + 4,
                   "ms_per_step": e2e_total / args.steps,
                   "mode": "two frames in flight: rt_render_host_async / rt_render_host_wait on "
                           "two streams with one scene copy each (a frame's buffers last touched "
                           "two frames before; each frame's upload and read-back timed)",
                   "sync_value": sync_value,
                   "sync_ms_per_step": statistics.median(sync_ms),
                   "sync_mode": "rt_render_host, one frame at a time, L2 flushed between frames"},
           "two_in_flight": {"value": pipe_value, "unit": UNIT,
                             "ms_per_step": pipe_total / args.steps,
                             "mode": "device-resident frames (vertex update from HBM, build, "
                                     "render), two in flight on two streams with one scene copy "
                                     "each, no host copies: the device-side counterpart of e2e"},
           "gpu_launches": launches_per_frame * args.steps,
           "render_config": {"variant": tuned.variant, "threads": ctx.variants()[tuned.variant][0],
                             "min_blocks_per_sm": ctx.variants()[tuned.variant][1],
                             "blocks_per_sm": tuned.blocks_per_sm, "chunk": tuned.chunk,
                             "stack_depth": 32, "autotune_best_ms": tuned_ms},
           "clocks": clocks, "device_status": dev_status,
           "wall_s_timed_loop": wall}
    print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=120)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--no-stress", action="store_true")
    ap.add_argument("--no-refit", action="store_true")
    ap.add_argument("--no-obj", action="store_true")
    ap.add_argument("--no-refraction", action="store_true")
    ap.add_argument("--no-instances", action="store_true")
    ap.add_argument("--no-sah", action="store_true")
    ap.add_argument("--render-variant", type=int, default=None,
                    help="render kernel variant instead of the autotuner's pick")
    ap.add_argument("--render-blocks", type=int, default=0, help="resident blocks per SM (0: all)")
    ap.add_argument("--render-chunk", type=int, default=128, help="pixels per work-counter grab")
    args = ap.parse_args()
    if args.warmup < 3:
        log("warmup raised to 3")
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
