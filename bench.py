"""Benchmark of the trace-and-accumulate path on GB300.

One step is one frame of the CSG-heavy scene, the largest configuration that runs on one GPU:
256 CSG objects (circle And / Or / AndNot rect, seed 3), 8 lights sharing 2^22 primary rays,
32 bounces, a string-mod overlay of 4096 chords (i -> 7 i mod 4096), 4096 x 4096 int64
fixed-point accumulation, resolve to RGBA16F, exact FP64 precision.  The frame's 1.5 G
segments exceed one accumulation pass, so the library accumulates between generations.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload csg|mid] [--precision exact|fast] [--no-extras] [--no-cpu-baseline]

``value``: traced segments per second over the whole job (all ranks), from CUDA events on
the library's stream around the captured frame graph, with the L2 flushed (a 512 MB write)
before every step.  ``e2e``: the same metric through the public C ABI with host buffers
(scene tables uploaded from the host and the RGBA16F image read back into pinned host
memory every step).  ``roofline``: the frame's longest kernel stage against the ceiling of
the resource it uses, measured in the same process (liblg_peaks.so).  ``cpu_baseline``: the
CPU restatement of the reference tracer (the reference is Rust and cannot be built) on all
host cores over a sample of the primaries, and the GPU's image of the same sample compared
with it.  The extra keys (``mid_scene``, ``image_errors``, ``fast_precision``, ``batch``,
``serve``, ``serve_load``) measure the other configurations on the same GPU.
``--impl reference`` times that CPU restatement alone, one sample per step.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "traced segments/s + accumulated px/s on 1 GB300; p50/p99 scene latency vs plain"
CULL = {"auto": 0, "off": 1, "on": 2}  # lg_culling
PRECISION = {"exact": 0, "fast": 1}  # lg_precision

WORKLOADS = {
    "csg": "csg_scene: 256 CSG objects (circle op rect, ops And/Or/AndNot, seed 3), 8 lights, 2^22 rays, "
           "32 bounces, 4096x4096, int64 Q31.32 accumulation, string-mod overlay m=4096 k=7, RGBA16F resolve",
    "mid": "mid_scene: 64 objects (rect/circle/mirror/curved mirror, seed 2), 8 lights x 2^18 rays, "
           "16 bounces, 1920x1080, int64 Q31.32 accumulation, RGBA16F resolve",
}
BATCH_WORKLOAD = ("batch: 512 seeded scenes (seed 4): objects log-uniform [4, 1024], rays log-uniform [2^12, 2^20], "
                  "bounces U{4..32}, canvases {256, 512, 1024, 2048}^2, int64 accumulation")
# CPU samples (primary stride per light): the baseline leg ~10-20 s, a reference-arm step ~5 s
CPU_STRIDE = {"csg": 1024, "mid": 16}
REF_STRIDE = {"csg": 2048, "mid": 32}

# Instructions per unit of work of the trace kernels and the tile raster in the exact mode,
# counted with ncu (smsp__sass_thread_inst_executed_op_{fadd,fmul,ffma,dadd,dmul,dfma}
# _pred_on.sum and smsp__sass_inst_executed_op_shared_atom.sum over the frame of
# ``bench.py --count-case``: csg 2^18 rays at 1024^2, mid 2^14 rays per light).
#   scan:   FP32 thread instructions per ray visit
#   solve:  FP64 thread instructions per object solved (lg_trace_stats.fp64_solves)
#   bounce: FP64 thread instructions per ray visit
#   raster: shared-memory atomic warp instructions per accumulated pixel
INST_PER_UNIT = {
    "csg": {"scan": 631.1, "solve": 80.2, "bounce": 71.7, "raster": 0.2805},
    "mid": {"scan": 952.3, "solve": 67.4, "bounce": 55.9, "raster": 0.3005},
}
# Warp instructions issued (smsp__inst_executed.sum) per unit of the same frames: the trace
# stages against the SM's issue ceiling (4 schedulers x 1 warp instruction per cycle per SM).
WARP_INST_PER_UNIT = {
    "csg": {"scan": 323.2, "solve": 52.0, "bounce": 75.2},
    "mid": {"scan": 270.3, "solve": 66.2, "bounce": 49.8},
}


def measured_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class PeaksLib(C.Structure):
    _fields_ = [("smem_atomics_per_s", C.c_double), ("fp32_fma_per_s", C.c_double), ("fp64_op_per_s", C.c_double),
                ("n_sm", C.c_int32), ("status", C.c_int32)]


def live_peaks(device: int) -> dict:
    """Throughput ceilings measured on this GPU now (light_garden_gb300/csrc/lg_peaks.cu)."""
    lib = C.CDLL(str(ROOT / "light_garden_gb300" / "_lib" / "liblg_peaks.so"))
    lib.lgp_measure.argtypes = [C.c_int, C.POINTER(PeaksLib)]
    p = PeaksLib()
    if lib.lgp_measure(device, C.byref(p)) != 0:
        raise RuntimeError(f"lgp_measure failed: {p.status}")
    return {"smem_atomics_per_s": p.smem_atomics_per_s, "fp32_fma_per_s": p.fp32_fma_per_s,
            "fp64_op_per_s": p.fp64_op_per_s}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
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
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(ws, v: float, device) -> float:
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate(ws: int, units: int, ms: float, device) -> tuple:
    """Whole-job throughput of ``ws`` replicas that each processed ``units`` in ``ms``: the
    slowest rank's time bounds the job (max over ranks)."""
    ms_max = allmax(ws, ms, device)
    return ws * units / (ms_max * 1e-3), ms_max


def packed_workload(name: str, precision: str, ray_scale: float = 1.0):
    from light_garden_gb300 import abi, workloads as W
    if name == "plain":  # 1 point light (4096 rays), circle + mirror, 8 bounces, 512x512
        pk = W.plain_small(accum=abi.LG_ACCUM_FIXED64).packed()
    elif name == "csg":
        pk = W.csg_scene(total_rays=max(8, int(round((1 << 22) * ray_scale)))).packed()
    else:
        pk = W.mid_scene(rays_per_light=max(1, int(round((1 << 18) * ray_scale)))).packed()
    pk.params.precision = PRECISION[precision]
    return pk


# ------------------------------------------------------------------------ CPU restatement
def cpu_sample(name: str, stride: int):
    """Oracle (CPU restatement of tracer.rs) on every stride-th primary: trace + raster."""
    from oracle import oracle as O
    pk = packed_workload(name, "exact")
    t0 = time.perf_counter()
    segs, paths, _, st = O.trace(pk, ray_stride=stride, threads=0)
    chords = O.string_mod_chords(pk.params)  # the sample starts at primary 0: the overlay is drawn
    t1 = time.perf_counter()
    acc, px = O.raster(segs, pk.params, threads=0, chords=chords)
    t2 = time.perf_counter()
    return pk, segs, paths, acc, px, t1 - t0, t2 - t1, int(st.primary_rays)


def sample_parity(pk, stride, o_segs, o_paths, o_acc, local):
    """The GPU's trace and image of the same sampled frame against the CPU restatement's:
    exact mode bit for bit; the FP32 accumulation and the double-float trace as errors."""
    import numpy as np
    from light_garden_gb300 import abi
    from light_garden_gb300.runtime import Context
    from oracle import oracle as O
    sys.path.insert(0, str(ROOT / "tests"))
    from parity import exact

    def rel(a, b):
        a = a.astype(np.float64).ravel()
        b = b.astype(np.float64).ravel()
        n1, n2 = np.abs(b).sum(), np.sqrt((b * b).sum())
        return float(np.abs(a - b).sum() / n1), float(np.sqrt(((a - b) ** 2).sum()) / n2)

    out = {"sample": f"every {stride}th primary of each light"}
    orig = abi.lg_params.from_buffer_copy(pk.params)
    with Context(device=local) as ctx:
        pk.params.record_paths = 1
        pk.params.ray_stride, pk.params.ray_offset = stride, 0
        pk.params.precision = abi.LG_PRECISION_EXACT
        ctx.upload(pk)
        ctx.trace()
        gs, gp = ctx.segments(paths=True)
        rep = exact(gs, gp, o_segs, o_paths)
        o_ch = O.string_mod_chords(pk.params)
        ctx.accumulate()
        acc = ctx.accum()
        out["exact"] = {"segments": rep.segments, "bit_exact_segments": rep.ok(),
                        "string_mod_lines": len(o_ch), "bit_exact_lines": ctx.chords().tobytes() == o_ch.tobytes(),
                        "image_bit_exact": bool(np.array_equal(acc, o_acc)),
                        "near_flag_differs": rep.near_flag_differs}
        del acc
        scale = 2.0 ** -32
        # the FP64 image of the oracle's segments and lines: the reference for the accumulation error
        f64, _ = O.raster_f64(o_segs, pk.params, chords=o_ch)
        l1, l2 = rel(o_acc.astype(np.float64) * scale, f64)
        out["fixed64_vs_fp64_raster"] = {"rel_l1": l1, "rel_l2": l2}
        pk.params.accum = abi.LG_ACCUM_F32
        pk.params.record_paths = 0
        ctx.upload(pk)
        ctx.trace()  # the same exact trace, accumulated in FP32
        ctx.accumulate()
        l1, l2 = rel(ctx.accum(), f64)
        out["fp32_accum_vs_fp64_raster"] = {"rel_l1": l1, "rel_l2": l2}
        # the double-float trace of the same sample, accumulated in fixed point
        pk.params.accum = abi.LG_ACCUM_FIXED64
        pk.params.precision = abi.LG_PRECISION_FAST
        pk.params.record_paths = 0
        ctx.upload(pk)
        ctx.trace()
        ctx.accumulate()
        l1, l2 = rel(ctx.accum().astype(np.float64) * scale, f64)
        out["fast_precision_image_vs_fp64"] = {"rel_l1": l1, "rel_l2": l2}
    pk.params = orig
    return out


def run_reference(args, ws, rank):
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    stride = args.cpu_stride or REF_STRIDE[args.workload]
    times, nseg, npx, nprim = [], 0, 0, 0
    for _ in range(args.warmup):
        cpu_sample(args.workload, stride)
    for _ in range(args.steps):
        _, segs, _, _, px, tt, tr, prim = cpu_sample(args.workload, stride)
        times.append(tt + tr)
        nseg, npx, nprim = len(segs), px, prim
    step_s = statistics.mean(times)
    value = nseg / step_s
    sample = (f"every {stride}th primary ray of each light ({nprim} primaries) traced and rasterised per step: "
              f"{nseg} segments, {npx} pixel updates")
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "segments/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload], "sample": sample},
        "px_per_s": npx / step_s,
        "cpu_baseline": {"value": value, "unit": "segments/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "segments/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference is Rust (no toolchain here) and its geometry crate is not vendored; this is the C "
                "restatement of tracer.rs (oracle/lg_oracle.c) timed on all host cores",
    }
    print(json.dumps(out), flush=True)


# ------------------------------------------------------------------------ frames on the GPU
def frame_bench(pk, local, steps, warmup, args, clocks=True):
    """Frames of one packed scene through lg_render: device time per step (CUDA events in
    the frame graph), L2 flushed before each step."""
    import torch
    from light_garden_gb300.runtime import Context
    dev = torch.device("cuda", local)
    Wd, Hd = pk.params.width, pk.params.height
    ctx = Context(device=local, raster_variant=args.raster_variant, culling=CULL[args.culling],
                  grid_density=args.grid_density)
    ctx.upload(pk)
    out = torch.empty((Hd, Wd * 4), dtype=torch.int16, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    for _ in range(max(1, warmup)):
        st = ctx.render_into(out.data_ptr(), Wd * 8, True)
    torch.cuda.synchronize()
    keys = ("trace_ms", "bin_ms", "raster_ms", "resolve_ms", "total_ms", "scan_ms", "solve_ms", "bounce_ms")
    tot = {k: 0.0 for k in keys}
    sampler = ClockSampler(local) if clocks else None
    if sampler:
        sampler.__enter__()
    try:
        for _ in range(steps):
            flush.zero_()  # write 512 MB > L2 before every step (not timed)
            torch.cuda.synchronize()
            st = ctx.render_into(out.data_ptr(), Wd * 8, True)
            for k in keys:
                tot[k] += st[k]
    finally:
        if sampler:
            sampler.__exit__(None, None, None)
    torch.cuda.synchronize()
    avg = {k: v / steps for k, v in tot.items()}
    return ctx, st, avg, (sampler.summary() if sampler else None)


def issue_ceiling(local, clk):
    """Warp instructions per second the GPU can issue: SMs x 4 schedulers x the median SM clock
    sampled during the timed region (or the maximum clock when unsampled)."""
    import torch
    mhz = (clk or {}).get("sm_mhz") or (clk or {}).get("sm_max_mhz")
    if not mhz:
        return None
    n_sm = torch.cuda.get_device_properties(local).multi_processor_count
    return n_sm * 4 * mhz * 1e6, f"{n_sm} SMs x 4 schedulers x {mhz:g} MHz (sampled)"


def rooflines(name, st, avg, peaks, hbm, issue=None):
    """Each kernel stage against the ceiling of the resource it uses (exact mode); with
    ``issue`` = (warp instructions per second the SMs can issue, how it was found), the trace
    stages also carry their share of the issue slots."""
    ipu = INST_PER_UNIT[name]
    vis, solves, px = st["ray_visits"], st["fp64_solves"], st["pixels"]
    r = {}

    def entry(kernel, bound, inst, ms, peak, unit_name, note):
        achieved = inst / (ms * 1e-3) / 1e9 if ms > 0 else 0.0
        return {"kernel": kernel, "bound": bound, "achieved": achieved, "peak": peak / 1e9, "unit": unit_name,
                "frac": achieved / (peak / 1e9) if peak else None, "traffic": None, "ms": ms, "peak_source":
                "measured live (liblg_peaks.so)", "note": note}

    r["scan"] = entry("k_scan (FP32 nearest-hit search)", "fp32_pipe", ipu["scan"] * vis, avg["scan_ms"],
                      peaks["fp32_fma_per_s"], "G FP32 inst/s",
                      f"{ipu['scan']} FP32 instructions per ray visit (ncu count) x {vis} visits")
    r["solve"] = entry("k_solve_x (exact FP64 nearest hit)", "fp64_pipe", ipu["solve"] * solves, avg["solve_ms"],
                       peaks["fp64_op_per_s"], "G FP64 inst/s",
                       f"{ipu['solve']} FP64 instructions per object solve (ncu count) x {solves} solves")
    r["bounce"] = entry("k_bounce_x (exact FP64 bounce and canvas exit)", "fp64_pipe", ipu["bounce"] * vis,
                        avg["bounce_ms"], peaks["fp64_op_per_s"], "G FP64 inst/s",
                        f"{ipu['bounce']} FP64 instructions per ray visit (ncu count) x {vis} visits")
    if issue and issue[0]:
        wpu = WARP_INST_PER_UNIT[name]
        for stage, units, uname in (("scan", vis, "ray visit"), ("solve", solves, "object solve"),
                                    ("bounce", vis, "ray visit")):
            ms = avg[stage + "_ms"]
            achieved = wpu[stage] * units / (ms * 1e-3) / 1e9 if ms > 0 else 0.0
            r[stage]["issue"] = {"achieved": achieved, "peak": issue[0] / 1e9, "unit": "G warp inst/s",
                                 "frac": achieved / (issue[0] / 1e9),
                                 "note": f"{wpu[stage]} warp instructions per {uname} (ncu count); peak {issue[1]}"}
    ra = entry("k_raster (tile accumulation in shared memory)", "smem_atomics", ipu["raster"] * 32 * px,
               avg["raster_ms"], peaks["smem_atomics_per_s"], "G shared atomics/s",
               f"{ipu['raster'] * 32:.2f} shared-memory atomic lane operations per pixel (ncu count) x {px} pixels")
    ra["hbm_equivalent"] = {"achieved_gbs": 64.0 * px / (avg["raster_ms"] * 1e-3) / 1e9, "peak_gbs": hbm[0],
                            "note": "64 B per pixel (an int64 RGBA read-modify-write) if the update went through "
                                    "HBM; the update runs in shared memory, so this can exceed 1 of the copy "
                                    "bandwidth (" + hbm[1] + ")"}
    r["raster"] = ra
    return r


def batch_bench(local, args, ray_scale=None):
    """512 mixed scenes: one multi-scene trace (lg_batch_render) against the plain path
    (lg_render of each scene in turn), at a fraction of the rays."""
    import torch
    ray_scale = args.batch_scale if ray_scale is None else ray_scale
    from light_garden_gb300 import workloads as W
    from light_garden_gb300.runtime import Context
    dev = torch.device("cuda", local)
    scenes = [W.scale_rays(w, ray_scale).packed() for w in W.batch_scenes(count=512)]
    for pk in scenes:
        pk.params.precision = PRECISION[args.precision]
    n = len(scenes)
    ctx = Context(device=local, culling=CULL[args.culling])
    ctx.batch_upload(scenes)
    out = torch.empty(ctx.batch_pixels() * 4, dtype=torch.int16, device=dev)
    ctx.batch_render_into(out.data_ptr(), out.numel() * 2, True)
    ms, stages = [], None
    for _ in range(2):
        st = ctx.batch_render_into(out.data_ptr(), out.numel() * 2, True)
        ms.append(st["total_ms"])
        if st["total_ms"] == min(ms):
            stages = {k: st[k] for k in ("trace_ms", "accumulate_ms", "resolve_ms", "segments", "pixels", "ray_visits",
                                         "primary_rays")}
    ctx.close()
    plain = Context(device=local, culling=CULL[args.culling])
    big = torch.empty(max(pk.params.width * pk.params.height for pk in scenes) * 4, dtype=torch.int16, device=dev)
    for pk in scenes[:4]:
        plain.upload(pk)
        plain.render_into(big.data_ptr(), pk.params.width * 8, True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for pk in scenes:
        plain.upload(pk)
        plain.render_into(big.data_ptr(), pk.params.width * 8, True)
    plain_s = time.perf_counter() - t0
    # the ceiling of batching: every 8th scene rendered alone at its reduced ray count and at
    # full rays; batching can at best run a scene at the per-ray efficiency the same scene
    # reaches with 1/ray_scale times the rays, where it fills far more of the GPU
    full = [w.packed() for w in W.batch_scenes(count=512)[::8]]
    t_small = t_full = 0.0
    for pk_s, pk_f in zip(scenes[::8], full):
        pk_f.params.precision = PRECISION[args.precision]
        for pk, acc in ((pk_s, "s"), (pk_f, "f")):  # same canvases: `big` holds either
            plain.upload(pk)
            for _ in range(2):  # graph capture, then the scan autotune of the scene's second render
                plain.render_into(big.data_ptr(), pk.params.width * 8, True)
            torch.cuda.synchronize()
            a = time.perf_counter()
            plain.render_into(big.data_ptr(), pk.params.width * 8, True)
            dt = time.perf_counter() - a
            if acc == "s":
                t_small += dt
            else:
                t_full += dt * ray_scale
    plain.close()
    b = n / (min(ms) * 1e-3)
    ceiling = t_small / t_full if t_full > 0 else None
    return {"workload": BATCH_WORKLOAD + f", rays x {ray_scale:g}", "scenes": n, "batched_scenes_per_s": b,
            "batch_ms": min(ms), "plain_scenes_per_s": n / plain_s, "batched_vs_plain": b / (n / plain_s),
            "ceiling_vs_plain": ceiling, "batch_stages": stages,
            "note": "batched: device time of the batch graph; plain: host wall time of upload + lg_render per scene; "
                    "ceiling: 64 scenes (every 8th) alone, time at these rays over time at full rays x ray scale"}


def batch_graph(local, args, ray_scale=None):
    """The 512-scene batch alone: upload, three lg_batch_render calls, the last one's stages."""
    import torch
    ray_scale = args.batch_scale if ray_scale is None else ray_scale
    from light_garden_gb300 import workloads as W
    from light_garden_gb300.runtime import Context
    scenes = [W.scale_rays(w, ray_scale).packed() for w in W.batch_scenes(count=512)]
    for pk in scenes:
        pk.params.precision = PRECISION[args.precision]
    ctx = Context(device=local, culling=CULL[args.culling])
    ctx.batch_upload(scenes)
    out = torch.empty(ctx.batch_pixels() * 4, dtype=torch.int16, device=torch.device("cuda", local))
    for _ in range(3):
        st = ctx.batch_render_into(out.data_ptr(), out.numel() * 2, True)
    ctx.close()
    return {k: st[k] for k in ("total_ms", "trace_ms", "accumulate_ms", "resolve_ms", "segments", "pixels", "ray_visits",
                               "primary_rays", "fp64_solves", "bound_tests", "object_tests")}


def serve_bench(local, args, rate=100.0, count=256, ray_scale=1.0 / 16):
    """Poisson arrivals: scenes/s and p50/p99 latency of the continuous-batching server against
    the plain path serving the same arrivals in order.  At 100 requests/s the load is below
    either path's capacity (the latencies are service times); at 200 requests/s, the bottom of
    the serving configuration's range, it is above it and the latencies include queueing."""
    import numpy as np
    import torch
    from light_garden_gb300 import workloads as W
    from light_garden_gb300.runtime import Context
    dev = torch.device("cuda", local)
    scenes = [W.scale_rays(w, ray_scale).packed() for w in W.batch_scenes(seed=6, count=count)]
    for pk in scenes:
        pk.params.precision = PRECISION[args.precision]
    rng = np.random.default_rng(7)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, count))
    ctx = Context(device=local, culling=CULL[args.culling])
    ctx.serve_begin(hbm_budget_bytes=int(120 * (1 << 30)), max_slots=4096)
    for sc in scenes[:2]:  # warm-up
        ctx.serve_submit(sc)
    while ctx.serve_step()["in_flight"] or any(ctx.serve_poll(r) is None for r in list(ctx.serve_shapes)):
        pass
    done_at, arrive_of = {}, {}
    inflight = set()
    t0 = time.perf_counter()
    nxt = 0
    while len(done_at) < count:
        now = time.perf_counter() - t0
        while nxt < count and arrivals[nxt] <= now:
            rid = ctx.serve_submit(scenes[nxt])
            arrive_of[rid] = arrivals[nxt]
            inflight.add(rid)
            nxt += 1
        if not inflight:
            time.sleep(max(0.0, arrivals[nxt] - now))
            continue
        st = ctx.serve_step()
        if st["finished"] or st["in_flight"] == 0:
            t = time.perf_counter() - t0
            for rid in list(inflight):
                if ctx.serve_poll(rid) is not None:
                    done_at[rid] = t
                    inflight.discard(rid)
    makespan = time.perf_counter() - t0
    lat = np.array([done_at[r] - arrive_of[r] for r in done_at]) * 1e3
    ctx.serve_end()
    ctx.close()
    plain = Context(device=local, culling=CULL[args.culling])
    big = torch.empty(max(pk.params.width * pk.params.height for pk in scenes) * 4, dtype=torch.int16, device=dev)
    for pk in scenes[:2]:
        plain.upload(pk)
        plain.render_into(big.data_ptr(), pk.params.width * 8, True)
    service = []
    for pk in scenes:
        a = time.perf_counter()
        plain.upload(pk)
        plain.render_into(big.data_ptr(), pk.params.width * 8, True)
        service.append(time.perf_counter() - a)
    plain.close()
    end, plat = 0.0, []
    for a, s in zip(arrivals, service):
        end = max(end, a) + s
        plat.append((end - a) * 1e3)
    plat = np.array(plat)
    return {"workload": BATCH_WORKLOAD.replace("seed 4", "seed 6") + f", rays x {ray_scale:g}",
            "requests": count, "arrivals": f"Poisson, {rate:g} requests/s", "hbm_budget_gb": 120,
            "scenes_per_s": count / makespan, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "makespan_s": makespan,
            "plain": {"scenes_per_s": count / end, "p50_ms": float(np.percentile(plat, 50)),
                      "p99_ms": float(np.percentile(plat, 99)), "mean_service_ms": float(np.mean(service) * 1e3)}}


def count_case(args):
    """One frame of a small case of the workload (csg: 2^18 rays at 1024^2; mid: 2^14 rays per
    light), no autotuning, printing the frame's units of work.  Run under ncu with instruction
    counters, it gives the instructions per unit of INST_PER_UNIT."""
    from light_garden_gb300 import workloads as W
    from light_garden_gb300.runtime import Context
    if args.workload == "csg":
        pk = W.csg_scene(total_rays=1 << 18, width=1024, height=1024).packed()
    else:
        pk = W.mid_scene(rays_per_light=1 << 14).packed()
    pk.params.precision = PRECISION[args.precision]
    with Context(raster_variant=1, culling=CULL[args.culling]) as ctx:
        ctx.upload(pk)
        _, st = ctx.render()
    keys = ("ray_visits", "fp64_solves", "pixels", "bound_tests", "object_tests", "segments", "scan_ms", "solve_ms",
            "bounce_ms", "raster_ms", "trace_ms", "total_ms")
    print(json.dumps({"count_case": args.workload, "precision": args.precision, **{k: st[k] for k in keys}}),
          flush=True)


def run_ours(args, ws, rank, local):
    import torch

    from light_garden_gb300 import abi

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    name = args.workload
    pk = packed_workload(name, args.precision)
    Wd, Hd = pk.params.width, pk.params.height
    peaks = live_peaks(local)
    hbm = measured_hbm()
    barrier(ws)
    ctx, st, avg, clk = frame_bench(pk, local, args.steps, max(3, args.warmup), args)
    barrier(ws)
    value, ms_max = aggregate(ws, st["segments"], avg["total_ms"], dev)
    px_per_s = ws * st["pixels"] / (ms_max * 1e-3)

    # end to end through the C ABI: scene tables from the host, image back to pinned host memory
    h2d = C.sizeof(abi.lg_geo) * pk.n_geo + C.sizeof(abi.lg_object) * pk.n_objects + \
        C.sizeof(abi.lg_light) * pk.n_lights + C.sizeof(abi.lg_params)
    d2h = Hd * Wd * 8
    host = torch.empty((Hd, Wd * 4), dtype=torch.int16, pin_memory=True)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    ctx.upload(pk)
    ctx.render_into(host.data_ptr(), Wd * 8, False)
    barrier(ws)
    e2e_steps = max(1, min(args.steps, 3))
    e2e_times = []
    for _ in range(e2e_steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.upload(pk)
        est = ctx.render_into(host.data_ptr(), Wd * 8, False)
        e2e_times.append(time.perf_counter() - t0)
    e2e_value, e2e_ms = aggregate(ws, est["segments"], statistics.mean(e2e_times) * 1e3, dev)
    ctx.close()
    del flush

    issue = issue_ceiling(local, clk)
    roof = rooflines(name, st, avg, peaks, hbm, issue) if args.precision == "exact" else {}
    dominant = max(roof.values(), key=lambda e: e["ms"]) if roof else None

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        stride = args.cpu_stride or CPU_STRIDE[name]
        spk, segs, paths, o_acc, px, tt, tr, prim = cpu_sample(name, stride)
        cpu = {"value": len(segs) / (tt + tr), "unit": "segments/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"every {stride}th primary of each light ({prim} primaries): {len(segs)} segments traced in "
                         f"{tt:.2f} s and rasterised ({px} px) in {tr:.2f} s",
               "trace_segments_per_s": len(segs) / tt, "raster_px_per_s": px / tr}
        try:
            cpu["parity"] = sample_parity(spk, stride, segs, paths, o_acc, local)
        except Exception as e:  # the headline line is printed either way
            cpu["parity"] = {"error": repr(e)}

    extras = {}
    if rank == 0 and ws == 1 and not args.no_extras:
        def extra(key, fn):
            try:
                extras[key] = fn()
            except Exception as e:
                extras[key] = {"error": repr(e)}

        def mid():
            mpk = packed_workload("mid", args.precision)
            c2, s2, a2, _ = frame_bench(mpk, local, 5, 3, args, clocks=False)
            c2.close()
            d = {"workload": WORKLOADS["mid"], "value": s2["segments"] / (a2["total_ms"] * 1e-3), "unit": "segments/s",
                 "ms_per_step": a2["total_ms"], "px_per_s": s2["pixels"] / (a2["total_ms"] * 1e-3),
                 "segments_per_step": s2["segments"], "pixels_per_step": s2["pixels"], "stage_ms": a2}
            if args.precision == "exact":
                d["rooflines"] = rooflines("mid", s2, a2, peaks, hbm, issue)
            return d

        def fast():
            fpk = packed_workload(name, "fast")
            c3, s3, a3, _ = frame_bench(fpk, local, 2, 1, args, clocks=False)
            c3.close()
            return {"workload": WORKLOADS[name] + ", double-float precision", "value": s3["segments"] / (a3["total_ms"] * 1e-3),
                    "unit": "segments/s", "ms_per_step": a3["total_ms"], "stage_ms": a3,
                    "flagged_per_step": {"decision_band": s3["near_degenerate"], "ill_conditioned": s3["ill_conditioned"],
                                         "segments": s3["segments"]}}

        def image_errors():
            # the other configurations' images against the FP64 raster of the oracle's own trace
            out = {}
            for wname, stride in (("plain", 1), ("mid", 64)):
                spk, segs, paths, o_acc, _, _, _, prim = cpu_sample(wname, stride)
                out["plain_small" if wname == "plain" else "mid_scene"] = {
                    "primaries": prim, **sample_parity(spk, stride, segs, paths, o_acc, local)}
            return out

        if name != "mid":
            extra("mid_scene", mid)
        extra("image_errors", image_errors)
        extra("fast_precision", fast)
        extra("batch", lambda: batch_bench(local, args))
        extra("serve", lambda: serve_bench(local, args))
        extra("serve_load", lambda: serve_bench(local, args, rate=200.0))

    # light setup, 3 trace kernels per generation, overlay, accumulation clear, resolve, string-mod lines
    G = pk.params.max_bounce
    launches = 1 + 3 * G + 1 + 1 + 1 + (1 if pk.params.string_mod.modulo else 0)
    if st["segments"] > (1 << 28):  # the frame streams: per generation decide, clear, count, scan, units, scatter, raster, rotate
        launches += 8 * G
    else:  # one accumulation: count, tile scan, units, scatter, raster
        launches += 5
    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": "segments/s", "n_gpus": ws, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 trace (exact), int64 accumulate" if args.precision == "exact"
            else "double-float trace, int64 accumulate", "data": "synthetic",
            "config": {"workload": WORKLOADS[name], "precision": args.precision,
                       "l2": "flushed before every step (512 MB write); working set > L2",
                       "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
            "px_per_s": px_per_s,
            "segments_per_step": st["segments"], "pixels_per_step": st["pixels"], "tile_refs_per_step": st["tile_refs"],
            "ray_visits_per_step": st["ray_visits"], "fp64_solves_per_step": st["fp64_solves"],
            "stage_ms": avg,
            "roofline": dominant,
            "rooflines": roof,
            "peaks": {"live": peaks, "hbm_gbs": hbm[0], "hbm_source": hbm[1]},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "segments/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": e2e_ms, "steps": e2e_steps},
            "gpu_launches": launches * args.steps,
            "clocks": clk,
        }
        out.update(extras)
        print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="csg", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="exact", choices=sorted(PRECISION),
                    help="exact: FP64 bit for bit with the FP64 formulas; fast: double-float refinement")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-stride", type=int, default=0,
                    help="primary stride of the CPU samples (0: the workload's default)")
    ap.add_argument("--no-extras", action="store_true", help="only the headline frame")
    ap.add_argument("--raster-variant", type=int, default=0, choices=[0, 1, 2],
                    help="0: autotuned; 1: shared-memory tile atomics; 2: warp-private tiles")
    ap.add_argument("--culling", default="auto", choices=sorted(CULL),
                    help="nearest-hit culling grid: auto (scenes of 96+ objects), off, on")
    ap.add_argument("--grid-density", type=float, default=0.0, help="culling grid cells per object (0: 2)")
    ap.add_argument("--count-case", action="store_true",
                    help="render one small frame of the workload and print its units of work (for ncu counts)")
    ap.add_argument("--batch-scale", type=float, default=1.0 / 16,
                    help="ray-count scale of the batch legs' scenes (default 1/16)")
    ap.add_argument("--only", choices=["batch", "serve", "batch-graph"], default=None,
                    help="run only that extra leg and print its JSON (for profiling); batch-graph: the 512-scene "
                         "batch at 1/16 of the rays rendered three times, nothing else")
    args = ap.parse_args()
    if args.count_case:
        count_case(args)
        return
    if args.only:
        import torch
        torch.cuda.set_device(0)
        fn = {"batch": batch_bench, "serve": serve_bench, "batch-graph": batch_graph}[args.only]
        print(json.dumps({args.only: fn(0, args)}), flush=True)
        return
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
