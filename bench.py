"""Benchmark: ms/frame of the deferred PBR + PCSS + SSAO frame at 1280x800.

Workload (the reference's headline configuration, synthetic and seeded): 20
icospheres (subdivision 5, 20,480 faces each) + ground plane = 409,602
triangles, per-mesh 1024^2 albedo / normal / roughness / metalness textures,
one point light, 2048^2 shadow map with PCSS (16 blocker taps, 25 PCF taps),
SSAO with 64 samples (radius 0.5) and the reference's in-place two-pass blur,
deferred Blinn-Phong / Cook-Torrance lighting, 1280x800, no SSAA.

One step = one fr_render_frame (shadow pass, geometry pass, SSAO + blur,
lighting) with the scene resident in HBM, replayed as the context's frame CUDA
graph; L2 is flushed (a 256 MiB write) before every timed step and each step
is timed with CUDA events on the context's stream (the frame's first and last
events only, fr_config.pass_timings = 0; the per-pass breakdowns come from the
same frames with an event at every pass boundary). `value` is the plain-SSAO
frame (the reference's method); `learned_ao` times the same frame with the
learned AO and reports its AO error against 256-sample SSAO on held-out views.
`e2e` runs frames through the public API with a camera that moves every step:
each step's frame matrices and eye come from host memory and the 8-bit frame is
read back to host memory inside the timed region (the frame graph is replayed
with the new camera's frame constants written into its kernel nodes;
`e2e_static_camera` repeats the scene's camera). `parity`
compares the GPU frame of the workload with the oracle's frame of the same
scene (the oracle run is also the CPU baseline).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

With --impl reference the reference's CPU path is timed instead: the CPU
restatement under oracle/ (the reference's own binary is x86-only and is not
built on aarch64 hosts) on all host cores, one bounded frame per step.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms/frame @1280x800 deferred PBR+PCSS+SSAO: plain vs learned AO (RMSE<=0.02)"
UNIT = "ms/frame"
WORKLOAD = ("deferred PBR + PCSS(16 blocker / 25 PCF) + SSAO(64 samples, r=0.5, in-place 2-pass blur), "
            "1280x800, 20 icospheres subdiv 5 + ground plane = 409,602 triangles, 1024^2 textures, "
            "2048^2 shadow map")
SCENE_KW = dict(seed=0, n_spheres=20, subdiv=5, tex=1024, width=1280, height=800, ssaa=0, ssao=True,
                shadow=True)
RENDER_CFG = dict(shadow_mode=2, shadow_size=2048, blocker_samples=16, pcf_samples=25, ssao_samples=64,
                  ssao_radius=0.5, ssao_bias=0.0005, ssao_range=0.01, blur_mode=0)
RENDER_W, RENDER_H = SCENE_KW["width"], SCENE_KW["height"]


# Triangles of the workload's scene: 20 icospheres of 20 * 4^5 faces and the 2-triangle ground.
TRIANGLES = 20 * 20 * 4 ** 5 + 2


def bench_config(ws: int) -> dict:
    """The `config` of the JSON line, the same in both arms."""
    return {"workload": WORKLOAD, "resolution": [SCENE_KW["width"], SCENE_KW["height"]], "triangles": TRIANGLES,
            "shadow_map": RENDER_CFG["shadow_size"], "ao": "plain SSAO",
            "l2": "flushed (256 MiB write) before every GPU step",
            "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"}


def scene_path() -> str:
    from forkerrenderer_gb300 import scenegen

    d = os.path.join(tempfile.gettempdir(), "fr_bench_c1_seed0")
    p = os.path.join(d, "scene.scene")
    if not os.path.exists(p):
        tmp = d + ".tmp%d" % os.getpid()
        scenegen.deferred_field_scene(tmp, **SCENE_KW)
        try:
            os.rename(tmp, d)
        except OSError:
            pass
    return p


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[0]))
                mx.append(float(s[1]))
            except ValueError:
                continue
            for n, v in zip(names, s[3:7]):
                if v.strip().lower() in ("active", "1"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def measured_bf16_peak() -> tuple[float, str]:
    """Dense BF16 TFLOP/s: the burst figure (a kernel timed alone)."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


def algorithmic_bytes(W: int, H: int, S: int) -> dict:
    """Algorithmic bytes per launch of the per-pixel passes (the minimum each
    kernel must move): lighting reads position 12 + normal 12 + albedo 4 +
    roughness/metalness/AO/type 4 + light-space NDC 12 + AO 1 and writes RGBA8 4
    per pixel, and touches the S^2 float shadow map once; SSAO reads view depth 4
    + normal 12 and writes AO 1 per pixel."""
    P = W * H
    return {"lighting": P * 49 + S * S * 4, "ssao": P * 17}


# DRAM bytes (read + write) and warp instructions (smsp__inst_executed.sum) per
# launch of the two per-pixel kernels at 1280x800 with a 2048^2 shadow map, from
# one ncu capture of this bench command:
#   ncu --section SpeedOfLight --section LaunchStats --metrics dram__bytes_read.sum,
#       dram__bytes_write.sum,smsp__inst_executed.sum,... --clock-control none
#       -k regex:"^k_ssao$|^k_tile_raster_shadow|^k_lighting|^k_setup" -c 5
#       python bench.py --steps 3 --warmup 3 --no-cpu-baseline --no-learned --batch-views 0
# Both kernels are bound by instruction issue, not DRAM: the issue roofline is the
# instruction count over the pass time against 4 warp instructions per SM per cycle.
NCU_DRAM_TRAFFIC = {"ssao": 20_000_512 + 768, "lighting": 48_232_448 + 62_464}
NCU_WARP_INSTRUCTIONS = {"ssao": 86_896_404, "lighting": 22_027_953}


def replica_ms_per_frame(dev_ms: float, steps: int, ws: int, device: str) -> tuple[float, float]:
    """Replicas: every rank renders `steps` frames; the job's time is the slowest
    rank's (MAX over ranks, an all-reduce on the process group's backend), and the
    whole job's ms per frame is that time over all ranks' frames. Returns (job
    milliseconds, ms per frame)."""
    if ws > 1:
        import torch

        tt = torch.tensor([dev_ms], dtype=torch.float64, device=device)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        dev_ms = float(tt.item())
    return dev_ms, dev_ms / (steps * ws)


def host_copy(m):
    import forkerrenderer_gb300 as fr

    h = fr.FrameMatrices()
    ctypes.memmove(ctypes.byref(h), ctypes.byref(m), ctypes.sizeof(m))
    return h


def orbit_matrices(scene, n: int) -> list:
    """n frames of a camera circling the scene centre at the scene camera's height
    and distance (0.5 degrees a step): (host-side FrameMatrices, eye) pairs."""
    import math

    ex, ey, ez = scene.info.eye
    rad = math.hypot(ex, ez)
    a0 = math.atan2(ex, ez)
    out = []
    for i in range(n):
        a = a0 + math.radians(0.5 * (i + 1))
        eye = (rad * math.sin(a), ey, rad * math.cos(a))
        out.append((host_copy(scene.view_matrices(eye, (0, 0, 0), RENDER_CFG["shadow_size"])), eye))
    return out


def e2e_frames(r, mats: list, pinned, flush, warmup: int):
    """Wall milliseconds of fr_render_frame (frame matrices and eye mats[i] from
    host memory) + the 8-bit frame's download into pinned memory, per frame
    after `warmup`."""
    import torch

    times = []
    for i, (m, eye) in enumerate(mats):
        flush.fill_(1)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        r.set_matrices(m, eye)
        r.Render()
        img = r.frame8(pinned)
        t2 = time.perf_counter()
        if i >= warmup:
            times.append((t2 - t1) * 1e3)
    return times, img


PARITY_BUFFERS = ["depth", "shadow", "gb_normal", "gb_position", "gb_lightndc", "gb_albedo", "gb_emissive",
                  "gb_param", "gb_type"]


def parity_record(r, scene) -> tuple[dict, float]:
    """The workload's frame on the GPU (scene camera, a fresh frame of the timed
    renderer) against the oracle's frame of the same scene, with the oracle's
    wall seconds on all host cores. Bar: visibility-derived buffers bit-exact,
    AO within 2e-6, 8-bit frame within 1 LSB on >= 99.9% of channels at >= 50 dB."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_bridge as OB

    r.set_matrices(None)
    r.Render()
    got = {"depth": r.depth(), "shadow": r.shadow_map(), "ao": r.ambient_occlusion(), "frame8": r.frame8()}
    for g in ("normal", "position", "lightndc", "albedo", "emissive", "param", "type"):
        got["gb_" + g] = r.gbuffer(g)
    want = OB.oracle_render(scene.handle, OB.reference_config(**RENDER_CFG, threads=os.cpu_count() or 1))
    mism = {k: int(np.count_nonzero(got[k].reshape(-1).view(np.uint32) != want[k].reshape(-1).view(np.uint32)))
            for k in PARITY_BUFFERS}
    d = np.abs(got["frame8"].astype(np.int32) - want["frame8"].astype(np.int32)).reshape(-1)
    mse = float((d.astype(np.float64) ** 2).mean())
    psnr = float("inf") if mse == 0 else 10 * np.log10(255.0 ** 2 / mse)
    ao = float(np.abs(got["ao"] - want["ao"]).max())
    within = float((d <= 1).mean())
    rec = {"against": "oracle (CPU restatement pinned bit for bit on the reference's output)",
           "visibility_bit_exact": all(v == 0 for v in mism.values()), "mismatched_elements": mism,
           "ao_max_abs": ao, "ao_tolerance": 2e-6, "frame8_within_1lsb": round(within, 6),
           "frame8_max_lsb": int(d.max()), "psnr_db": round(psnr, 2) if psnr != float("inf") else "inf"}
    rec["pass"] = bool(rec["visibility_bit_exact"] and ao <= 2e-6 and within >= 0.999 and
                       (psnr == float("inf") or psnr >= 50.0))
    return rec, float(want["seconds"])


def pass_medians(r, args, flush) -> dict:
    """Median CUDA-event pass times (ms) of args.steps frames of renderer r, L2
    flushed before each, after args.warmup untimed frames."""
    import torch

    for _ in range(args.warmup):
        r.Render()
        r.timings()
    passes = []
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        r.Render()
        passes.append(r.timings())
    return {k: statistics.median([p[k] for p in passes]) for k in passes[0]}


def run_gpu(args) -> dict:
    import numpy as np
    import torch

    import forkerrenderer_gb300 as fr

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    path = scene_path()
    t0 = time.perf_counter()
    scene = fr.Scene(path)  # host ingest: .scene / .obj / .mtl / .tga, models and textures in parallel
    t1 = time.perf_counter()
    # the timed renderer records only the frame's first and last events; the
    # per-pass breakdowns below come from renderers with pass events
    r = fr.Renderer(device=local, frame_graph=1, pass_timings=0, **RENDER_CFG)
    t2 = time.perf_counter()
    r.Preconfigure(scene)  # upload
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    scene_times = {"load_s": round(t1 - t0, 3), "upload_s": round(t3 - t2, 3), "threads": os.cpu_count()}
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        r.Render()
        r.timings()
    per_step = []
    barrier()
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            r.Render()
            t = r.timings()  # CUDA-event time of the frame on the render stream (waits for it)
            per_step.append(t["total"])
        barrier()
        wall = time.perf_counter() - t0
    launches = r.launch_count() * args.steps
    dev_ms, ms_per_frame = replica_ms_per_frame(sum(per_step), args.steps, ws, f"cuda:{local}")

    # e2e: each step's frame matrices from host memory in, the 8-bit frame out to
    # pinned host memory, inside the timed region
    m = scene.frame_matrices(RENDER_CFG["shadow_size"])
    pinned = torch.empty(m.width * m.height * 3, dtype=torch.uint8, pin_memory=True).numpy()
    h2d = ctypes.sizeof(fr.FrameMatrices) + 12  # the matrices and the eye
    e2e_times, img = e2e_frames(r, orbit_matrices(scene, args.warmup + args.steps), pinned, flush, args.warmup)
    static_times, _ = e2e_frames(r, [(host_copy(m), None)] * (args.warmup + args.steps), pinned, flush,
                                 args.warmup)
    d2h = int(img.nbytes)
    r.set_matrices(None)

    W, H, S = m.width, m.height, m.shadow_width
    alg = algorithmic_bytes(W, H, S)
    # The same frames with an event at every pass boundary (the breakdown; its total
    # carries those events' time). The timed frames overlap the shadow pass with
    # geometry, SSAO and blur; the per-kernel roofline uses the frame with every
    # pass in order, so each kernel's time is its own.
    rp = fr.Renderer(device=local, frame_graph=1, **RENDER_CFG)
    rp.Preconfigure(scene)
    med = pass_medians(rp, args, flush)
    rp.close()
    rs = fr.Renderer(device=local, frame_graph=1, concurrent_passes=0, **RENDER_CFG)
    rs.Preconfigure(scene)
    seq = pass_medians(rs, args, flush)
    rs.close()
    dominant = max(("ssao", "lighting"), key=lambda k: seq[k])
    peak, peak_kind = measured_peaks()
    achieved = alg[dominant] / (seq[dominant] * 1e-3) / 1e9
    res = {
        "metric": METRIC, "value": round(ms_per_frame, 4), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dev_ms / args.steps, 4),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generator, seed 0)",
        "config": bench_config(ws),
        "passes_ms_median": {k: round(v, 4) for k, v in med.items()},
        "passes_ms_median_sequential": {k: round(v, 4) for k, v in seq.items()},
        "passes_note": ("timed frames run the shadow pass beside geometry + SSAO + blur (two streams, "
                        "joined before lighting) and record only their first and last events; the "
                        "breakdowns come from the same frames with an event at every pass boundary "
                        "(their totals include those events' time); the sequential frame times each "
                        "pass alone"),
        "scene_ingest": scene_times,
        "clocks": clocks.summary(),
        "e2e": {"value": round(statistics.mean(e2e_times), 4), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "camera": ("moves every step (orbit about the scene centre): the frame graph is replayed "
                           "with each camera's frame constants"),
                "path": "fr_render_frame with host frame matrices + fr_download of the 8-bit frame"},
        "e2e_static_camera": {"value": round(statistics.mean(static_times), 4), "unit": UNIT,
                              "camera": "the scene's, every step: the frame graph is replayed"},
        "Mtri_per_s": round(scene.info.num_triangles / (ms_per_frame * 1e3), 1),
        "Mpix_per_s": round(W * H / (ms_per_frame * 1e3), 1),
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": "k_" + dominant, "achieved": round(achieved, 1),
                     "timed_in": "sequential frame (pass alone on the GPU)",
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_kind": peak_kind,
                     "traffic": NCU_DRAM_TRAFFIC[dominant] if (W, H, S) == (1280, 800, 2048) else None,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch",
                     "algorithmic_bytes_per_launch": alg[dominant]},
        "wall_s": round(wall, 3),
    }
    sm_mhz = res["clocks"].get("sm_mhz") or 2070.0
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    if (W, H, S) == (1280, 800, 2048):
        issue_peak = sms * 4 * sm_mhz * 1e6 / 1e12  # T warp instructions / s
        res["issue_roofline"] = {
            k: {"bound": "issue", "achieved": round(NCU_WARP_INSTRUCTIONS[k] / (seq[k] * 1e-3) / 1e12, 3),
                "peak": round(issue_peak, 3), "unit": "T warp-inst/s",
                "frac": round(NCU_WARP_INSTRUCTIONS[k] / (seq[k] * 1e-3) / 1e12 / issue_peak, 3),
                "warp_instructions_per_launch": NCU_WARP_INSTRUCTIONS[k]}
            for k in ("ssao", "lighting")}
    assert scene.info.num_triangles == TRIANGLES and (W, H, S) == (1280, 800, 2048)
    if rank == 0 and not args.no_cpu_baseline:
        res["parity"], sec = parity_record(r, scene)
        res["cpu_baseline"] = {"value": round(sec * 1e3, 3), "unit": UNIT, "cores": os.cpu_count() or 1,
                               "kind": "port",
                               "sample": "1 full frame of the workload (CPU restatement, all cores)"}
    res["outputs"] = tga_outputs(args, r, flush, rank == 0 and not args.no_cpu_baseline)
    if not args.no_learned:
        res["learned_ao"] = learned_ao(args, scene, flush, local, med, seq, rank == 0)
    if args.batch_views > 0:
        res["batched_views"] = batched_views(args, scene, flush, local)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return res if rank == 0 else None


# The shipped learned-AO model: input view depth, normal x / y and a 16-sample SSAO
# (aonet_field20.f32 is the geometry-only variant: view depth and normal).
WEIGHTS = os.path.join(ROOT, "forkerrenderer_gb300", "weights", "aonet_field20_ssao16.f32")

# Bytes the encoder must read per pixel of each output's device source
# (8-bit frame: 4; float buffers: 4; G-buffer fields: one 16-byte plane).
TGA_SOURCE_BYTES = {"framebuffer.tga": 4, "framebuffer_SSAA.tga": 4, "shadowmap.tga": 4, "zbuffer.tga": 4,
                    "gbuffer_normal.tga": 16, "gbuffer_worldpos.tga": 16, "gbuffer_albedo.tga": 16,
                    "gbuffer_param.tga": 16, "gbuffer_shading_type.tga": 16, "gbuffer_ambient_occlusion.tga": 4}


def tga_outputs(args, r, flush, cpu_baseline):
    """The reference's output stage (main.cpp:45-54: every Output:: TGA file of
    the frame) on the last frame: device time of the encoding kernels, end to end
    through fr_output_encode_all (files in host memory), and the oracle's CPU
    encoding of the same images (conversion + RLE, one core)."""
    import torch

    from forkerrenderer_gb300 import output

    files, _ = output.encode_all(r)  # the files themselves, for the checks below
    pinned = torch.empty(output.max_bytes(r), dtype=torch.uint8, pin_memory=True)
    for _ in range(args.warmup):
        output.encode_all_into(r, pinned.data_ptr())
    dev, e2e = [], []
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sizes, ms = output.encode_all_into(r, pinned.data_ptr())  # every file, in pinned host memory
        e2e.append((time.perf_counter() - t0) * 1e3)
        dev.append(ms)
    assert sum(sizes) == sum(len(d) for d in files.values())
    pixels = {fn: int.from_bytes(d[12:14], "little") * int.from_bytes(d[14:16], "little") for fn, d in files.items()}
    out_bytes = sum(len(d) for d in files.values())
    alg = out_bytes + sum(pixels[fn] * TGA_SOURCE_BYTES[fn] for fn in files)
    dmed = statistics.median(dev)
    res = {"files": len(files), "file_bytes": out_bytes, "pixels": sum(pixels.values()),
           "device_ms_median": round(dmed, 4), "e2e_ms_median": round(statistics.median(e2e), 4),
           "algorithmic_bytes": alg, "achieved_GBps": round(alg / (dmed * 1e-3) / 1e9, 1),
           "kernels_per_frame": 3, "rle": True,
           "e2e_path": "fr_output_encode_all: encode on the device, every file copied into pinned host memory"}
    if cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle_bridge as OB
        import tga_util as T

        bufs = {"frame8": r.frame8(), "depth": r.depth(), "shadow": r.shadow_map(), "ao": r.ambient_occlusion()}
        for g, key in (("normal", "gb_normal"), ("position", "gb_position"), ("albedo", "gb_albedo"),
                       ("param", "gb_param"), ("type", "gb_type")):
            bufs[key] = r.gbuffer(g)
        t0 = time.perf_counter()
        n = 0
        for fn, key, kind in T.OUTPUTS:
            if fn in files:
                assert OB.oracle_tga(T.reference_image(key, kind, bufs)) == files[fn], fn
                n += 1
        cpu_ms = (time.perf_counter() - t0) * 1e3
        res["cpu_baseline"] = {"value": round(cpu_ms, 2), "unit": "ms", "cores": 1, "kind": "port",
                               "sample": f"the {n} files of one frame, conversion + RLE (oracle restatement)"}
        res["matches_oracle"] = True
    return res


def learned_ao(args, scene, flush, local, plain_med, plain_seq, evaluate):
    """The same frames with the learned AO (U-Net + 1-in-64 probe, plain SSAO as the
    gated fallback), timed with the same protocol, and its AO error against
    256-sample SSAO (+ blur) on held-out views, next to plain 64-sample SSAO. The
    frame times compare the concurrent frames; the AO stage times compare
    sequential frames (each pass alone on the GPU)."""
    import torch

    import forkerrenderer_gb300 as fr
    from forkerrenderer_gb300 import _native as N
    from forkerrenderer_gb300.aonet import AONet, train
    from forkerrenderer_gb300.train_ao import load_params

    weights = args.ao_weights or WEIGHTS
    with open(os.path.splitext(weights)[0] + ".json") as f:
        meta = json.load(f)
    thr = float(meta.get("probe_threshold", 0.06))
    ins = int(meta.get("input_samples", 0))
    net = AONet(local)
    net.set_params(load_params(weights))
    meds = []
    for concurrent in (1, 0):
        r = fr.Renderer(device=local, frame_graph=1, ao_mode=N.FR_AO_LEARNED, ao_probe_threshold=thr,
                        ao_input_samples=ins, concurrent_passes=concurrent, **RENDER_CFG)
        r.Preconfigure(scene)
        r.set_ao_net(net)
        meds.append(pass_medians(r, args, flush))
        if concurrent:
            mean_sq, fell = r.ao_probe_result()
            launches = r.launch_count()
            net_ms = network_ms(args, r, net, flush, local)
        r.close()
    med, seq = meds
    ao_l = seq["ssao"] + seq["blur"]
    ao_p = plain_seq["ssao"] + plain_seq["blur"]
    out = {
        "ms_per_frame": round(med["total"], 4),
        "passes_ms_median": {k: round(v, 4) for k, v in med.items()},
        "passes_ms_median_sequential": {k: round(v, 4) for k, v in seq.items()},
        "ao_stage_ms": round(ao_l, 4), "plain_ao_stage_ms": round(ao_p, 4),
        "ao_stage_speedup": round(ao_p / ao_l, 3), "frame_speedup": round(plain_med["total"] / med["total"], 3),
        "probe": {"mean_sq_diff": round(mean_sq, 5), "threshold": thr, "fell_back": fell},
        "gpu_launches_per_frame": launches,
        "network": "U-Net 3 levels 16/32/64, level 0 on 2x2 pixel blocks, BF16 tcgen05 convs",
        "tensor_roofline": tensor_roofline(net_ms),
        "input": (("view depth, normal x / y, %d-sample SSAO (no blur)" % ins) if ins > 0 else
                  "view depth (BF16 value + its rounding residual) and normal x / y" if ins < 0 else
                  "view depth and normal"),
        "weights": os.path.relpath(weights, ROOT),
        "training": {k: meta.get(k) for k in ("steps_done", "command", "train_seconds", "label_seconds")},
    }
    if evaluate and args.ao_eval_views > 0:
        rep, _ = train(scene, net, fr.default_config(device=local, ao_input_samples=ins, **RENDER_CFG), steps=0,
                       train_views=1,
                       eval_views=args.ao_eval_views, seed=1, log_every=0)
        out.update({
            "eval_views": args.ao_eval_views,
            "rmse_vs_256spp_ssao": round(rep["eval_rmse_covered"], 5),
            "rmse_vs_256spp_ssao_all_pixels": round(rep["eval_rmse"], 5),
            "max_abs_err": round(rep["eval_max_err"], 5),
            "plain64_rmse_vs_256spp": round(rep["plain_rmse_covered"], 5),
            "no_ao_rmse_vs_256spp": round(rep["none_rmse_covered"], 5),
            "rmse_target": 0.02, "meets_rmse_target": bool(rep["eval_rmse_covered"] <= 0.02),
        })
    net.close()
    return out


# The network's 3x3 convolutions (input channels, output channels, level) and its
# 1x1 head (16 -> 4 sub-pixel values); level 0 works on 2x2 pixel blocks, each
# level 4x coarser than the one above.
UNET_LAYERS = [(16, 16, 0), (16, 16, 0), (16, 32, 1), (32, 32, 1), (32, 64, 2), (64, 64, 2), (96, 32, 1),
               (32, 32, 1), (48, 16, 0), (16, 16, 0)]
# ncu --set full capture of the level-0 16 -> 16 convolution (k_conv3x3, 760 CTAs) in
# the 1280x800 learned frame: sm__pipe_tensor_cycles_active.avg.pct_of_peak_sustained_active
NCU_TENSOR_PIPE_LEVEL0 = 0.050


def network_flops(W: int, H: int) -> int:
    """Algorithmic FLOPs of one forward of the network on a W x H frame (2 per MAC)."""
    pos0 = (W // 2) * (H // 2)
    total = sum(pos0 // 16 ** lv * cin * cout * 9 * 2 for cin, cout, lv in UNET_LAYERS)
    return total + pos0 * 16 * 4 * 2


def network_ms(args, r, net, flush, local) -> float:
    """Median device time (CUDA events on the launching stream, L2 flushed before
    each) of the network's forward on the frame's own input (fr_ao_features of the
    renderer's last frame): its 14 kernels plus the space-to-depth pass of the
    full-resolution input that the frame's own blocked input skips."""
    import torch

    W, H = RENDER_W, RENDER_H
    dev = f"cuda:{local}"
    feat = torch.zeros((1, 1, H, W, 8), dtype=torch.int16, device=dev)
    r.ao_features(feat)
    torch.cuda.synchronize(dev)  # the features come from the renderer's stream
    out = torch.empty((1, H, W), dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        net.forward(feat, 1, H, W, out, st)
    times = []
    for _ in range(args.steps):
        flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        net.forward(feat, 1, H, W, out, st)
        e1.record(st)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    net.check(st)
    return statistics.median(times)


def tensor_roofline(net_ms: float) -> dict:
    """The network's tensor-core use: algorithmic FLOPs / its forward time against
    the measured dense BF16 peak, and the ncu tensor-pipe activity of its largest layer."""
    peak, kind = measured_bf16_peak()
    flops = network_flops(RENDER_W, RENDER_H)
    achieved = flops / (net_ms * 1e-3) / 1e12
    return {"bound": "tensor", "flops_per_forward": flops, "forward_ms": round(net_ms, 4),
            "achieved": round(achieved, 2), "peak": peak, "unit": "TFLOP/s", "frac": round(achieved / peak, 4),
            "peak_kind": kind, "ncu_tensor_pipe_active_level0": NCU_TENSOR_PIPE_LEVEL0}


BATCH_SIZES = [(256, 256), (640, 400), (1280, 800), (1920, 1080)]


def batched_views(args, scene, flush, local):
    """Many views of the scene in one batch: camera views of sizes drawn uniformly
    from 256x256, 640x400, 1280x800, 1920x1080 (cameras on a hemisphere of radius
    4..8 around the scene centre) plus 4 directional lights with 2048^2 shadow
    maps; deferred PBR + PCF; learned AO on the views whose size the network
    takes (multiples of 32), plain SSAO on the others. Autotuned, then timed
    (one step = one batch = one CUDA graph launch)."""
    import math
    import random

    import torch

    import forkerrenderer_gb300 as fr
    from forkerrenderer_gb300 import _native as N
    from forkerrenderer_gb300.aonet import AONet
    from forkerrenderer_gb300.batch import Batch, directional_light, view
    from forkerrenderer_gb300.train_ao import load_params

    rng = random.Random(4)
    cfg = dict(RENDER_CFG, shadow_mode=N.FR_SHADOW_PCF, shadow_size=2048)
    weights = args.ao_weights or WEIGHTS
    with open(os.path.splitext(weights)[0] + ".json") as f:
        ins = int(json.load(f).get("input_samples", 0))
    r = fr.Renderer(device=local, **cfg, ao_probe_threshold=1e9, ao_input_samples=ins)
    r.Preconfigure(scene)
    net = AONet(local)
    net.set_params(load_params(weights))
    r.set_ao_net(net)
    import ctypes as C

    views, n_learned = [], 0
    for _ in range(args.batch_views):
        w, h = BATCH_SIZES[rng.randrange(len(BATCH_SIZES))]
        rad, ct, ph = rng.uniform(4, 8), rng.uniform(0.25, 0.95), rng.uniform(0, 2 * math.pi)
        st = math.sqrt(1 - ct * ct)
        eye = (rad * st * math.cos(ph), rad * ct, rad * st * math.sin(ph))
        m = scene.view_matrices(eye, (0, 0, 0), 2048)
        vm = fr.FrameMatrices()
        C.memmove(C.byref(vm), C.byref(m), C.sizeof(m))
        vm.width, vm.height = w, h
        vm.viewport[:] = [w / 2, 0, 0, w / 2, 0, h / 2, 0, h / 2, 0, 0, 0.5, 0.5, 0, 0, 0, 1]
        learned = w % 32 == 0 and h % 32 == 0
        n_learned += learned
        views.append(view(vm, eye, N.FR_AO_LEARNED if learned else N.FR_AO_SSAO))
    lights = [directional_light((0.35, -1.0, 0.25), (0.9, 0.85, 0.8), 2048, 6.0),
              directional_light((-0.6, -0.7, 0.3), (0.3, 0.35, 0.45), 2048, 6.0),
              directional_light((0.1, -0.9, -0.6), (0.25, 0.25, 0.2), 2048, 6.0),
              directional_light((-0.2, -1.0, -0.1), (0.2, 0.2, 0.25), 2048, 6.0)]
    b = Batch(r, views, lights)
    t0 = time.perf_counter()
    best, best_ms = b.autotune(reps=2)
    tune_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        b.render()
        b.timings()
    stages = []
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        b.render()
        stages.append(b.timings())
    med = {k: statistics.median([s[k] for s in stages]) for k in stages[0]}
    w = b.work()
    ms = med["total"]
    out = {
        "ms_per_batch": round(ms, 3), "views": len(views), "learned_ao_views": n_learned,
        "view_sizes": {f"{a}x{c}": sum(1 for v in views if (v.matrices.width, v.matrices.height) == (a, c))
                       for a, c in BATCH_SIZES},
        "lights": "4 directional, 2048^2 shadow maps, PCF 25", "stages_ms_median": {k: round(v, 3) for k, v in med.items()},
        "triangles_per_batch": w["triangles"], "pixels_per_batch": w["pixels"],
        "Mtri_per_s": round(w["triangles"] / (ms * 1e3), 1), "Mpix_per_s": round(w["pixels"] / (ms * 1e3), 1),
        "ms_per_view": round(ms / len(views), 4),
        "autotuned": {"light_tile": best[0], "bin_batch": best[1], "ctas_per_sm": best[2],
                      "best_ms": round(best_ms, 3), "sweep_seconds": round(tune_s, 1)},
        "graph": "one CUDA graph per batch; fine raster and lighting are persistent (view, tile) queue launches",
    }
    b.close()
    r.close()
    net.close()
    return out


def cpu_oracle_frame(threads: int) -> tuple[float, int]:
    """One full frame of the workload on the CPU restatement; returns seconds."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_bridge as OB

    import forkerrenderer_gb300 as fr

    scene = fr.Scene(scene_path())
    cfg = OB.reference_config(**RENDER_CFG, threads=threads)
    out = OB.oracle_render(scene.handle, cfg)
    return out["seconds"], threads


def run_reference(args) -> dict | None:
    ws, rank, _ = dist_env()
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    from forkerrenderer_gb300.build import build_oracle

    build_oracle()
    for _ in range(max(0, min(args.warmup, 1))):
        cpu_oracle_frame(threads)
    times = [cpu_oracle_frame(threads)[0] for _ in range(args.steps)]
    ms = statistics.mean(times) * 1e3
    sample = f"{args.steps} full frame(s) of the workload"
    return {"metric": METRIC, "value": round(ms, 3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator, seed 0)", "impl": "reference",
            "config": bench_config(ws),
            "cpu_baseline": {"value": round(ms, 3), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(ms, 3), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-AO frames")
    ap.add_argument("--ao-eval-views", type=int, default=200, help="held-out views for the learned-AO error")
    ap.add_argument("--batch-views", type=int, default=64, help="views of the batched multi-view line (0 = skip)")
    ap.add_argument("--ao-weights", default=None, help="learned-AO weights (default: the shipped field-scene model)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup) if args.impl == "gb300" else args.warmup
    if args.impl == "reference":
        res = run_reference(args)
        if res is not None:
            print(json.dumps(res))
        return
    from forkerrenderer_gb300.build import build_native

    build_native()
    res = run_gpu(args)
    if res is None:
        return
    print(json.dumps(res))


if __name__ == "__main__":
    main()
