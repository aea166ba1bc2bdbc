"""Benchmark of the GI/lighting stage: 1080p GI+denoise frames.

One step = one frame of the stage on the 1920x1080 workload (40-box room,
2048 VPLs with 6x128^2 FP16 distance cubes, 4 point lights, 4x2048^2 CSM,
<= 64 VPLs per 16x16 tile, K = 8 samples per pixel, 5 denoise passes):
VPL visibility cull, deferred PBR + CSM, tile cull, GI gather, merge +
4 a-trous passes with temporal reprojection and composite, through
sgi_render_frame. The 8-frame seeded camera path rotates, so consecutive steps
read different G-buffers and CSMs (8 x 126 MB of per-frame inputs, above the
129 MB L2) and L2 is additionally flushed before every timed step.

value  = Mpix/s with inputs resident in HBM (CUDA events around each frame).
e2e    = Mpix/s through the C ABI with the frame's G-buffer and light records
         copied from pinned host memory and the HDR frame copied back, every step.
--impl reference times the CPU restatement of the reference shaders (FP32
oracle, all host threads) on the same workload.
"""
from __future__ import annotations

import argparse
import datetime
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "1080p GI+denoise Mpix/s (plain a-trous path; neural vs plain at equal PSNR under equal_psnr)"
UNIT = "Mpix/s"
CPU_SAMPLE_S = 10.0   # seconds of oracle frames timed for the CPU baseline


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["hd", "small"], default="hd")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-uhd", action="store_true", help="skip the 3840x2160 neural/plain comparison")
    ap.add_argument("--no-batched", action="store_true", help="skip the 64-view CUDA graph batch")
    ap.add_argument("--profile", action="store_true",
                    help="profiling case for ncu: the same 1080p workload with a 2-frame path, "
                         "--warmup + --steps frames of sgi_render_frame only (no e2e or CPU legs)")
    ap.add_argument("--neural", action="store_true",
                    help="with --profile: frames of sgi_render_frame_neural (K = 2) instead")
    ap.add_argument("--persistent", action="store_true",
                    help="with --profile: 8 views of 960x540 of one room rendered by the persistent batch kernel")
    ap.add_argument("--atrous", choices=["direct", "staged"], default=None,
                    help="with --profile: the a-trous tap staging (default: the library's default)")
    ap.add_argument("--fast", action="store_true",
                    help="with --profile: the shading kernels in their tolerance mode (SGI_SHADING_FAST)")
    ap.add_argument("--fp8", action="store_true",
                    help="with --profile --neural: FP8 E4M3 convolutions (calibrated on another room) at K = 1")
    return ap.parse_args()


def workload(name):
    from stratusgfx_gb300 import scene as S
    return S.HD if name == "hd" else S.SMALL


# ------------------------------------------------------------- clocks ----
class ClockSampler:
    """nvidia-smi clock and throttle-reason samples every 50 ms. start() returns
    once the first sample is in, so the samples cover the timed region;
    window() marks that region and stop() keeps the samples taken inside it
    (all samples if none fell inside, which the result says)."""
    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None
        self.t0 = self.t1 = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "50"], stdout=open(self.path, "w"),
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        deadline = time.time() + 5.0
        while time.time() < deadline and os.path.getsize(self.path) == 0 and self.proc.poll() is None:
            time.sleep(0.01)

    def window(self, begin: bool):
        if begin:
            self.t0 = datetime.datetime.now()
        else:
            self.t1 = datetime.datetime.now()

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.06)   # one more sample after the timed region
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 10:
                    continue
                try:
                    ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f")
                    rows.append((ts, float(parts[2]), float(parts[3]),
                                 {n for n, v in zip(names, parts[6:10]) if v.lower().startswith("active")}))
                except ValueError:
                    continue
        os.unlink(self.path)
        inside = [r for r in rows if self.t0 and self.t1 and
                  self.t0 - datetime.timedelta(milliseconds=50) <= r[0] <= self.t1 + datetime.timedelta(milliseconds=50)]
        use = inside or rows
        reasons = set().union(*[r[3] for r in use]) if use else set()
        out = {"sm_mhz": statistics.median([r[1] for r in use]) if use else None,
               "sm_max_mhz": use[-1][2] if use else None, "reasons": sorted(reasons), "samples": len(use)}
        if rows and not inside:
            out["note"] = "no sample fell inside the timed region; all samples of the run reported"
        return out


# ------------------------------------------------- algorithmic bytes ----
def kernel_bytes(w) -> dict:
    """Bytes each kernel (group) must move per frame: each input read once, each output written once, in the
    layouts these kernels use (the gather writes the per-pixel guide the later passes read)."""
    P = w.width * w.height
    cube = 2 if w.cube_format == 1 else 4
    # gather: depth, normal, albedo, rma (4 B each), reflectivity, ssao (2 B each), K cube texels;
    # writes the pass-0 reservoir (8 B) and the guide (16 B)
    gather = P * (4 + 4 + 4 + 4 + 2 + 2 + w.samples * cube + 8 + 16)
    atrous = P * (8 + 16 + 8) * (w.denoise_passes - 2)
    # final: reservoir, guide, albedo, screen, velocity, id, prev depth/normal/id, prev GI, history in;
    # HDR, GI, history out
    final = P * (8 + 16 + 4 + 8 + 4 + 4 + 4 + 4 + 4 + 8 + 2 + 8 + 8 + 2)
    deferred = P * (4 + 4 + 4 + 4 + 2 + 2 + 8) + 4 * w.csm_resolution ** 2 * 4
    tiles = P * (4 + 4)
    vis = w.num_vpls * (64 + 8 + 4 + 1)
    return {"vpl_cull": vis, "deferred_pbr_csm": deferred, "tile_cull": tiles, "vpl_gather": gather,
            "atrous": atrous, "denoise_final": final}


# kernel (group) -> index into sgi_get_pass_times with the denoise split, and the CUDA kernels it holds
KERNELS = {"vpl_cull": (0, "vpl_cull_kernel (visibility flags and, in its last block, the compaction)"),
           "deferred_pbr_csm": (1, "deferred_pbr_csm_kernel"),
           "tile_cull": (2, "tile_stage1_kernel + tile_cull_kernel"),
           "vpl_gather": (3, "vpl_gather_kernel (gather + denoise pass 0 merge + guide)"),
           "atrous": (5, "atrous_staged_kernel x (denoise passes - 2) (strides 2, 4, 8; atrous_kernel beyond)"),
           "denoise_final": (6, "denoise_final_kernel")}


def kernel_flops(fl: dict) -> dict:
    """Algorithmic FLOPs per frame of each kernel (group) from the oracle's counting instantiation."""
    return {"vpl_cull": fl["vpl_cull"][0], "deferred_pbr_csm": fl["direct"][0],
            "tile_cull": fl["tile_stage1"][0] + fl["tile_stage2"][0],
            "vpl_gather": fl["gather"][0] + fl["denoise_pass0"][0], "atrous": fl["atrous"][0],
            "denoise_final": fl["denoise_final"][0]}


def fp32_peak_tflops(sm_mhz) -> tuple[float, str]:
    """FP32 rate of the GPU at the sampled SM clock: SMs x 128 FP32 lanes x 2 FLOP (FMA) per cycle."""
    import torch
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = sm_mhz or 2070.0
    return sms * 128 * 2 * mhz * 1e6 / 1e12, (f"nominal FP32 rate at the sampled SM clock: {sms} SMs x 128 lanes "
                                               f"x 2 FLOP x {mhz:.0f} MHz")


def traffic_from_profiles(kernel: str):
    """DRAM bytes per frame of a kernel group (ncu dram__bytes_read.sum + dram__bytes_write.sum summed over its
    launches in one frame) recorded in profiles/traffic.json (None if absent)."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get(kernel)
    except Exception:
        return None


# --------------------------------------------------------- our arm ----
def run_ours(args, rank, world, local_rank):
    import torch

    from stratusgfx_gb300 import abi, replicas, stage
    from stratusgfx_gb300 import scene as S

    torch.cuda.set_device(local_rank)
    w = workload(args.workload)
    P = w.width * w.height
    sc = S.workload_scene(w, 1234 + 2 + rank)
    ds = stage.DeviceScene(sc, w)
    cfg = stage.workload_config(w)
    st = stage.GiStage(cfg)
    st.set_lights(ds.vpls, ds.entries, ds.points)
    frames = len(sc.cameras) - 1
    out = torch.empty((w.height, w.width, 4), dtype=torch.float16, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    fps = 60.0
    torch.cuda.synchronize()
    launches0 = st.launch_count()

    def frame(step):
        k = step % frames + 1
        st.set_shadow_maps(ds.csms[k], ds.cubes)
        st.render_frame(ds.gbuffers[k], ds.gbuffers[k - 1], ds.camera(k), out, 1000.0 + 16.0 * step, fps)

    for s in range(args.warmup):
        frame(s)
    torch.cuda.synchronize()
    replicas.barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(local_rank)
    clocks.start()
    launches_before = st.launch_count()
    torch.cuda.synchronize()
    clocks.window(True)
    for s in range(args.steps):
        flush.fill_(float(s))                    # evict L2 (256 MB > 129 MB), outside the events
        starts[s].record()
        frame(args.warmup + s)                   # direct lighting overlaps the culls and the gather
        ends[s].record()
    torch.cuda.synchronize()
    clocks.window(False)
    launches_timed = st.launch_count() - launches_before
    clock = clocks.stop()
    ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    # per-pass breakdown: the same frames with per-pass events (the passes then run in sequence)
    def per_pass(stage_obj, render):
        stage_obj.set_timing(True)
        acc = np.zeros(7)
        for s in range(args.steps):
            flush.fill_(float(s))
            render(args.warmup + s)
            acc += np.array(stage_obj.pass_times(split=True))   # synchronises on the frame's last event
        stage_obj.set_timing(False)
        torch.cuda.synchronize()
        return acc

    pass_ms = per_pass(st, frame)

    # ---- the same frames in the tolerance mode of the shading kernels (SGI_SHADING_FAST)
    stf = stage.GiStage(cfg)
    abi.check(stf.lib.sgi_set_shading_precision(stf.ctx, abi.SGI_SHADING_FAST), stf.ctx)
    stf.set_lights(ds.vpls, ds.entries, ds.points)

    def frame_fast(step):
        k = step % frames + 1
        stf.set_shadow_maps(ds.csms[k], ds.cubes)
        stf.render_frame(ds.gbuffers[k], ds.gbuffers[k - 1], ds.camera(k), out, 1000.0 + 16.0 * step, fps)

    for s in range(args.warmup):
        frame_fast(s)
    torch.cuda.synchronize()
    fast_ms = 0.0
    for s in range(args.steps):
        flush.fill_(float(s))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        frame_fast(args.warmup + s)
        e1.record()
        torch.cuda.synchronize()
        fast_ms += e0.elapsed_time(e1)
    fast_ms /= args.steps
    fast_pass_ms = per_pass(stf, frame_fast)
    stf.close()

    # ---- a-trous passes with the other tap staging (SGI_ATROUS_DIRECT / _STAGED), per-pass times
    def staging_leg(fast_mode, staged):
        sx = stage.GiStage(cfg)
        if fast_mode:
            abi.check(sx.lib.sgi_set_shading_precision(sx.ctx, abi.SGI_SHADING_FAST), sx.ctx)
        abi.check(sx.lib.sgi_set_atrous_staging(sx.ctx, abi.SGI_ATROUS_STAGED if staged else abi.SGI_ATROUS_DIRECT),
                  sx.ctx)
        sx.set_lights(ds.vpls, ds.entries, ds.points)

        def frame_x(step):
            k = step % frames + 1
            sx.set_shadow_maps(ds.csms[k], ds.cubes)
            sx.render_frame(ds.gbuffers[k], ds.gbuffers[k - 1], ds.camera(k), out, 1000.0 + 16.0 * step, fps)

        for s in range(args.warmup):
            frame_x(s)
        acc = per_pass(sx, frame_x)
        abi.check(sx.lib.sgi_device_status(sx.ctx), sx.ctx)
        sx.close()
        return acc

    default_staged = st.lib.sgi_get_atrous_staging(st.ctx) == abi.SGI_ATROUS_STAGED
    other_ms = staging_leg(False, not default_staged)
    other_fast_ms = staging_leg(True, not default_staged)
    atrous_ms = {False: (pass_ms[5], fast_pass_ms[5]), True: (other_ms[5], other_fast_ms[5])}
    if default_staged:
        atrous_ms = {True: atrous_ms[False], False: atrous_ms[True]}
    staging = {"default": "staged" if default_staged else "direct",
               "passes": "a-trous passes 1 .. n-2 (strides 2, 4, 8), ms per frame from per-pass events",
               "exact": {"direct_ms": round(atrous_ms[False][0] / args.steps, 4),
                         "staged_ms": round(atrous_ms[True][0] / args.steps, 4)},
               "fast": {"direct_ms": round(atrous_ms[False][1] / args.steps, 4),
                        "staged_ms": round(atrous_ms[True][1] / args.steps, 4)}}
    total_ms = replicas.max_over_ranks(float(sum(ms)), device="cuda")
    ms_per_step = total_ms / args.steps
    value = replicas.job_throughput(P * args.steps, world, total_ms) / 1e6

    # ---- e2e: host buffers through the public API (ABI), copies inside the timed region.
    # Three G-buffer slots and two output buffers: the host->device copy of frame s+1 and the
    # device->host copy of frame s-1 run on a copy stream while frame s renders.
    host_g = [g.pinned_clone() for g in ds.gbuffers]
    host_vpls = ds.vpls.cpu().pin_memory()
    host_entries = ds.entries.cpu().pin_memory()
    host_points = ds.points.cpu().pin_memory() if ds.points is not None else None
    dev_vpls = [torch.empty_like(ds.vpls) for _ in range(2)]
    dev_entries = [torch.empty_like(ds.entries) for _ in range(2)]
    dev_points = [torch.empty_like(ds.points) for _ in range(2)] if ds.points is not None else [None, None]
    slots = [stage.GBufferTensors(w.height, w.width, "cuda") for _ in range(3)]
    outs = [torch.empty((w.height, w.width, 4), dtype=torch.float16, device="cuda") for _ in range(2)]
    host_out = torch.empty((w.height, w.width, 4), dtype=torch.float16).pin_memory()
    st2 = stage.GiStage(cfg)
    h2d = slots[0].nbytes()
    h2d += host_vpls.numel() * 4 + host_entries.numel() * 4 + (host_points.numel() * 4 if host_points is not None else 0)
    d2h = host_out.numel() * 2
    comp = torch.cuda.current_stream()
    copy = torch.cuda.Stream()

    def upload(step):
        """Frame `step`'s inputs -> slot step % 3 and light buffers step % 2, on the copy stream."""
        k = step % frames + 1
        with torch.cuda.stream(copy):
            slots[step % 3].copy_from(host_g[k], non_blocking=True)
            dev_vpls[step % 2].copy_(host_vpls, non_blocking=True)
            dev_entries[step % 2].copy_(host_entries, non_blocking=True)
            if dev_points[0] is not None:
                dev_points[step % 2].copy_(host_points, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(copy)
        return ev

    def e2e_run(first, n, start_event=None):
        """Renders frames first .. first+n-1 from host inputs to host outputs (asynchronous)."""
        if start_event is not None:
            copy.wait_event(start_event)
        ready = upload(first)
        done = [None, None]       # compute finished frame s (its inputs and lights are free)
        fetched = [None, None]    # device->host copy of frame s finished (its output buffer is free)
        for step in range(first, first + n):
            k = step % frames + 1
            comp.wait_event(ready)
            if fetched[step % 2] is not None:
                comp.wait_event(fetched[step % 2])
            if step + 1 < first + n:
                if done[(step + 1) % 2] is not None:
                    copy.wait_event(done[(step + 1) % 2])
                ready = upload(step + 1)
            st2.set_lights(dev_vpls[step % 2], dev_entries[step % 2], dev_points[step % 2])
            st2.set_shadow_maps(ds.csms[k], ds.cubes)
            st2.render_frame(slots[step % 3], slots[(step - 1) % 3], ds.camera(k), outs[step % 2],
                             1000.0 + 16.0 * step, fps)
            ev = torch.cuda.Event()
            ev.record(comp)
            done[step % 2] = ev
            with torch.cuda.stream(copy):
                copy.wait_event(ev)
                host_out.copy_(outs[step % 2], non_blocking=True)
                f = torch.cuda.Event()
                f.record(copy)
                fetched[step % 2] = f

    slots[2].copy_from(host_g[0])              # the frame before the first one
    e2e_run(0, args.warmup)
    torch.cuda.synchronize()
    replicas.barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(comp)
    e2e_run(args.warmup, args.steps, e0)
    e1.record(copy)                            # after the last device->host copy
    torch.cuda.synchronize()
    e2e_ms = replicas.max_over_ranks(e0.elapsed_time(e1), device="cuda")
    e2e_value = replicas.job_throughput(P * args.steps, world, e2e_ms) / 1e6

    # ---- per-kernel roofline: algorithmic bytes against HBM, algorithmic FLOPs against the FP32 rate
    parity = cpu = None
    flops = None
    if rank == 0 and not args.no_cpu_baseline:
        parity, cpu, fl = parity_and_cpu_baseline(ds, sc, w, cfg)
        flops = kernel_flops(fl)
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs") or 6800.0
    peak_src = "measured" if peaks.get("hbm_gbs") else "fallback"
    fp32_peak, fp32_src = fp32_peak_tflops(clock.get("sm_mhz"))
    kb = kernel_bytes(w)

    def kernel_table(pms):
        table = {}
        for name, (idx, what) in KERNELS.items():
            avg = pms[idx] / args.steps
            gbs = kb[name] / (avg / 1e3) / 1e9 if avg > 0 else 0.0
            k = {"kernels": what, "ms": round(avg, 4), "alg_bytes": kb[name], "gbs": round(gbs, 1),
                 "frac_hbm": round(gbs / hbm_peak, 4)}
            if flops is not None:
                tf = flops[name] / (avg / 1e3) / 1e12 if avg > 0 else 0.0
                k.update({"alg_flops": int(flops[name]), "tflops": round(tf, 2),
                          "frac_fp32": round(tf / fp32_peak, 4)})
                k["bound"] = "fp32" if k["frac_fp32"] > k["frac_hbm"] else "hbm"
            else:
                k["bound"] = "hbm"
            table[name] = k
        return table

    kernels = kernel_table(pass_ms)
    fast = {"shading": "SGI_SHADING_FAST (approximate division, square root and exponential, contraction; "
                       "decisions and texel choices correctly rounded)",
            "ms_per_frame": round(fast_ms, 4), "mpix_s": round(P / fast_ms / 1e3, 1),
            "speedup_vs_exact": round(ms_per_step / fast_ms, 3), "kernels": kernel_table(fast_pass_ms)}
    dom = max(kernels, key=lambda n: kernels[n]["ms"])
    dk = kernels[dom]
    if dk["bound"] == "fp32":
        roof = {"bound": "fp32", "kernel": dom, "achieved": dk["tflops"], "peak": round(fp32_peak, 1),
                "unit": "TFLOP/s", "frac": dk["frac_fp32"], "peak_source": fp32_src,
                "alg_flops_per_launch": dk["alg_flops"], "frac_hbm": dk["frac_hbm"]}
    else:
        roof = {"bound": "hbm", "kernel": dom, "achieved": dk["gbs"], "peak": hbm_peak, "unit": "GB/s",
                "frac": dk["frac_hbm"], "peak_source": peak_src}
    roof["alg_bytes_per_launch"] = dk["alg_bytes"]
    roof["traffic"] = traffic_from_profiles(dom)
    roof["hbm_peak_gbs"] = hbm_peak
    roof["hbm_peak_source"] = peak_src

    result = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": w.name, "resolution": f"{w.width}x{w.height}", "vpls": w.num_vpls,
                   "cube": f"6x{w.cube_size}^2 {'fp16' if w.cube_format == 1 else 'fp32'}",
                   "csm": f"4x{w.csm_resolution}^2 fp32", "point_lights": w.num_points, "tile": w.tile_size,
                   "max_vpls_per_tile": w.max_per_tile, "samples_per_pixel": w.samples,
                   "denoise_passes": w.denoise_passes, "frames": frames, "gi_mode": "tiled",
                   "l2": "flushed (256 MB write) before every timed frame; 8 rotating frames of inputs",
                   "parallelism": f"replicas{world}"},
        "e2e": {"value": round(e2e_value, 2), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": round(e2e_ms / args.steps, 4)},
        "gpu_launches": int(launches_timed),
        "roofline": roof,
        "kernels": kernels,
        "fast": fast,
        "atrous_staging": staging,
        "clocks": clock,
    }
    if rank == 0:
        result.update(neural_vs_plain(args, ds, sc, w, cfg, flush))
    if parity is not None:
        result["parity"], result["cpu_baseline"] = parity, cpu
    if rank == 0 and not args.no_uhd and w.name == S.HD.name:
        del ds
        result.update(uhd_comparison(args, flush))
    if rank == 0 and not args.no_batched and w.name == S.HD.name:
        result.update(batched_views(args, flush))
    st.close()
    st2.close()
    return result


def converged_targets(ds, sc, w, cfg, batches=64):
    """Converged GI per frame: sgi_gi_target with 64 batches of 8 samples (FP64 sums), seeded
    independently of the frames it judges. Returns (targets, ms per frame)."""
    import torch

    from stratusgfx_gb300 import stage
    tcfg = stage.workload_config(w, samples_per_pixel=8)
    st = stage.GiStage(tcfg)
    st.set_lights(ds.vpls, ds.entries, ds.points)
    frames = len(sc.cameras) - 1
    out = []
    ms = 0.0
    for k in range(1, frames + 1):
        st.set_shadow_maps(ds.csms[k], ds.cubes)
        cam = ds.camera(k)
        st.cull_vpls()
        st.cull_tiles(ds.gbuffers[k], cam)
        t = torch.empty((w.height, w.width, 4), dtype=torch.float32, device="cuda")
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        st.gi_target(ds.gbuffers[k], cam, 1000.0 + 16.0 * k + 7.0e6, batches, t)
        e1.record()
        torch.cuda.synchronize()
        ms += e0.elapsed_time(e1)
        out.append(t)
    st.close()
    return out, ms / frames


def psnr_vs_converged(render, ds, sc, w, cfg, targets):
    """Renders frames 1..8 in order with render(st, k, out) on a fresh context and returns the mean
    PSNR (dB) of the HDR frame against the converged frame screen + gi * target, and of the GI term
    alone (sgi_gi_error_stats: FP64 reductions on the device)."""
    import torch

    from stratusgfx_gb300 import stage
    st = stage.GiStage(cfg)
    st.set_lights(ds.vpls, ds.entries, ds.points)
    H, W = w.height, w.width
    out = torch.empty((H, W, 4), dtype=torch.float16, device="cuda")
    direct = torch.empty((H, W, 4), dtype=torch.float16, device="cuda")
    full, gi_only = [], []
    for k in range(1, len(targets) + 1):
        st.set_shadow_maps(ds.csms[k], ds.cubes)
        render(st, k, out)
        st.direct_lighting(ds.gbuffers[k], ds.camera(k), direct)
        es = stage.gi_error_stats(ds.gbuffers[k], out, direct, targets[k - 1])   # FP64 on the device
        full.append(es["psnr_frame"])
        gi_only.append(es["psnr_gi"])
    st.close()
    return round(sum(full) / len(full), 2), round(sum(gi_only) / len(gi_only), 2)


def _host_scene(ds, sc, w, frames):
    """The oracle's view of the device-generated inputs (copied to host) for the listed frames."""
    from oracle import binding as O
    g = [None] * len(ds.gbuffers)
    for k in frames:
        g[k] = ds.gbuffers[k].numpy()
    csm = {k: ds.csm_depth[k].cpu().numpy() for k in frames}
    return O.HostScene.from_arrays(sc, w, g, csm, ds.cube_storage.cpu().numpy())


def parity_and_cpu_baseline(ds, sc, w, cfg):
    """Frames 1 and 2 of the workload (the second reading the first's history) through the FP32 oracle,
    timed with all host threads (the CPU baseline), and through sgi_render_frame on a fresh context with
    the same inputs and frame parameters: the visible list, every per-tile list and the HDR output are
    compared, then frame 1 is compared with the FP64 oracle (PSNR). Frame 1 also runs through the oracle's
    operation-counting instantiation for the algorithmic FLOPs of each kernel."""
    import torch

    from oracle import binding as O
    from stratusgfx_gb300 import abi, stage
    hs = _host_scene(ds, sc, w, (0, 1, 2))
    H, W = w.height, w.width
    gi = np.zeros((H, W, 4), np.float32)
    hist = np.zeros((H, W), np.float32)
    refs = []
    t0 = time.perf_counter()
    for k in (1, 2):
        r = O.frame(32, cfg, hs, k, gi, hist, 1000.0 + 16.0 * k, 60.0)
        gi, hist = r["gi"], r["hist"]
        refs.append(r)
    # more frames for the timing alone (frames 1 and 2 again, the history carried on), about 10 s in all
    n_cpu = len(refs)
    while time.perf_counter() - t0 < CPU_SAMPLE_S and n_cpu < 64:
        k = 1 + n_cpu % 2
        r = O.frame(32, cfg, hs, k, gi, hist, 1000.0 + 16.0 * k, 60.0)
        gi, hist = r["gi"], r["hist"]
        n_cpu += 1
    dt = time.perf_counter() - t0
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    cpu = {"value": round(n_cpu * W * H / dt / 1e6, 4), "unit": UNIT, "cores": cores, "kind": "port",
           "sample": f"{n_cpu} full {W}x{H} frames of the same workload through the FP32 oracle (OpenMP), "
                     f"{dt:.1f} s"}
    st = stage.GiStage(cfg)
    st.set_lights(ds.vpls, ds.entries, ds.points)
    out = torch.empty((H, W, 4), dtype=torch.float16, device="cuda")
    L = cfg.max_vpls_per_tile
    lists_ok = vis_ok = True
    differ = 0
    max_rel = 0.0
    frame1 = None
    for k, ref in zip((1, 2), refs):
        st.set_shadow_maps(ds.csms[k], ds.cubes)
        st.render_frame(ds.gbuffers[k], ds.gbuffers[k - 1], ds.camera(k), out, 1000.0 + 16.0 * k, 60.0)
        torch.cuda.synchronize()
        idx = st.read_debug(abi.SGI_DEBUG_VISIBLE_INDEX, np.int32)
        cnt = ref["count"]
        vis_ok &= bool(idx[0] == cnt and np.array_equal(idx[1:1 + cnt], ref["visible_index"][1:1 + cnt]))
        lists = st.read_debug(abi.SGI_DEBUG_TILE_LISTS, np.int32).reshape(-1, 1 + L)
        lists_ok &= bool(np.array_equal(lists, ref["lists"]))
        got = out.cpu().numpy().astype(np.float32)[..., :3]
        exp = ref["combined"][..., :3].astype(np.float32)
        same = (got == exp) | (np.isnan(got) & np.isnan(exp))
        differ += int((~same).sum())
        ok = np.isfinite(got) & np.isfinite(exp)
        rel = np.abs(got[ok].astype(np.float64) - exp[ok]) / np.maximum(np.abs(exp[ok]), 1e-6)
        max_rel = max(max_rel, float(rel.max()) if rel.size else 0.0)
        if k == 1:
            frame1 = got.astype(np.float64)
    st.close()
    # the tolerance mode on the same two frames: identical lists, radiance within tolerance of the oracle
    stf = stage.GiStage(cfg)
    abi.check(stf.lib.sgi_set_shading_precision(stf.ctx, abi.SGI_SHADING_FAST), stf.ctx)
    stf.set_lights(ds.vpls, ds.entries, ds.points)
    f_lists_ok = True
    f_max_rel = 0.0
    f_over = 0
    fast1 = None
    for k, ref in zip((1, 2), refs):
        stf.set_shadow_maps(ds.csms[k], ds.cubes)
        stf.render_frame(ds.gbuffers[k], ds.gbuffers[k - 1], ds.camera(k), out, 1000.0 + 16.0 * k, 60.0)
        torch.cuda.synchronize()
        lists = stf.read_debug(abi.SGI_DEBUG_TILE_LISTS, np.int32).reshape(-1, 1 + L)
        f_lists_ok &= bool(np.array_equal(lists, ref["lists"]))
        got = out.cpu().numpy().astype(np.float64)[..., :3]
        exp = ref["combined"][..., :3].astype(np.float64)
        rel = np.abs(got - exp) / np.maximum(np.abs(exp), 2.0 ** -14)
        rel[np.isnan(got) & np.isnan(exp)] = 0.0
        f_max_rel = max(f_max_rel, float(np.nanmax(rel)))
        f_over += int((rel.max(axis=2) > 1e-3).sum())
        if k == 1:
            fast1 = got
    stf.close()
    t1 = time.perf_counter()
    r64 = O.frame(64, cfg, hs, 1, np.zeros((H, W, 4)), np.zeros((H, W)), 1016.0, 60.0)
    t64 = time.perf_counter() - t1
    ref64 = r64["combined"][..., :3]
    mse = float(np.mean((frame1 - ref64) ** 2))
    peak = float(np.max(np.abs(ref64)))
    t2 = time.perf_counter()
    fl = O.frame_flops(cfg, hs, 1, np.zeros((H, W, 4), np.float32), np.zeros((H, W), np.float32), 1016.0, 60.0)
    t_count = time.perf_counter() - t2
    parity = {"workload": w.name, "frames": 2, "visible_lists_equal": vis_ok, "tile_lists_equal": lists_ok,
              "tiles_per_frame": int(refs[0]["lists"].shape[0]), "hdr_bit_exact": differ == 0,
              "hdr_values_differing": differ, "max_rel_err_vs_fp32_oracle": max_rel,
              "psnr_vs_fp64_oracle_db": round(10.0 * np.log10(peak * peak / mse), 2) if mse > 0 else None,
              "fp64_oracle_frame_s": round(t64, 2),
              "oracle": "CPU restatement of the reference shaders (parity unpinned by the reference)",
              "fast": {"tile_lists_equal": f_lists_ok,
                       "max_rel_err_vs_fp32_oracle": f_max_rel,
                       "pixels_over_1e-3": f_over, "pixels": 2 * H * W,
                       "rel_err": "|gpu - oracle| / max(|oracle|, 2^-14) over the HDR frame after all passes",
                       "psnr_vs_fp64_oracle_db": round(10.0 * np.log10(peak * peak /
                                                                       float(np.mean((fast1 - ref64) ** 2))), 2)},
              "flop_count_s": round(t_count, 2)}
    return parity, cpu, fl


def time_frames(render, ds, frames, steps, warmup, flush):
    """Mean ms per frame of render(k) over `steps` frames (L2 flushed before each, outside the events)."""
    import torch
    for s in range(warmup):
        render(s % frames + 1, s)
    torch.cuda.synchronize()
    ms = 0.0
    for s in range(steps):
        flush.fill_(float(s))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        render((warmup + s) % frames + 1, warmup + s)
        e1.record()
        torch.cuda.synchronize()
        ms += e0.elapsed_time(e1)
    return ms / steps


def measure_runs(runs, res, net, ds, sc, w, targets, flush, steps):
    """For each (name, render, label, config overrides): ms/frame over `steps` frames (device-resident,
    L2 flushed) and PSNR of the HDR frame and of its GI term against the converged frames;
    res[name][label] receives the numbers. Names starting with "neural_fp8" run the U-Net in FP8."""
    import torch

    from stratusgfx_gb300 import abi, stage
    H, W = w.height, w.width
    frames = len(sc.cameras) - 1
    out = torch.empty((H, W, 4), dtype=torch.float16, device="cuda")
    for name, render, label, kw in runs:
        if net is not None:
            net.set_precision(abi.SGI_NN_FP8 if name.startswith("neural_fp8") else abi.SGI_NN_BF16)
        kcfg = stage.workload_config(w, **kw)
        st = stage.GiStage(kcfg)
        st.set_lights(ds.vpls, ds.entries, ds.points)

        def one(k, s, st=st, render=render):
            st.set_shadow_maps(ds.csms[k], ds.cubes)
            render(st, k, out)

        ms = time_frames(one, ds, frames, steps, 3, flush)
        st.close()
        p_full, p_gi = psnr_vs_converged(render, ds, sc, w, kcfg, targets)
        res.setdefault(name, {})[label] = {"ms_per_frame": round(ms, 4), "mpix_s": round(W * H / ms / 1e3, 1),
                                           "psnr_db": p_full, "psnr_gi_db": p_gi}


def render_fns(ds, net):
    """The plain and the neural frame of frame k into `out`, on context `st`."""
    import ctypes as C

    from stratusgfx_gb300 import abi, stage

    def plain_render(st, k, out):
        st.render_frame(ds.gbuffers[k], ds.gbuffers[k - 1], ds.camera(k), out, 1000.0 + 16.0 * k, 60.0)

    def neural_render(st, k, out):
        fp = abi.FrameParams(1000.0 + 16.0 * k, 60.0)
        abi.check(st.lib.sgi_render_frame_neural(st.ctx, net.h, C.byref(ds.gbuffers[k].struct()),
                                                 C.byref(ds.gbuffers[k - 1].struct()), C.byref(ds.camera(k)),
                                                 C.byref(fp), C.c_void_p(out.data_ptr()),
                                                 stage._stream_ptr(None)), st.ctx)
    return plain_render, neural_render


def uhd_comparison(args, flush):
    """3840x2160 with 4096 VPLs at K = 4: the plain a-trous frame, the BF16 U-Net frame and the FP8
    U-Net frame (scales calibrated on a frame of another room); ms/frame and PSNR against the
    converged (K = 512, FP64) frames."""
    from stratusgfx_gb300 import denoiser, stage
    from stratusgfx_gb300 import scene as S
    if not os.path.exists(denoiser.WEIGHTS):
        return {"uhd": {"unavailable": f"no trained weights at {denoiser.WEIGHTS}"}}
    w = S.UHD
    sc = S.workload_scene(w, 1234 + 4)
    ds = stage.DeviceScene(sc, w)
    cfg = stage.workload_config(w)
    targets, target_ms = converged_targets(ds, sc, w, cfg)
    net = denoiser.KpcnDenoiser(1, w.height, w.width)
    net.load(denoiser.WEIGHTS)
    calib = denoiser.make_dataset(1, H=w.height, W=w.width, frames_per_room=2, seed=778, samples=(2,), batches=1,
                                  log=lambda *a: None)
    net.calibrate_fp8(calib.feat[:1])
    del calib
    plain_render, neural_render = render_fns(ds, net)
    K = w.samples
    runs = [("plain", plain_render, f"K{K}", {}), ("neural_bf16", neural_render, f"K{K}", {}),
            ("neural_fp8", neural_render, f"K{K}", {})]
    # the FP8 network at fewer samples, for the equal-PSNR point at 4K
    runs += [("neural_fp8_low", neural_render, f"K{k}", dict(samples_per_pixel=k)) for k in (2, 1)]
    res = {}
    measure_runs(runs, res, net, ds, sc, w, targets, flush, max(6, args.steps // 4))
    net.close()
    out = {"workload": w.name, "resolution": f"{w.width}x{w.height}", "vpls": w.num_vpls,
           "cube": f"6x{w.cube_size}^2 fp16", "samples_per_pixel": K, "frames": len(sc.cameras) - 1}
    for name in ("plain", "neural_bf16", "neural_fp8"):
        out[name] = res[name][f"K{K}"]
    for k, v in res["neural_fp8_low"].items():
        out[f"neural_fp8_{k}"] = v
    plain = out["plain"]
    ok = [(v["ms_per_frame"], n) for n, v in out.items()
          if n.startswith("neural") and isinstance(v, dict) and v["psnr_gi_db"] >= plain["psnr_gi_db"]]
    if ok:
        best = min(ok)
        out["equal_psnr"] = {"plain_ms": plain["ms_per_frame"], "plain_gi_psnr_db": plain["psnr_gi_db"],
                             "neural_config": best[1], "neural_ms": best[0],
                             "neural_gain_gi_db": round(out[best[1]]["psnr_gi_db"] - plain["psnr_gi_db"], 2),
                             "speedup_at_equal_or_better_psnr": round(plain["ms_per_frame"] / best[0], 3)}
    out["converged_target"] = {"samples_per_pixel": 512, "accumulation": "fp64", "ms_per_frame": round(target_ms, 2)}
    return {"uhd": out}


def batched_views(args, flush):
    """64 views of uneven resolution (width and height log-uniform between 256x256 and 1920x1080) of 8
    seeded rooms, each view a context of its own. sgi_batch tunes every view's block shapes and captures a
    frame of every view - VPL and tile cull, K-sample gather, the plain a-trous or the FP8 U-Net - into one
    CUDA graph; one graph launch renders all 64. Reports views/s and Mpix/s of the graph, of the same
    frames issued view by view, and the mean GI PSNR of each path against the converged frames."""
    import ctypes as C

    import torch

    from stratusgfx_gb300 import abi, denoiser, stage
    from stratusgfx_gb300 import scene as S
    if not os.path.exists(denoiser.WEIGHTS):
        return {"batched": {"unavailable": f"no trained weights at {denoiser.WEIGHTS}"}}
    lib = abi.load()
    rng = np.random.default_rng(4242)
    n_views, n_rooms = 64, 8
    rooms, views = {}, []
    for i in range(n_views):
        t = rng.uniform()
        W = max(256, int(round(256 * (1920 / 256) ** t / 8)) * 8)
        H = max(256, int(round(256 * (1080 / 256) ** t / 8)) * 8)
        r = i % n_rooms
        w = S.Workload(f"view{i}_{W}x{H}", W, H, 40, 2048, 4, 2048, 128, abi.SGI_CUBE_F16, 8, 5, 1)
        sc = S.make_scene(6000 + r, W, H, w.num_boxes, w.num_vpls, 1, vpl_radius=w.vpl_radius,
                          num_points=w.num_points, csm_resolution=w.csm_resolution, camera_seed=7000 + i)
        if r not in rooms:
            rooms[r] = stage.DeviceScene(sc, w)
            vs = rooms[r]
        else:
            vs = stage.ViewScene(rooms[r], sc, w)
        tgt, _ = converged_targets(vs, sc, w, stage.workload_config(w))
        views.append((w, sc, vs, tgt[0]))
    total_px = sum(w.width * w.height for w, _, _, _ in views)
    net = denoiser.KpcnDenoiser(1, 1080, 1920)
    net.load(denoiser.WEIGHTS)
    calib = denoiser.make_dataset(1, H=1080, W=1920, frames_per_room=2, seed=779, samples=(2,), batches=1,
                                  log=lambda *a: None)
    net.calibrate_fp8(calib.feat[:1])
    del calib
    steps = max(6, args.steps // 4)
    res = {"views": n_views, "rooms": n_rooms, "resolutions": "log-uniform 256x256 .. 1920x1080",
           "total_mpix": round(total_px / 1e6, 2), "runs": {}}

    for name, K, nn in (("plain_K8", 8, None), ("plain_K8_persistent", 8, None), ("neural_fp8_K1", 1, net),
                        ("neural_fp8_K2", 2, net)):
        persistent = name.endswith("_persistent")
        if nn is not None:
            nn.set_precision(abi.SGI_NN_FP8)
        objs = []
        for w, sc, vs, tgt in views:
            st = stage.GiStage(stage.workload_config(w, samples_per_pixel=K))
            st.set_lights(vs.vpls, vs.entries, vs.points)
            st.set_shadow_maps(vs.csms[1], vs.cubes)
            o = dict(w=w, vs=vs, tgt=tgt, st=st, out=torch.empty((w.height, w.width, 4), dtype=torch.float16,
                                                                  device="cuda"),
                     cur=vs.gbuffers[1].struct(), prev=vs.gbuffers[0].struct(), cam=vs.camera(1))
            objs.append(o)

        def frame(o, t):
            fp = abi.FrameParams(t, 60.0)
            if nn is None:
                stt = lib.sgi_render_frame(o["st"].ctx, C.byref(o["cur"]), C.byref(o["prev"]), C.byref(o["cam"]),
                                           C.byref(fp), C.c_void_p(o["out"].data_ptr()), None)
            else:
                stt = lib.sgi_render_frame_neural(o["st"].ctx, nn.h, C.byref(o["cur"]), C.byref(o["prev"]),
                                                  C.byref(o["cam"]), C.byref(fp), C.c_void_p(o["out"].data_ptr()),
                                                  None)
            abi.check(stt, o["st"].ctx)

        # quality: four frames of each view with fresh sample seeds, GI term of the last against the target
        psnr = []
        for o in objs:
            for j in range(4):
                frame(o, 1000.0 + 16.0 * j)
            w = o["w"]
            direct = torch.empty((w.height, w.width, 4), dtype=torch.float16, device="cuda")
            o["st"].direct_lighting(o["vs"].gbuffers[1], o["cam"], direct)
            psnr.append(stage.gi_error_stats(o["vs"].gbuffers[1], o["out"], direct, o["tgt"])["psnr_gi"])
        # the same frames issued view by view
        ms_seq = 0.0
        for s in range(steps + 2):
            flush.fill_(float(s))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for o in objs:
                frame(o, 1016.0)
            e1.record()
            torch.cuda.synchronize()
            if s >= 2:
                ms_seq += e0.elapsed_time(e1)
        ms_seq /= steps
        # one graph launch per batch of 64 frames, block shapes tuned per view
        arr = (abi.View * n_views)(*[abi.View(o["st"].ctx.value, C.addressof(o["cur"]), C.addressof(o["prev"]),
                                              C.addressof(o["cam"]), abi.FrameParams(1016.0, 60.0),
                                              o["out"].data_ptr()) for o in objs])
        h = C.c_void_p()
        t0 = time.perf_counter()
        if persistent:   # one persistent kernel per batch, CTA count tuned over 2 frames
            stt = lib.sgi_batch_create_persistent(arr, n_views, 2, None, C.byref(h))
        else:
            stt = lib.sgi_batch_create(arr, n_views, nn.h if nn is not None else None, 2, None, C.byref(h))
        if stt != abi.SGI_OK:
            raise abi.SgiError(stt, f"sgi_batch_create: {lib.sgi_batch_last_error(h)}")
        build_s = time.perf_counter() - t0
        for s in range(3):
            abi.check(lib.sgi_batch_launch(h, None))
        torch.cuda.synchronize()
        ms_graph = 0.0
        for s in range(steps):
            flush.fill_(float(s))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            abi.check(lib.sgi_batch_launch(h, None))
            e1.record()
            torch.cuda.synchronize()
            ms_graph += e0.elapsed_time(e1)
        ms_graph /= steps
        abi.check(lib.sgi_batch_status(h))
        kernels = int(lib.sgi_batch_kernel_count(h))
        pshape = None
        if persistent:
            regs, ctas = C.c_int32(), C.c_int32()
            abi.check(lib.sgi_batch_persistent_shape(h, C.byref(regs), C.byref(ctas)))
            pshape = {"registers_per_thread": regs.value, "ctas": ctas.value}
        shapes = {}
        bx, by = C.c_int32(), C.c_int32()
        for o in objs:
            lib.sgi_get_block_shape(o["st"].ctx, abi.SGI_BLOCK_GATHER, C.byref(bx), C.byref(by))
            key = f"{bx.value}x{by.value}"
            shapes[key] = shapes.get(key, 0) + 1
        abi.check(lib.sgi_batch_destroy(h))
        for o in objs:
            o["st"].close()
        res["runs"][name] = {"ms_per_batch": round(ms_graph, 3), "views_s": round(n_views / ms_graph * 1e3, 1),
                             "mpix_s": round(total_px / ms_graph / 1e3, 1),
                             "view_by_view_ms": round(ms_seq, 3), "graph_speedup": round(ms_seq / ms_graph, 3),
                             "mean_gi_psnr_db": round(sum(psnr) / len(psnr), 2),
                             "kernels_per_launch": kernels,
                             "tuned": pshape if persistent else {"gather_blocks": shapes},
                             "tune_and_capture_s": round(build_s, 2)}
    net.close()
    plain = res["runs"]["plain_K8"]
    ok = [(v["ms_per_batch"], k) for k, v in res["runs"].items()
          if k.startswith("neural") and v["mean_gi_psnr_db"] >= plain["mean_gi_psnr_db"]]
    if ok:
        best = min(ok)
        res["matched_psnr"] = {"plain": "plain_K8", "neural": best[1],
                               "views_s_plain": plain["views_s"], "views_s_neural": res["runs"][best[1]]["views_s"],
                               "speedup": round(plain["ms_per_batch"] / best[0], 3)}
    else:
        res["matched_psnr"] = {"plain": "plain_K8", "neural": None}
    return {"batched": res}


# U-Net multiply-adds per pixel: 3x3 convolutions at full, half and quarter resolution
UNET_MACS_PER_PIXEL = 9 * (16 * 32 + 32 * 32 + 96 * 32 + 32 * 32 + 32 * 32) + \
    9 * (32 * 64 + 64 * 64 + 192 * 64 + 64 * 64) / 4 + 9 * (64 * 128 + 128 * 128) / 16


def unet_roofline(net, H, W, flush, iters=10):
    """The learned denoiser's forward pass (11 convolutions, upsampling, kernel apply) at H x W in BF16 and
    FP8: ms (CUDA events, L2 flushed before each), achieved dense TFLOP/s (2 x multiply-adds of the 3x3
    convolutions) and its fraction of the measured BF16 tensor peak (FP8: of twice that, the E4M3 rate)."""
    import torch

    from stratusgfx_gb300 import abi
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    bf16 = peaks.get("bf16_tflops") or 1900.0
    src = "measured" if peaks.get("bf16_tflops") else "fallback"
    g = torch.Generator(device="cpu").manual_seed(5)
    feat = torch.randn((1, H, W, 16), generator=g).clamp(-3, 3).to("cuda", torch.bfloat16)
    noisy = torch.rand((1, H, W, 4), generator=g).cuda()
    prev = torch.rand((1, H, W, 4), generator=g).cuda()
    out = torch.empty((1, H, W, 4), device="cuda")
    flops = 2.0 * UNET_MACS_PER_PIXEL * H * W
    res = {"flops_per_forward": flops, "peak_source": src}
    for name, prec, peak in (("bf16", abi.SGI_NN_BF16, bf16), ("fp8", abi.SGI_NN_FP8, 2.0 * bf16)):
        net.set_precision(prec)
        for _ in range(3):
            net.forward(feat, noisy, prev, out)
        torch.cuda.synchronize()
        ms = 0.0
        for i in range(iters):
            flush.fill_(float(i))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            net.forward(feat, noisy, prev, out)
            e1.record()
            torch.cuda.synchronize()
            ms += e0.elapsed_time(e1)
        ms /= iters
        tf = flops / (ms / 1e3) / 1e12
        res[name] = {"ms": round(ms, 4), "tflops": round(tf, 1), "peak_tflops": round(peak, 1),
                     "frac": round(tf / peak, 4)}
    net.set_precision(abi.SGI_NN_BF16)
    return res


def neural_vs_plain(args, ds, sc, w, cfg, flush):
    """The metric's comparison: plain a-trous at K = 8..64 against the learned denoiser at K = 8, 4, 2;
    ms/frame (device-resident) and PSNR against the converged frame (equal_psnr below)."""
    from stratusgfx_gb300 import denoiser
    if not os.path.exists(denoiser.WEIGHTS):
        return {"neural": {"unavailable": f"no trained weights at {denoiser.WEIGHTS}"}}
    targets, target_ms = converged_targets(ds, sc, w, cfg)
    H, W = w.height, w.width
    net = denoiser.KpcnDenoiser(1, H, W)
    net.load(denoiser.WEIGHTS)
    # FP8 scales calibrated on a frame of another room (seed 777), not on the measured frames
    calib = denoiser.make_dataset(1, H=H, W=W, frames_per_room=2, seed=777, samples=(2,), batches=1,
                                  log=lambda *a: None)
    net.calibrate_fp8(calib.feat[:1])
    del calib
    res = {"plain": {}, "neural": {}, "neural_fp8": {}}
    plain_render, neural_render = render_fns(ds, net)

    runs = [("plain", plain_render, f"K{K}", dict(samples_per_pixel=K)) for K in (8, 16, 32, 64)]
    runs += [("neural", neural_render, f"K{K}", dict(samples_per_pixel=K)) for K in (8, 4, 2, 1)]
    runs += [("neural_fp8", neural_render, f"K{K}", dict(samples_per_pixel=K)) for K in (8, 4, 2, 1)]
    measure_runs(runs, res, net, ds, sc, w, targets, flush, max(8, args.steps // 2))
    res["unet"] = unet_roofline(net, H, W, flush)
    net.close()
    # Equal PSNR. The plain path's quality saturates with K (the a-trous filter's bias, not
    # the sample count, bounds its error against the converged frame), so the comparison is:
    # the plain path at its best GI PSNR, reached by its cheapest K (within 0.1 dB), against
    # the fastest neural configuration whose GI PSNR is at least that high.
    best_plain = max(v["psnr_gi_db"] for v in res["plain"].values())
    plain_ref = min(((v["ms_per_frame"], k) for k, v in res["plain"].items() if v["psnr_gi_db"] >= best_plain - 0.1))
    eq = {"plain_best_gi_psnr_db": best_plain, "plain_config": plain_ref[1], "plain_ms": plain_ref[0],
          "plain_K8_gi_psnr_db": res["plain"]["K8"]["psnr_gi_db"], "plain_K8_ms": res["plain"]["K8"]["ms_per_frame"]}
    ok = [(v["ms_per_frame"], f"{n}_{k}") for n in ("neural", "neural_fp8") for k, v in res[n].items()
          if v["psnr_gi_db"] >= best_plain]
    if ok:
        nk = min(ok)[1]
        prec, kk = nk.rsplit("_", 1)
        eq.update({"neural_config": nk, "neural_ms": min(ok)[0],
                   "neural_gain_gi_db": round(res[prec][kk]["psnr_gi_db"] - best_plain, 2),
                   "speedup_at_equal_or_better_psnr": round(plain_ref[0] / min(ok)[0], 3)})
    else:
        eq["neural_config"] = None
    res["equal_psnr"] = eq
    res["converged_target"] = {"samples_per_pixel": 512, "accumulation": "fp64", "ms_per_frame": round(target_ms, 2)}
    return res


# ---------------------------------------------------- reference arm ----
def _mapped_libraries() -> list[str]:
    """Shared objects of this repository mapped into the process (from /proc/self/maps)."""
    out = set()
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                path = line.split()[-1] if len(line.split()) >= 6 else ""
                if path.startswith(ROOT) and path.endswith(".so"):
                    out.add(os.path.relpath(path, ROOT))
    except OSError:
        pass
    return sorted(out)


def run_reference(args):
    """The reference's path restated on the CPU (its GLSL needs an OpenGL driver, unavailable on this machine):
    FP32 oracle with all host threads, inputs from the oracle's CPU ray caster, one full frame per step
    and the same --steps / --warmup as the GPU arm. Nothing of the GPU library is loaded: the config
    comes from abi.config_defaults (Python), and the arm checks its own mappings before printing."""
    from oracle import binding as O
    from stratusgfx_gb300 import stage
    from stratusgfx_gb300 import scene as S
    w = workload(args.workload)
    sc = S.workload_scene(w, 1234 + 2)
    t0 = time.perf_counter()
    hs = O.HostScene(sc, w)
    gen_s = time.perf_counter() - t0
    cfg = stage.workload_config(w)
    H, W = w.height, w.width
    frames = len(sc.cameras) - 1
    gi = np.zeros((H, W, 4), np.float32)
    hist = np.zeros((H, W), np.float32)
    steps = max(1, args.steps)
    warm = max(0, args.warmup)
    for s in range(warm):
        k = s % frames + 1
        r = O.frame(32, cfg, hs, k, gi, hist, 1000.0 + 16.0 * s, 60.0)
        gi, hist = r["gi"], r["hist"]
    t0 = time.perf_counter()
    for s in range(steps):
        k = (warm + s) % frames + 1
        r = O.frame(32, cfg, hs, k, gi, hist, 1000.0 + 16.0 * s, 60.0)
        gi, hist = r["gi"], r["hist"]
    dt = time.perf_counter() - t0
    value = steps * W * H / dt / 1e6
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    libs = _mapped_libraries()
    if any("libsgi" in p for p in libs):
        raise RuntimeError(f"the reference arm mapped the GPU library: {libs}")
    return {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": warm,
            "ms_per_step": round(dt / steps * 1e3, 2), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": {"workload": w.name, "resolution": f"{W}x{H}", "gi_mode": "tiled",
                       "samples_per_pixel": w.samples, "denoise_passes": w.denoise_passes,
                       "vpls": w.num_vpls, "point_lights": w.num_points, "frames": frames},
            "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{steps} full {W}x{H} frames (one per step) through the FP32 CPU "
                                       f"restatement of the reference shaders; input generation {gen_s:.1f} s "
                                       f"untimed"},
            "native_libraries": libs,
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_profile_persistent(args):
    """Frames of 8 views (960x540, one 40-box room with 2048 VPLs, K = 8) through the persistent batch kernel
    (untuned shape), for kernel captures (about 1 GB on the device)."""
    import ctypes as C

    import torch

    from stratusgfx_gb300 import abi, stage
    from stratusgfx_gb300 import scene as S
    lib = abi.load()
    views = []
    room = None
    for i in range(8):
        w = S.Workload(f"view{i}_960x540", 960, 540, 40, 2048, 4, 2048, 128, abi.SGI_CUBE_F16, 8, 5, 1)
        sc = S.make_scene(1234 + 2, w.width, w.height, w.num_boxes, w.num_vpls, 1, num_points=w.num_points,
                          csm_resolution=w.csm_resolution, camera_seed=300 + i)
        vs = stage.DeviceScene(sc, w) if room is None else stage.ViewScene(room, sc, w)
        room = room or vs
        st = stage.GiStage(stage.workload_config(w))
        if args.fast:
            abi.check(lib.sgi_set_shading_precision(st.ctx, abi.SGI_SHADING_FAST), st.ctx)
        st.set_lights(vs.vpls, vs.entries, vs.points)
        st.set_shadow_maps(vs.csms[1], vs.cubes)
        out = torch.empty((w.height, w.width, 4), dtype=torch.float16, device="cuda")
        st.render_frame(vs.gbuffers[1], vs.gbuffers[0], vs.camera(1), out, 1016.0, 60.0)
        o = dict(st=st, out=out, cur=vs.gbuffers[1].struct(), prev=vs.gbuffers[0].struct(), cam=vs.camera(1), vs=vs)
        views.append(o)
    arr = (abi.View * len(views))(*[abi.View(o["st"].ctx.value, C.addressof(o["cur"]), C.addressof(o["prev"]),
                                             C.addressof(o["cam"]), abi.FrameParams(1032.0, 60.0),
                                             o["out"].data_ptr()) for o in views])
    h = C.c_void_p()
    abi.check(lib.sgi_batch_create_persistent(arr, len(views), 0, None, C.byref(h)))
    for _ in range(args.warmup + args.steps):
        abi.check(lib.sgi_batch_launch(h, None))
    torch.cuda.synchronize()
    abi.check(lib.sgi_batch_status(h))
    regs, ctas = C.c_int32(), C.c_int32()
    abi.check(lib.sgi_batch_persistent_shape(h, C.byref(regs), C.byref(ctas)))
    abi.check(lib.sgi_batch_destroy(h))
    print(json.dumps({"profile_case": "8 views 960x540 persistent" + (" fast" if args.fast else ""),
                      "launches": args.warmup + args.steps, "registers": regs.value, "ctas": ctas.value}))
    for o in views:
        o["st"].close()


def run_profile(args):
    """Frames of the workload only, for kernel captures (about 0.7 GB on the device)."""
    import torch

    from stratusgfx_gb300 import stage
    from stratusgfx_gb300 import scene as S
    if args.persistent:
        run_profile_persistent(args)
        return
    w = workload(args.workload)
    sc = S.make_scene(1234 + 2, w.width, w.height, w.num_boxes, w.num_vpls, 2, vpl_radius=w.vpl_radius,
                      num_points=w.num_points, csm_resolution=w.csm_resolution)
    ds = stage.DeviceScene(sc, w)
    spp = (1 if args.fp8 else 2) if args.neural else None
    st = stage.GiStage(stage.workload_config(w, samples_per_pixel=spp) if spp else stage.workload_config(w))
    from stratusgfx_gb300 import abi
    if args.fast:
        abi.check(st.lib.sgi_set_shading_precision(st.ctx, abi.SGI_SHADING_FAST), st.ctx)
    if args.atrous is not None:
        abi.check(st.lib.sgi_set_atrous_staging(st.ctx, {"direct": abi.SGI_ATROUS_DIRECT,
                                                         "staged": abi.SGI_ATROUS_STAGED}[args.atrous]), st.ctx)
    st.set_lights(ds.vpls, ds.entries, ds.points)
    out = torch.empty((w.height, w.width, 4), dtype=torch.float16, device="cuda")
    net = None
    if args.neural:
        import ctypes as C

        from stratusgfx_gb300 import abi, denoiser
        net = denoiser.KpcnDenoiser(1, w.height, w.width)
        net.load(denoiser.WEIGHTS)
        if args.fp8:
            calib = denoiser.make_dataset(1, H=w.height, W=w.width, frames_per_room=2, seed=777, samples=(2,),
                                          batches=1, log=lambda *a: None)
            net.calibrate_fp8(calib.feat[:1])
            net.set_precision(abi.SGI_NN_FP8)
            del calib
    for s in range(args.warmup + args.steps):
        k = s % 2 + 1
        st.set_shadow_maps(ds.csms[k], ds.cubes)
        if net is None:
            st.render_frame(ds.gbuffers[k], ds.gbuffers[k - 1], ds.camera(k), out, 1000.0 + 16.0 * s, 60.0)
        else:
            fp = abi.FrameParams(1000.0 + 16.0 * s, 60.0)
            abi.check(st.lib.sgi_render_frame_neural(st.ctx, net.h, C.byref(ds.gbuffers[k].struct()),
                                                     C.byref(ds.gbuffers[k - 1].struct()), C.byref(ds.camera(k)),
                                                     C.byref(fp), C.c_void_p(out.data_ptr()), None), st.ctx)
    torch.cuda.synchronize()
    if net is not None:
        net.close()
    print(json.dumps({"profile_case": w.name + ("_neural_fp8_k1" if args.fp8 else "_neural_k2" if net else "") +
                      ("_fast" if args.fast else ""),
                      "frames": args.warmup + args.steps,
                      "launches_per_frame": st.launch_count() // (args.warmup + args.steps)}))
    st.close()


def main():
    args = parse()
    if args.profile:
        from __graft_entry__ import build
        build()
        run_profile(args)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one process per GPU: relaunch under torch.distributed.run with N local ranks
        import socket
        with socket.socket() as sk:
            sk.bind(("127.0.0.1", 0))
            port = sk.getsockname()[1]
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
               "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + sys.argv[1:]
        sys.exit(subprocess.call(cmd))
    if world != args.gpus:
        sys.exit(f"bench.py: --gpus {args.gpus} but WORLD_SIZE is {world}")
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)))
        return
    from __graft_entry__ import build
    build()
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    res = run_ours(args, rank, world, local_rank)
    if rank == 0:
        print(json.dumps(res))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
