"""Benchmark: depth-map layered angular-spectrum CGH frames/s at 1920x1080.

Workload (one "step" = one frame): 1920x1080 uint8 intensity + uint8 depth
(seeded Gaussian-sum scenes), 32 depth layers over z in [0.30, 0.35] m, 8 um
pitch, 532 nm, per-pixel random phase (seeded SplitMix64 stream generated on
the device), 2x zero-padded angular-spectrum propagation on a 3840x2160
grid, symmetrization encoding to a real fringe; FP32 compute.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value      frames/s with inputs resident in HBM, CUDA events around each
           step on the launching stream; L2 flushed (512 MiB write) between
           timed steps, outside the events.
e2e        the same frames through oh_depthmap_generate_host from pinned
           host buffers on a stream of its own: the row pass reads the image
           and depth bytes from host memory and the output pass writes the
           fringe there (through the buffers' device mappings), wall clock
           per call.
roofline   the dominant kernel's device time (events around its launches on
           its stream) against the measured HBM peak.
cpu_baseline  the oracle port (numpy/scipy pocketfft, all host cores) on one
           whole frame.
--impl reference  times that CPU restatement of the reference's depth-map
           path (Calc_Holo_CPU + encoding_CPU) alone; the reference's own CPU
           code needs Qt and FFTW and cannot be built.
N > 1: one process per GPU (torchrun), independent frames per rank (weak
scaling), no collective on the data path; max of per-rank times.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "CGH frames/s at 1920×1080 vs plain GPU path at ≤1e-3 rel err; % roofline"
NX, NY, LAYERS, PAD = 1920, 1080, 32, 2
SCENE_SEED, PHASE_SEED = 2024, 77
WORKLOAD = ("depth-map layered angular-spectrum CGH 1920x1080, 32 layers z 0.30-0.35 m, 2x zero-padded "
            "3840x2160 FFT grid, per-pixel seeded random phase, symmetrization encoding, fp32")


def profile_figure(fname, kernel):
    """A per-launch figure of `kernel` from a JSON summary under profiles/
    (ncu captures), or None."""
    path = ROOT / "profiles" / fname
    if not path.exists():
        return None
    return json.loads(path.read_text()).get(kernel)


def compute_roofline(kernel, ms_per_launch, peaks):
    """Issue-side roofline of one kernel: warp instructions per launch (ncu,
    profiles/instructions.json) over its measured launch time, against the
    peak issue rate and the FMA and MUFU pipe rates measured by
    oh_measure_issue_peaks on this GPU."""
    inst = profile_figure("instructions.json", kernel)
    if not inst or not peaks or ms_per_launch <= 0:
        return {"kernel": kernel, "ms_per_launch": ms_per_launch, "instructions": None}
    s = ms_per_launch * 1e-3
    r = {"kernel": kernel, "ms_per_launch": ms_per_launch, "bound": "issue", "unit": "warp inst/s",
         "achieved": inst["warp_inst"] / s, "peak": peaks["ffma_warp_inst_per_s"], "peak_source": "measured"}
    r["frac"] = r["achieved"] / r["peak"]
    if inst.get("fma"):
        r["fma_pipe_frac"] = inst["fma"] / s / peaks["ffma_warp_inst_per_s"]
    if inst.get("xu"):
        r["mufu_frac"] = inst["xu"] * 32 / s / peaks["mufu_per_s"]
    return r


def load_bf16_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text()).get("bf16_tflops", 1900.0)), "measured"
    return 1900.0, "fallback"


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """SM clock and throttle reasons sampled while the timed region runs.

    Polls NVML through ctypes every 2 ms (reads only); falls back to
    nvidia-smi at 200 ms when NVML cannot be loaded."""
    # NVML clocks-event reason bits
    REASONS = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown", 0x20: "sw_thermal_slowdown", 0x4: "sw_power_cap"}

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.samples = []
        self.stop = None
        self.max_mhz = None
        self.proc = None

    def _nvml(self):
        import ctypes as C
        for name in ("libnvidia-ml.so.1", "libnvidia-ml.so"):
            try:
                lib = C.CDLL(name)
                break
            except OSError:
                lib = None
        if lib is None or lib.nvmlInit_v2() != 0:
            return None
        h = C.c_void_p()
        bus = None
        try:
            import torch
            pr = torch.cuda.get_device_properties(self.gpu)
            bus = "%08x:%02x:%02x.0" % (getattr(pr, "pci_domain_id"), getattr(pr, "pci_bus_id"),
                                        getattr(pr, "pci_device_id"))
        except Exception:
            bus = None
        if bus is None or lib.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), C.byref(h)) != 0:
            if lib.nvmlDeviceGetHandleByIndex_v2(self.gpu, C.byref(h)) != 0:
                return None
        return lib, h

    def __enter__(self):
        import threading
        import ctypes as C
        nv = self._nvml()
        if nv is not None:
            lib, h = nv
            mx = C.c_uint()
            if lib.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx)) == 0:
                self.max_mhz = mx.value
            self.stop = threading.Event()

            def run():
                clk = C.c_uint()
                rs = C.c_ulonglong()
                get_r = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                    lib.nvmlDeviceGetCurrentClocksThrottleReasons
                while not self.stop.is_set():
                    if lib.nvmlDeviceGetClockInfo(h, 1, C.byref(clk)) == 0 and get_r(h, C.byref(rs)) == 0:
                        self.samples.append((clk.value, rs.value))
                    time.sleep(0.002)
            self.thread = threading.Thread(target=run, daemon=True)
            self.thread.start()
            return self
        try:
            self.path = Path(tempfile.gettempdir()) / f"oh_clocks_{os.getpid()}.csv"
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=clocks.sm,clocks.max.sm,"
                                          "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                                          "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.stop is not None:
            self.stop.set()
            self.thread.join(timeout=2)
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()
            for ln in self.path.read_text().splitlines():
                f = [x.strip() for x in ln.split(",")]
                if len(f) >= 6 and f[0].replace(".", "").isdigit():
                    bits = sum(b for b, x in zip((0x8, 0x40, 0x20, 0x4), f[2:6]) if x.lower() == "active")
                    self.samples.append((float(f[0]), bits))
                    self.max_mhz = float(f[1]) if f[1].replace(".", "").isdigit() else self.max_mhz
            try:
                self.path.unlink()
            except Exception:
                pass

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": ["no samples"], "samples": 0}
        reasons = sorted({name for _, r in self.samples for bit, name in self.REASONS.items() if r & bit})
        return {"sm_mhz": statistics.median(c for c, _ in self.samples), "sm_max_mhz": self.max_mhz,
                "reasons": reasons, "samples": len(self.samples),
                "source": "nvml" if self.stop is not None else "nvidia-smi"}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_frame(img, depth, phase, workers=None, layers=None):
    """The oracle port on the host cores: the whole 32-layer frame (or the
    render entries in `layers`) plus the encode, float64 numpy/scipy
    pocketfft with `workers` threads.  Returns (seconds, fringe, field)."""
    from oracle import depthmap as odm
    workers = workers or os.cpu_count()
    p = odm.DMParams(pnx=NX, pny=NY, num_of_depth=LAYERS, pad=PAD)
    t0 = time.perf_counter()
    U = odm.calc_holo(img, depth, p, phase=phase, workers=workers, layers=layers)
    fringe, field = odm.encode_symmetrization(U, p, workers=workers, return_field=True)
    return time.perf_counter() - t0, fringe, field


CPU_SAMPLE = ("one whole 1920x1080 32-layer frame per step (all layers, 2x pad, encode), float64 numpy/scipy "
              "pocketfft with {w} threads; the reference's depth-map CPU code needs Qt and FFTW, so its "
              "line-by-line restatement (oracle/depthmap.py) runs")


def run_reference(args, world, rank):
    """--impl reference: the CPU restatement of the reference's depth-map path,
    whole frames.  Warm-up steps run one layer plus the encode (they only
    warm the FFT plans and caches); every timed step is a full frame."""
    if rank != 0:
        return
    from openholo_gb300 import scenes
    img, depth = scenes.depthmap_scene(SCENE_SEED, NY, NX)
    phase = scenes.seeded_phase(PHASE_SEED, NY, NX)
    cores = os.cpu_count()
    for _ in range(args.warmup):
        cpu_frame(img, depth, phase, workers=cores, layers=[LAYERS // 2])
    secs = []
    t_all = time.perf_counter()
    for _ in range(args.steps):
        secs.append(cpu_frame(img, depth, phase, workers=cores)[0])
    wall = time.perf_counter() - t_all
    fps = len(secs) / sum(secs)
    line = {"metric": METRIC, "value": fps, "unit": "frames/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 / fps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD.replace("fp32", "float64 CPU"), "pnx": NX, "pny": NY, "layers": LAYERS,
                       "pad": PAD},
            "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": cores, "kind": "port",
                             "sample": CPU_SAMPLE.format(w=cores) + "; warm-up steps: one layer + encode"},
            "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "timed_region_s": wall, "frame_s": {"min": min(secs), "max": max(secs)}}
    print(json.dumps(line), flush=True)


def reconstruct_intensity(fringe, z, lam=532e-9, pitch=8e-6):
    """Numerical reconstruction used for PSNR: the real fringe propagated by
    the angular spectrum over +z (back to a layer plane; the frame was formed
    with d = -z), intensity |U|^2, float64 numpy on the host."""
    ny, nx = fringe.shape
    fx = np.fft.fftfreq(nx, pitch)
    fy = np.fft.fftfreq(ny, pitch)
    s = 1.0 - (lam * fx[None, :]) ** 2 - (lam * fy[:, None]) ** 2
    H = np.exp(1j * (2 * math.pi / lam) * z * np.sqrt(np.maximum(s, 0.0)))
    u = np.fft.ifft2(np.fft.fft2(fringe.astype(np.float64)) * H)
    return np.abs(u) ** 2


def error_report(got_fringe, got_field, ref_fringe, ref_field, focus_z=(0.30, 0.325, 0.35)):
    """Max and RMS complex error of the field, relative L2 of field and fringe
    against the FP64 oracle, and the reconstruction PSNR (intensities
    normalised by the oracle reconstruction's maximum) at the nearest, middle
    and farthest layer depths."""
    d = got_field.astype(np.complex128) - ref_field
    scale = np.abs(ref_field).max()
    rep = {"field_rel_l2": float(np.linalg.norm(d) / np.linalg.norm(ref_field)),
           "field_max_abs": float(np.abs(d).max()), "field_max_abs_rel": float(np.abs(d).max() / scale),
           "field_rms": float(np.sqrt(np.mean(np.abs(d) ** 2))),
           "field_rms_rel": float(np.sqrt(np.mean(np.abs(d) ** 2)) / np.sqrt(np.mean(np.abs(ref_field) ** 2))),
           "fringe_rel_l2": float(np.linalg.norm(got_fringe.astype(np.float64) - ref_fringe) /
                                  np.linalg.norm(ref_fringe))}
    ps = {}
    for z in focus_z:
        a = reconstruct_intensity(got_fringe, z)
        b = reconstruct_intensity(ref_fringe, z)
        m = b.max()
        mse = float(np.mean((a / m - b / m) ** 2))
        ps[f"{z:.3f}"] = 10 * math.log10(1.0 / mse) if mse > 0 else float("inf")
    rep["psnr_db"] = ps
    rep["psnr_db_min"] = min(ps.values())
    return rep


def plain_gpu_path(img_t, depth_t, zt, lut, torch):
    """The reference's per-layer structure (mask kernel, centred FFT, AS
    multiply-accumulate, crop, centred IFFT, shift phase, real part) in FP32
    with cuFFT C2C (torch.fft, plans cached) and transfer functions
    precomputed once in FP64.  Comparison baseline only."""
    dev = img_t.device
    Px, Py = PAD * NX, PAD * NY
    ox, oy = (Px - NX) // 2, (Py - NY) // 2
    lam, pp = 532e-9, 8e-6
    k = 2 * math.pi / lam
    ssx, ssy = Px * pp, Py * pp
    x = torch.arange(Px, device=dev, dtype=torch.float64)
    y = torch.arange(Py, device=dev, dtype=torch.float64)
    fx = (-1.0 / (2 * pp)) + x / ssx
    fy = (1.0 / (2 * pp)) - 1.0 / ssy - y / ssy
    s = torch.sqrt(1 - (lam * fx[None, :]) ** 2 - (lam * fy[:, None]) ** 2)
    H = []
    for z in zt:
        ph = torch.remainder(k * (-z) * s + k * z, 2 * math.pi)     # carrier folded in (FP64)
        H.append(torch.polar(torch.ones_like(ph), ph).to(torch.complex64))
    from openholo_gb300 import scenes
    ph0 = torch.from_numpy(scenes.seeded_phase(PHASE_SEED, NY, NX)).to(dev)
    src = (img_t.to(torch.float32) / 255.0) * torch.polar(torch.ones_like(ph0), ph0)
    layer_idx = torch.from_numpy(lut.astype(np.int64)).to(dev)[depth_t.long()]
    cx1, cx2, cy1, cy2 = 0, Px - 1, Py // 2 - (Py // 2) // 2 - 1, Py // 2 - (Py // 2) // 2 - 1 + Py // 2 - 1
    r = torch.arange(NY, device=dev, dtype=torch.float64)
    yy = NY * pp / 2.0 - pp * r - pp
    shy = torch.polar(torch.ones_like(yy), 2 * math.pi * (yy / (4 * pp))).to(torch.complex64)
    u = torch.zeros((Py, Px), dtype=torch.complex64, device=dev)

    def frame():
        U = torch.zeros((Py, Px), dtype=torch.complex64, device=dev)
        for li in range(LAYERS):
            u.zero_()
            u[oy:oy + NY, ox:ox + NX] = torch.where(layer_idx == li + 1, src, 0)
            S = torch.fft.fftshift(torch.fft.fft2(torch.fft.fftshift(u)))
            U += H[li] * S
        Uc = torch.zeros_like(U)
        Uc[cy1:cy2 + 1, cx1:cx2 + 1] = U[cy1:cy2 + 1, cx1:cx2 + 1]
        h = torch.fft.fftshift(torch.fft.ifft2(torch.fft.fftshift(Uc)))[oy:oy + NY, ox:ox + NX]
        return (h * shy[:, None]).real
    return frame


SECONDARY_OPS = ("pointcloud", "pls", "wrp", "batch", "square", "unet")
UNET_SIDE, UNET_SAMPLES, UNET_BATCH, UNET_LR, UNET_ZMID = 1024, 20000, 4, 1e-3, 0.325
SQUARE_SIDE, SQUARE_LAYERS = 2048, 16     # --op square: the batch's largest frame shape


def secondary_measurements(ctx, dev, torch, reps=5, ops=SECONDARY_OPS, warmup=1, peaks=None,
                           samples=UNET_SAMPLES, batch_frames=None, batch_tune=True):
    """The other operators at their own workloads (seeded synthetic inputs):
    pointcloud: KETI exact-r sum 1024x1024 x 5000 points + phase-only encoding;
    pls: the same shape through the paraxial cwoPLS::Fresnel sum (tensor-core
    and CUDA-core engines); wrp: WRP (200,000 points, 64x64 windows) +
    zero-padded Fresnel propagation to 3840x2160 at 3.74 um + phase-only
    encoding.  Each is timed over `reps` calls after `warmup` calls."""
    import ctypes as C
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    out = {}

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    n, nx, ny = 5000, 1024, 1024
    if "pointcloud" in ops:
        _sec_pointcloud(ctx, dev, torch, st, timed, out, n, nx, ny, peaks)
    if "pls" in ops:
        _sec_pls(ctx, dev, torch, st, timed, out, n, nx, ny, reps + warmup, peaks)
    if "wrp" in ops:
        _sec_wrp(ctx, dev, torch, st, timed, out, reps + warmup, peaks)
    if "batch" in ops:
        _sec_batch(ctx, dev, torch, out, reps, warmup, batch_frames, batch_tune)
    if "square" in ops:
        _sec_square(ctx, dev, torch, timed, out)
    if "unet" in ops:
        _sec_unet(ctx, dev, torch, timed, out, samples)
    return out


def unet_fwd_flops(side):
    """Forward FLOPs of one side x side frame through the U-Net (multiply-adds
    x 2, the first layer's 4 input channels padded to 32 as computed)."""
    from openholo_gb300 import surrogate
    f = 0
    for name, cin, cout, taps in surrogate.layer_shapes():
        lvl = int(name[3]) if name[:3] in ("enc", "dec") else 0
        f += 2 * (side >> lvl) ** 2 * taps * (32 if cin == 4 else cin) * cout
    return f


def _sec_unet(ctx, dev, torch, timed, out, samples):
    """The learned form: a U-Net (32/64/128/256 channels, 3x3 convolutions,
    BF16, FP32 accumulation, all convolutions on the tensor cores) trained on
    the GPU on `samples` seeded 1024x1024 RGB-D frames against the plain
    method's mid-plane field (32 layers over 0.30-0.35 m, mid plane 0.325 m,
    2x pad), then evaluated on 32 held-out frames with the 40 dB PSNR gate."""
    from openholo_gb300 import depthmap as dm, surrogate
    side, B = UNET_SIDE, UNET_BATCH
    p = dm.make_params(pnx=side, pny=side, num_of_depth=32, pad=2)
    lut, _ = dm.levels(p)
    dl = np.where(lut > 0, (lut - 1) / 31.0, 0.0).astype(np.float32)
    probe = surrogate.scenes_rgbd(ctx, 10 ** 6, 1, side, side)[0]
    rms = float(torch.sqrt((surrogate.mid_field(ctx, p, UNET_ZMID, probe).abs() ** 2).mean()))
    net = surrogate.UNet(ctx, max_batch=B, max_height=side, max_width=side, seed=1, out_scale=rms, depth_lut=dl)
    try:
        # training throughput of the step alone (fixed batch)
        x = surrogate.scenes_rgbd(ctx, 5, B, side, side)
        tg = torch.zeros((B, side, side, 2), dtype=torch.float32, device=dev)
        step_ms = timed(lambda: net.train_step(x, tg, 0.0))
        f1 = unet_fwd_flops(side)
        res = {"train_step_ms_batch4": step_ms, "train_samples_per_s": B * 1000.0 / step_ms,
               "fwd_gflop_per_frame": f1 / 1e9, "train_tflops": 3 * f1 * B / (step_ms * 1e-3) / 1e12,
               "train_kernels_ms": kernel_breakdown(ctx, torch, lambda: net.train_step(x, tg, 0.0), calls=2)}
        bf16, kind = load_bf16_peak()
        res["roofline"] = {"bound": "tensor", "unit": "TFLOP/s", "achieved": res["train_tflops"], "peak": bf16,
                           "frac": res["train_tflops"] / bf16, "peak_source": kind,
                           "what": "forward + input-gradient + weight-gradient convolutions (3 x forward FLOPs) per "
                                   "training step time"}
        net.set_params(net.get_params())     # fresh Adam state for the real run
        t0 = time.perf_counter()
        losses = surrogate.train(ctx, net, p, UNET_ZMID, samples, B, UNET_LR, seed=1000)
        torch.cuda.synchronize()
        res["training"] = {"samples": samples, "batch": B, "lr": UNET_LR, "seconds": time.perf_counter() - t0,
                           "loss_first": float(np.mean(losses[:10])), "loss_last": float(np.mean(losses[-10:])),
                           "what": "each sample a fresh seeded scene, target generated on the GPU by the plain "
                                   "method inside the timed loop"}
        # held-out evaluation with the 40 dB gate
        reps = []
        for s in range(32):
            r = surrogate.scenes_rgbd(ctx, 9 * 10 ** 6 + s, 1, side, side)[0]
            reps.append(surrogate.generate(ctx, net, p, UNET_ZMID, r, check=True, psnr_threshold_db=40.0)[1])
        ps = [r["psnr_db"] for r in reps]
        res["accuracy"] = {"psnr_db_mean": float(np.mean(ps)), "psnr_db_min": float(np.min(ps)),
                           "psnr_db_max": float(np.max(ps)), "rel_err_mean": float(np.mean([r["rel_err"] for r in reps])),
                           "max_abs_err_mean": float(np.mean([r["max_abs_err"] for r in reps])),
                           "rms_err_mean": float(np.mean([r["rms_err"] for r in reps])),
                           "fallbacks": int(sum(r["fell_back"] for r in reps)), "frames": len(reps),
                           "threshold_db": 40.0,
                           "what": "mid-plane intensity PSNR of the prediction against the plain method (peak = "
                                   "max plain intensity); complex errors relative to the plain field"}
        # throughput: surrogate alone, surrogate judged on every frame, plain frame
        r = surrogate.scenes_rgbd(ctx, 9 * 10 ** 6, 1, side, side)[0]
        fr = torch.empty((side, side), dtype=torch.float32, device=dev)
        ms_sg = timed(lambda: surrogate.generate(ctx, net, p, UNET_ZMID, r, check=False, fringe=fr))
        ms_chk = timed(lambda: surrogate.generate(ctx, net, p, UNET_ZMID, r, check=True, fringe=fr))
        g, d = r[..., 1].contiguous(), r[..., 3].contiguous()
        ms_plain = timed(lambda: dm.generate(ctx, p, g, d, fringe=fr))
        res["frames_per_s"] = {"surrogate": 1000.0 / ms_sg, "surrogate_checked_every_frame": 1000.0 / ms_chk,
                               "plain_method": 1000.0 / ms_plain}
        res["what"] = ("1024x1024 RGB-D -> U-Net mid-plane field -> angular-spectrum propagation over 0.325 m, "
                       "2x pad, symmetrization encoding; plain method: the same frame's 32 layers")
        out["unet_surrogate_1024"] = res
    finally:
        net.close()


def _sec_square(ctx, dev, torch, timed, out):
    """One square depth-map frame of the batch workload's largest shape
    (2048 x 2048, 16 layers, 2x pad: a 4096 x 4096 FFT grid), seeded scene."""
    from openholo_gb300 import depthmap as dm, scenes
    side, L = SQUARE_SIDE, SQUARE_LAYERS
    img, depth = scenes.depthmap_scene(5, side, side)
    p = dm.make_params(pnx=side, pny=side, num_of_depth=L, pad=2, phase_mode=dm.OH_PHASE_SEEDED, seed=3)
    ti, td = torch.from_numpy(img).to(dev), torch.from_numpy(depth).to(dev)
    fr = torch.empty((side, side), dtype=torch.float32, device=dev)
    ms = timed(lambda: dm.generate(ctx, p, ti, td, fringe=fr))
    npad = (2 * side) ** 2
    model = L * 32 * npad + 32 * npad + 2 * side * side        # the frame's HBM model, as for the headline frame
    peak, src = load_peaks()
    gbs = model / (ms * 1e-3) / 1e9
    out[f"depthmap_{side}x{side}_L{L}"] = {
        "ms_per_frame": ms, "frames_per_s": 1000.0 / ms,
        "roofline": {"bound": "hbm", "unit": "GB/s", "achieved": gbs, "peak": peak, "frac": gbs / peak,
                     "peak_source": src, "algorithmic_bytes_per_frame": model,
                     "what": "model bytes (L*32*Np + 32*Np + 2N) per frame time; the kernels skip the zero padding"},
        "what": "one frame of the batch workload's largest shape, 2x pad"}


def batch_workload():
    from openholo_gb300 import scenes
    return scenes.batch_workload()


def _sec_batch(ctx, dev, torch, out, reps, warmup, nframes=None, tune=True):
    from openholo_gb300 import depthmap as dm, launch_count, scenes
    work = batch_workload()[:nframes]
    scene = {}
    frames = []
    for i, (side, L, lam) in enumerate(work):
        if side not in scene:
            img, depth = scenes.depthmap_scene(scenes.BATCH_SCENE_SEED + side, side, side)
            scene[side] = (torch.from_numpy(img).to(dev), torch.from_numpy(depth).to(dev))
        p = dm.make_params(pnx=side, pny=side, num_of_depth=L, lam=lam, pad=2, phase_mode=dm.OH_PHASE_SEEDED,
                           seed=scenes.BATCH_PHASE_SEED + i)
        frames.append((p, scene[side][0], scene[side][1],
                       torch.empty((side, side), dtype=torch.float32, device=dev)))
    model = sum(L * 32 * (2 * side) ** 2 + 32 * (2 * side) ** 2 + 2 * side * side for side, L, _ in work)
    stream = torch.cuda.Stream(device=dev)

    def run(persistent):
        from openholo_gb300 import _lib
        _lib.call("oh_ctx_set_depthmap_batch_mode", ctx.handle, persistent)
        with torch.cuda.stream(stream):
            for _ in range(max(2, warmup)):
                dm.generate_batch(ctx, frames, graph=True)
            stream.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            n0 = launch_count()
            a.record(stream)
            for _ in range(reps):
                dm.generate_batch(ctx, frames, graph=True)
            b.record(stream)
            stream.synchronize()
        _lib.call("oh_ctx_set_depthmap_batch_mode", ctx.handle, 1)
        return a.elapsed_time(b) / reps, (launch_count() - n0) / reps

    ms_pf, k_pf = run(0)
    tune_s = None
    if tune:
        with torch.cuda.stream(stream):
            t0 = time.perf_counter()
            dm.autotune_batch(ctx, frames, reps=2, stream=stream)
            stream.synchronize()
            tune_s = time.perf_counter() - t0
    ms, kernels = run(1)
    peak_bw, peak_src = load_peaks()
    out["batch_64_frames_mixed_per_frame_launches"] = {
        "ms_per_batch": ms_pf, "frames_per_s": len(work) * 1000.0 / ms_pf, "kernels_per_batch": k_pf,
        "roofline": {"bound": "hbm", "unit": "GB/s", "achieved": model / (ms_pf * 1e-3) / 1e9, "peak": peak_bw,
                     "frac": model / (ms_pf * 1e-3) / 1e9 / peak_bw, "peak_source": peak_src,
                     "what": "the batch's model bytes per batch time, as for the persistent kernel"},
        "what": "the same batch as per-frame launches (set-up, row, column and output pass per frame) replayed "
                "from one CUDA graph"}
    out["batch_64_frames_mixed"] = {
        "frames": len(work),
        "ms_per_batch": ms, "frames_per_s": len(work) * 1000.0 / ms,
        "model_bytes_per_batch": model, "model_gbs": model / (ms * 1e-3) / 1e9,
        "kernels_per_batch": kernels,
        "autotune": {"seconds": tune_s, **{str(n): dm.batch_tuning(ctx, n) for n in (1024, 1536, 2048, 3072, 4096)}},
        "roofline": {"bound": "hbm", "unit": "GB/s", "achieved": model / (ms * 1e-3) / 1e9,
                     "peak": load_peaks()[0], "frac": model / (ms * 1e-3) / 1e9 / load_peaks()[0],
                     "peak_source": load_peaks()[1],
                     "what": "model bytes (the reference pipeline's FFT passes over the padded grid) per batch "
                             "time; the kernels skip the zero padding and empty rows, so the model can exceed "
                             "the bytes they move"},
        "what": "64 depth-map frames, one launch of the persistent batch kernel replayed from a CUDA graph: "
                "side 512-2048 px, 8-64 layers, 450/532/633 nm, 2x pad, FP32; model bytes = sum over frames of "
                "L*32*Np + 32*Np + 2N"}


def gpu_error_report(got, ref, torch, pitch, lam, z):
    """Field errors of `got` against the FP64 `ref` (device tensors): relative
    L2, max and RMS complex error (relative to max |ref| and RMS |ref|), and
    the PSNR of the angular-spectrum reconstruction at distance z
    (intensities normalised by the reference reconstruction's maximum),
    computed in float64 with torch.fft."""
    g = got.to(torch.complex128)
    d = g - ref
    rep = {"rel_l2": float(torch.linalg.norm(d) / torch.linalg.norm(ref)),
           "max_abs_rel": float(d.abs().max() / ref.abs().max()),
           "rms_rel": float(torch.sqrt((d.abs() ** 2).mean()) / torch.sqrt((ref.abs() ** 2).mean()))}
    ny, nx = ref.shape
    fx = torch.fft.fftfreq(nx, pitch, dtype=torch.float64, device=ref.device)
    fy = torch.fft.fftfreq(ny, pitch, dtype=torch.float64, device=ref.device)
    sq = torch.sqrt(torch.clamp(1.0 - (lam * fx[None, :]) ** 2 - (lam * fy[:, None]) ** 2, min=0.0))
    H = torch.polar(torch.ones_like(sq), (2 * math.pi / lam) * z * sq)
    ia = torch.fft.ifft2(torch.fft.fft2(g) * H).abs() ** 2
    ib = torch.fft.ifft2(torch.fft.fft2(ref) * H).abs() ** 2
    m = ib.max()
    mse = float(((ia - ib) / m).pow(2).mean())
    rep["psnr_db"] = 10 * math.log10(1.0 / mse) if mse > 0 else float("inf")
    rep["psnr_plane_z"] = z
    return rep


def _sec_pointcloud(ctx, dev, torch, st, timed, out, n, nx, ny, peaks=None):
    import ctypes as C
    from openholo_gb300 import _lib, scenes
    pts_np = scenes.pointcloud_scene(11, n).astype(np.float32)
    pts = torch.from_numpy(pts_np).to(dev)
    p = _lib.PcParams(1.0, 1.0, 1.0, 0.0, 8e-6, 8e-6, nx, ny, 532e-9, 0.0, 0.0)
    f32 = torch.empty((ny, nx), dtype=torch.complex64, device=dev)
    u8 = torch.empty((ny, nx), dtype=torch.uint8, device=dev)

    def pc():
        _lib.call("oh_pointcloud", ctx.handle, 0, C.byref(p), C.c_void_p(pts.data_ptr()), n,
                  C.c_void_p(f32.data_ptr()), None, st)
        _lib.call("oh_encode", ctx.handle, 0, 9, nx, ny, C.c_void_p(f32.data_ptr()), C.c_void_p(u8.data_ptr()), st)
    ms = timed(pc)
    kms = kernel_breakdown(ctx, torch, pc)
    f64 = torch.empty((ny, nx), dtype=torch.complex128, device=dev)
    _lib.call("oh_pointcloud", ctx.handle, 1, C.byref(p), C.c_void_p(pts.data_ptr()), n,
              C.c_void_p(f64.data_ptr()), None, st)
    torch.cuda.synchronize()
    acc = gpu_error_report(f32, f64, torch, 8e-6, 532e-9, -float(np.mean(pts_np[:, 2])))
    acc["reference"] = "the FP64 path (equal to the CPU oracle to 1e-9 in the tests)"
    res = {"ms_per_hologram": ms, "holograms_per_s": 1000.0 / ms,
           "point_pixel_terms_per_s": n * nx * ny / (ms / 1000.0), "kernels_ms": kms,
           "rel_err_vs_fp64": acc["rel_l2"], "accuracy": acc, "dtype": "f32 (FP64-reduced phase tables)"}
    t_direct = kms.get("pc_direct_f32")
    if peaks and t_direct:
        mufu = 3.0 * n * nx * ny          # per term: sqrt.approx, rcp.approx, sin.approx
        res["roofline"] = {"bound": "mufu", "kernel": "pc_direct_f32", "unit": "MUFU results/s",
                           "achieved": mufu / (t_direct * 1e-3), "peak": peaks["mufu_per_s"],
                           "frac": mufu / (t_direct * 1e-3) / peaks["mufu_per_s"], "peak_source": "measured",
                           "algorithmic_per_launch": mufu,
                           "issue": compute_roofline("pc_direct_f32", t_direct, peaks)}
    out["pointcloud_1024x1024_5000pts"] = res
    del f64


def kernel_breakdown(ctx, torch, fn, calls=5):
    """Per-kernel milliseconds per call, from the library's stream events, in
    a separate pass (the timed pass above runs with these events off)."""
    torch.cuda.synchronize()
    ctx.set_timing(True)
    ctx.read_timing(reset=True)
    for _ in range(calls):
        fn()
    torch.cuda.synchronize()
    kt = ctx.read_timing(reset=True)
    ctx.set_timing(False)
    return {k: v[0] / calls for k, v in kt.items()}


def _sec_pls(ctx, dev, torch, st, timed, out, n, nx, ny, calls, peaks=None):
    import ctypes as C
    from openholo_gb300 import _lib, scenes
    pls_pts = torch.from_numpy(scenes.pls_scene(11, n)).to(dev)
    pls_out = torch.empty((ny, nx), dtype=torch.complex64, device=dev)
    pls_res = {}
    for eng_name, eng in (("tensor", _lib.PLS_ENGINE_TENSOR), ("cuda_core_gemm", _lib.PLS_ENGINE_GEMM)):
        pp = _lib.PlsParams(nx, ny, 8e-6, 8e-6, 0.0, 0.0, 0.0, 0.0, 532e-9, 0.0, 0.0, _lib.PLS_FRESNEL, 1, eng)

        def pls_frame(pp=pp):
            _lib.call("oh_pls", ctx.handle, 0, C.byref(pp), C.c_void_p(pls_pts.data_ptr()), n,
                      C.c_void_p(pls_out.data_ptr()), st)
        ms_p = timed(pls_frame)
        pls_res[eng_name] = {"ms_per_hologram": ms_p, "kernels_ms": kernel_breakdown(ctx, torch, pls_frame)}
    tc_ms = pls_res["tensor"]["kernels_ms"].get("pls_tc_gemm")
    if tc_ms:
        useful = 8.0 * nx * ny * n          # complex multiply-adds as real flops, counted once
        pls_res["tensor"]["gemm_useful_tflops"] = useful / (tc_ms * 1e-3) / 1e12
        pls_res["tensor"]["gemm_issued_tflops"] = 3 * 2.0 * ny * (2 * nx) * (2 * n) / (tc_ms * 1e-3) / 1e12
        bf16, kind = load_bf16_peak()
        pls_res["roofline"] = {"bound": "tensor", "kernel": "pls_tc_gemm", "unit": "TFLOP/s",
                               "achieved": pls_res["tensor"]["gemm_issued_tflops"], "peak": bf16,
                               "frac": pls_res["tensor"]["gemm_issued_tflops"] / bf16, "peak_source": kind,
                               "what": "issued BF16 flops (three split products of the real embedding)"}
    out["pls_fresnel_1024x1024_5000pts"] = pls_res
    del pls_out


def _sec_wrp(ctx, dev, torch, st, timed, out, calls, peaks=None):
    import ctypes as C
    from openholo_gb300 import _lib, scenes
    npts, hx, hy, dp, lam = 200_000, 3840, 2160, 3.74e-6, 532e-9
    xyz = scenes.wrp_scene(12, npts)
    z_wrp = float(xyz[:, 2].min()) - 5e-3
    t_xyz = torch.from_numpy(xyz).to(dev)
    wrp = torch.zeros((hy, hx), dtype=torch.complex64, device=dev)
    hol = torch.empty((hy, hx), dtype=torch.uint8, device=dev)
    wp = _lib.WrpParams(hx, hy, dp, lam, z_wrp, 32)

    def wrp_frame():
        wrp.zero_()
        _lib.call("oh_wrp_accumulate", ctx.handle, 0, C.byref(wp), C.c_void_p(t_xyz.data_ptr()), npts,
                  C.c_void_p(wrp.data_ptr()), st)
        _lib.call("oh_fresnel_propagate", ctx.handle, 0, hx, hy, dp, lam, z_wrp, C.c_void_p(wrp.data_ptr()), st)
        _lib.call("oh_encode", ctx.handle, 0, 9, hx, hy, C.c_void_p(wrp.data_ptr()), C.c_void_p(hol.data_ptr()), st)
    ms3 = timed(wrp_frame)
    kms = kernel_breakdown(ctx, torch, wrp_frame)
    res = {"ms_per_hologram": ms3, "holograms_per_s": 1000.0 / ms3, "kernels_ms": kms, "dtype": "f32"}
    # accuracy of the propagated hologram field against the FP64 path (WRP and
    # padded-grid Fresnel in double; both equal the CPU oracle in the tests)
    w64 = torch.zeros((hy, hx), dtype=torch.complex128, device=dev)
    _lib.call("oh_wrp_accumulate", ctx.handle, 1, C.byref(wp), C.c_void_p(t_xyz.data_ptr()), npts,
              C.c_void_p(w64.data_ptr()), st)
    _lib.call("oh_fresnel_propagate", ctx.handle, 1, hx, hy, dp, lam, z_wrp, C.c_void_p(w64.data_ptr()), st)
    wrp.zero_()
    _lib.call("oh_wrp_accumulate", ctx.handle, 0, C.byref(wp), C.c_void_p(t_xyz.data_ptr()), npts,
              C.c_void_p(wrp.data_ptr()), st)
    _lib.call("oh_fresnel_propagate", ctx.handle, 0, hx, hy, dp, lam, z_wrp, C.c_void_p(wrp.data_ptr()), st)
    torch.cuda.synchronize()
    acc = gpu_error_report(wrp, w64, torch, dp, lam, -z_wrp - 5e-3)
    acc["reference"] = "the FP64 path (WRP and padded-grid Fresnel in double)"
    res["accuracy"] = acc
    del w64
    torch.cuda.empty_cache()
    if peaks:
        bf16 = load_bf16_peak()
        t_tc = kms.get("wrp_tc")
        if t_tc:
            flops = 3 * 8.0 * npts * 64 * 64          # complex window MACs as real flops, x3 split products
            res["roofline"] = {"bound": "tensor", "kernel": "wrp_tc", "unit": "TFLOP/s",
                               "achieved": flops / (t_tc * 1e-3) / 1e12, "peak": bf16[0],
                               "frac": flops / (t_tc * 1e-3) / 1e12 / bf16[0], "peak_source": bf16[1],
                               "algorithmic_flops_per_launch": flops,
                               "issue": compute_roofline("wrp_tc", t_tc, peaks)}
        fr_ms = sum(v for k, v in kms.items() if k.startswith("fresnel_"))
        if fr_ms:
            hbm, kind = load_peaks()
            fb = 2 * 32 * (2 * hx) * (2 * hy)          # two padded 2-pass FFTs, 8 B read + 8 B written per pass
            res["roofline_fresnel"] = {"bound": "hbm", "unit": "GB/s", "achieved": fb / (fr_ms * 1e-3) / 1e9,
                                       "peak": hbm, "frac": fb / (fr_ms * 1e-3) / 1e9 / hbm,
                                       "peak_source": kind, "algorithmic_bytes": fb,
                                       "issue_rowconv": compute_roofline("fresnel_rowconv",
                                                                         kms.get("fresnel_rowconv", 0), peaks)}
    out["wrp_200k_64x64_fresnel_3840x2160"] = res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-baselines", action="store_true", help="skip the CPU and plain-GPU comparison legs")
    ap.add_argument("--no-secondary", action="store_true", help="skip the point-cloud and WRP workloads")
    ap.add_argument("--unet-samples", type=int, default=UNET_SAMPLES,
                    help="training samples of the learned form (other_operators.unet_surrogate_1024)")
    ap.add_argument("--record", default=None,
                    help="append one JSON-lines accuracy record (max/RMS error, PSNR, fallbacks) to this file")
    ap.add_argument("--batch-frames", type=int, default=None,
                    help="--op batch: the first N frames of the 64-frame workload (small profiling case)")
    ap.add_argument("--no-tune", action="store_true",
                    help="--op batch: time the batch kernel with its default settings (no autotuning first)")
    ap.add_argument("--op", choices=SECONDARY_OPS, default=None,
                    help="time one secondary workload alone (steps calls after warmup) and print its line")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.op:
        import torch
        from openholo_gb300 import Context
        torch.cuda.set_device(local)
        res = secondary_measurements(Context(local), torch.device("cuda", local), torch, reps=args.steps,
                                     ops=(args.op,), warmup=args.warmup, samples=args.unet_samples,
                                     batch_frames=args.batch_frames, batch_tune=not args.no_tune)
        if rank == 0:
            print(json.dumps({"op": args.op, "steps": args.steps, "warmup": args.warmup, **res}), flush=True)
        return

    import torch
    from openholo_gb300 import Context, depthmap as dm, launch_count, scenes
    from openholo_gb300.shard import max_over_ranks, rank_seed

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
        pg = dist
    ctx = Context(local)
    stream = torch.cuda.current_stream()
    img, depth = scenes.depthmap_scene(rank_seed(SCENE_SEED, rank), NY, NX)
    p = dm.make_params(pnx=NX, pny=NY, num_of_depth=LAYERS, pad=PAD, phase_mode=dm.OH_PHASE_SEEDED,
                       seed=rank_seed(PHASE_SEED, rank))
    d_img = torch.from_numpy(img).to(dev)
    d_depth = torch.from_numpy(depth).to(dev)
    fringe = torch.empty((NY, NX), dtype=torch.float32, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    for _ in range(args.warmup):
        dm.generate(ctx, p, d_img, d_depth, fringe=fringe)
    torch.cuda.synchronize()

    # ---- device-resident timed region
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    n0 = launch_count()
    ctx.set_timing(True)
    ctx.read_timing(reset=True)
    with ClockSampler(local) as clk:
        for a, b in ev:
            flush.fill_(1.0)
            a.record(stream)
            dm.generate(ctx, p, d_img, d_depth, fringe=fringe)
            b.record(stream)
        torch.cuda.synchronize()
    launches = launch_count() - n0
    ctx.set_timing(False)
    ktimes = ctx.read_timing(reset=True)
    clocks = clk.summary()
    total_ms = sum(a.elapsed_time(b) for a, b in ev)
    total_ms = max_over_ranks(total_ms, pg, dev)
    ms_step = total_ms / args.steps
    fps = world * 1000.0 / ms_step

    # ---- end to end through the host-buffer C entry point
    h_img = torch.from_numpy(img).pin_memory()
    h_depth = torch.from_numpy(depth).pin_memory()
    h_out = torch.empty((NY, NX), dtype=torch.float32).pin_memory()
    # a stream of its own, as a serving loop would use: repeated calls with
    # the same page-locked buffers replay one graph of copies and passes
    e2e_stream = torch.cuda.Stream(device=dev)
    for _ in range(2):
        dm.generate_host(ctx, p, h_img.numpy(), h_depth.numpy(), out=h_out.numpy(), stream=e2e_stream)
    if pg:
        pg.barrier()
    wall = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dm.generate_host(ctx, p, h_img.numpy(), h_depth.numpy(), out=h_out.numpy(), stream=e2e_stream)
        wall.append(time.perf_counter() - t0)
    e2e_ms = 1000.0 * sum(wall) / len(wall)
    e2e_ms = max_over_ranks(e2e_ms, pg, dev)

    # ---- roofline of the dominant kernel
    peak, peak_kind = load_peaks()
    dom = max(ktimes.items(), key=lambda kv: kv[1][0]) if ktimes else ("?", (0.0, 1))
    dom_name, (dom_ms, dom_n) = dom
    Np = (PAD * NX) * (PAD * NY)
    # per-kernel share of the frame HBM model: per layer a 2-pass FFT that reads and
    # writes 8 B/sample per pass, plus one inverse 2-pass FFT and the uint8 inputs
    model = {"dm_row_pass": LAYERS * 16 * Np + 2 * NX * NY,
             "dm_col_pass": LAYERS * 16 * Np + 16 * Np,
             "dm_out_pass": 16 * Np}
    alg_bytes = model.get(dom_name, 0)
    launch_s = dom_ms / dom_n / 1000.0 if dom_ms > 0 else float("inf")
    achieved = alg_bytes / launch_s / 1e9
    traffic = profile_figure("traffic.json", dom_name)
    roof = {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
            "algorithmic_bytes_per_launch": alg_bytes}
    if traffic:
        roof["traffic_gbs"] = traffic / launch_s / 1e9
        roof["traffic_frac"] = roof["traffic_gbs"] / peak

    out = {"metric": METRIC, "value": fps, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32",
           "data": "synthetic: seeded Gaussian-sum uint8 intensity/depth, SplitMix64 per-pixel phase",
           "config": {"workload": WORKLOAD, "pnx": NX, "pny": NY, "layers": LAYERS, "pad": PAD,
                      "fft_grid": [PAD * NX, PAD * NY], "l2": "flushed between timed steps (512 MiB write)"},
           "e2e": {"value": world * 1000.0 / e2e_ms, "unit": "frames/s", "h2d_bytes_per_step": 2 * NX * NY,
                   "d2h_bytes_per_step": 4 * NX * NY,
                   "call_ms": {"min": 1000.0 * min(wall), "median": 1000.0 * sorted(wall)[len(wall) // 2],
                               "max": 1000.0 * max(wall)}},
           "gpu_launches": launches,
           "kernels_ms_per_frame": {k: v[0] / args.steps for k, v in ktimes.items()},
           "roofline": roof,
           "clocks": clocks}

    peaks = None
    if rank == 0 and world == 1:
        from openholo_gb300 import _lib
        try:
            peaks = _lib.measure_issue_peaks(local)
            out["compute_peaks"] = peaks
            out["roofline_compute"] = {k: compute_roofline(k, v[0] / v[1], peaks) for k, v in ktimes.items()}
        except Exception as e:  # pragma: no cover
            out["compute_peaks"] = {"error": str(e)[:200]}

    if rank == 0 and world == 1 and not args.no_secondary:
        try:
            out["other_operators"] = secondary_measurements(ctx, dev, torch, peaks=peaks,
                                                            samples=args.unet_samples)
        except Exception as e:  # pragma: no cover
            out["other_operators"] = {"error": str(e)[:300]}
        torch.cuda.empty_cache()
    if rank == 0 and world == 1 and not args.no_baselines:
        # FP64 mode of the same frame (the reference computes in double)
        f64 = dm.generate(ctx, p, d_img, d_depth, precision="fp64")
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(3):
            dm.generate(ctx, p, d_img, d_depth, precision="fp64", fringe=f64)
        b.record()
        torch.cuda.synchronize()
        ms64 = a.elapsed_time(b) / 3
        out["fp64_mode"] = {"value": 1000.0 / ms64, "unit": "frames/s", "ms_per_frame": ms64}
        # plain FP32 GPU path (reference structure on cuFFT)
        try:
            lut, zt = dm.levels(p)
            frame = plain_gpu_path(d_img, d_depth, list(zt), lut, torch)
            for _ in range(2):
                ref_plain = frame()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            reps = 3
            a.record()
            for _ in range(reps):
                ref_plain = frame()
            b.record()
            torch.cuda.synchronize()
            plain_ms = a.elapsed_time(b) / reps
            out["plain_gpu_path"] = {"value": 1000.0 / plain_ms, "unit": "frames/s",
                                     "rel_err_vs_fp64": float(torch.linalg.norm(ref_plain.double() - f64) /
                                                              torch.linalg.norm(f64)),
                                     "what": "reference per-layer structure, FP32, cuFFT C2C via torch.fft, "
                                             "FP64-precomputed transfer functions"}
            del frame
        except Exception as e:  # pragma: no cover
            out["plain_gpu_path"] = {"error": str(e)[:200]}
        # the FP32 frame's field, for the error report
        field32 = torch.empty((NY, NX), dtype=torch.complex64, device=dev)
        field64 = torch.empty((NY, NX), dtype=torch.complex128, device=dev)
        dm.generate(ctx, p, d_img, d_depth, fringe=fringe, field=field32)
        dm.generate(ctx, p, d_img, d_depth, precision="fp64", fringe=f64, field=field64)
        torch.cuda.synchronize()
        got_fr, got_field = fringe.cpu().numpy(), field32.cpu().numpy()
        got64_fr, got64_field = f64.cpu().numpy(), field64.cpu().numpy()
        del f64, field32, field64
        torch.cuda.empty_cache()
        # CPU baseline: one whole frame of the oracle port, whose output is also
        # the FP64 reference of the error report
        phase = scenes.seeded_phase(rank_seed(PHASE_SEED, rank), NY, NX)
        cores = os.cpu_count()
        secs, ref_fr, ref_field = cpu_frame(img, depth, phase, workers=cores)
        out["cpu_baseline"] = {"value": 1.0 / secs, "unit": "frames/s", "cores": cores, "kind": "port",
                               "sample": CPU_SAMPLE.format(w=cores)}
        out["accuracy"] = {"fp32_vs_fp64_oracle": error_report(got_fr, got_field, ref_fr, ref_field),
                           "fp64_vs_fp64_oracle": error_report(got64_fr, got64_field, ref_fr, ref_field,
                                                               focus_z=(0.325,)),
                           "what": "whole 1920x1080 frame against the CPU oracle (float64); PSNR of "
                                   "angular-spectrum reconstructions of the fringe at the given depths"}
        out["accuracy"]["rel_err_vs_fp64"] = out["accuracy"]["fp32_vs_fp64_oracle"]["fringe_rel_l2"]
    if rank == 0:
        print(json.dumps(out), flush=True)
        if args.record:
            with open(args.record, "a") as fh:
                rec = {"when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()), "workload": WORKLOAD,
                       "value": out["value"], "accuracy": out.get("accuracy"),
                       "other_operators_accuracy": {k: v.get("accuracy") for k, v in
                                                    (out.get("other_operators") or {}).items()
                                                    if isinstance(v, dict) and "accuracy" in v}}
                fh.write(json.dumps(rec) + "\n")
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
