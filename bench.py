#!/usr/bin/env python
"""Benchmark of the 3D FFT convolution on GB300.

Workload (default): the plain forward convolution at microscope size -- a
512x512x128 (x,y,z) float32 stack (background 100 + 2000 Gaussian spots,
Poisson noise, seed 2) with a 31x31x63 anisotropic Gaussian PSF.  One step is
one full convolution (kernel spectrum + image transforms + product + inverse)
of that volume.  Inputs are seeded synthetic data of the configuration's
shapes and value distribution.

Line fields (one JSON line from rank 0):
  value     Gvoxel/s with inputs resident in HBM (fc_conv3d_device), per-step
            CUDA events on the launch stream, L2 flushed before every step
            (256 MiB write, outside the step events), mean over K steps, max
            over ranks; whole-job aggregate over N replicas.
  e2e       the same metric through convolution3DfftCUDAInPlace with host
            buffers (pinned), H2D + compute + D2H inside the timed call;
            e2e.link holds the measured pinned copy bandwidth of the host
            link and the time the call's bytes need over it.
  roofline  the dominant pass, algorithmic bytes / its mean event duration,
            against the measured HBM copy bandwidth.
  fp64_error  rel-L2 and max-abs error of the headline output against an
            FP64 FFT convolution on the host (every form carries its own).
  cpu_baseline  the reference algorithm on the host cores (oracle port).
  ref_gpu_build  the reference library's own GPU build (compiled from its
            sources with cuFFT) through its InPlace entry on the same GPU,
            wall time per call, beside the same call of this library.
  ref_cufft the reference's device sequence (cuFFT R2C x2, modulate, C2R)
            with plans built beforehand, CUDA events, on the same GPU.
  forms     the non-power-of-two stack, adjoint, batched, tensor-core,
            kernel-spectrum reuse, subsampled kernel and Richardson-Lucy
            forms against the plain path, each with its FP64-oracle error.
`--impl reference` times the reference algorithm on the host cores (the
oracle's float32 port with scipy.fft standing in for cuFFT; the reference
library itself has no CPU path).  Both arms print the same `config`.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

CONFIGS = {
    "c2a": dict(workload="plain_conv_512x512x128_psf31x31x63", fn="c2", kw=dict(nonpow2=False)),
    "c2b": dict(workload="plain_conv_384x448x96_psf31x31x63", fn="c2", kw=dict(nonpow2=True)),
    "c1": dict(workload="plain_conv_64x64x64_psf7x7x7", fn="c1", kw={}),
    "c5": dict(workload="plain_conv_1024x1024x256_psf63x63x63", fn="c5", kw={}),
    # the 256-long fused z pass on a quarter of the columns (profiler captures)
    "c5s": dict(workload="plain_conv_512x512x256_psf63x63x63", fn="c5", kw=dict(plane=512)),
}
METRIC = "Gvoxel/s per 3D FFT conv (plain/batched/adjoint/TC) vs plain & ref cuFFT, rel-L2<=1e-5"


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "100", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append((time.perf_counter(), parts))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.t:
            self.t.join(timeout=5)

    def summary(self, t0: float, t1: float):
        inside = [r for t, r in self.rows if t0 <= t <= t1] or [r for _, r in self.rows]
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm = [float(r[1]) for r in inside if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in inside if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in inside for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(inside)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if os.environ.get("FC_BENCH_BACKEND", "nccl") == "nccl" else "gloo")
    return world, rank, local


def reduce_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def make_data(cfg):
    from fourierconvolutioncudalib_gb300 import workloads as W

    return getattr(W, cfg["fn"])(**cfg["kw"])


def config_dict(cfg, im_shape, k_shape, world, suffix=""):
    """The `config` object of the JSON line; both arms print the same one."""
    nz, ny, nx = im_shape
    kz, ky, kx = k_shape
    return {"workload": cfg["workload"] + suffix, "image_xyz": [nx, ny, nz], "kernel_xyz": [kx, ky, kz],
            "l2": "flushed before every GPU step (256 MiB write outside the step timing)",
            "parallelism": f"replicas x{world}"}


def fp64_conv(im, k, workers=None):
    """Circular convolution in double precision (scipy.fft on all host cores),
    kernel centre at k//2 moved to the origin; returns (result, padded kernel)."""
    import scipy.fft as sfft

    workers = workers or os.cpu_count() or 1
    pk = np.zeros(im.shape, np.float64)
    kz, ky, kx = k.shape
    nz, ny, nx = im.shape
    pk[np.ix_((np.arange(kz) - kz // 2) % nz, (np.arange(ky) - ky // 2) % ny, (np.arange(kx) - kx // 2) % nx)] = k
    a = sfft.rfftn(im.astype(np.float64), workers=workers)
    a *= sfft.rfftn(pk, workers=workers)
    return sfft.irfftn(a, s=im.shape, axes=(0, 1, 2), workers=workers), pk


def fp64_error(out, exact):
    """rel-L2 and max-abs / max|exact| of a float32 result against FP64."""
    o = np.asarray(out, np.float64)
    e = np.asarray(exact, np.float64)
    return {"rel_l2": float(np.linalg.norm((o - e).ravel()) / np.linalg.norm(e.ravel())),
            "max_abs_rel": float(np.max(np.abs(o - e)) / np.max(np.abs(e)))}


# ------------------------------------------------------------------ reference arm
def run_reference(args, cfg, world, rank):
    if rank != 0:
        return
    from oracle import oracle as orc

    d = make_data(cfg)
    im, k = d["image"], d["kernel"]
    cores = os.cpu_count() or 1
    budget_s = float(os.environ.get("FC_BENCH_REF_BUDGET_S", "120"))
    t = time.perf_counter()
    orc.reference_path_fp32(im, k, "centered", workers=cores)
    first = time.perf_counter() - t
    warm = min(args.warmup, max(0, int(10 / max(first, 1e-3))))
    for _ in range(warm):
        orc.reference_path_fp32(im, k, "centered", workers=cores)
    steps = max(1, min(args.steps, int(budget_s / max(first, 1e-3))))
    times = []
    for _ in range(steps):
        t = time.perf_counter()
        orc.reference_path_fp32(im, k, "centered", workers=cores)
        times.append(time.perf_counter() - t)
    ms = 1e3 * statistics.mean(times)
    val = im.size / (ms / 1e3) / 1e9
    sample = f"{steps} full-volume steps of {args.steps} requested (budget {budget_s:.0f} s), {warm} warm-up"
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "Gvoxel/s", "n_gpus": world, "steps": steps,
        "warmup": warm, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded, configuration shapes and distribution)",
        "config": config_dict(cfg, im.shape, k.shape, world),
        "impl_detail": "reference algorithm on host cores: pad+shift, R2C x2, modulate 1/N, C2R "
                       "(float32, scipy.fft transforms standing in for cuFFT)",
        "cpu_baseline": {"value": val, "unit": "Gvoxel/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": val, "unit": "Gvoxel/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ our arm
def run_ours(args, cfg, world, rank, local):
    import torch

    import fourierconvolutioncudalib_gb300 as fc
    from fourierconvolutioncudalib_gb300 import build as fcbuild
    from fourierconvolutioncudalib_gb300 import device as fcd

    fcbuild.build()
    fc.load_library()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    d = make_data(cfg)
    im_np, k_np = d["image"], d["kernel"]
    nz, ny, nx = im_np.shape
    kz, ky, kx = k_np.shape
    N = im_np.size
    img = torch.from_numpy(im_np).to(dev)
    ker = torch.from_numpy(k_np).to(dev)
    out = torch.empty_like(img)
    ws = torch.empty(fcd.workspace_bytes(im_np.shape, k_np.shape), dtype=torch.uint8, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()

    tc_flag = {"fp16": fc.FC_FLAG_TC_FP16, "bf16": fc.FC_FLAG_TC_BF16}.get(args.tc, 0)

    def step():
        fcd.conv3d(img, ker, out=out, workspace=ws, flags=tc_flag)

    for _ in range(args.warmup):
        flush.zero_()
        step()
    torch.cuda.synchronize()

    # ---- per-pass breakdown (untimed steps): mean event duration of every pass
    peak, peak_kind = load_peaks()
    fcd.profile(True)
    for _ in range(max(3, min(args.steps, 10))):
        flush.zero_()
        step()
    torch.cuda.synchronize()
    fcd.profile(False)
    agg = {}
    for name, pms, by in fcd.profile():
        a = agg.setdefault(name, [0.0, 0.0, 0])
        a[0] += pms
        a[1] += by
        a[2] += 1
    table = []
    for name, (tms, tby, cnt) in agg.items():
        mean_ms = tms / cnt
        gbs = (tby / cnt) / (mean_ms / 1e3) / 1e9 if mean_ms > 0 else 0.0
        table.append({"pass": name, "launches": cnt, "mean_us": 1e3 * mean_ms, "alg_bytes": tby / cnt, "GB/s": gbs,
                      "frac": gbs / peak})
    table.sort(key=lambda r: -r["mean_us"] * r["launches"])
    dom_name = table[0]["pass"] if table else None

    # ---- timed region: K steps with per-step events; inside the steps only the
    # dominant pass records events (its launch durations give the roofline)
    K = args.steps
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    fcd.profile(True, only=dom_name)
    launches = 0
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(K):
        flush.zero_()
        evs[i][0].record(stream)
        step()
        evs[i][1].record(stream)
        launches += fcd.launch_count()
    torch.cuda.synchronize()
    barrier(world)
    t1 = time.perf_counter()
    fcd.profile(False)
    time.sleep(0.2)
    clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    dom_recs = fcd.profile()
    ms_local = statistics.mean(step_ms)
    ms = reduce_max(ms_local, world)
    value = world * N / (ms / 1e3) / 1e9

    # dominant kernel roofline from its launches inside the timed region
    dom = None
    if dom_recs:
        d_ms = statistics.mean(r[1] for r in dom_recs)
        d_by = statistics.mean(r[2] for r in dom_recs)
        d_gbs = d_by / (d_ms / 1e3) / 1e9
        dom = {"pass": dom_name, "launches": len(dom_recs), "mean_us": 1e3 * d_ms, "alg_bytes": d_by, "GB/s": d_gbs,
               "frac": d_gbs / peak}
    traffic = None
    tf = ROOT / "profiles" / "ncu_traffic.json"
    if dom and tf.exists():
        try:
            wl = cfg["workload"] + (f"_tc_{args.tc}" if tc_flag else "")
            traffic = json.loads(tf.read_text()).get(wl, {}).get(dom["pass"])
        except Exception:
            traffic = None
    Mc = (nx // 2 + 1) * ny * nz
    model_bytes = 8 * N + 4 * k_np.size + 80 * Mc
    roofline = {"bound": "hbm", "kernel": dom["pass"] if dom else None, "achieved": dom["GB/s"] if dom else None,
                "peak": peak, "unit": "GB/s", "frac": dom["frac"] if dom else None, "traffic": traffic,
                "peak_source": peak_kind,
                "step_model_bytes": model_bytes, "step_model_frac": model_bytes / (ms / 1e3) / 1e9 / peak}

    # ---- end to end through the reference-facing C ABI, host buffers
    e2e = None
    if not args.no_e2e:
        pin = torch.empty(N, dtype=torch.float32, pin_memory=True).numpy().reshape(im_np.shape)
        kpin = torch.empty(k_np.size, dtype=torch.float32, pin_memory=True).numpy().reshape(k_np.shape)
        kpin[...] = k_np
        e2e_t = []
        page = im_np.copy()
        page_t = []
        reps = max(3, min(args.steps, 20))
        for i in range(reps + 2):
            np.copyto(pin, im_np)
            torch.cuda.synchronize()
            t = time.perf_counter()
            fc.convolution3DfftCUDAInPlace(pin, (nx, ny, nz), kpin, (kx, ky, kz), local)
            dt = time.perf_counter() - t
            if i >= 2:
                e2e_t.append(dt)
        for i in range(min(reps, 5) + 1):
            np.copyto(page, im_np)
            t = time.perf_counter()
            fc.convolution3DfftCUDAInPlace(page, (nx, ny, nz), k_np, (kx, ky, kz), local)
            dt = time.perf_counter() - t
            if i >= 1:
                page_t.append(dt)
        ok_err = float(np.max(np.abs(pin - out.cpu().numpy())) / max(1e-30, float(np.max(np.abs(pin)))))
        # the same call with staged copies instead of direct host access
        fc.lib().fc_set_host_io(0)
        copy_t = []
        for i in range(min(reps, 5) + 1):
            np.copyto(pin, im_np)
            t = time.perf_counter()
            fc.convolution3DfftCUDAInPlace(pin, (nx, ny, nz), kpin, (kx, ky, kz), local)
            dt = time.perf_counter() - t
            if i >= 1:
                copy_t.append(dt)
        fc.lib().fc_set_host_io(2)
        e2e_s = reduce_max(statistics.median(e2e_t), world)
        link = measure_link(torch, dev, N)
        h2d_b, d2h_b = 4 * (N + k_np.size), 4 * N
        link["bound_ms_per_call"] = 1e3 * (h2d_b / (link["h2d_GBps"] * 1e9) + d2h_b / (link["d2h_GBps"] * 1e9))
        link["bound_ms_overlapped"] = 1e3 * max(h2d_b / (link["h2d_GBps"] * 1e9), d2h_b / (link["d2h_GBps"] * 1e9))
        e2e = {"value": world * N / e2e_s / 1e9, "unit": "Gvoxel/s", "h2d_bytes_per_step": h2d_b,
               "d2h_bytes_per_step": d2h_b, "host_buffer": "pinned", "ms_per_call": 1e3 * e2e_s,
               "link": link, "link_frac": link["bound_ms_per_call"] / (1e3 * e2e_s),
               "host_io": "auto: pinned buffer read/written in place by the passes over NVLink-C2C; pageable "
                          "buffers staged with copies",
               "pageable_ms_per_call": 1e3 * statistics.median(page_t),
               "staged_copy_ms_per_call": 1e3 * statistics.median(copy_t), "api": "convolution3DfftCUDAInPlace",
               "max_rel_diff_vs_device_path": ok_err}

    # ---- reference device sequence on cuFFT, same GPU
    ref_cufft = None
    if not args.no_ref_cufft:
        try:
            ref_cufft = time_ref_cufft(im_np, k_np, dev, args, value)
        except Exception as e:  # the cuFFT harness is optional for the line
            ref_cufft = {"error": str(e)[:200]}

    # ---- the other forms (adjoint, batched) against the plain path on the same GPU
    forms = None
    if rank == 0 and not args.no_forms:
        try:
            forms = time_forms(dev, fcd, torch)
        except Exception as e:  # reported, not fatal for the headline line
            forms = {"error": str(e)[:300]}

    # ---- FP64-oracle error of the headline result (the output of the last timed step)
    fp64 = None
    if rank == 0 and not args.no_fp64:
        fp64 = fp64_error(out.cpu().numpy(), fp64_conv(im_np, k_np)[0])

    # ---- baselines (rank 0, N = 1 only): the reference algorithm on the host
    # cores, and the reference library's own GPU build on this GPU
    cpu = None
    ref_gpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = time_cpu_baseline(im_np, k_np)
    if rank == 0 and world == 1 and not args.no_ref_gpu:
        try:
            ref_gpu = time_ref_gpu_build(im_np, k_np, local, fc, e2e)
        except Exception as e:  # reported, not fatal for the headline line
            ref_gpu = {"error": str(e)[:300]}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Gvoxel/s", "n_gpus": world, "steps": K,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if not tc_flag else f"f32 data, {args.tc} hi+lo tensor-core DFT stages",
            "data": "synthetic (seeded, configuration shapes and distribution)",
            "config": config_dict(cfg, im_np.shape, k_np.shape, world, f"_tc_{args.tc}" if tc_flag else ""),
            "impl_detail": "fc_conv3d_device on HBM-resident buffers (value); convolution3DfftCUDAInPlace on host "
                           "buffers (e2e)",
            "fp64_error": fp64,
            "wall_s_timed_region": t1 - t0,
            "e2e": e2e, "roofline": roofline, "passes": table, "cpu_baseline": cpu, "ref_gpu_build": ref_gpu,
            "ref_cufft": ref_cufft, "forms": forms,
            "gpu_launches": launches, "clocks": clocks.summary(t0, t1),
        }
        print(json.dumps(line), flush=True)


def measure_link(torch, dev, n_floats):
    """Pinned host <-> device copy bandwidth of one volume (GB/s), best of 5."""
    h = torch.empty(n_floats, dtype=torch.float32, pin_memory=True)
    d = torch.empty(n_floats, dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream()
    res = {}
    for name, fn in (("h2d_GBps", lambda: d.copy_(h, non_blocking=True)),
                     ("d2h_GBps", lambda: h.copy_(d, non_blocking=True))):
        best = None
        for _ in range(6):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            fn()
            b.record(st)
            torch.cuda.synchronize()
            t = a.elapsed_time(b)
            best = t if best is None else min(best, t)
        res[name] = 4 * n_floats / (best / 1e3) / 1e9
    res["how"] = "torch copy of one volume between page-locked host memory and HBM, CUDA events, best of 6"
    return res


def time_ref_gpu_build(im_np, k_np, local, fc, e2e):
    """The reference library's own GPU build (compiled from its sources with
    cuFFT, oracle/build_ref.sh) through its convolution3DfftCUDAInPlace on
    pageable host buffers, wall time per call, beside the same call of this
    library.  The reference's kernel placement differs from the centred one on
    non-cubic shapes, so its output is compared with this library's
    reference-arithmetic placement (fc_set_shift_compat)."""
    from oracle import reference_gpu

    if not reference_gpu.available():
        return {"unavailable": "the reference library could not be built on this host"}
    nz, ny, nx = im_np.shape
    kz, ky, kx = k_np.shape
    r = reference_gpu.time_inplace(im_np, k_np, reps=8, warmup=2, device=local)
    ref_s = statistics.median(r["seconds"])
    L = fc.lib()
    ours = im_np.copy()
    L.fc_set_shift_compat(1)
    try:
        fc.convolution3DfftCUDAInPlace(ours, (nx, ny, nz), k_np, (kx, ky, kz), local)
        page_t = []
        for i in range(6):
            np.copyto(ours, im_np)
            t = time.perf_counter()
            fc.convolution3DfftCUDAInPlace(ours, (nx, ny, nz), k_np, (kx, ky, kz), local)
            if i >= 1:
                page_t.append(time.perf_counter() - t)
    finally:
        L.fc_set_shift_compat(0)
    ref_out = r["output"].astype(np.float64)
    d = ours.astype(np.float64) - ref_out
    our_page_s = statistics.median(page_t)
    res = {"value": im_np.size / ref_s / 1e9, "unit": "Gvoxel/s", "ms_per_call": 1e3 * ref_s,
           "calls": len(r["seconds"]), "host_buffer": "pageable",
           "ours_same_call_ms": 1e3 * our_page_s, "speedup_of_ours_same_call": ref_s / our_page_s,
           "rel_l2_ours_vs_reference": float(np.linalg.norm(d) / np.linalg.norm(ref_out)),
           "max_abs_rel_ours_vs_reference": float(np.max(np.abs(d)) / np.max(np.abs(ref_out))),
           "what": "reference convolution3DfftCUDAInPlace built from its own sources (nvcc sm_103a, cuFFT), median "
                   "wall time per call (host pad, plans, H2D, cuFFT R2C x2, modulate, C2R, D2H, un-pad); ours: "
                   "the same call with the reference's kernel placement"}
    if e2e:
        res["speedup_of_ours_e2e_pinned"] = ref_s / (e2e["ms_per_call"] / 1e3)
    return res


def time_ref_cufft(im_np, k_np, dev, args, our_value):
    """The reference's device sequence (R2C image, R2C kernel, modulate, C2R) on
    cuFFT with plans built beforehand, CUDA events around each sequence."""
    import torch
    from baseline import refseq

    L = refseq.lib()
    nz, ny, nx = im_np.shape
    nxh = nx // 2 + 1
    base_img = torch.zeros((nz, ny, 2 * nxh), dtype=torch.float32, device=dev)
    base_img[..., :nx] = torch.from_numpy(im_np).to(dev)
    kz, ky, kx = k_np.shape
    pk = np.zeros(im_np.shape, np.float32)  # centred placement, same as the library's default
    iz = (np.arange(kz) - kz // 2) % nz
    iy = (np.arange(ky) - ky // 2) % ny
    ix = (np.arange(kx) - kx // 2) % nx
    pk[np.ix_(iz, iy, ix)] = k_np
    base_ker = torch.zeros_like(base_img)
    base_ker[..., :nx] = torch.from_numpy(pk).to(dev)
    wi = torch.empty_like(base_img)
    wk = torch.empty_like(base_img)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    st = torch.cuda.current_stream()
    reps = max(3, min(args.steps, 50))
    times = []
    for i in range(reps + 3):
        wi.copy_(base_img)
        wk.copy_(base_ker)
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        rc = L.refseq_device_only(wi.data_ptr(), wk.data_ptr(), nx, ny, nz, st.cuda_stream)
        b.record(st)
        if rc != 0:
            raise RuntimeError(L.refseq_last_error().decode())
        torch.cuda.synchronize()
        if i >= 3:
            times.append(a.elapsed_time(b))
    L.refseq_release()
    ms = statistics.mean(times)
    v = im_np.size / (ms / 1e3) / 1e9
    return {"value": v, "unit": "Gvoxel/s", "ms_per_step": ms, "speedup_of_ours": our_value / v,
            "what": "cuFFT 3D R2C(image), R2C(padded kernel), modulate x 1/N, C2R; plans pre-built"}


def _events_ms(torch, fn, reps, flush):
    st = torch.cuda.current_stream()
    ts = []
    for i in range(reps + 2):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        fn()
        b.record(st)
        torch.cuda.synchronize()
        if i >= 2:
            ts.append(a.elapsed_time(b))
    return statistics.mean(ts)


def _rel64(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def time_forms(dev, fcd, torch):
    """Adjoint form on the differentiation configuration (256^3, 21^3) and the
    batched form on the multi-view configuration (6 uneven views), each
    against the plain path on the same GPU, with its error against FP64."""
    import tempfile

    from fourierconvolutioncudalib_gb300 import workloads as W

    # the batched form tunes its launch choices on its first (untimed) call; a
    # fresh cache file makes it tune against the kernels of this build
    os.environ.setdefault("FC_TUNE_CACHE", os.path.join(tempfile.mkdtemp(prefix="fc_tune_"), "tune.txt"))

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    out = {}
    # adjoint: both gradients of 0.5*||conv(x,k) - y||^2 for a given residual
    d = W.c3()
    x, k = d["image"], d["kernel"]
    rng = np.random.default_rng(44)
    g = rng.standard_normal(x.shape).astype(np.float32)
    xt, kt, gt = (torch.from_numpy(a).to(dev) for a in (x, k, g))
    ms_adj = _events_ms(torch, lambda: fcd.conv3d_adjoint(xt, kt, gt, k.shape), 10, flush)
    ms_fwd = _events_ms(torch, lambda: fcd.conv3d(xt, kt), 10, flush)
    gi, gk = fcd.conv3d_adjoint(xt, kt, gt, k.shape)
    torch.cuda.synchronize()
    import scipy.fft as sfft

    wk = os.cpu_count() or 1
    _, pk = fp64_conv(x, k)
    G = sfft.rfftn(g.astype(np.float64), workers=wk)
    ax = (0, 1, 2)
    ex = sfft.irfftn(G * np.conj(sfft.rfftn(pk, workers=wk)), s=x.shape, axes=ax, workers=wk)
    gP = sfft.irfftn(np.conj(sfft.rfftn(x.astype(np.float64), workers=wk)) * G, s=x.shape, axes=ax, workers=wk)
    kz, ky, kx = k.shape
    nz, ny, nx = x.shape
    ek = gP[np.ix_((np.arange(kz) - kz // 2) % nz, (np.arange(ky) - ky // 2) % ny, (np.arange(kx) - kx // 2) % nx)]
    out["adjoint"] = {"workload": "adjoint_256x256x256_psf21x21x21", "value": x.size / (ms_adj / 1e3) / 1e9,
                      "unit": "Gvoxel/s", "ms": ms_adj, "plain_forward_ms": ms_fwd,
                      "vs_plain": ms_fwd / ms_adj,
                      "fp64_error_grad_image": fp64_error(gi.cpu().numpy(), ex),
                      "fp64_error_grad_kernel": fp64_error(gk.cpu().numpy(), ek)}
    # batched: six views, one call, against six sequential plain calls
    views = W.c4()
    imgs = [torch.from_numpy(v["image"]).to(dev) for v in views]
    kers = [torch.from_numpy(v["kernel"]).to(dev) for v in views]
    outs = [torch.empty_like(i) for i in imgs]
    dims = []
    for i, kk in zip(imgs, kers):
        dims += [i.shape[2], i.shape[1], i.shape[0], kk.shape[2], kk.shape[1], kk.shape[0]]
    need = fcd.lib().fc_conv3d_batched_workspace_bytes(len(imgs), fcd._iarr(dims), 0)
    ws = torch.empty(need, dtype=torch.uint8, device=dev)
    ws1 = torch.empty(max(fcd.workspace_bytes(i.shape, kk.shape) for i, kk in zip(imgs, kers)), dtype=torch.uint8,
                      device=dev)
    nvox = sum(i.numel() for i in imgs)
    ms_b = _events_ms(torch, lambda: fcd.conv3d_batched(imgs, kers, outs=outs, workspace=ws), 10, flush)

    def seq():
        for i, kk, o in zip(imgs, kers, outs):
            fcd.conv3d(i, kk, out=o, workspace=ws1)

    ms_s = _events_ms(torch, seq, 10, flush)
    fcd.conv3d_batched(imgs, kers, outs=outs, workspace=ws)
    torch.cuda.synchronize()
    errs = [fp64_error(o.cpu().numpy(), fp64_conv(v["image"], v["kernel"])[0]) for o, v in zip(outs, views)]
    ch = (ctypes.c_int * 5)()
    sched = fcd.lib().fc_batched_last_plan(ch)
    sched_names = ["pass-major", "view-major", "view-concurrent", "single-volume sequence per view",
                   "single-volume sequences concurrently"]
    choice_names = ["persistent work-list launch", "persistent, one CTA per SM", "one launch per view"]
    out["batched"] = {"workload": "batched_6_views_87M_voxels", "value": nvox / (ms_b / 1e3) / 1e9,
                      "unit": "Gvoxel/s", "ms": ms_b, "sequential_plain_ms": ms_s, "vs_sequential_plain": ms_s / ms_b,
                      "fp64_error_max_over_views": {"rel_l2": max(e["rel_l2"] for e in errs),
                                                    "max_abs_rel": max(e["max_abs_rel"] for e in errs)},
                      "tuned_schedule": sched_names[sched] if 0 <= sched < 5 else None,
                      "tuned_pass_choices": [choice_names[c] if 0 <= c < 3 else None for c in ch],
                      "how": "one call; the tuner times persistent work-list launches per pass against per-view "
                             "launches and five schedules, caches the choice, and the call replays a CUDA graph"}
    # tensor-core precision mode at 1024x1024x256 (63^3 PSF): time and FP64-oracle
    # error of the fp32 path and of the fp16 and bf16 modes
    import fourierconvolutioncudalib_gb300 as fc

    d5 = W.c5()
    im5, k5 = d5["image"], d5["kernel"]
    ref5 = fp64_conv(im5, k5)[0]
    i5 = torch.from_numpy(im5).to(dev)
    k5t = torch.from_numpy(k5).to(dev)
    ws5 = torch.empty(fcd.workspace_bytes(im5.shape, k5.shape), dtype=torch.uint8, device=dev)
    o5 = torch.empty_like(i5)
    tc = {"workload": "tc_1024x1024x256_psf63x63x63"}
    ms32 = None
    for name, flag in (("fp32", 0), ("fp16", fc.FC_FLAG_TC_FP16), ("bf16", fc.FC_FLAG_TC_BF16)):
        ms = _events_ms(torch, lambda: fcd.conv3d(i5, k5t, out=o5, workspace=ws5, flags=flag), 5, flush)
        torch.cuda.synchronize()
        ms32 = ms if flag == 0 else ms32
        tc[name] = {"value": im5.size / (ms / 1e3) / 1e9, "unit": "Gvoxel/s", "ms": ms, "vs_fp32_path": ms32 / ms,
                    "fp64_error": fp64_error(o5.cpu().numpy(), ref5)}
    del i5, k5t, ws5, o5, ref5
    d2 = W.c2()
    im2, k2 = d2["image"], d2["kernel"]
    ref2, _ = fp64_conv(im2, k2)
    i2 = torch.from_numpy(im2).to(dev)
    k2t = torch.from_numpy(k2).to(dev)
    tc["how"] = ("radix-16 stages as real 128x32x32 DFT products on tcgen05 (kind::f16, M=128 butterflies per "
                 "128-thread group, fp32 accumulator in TMEM, operands in shared memory), per-row power-of-two "
                 "scaling, hi+lo 16-bit operands (3 products), fp32 accumulation")
    out["tensor_core"] = tc
    # the non-power-of-two microscope stack (384x448x96, same generator and PSF): radices 16, 14, 12, 6, 2
    db = W.c2(nonpow2=True)
    imb, kb = db["image"], db["kernel"]
    ib = torch.from_numpy(imb).to(dev)
    kbt = torch.from_numpy(kb).to(dev)
    ob = torch.empty_like(ib)
    wsb = torch.empty(fcd.workspace_bytes(imb.shape, kb.shape), dtype=torch.uint8, device=dev)
    ms_b2 = _events_ms(torch, lambda: fcd.conv3d(ib, kbt, out=ob, workspace=wsb), 20, flush)
    torch.cuda.synchronize()
    out["plain_nonpow2"] = {"workload": "plain_conv_384x448x96_psf31x31x63", "value": imb.size / (ms_b2 / 1e3) / 1e9,
                            "unit": "Gvoxel/s", "ms": ms_b2, "fp64_error": fp64_error(ob.cpu().numpy(),
                                                                                      fp64_conv(imb, kb)[0])}
    del ib, kbt, ob, wsb
    # kernel-spectrum reuse: the image passes only, against the plain call (512x512x128, 31x31x63)
    ks = fcd.kernel_spectrum(k2t, im2.shape)
    o2 = torch.empty_like(i2)
    ws2 = torch.empty(fcd.workspace_bytes(im2.shape, k2.shape), dtype=torch.uint8, device=dev)
    ms_plain = _events_ms(torch, lambda: fcd.conv3d(i2, k2t, out=o2, workspace=ws2), 10, flush)
    ms_reuse = _events_ms(torch, lambda: fcd.conv3d_kspec(i2, ks, k2.shape, out=o2, workspace=ws2), 10, flush)
    fcd.conv3d_kspec(i2, ks, k2.shape, out=o2, workspace=ws2)
    torch.cuda.synchronize()
    out["kernel_spectrum_reuse"] = {
        "workload": "plain_conv_512x512x128_psf31x31x63", "value": im2.size / (ms_reuse / 1e3) / 1e9,
        "unit": "Gvoxel/s", "ms": ms_reuse, "plain_ms": ms_plain, "vs_plain": ms_plain / ms_reuse,
        "fp64_error": fp64_error(o2.cpu().numpy(), ref2)}
    # subsampled kernel (the memory-saving variant): the kernel transformed at
    # its own size and read at the nearest kernel frequency; an approximation,
    # so its error is reported against the exact convolution
    wss = torch.empty(fcd.subsampled_workspace_bytes(im2.shape, k2.shape), dtype=torch.uint8, device=dev)
    ms_sub = _events_ms(torch, lambda: fcd.conv3d_subsampled(i2, k2t, out=o2, workspace=wss), 10, flush)
    fcd.conv3d_subsampled(i2, k2t, out=o2, workspace=wss)
    torch.cuda.synchronize()
    gs = o2.cpu().numpy()
    out["subsampled_kernel"] = {
        "workload": "subsampled_conv_512x512x128_psf31x31x63", "value": im2.size / (ms_sub / 1e3) / 1e9,
        "unit": "Gvoxel/s", "ms": ms_sub, "plain_ms": ms_plain, "vs_plain": ms_plain / ms_sub,
        "workspace_bytes": wss.numel(), "plain_workspace_bytes": ws2.numel(),
        "rel_l2_vs_exact_convolution": _rel64(gs, ref2),
        "max_abs_rel_vs_exact_convolution": float(np.max(np.abs(gs - ref2)) / np.max(np.abs(ref2)))}
    del i2, k2t, o2, ws2, ks, wss
    # Richardson-Lucy: 10 iterations on the 256^3 spot volume blurred by the 21^3 PSF
    y3 = fcd.conv3d(torch.from_numpy(d["x_true"]).to(dev), torch.from_numpy(d["k_true"]).to(dev)).clamp_(min=0)
    k3 = torch.from_numpy(d["k_true"]).to(dev)
    iters = 10
    est = torch.empty_like(y3)

    def rl():
        est.copy_(y3)
        fcd.rl_deconvolve(y3, k3, iters, estimate=est)

    ms_rl = _events_ms(torch, rl, 3, flush)
    ms_c = _events_ms(torch, lambda: fcd.conv3d(y3, k3), 5, flush)
    # FP64 restatement of the update, 2 iterations (numpy)
    est.copy_(y3)
    fcd.rl_deconvolve(y3, k3, 2, estimate=est)
    torch.cuda.synchronize()
    yn = y3.double().cpu().numpy()
    _, pk3 = fp64_conv(yn.astype(np.float32), d["k_true"])
    K3 = np.fft.rfftn(pk3)
    xr = yn.copy()
    for _ in range(2):
        e = np.fft.irfftn(np.fft.rfftn(xr) * K3, s=yn.shape, axes=(0, 1, 2))
        r = np.divide(yn, e, out=np.zeros_like(yn), where=e > 0)
        xr = xr * np.fft.irfftn(np.fft.rfftn(r) * np.conj(K3), s=yn.shape, axes=(0, 1, 2))
    out["richardson_lucy"] = {
        "workload": "rl_256x256x256_psf21x21x21_10_iterations", "value": y3.numel() * iters / (ms_rl / 1e3) / 1e9,
        "unit": "Gvoxel-iterations/s", "ms": ms_rl, "ms_per_iteration": ms_rl / iters,
        "plain_conv_ms": ms_c, "iteration_vs_two_plain_convs": 2 * ms_c / (ms_rl / iters),
        "fp64_error_after_2_iterations": fp64_error(est.cpu().numpy(), xr),
        "how": "kernel spectrum once per call; per iteration conv and correlation against it + 2 pointwise passes"}
    return out


def time_cpu_baseline(im_np, k_np):
    from oracle import oracle as orc

    cores = os.cpu_count() or 1
    t = time.perf_counter()
    orc.reference_path_fp32(im_np, k_np, "centered", workers=cores)
    first = time.perf_counter() - t
    n = max(1, min(5, int(15.0 / max(first, 1e-3))))
    ts = []
    for _ in range(n):
        t = time.perf_counter()
        orc.reference_path_fp32(im_np, k_np, "centered", workers=cores)
        ts.append(time.perf_counter() - t)
    s = statistics.mean(ts)
    out = {"value": im_np.size / s / 1e9, "unit": "Gvoxel/s", "cores": cores, "kind": "port",
           "sample": f"{n} full-volume convolutions (after 1 warm-up): the reference algorithm in float32 on the "
                     f"host, scipy.fft transforms on {cores} threads"}
    # the reference test suite's CPU convolution (tests/test_algorithms.hpp:10-58: direct spatial sum, float
    # accumulator, periodic here) on output crops at the volume's centre, all cores and one thread; the
    # full-volume time is extrapolated from the crop
    try:
        ds = {}
        for label, crop, threads in (("all_cores", (16, 32, 32), cores), ("one_thread", (4, 16, 16), 1)):
            c0 = tuple((nn - cc) // 2 for nn, cc in zip(im_np.shape, crop))
            t = time.perf_counter()
            orc.convolve_direct_crop(im_np, k_np, c0, crop, threads=threads)
            dt = time.perf_counter() - t
            nv = int(np.prod(crop))
            ds[label] = {"value": nv / dt / 1e9, "unit": "Gvoxel/s", "cores": threads,
                         "crop_zyx": list(crop), "seconds": dt,
                         "full_volume_seconds_extrapolated": dt * im_np.size / nv}
        ds["what"] = "direct spatial sum of the reference test suite's CPU convolution, on output crops"
        out["direct_sum"] = ds
    except Exception as e:  # the FFT-based baseline above stands on its own
        out["direct_sum"] = {"unavailable": repr(e)[:200]}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", choices=sorted(CONFIGS), default="c2a")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-ref-cufft", action="store_true")
    ap.add_argument("--no-forms", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-ref-gpu", action="store_true")
    ap.add_argument("--tc", choices=["fp16", "bf16"], default=None,
                    help="time the tensor-core precision mode instead of the fp32 path")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    cfg = CONFIGS[args.config]
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, cfg, world, rank)
    else:
        run_ours(args, cfg, world, rank, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
