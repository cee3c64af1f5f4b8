#!/usr/bin/env python
"""FDK cone-beam reconstruction benchmark on GB300.

Workload: 1024^3 FP32 volume from 720 x 1024^2 uint16 projections (0.15 mm
pitch, SOD 300 mm, SDD 900 mm), log transform + Hann ramp + voxel-driven
backprojection.  Seeded synthetic 40-ellipsoid phantom (densities
0.1-2.0 /cm), Poisson counts at I0 = 60000.  One step = one full
reconstruction.  Metric: GUPS (voxel-projection updates per second); the
chosen form stores filtered projections in FP16 (FP32 math and
accumulation), the plain form in FP32.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank reconstructs its own volume (independent
scans, no data exchange): weak scaling, time = max over ranks.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

I0 = 60000.0
N_ELLIPSOIDS = 40
PHANTOM_SEED = 11
FLOPS_PER_UPDATE = 14  # z-column walk: v, floor/frac, 3 lerps, weighted accumulate
PEAK_FP32_NOMINAL = 152 * 128 * 2 * 2.070e9 / 1e12  # TFLOP/s at the 2070 MHz max SM clock
CPU_SAMPLE_SLICES = (508, 509, 510, 511, 512, 513, 514, 515)
RMSE_SLICES = ((480, 512, 544), (1010,))


def bp_kernel_name(variant, precision=None):
    """Name of the backprojection variant a storage format runs at 1024^3 (the selected one, else the
    format's default, a quarter-turn kernel for this symmetric scan)."""
    from tomokvas_gb300 import _lib

    L = _lib.load()
    precision = _lib.TK_F16 if precision is None else precision
    if variant < 0 or L.tk_bp_variant_precision(variant) != precision:
        variant = next(i for i in range(L.tk_bp_variant_count()) if L.tk_bp_variant_precision(i) == precision)
    return "bp_" + L.tk_bp_variant_name(variant).decode()


def half_math_variant():
    """Index of the selectable FP16 half-math quarter-turn kernel (16 x 8 tiles; FP16 interpolation
    arithmetic), reported beside the headline, never as it."""
    from tomokvas_gb300 import _lib

    L = _lib.load()
    return next(i for i in range(L.tk_bp_variant_count())
                if L.tk_bp_variant_name(i).decode().startswith("quad<f16,16,8,") and ",h16row1," in
                L.tk_bp_variant_name(i).decode())


# DRAM traffic of the default FP16 backprojection kernel at the 1024^3 / 720-projection launch:
# dram__bytes_read.sum + dram__bytes_write.sum of one launch, captured with those two metrics alone
# (one ncu pass on the 64-slice slab case, so the full-size launch is captured in one pass, nothing saved or
# restored).  source_sha1 is the sha1 of tk_bp.cu + tk_bp_core.cuh at capture: a later source reports the
# traffic as stale (null) instead of a frozen number.
BP_TRAFFIC = {"kernel": "bp_quad<f16,16,8,16,2,cap6144,f32i,issue1,geo1>", "bytes_per_launch": 310.51e9 + 4.30e9,
              "source_sha1": "a79e5ca07db27cf4acb4799b067280a168fc95b7",
              "capture": "ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum --clock-control none "
                         "-k regex:bp_quad -c 1 python bench.py --steps 1 --warmup 1 --no-e2e --no-rmse --no-extras"}


def bp_source_sha1():
    import hashlib

    h = hashlib.sha1()
    for f in ("tk_bp.cu", "tk_bp_core.cuh"):
        with open(os.path.join(ROOT, "tomokvas_gb300", "csrc", f), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-rmse", action="store_true", help="skip the FP64 oracle accuracy check")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the batch and adjoint summaries")
    ap.add_argument("--variant", type=int, default=-1, help="backprojection kernel variant (-1 = default)")
    ap.add_argument("--adjoint", action="store_true",
                    help="differentiation workload: 512^3 (scale 1.5) from 360 x 768^2 FP32 projections, "
                         "time A (FDK) and A^T (transpose) and check the dot-product test")
    ap.add_argument("--outofcore", action="store_true",
                    help="out-of-core workload: 2048^3 from 1440 x 2048^2 uint16 streamed from pinned host "
                         "memory in chunks (FP16 filtered chunks), RMSE vs FP64 on 32 sampled slices")
    ap.add_argument("--batch", action="store_true",
                    help="batched workload: 64 seeded phantoms of uneven sizes (W in {128..512}, 90-360 "
                         "projections, SOD/SDD 0.3-0.6, 96^3-384^3), one persistent launch / CUDA graph vs one "
                         "launch per volume")
    ap.add_argument("--reference-gpu", action="store_true",
                    help="time the reference's own kernels (FBPG/kernel.cu built for sm_103a, cuFFT) on this GPU "
                         "at the 256^3 and 1024^3 workloads beside ours on the same log sinograms (Ram-Lak), "
                         "with the relative RMSE between the two")
    ap.add_argument("--chunk", type=int, default=480, help="projections per streamed chunk (--outofcore)")
    ap.add_argument("--items", type=int, default=64, help="with --batch: only the first ITEMS volumes (small case for ncu)")
    ap.add_argument("--profile-adjoint", action="store_true",
                    help="with --adjoint: small case for ncu, 120 instead of 360 projections (same 512^3 volume, "
                         "same row step 1.43)")
    ap.add_argument("--profile-filter", choices=["f32", "f16", "bf16", "f32c"], default=None,
                    help="small case for ncu: the u16 log + Hann filter of 90 x 1024^2 projections into one "
                         "storage format; one untimed and two timed launches")
    ap.add_argument("--sweep", action="store_true", help="with --profile-bp: time every variant of that precision")
    ap.add_argument("--filter-width", type=int, default=1024, help="with --profile-filter: detector width (and height)")
    ap.add_argument("--filter-form", choices=["auto", "fft", "toeplitz"], default="auto",
                    help="with --profile-filter: the filter form (tk_filter_select_form)")
    ap.add_argument("--probe-link", action="store_true",
                    help="time host<->device copies of the e2e leg's buffer sizes, alone and beside a busy GPU")
    ap.add_argument("--profile-bp", choices=["f32", "f16", "bf16", "f32c"], default=None,
                    help="small case for ncu: 180 x 1024^2 projections, a 64-slice slab of the 1024^2 volume; "
                         "one untimed and two timed backprojection launches")
    return ap.parse_args()


def workload():
    from tomokvas_gb300.geometry import config

    return config("c2")


def phantom(g):
    from tomokvas_gb300.phantom import random_ellipsoids

    return random_ellipsoids(N_ELLIPSOIDS, g.fov_radius_cm, g.Z * g.voxel_cm / 2, seed=PHANTOM_SEED)


CONFIG = {
    "workload": "fdk_1024cube_from_720x1024sq_u16",
    "projections": [720, 1024, 1024],
    "volume": [1024, 1024, 1024],
    "geometry": "circular 360 deg, pitch 0.15 mm, SOD 300 mm, SDD 900 mm, voxel 0.05 mm",
    "filter": "log + cosine weight + Hann-windowed ramp, pad 2048 (shared-memory FFT)",
    "input": "uint16 counts, I0=60000 (resident in HBM for value; pinned host for e2e)",
    "l2": "inputs (1.51 GB raw, 3.0 GB filtered) exceed the 129 MB L2; no flush needed",
}


# ------------------------------------------------------------------ helpers
class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    Q = ("uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid=None):
        self.uuid = uuid
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        rows = []
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            if self.uuid and self.uuid not in f[0]:
                continue
            rows.append(f)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[4 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max((float(r[3]) for r in rows if r[3].replace(".", "").isdigit()), default=None)}


def cpu_sample(g, nthreads, slices=CPU_SAMPLE_SLICES):
    """FP32 restatement of the reference (oracle port) on sampled slices, from
    raw uint16 projections generated on the CPU for the detector rows they need."""
    from oracle import oracle as orc

    G = orc.geom_from(g)
    z = np.array(slices, dtype=np.int32)
    lo, hi = orc.rows_needed(G, z)
    band = g.replace(H=hi - lo + 1, cZ=g.cZ - lo)
    line = orc.project_ellipsoids(phantom(g), orc.geom_from(band), "proj", nthreads)  # [N][band][W]
    rng = np.random.default_rng(5)
    raw = np.zeros((g.N, g.H, g.W), dtype=np.uint16)  # rows outside the band are never read
    raw[:, lo:hi + 1] = np.clip(rng.poisson(I0 * np.exp(-line.astype(np.float64))), 0, 65535)
    t0 = time.perf_counter()
    orc.fdk_u16_f32_sampled(raw, G, I0, window="hann", zlist=z, nthreads=nthreads)
    dt = time.perf_counter() - t0
    upd = len(slices) * g.X * g.Y * g.N
    return upd / dt / 1e9, dt, f"{len(slices)} central slices of the 1024^3 volume x 720 projections " \
                               f"(log/weight/filter of detector rows {lo}-{hi} only)"


def emit(obj):
    print(json.dumps(obj), flush=True)


# ------------------------------------------------- replicas (N > 1 ranks)
# One process per GPU, each reconstructing its own volume: no collective on
# the data path.  The only cross-rank steps are the barriers around the timed
# region and the maximum of the per-rank times.
def ranks_max(x: float, dist=None, device="cuda") -> float:
    """Maximum of x over all ranks (x itself without a process group)."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_gups(updates_per_rank: int, world: int, seconds: float) -> float:
    """Whole-job throughput: every rank did updates_per_rank in at most `seconds`."""
    return world * updates_per_rank / seconds / 1e9


# --------------------------------------------------------- reference arm
def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    g = workload()
    cores = os.cpu_count() or 1
    vals, secs = [], []
    sample = ""
    for i in range(args.warmup + args.steps):
        gups, dt, sample = cpu_sample(g, cores)
        if i >= args.warmup:
            vals.append(gups)
            secs.append(dt)
    v = statistics.mean(vals)
    upd = g.updates
    emit({"impl": "reference", "metric": "GUPS", "value": v, "unit": "GUPS", "n_gpus": args.gpus,
          "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(secs),
          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
          "data": "synthetic: seeded 40-ellipsoid phantom, Poisson counts I0=60000", "config": CONFIG,
          "s_per_volume": upd / (v * 1e9),
          "cpu_baseline": {"value": v, "unit": "GUPS", "cores": cores, "kind": "port", "sample": sample,
                           "what": "FP32 restatement of the reference FDK (oracle/tk_oracle.c), the reference "
                                   "has no CPU implementation of the path"},
          "e2e": {"value": v, "unit": "GUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
    return 0


# ---------------------------------------------------------------- our arm
def run_ours(args):
    import torch

    from tomokvas_gb300 import _build, _lib, device
    from tomokvas_gb300.fbp import FilteredBackProjection

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        dist = None
        torch.cuda.set_device(0)
    _build.build()
    _lib.load()
    if args.variant >= 0:  # applies to the backprojections of that variant's storage format
        _lib.check(_lib.load().tk_bp_select_variant(args.variant))

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x):
        return ranks_max(x, dist)

    g = workload()
    ell = phantom(g)
    stream = torch.cuda.current_stream()
    # synthetic raw counts, resident in HBM
    line = device.phantom_project(g, ell, _lib.TK_LAYOUT_PROJECTION)
    gen = torch.Generator(device="cuda").manual_seed(PHANTOM_SEED + rank)
    counts = torch.poisson(I0 * torch.exp(-line), generator=gen).clamp_(0, 65535)
    raw = counts.to(torch.int32).to(torch.int16)  # uint16 bits
    del line, counts
    ff = device.flatfield(flat_value=I0, A=1.0, B=0.0, invert=True, floor_counts=0.5)
    vol = torch.empty((g.Z, g.Y, g.X), dtype=torch.float32, device="cuda")
    upd = g.updates

    L = _lib.load()
    launches = {}

    def timed(precision, steps, warmup, sample_clocks=False):
        q, scale = device.alloc_filtered(g, precision)
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]

        def one(e=None):
            if e:
                e[0].record(stream)
            device.filter_projections(g, raw, _lib.TK_INPUT_U16, _lib.TK_LAYOUT_PROJECTION, ff,
                                      _lib.TK_WINDOW_HANN, precision, out=(q, scale))
            if e:
                e[1].record(stream)
            device.backproject(g, q, scale if precision in (_lib.TK_F16, _lib.TK_BF16) else None, precision,
                               vol=vol)
            if e:
                e[2].record(stream)

        for _ in range(warmup):
            one()
        barrier()
        uuid = str(getattr(torch.cuda.get_device_properties(torch.cuda.current_device()), "uuid", "") or "")
        sampler = ClockSampler(uuid or None) if sample_clocks else None
        if sampler:
            sampler.start()
            time.sleep(0.4)
        barrier()
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        n0 = L.tk_kernel_launches()
        t_start.record(stream)
        for i in range(steps):
            one(ev[i])
        t_end.record(stream)
        barrier()
        launches[precision] = L.tk_kernel_launches() - n0
        clocks = sampler.stop() if sampler else None
        total_ms = t_start.elapsed_time(t_end)
        filt = [e[0].elapsed_time(e[1]) for e in ev]
        bp = [e[1].elapsed_time(e[2]) for e in ev]
        total_ms = max_over_ranks(total_ms)
        del q, scale
        return total_ms / steps, statistics.mean(filt), statistics.mean(bp), clocks

    K, W = args.steps, args.warmup

    def slices():
        return {tuple(zs): vol[torch.tensor(zs, device="cuda")].cpu().numpy() for zs in RMSE_SLICES}

    # chosen form: FP16 storage, FP32 interpolation (the default FP16 kernel)
    ms16, f16_filter, f16_bp, clocks = timed(_lib.TK_F16, K, W, sample_clocks=(rank == 0))
    vol16 = slices()
    # the same form with bfloat16 storage (widening on the integer pipe)
    ms_bf, bf_filter, bf_bp, _ = timed(_lib.TK_BF16, K, W)
    vol_bf = slices()
    # plain form: the faster of the two FP32 storage formats (samples / coefficients)
    plain_runs = {}
    for pname, pcode in (("f32", _lib.TK_F32), ("f32c", _lib.TK_F32_COEF)):
        r = timed(pcode, K, W)
        plain_runs[pname] = (r, slices())
    plain_name = min(plain_runs, key=lambda k: plain_runs[k][0][0])
    (ms32, f32_filter, f32_bp, _), vol32 = plain_runs[plain_name]
    plain_code = _lib.TK_F32 if plain_name == "f32" else _lib.TK_F32_COEF
    plain_alt = {k: {"ms_per_step": v[0][0], "bp_ms": v[0][2], "filter_ms": v[0][1],
                     "kernel": bp_kernel_name(-1, _lib.TK_F32 if k == "f32" else _lib.TK_F32_COEF)}
                 for k, v in plain_runs.items()}
    # the FP32-coefficient quarter-turn kernel (selectable; the general walk is the faster FP32 form): the
    # chosen form's algorithm with FP32 storage, for the ratio on matched kernels
    qf32 = next(i for i in range(L.tk_bp_variant_count()) if L.tk_bp_variant_name(i).decode().startswith("quad<f32c,"))
    _lib.check(L.tk_bp_select_variant(qf32))
    try:
        ms_q32, _, q32_bp, _ = timed(_lib.TK_F32_COEF, K, W)
    finally:
        _lib.check(L.tk_bp_select_variant(args.variant))
    # the selectable FP16 half-math form (FP16 interpolation arithmetic): reported beside, not the headline
    hm = half_math_variant()
    _lib.check(L.tk_bp_select_variant(hm))
    try:
        ms_hm, hm_filter, hm_bp, _ = timed(_lib.TK_F16, K, W)
        vol_hm = slices()
    finally:
        _lib.check(L.tk_bp_select_variant(args.variant))
    value = replica_gups(upd, world, ms16 * 1e-3)
    plain = replica_gups(upd, world, ms32 * 1e-3)
    flags = device.device_error_flags()

    # end to end through the reference-facing handle: pinned host raw in, pinned host volume out
    e2e = None
    if not args.no_e2e:
        raw_h = torch.empty(raw.shape, dtype=torch.int16, pin_memory=True)
        raw_h.copy_(raw)
        vol_h = torch.empty((g.Z, g.Y, g.X), dtype=torch.float32, pin_memory=True)
        del vol
        torch.cuda.empty_cache()
        from tomokvas_gb300.fbp import VolumeSink

        zb = 128
        sink = VolumeSink(g.X, g.Y, g.Z, zb, out=vol_h.numpy())
        fbp = FilteredBackProjection(raise_on_error=True)
        fbp.SetGPUid(torch.cuda.current_device())
        fbp.SetBlockSize(zb)
        fbp.SetSinogramProperties(None, g.W, g.cX, g.N, g.H, g.cZ, g.dfi, g.D, g.tau)
        fbp.SetReconstructionProperties(sink, g.X, g.cx, g.Y, g.cy, g.Z, g.cz, g.rot)
        fbp.SetScaleXYZ(g.scale)
        fbp.SetFilter("hann")
        fbp.SetPrecision("f16")
        fbp.SetPipeline(True)  # as the C++ FilteredBackProjection: reconstruct while the chunks land
        raw_np = raw_h.numpy().view(np.uint16)

        parts = {"initialize_s": [], "reconstruction_s": [], "upload_ms": [], "d2h_tail_ms": [], "gpu_ms": []}

        def e2e_step(record=False):
            fbp.SetProjectionsU16(raw_np, "projection", flat_value=I0)
            t_a = time.perf_counter()
            fbp.Initialize()  # upload in 4 angle chunks, each filtered and backprojected as it lands
            t_b = time.perf_counter()
            fbp.CalculateReconstruction()  # D2H of each Z block once its last backprojection has run
            if record:
                parts["initialize_s"].append(t_b - t_a)
                parts["reconstruction_s"].append(time.perf_counter() - t_b)
                tm = fbp.Timings()
                parts["upload_ms"].append(round(tm["h2d_ms"], 2))
                parts["d2h_tail_ms"].append(round(tm["d2h_ms"], 2))
                parts["gpu_ms"].append(round(tm["bp_ms"], 2))  # pipelined: filter + backprojection span

        for _ in range(W):
            e2e_step()
        barrier()
        t0 = time.perf_counter()
        for _ in range(K):
            e2e_step(True)
        barrier()
        e2e_s = max_over_ranks((time.perf_counter() - t0) / K)
        timings = fbp.Timings()
        fbp.close()
        e2e = {"value": replica_gups(upd, world, e2e_s), "unit": "GUPS", "s_per_volume": e2e_s,
               "initialize_s": statistics.mean(parts["initialize_s"]),
               "reconstruction_s": statistics.mean(parts["reconstruction_s"]),
               "steps_s": [round(a + b, 5) for a, b in zip(parts["initialize_s"], parts["reconstruction_s"])],
               "initialize_steps_s": [round(a, 5) for a in parts["initialize_s"]],
               "upload_ms": timings["h2d_ms"], "upload_steps_ms": parts["upload_ms"],
               "d2h_tail_steps_ms": parts["d2h_tail_ms"], "gpu_span_steps_ms": parts["gpu_ms"],
               "h2d_bytes_per_step": int(raw.numel() * 2), "d2h_bytes_per_step": int(g.X * g.Y * g.Z * 4),
               "api": "C ABI tk_fdk_* (FilteredBackProjection mirror): u16 projections from pinned host, "
                      "volume to pinned host via the bin_siz-style block sink, 128-slice blocks, pipelined "
                      "(tk_fdk_set_pipeline)"}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    # compact summaries of the batched (64 uneven volumes) and differentiation (512^3 from
    # 360 x 768^2) workloads, after the headline's timed regions
    extras = {}
    if not args.no_extras:
        torch.cuda.empty_cache()
        extras["c3_batch"] = batch_summary(steps=3, warmup=1)
        torch.cuda.empty_cache()
        extras["c4_adjoint"] = adjoint_summary(steps=3, warmup=1)
        torch.cuda.empty_cache()

    # accuracy on sampled slices vs the FP64 oracle (untimed)
    rmse = None
    if not args.no_rmse:
        from oracle import oracle as orc

        G = orc.geom_from(g)
        raw_np = raw.cpu().numpy().view(np.uint16)
        sino = orc.log_u16(raw_np, np.float32(I0))
        num16 = num32 = numhm = numbf = den = 0.0
        for zs in RMSE_SLICES:
            ref = orc.fdk_f64(sino, G, "hann", np.array(zs, dtype=np.int32))
            num16 += float(np.sum((vol16[tuple(zs)] - ref) ** 2))
            numbf += float(np.sum((vol_bf[tuple(zs)] - ref) ** 2))
            num32 += float(np.sum((vol32[tuple(zs)] - ref) ** 2))
            numhm += float(np.sum((vol_hm[tuple(zs)] - ref) ** 2))
            den += float(np.sum(ref ** 2))
        del sino
        rmse = {"chosen_f16_vs_fp64": (num16 / den) ** 0.5, "plain_f32_vs_fp64": (num32 / den) ** 0.5,
                "half_math_f16_vs_fp64": (numhm / den) ** 0.5, "bf16_vs_fp64": (numbf / den) ** 0.5,
                "slices": [z for zs in RMSE_SLICES for z in zs], "metric": "relative RMSE"}

    cores = os.cpu_count() or 1
    cpu_gups, cpu_s, sample = cpu_sample(g, cores)

    bp_tflops = upd * FLOPS_PER_UPDATE / (f16_bp * 1e-3) / 1e12
    fma_peak = ctypes.c_double(0.0)
    _lib.check(L.tk_measure_fp32_fma_rate(ctypes.byref(fma_peak)))
    fp32_peak = fma_peak.value
    kname = bp_kernel_name(args.variant)
    traffic, traffic_note = None, "no capture recorded for this kernel"
    if BP_TRAFFIC["kernel"] == kname:
        if BP_TRAFFIC["source_sha1"] == bp_source_sha1():
            traffic = int(BP_TRAFFIC["bytes_per_launch"])
            traffic_note = f"one-pass ncu capture of a full-size launch: {BP_TRAFFIC['capture']}"
        else:
            traffic_note = "stale: the backprojection source changed after the capture"
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    bp_bytes = g.N * g.H * g.W * 8 + g.X * g.Y * g.Z * 4  # FP16 coefficient image read once + volume written once
    out = {
        "metric": "GUPS", "value": value, "unit": "GUPS", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms16, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f16-stored filtered projections (bilinear coefficient image, 8 B/entry); f32 geometry, "
                 "f32 bilinear interpolation (16-bit values converted exactly to f32), f32 U^2 weighting and "
                 "accumulation", "data": "synthetic: seeded 40-ellipsoid phantom, "
        "Poisson counts I0=60000 (no dataset)", "config": CONFIG,
        "s_per_volume": ms16 * 1e-3,
        "kernel": kname,
        "plain": {"value": plain, "unit": "GUPS", "ms_per_step": ms32, "s_per_volume": ms32 * 1e-3,
                  "dtype": "f32 math, f32-stored filtered projections", "storage": plain_name,
                  "kernel": plain_alt[plain_name]["kernel"],
                  "filter_ms": f32_filter, "bp_ms": f32_bp, "formats": plain_alt},
        "chosen_vs_plain": plain and value / plain,
        "chosen_vs_plain_kernels": [kname, plain_alt[plain_name]["kernel"]],
        "chosen_vs_plain_matched": {"ratio": ms_q32 / ms16, "kernels": [kname, "bp_" + L.tk_bp_variant_name(qf32).decode()],
                                    "plain_ms_per_step": ms_q32, "plain_bp_ms": q32_bp,
                                    "note": "both quarter-turn kernels with FP32 interpolation; storage FP16 vs FP32 "
                                            "coefficients (8 vs 16 B per entry)"},
        "bf16": {"value": replica_gups(upd, world, ms_bf * 1e-3), "unit": "GUPS", "ms_per_step": ms_bf,
                 "bp_ms": bf_bp, "filter_ms": bf_filter, "kernel": bp_kernel_name(-1, _lib.TK_BF16),
                 "dtype": "bf16-stored filtered projections, f32 bilinear interpolation and accumulation",
                 "rmse_vs_fp64": rmse and rmse["bf16_vs_fp64"],
                 "vs_plain": plain and replica_gups(upd, world, ms_bf * 1e-3) / plain},
        "half_math": {"value": replica_gups(upd, world, ms_hm * 1e-3), "unit": "GUPS", "ms_per_step": ms_hm,
                      "bp_ms": hm_bp, "filter_ms": hm_filter, "kernel": bp_kernel_name(hm),
                      "dtype": "f16 storage with f16 interpolation arithmetic (HFMA2 column and FP16 row "
                               "interpolation, U^2 rounded to f16, f32 accumulation): a selectable form, not "
                               "the headline",
                      "rmse_vs_fp64": rmse and rmse["half_math_f16_vs_fp64"]},
        "stages_ms": {"filter": f16_filter, "backprojection": f16_bp},
        "rmse": rmse,
        "e2e": e2e,
        "gpu_launches": launches[_lib.TK_F16],
        "device_error_flags": flags,
        "roofline": {"bound": "fp32", "kernel": bp_kernel_name(args.variant),
                     "achieved": bp_tflops, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": bp_tflops / fp32_peak, "traffic": traffic, "traffic_note": traffic_note,
                     "flops_per_update": FLOPS_PER_UPDATE, "peak_nominal": PEAK_FP32_NOMINAL,
                     "frac_of_nominal": bp_tflops / PEAK_FP32_NOMINAL,
                     "peak_source": "measured live on this GPU: FP32 FMA throughput kernel "
                                    "(tk_measure_fp32_fma_rate); MEASURED_PEAKS.json has no FP32 figure and the "
                                    "kernel is bound by the FP32 pipe, not by HBM or the tensor cores; nominal "
                                    "152 SM x 128 lanes x 2 x 2070 MHz beside it"},
        "roofline_hbm": {"bound": "hbm", "achieved": bp_bytes / (f16_bp * 1e-3) / 1e9, "peak": hbm_peak,
                         "unit": "GB/s", "frac": bp_bytes / (f16_bp * 1e-3) / 1e9 / hbm_peak,
                         "note": "algorithmic bytes of the backprojection (informational)"},
        "cpu_baseline": {"value": cpu_gups, "unit": "GUPS", "cores": cores, "kind": "port", "sample": sample,
                         "seconds": cpu_s},
        "clocks": clocks,
        **extras,
    }
    emit(out)
    if dist:
        dist.destroy_process_group()
    return 0


def run_profile_bp(args):
    """Backprojection-only case small enough for an ncu capture (inputs > L2)."""
    import torch

    from tomokvas_gb300 import _build, _lib, device

    _build.build()
    torch.cuda.set_device(0)
    g = workload().replace(N=180, dfi=float(np.float32(2.0 * np.pi / 180)))
    prec = _lib.PRECISIONS[args.profile_bp]
    line = device.phantom_project(g, phantom(g), _lib.TK_LAYOUT_PROJECTION)
    q, scale = device.filter_projections(g, line, _lib.TK_INPUT_F32, _lib.TK_LAYOUT_PROJECTION,
                                         window=_lib.TK_WINDOW_HANN, precision=prec)
    del line
    nz = 64
    vol = torch.empty((nz, g.Y, g.X), dtype=torch.float32, device="cuda")
    zoff = -(g.Z - 1) / 2.0 + (g.Z - nz) / 2.0  # the central slab
    sc = scale if prec in (_lib.TK_F16, _lib.TK_BF16) else None
    L = _lib.load()
    variants = [args.variant]
    if args.sweep:
        variants = [i for i in range(L.tk_bp_variant_count()) if L.tk_bp_variant_precision(i) == prec]
    upd = nz * g.X * g.Y * g.N
    for vi in variants:
        _lib.check(L.tk_bp_select_variant(vi))
        device.backproject(g, q, sc, prec, vol=vol, nz=nz, zoff=zoff)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(2):
            device.backproject(g, q, sc, prec, vol=vol, nz=nz, zoff=zoff)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 2
        name = L.tk_bp_variant_name(vi).decode() if vi >= 0 else "default"
        emit({"profile_bp": args.profile_bp, "variant": name, "ms_per_launch": ms,
              "gups": upd / (ms * 1e-3) / 1e9, "updates_per_launch": upd, "flags": device.device_error_flags()})
    _lib.check(L.tk_bp_select_variant(-1))
    return 0


def run_probe_link(args):
    """The host link, for the e2e leg's step-to-step spread: the 1.51 GB uint16 projections
    host -> device and the 4.29 GB volume device -> host, as one copy each and as eight chunk copies,
    from the same page-locked buffers in a loop with no kernel launched; the same copies while
    device-to-device copies or the backprojection kernel run on another stream; the e2e leg's
    handle steps, each after a bare upload of the same buffer; then copies from buffers page-locked
    afresh for every copy.  CUDA events on the copy stream time each copy."""
    import torch

    torch.cuda.set_device(0)
    g = workload()
    n_in, n_vol = g.N * g.H * g.W, g.X * g.Y * g.Z
    raw_h = torch.empty(n_in, dtype=torch.int16, pin_memory=True)
    vol_h = torch.empty(n_vol, dtype=torch.float32, pin_memory=True)
    raw_d = torch.randint(0, 32767, (n_in,), dtype=torch.int16, device="cuda")
    raw_h.copy_(raw_d)  # filled from the device, as the e2e leg fills its buffer
    vol_d = torch.zeros(n_vol, dtype=torch.float32, device="cuda")
    st = torch.cuda.Stream()
    reps = max(args.steps, 4)

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(st):
            e0.record(st)
            fn()
            e1.record(st)
        e1.synchronize()
        return round(e0.elapsed_time(e1), 2)

    def chunks(dst, src, k=8):
        step = (dst.numel() + k - 1) // k
        for a in range(0, dst.numel(), step):
            dst[a:a + step].copy_(src[a:a + step], non_blocking=True)

    out = {"h2d_ms": [], "d2h_ms": [], "h2d_chunked_ms": [], "d2h_chunked_ms": [], "h2d_fresh_ms": [],
           "d2h_fresh_ms": []}
    for _ in range(reps):
        out["h2d_ms"].append(timed(lambda: raw_d.copy_(raw_h, non_blocking=True)))
        out["d2h_ms"].append(timed(lambda: vol_h.copy_(vol_d, non_blocking=True)))
    for _ in range(reps):
        out["h2d_chunked_ms"].append(timed(lambda: chunks(raw_d, raw_h)))
        out["d2h_chunked_ms"].append(timed(lambda: chunks(vol_h, vol_d)))
    # the same copies while the GPU is busy on another stream: device-to-device copies (HBM bound),
    # then the backprojection kernel of the 1024^3 workload (on zero-filled FP16 entries)
    busy = torch.cuda.Stream()
    big_a = torch.zeros(1 << 30, dtype=torch.float32, device="cuda")
    big_b = torch.empty_like(big_a)
    out["h2d_under_d2d_ms"], out["h2d_under_bp_ms"], out["d2h_under_bp_ms"] = [], [], []
    for _ in range(reps):
        with torch.cuda.stream(busy):
            for _ in range(8):
                big_b.copy_(big_a)
        out["h2d_under_d2d_ms"].append(timed(lambda: raw_d.copy_(raw_h, non_blocking=True)))
        torch.cuda.synchronize()
    del big_a, big_b
    from tomokvas_gb300 import _lib, device

    q, sc = device.alloc_filtered(g, _lib.TK_F16)
    q.zero_()
    vol = torch.empty((g.Z, g.Y, g.X), dtype=torch.float32, device="cuda")
    for _ in range(reps):
        device.backproject(g, q, sc, _lib.TK_F16, vol=vol, stream=busy)
        out["h2d_under_bp_ms"].append(timed(lambda: raw_d.copy_(raw_h, non_blocking=True)))
        out["d2h_under_bp_ms"].append(timed(lambda: vol_h.copy_(vol_d, non_blocking=True)))
        torch.cuda.synchronize()
    del q, vol
    # the e2e leg's handle steps, each preceded by a 1 MB and a whole bare upload, of the handle's
    # buffer or of another buffer of the same size: whether the first upload after a step is slow
    # whoever issues it and whatever it reads, and whether a small copy takes the delay
    from tomokvas_gb300.fbp import FilteredBackProjection, VolumeSink

    sink = VolumeSink(g.X, g.Y, g.Z, 128, out=vol_h.numpy().reshape(g.Z, g.Y, g.X))
    fbp = FilteredBackProjection(raise_on_error=True)
    fbp.SetBlockSize(128)
    fbp.SetSinogramProperties(None, g.W, g.cX, g.N, g.H, g.cZ, g.dfi, g.D, g.tau)
    fbp.SetReconstructionProperties(sink, g.X, g.cx, g.Y, g.cy, g.Z, g.cz, g.rot)
    fbp.SetScaleXYZ(g.scale)
    fbp.SetFilter("hann")
    fbp.SetPrecision("f16")
    fbp.SetPipeline(True)
    raw_np = raw_h.numpy().view(np.uint16)
    out["h2d_1mb_before_handle_ms"], out["before_handle_source"] = [], []
    out["h2d_before_handle_ms"], out["handle_upload_ms"], out["handle_step_s"] = [], [], []
    small = 1 << 19  # 1 MB of the same buffer
    other_h = torch.empty_like(raw_h, pin_memory=True)  # a second page-locked buffer of the same size
    other_h.copy_(raw_d)
    for i in range(reps + 2):
        src = raw_h if i % 2 else other_h  # the bare upload reads the handle's buffer or another one
        pre_small = timed(lambda: raw_d[:small].copy_(src[:small], non_blocking=True))
        pre = timed(lambda: raw_d.copy_(src, non_blocking=True))
        fbp.SetProjectionsU16(raw_np, "projection", flat_value=I0)
        t0 = time.perf_counter()
        fbp.Initialize()
        fbp.CalculateReconstruction()
        dt = time.perf_counter() - t0
        if i >= 2:  # two warm-up steps
            out["h2d_1mb_before_handle_ms"].append(pre_small)
            out["before_handle_source"].append("same" if i % 2 else "other")
            out["h2d_before_handle_ms"].append(pre)
            out["handle_upload_ms"].append(round(fbp.Timings()["h2d_ms"], 2))
            out["handle_step_s"].append(round(dt, 4))
    fbp.close()
    del raw_h, vol_h, other_h
    for _ in range(min(reps, 4)):
        rh = torch.zeros(n_in, dtype=torch.int16, pin_memory=True)
        vh = torch.empty(n_vol, dtype=torch.float32, pin_memory=True)
        out["h2d_fresh_ms"].append(timed(lambda: raw_d.copy_(rh, non_blocking=True)))
        out["d2h_fresh_ms"].append(timed(lambda: vh.copy_(vol_d, non_blocking=True)))
        del rh, vh
    gb_in, gb_vol = n_in * 2 / 1e9, n_vol * 4 / 1e9
    out["h2d_gbs"] = [round(gb_in / (t * 1e-3), 1) for t in out["h2d_ms"]]
    out["d2h_gbs"] = [round(gb_vol / (t * 1e-3), 1) for t in out["d2h_ms"]]
    emit({"probe_link": out, "h2d_bytes": n_in * 2, "d2h_bytes": n_vol * 4,
          "note": "each copy timed with CUDA events on its own stream; *_under_* copies run beside "
                  "device-to-device copies or the backprojection kernel on another stream"})
    return 0


def run_profile_filter(args):
    """Filter-only case small enough for an ncu capture: 90 x 1024^2 uint16 projections (189 MB in,
    0.38-1.5 GB out, above L2)."""
    import torch

    from tomokvas_gb300 import _build, _lib, device

    _build.build()
    torch.cuda.set_device(0)
    g = workload().replace(N=90, dfi=float(np.float32(2.0 * np.pi / 90)))
    if args.filter_width != g.W:  # 360 frames of W x W at the same geometry
        Wf = args.filter_width
        g = g.replace(N=360, dfi=float(np.float32(2.0 * np.pi / 360)), W=Wf, H=Wf, cX=(Wf - 1) / 2.0,
                      cZ=(Wf - 1) / 2.0, X=min(g.X, Wf), Y=min(g.Y, Wf), Z=min(g.Z, Wf))
    prec = _lib.PRECISIONS[args.profile_filter]
    L = _lib.load()
    _lib.check(L.tk_filter_select_form({"auto": _lib.TK_FILTER_AUTO, "fft": _lib.TK_FILTER_FFT,
                                        "toeplitz": _lib.TK_FILTER_TOEPLITZ}[args.filter_form]))
    line = device.phantom_project(g, phantom(g), _lib.TK_LAYOUT_PROJECTION)
    gen = torch.Generator(device="cuda").manual_seed(PHANTOM_SEED)
    raw = torch.poisson(I0 * torch.exp(-line), generator=gen).clamp_(0, 65535).to(torch.int32).to(torch.int16)
    del line
    ff = device.flatfield(flat_value=I0, A=1.0, B=0.0, invert=True, floor_counts=0.5)
    q, scale = device.alloc_filtered(g, prec)

    def one():
        device.filter_projections(g, raw, _lib.TK_INPUT_U16, _lib.TK_LAYOUT_PROJECTION, ff, _lib.TK_WINDOW_HANN,
                                  prec, out=(q, scale))

    one()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(2):
        one()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 2
    samples = g.N * g.H * g.W
    out_bytes = device.filtered_bytes(g, prec)
    emit({"profile_filter": args.profile_filter, "W": g.W, "N": g.N,
          "form": "toeplitz" if L.tk_filter_form_for(g.W, prec) == _lib.TK_FILTER_TOEPLITZ else "fft",
          "ms_per_call": ms, "samples": samples,
          "gsamples_per_s": samples / (ms * 1e-3) / 1e9,
          "hbm_algorithmic_gbs": (samples * 2 + out_bytes) / (ms * 1e-3) / 1e9,
          "flags": device.device_error_flags()})
    return 0


def adjoint_summary(steps, warmup, column_lanes=False, descent_p=False, refine_steps=20, profile=False):
    """A and A^T on the 512^3 / 360 x 768^2 differentiation workload: times, the full-size dot-product
    test, and data-consistency steps on the volume from the FDK volume (tk_refine_volume, filtered
    projections checkpointed in FP16)."""
    import torch

    from tomokvas_gb300 import _lib, device
    from tomokvas_gb300.geometry import FDKGeometry, config
    from tomokvas_gb300.phantom import random_ellipsoids

    g = config("c4")
    if profile:
        g = FDKGeometry.circular(120, 768, 768, 0.2, 400.0, 800.0, (512, 512, 512), 0.15)
    ell = random_ellipsoids(20, g.fov_radius_cm, g.Z * g.voxel_cm / 2, seed=4)
    p = device.phantom_project(g, ell, _lib.TK_LAYOUT_SINOGRAM)
    gen = torch.Generator(device="cuda").manual_seed(9)
    p += 0.01 * float(p.max().item()) * torch.randn(p.shape, device="cuda", generator=gen)
    y = torch.randn((g.Z, g.Y, g.X), device="cuda", generator=gen)
    ws = torch.empty(device.workspace_bytes(g, _lib.TK_F32), dtype=torch.uint8, device="cuda")
    vol = torch.empty((g.Z, g.Y, g.X), device="cuda")
    grad = torch.empty_like(p)

    def fwd():
        device.fdk_device(g, p, workspace=ws, vol=vol)

    def bwd():
        device.fdk_backward(g, y, workspace=ws, out=grad)

    def timeit(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    res = {}
    L = _lib.load()
    if column_lanes:  # the other forward-projector forms, timed beside the default
        for v, key in ((1, "backward_column_lanes"), (2, "backward_fp32_atomics")):
            try:
                _lib.check(L.tk_fp_select_variant(v))
                ms = timeit(bwd)
                res[key] = {"ms": ms, "gups": g.updates / (ms * 1e-3) / 1e9}
            finally:
                _lib.check(L.tk_fp_select_variant(0))
    for name, fn in (("forward", fwd), ("backward", bwd)):
        ms = timeit(fn)
        res[name] = {"ms": ms, "gups": g.updates / (ms * 1e-3) / 1e9}
    res["backward_over_forward"] = res["backward"]["ms"] / res["forward"]["ms"]
    lhs = float(torch.sum(vol.double() * y.double()).item())
    rhs = float(torch.sum(p.double() * grad.double()).item())
    res["dot_product_rel_err"] = abs(lhs - rhs) / abs(lhs)
    if column_lanes:
        try:
            _lib.check(L.tk_fp_select_variant(2))
            bwd()
            rhs2 = float(torch.sum(p.double() * grad.double()).item())
            res["backward_fp32_atomics"]["dot_product_rel_err"] = abs(lhs - rhs2) / abs(lhs)
        finally:
            _lib.check(L.tk_fp_select_variant(0))
    if descent_p:
        # 20 steps p <- p - a grad ||A p - t||^2 from the noisy projections toward the volume of the
        # noise-free ones (t = A p_clean); a from a power-iteration estimate of ||A||^2
        clean = device.phantom_project(g, ell, _lib.TK_LAYOUT_SINOGRAM)
        t = torch.empty_like(vol)
        device.fdk_device(g, clean, workspace=ws, vol=t)
        del clean
        v = torch.randn(p.shape, device="cuda", generator=gen)
        for _ in range(6):
            device.fdk_device(g, v, workspace=ws, vol=vol)
            device.fdk_backward(g, vol, workspace=ws, out=grad)
            nrm = float(torch.linalg.vector_norm(grad).item())
            v = grad / nrm
        del v
        a = 0.9 / nrm
        pk = p.clone()
        losses = []
        float(torch.sum(t.double() ** 2).item())  # the loss reduction's first use loads its kernel (seconds)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(20):
            device.fdk_device(g, pk, workspace=ws, vol=vol)
            vol -= t
            losses.append(torch.sum(vol.double() ** 2))
            device.fdk_backward(g, vol, workspace=ws, out=grad)
            pk.add_(grad, alpha=-a)
        e1.record()
        torch.cuda.synchronize()
        ls = [float(x.item()) for x in losses]
        res["descent_on_projections"] = {
            "steps": 20, "ms_per_step": e0.elapsed_time(e1) / 20, "step_size": a, "loss_ratio": ls[-1] / ls[0],
            "monotone": all(b < c for c, b in zip(ls, ls[1:]))}
        del pk, t
    if refine_steps > 0:
        # volume refinement x <- x - alpha B (B^T x - q) from the FDK volume, q checkpointed in FP16
        del grad
        rws = device.refine_workspace(g)
        ck = device.refine_checkpoint(g, p, precision=_lib.TK_F16, workspace=rws)
        alpha = device.refine_step_size(g, iters=6, vol_tmp=y, workspace=rws)
        x = torch.empty((g.Z, g.Y, g.X), device="cuda")
        device.fdk_device(g, p, workspace=ws, vol=x)
        loss = torch.zeros(refine_steps, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n0 = L.tk_kernel_launches()
        e0.record()
        device.refine_volume(g, ck, x, alpha, refine_steps, loss=loss, workspace=rws)
        e1.record()
        torch.cuda.synchronize()
        ls = loss.cpu().numpy()
        res["refine_volume"] = {
            "steps": refine_steps, "ms_per_step": e0.elapsed_time(e1) / refine_steps, "step_size": alpha,
            "loss_first": float(ls[0]), "loss_last": float(ls[-1]), "loss_ratio": float(ls[-1] / ls[0]),
            "monotone": bool(np.all(np.diff(ls) < 0)),
            "launches_per_step": (L.tk_kernel_launches() - n0) / refine_steps,
            "checkpoint": "filtered projections q = F W p as FP16 samples (0.42 GB instead of 0.85 GB FP32)",
            "per_step": "B^T x (scatter forward projector) + residual -alpha (B^T x - q) with the loss + "
                        "B r accumulated into x (FP32 backprojector)"}
        del rws, ck, x
    res["flags"] = device.device_error_flags()
    return {"workload": f"fdk_adjoint_512cube_scale1.5_from_{g.N}x768sq_f32", "updates": g.updates, **res}


def run_adjoint(args):
    import torch

    from tomokvas_gb300 import _build

    _build.build()
    torch.cuda.set_device(0)
    emit(adjoint_summary(args.steps, args.warmup, column_lanes=True, descent_p=not args.profile_adjoint,
                         refine_steps=0 if args.profile_adjoint else 20, profile=args.profile_adjoint))
    return 0


def run_outofcore(args):
    """2048^3 FP32 volume held in HBM from 1440 x 2048^2 uint16 projections that
    stay in pinned host memory and stream to the GPU in chunks (tk_fdk_stream):
    the copy of the next chunks overlaps the filter and backprojection of the
    current one.  Synthetic: seeded 100-ellipsoid phantom, Poisson counts
    I0 = 50000, Hann ramp padded to 4096."""
    import torch

    from tomokvas_gb300 import _build, _lib, device
    from tomokvas_gb300.geometry import config
    from tomokvas_gb300.phantom import random_ellipsoids

    _build.build()
    torch.cuda.set_device(0)
    g = config("c5")
    I0c = 50000.0
    ell = random_ellipsoids(100, g.fov_radius_cm, g.Z * g.voxel_cm / 2, seed=5)
    # raw counts: generated on the GPU, kept in page-locked host memory (12.1 GB)
    raw_h = torch.empty((g.N, g.H, g.W), dtype=torch.int16, pin_memory=True)
    line = device.phantom_project(g, ell, _lib.TK_LAYOUT_PROJECTION)
    gen = torch.Generator(device="cuda").manual_seed(55)
    for b0 in range(0, g.N, 96):
        c = torch.poisson(I0c * torch.exp(-line[b0:b0 + 96]), generator=gen).clamp_(0, 65535)
        raw_h[b0:b0 + 96].copy_(c.to(torch.int32).to(torch.int16))
        del c
    del line
    torch.cuda.empty_cache()
    ff = device.flatfield(flat_value=I0c, A=1.0, B=0.0, invert=True, floor_counts=0.5)
    prec = _lib.TK_F16
    ws = torch.empty(device.stream_workspace_bytes(g, _lib.TK_INPUT_U16, prec, args.chunk), dtype=torch.uint8,
                     device="cuda")
    vol = torch.empty((g.Z, g.Y, g.X), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def step():
        device.fdk_stream(g, raw_h, _lib.TK_INPUT_U16, ff=ff, window=_lib.TK_WINDOW_HANN, precision=prec,
                          chunk=args.chunk, workspace=ws, vol=vol, stream=stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) / args.steps
    ms = e0.elapsed_time(e1) / args.steps
    flags = device.device_error_flags()
    zs = np.linspace(0, g.Z - 1, 32).round().astype(np.int32)
    sl = vol[torch.from_numpy(zs).long().cuda()].cpu().numpy()
    rmse = None
    if not args.no_rmse:
        from oracle import oracle as orc

        t1 = time.perf_counter()
        ref = orc.fdk_u16_f64_sampled(raw_h.numpy().view(np.uint16), orc.geom_from(g), I0c, window="hann",
                                      zlist=zs, nthreads=os.cpu_count() or 1)
        rmse = {"chosen_f16_vs_fp64": float(np.sqrt(np.sum((sl - ref) ** 2) / np.sum(ref ** 2))),
                "max_abs_rel": float(np.abs(sl - ref).max() / np.abs(ref).max()), "slices": zs.tolist(),
                "metric": "relative RMSE over 32 full 2048^2 slices", "oracle_s": time.perf_counter() - t1}
    emit({"workload": "fdk_outofcore_2048cube_from_1440x2048sq_u16_streamed", "metric": "GUPS",
          "value": g.updates / (ms * 1e-3) / 1e9, "unit": "GUPS", "s_per_volume": ms * 1e-3,
          "wall_s_per_volume": wall, "steps": args.steps, "warmup": args.warmup, "chunk": args.chunk,
          "updates": g.updates, "h2d_bytes_per_step": int(raw_h.numel() * 2), "storage": "f16 coefficients",
          "device_bytes": int(ws.numel() + vol.numel() * 4), "rmse": rmse, "flags": flags,
          "data": "synthetic: seeded 100-ellipsoid phantom, Poisson counts I0=50000 (no dataset)"})
    return 0


def batch_geometries(n=64, seed=3):
    """The uneven batch: square detectors W in {128,192,256,384,512} at 0.2 mm, 90-360 projections,
    SOD 300 mm with SOD/SDD in [0.3, 0.6], cubic volumes of 96-384 voxels covering the field of view
    where the tile footprint allows (scale <= 1.5)."""
    from tomokvas_gb300.geometry import FDKGeometry

    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        W = int(rng.choice([128, 192, 256, 384, 512]))
        N = int(rng.integers(90, 361))
        ratio = float(rng.uniform(0.3, 0.6))
        nv = int(rng.integers(96, 385))
        sod, pitch = 300.0, 0.2
        sdd = sod / ratio
        s = min(0.9 * W / nv, 1.5)
        out.append(FDKGeometry.circular(N, W, W, pitch, sod, sdd, (nv, nv, nv), s * pitch * sod / sdd))
    return out


def batch_summary(steps, warmup, items=64):
    """64 uneven reconstructions: one launch per volume vs the batched persistent launch (eager and as a
    CUDA graph), after the autotuner picked each item's filter form and the batch's tile shape."""
    import torch

    from tomokvas_gb300 import _lib, device
    from tomokvas_gb300.batch import Batch
    from tomokvas_gb300.phantom import random_ellipsoids

    geos = batch_geometries()[:max(1, items)]
    prec = _lib.TK_F16
    ins, vols, wss = [], [], []
    for k, g in enumerate(geos):
        ell = random_ellipsoids(20, g.fov_radius_cm, g.Z * g.voxel_cm / 2, seed=100 + k)
        ins.append(device.phantom_project(g, ell, _lib.TK_LAYOUT_SINOGRAM))
        vols.append(torch.empty((g.Z, g.Y, g.X), device="cuda"))
        wss.append(torch.empty(device.workspace_bytes(g, prec), dtype=torch.uint8, device="cuda"))
    updates = sum(g.updates for g in geos)
    stream = torch.cuda.current_stream()

    def timeit(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    def per_volume():
        for g, x, v, w in zip(geos, ins, vols, wss):
            device.fdk_device(g, x, precision=prec, workspace=w, vol=v)

    ms_single = timeit(per_volume)
    ref = [v[v.shape[0] // 2].cpu().numpy() for v in vols]
    b = Batch(prec)
    for g, x, v in zip(geos, ins, vols):
        b.submit(g, x, v)
    b.plan()
    tuned, tune_ms = b.autotune()
    forms = b.filter_forms()
    ms_eager = timeit(lambda: b.run(graph=False))
    filt_ms, bp_ms = b.timings()  # phases of the last eager run
    ms_graph = timeit(lambda: b.run(graph=True))
    diff = max(float(np.abs(v[v.shape[0] // 2].cpu().numpy() - r).max() / max(np.abs(r).max(), 1e-30))
               for v, r in zip(vols, ref))
    flags = device.device_error_flags()
    by_width = {}
    for g, f in zip(geos, forms):
        k = "toeplitz" if f == _lib.TK_FILTER_TOEPLITZ else "fft"
        by_width.setdefault(str(g.W), {"fft": 0, "toeplitz": 0})[k] += 1
    b.close()
    return {"workload": f"batch_{len(geos)}_uneven_fdk", "metric": "GUPS", "unit": "GUPS", "items": len(geos),
            "updates": updates, "storage": "f16 coefficients, f32 interpolation", "steps": steps, "warmup": warmup,
            "per_volume": {"ms": ms_single, "gups": updates / (ms_single * 1e-3) / 1e9},
            "batch_eager": {"ms": ms_eager, "gups": updates / (ms_eager * 1e-3) / 1e9,
                            "filter_phase_ms": filt_ms, "backprojection_ms": bp_ms},
            "batch_graph": {"ms": ms_graph, "gups": updates / (ms_graph * 1e-3) / 1e9},
            "speedup_graph_vs_per_volume": ms_single / ms_graph, "autotuned_variant": tuned,
            "autotune_ms": tune_ms, "filter_forms_by_width": by_width,
            "max_rel_diff_vs_per_volume_mid_slices": diff, "flags": flags,
            "data": f"synthetic: {len(geos)} seeded 20-ellipsoid phantoms, analytic FP32 line integrals (no dataset)"}


def run_batch(args):
    import torch

    from tomokvas_gb300 import _build

    _build.build()
    torch.cuda.set_device(0)
    emit(batch_summary(args.steps, args.warmup, args.items))
    return 0


def run_reference_gpu(args):
    """The reference's FDK kernels vs ours on the same GPU and inputs.  The
    reference reads FP32 log sinograms [H][N][W] and has only the Ram-Lak
    filter, so both sides get that; its Z blocks are 30 slices (setting.xml)."""
    import torch

    from oracle import ref_build, refrun
    from tomokvas_gb300 import _build, _lib, device
    from tomokvas_gb300.geometry import config

    _build.build()
    torch.cuda.set_device(0)
    if ref_build.build_fatbin() is None:
        emit({"reference_gpu": "unavailable: oracle/_ref/tk_ref_kernels.fatbin missing"})
        return 0
    out = {}
    for name, seed in (("c1", 1), ("c2", 2), ("c4", 4)):
        g = config(name).replace(zb=30)
        from tomokvas_gb300.phantom import random_ellipsoids

        ell = random_ellipsoids(40, g.fov_radius_cm, g.Z * g.voxel_cm / 2, seed=seed)
        line = device.phantom_project(g, ell, _lib.TK_LAYOUT_SINOGRAM)
        gen = torch.Generator(device="cuda").manual_seed(seed)
        counts = torch.poisson(I0 * torch.exp(-line), generator=gen).clamp_(min=0.5)
        sino = -torch.log(counts / I0)  # FP32 log sinogram [H][N][W], the reference's input
        del line, counts
        host = sino.cpu().numpy()
        # ours, same input, Ram-Lak: FP32 samples (the reference's arithmetic) and the chosen FP16 form
        res = {}
        vols = {}
        for pname, prec in (("f32", _lib.TK_F32), ("f16", _lib.TK_F16)):
            ws = torch.empty(device.workspace_bytes(g, prec), dtype=torch.uint8, device="cuda")
            vol = torch.empty((g.Z, g.Y, g.X), device="cuda")
            for _ in range(2):
                device.fdk_device(g, sino, precision=prec, workspace=ws, vol=vol)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(3):
                device.fdk_device(g, sino, precision=prec, workspace=ws, vol=vol)
            e1.record()
            torch.cuda.synchronize()
            res[pname] = e0.elapsed_time(e1) / 3
            vols[pname] = vol.cpu().numpy()
            del ws, vol
        del sino
        torch.cuda.empty_cache()
        times = {}
        refrun.fdk(host, g, times) if name == "c1" else None  # warm-up (module load, cuFFT plans) on the small case
        t0 = time.perf_counter()
        ref = refrun.fdk(host, g, times)
        wall = time.perf_counter() - t0
        computed = slice(0, g.Z - 1) if (g.Z - 1) % g.zb == 0 else slice(0, g.Z)  # the reference's last-slice quirk
        den = float(np.sqrt(np.mean(ref[computed].astype(np.float64) ** 2)))
        rm = {k: float(np.sqrt(np.mean((v[computed].astype(np.float64) - ref[computed]) ** 2)) / den)
              for k, v in vols.items()}
        out[name] = {"volume": [g.X, g.Y, g.Z], "projections": [g.N, g.H, g.W], "updates": g.updates,
                     "reference": {**times, "wall_s": wall, "gups_bp_kernels": g.updates / (times["bp_kernels_ms"] * 1e-3) / 1e9,
                                   "gups_total": g.updates / (times["total_ms"] * 1e-3) / 1e9},
                     "ours_ms": {"f32_samples": res["f32"], "f16_coefficients": res["f16"]},
                     "ours_gups": {k: g.updates / (v * 1e-3) / 1e9 for k, v in res.items()},
                     "speedup_total_f32": times["total_ms"] / res["f32"],
                     "speedup_total_f16": times["total_ms"] / res["f16"],
                     "rel_rmse_vs_reference": rm}
        del host, ref, vols
    emit({"reference_gpu": out, "note": "reference = FBPG/kernel.cu compiled for sm_103a and driven in its own "
          "stage order with cuFFT (oracle/tk_refrun.cpp); times are its wall clock with its own device "
          "synchronisations; ours = tk_fdk_device, inputs resident in HBM, CUDA events"})
    return 0


def main():
    args = parse()
    if args.reference_gpu:
        return run_reference_gpu(args)
    if args.batch:
        return run_batch(args)
    if args.adjoint:
        return run_adjoint(args)
    if args.profile_filter:
        return run_profile_filter(args)
    if args.outofcore:
        return run_outofcore(args)
    if args.profile_bp:
        return run_profile_bp(args)
    if args.probe_link:
        return run_probe_link(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
