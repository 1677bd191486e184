"""Capon/MVDR throughput benchmark (one JSON line on stdout).

Workload: Xd [Nx=256][Ny=2048][M=64] complex64 (synthetic, 8 scatterers at
20 dB per element), L=32, K=2 (5 range samples), loading 0.01*tr(R)/L,
a = ones(32): 256 x 2044 = 523,264 pixels per step.  Outputs per pixel:
complex amplitude z and power P.

  value   pixels/s of the fused kernel with the cube resident in HBM
          (one launch per step; the 268 MB cube exceeds the 126 MB L2, so
          every step streams it from HBM)
  e2e     pixels/s through cos_capon_get_capon_ex with pinned host buffers:
          H2D of the cube, the launch and D2H of z and P inside each step
  plain   pixels/s of the plain FP32 three-stage form (the denominator of the
          metric), same workload

``--impl reference`` times the reference's own CPU Capon path
(getCaponC.getCaponCPy, compiled from the reference sources into oracle/_ref)
on all host cores, or the FP64 C oracle when that module is not built.
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
sys.path.insert(0, ROOT)

M, L, K, NX, NY, D = 64, 32, 2, 256, 2048, 0.01
NS, T = M - L + 1, 2 * K + 1
NPIX = NX * (NY - 2 * K)
# Algorithmic work per pixel (canonical count: full-array Gram covariance with
# diagonal smoothing 8 M^2 T + 2 L^2 Ns, Cholesky 4/3 L^3, two triangular
# solves 8 L^2, weights/outputs 32 L + 8 M).
FLOP_PER_PIXEL = 8 * M * M * T + 2 * L * L * NS + (4.0 / 3.0) * L ** 3 + 8 * L * L + 32 * L + 8 * M
# Floating-point work the fused kernel actually executes per pixel (useful
# operations, complex MAC = 8 flop): covariance rows 1..L-1 by the diagonal
# recurrence (2T MACs per upper-triangle entry), row 0 and subarray sums
# amortised per range row, Cholesky, two forward solves, outputs.
EXEC_FLOP_PER_PIXEL = (8 * 2 * T * (L * (L + 1) // 2 - L) + 8 * NS * L + 2 * NS * L + 2 * T * L
                       + (4.0 / 3.0) * L ** 3 + 2 * 8 * L * L / 2 * 2 + 16 * L)
# Algorithmic HBM bytes per pixel: the cube once (8 M Ny/(Ny-2K)) + z + P.
BYTES_PER_PIXEL = 8 * M * NY / (NY - 2 * K) + 8 + 4
# DRAM bytes per pixel of the fused kernel from one ncu capture (dram__bytes_read
# + dram__bytes_write = 168.42 + 5.63 MB over 327,040 pixels, the 160-beam
# profiling case), scaled to a full launch by the pixels it processes.
TRAFFIC_PER_PIXEL = (168.418816e6 + 5.626368e6) / 327040
CONFIG = {"workload": "capon-element-space M=64 L=32 K=2 [Nx=256,Ny=2048]", "M": M, "L": L, "K": K,
          "Nx": NX, "Ny": NY, "pixels_per_step": NPIX, "loading": D, "outputs": "z,P",
          "l2": "inputs larger than L2 (268 MB cube vs 126 MB L2)", "parallelism": "replicas"}


def _peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


class Clocks:
    """nvidia-smi sampling around the timed region.  The sampler starts before
    the warm-up, polls every 20 ms and stamps each sample with nvidia-smi's own
    clock; `window(t0, t1)` marks the timed region (time.time() bounds), and
    the summary keeps the samples inside it -- or, when the region is shorter
    than one polling interval, the samples of the whole sampled span, and says
    so."""

    def __init__(self, dev: int):
        self.dev, self.proc, self.out, self.win = dev, None, [], None

    def __enter__(self):
        q = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)   # nvidia-smi start-up, so that sampling covers the warm-up and the timed region
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.out.append(line.strip())

    def window(self, t0: float, t1: float):
        self.win = (t0, t1)

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.05)
            self.proc.terminate()
            self.proc.wait()
            self.t.join(timeout=2)

    @staticmethod
    def _stamp(s: str):
        import datetime
        for fmt in ("%Y/%m/%d %H:%M:%S.%f", "%Y/%m/%d %H:%M:%S"):
            try:
                return datetime.datetime.strptime(s, fmt).timestamp()
            except ValueError:
                pass
        return None

    def summary(self) -> dict:
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        rows = []
        for line in self.out:
            f = [v.strip() for v in line.split(",")]
            if len(f) < 8:
                continue
            try:
                rows.append((self._stamp(f[0]), float(f[1]), float(f[2]), f[4:8]))
            except ValueError:
                continue
        inside = [r for r in rows if self.win and r[0] is not None and self.win[0] <= r[0] <= self.win[1]]
        use, span = (inside, "timed region") if inside else (rows, "warm-up and timed region (region shorter "
                                                                   "than the 20 ms polling interval)")
        reasons = sorted({n for r in use for n, v in zip(names, r[3]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median([r[1] for r in use]) if use else None,
                "sm_max_mhz": use[-1][2] if use else None, "samples": len(use), "span": span,
                "reasons": reasons}


def mixed_roofline(ms: float, fp32_tflops: float, peaks: dict) -> dict:
    """The mixed bound of the per-pixel work: the covariance (F_cov) at the
    tensor-core TF32 rate, the Cholesky, solves and outputs at the FP32 rate,
    t_roof = F_cov/P_TC + (F_chol + F_sol + F_out)/P_FP32 per pixel, and the
    measured time's fraction of it.  P_TC is half the measured dense bf16 rate
    (TF32 issues at half the bf16 rate)."""
    bf16 = peaks.get("bf16_tflops")
    if not bf16:
        return None
    f_cov = 8 * M * M * T + 2 * L * L * NS
    f_rest = (4.0 / 3.0) * L ** 3 + 8 * L * L + 32 * L + 8 * M
    p_tc = bf16 / 2.0
    t_roof_ms = NPIX * (f_cov / (p_tc * 1e12) + f_rest / (fp32_tflops * 1e12)) * 1e3
    return {"t_roof_ms": t_roof_ms, "t_measured_ms": ms, "frac": t_roof_ms / ms, "p_tc_tflops": p_tc,
            "p_fp32_tflops": fp32_tflops, "f_cov_per_pixel": f_cov, "f_rest_per_pixel": f_rest,
            "peak_source": "TF32 = half of MEASURED_PEAKS.json bf16_tflops; FP32 = SGEMM measured here"}


def headline_roofline(ms: float, fp32_tflops: float, peaks: dict) -> dict:
    """The headline roofline: the mixed bound of the per-pixel work (the
    canonical covariance F_cov at the tensor-core TF32 rate, the Cholesky,
    solves and outputs at the FP32 rate).  `achieved` is the canonical flop
    rate of the measured launch, `peak` the canonical flop rate a launch at the
    bound would reach, so frac = t_roof / t_measured."""
    mix = mixed_roofline(ms, fp32_tflops, peaks)
    if mix is None:
        return None
    flops = FLOP_PER_PIXEL * NPIX
    return {"bound": "tensor", "bound_detail": "mixed: F_cov at the TF32 tensor rate + F_chol+F_sol+F_out at FP32",
            "achieved": flops / (ms * 1e-3) / 1e12, "peak": flops / (mix["t_roof_ms"] * 1e-3) / 1e12,
            "unit": "TFLOP/s", "frac": mix["frac"], "traffic": TRAFFIC_PER_PIXEL * NPIX, "traffic_unit": "bytes",
            "traffic_source": "ncu dram__bytes_read+write of a smaller capture, scaled by pixels",
            "t_roof_ms": mix["t_roof_ms"], "t_measured_ms": ms, "p_tc_tflops": mix["p_tc_tflops"],
            "p_fp32_tflops": fp32_tflops, "f_cov_per_pixel": mix["f_cov_per_pixel"],
            "f_rest_per_pixel": mix["f_rest_per_pixel"],
            "peak_source": "P_TC assumed = half of MEASURED_PEAKS.json bf16_tflops (TF32 issues at half the bf16 "
                           "rate; not a measured TF32 rate); P_FP32 = cuBLAS SGEMM measured in this process"}


def fp32_peak_tflops(torch) -> float:
    """cuBLAS FP32 SGEMM throughput (TF32 off): the measured CUDA-core FP32 peak."""
    torch.backends.cuda.matmul.allow_tf32 = False
    n = 8192
    a = torch.randn(n, n, device="cuda")
    b = torch.randn(n, n, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = max(best, 2 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b
    return best


def cpu_reference_rate(cores: int, beams: int, seed: int = 1) -> dict:
    """Reference CPU Capon on `beams` beams of the workload, all `cores`
    processes; returns pixels/s and what ran."""
    from cos_gb300 import synth
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref  # noqa: E402
    x = synth.cube(NY, beams, M, [10.0] * 8, seed)
    if ref.available():
        import multiprocessing as mp
        ctx = mp.get_context("spawn")
        slabs = np.array_split(np.arange(beams), cores)
        slabs = [s for s in slabs if len(s)]
        with ctx.Pool(len(slabs), initializer=_ref_init) as pool:
            pool.map(_ref_slab, [np.ascontiguousarray(x[s[:1], :64]) for s in slabs])   # warm-up
            t0 = time.perf_counter()
            pool.map(_ref_slab, [np.ascontiguousarray(x[s]) for s in slabs])
            dt = time.perf_counter() - t0
        kind = "reference"
        what = "getCaponC.getCaponCPy (reference Cython, FP64) in a spawn pool"
    else:
        import oracle  # noqa: E402
        oracle.capon(x[:1, :64], D, L, K, nthreads=1)
        t0 = time.perf_counter()
        oracle.capon(x, D, L, K, nthreads=cores)
        dt = time.perf_counter() - t0
        kind = "port"
        what = "FP64 C restatement (oracle/capon_oracle.c), pthreads"
    npx = beams * (NY - 2 * K)
    return {"value": npx / dt, "unit": "pixels/s", "cores": cores, "kind": kind,
            "sample": f"{beams} beams x {NY - 2 * K} pixels of the workload ({npx} pixels), {what}",
            "seconds": dt}


def _ref_init():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref  # noqa: E402
    global _REF
    _REF = ref.load()


def _ref_slab(x):
    _REF.getCaponCPy(x.astype(np.complex128), D, L, K, np.array([]), False, False)
    return 0


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    beams = max(cores, 8)
    vals = []
    last = None
    for i in range(args.warmup + args.steps):
        r = cpu_reference_rate(cores, beams, seed=1 + i)
        if i >= args.warmup:
            vals.append(r["value"])
        last = r
    v = statistics.median(vals)
    npx_step = beams * (NY - 2 * K)
    line = {"metric": METRIC, "value": v, "unit": "pixels/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": npx_step / v * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic", "config": CONFIG,
            "cpu_baseline": {k: last[k] for k in ("unit", "cores", "kind", "sample")} | {"value": v},
            "e2e": {"value": v, "unit": "pixels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


METRIC = "Capon pixels/s at L=32 (fast vs plain FP32 GPU; <=1e-4 rel err vs FP64)"


def run_gpu(args) -> None:
    import torch
    from cos_gb300 import _lib, capon, synth

    from cos_gb300 import replicas
    rank, local, world = replicas.env()
    torch.cuda.set_device(local)
    dist = replicas.init("nccl")

    x_host = synth.config1(seed=1 + rank)["x"]
    xt = torch.from_numpy(x_host).cuda()
    npy = NY - 2 * K
    ctx = capon.Context()
    stream = torch.cuda.Stream()

    def frame(form_P=True):
        f = capon.DeviceFrame(x=xt, L=L, K=K, d=D,
                              z=torch.empty((NX, npy), dtype=torch.complex64, device="cuda"),
                              P=torch.empty((NX, npy), dtype=torch.float32, device="cuda"))
        return f

    def time_form(form: int, steps: int, warmup: int, clk=None, refine: int = 0):
        f = frame()
        o = capon.opts(form=form, refine=refine)
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                capon.capon_frames([f], ctx, o, stream)
        stream.synchronize()
        replicas.barrier(dist)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.time()
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(steps):
                capon.capon_frames([f], ctx, o, stream)
            e1.record(stream)
        e1.synchronize()
        torch.cuda.synchronize()
        if clk is not None:
            clk.window(t0, time.time())
        ms = replicas.max_over_ranks(dist, e0.elapsed_time(e1) / steps, device="cuda")
        return ms, f

    # fused (headline), with clocks sampled during the timed region
    with Clocks(local) as clk:
        ms, f = time_form(_lib.FORM_FUSED, args.steps, args.warmup, clk)
    clocks = clk.summary()
    value = replicas.aggregate_rate(NPIX, ms, world)

    # plain FP32 three-stage form (denominator), fewer steps
    ms_plain, _ = time_form(_lib.FORM_PLAIN, max(2, min(args.steps, 5)), max(1, min(args.warmup, 2)))

    # the tensor-core fused form (per-row Hankel Gram on tcgen05, R on chip)
    tcf = None
    try:
        ms_tcf, f_tcf = time_form(_lib.FORM_TC_FUSED, args.steps, args.warmup)
        tcf = {"value": replicas.aggregate_rate(NPIX, ms_tcf, world), "unit": "pixels/s", "ms_per_step": ms_tcf,
               "speedup_over_plain": ms_plain / ms_tcf, "fused_fp32_over_tc": ms_tcf / ms,
               "precision": "FP16 hi/lo split of row-scaled samples, 3 products, FP32 accumulation; FP32 Cholesky"}
    except Exception as exc:
        f_tcf = None
        tcf = {"error": str(exc)[:200]}

    # the FP32 Cholesky with one FP64-residual refinement step, in the fused
    # path: on every pixel, and on the ill-conditioned ones (pivot spread > 32)
    refined, f_ref = {}, {}
    for name, rv in (("all_pixels", _lib.REFINE_ALL), ("adaptive", _lib.REFINE_ADAPTIVE)):
        try:
            ms_r, f_ref[name] = time_form(_lib.FORM_FUSED, max(2, min(args.steps, 5)), max(1, min(args.warmup, 2)),
                                          refine=rv)
            refined[name] = {"ms_per_step": ms_r, "value": replicas.aggregate_rate(NPIX, ms_r, world),
                             "unit": "pixels/s"}
        except Exception as exc:
            refined[name] = {"error": str(exc)[:200]}

    # e2e through the host-pointer C-ABI call, pinned host buffers
    xp = torch.from_numpy(x_host).pin_memory()
    zp = torch.empty((NX, npy), dtype=torch.complex64).pin_memory()
    Pp = torch.empty((NX, npy), dtype=torch.float32).pin_memory()
    cctx = capon.Capon()
    xn, zn, Pn = xp.numpy(), zp.numpy(), Pp.numpy()
    for _ in range(max(1, args.warmup)):
        _lib.check(cctx.getCaponEx(zn, Pn, None, None, xn, D, L, K, M, NX, NY, 0))
    replicas.barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _lib.check(cctx.getCaponEx(zn, Pn, None, None, xn, D, L, K, M, NX, NY, 0))
    e2e_ms = replicas.max_over_ranks(dist, (time.perf_counter() - t0) * 1e3 / args.steps, device="cuda")

    # the reference-facing drop-in call (Capon::getCapon semantics: z and w, no
    # P), end to end from pinned host buffers
    wp = torch.empty((NX, npy, L), dtype=torch.complex64).pin_memory()
    wn = wp.numpy()
    for _ in range(max(1, args.warmup)):
        _lib.check(cctx.getCapon(zn, wn, None, xn, D, L, K, M, NX, NY, 0))
    replicas.barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _lib.check(cctx.getCapon(zn, wn, None, xn, D, L, K, M, NX, NY, 0))
    dropin_ms = replicas.max_over_ranks(dist, (time.perf_counter() - t0) * 1e3 / args.steps, device="cuda")

    # adjoint cost: forward with the weights saved (absolute loading, as the
    # differentiable path runs it) and the adjoint kernel over the full frame
    adj = None
    try:
        from cos_gb300.autograd import capon_power
        delta = torch.tensor(0.5, dtype=torch.float32, device="cuda", requires_grad=True)
        tau = torch.zeros(M, dtype=torch.float32, device="cuda", requires_grad=True)
        xg = xt.clone().requires_grad_(True)
        for _ in range(2):
            Pd = capon_power(xg, delta, tau, L, K, 0.25, ctx)
            Pd.sum().backward()
        torch.cuda.synchronize()
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        nrep = max(2, min(args.steps, 5))
        fw = bw = 0.0
        for _ in range(nrep):
            e0.record()
            Pd = capon_power(xg, delta, tau, L, K, 0.25, ctx)
            e1.record()
            Pd.sum().backward()
            e2.record()
            e2.synchronize()
            fw += e0.elapsed_time(e1)
            bw += e1.elapsed_time(e2)
        adj = {"forward_ms": fw / nrep, "backward_ms": bw / nrep, "backward_over_forward": bw / fw,
               "note": "full frame, loss = sum of P; forward saves w (the ms include the torch glue: phase, "
                       "gradient buffers)"}
    except Exception as exc:  # reported, not fatal to the throughput line
        adj = {"error": str(exc)[:200]}

    # config 2: four frames of uneven (M, L, Nb), one CUDA graph per step
    cfg2 = None
    try:
        frames2 = []
        npix2 = 0
        for fr in synth.config2(seed=2):
            x2 = torch.from_numpy(fr["x"]).cuda()
            Nx2, Ny2, _ = fr["x"].shape
            npy2 = Ny2 - 2 * fr["K"]
            npix2 += Nx2 * npy2
            frames2.append(capon.DeviceFrame(x=x2, L=fr["L"], K=fr["K"], d=fr["d"], Nb=fr["Nb"],
                                             z=torch.empty((Nx2, npy2), dtype=torch.complex64, device="cuda"),
                                             P=torch.empty((Nx2, npy2), dtype=torch.float32, device="cuda")))
        with torch.cuda.stream(stream):
            for _ in range(2):
                capon.capon_frames(frames2, ctx, stream=stream)
        stream.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream):
            capon.capon_frames(frames2, ctx, stream=stream)
        for _ in range(args.warmup):
            graph.replay()
        torch.cuda.synchronize()
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        g0.record()
        for _ in range(args.steps):
            graph.replay()
        g1.record()
        g1.synchronize()
        ms2 = g0.elapsed_time(g1) / args.steps
        cfg2 = {"workload": "4 frames [Ny=1024, Nx=256]: (M,L,Nb) = (32,16,0), (64,32,0), (96,48,3), (128,64,5), K=1",
                "pixels_per_step": npix2, "ms_per_step": ms2, "pixels_per_s": npix2 / (ms2 * 1e-3),
                "launch": "one CUDA graph replay per step"}
        del frames2
    except Exception as exc:
        cfg2 = {"error": str(exc)[:200]}

    steering = None
    try:
        steering = steering_rate(stream, _peaks().get("hbm_gbs"))
    except Exception as exc:
        steering = {"error": str(exc)[:200]}

    lca_line = None
    try:
        lca_line = lca_rate(stream, _peaks().get("hbm_gbs"))
    except Exception as exc:
        lca_line = {"error": str(exc)[:200]}

    sliding = None
    if not args.no_precision and rank == 0:
        try:
            sliding = sliding_inverse_study(ctx, stream, xt, x_host)
        except Exception as exc:
            sliding = {"error": str(exc)[:200]}

    precision = None
    if not args.no_precision and rank == 0:
        try:
            precision = precision_study(ctx, stream)
        except Exception as exc:
            precision = {"error": str(exc)[:200]}

    # parity of this very run against the FP64 oracle on sampled beams
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # noqa: E402
    beams = [0, 128, 255]
    refo = oracle.capon(np.ascontiguousarray(x_host[beams]), D, L, K, want_w=False, nthreads=3)
    Pg = f.P.cpu().numpy()[beams]
    relP = np.abs(Pg - refo["P"]) / refo["P"]
    if f_tcf is not None:
        eT = np.abs(f_tcf.P.cpu().numpy()[beams] - refo["P"]) / refo["P"]
        tcf["P_rel_err_max"], tcf["P_rel_err_median"] = float(eT.max()), float(np.median(eT))
    for name, fr in f_ref.items():
        eR = np.abs(fr.P.cpu().numpy()[beams] - refo["P"]) / refo["P"]
        refined[name]["P_rel_err_max"], refined[name]["P_rel_err_median"] = float(eR.max()), float(np.median(eR))

    peaks = _peaks()
    fp32 = fp32_peak_tflops(torch)
    hbm_peak = peaks.get("hbm_gbs")
    kernel_s = ms * 1e-3
    achieved_tf = FLOP_PER_PIXEL * NPIX / kernel_s / 1e12
    exec_tf = EXEC_FLOP_PER_PIXEL * NPIX / kernel_s / 1e12
    achieved_gbs = BYTES_PER_PIXEL * NPIX / kernel_s / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "pixels/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator, 8 scatterers, 20 dB)",
        "config": CONFIG,
        "tc_fused": tcf,
        "refined": refined,
        "plain": {"value": NPIX * world / (ms_plain * 1e-3), "ms_per_step": ms_plain,
                  "speedup_fused_over_plain": ms_plain / ms},
        "parity": {"P_rel_err_max": float(relP.max()), "P_rel_err_median": float(np.median(relP)),
                   "sample": "beams 0,128,255 vs FP64 oracle"},
        "e2e": {"value": NPIX * world / (e2e_ms * 1e-3), "unit": "pixels/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": int(x_host.nbytes), "d2h_bytes_per_step": int(zn.nbytes + Pn.nbytes)},
        "e2e_getcapon_zw": {"value": replicas.aggregate_rate(NPIX, dropin_ms, world), "unit": "pixels/s",
                            "ms_per_step": dropin_ms, "h2d_bytes_per_step": int(x_host.nbytes),
                            "d2h_bytes_per_step": int(zn.nbytes + wn.nbytes),
                            "call": "cos_capon_get_capon (Capon::getCapon drop-in: z and w)"},
        "gpu_launches": args.steps,
        "roofline": headline_roofline(ms, fp32, peaks),
        "roofline_fp32_canonical": {
            "bound": "fp32", "achieved": achieved_tf, "peak": fp32, "unit": "TFLOP/s",
            "frac": achieved_tf / fp32, "traffic": TRAFFIC_PER_PIXEL * NPIX, "traffic_unit": "bytes",
            "note": "canonical flops (non-recursive covariance) over the FP32 rate: the kernel never executes "
                    "those flops, so this can exceed 1; executed_frac is the FP32-pipe figure",
            "peak_source": "measured here: cuBLAS FP32 SGEMM 8192^3, TF32 off",
            "flop_per_pixel": FLOP_PER_PIXEL,
            "executed_flop_per_pixel": EXEC_FLOP_PER_PIXEL, "executed_tflops": exec_tf,
            "executed_frac": exec_tf / fp32},
        "roofline_hbm": {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                         "frac": (achieved_gbs / hbm_peak) if hbm_peak else None,
                         "bytes_per_pixel": BYTES_PER_PIXEL, "peak_source": "MEASURED_PEAKS.json hbm_gbs"},
        "clocks": clocks,
        "adjoint": adj,
        "config2": cfg2,
        "precision": precision,
        "steering": steering,
        "lca": lca_line,
        "sliding_inverse": sliding,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = {k: v for k, v in cpu_reference_rate(os.cpu_count() or 1, 16).items()
                                if k != "seconds"}
        line["cpu_baseline"]["sample_fraction"] = f"16 of {NX} beams ({16 / NX:.4f} of the frame); value is the rate"
    if rank == 0:
        print(json.dumps(line))
    replicas.finalize(dist)


SLIDING_D = 0.5          # absolute loading on the normalised covariance
SLIDING_SEGMENTS = (4, 8, 32)


def sliding_inverse_study(ctx, stream, xt, x_host) -> dict:
    """The config-1 frame through FORM_SLIDING_INVERSE (R_d^-1 carried along
    range by Sherman-Morrison changes) at a few build-up intervals, beside the
    fused kernel at the same absolute loading; P errors on sampled beams
    against the FP64 direct solve."""
    import torch
    from cos_gb300 import _lib, capon
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # noqa: E402
    npy = NY - 2 * K
    beams = [0, 128, 255]
    ref = oracle.capon(np.ascontiguousarray(x_host[beams]), SLIDING_D, L, K, want_w=False, nthreads=3,
                       absolute=True, fp32_scalars=False)

    def run(o, steps=3):
        f = capon.DeviceFrame(x=xt, L=L, K=K, d=SLIDING_D,
                              z=torch.empty((NX, npy), dtype=torch.complex64, device="cuda"),
                              P=torch.empty((NX, npy), dtype=torch.float32, device="cuda"))
        with torch.cuda.stream(stream):
            capon.capon_frames([f], ctx, o, stream)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                capon.capon_frames([f], ctx, o, stream)
            e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / steps
        P = f.P.cpu().numpy()[beams]
        e = np.abs(P - ref["P"]) / ref["P"]
        return {"ms": ms, "pixels_per_s": NPIX / (ms * 1e-3), "P_rel_err_max": float(np.nanmax(e)),
                "P_rel_err_median": float(np.nanmedian(e)), "nonfinite": int(np.sum(~np.isfinite(P)))}

    out = {"workload": f"config-1 frame, absolute loading {SLIDING_D} on the normalised R",
           "fused_same_loading": run(capon.opts(form=_lib.FORM_FUSED, loading=_lib.LOAD_ABSOLUTE))}
    for seg in SLIDING_SEGMENTS:
        out[f"segment_{seg}"] = run(capon.opts(form=_lib.FORM_SLIDING_INVERSE, loading=_lib.LOAD_ABSOLUTE,
                                               segment=seg))
    out["error_sample"] = "beams 0,128,255 vs the FP64 direct solve (oracle, absolute loading)"
    return out


PRECISION_FORMS = [  # name, form, refine
    ("all_fp32", 1, 0),                       # plain FP32 pipeline, the reference GPU algorithm
    # fused kernel (L = 64: one warp per pixel, registers): float-float
    # covariance, FP32 Cholesky; then with one FP64-residual refinement step
    ("fused_ff_cov_fp32_chol", 0, 0),
    ("fused_ff_cov_fp32_chol_fp64_refine", 0, 1),
    # ... the refinement step only on the pixels whose pivot spread exceeds 32
    ("fused_ff_cov_fp32_chol_adaptive_refine", 0, 2),
    # the same arithmetic with R materialised per pixel (precise pipeline)
    ("precise_ff_cov_fp32_chol_fp64_refine", 1, 1),
    ("tc_tf32", 2, 0), ("tc_tf32_refine", 2, 1),
    ("tc_bf16x3", 3, 0), ("tc_bf16x3_refine", 3, 1),
    ("tc_tf32x3", 4, 0), ("tc_tf32x3_refine", 4, 1),
]


def precision_study(ctx, stream) -> dict:
    """Precision stress workload: per-pixel relative errors of R, w and P for
    every form against the FP64 oracle on the three beams with the most energy
    (the coherent pair), and each form's time on the full frame."""
    import torch
    from cos_gb300 import _lib, capon, synth
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # noqa: E402
    c = synth.config3(seed=3)
    x, L, K, d = c["x"], c["L"], c["K"], c["d"]
    Nx, Ny, M = x.shape
    npy = Ny - 2 * K
    beams = sorted(np.argsort(np.sum(np.abs(x) ** 2, axis=(1, 2)))[-3:].tolist())
    sub = np.ascontiguousarray(x[beams])
    ref = oracle.capon(sub, d, L, K, want_R=True, want_w=True, nthreads=os.cpu_count() or 1)
    Rn = np.abs(ref["R"]).reshape(len(beams), npy, -1).max(-1)
    wn = np.linalg.norm(ref["w"], axis=-1)
    xt = torch.from_numpy(x).cuda()
    cap = capon.Capon()
    out = {"workload": f"[Nx={Nx}][Ny={Ny}][M={M}] L={L} K={K} loading {d}, two coherent scatterers 40 dB",
           "error_sample": f"beams {beams} ({len(beams) * npy} pixels) vs FP64 oracle; R as max|dR|/max|R| per "
                           "pixel, w as |dw|/|w|, P as |dP|/P", "forms": {}}
    for name, form, refine in PRECISION_FORMS:
        z = np.zeros((len(beams), npy), np.complex64)
        P = np.zeros((len(beams), npy), np.float32)
        w = np.zeros((len(beams), npy, L), np.complex64)
        R = np.zeros((len(beams), npy, L, L), np.complex64)
        o = capon.opts(form=form, r_layout=_lib.R_NORMALISED, refine=refine)
        e = cap.getCaponEx(z, P, w, R, sub, d, L, K, M, len(beams), Ny, 0, o)
        if e:
            out["forms"][name] = {"status": e}
            continue
        eR = np.abs(R - ref["R"]).reshape(len(beams), npy, -1).max(-1) / Rn
        ew = np.linalg.norm(w - ref["w"], axis=-1) / wn
        eP = np.abs(P - ref["P"]) / ref["P"]
        fr = capon.DeviceFrame(x=xt, L=L, K=K, d=d, P=torch.empty((Nx, npy), device="cuda"))
        with torch.cuda.stream(stream):
            capon.capon_frames([fr], ctx, o, stream)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(2):
                capon.capon_frames([fr], ctx, o, stream)
            e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / 2
        out["forms"][name] = {"R_max": float(eR.max()), "R_median": float(np.median(eR)),
                              "w_max": float(ew.max()), "w_median": float(np.median(ew)),
                              "P_max": float(eP.max()), "P_median": float(np.median(eP)),
                              "ms_full_frame": ms, "pixels_per_s": Nx * npy / (ms * 1e-3)}
        del fr
    del xt
    torch.cuda.empty_cache()
    # the stress target: P within 1e-4 of FP64 at <= 30 ms per frame; the
    # fastest form that meets it
    ok = [(v["ms_full_frame"], k) for k, v in out["forms"].items() if "P_max" in v and v["P_max"] <= 1e-4]
    best = min(ok) if ok else None
    out["target"] = {"P_max": 1e-4, "ms_per_frame": 30.0, "fastest_form_within_P": best[1] if best else None,
                     "its_ms": best[0] if best else None, "met": bool(best and best[0] <= 30.0)}
    return out


def steering_rate(stream, hbm_peak) -> dict:
    """Time-domain steering (cos_capon_tdib) producing a config-1-sized cube
    [Nx=256][Ny=2048][64 hydrophones] plus its delay-and-sum image, device
    pointers; HBM roofline over the algorithmic bytes (cube and image written,
    pixel geometry and channel data read once)."""
    import ctypes
    import torch
    from cos_gb300 import _lib, capon
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import tdib_oracle  # noqa: E402
    sc = tdib_oracle.scenario(seed=4, n_h=M, n_s=4096, n_x=NX, n_y=NY)
    dev = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).cuda()   # noqa: E731
    mf = dev(sc["mfdata"], np.complex64)
    xr, dd = dev(sc["x_r"], np.float64), dev(sc["D"], np.float64)
    xa, ya = dev(sc["xarr"], np.float64), dev(sc["yarr"], np.float64)
    Xd = torch.empty((NX, NY, M), dtype=torch.complex64, device="cuda")
    img = torch.empty((NY, NX), dtype=torch.complex64, device="cuda")
    t = sc["mtaxe"]
    ctx = capon.Context()
    args = (ctx.handle, mf.data_ptr(), M, t.size, float(t[0]), float(t[1] - t[0]), ctypes.c_void_p(xr.data_ptr()),
            ctypes.c_void_p(dd.data_ptr()), sc["c"], sc["fc"], ctypes.c_void_p(xa.data_ptr()),
            ctypes.c_void_p(ya.data_ptr()), NX, NY, Xd.data_ptr(), img.data_ptr(), 1, stream.cuda_stream)
    for _ in range(3):
        _lib.check(_lib.lib.cos_capon_tdib(*args), "cos_capon_tdib")
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n = 10
    e0.record(stream)
    for _ in range(n):
        _lib.lib.cos_capon_tdib(*args)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / n
    nbytes = NX * NY * M * 8 + NX * NY * 8 + 2 * NX * NY * 8 + M * t.size * 8
    gbs = nbytes / (ms * 1e-3) / 1e9
    return {"workload": f"[Nx={NX}][Ny={NY}] pixels x {M} hydrophones, 4096 samples each; cube + image",
            "ms": ms, "pixels_per_s": NX * NY / (ms * 1e-3), "bytes": nbytes,
            "roofline_hbm": {"achieved": gbs, "peak": hbm_peak, "unit": "GB/s",
                             "frac": gbs / hbm_peak if hbm_peak else None}}


def lca_rate(stream, hbm_peak) -> dict:
    """LCA window selection (cos_capon_lca) over the config-1 pixel grid with 8
    windows and a 5 x 1 range filter, device pointers; HBM roofline over the
    algorithmic bytes (Z read once, the image and window index written)."""
    import ctypes
    import torch
    from cos_gb300 import _lib, capon
    Nw = 8
    g = torch.Generator(device="cuda").manual_seed(5)
    Z = torch.randn((NY, NX, Nw), dtype=torch.complex64, device="cuda", generator=g)
    img = torch.empty((NY, NX), dtype=torch.complex64, device="cuda")
    win = torch.empty((NY, NX), dtype=torch.int32, device="cuda")
    wrf = np.ones((5, 1))
    ctx = capon.Context()
    args = (ctx.handle, Z.data_ptr(), NY, NX, Nw, wrf.ctypes.data, 5, 1, img.data_ptr(),
            ctypes.c_void_p(win.data_ptr()), 1, stream.cuda_stream)
    for _ in range(3):
        _lib.check(_lib.lib.cos_capon_lca(*args), "cos_capon_lca")
    stream.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n = 10
    e0.record(stream)
    for _ in range(n):
        _lib.lib.cos_capon_lca(*args)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / n
    nbytes = NY * NX * Nw * 8 + NY * NX * 12
    gbs = nbytes / (ms * 1e-3) / 1e9
    return {"workload": f"Z [Ny={NY}][Nx={NX}][Nw={Nw}], filter 5 x 1", "ms": ms,
            "pixels_per_s": NX * NY / (ms * 1e-3), "bytes": nbytes,
            "roofline_hbm": {"achieved": gbs, "peak": hbm_peak, "unit": "GB/s",
                             "frac": gbs / hbm_peak if hbm_peak else None}}


RTC_STAGES = ["memcpy_x_h2d", "sliding_beamspace", "build_R", "memcpy_R_d2h", "init_a", "beamspace_part1",
              "solve", "beamspace_part2", "weights_output", "memcpy_wz_d2h"]


def run_rtc(args) -> None:
    """The reference's own RealTimeCapon GPU library (built from its sources by
    oracle/build_rtc.py) on the same workload: its per-stage wall times (the
    library's timer file), the kernel-stage sum, and its P error vs the oracle."""
    import ctypes
    import tempfile
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build_rtc  # noqa: E402
    import oracle  # noqa: E402
    from cos_gb300 import synth
    libpath = build_rtc.build()
    if not libpath:
        print(json.dumps({"impl": "reference-gpu-library", "unavailable": "reference sources not staged"}))
        return
    rtc = ctypes.CDLL(libpath)
    vp, fl, i = ctypes.c_void_p, ctypes.c_float, ctypes.c_int
    rtc.rtc_get_capon.argtypes = [vp, vp, vp, vp, fl, i, i, i, i, i, i]
    x = synth.config1(seed=1)["x"]
    npy = NY - 2 * K
    z = np.zeros((NX, npy), np.complex64)
    w = np.zeros((NX, npy, L), np.complex64)
    R = np.zeros((NX, npy, L, L), np.complex64)   # the library copies R back (COPY_R_DEVICE_HOST)
    cwd = os.getcwd()
    tmp = tempfile.mkdtemp(prefix="rtc_")
    os.chdir(tmp)
    try:
        calls = []
        for it in range(1 + max(1, args.steps)):
            t0 = time.perf_counter()
            e = rtc.rtc_get_capon(z.ctypes.data, w.ctypes.data, R.ctypes.data, x.ctypes.data, D, L, K, M, NX, NY, 0)
            calls.append((time.perf_counter() - t0) * 1e3)
            if e:
                print(json.dumps({"impl": "reference-gpu-library", "error": int(e)}))
                return
        rows = [[float(v) for v in ln.split()] for ln in open("timer_values.txt") if ln.strip()]
    finally:
        os.chdir(cwd)
    rows = rows[1:]   # the first call allocates
    med = {n: statistics.median(r[k] for r in rows) for k, n in enumerate(RTC_STAGES)}
    kern = med["build_R"] + med["init_a"] + med["solve"] + med["weights_output"]
    beams = [0, 128, 255]
    ref = oracle.capon(np.ascontiguousarray(x[beams]), D, L, K, want_w=False, nthreads=3)
    # the library returns z and w; its power is 1/Re(sum Ria) = w^H R w with w = Ria/sum(Ria)
    Rb = R[beams].astype(np.complex128) / (NS * T)    # column-major, loaded, unnormalised -> normalised
    wb = w[beams].astype(np.complex128)
    P = np.real(np.einsum("bpi,bpji,bpj->bp", wb.conj(), Rb, wb))
    relP = np.abs(P - ref["P"]) / ref["P"]
    relz = np.abs(z[beams] - ref["z"]) / np.sqrt(ref["P"])
    print(json.dumps({
        "impl": "reference-gpu-library", "workload": CONFIG["workload"], "pixels": NPIX,
        "stages_ms_median": med, "kernel_stages_ms": kern, "pixels_per_s_kernel_stages": NPIX / (kern * 1e-3),
        "call_ms_median": statistics.median(calls[1:]), "calls": len(calls) - 1,
        "P_rel_err_max": float(relP.max()), "z_err_max_rel_sqrtP": float(relz.max()),
        "note": "RealTimeCapon built from its own sources for sm_103a; stage times are the library's own "
                "host wall-clock timers around synchronised stages (Capon.cpp:171-459)"}))


def run_profile_case(args) -> None:
    """One form (default: fused) alone on the first Nx=profile_nx beams of a
    workload (config1, config2 = its four frames, config3), for ncu captures."""
    import torch
    from cos_gb300 import capon, synth
    wl = args.profile_workload
    if wl == "config2":
        cfgs = synth.config2(seed=2, Nx=args.profile_nx)
    elif wl == "config3":
        cfgs = [synth.config3(seed=3, Nx=args.profile_nx)]
    else:
        cfgs = [synth.config1(seed=1, Nx=args.profile_nx)]
    frames = []
    for c in cfgs:
        Nx, Ny, _ = c["x"].shape
        frames.append(capon.DeviceFrame(x=torch.from_numpy(c["x"]).cuda(), L=c["L"], K=c["K"], d=c["d"],
                                        Nb=c["Nb"],
                                        P=torch.empty((Nx, Ny - 2 * c["K"]), dtype=torch.float32, device="cuda"),
                                        w=torch.empty((Nx, Ny - 2 * c["K"], c["L"]), dtype=torch.complex64,
                                                      device="cuda") if args.profile_w else None))
    ctx = capon.Context()
    for _ in range(args.warmup + args.steps):
        capon.capon_frames(frames, ctx, capon.opts(form=args.profile_form, refine=args.profile_refine))
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": {"workload": wl, "Nx": args.profile_nx, "refine": args.profile_refine,
                                       "launches": args.warmup + args.steps}}))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-precision", action="store_true", help="skip the precision-stress study")
    ap.add_argument("--rtc", action="store_true",
                    help="time the reference's RealTimeCapon GPU library (oracle/build_rtc.py) on the workload")
    ap.add_argument("--profile-form", type=int, default=0, help="form of the profiling case (COS_CAPON_FORM_*)")
    ap.add_argument("--profile-workload", default="config1", choices=["config1", "config2", "config3"])
    ap.add_argument("--profile-w", action="store_true", help="the profiling case also writes the weights w")
    ap.add_argument("--profile-refine", type=int, default=0, help="the profiling case's opts.refine (COS_CAPON_REFINE_*)")
    ap.add_argument("--profile-nx", type=int, default=0,
                    help="profiling case: only the fused kernel, warmup+steps launches on Nx beams of the workload")
    args = ap.parse_args()
    if args.rtc:
        run_rtc(args)
    elif args.profile_nx:
        run_profile_case(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
