"""Benchmark: effective FP64 TFLOP/s of the GB300 Ozaki DGEMM.

Workload (one step = one full DGEMM through stages (a)-(d)):
  C = A B, M = N = K = 4096, row-major FP64, a_ij = (U(0,1) - 0.5) exp(phi N(0,1)),
  phi = 1, A and B from independent seeds; slices chosen by the precision knob for a
  requested normwise relative error of 1e-15 (b = 7, triangular pair set).
  Effective FP64 TFLOP/s = 2 M N K / time (the reference's GFLOPS formula,
  test.cpp:302, 595-604).  The result is checked on 1000 sampled entries against
  the exact product (and MPFR when available); a step that misses the bound is
  reported as invalid.

value : device-resident inputs (A, B in HBM before the timed region, 268 MB of
        inputs + 600 MB of slice planes per step, larger than the 126 MB L2),
        CUDA events on the launching stream, max over ranks.
valid : the normwise relative error on 1000 sampled entries, against the exact
        products and MPFR-106, is <= 1e-15 (accuracy_gate says why normwise);
        the elementwise form of the bound is measured under elementwise_mode.
e2e   : the reference-facing host-array call (ozAIE_DGEMM semantics) with host
        copies in and out inside the timed region, on pageable numpy arrays
        (pinned arrays reported beside it).
Also, by default: the batched workload (512 uneven problems, grouped vs per
call), the long-K workload (8192 x 8192 x 65536 and its ill-conditioned
variant), the accuracy-adaptive mix (65 problems up to 16384^3) and the 4096^3
sweep (both pair sets, s = 3..8, phi in {0.5, 1, 2, 4}); --quick skips them.
--impl reference : the reference's arithmetic on the host cores (the oracle port,
        OpenMP), bounded row sample of the same workload.
"""
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

M = N = K = 4096
PHI = 1.0
BOUND = 1e-15
METRIC = "effective FP64 TFLOP/s at rel-err<=1e-15 vs MPFR: batched/adaptive vs plain Ozaki"
UNIT = "TFLOP/s"
WORKLOAD = "ozaki_dgemm_4096x4096x4096_phi1_adaptive_1e-15"


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": d.get("hbm_gbs", 6800.0), "bf16_tflops": d.get("bf16_tflops", 1900.0),
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained", 1700.0), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "source": "fallback"}


def profile_traffic():
    """Per-launch DRAM bytes of the slice-pair GEMM from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "oz_gemm_kernel_4096_s8_j9.md")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            if line.startswith("traffic_bytes_per_launch:"):
                try:
                    return float(line.split(":", 1)[1].strip())
                except ValueError:
                    return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(x, device="cpu"):
    """Largest value of x over the ranks of the process group (x itself when
    there is none): the timing that a whole job reports."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return x
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_baseline(A, B, s, J, rows=512):
    """The reference's arithmetic on the host cores: oracle port of split + int8
    slice-pair GEMMs + bin sum + decode over a bounded row sample of A, with the
    slice schedule (s, J) the GPU path used."""
    from oracle import ozoracle as O
    O.dgemm_rows(A, B, 7, s, J, 0, 0, 4)  # warm-up
    t0 = time.perf_counter()
    O.dgemm_rows(A, B, 7, s, J, 0, 0, rows)
    dt = time.perf_counter() - t0
    return {"value": 2.0 * rows * N * K / dt / 1e12, "unit": UNIT, "cores": O.num_threads(), "kind": "port",
            "sample": "%d of %d rows of A against all of B (s=%d, pairs p+q<=%d), exponents over full K, %.1f s" %
                      (rows, M, s, J - 1, dt)}


def cpu_blas_dgemm(A, B):
    """numpy's OpenBLAS DGEMM on the host cores (bounded: 1024 rows)."""
    a = np.ascontiguousarray(A[:1024])
    a @ B[:, :256]
    t0 = time.perf_counter()
    a @ B
    dt = time.perf_counter() - t0
    return {"value": 2.0 * 1024 * N * K / dt / 1e12, "unit": UNIT, "sample": "1024 x 4096 x 4096"}


def batched_workload(n, seed=7, lo=32, hi=2048):
    """Sizes of the batched workload: M, N, K each log-uniform in [lo, hi]."""
    g = np.random.default_rng(seed)
    return np.exp(g.uniform(np.log(lo), np.log(hi), size=(n, 3))).astype(np.int64)


def batched_run(n_probs, dev, stream, oz, O, torch):
    """Many uneven DGEMMs: the grouped, accuracy-adaptive call (replayed CUDA
    graphs) against plain per-call DGEMMs with the fixed accurate configuration
    (s = 8, full pair set), both on device-resident operands."""
    sizes = batched_workload(n_probs)
    probs, hosts, flops = [], [], 0.0
    for i, (m, n, k) in enumerate(sizes):
        m, n, k = int(m), int(n), int(k)
        A = O.gen_phi((m, k), 10000 + i, PHI)
        B = O.gen_phi((k, n), 20000 + i, PHI)
        dA, dB = torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)
        dC = torch.empty((m, n), dtype=torch.float64, device=dev)
        probs.append({"M": m, "N": n, "K": k, "A": dA.data_ptr(), "lda": k, "B": dB.data_ptr(), "ldb": n,
                      "C": dC.data_ptr(), "ldc": n, "error_bound": BOUND})
        hosts.append((A, B, dA, dB, dC))
        flops += 2.0 * m * n * k
    hg = oz.Handle()
    hg.set_graph(1)

    def grouped():
        rc, used = hg.dgemm_grouped(probs, stream.cuda_stream, with_bins=True)
        if rc:
            raise RuntimeError(hg.last_error())
        return used

    def time_grouped(reps=5):
        for _ in range(3):
            u = grouped()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            grouped()
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) / reps * 1e3
        if hg.sync():
            raise RuntimeError(hg.last_error())
        return ms, u

    untuned_ms, used = time_grouped()
    # the autotuner over the workload's size classes (ceil log2 of M, N, K), for the
    # slice schedules the grouped call picked; one representative problem per class
    classes = {}
    for (m, n, k), sj in zip(sizes, used):
        key = (int(np.ceil(np.log2(m))), int(np.ceil(np.log2(n))), int(np.ceil(np.log2(k))), sj)
        classes.setdefault(key, (int(m), int(n), int(k)))
    ht = oz.Handle()
    t0 = time.perf_counter()
    for (_, _, _, (s_, j_)), (m, n, k) in classes.items():
        ht.autotune(m, n, k, 7, s_, j_, max_candidates=12)
    tune_s = time.perf_counter() - t0
    ht.close()
    tuned_ms, _ = time_grouped()
    # the per-class winners, each timed alone, spread the problems over more plan
    # classes (grouped launches); the grouped call is timed again with the
    # planner's own plans (the tuning table cleared), which measured faster
    oz.load().ozgb_tuning_clear()
    g_ms, used = time_grouped()
    # accuracy: 64 sampled entries of 8 problems against the exact products
    worst = 0.0
    for i in range(0, n_probs, max(1, n_probs // 8)):
        A, B, _, _, dC = hosts[i]
        r, c = O.sample_indices(A.shape[0], B.shape[1], 64, i)
        ex, _ = O.exact_entries(A, B, r, c)
        got = dC.cpu().numpy()[r, c]
        worst = max(worst, float(np.linalg.norm(got - ex) / max(np.linalg.norm(ex), 1e-300)))
    hg.close()

    def per_call(configure):
        """Every problem through its own ozgb_dgemm_device call on one handle."""
        hp = oz.Handle()
        configure(hp)

        def run():
            for pb in probs:
                if hp.dgemm_device(pb["M"], pb["N"], pb["K"], pb["A"], pb["lda"], pb["B"], pb["ldb"], pb["C"],
                                   pb["ldc"], stream.cuda_stream):
                    raise RuntimeError(hp.last_error())

        run()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(2):
            run()
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) / 2 * 1e3
        if hp.sync():
            raise RuntimeError(hp.last_error())
        hp.close()
        return ms

    def fixed(s, J):
        def f(h):
            h.set_slices(s)
            h.set_bins(J)
        return f

    # the grouped call's most frequent slice schedule, run per call
    sched = {}
    for sj in used:
        sched[sj] = sched.get(sj, 0) + 1
    s_used, j_used = max(sched, key=sched.get)
    p_ms = per_call(fixed(8, 15))                       # plain: the accurate configuration
    a_ms = per_call(lambda h: h.set_error_bound(BOUND))  # per-call precision knob
    e_ms = per_call(fixed(s_used, j_used))               # per-call, the grouped call's s and pair set
    return {"workload": "%d DGEMMs, M, N, K log-uniform in [32, 2048] (seed 7), phi=1, bound 1e-15 each" % n_probs,
            "effective_flop": flops,
            "autotuned_size_classes": {"classes": len(classes), "tuning_s": tune_s, "grouped_tuned_ms": tuned_ms,
                                       "grouped_untuned_first_ms": untuned_ms,
                                       "note": "per-class winners timed alone; the grouped call below uses the "
                                               "planner's plans (the tuning table cleared)"},
            "grouped_adaptive_graph": {"value": flops / (g_ms * 1e-3) / 1e12, "unit": UNIT, "ms": g_ms,
                                       "schedule_hist": {"s%d_J%d" % k: v for k, v in sorted(sched.items())},
                                       "max_normwise_rel_err_sampled": worst},
            "per_call_same_s_triangular": {"value": flops / (e_ms * 1e-3) / 1e12, "unit": UNIT, "ms": e_ms,
                                           "slices": s_used, "bins": j_used},
            "per_call_adaptive": {"value": flops / (a_ms * 1e-3) / 1e12, "unit": UNIT, "ms": a_ms},
            "plain_per_call_s8_full": {"value": flops / (p_ms * 1e-3) / 1e12, "unit": UNIT, "ms": p_ms},
            "ratios": {
                "grouping_at_equal_s_and_pairs": e_ms / g_ms,
                "adaptive_vs_plain_per_call": p_ms / a_ms,
                "grouped_adaptive_vs_plain_per_call": p_ms / g_ms},
            "speedup": p_ms / g_ms}


def device_phi(shape, seed, phi, dev, torch):
    """a_ij = (U(0,1) - 0.5) exp(phi N(0,1)) drawn on the device (torch's Philox
    generator): the same family as the oracle's gen_phi, for operands too large
    to draw on the host."""
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    x = torch.rand(shape, generator=g, dtype=torch.float64, device=dev).sub_(0.5)
    x.mul_(torch.randn(shape, generator=g, dtype=torch.float64, device=dev).mul_(phi).exp_())
    return x


def sampled_errors(dA, dB, dC, n, seed, O, torch, tail=1e-4, mpfr=True):
    """Errors of n sampled entries of dC against the exact products (and MPFR-106
    when libmpfr loads): only the sampled rows of A and columns of B leave the GPU.
    max_rel is the largest elementwise relative error (the reference's reported
    metric, common.h:585-592); max_rel_kept the same over the entries at least
    tail |a_i| |b_j| / sqrt(K) away from zero (the elementwise criterion's set)."""
    M, N = dC.shape
    K = dA.shape[1]
    r, c = O.sample_indices(M, N, n, seed)
    ri = torch.from_numpy(r.astype(np.int64)).to(dA.device)
    ci = torch.from_numpy(c.astype(np.int64)).to(dA.device)
    As = dA.index_select(0, ri).cpu().numpy()
    Bs = dB.index_select(1, ci).cpu().numpy()
    got = dC[ri, ci].cpu().numpy()
    idx = np.arange(n, dtype=np.int32)
    ex, absdot = O.exact_entries(As, Bs, idx, idx)
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = np.where(ex != 0, np.abs(got - ex) / np.abs(ex), np.where(got == ex, 0.0, np.inf))
    scale = np.sqrt(np.sum(As * As, axis=1) * np.sum(Bs * Bs, axis=0) / K)
    kept = np.abs(ex) >= tail * scale
    out = {"normwise_rel_vs_exact": float(np.linalg.norm(got - ex) / max(np.linalg.norm(ex), 1e-300)),
           "max_rel_vs_exact": float(np.max(rel)),
           "max_rel_kept_vs_exact": float(np.max(rel[kept])) if kept.any() else 0.0,
           "kept": int(kept.sum()),
           "max_componentwise_vs_exact": float(np.max(np.abs(got - ex) / np.maximum(absdot, 1e-300))),
           "entries": n}
    mp = O.mpfr_entries(As, Bs, idx, idx) if mpfr else None
    if mp is not None:
        out["normwise_rel_vs_mpfr106"] = float(np.linalg.norm(got - mp) / max(np.linalg.norm(mp), 1e-300))
        with np.errstate(divide="ignore", invalid="ignore"):
            relm = np.where(mp != 0, np.abs(got - mp) / np.abs(mp), np.where(got == mp, 0.0, np.inf))
        out["max_rel_vs_mpfr106"] = float(np.max(relm))
    return out


def cublas_emulated_run(dA, dB, dC, A, B, r, c, exact, absdot, O, torch):
    """cuBLAS's own fixed-point FP64 emulation on the headline workload, for
    comparison, with the eager strategy: through cublasGemmEx's compute type
    CUBLAS_COMPUTE_64F_EMULATED_FIXEDPOINT, and through cublasDgemm under the math
    mode CUBLAS_FP64_EMULATED_FIXEDPOINT_MATH (mantissa bits chosen by cuBLAS at run
    time, and fixed at 53).  tests/perf/cublas_dgemm.cu is compiled here when nvcc is
    present; any failure is reported, not raised."""
    import ctypes
    import shutil
    import subprocess
    import tempfile
    try:
        nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
        nvcc = nvcc if os.path.exists(nvcc) else shutil.which("nvcc")
        if not nvcc:
            return {"unavailable": "nvcc not found"}
        with tempfile.TemporaryDirectory(prefix="oz_cublas_") as tmp:
            so = os.path.join(tmp, "libcublas_dgemm.so")
            subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-Xcompiler",
                            "-fPIC", "-shared", "-o", so, os.path.join(ROOT, "tests", "perf", "cublas_dgemm.cu"),
                            "-lcublas"], check=True, capture_output=True, timeout=300)
            L = ctypes.CDLL(so)  # stays mapped after the directory is removed
        L.cublas_dgemm_timed.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p] * 3 + [ctypes.c_int] * 3 + \
            [ctypes.POINTER(ctypes.c_float)]
        M, K = dA.shape
        N = dB.shape[1]
        out = {}
        for name, mode, bits in (("gemmex_compute_type", 1, 0), ("math_mode", 2, 0), ("math_mode_53_bits", 2, 53)):
            ms = ctypes.c_float(0.0)
            torch.cuda.synchronize()
            rc = L.cublas_dgemm_timed(M, N, K, dA.data_ptr(), dB.data_ptr(), dC.data_ptr(), mode, bits, 5,
                                      ctypes.byref(ms))
            torch.cuda.synchronize()
            if rc:
                out[name] = {"unavailable": "cublas_dgemm_timed returned %d" % rc}
                continue
            out[name] = {"value": 2.0 * M * N * K / (ms.value * 1e-3) / 1e12, "unit": UNIT, "ms": ms.value,
                         "accuracy_vs_exact": O.error_report(dC.cpu().numpy(), A, B, r, c, exact, absdot)}
        return out
    except Exception as e:  # the comparison line must not stop the benchmark
        return {"unavailable": "%s: %s" % (type(e).__name__, str(e)[:200])}


def time_device(fn, torch, stream, reps=1):
    """Mean device time (ms) of fn() over reps calls, CUDA events on the stream."""
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def long_k_run(dev, stream, oz, O, torch):
    """The long-K workload: M = N = 8192, K = 65536, phi = 1, and the
    ill-conditioned variant with row i of A scaled by 2^(-40 i / M); the accurate
    mode (s = 8, full pair set) and the precision knob at 1e-15, against cuBLAS
    FP64 on the same operands."""
    Ml, Nl, Kl = 8192, 8192, 65536
    flops = 2.0 * Ml * Nl * Kl
    dB = device_phi((Kl, Nl), 32, 1.0, dev, torch)
    dC = torch.empty((Ml, Nl), dtype=torch.float64, device=dev)
    out = {"workload": "M = N = 8192, K = 65536, phi = 1 (device-drawn operands)", "effective_flop": flops}
    for name in ("phi1", "ill_conditioned"):
        dA = device_phi((Ml, Kl), 31, 1.0, dev, torch)
        if name == "ill_conditioned":
            dA.mul_(torch.exp2(-40.0 * torch.arange(Ml, dtype=torch.float64, device=dev) / Ml)[:, None])
        res = {}
        for label in ("accurate_s8_full", "adaptive_1e-15"):
            h = oz.Handle()
            if label == "accurate_s8_full":  # the accurate mode's configuration
                h.set_slices(8)
                h.set_bins(15)
            else:
                h.set_error_bound(BOUND)

            def call():
                if h.dgemm_device(Ml, Nl, Kl, dA.data_ptr(), Kl, dB.data_ptr(), Nl, dC.data_ptr(), Nl,
                                  stream.cuda_stream):
                    raise RuntimeError(h.last_error())

            call()
            ms = time_device(call, torch, stream, 2)
            if h.sync():
                raise RuntimeError(h.last_error())
            cfg = h.config()
            res[label] = {"value": flops / (ms * 1e-3) / 1e12, "unit": UNIT, "ms": ms, "slices": cfg["slices"],
                          "bins": cfg["bins"], "accuracy": sampled_errors(dA, dB, dC, 256, 5, O, torch)}
            h.close()
        if name == "phi1":
            ms = time_device(lambda: torch.matmul(dA, dB, out=dC), torch, stream, 1)
            res["cublas_dgemm"] = {"value": flops / (ms * 1e-3) / 1e12, "unit": UNIT, "ms": ms,
                                   "accuracy": sampled_errors(dA, dB, dC, 256, 5, O, torch)}
        out[name] = res
        del dA
    return out


def mix_sizes(n=64, seed=5, lo=1024, hi=16384):
    """The accuracy-adaptive mix: n square sizes log-uniform in [lo, hi] plus one
    hi^3, each with phi from {0.5, 1, 2, 4} and a bound from {1e-8, 1e-11, 1e-13,
    1e-15}."""
    g = np.random.default_rng(seed)
    sz = [int(x) for x in np.exp(g.uniform(np.log(lo), np.log(hi), n))] + [hi]
    phis = g.choice([0.5, 1.0, 2.0, 4.0], n + 1)
    bounds = g.choice([1e-8, 1e-11, 1e-13, 1e-15], n + 1)
    return list(zip(sz, phis.tolist(), bounds.tolist()))


def mix_run(n, dev, stream, oz, O, torch):
    """Per-problem calls over the mix, one problem resident at a time: the
    precision knob with each problem's own bound under both criteria (normwise,
    and elementwise with tail 1e-4), the plain accurate configuration (s = 8,
    full pair set) and cuBLAS FP64.  Every problem's results are checked on 256
    sampled entries against the exact products (normwise and elementwise on the
    samples); the normwise error over the whole of C is taken against a 16-slice
    Ozaki product, itself checked on those samples against the exact products
    (with heavy-tailed entries, phi = 4, a few large entries carry the norm of C,
    so a sampled normwise error says little about the whole matrix)."""
    probs = mix_sizes(n)

    def handle(slices=0, bins=0, bound=0.0, elementwise=False):
        h = oz.Handle()
        if slices:
            h.set_slices(slices)
            h.set_bins(bins)
        if bound:
            h.set_error_bound(bound)
        if elementwise:
            h.set_error_criterion(oz.Criterion.elementwise, 1e-4)
        return h

    # knob (normwise); knob (elementwise); accurate mode's configuration; 16-slice reference
    ha, he, hp, hr = handle(), handle(elementwise=True), handle(8, 15), handle(16, 16)
    tot = {"adaptive": 0.0, "adaptive_elementwise": 0.0, "plain_s8_full": 0.0, "cublas_dgemm": 0.0}
    flops_all, hist, hist_e, per = 0.0, {}, {}, []
    met = {"normwise_all_vs_16_slices": 0, "normwise_sampled_vs_exact": 0, "elementwise_kept_sampled_vs_exact": 0}
    worst = {"normwise_all_vs_16_slices": 0.0, "elementwise_kept_sampled_vs_exact": 0.0}
    ref_worst = 0.0
    for i, (m, phi, bound) in enumerate(probs):
        dA = device_phi((m, m), 100 + i, phi, dev, torch)
        dB = device_phi((m, m), 200 + i, phi, dev, torch)
        dR = torch.empty((m, m), dtype=torch.float64, device=dev)
        dC = torch.empty_like(dR)
        flops = 2.0 * m ** 3
        flops_all += flops
        ha.set_error_bound(bound)
        he.set_error_bound(bound)

        def call(h, out):
            if h.dgemm_device(m, m, m, dA.data_ptr(), m, dB.data_ptr(), m, out.data_ptr(), m, stream.cuda_stream):
                raise RuntimeError(h.last_error())

        call(hr, dR)
        ref_worst = max(ref_worst, sampled_errors(dA, dB, dR, 64, i, O, torch, mpfr=False)["normwise_rel_vs_exact"])
        rn = torch.linalg.norm(dR).item()
        call(hp, dC)
        tp = time_device(lambda: call(hp, dC), torch, stream)
        ep = torch.linalg.norm(dC - dR).item() / rn
        call(he, dC)
        te = time_device(lambda: call(he, dC), torch, stream)
        if he.sync():
            raise RuntimeError(he.last_error())
        ce = he.config()
        se = "s%d_J%d" % (ce["slices"], ce["bins"])
        ee = sampled_errors(dA, dB, dC, 256, 1000 + i, O, torch, mpfr=False)
        call(ha, dC)
        ta = time_device(lambda: call(ha, dC), torch, stream)
        for h in (ha, hp, hr):
            if h.sync():
                raise RuntimeError(h.last_error())
        ca_ = ha.config()
        s = "s%d_J%d" % (ca_["slices"], ca_["bins"])
        ea = torch.linalg.norm(dC - dR).item() / rn
        sa = sampled_errors(dA, dB, dC, 256, 1000 + i, O, torch, mpfr=False)
        tc = time_device(lambda: torch.matmul(dA, dB, out=dC), torch, stream)
        ec = torch.linalg.norm(dC - dR).item() / rn
        tot["adaptive"] += ta
        tot["adaptive_elementwise"] += te
        tot["plain_s8_full"] += tp
        tot["cublas_dgemm"] += tc
        met["normwise_all_vs_16_slices"] += int(ea <= bound)
        met["normwise_sampled_vs_exact"] += int(sa["normwise_rel_vs_exact"] <= bound)
        met["elementwise_kept_sampled_vs_exact"] += int(ee["max_rel_kept_vs_exact"] <= bound)
        worst["normwise_all_vs_16_slices"] = max(worst["normwise_all_vs_16_slices"], ea / bound)
        worst["elementwise_kept_sampled_vs_exact"] = max(worst["elementwise_kept_sampled_vs_exact"],
                                                         ee["max_rel_kept_vs_exact"] / bound)
        hist[s] = hist.get(s, 0) + 1
        hist_e[se] = hist_e.get(se, 0) + 1
        per.append([m, phi, bound, s, se, round(ta, 3), round(te, 3), round(tp, 3), round(tc, 3), ea,
                    sa["normwise_rel_vs_exact"], sa["max_rel_vs_exact"], ee["max_rel_kept_vs_exact"], ep, ec])
        del dA, dB, dR, dC
    for h in (ha, he, hp, hr):
        h.close()
    return {"workload": "%d square DGEMMs, size log-uniform in [1024, 16384] (seed 5), plus one 16384^3; "
                        "phi from {0.5, 1, 2, 4}, bound from {1e-8, 1e-11, 1e-13, 1e-15} per problem; "
                        "device-drawn operands" % n,
            "effective_flop": flops_all,
            "error_reference": {"sampled": "exact products on 256 sampled entries of every problem",
                                "whole_matrix": "Ozaki, 16 slices, triangular pair set, normwise over all of C",
                                "whole_matrix_reference_worst_sampled_normwise_vs_exact": ref_worst},
            "bounds_met": met, "problems": len(probs), "worst_err_over_bound": worst,
            "adaptive": {"value": flops_all / (tot["adaptive"] * 1e-3) / 1e12, "unit": UNIT, "ms": tot["adaptive"],
                         "criterion": "normwise", "schedule_hist": hist},
            "adaptive_elementwise": {"value": flops_all / (tot["adaptive_elementwise"] * 1e-3) / 1e12, "unit": UNIT,
                                     "ms": tot["adaptive_elementwise"], "criterion": "elementwise, tail 1e-4",
                                     "schedule_hist": hist_e},
            "plain_s8_full": {"value": flops_all / (tot["plain_s8_full"] * 1e-3) / 1e12, "unit": UNIT,
                              "ms": tot["plain_s8_full"]},
            "cublas_dgemm": {"value": flops_all / (tot["cublas_dgemm"] * 1e-3) / 1e12, "unit": UNIT,
                             "ms": tot["cublas_dgemm"]},
            "per_problem": {"columns": ["n", "phi", "bound", "schedule", "schedule_elementwise", "adaptive_ms",
                                        "elementwise_ms", "plain_ms", "cublas_ms", "adaptive_err_all_vs_16",
                                        "adaptive_err_sampled_normwise", "adaptive_err_sampled_max_rel",
                                        "elementwise_err_sampled_max_rel_kept", "plain_err_all_vs_16",
                                        "cublas_err_all_vs_16"], "rows": per}}


def sweep_run(dev, stream, oz, O, torch):
    """The square workload's full grid: M = N = K = 4096, both pair sets (fast:
    triangular, accurate: full), s = 3..8 slices of 7 bits, phi in {0.5, 1, 2, 4}
    (A seed 1, B seed 2).  Errors on 1000 sampled entries against the exact
    products and MPFR-106 (the reference's oracle), and normwise over all of C
    against a 16-slice product; cuBLAS FP64 beside each phi."""
    rows = []
    n = 4096
    for phi in (0.5, 1.0, 2.0, 4.0):
        A = O.gen_phi((n, n), 1, phi)
        B = O.gen_phi((n, n), 2, phi)
        dA, dB = torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)
        dC = torch.empty((n, n), dtype=torch.float64, device=dev)
        dR = torch.empty_like(dC)
        r, c = O.sample_indices(n, n, 1000, 3)
        exact, absdot = O.exact_entries(A, B, r, c)
        mp = O.mpfr_entries(A, B, r, c)
        hr = oz.Handle()
        hr.set_slices(16)
        hr.set_bins(16)
        if hr.dgemm_device(n, n, n, dA.data_ptr(), n, dB.data_ptr(), n, dR.data_ptr(), n, stream.cuda_stream):
            raise RuntimeError(hr.last_error())
        hr.close()
        rn = torch.linalg.norm(dR).item()

        def errs(C):
            got = C[r, c]
            e = {"sampled_normwise_vs_exact": float(np.linalg.norm(got - exact) / np.linalg.norm(exact)),
                 "sampled_max_rel_vs_exact": float(np.max(np.abs(got - exact) / np.maximum(np.abs(exact), 1e-300))),
                 "sampled_max_componentwise": float(np.max(np.abs(got - exact) / np.maximum(absdot, 1e-300)))}
            if mp is not None:
                e["sampled_normwise_vs_mpfr106"] = float(np.linalg.norm(got - mp) / np.linalg.norm(mp))
                e["sampled_max_rel_vs_mpfr106"] = float(np.max(np.abs(got - mp) / np.maximum(np.abs(mp), 1e-300)))
            return e

        ms = time_device(lambda: torch.matmul(dA, dB, out=dC), torch, stream, 1)
        e = errs(dC.cpu().numpy())
        e["normwise_all_vs_16_slices"] = torch.linalg.norm(dC - dR).item() / rn
        rows.append({"phi": phi, "impl": "cublas_dgemm", "ms": ms, "tflops": 2.0 * n ** 3 / ms / 1e9, **e})
        for mode in ("fast", "accurate"):
            for sl in range(3, 9):
                h = oz.Handle()
                h.set_slices(sl)
                h.set_bins(sl if mode == "fast" else 2 * sl - 1)

                def call():
                    if h.dgemm_device(n, n, n, dA.data_ptr(), n, dB.data_ptr(), n, dC.data_ptr(), n,
                                      stream.cuda_stream):
                        raise RuntimeError(h.last_error())

                call()
                ms = time_device(call, torch, stream, 3)
                if h.sync():
                    raise RuntimeError(h.last_error())
                h.close()
                e = errs(dC.cpu().numpy())
                e["normwise_all_vs_16_slices"] = torch.linalg.norm(dC - dR).item() / rn
                rows.append({"phi": phi, "impl": "ozaki_%s_s%d" % (mode, sl), "ms": ms,
                             "tflops": 2.0 * n ** 3 / ms / 1e9, **e})
        del dA, dB, dC, dR
    return {"workload": "M = N = K = 4096, a = (U - 0.5) exp(phi N), A seed 1, B seed 2", "rows": rows}


def profile_grouped(n_probs):
    """The batched workload's grouped call without graphs, per-stage device times,
    for each launch form (1: one GEMM launch per plan class, 0: one per problem);
    the sixth call of each form runs inside the NVTX range oz_grouped_step so that
    an ncu capture can select it."""
    import torch
    import ozaie_gb300 as oz
    from oracle import ozoracle as O
    dev = torch.device("cuda", 0)
    probs, keep = [], []
    for i, (m, n, k) in enumerate(batched_workload(n_probs)):
        m, n, k = int(m), int(n), int(k)
        dA = torch.from_numpy(O.gen_phi((m, k), 10000 + i, PHI)).to(dev)
        dB = torch.from_numpy(O.gen_phi((k, n), 20000 + i, PHI)).to(dev)
        dC = torch.empty((m, n), dtype=torch.float64, device=dev)
        probs.append({"M": m, "N": n, "K": k, "A": dA.data_ptr(), "lda": k, "B": dB.data_ptr(), "ldb": n,
                      "C": dC.data_ptr(), "ldc": n, "error_bound": BOUND})
        keep.append((dA, dB, dC))
    stream = torch.cuda.current_stream().cuda_stream
    out = {}
    for launch in (1, 0):
        h = oz.Handle()
        h.set_grouped_launch(launch)
        h.set_profiling(True)
        n0 = h.launch_count()
        for r in range(6):
            if r == 5:
                torch.cuda.nvtx.range_push("oz_grouped_step")
            rc, _ = h.dgemm_grouped(probs, stream)
            if r == 5:
                torch.cuda.nvtx.range_pop()
            if rc:
                raise RuntimeError(h.last_error())
            torch.cuda.synchronize()
        if h.sync():
            raise RuntimeError(h.last_error())
        out["launch_per_class" if launch else "launch_per_problem"] = {
            "stage_ms": h.stage_times(), "launches_per_call": (h.launch_count() - n0) / 6}
        h.close()
    # wall time per call (five calls back to back) of the default form, with and without graphs
    for graph in (0, 1):
        h = oz.Handle()
        h.set_graph(graph)
        for _ in range(3):
            h.dgemm_grouped(probs, stream)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(5):
            rc, _ = h.dgemm_grouped(probs, stream)
            if rc:
                raise RuntimeError(h.last_error())
        torch.cuda.synchronize()
        out["wall_ms_graph%d" % graph] = (time.perf_counter() - t0) / 5 * 1e3
        if h.sync():
            raise RuntimeError(h.last_error())
        h.close()
    print(json.dumps({"profile_grouped": True, "problems": n_probs, **out}))
    return 0


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import ozoracle as O
    A = O.gen_phi((M, K), 1, PHI)
    B = O.gen_phi((K, N), 2, PHI)
    # the slice schedule the GPU arm's precision knob picks for this workload and bound
    s, J = 8, 9
    rows = 64
    for _ in range(args.warmup):
        O.dgemm_rows(A, B, 7, s, J, 0, 0, 2)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.dgemm_rows(A, B, 7, s, J, 0, 0, rows)
        times.append(time.perf_counter() - t0)
    dt = statistics.median(times)
    v = 2.0 * rows * N * K / dt / 1e12
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int8 slices, int64 bins, f64 in/out", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample_rows": rows, "slices": s, "bins": J},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": O.num_threads(), "kind": "port",
                             "sample": "%d of %d rows per step" % (rows, M)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-only", action="store_true",
                    help="only the timed DGEMM steps (for ncu launch lists and captures)")
    ap.add_argument("--profile-grouped", action="store_true",
                    help="only the batched workload's grouped call, without graphs, both launch forms: per-stage "
                         "times, the sixth call of each form inside the NVTX range oz_grouped_step")
    ap.add_argument("--case", type=int, default=0, help="square size for --profile-only (default 4096)")
    ap.add_argument("--slices", type=int, default=0, help="fixed triangular slice count for --profile-only")
    ap.add_argument("--batched", type=int, default=512, help="problems in the batched comparison (0: skip)")
    ap.add_argument("--no-autotune", action="store_true", help="use the planner's cost-model plans")
    ap.add_argument("--no-longk", action="store_true", help="skip the long-K workload (8192^2 x 65536)")
    ap.add_argument("--mix", type=int, default=64, help="problems of the accuracy-adaptive mix (0: skip)")
    ap.add_argument("--no-sweep", action="store_true",
                    help="skip the 4096^3 grid: both pair sets, s = 3..8, phi in {0.5, 1, 2, 4}")
    ap.add_argument("--quick", action="store_true", help="headline only: no batched, long-K, mix or sweep runs")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.quick:
        args.batched, args.mix, args.no_longk, args.no_sweep = 0, 0, True, True
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import torch.distributed as dist

    import ozaie_gb300 as oz
    from oracle import ozoracle as O

    if args.profile_grouped:
        return profile_grouped(args.batched or 512)

    global M, N, K
    if args.profile_only and args.case:
        M = N = K = args.case
    ws, rank, local = dist_env()
    if ws > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    A = O.gen_phi((M, K), 1 + 1000 * rank, PHI)
    B = O.gen_phi((K, N), 2 + 1000 * rank, PHI)
    dA = torch.from_numpy(A).to(dev)
    dB = torch.from_numpy(B).to(dev)
    dC = torch.empty((M, N), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)

    h = oz.Handle()
    tuned = None
    if not args.no_autotune:
        # the precision knob picks s = 9 for this workload: tune that plan (and its
        # neighbours) before anything is timed
        # the slice schedules the knob picks here (normwise: s = 8 with the pair
        # set p + q <= 8; elementwise: s = 11, p + q <= 11) and their neighbours
        tuned = {"s%d_J%d" % (s, J): h.autotune(M, N, K, 7, s, J, max_candidates=24)
                 for s, J in ((8, 9), (9, 9), (9, 10), (11, 12), (12, 12))}
    h.set_error_bound(BOUND)
    if args.profile_only and args.slices:
        h.set_slices(args.slices)
        h.set_bins(args.slices)

    def step():
        rc = h.dgemm_device(M, N, K, dA.data_ptr(), K, dB.data_ptr(), N, dC.data_ptr(), N, stream.cuda_stream)
        if rc:
            raise RuntimeError(h.last_error())

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if h.sync():
        raise RuntimeError(h.last_error())
    cfg = h.config()
    if args.profile_only:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        if h.sync():
            raise RuntimeError(h.last_error())
        h.set_profiling(True)
        # the profiled step sits in an NVTX range, so an ncu capture can select it
        # (ncu --nvtx --nvtx-include oz_profile_step/) after the autotuner's trial launches
        torch.cuda.nvtx.range_push("oz_profile_step")
        step()
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        st_ms = h.stage_times()
        h.set_profiling(False)
        gemm_tf = 2.0 * cfg["pairs"] * M * N * K / (st_ms["gemm"] * 1e-3) / 1e12
        print(json.dumps({"profile_only": True, "M": M, "N": N, "K": K, "ms_per_step": ms,
                          "tflops": 2.0 * M * N * K / (ms * 1e-3) / 1e12, "stage_ms": st_ms,
                          "gemm_mma_tflops": gemm_tf, "config": cfg}))
        h.close()
        return 0

    # accuracy of this configuration on 1000 sampled entries (outside the timed region)
    C = dC.cpu().numpy()
    r, c = O.sample_indices(M, N, 1000, 3)
    exact, absdot = O.exact_entries(A, B, r, c)
    err = O.error_report(C, A, B, r, c, exact, absdot)
    mp = O.mpfr_entries(A, B, r, c) if rank == 0 else None
    err_mpfr = O.error_report(C, A, B, r, c, mp, absdot) if mp is not None else None

    # per-stage device times (events on the launching stream)
    h.set_profiling(True)
    stage = []
    for _ in range(3):
        step()
        torch.cuda.synchronize()
        stage.append(h.stage_times())
    h.set_profiling(False)
    gemm_ms = statistics.median([t["gemm"] for t in stage])

    clocks = ClockSampler(local)
    clocks.start()
    for _ in range(max(3, args.warmup)):  # keeps the GPU busy while the sampler starts
        step()
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    n_launch0 = h.launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    ms = e0.elapsed_time(e1) / args.steps
    gpu_launches = h.launch_count() - n_launch0
    clk = clocks.stop()
    if h.sync():
        raise RuntimeError(h.last_error())
    ms = max_over_ranks(ms, dev)
    flops = 2.0 * M * N * K
    value = flops * ws / (ms * 1e-3) / 1e12

    # e2e: host arrays through the reference-facing call (ozAIE_DGEMM semantics),
    # copies in and out inside the timed region.  Primary: plain pageable numpy
    # arrays, as the reference's own caller passes std::vector memory
    # (example/oztest.cpp); also pinned arrays, as a caller streaming many products
    # would keep them.
    e2e_steps = max(3, min(args.steps, 10))

    def e2e_time(Ah, Bh, Ch):
        he = oz.Handle()
        he.set_error_bound(BOUND)
        assert he.setup(M, N, K, oz.Mode.fast) == 0, he.last_error()
        for _ in range(2):
            assert he.dgemm(M, N, K, Ah, Bh, Ch) == 0, he.last_error()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            assert he.dgemm(M, N, K, Ah, Bh, Ch) == 0, he.last_error()
        t = (time.perf_counter() - t0) / e2e_steps * 1e3
        he.close()
        return t

    e2e_ms = e2e_time(np.ascontiguousarray(A), np.ascontiguousarray(B), np.empty((M, N)))
    e2e_pinned_ms = e2e_time(torch.from_numpy(A).pin_memory().numpy(), torch.from_numpy(B).pin_memory().numpy(),
                             torch.empty((M, N), dtype=torch.float64).pin_memory().numpy())

    # the same product with the knob's elementwise criterion: relative error of
    # every entry at least 1e-4 |a_i| |b_j| / sqrt(K) away from zero <= 1e-15
    hq = oz.Handle()
    hq.set_error_bound(BOUND)
    hq.set_error_criterion(oz.Criterion.elementwise, 1e-4)

    def step_e():
        if hq.dgemm_device(M, N, K, dA.data_ptr(), K, dB.data_ptr(), N, dC.data_ptr(), N, stream.cuda_stream):
            raise RuntimeError(hq.last_error())

    for _ in range(3):
        step_e()
    el_ms = time_device(step_e, torch, stream, max(3, min(args.steps, 20)))
    if hq.sync():
        raise RuntimeError(hq.last_error())
    el_cfg = hq.config()
    hq.close()
    el_err = sampled_errors(dA, dB, dC, 1000, 3, O, torch) if rank == 0 else None
    elementwise_mode = {
        "value": 2.0 * M * N * K / (el_ms * 1e-3) / 1e12, "unit": UNIT, "ms_per_step": el_ms,
        "criterion": "elementwise relative error <= 1e-15 for every entry with |c_ij| >= 1e-4 |a_i| |b_j| / sqrt(K)",
        "slices": el_cfg["slices"], "bins": el_cfg["bins"], "pairs": el_cfg["pairs"], "accuracy": el_err,
        "valid_elementwise_all_sampled_vs_mpfr106": bool(el_err and el_err.get("max_rel_vs_mpfr106", 1.0) <= BOUND),
        "valid_elementwise_kept_sampled_vs_exact": bool(el_err and el_err["max_rel_kept_vs_exact"] <= BOUND)}

    # native FP64 DGEMM (cuBLAS through torch) on the same GPU, and its accuracy
    for _ in range(2):
        torch.matmul(dA, dB, out=dC)
    torch.cuda.synchronize()
    c0 = torch.cuda.Event(enable_timing=True)
    c1 = torch.cuda.Event(enable_timing=True)
    c0.record(stream)
    for _ in range(3):
        torch.matmul(dA, dB, out=dC)
    c1.record(stream)
    torch.cuda.synchronize()
    cublas_ms = c0.elapsed_time(c1) / 3
    err_cublas = O.error_report(dC.cpu().numpy(), A, B, r, c, exact, absdot)
    cublas_emulated = cublas_emulated_run(dA, dB, dC, A, B, r, c, exact, absdot, O, torch) if rank == 0 else None

    batched = batched_run(args.batched, dev, stream, oz, O, torch) if args.batched > 0 and rank == 0 else None
    long_k = long_k_run(dev, stream, oz, O, torch) if not args.no_longk and rank == 0 else None
    mix = mix_run(args.mix, dev, stream, oz, O, torch) if args.mix > 0 and rank == 0 else None
    sweep = sweep_run(dev, stream, oz, O, torch) if not args.no_sweep and rank == 0 else None

    peaks = load_peaks()
    mma_flops = 2.0 * cfg["pairs"] * M * N * K
    achieved = mma_flops / (gemm_ms * 1e-3) / 1e12
    traffic = profile_traffic()

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64 in/out; int8-valued bf16 slices on tcgen05 kind::f16, exact fp32->int accumulation",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "M": M, "N": N, "K": K, "phi": PHI, "error_bound": BOUND,
                       "slices": cfg["slices"], "bits": cfg["bits"], "bins": cfg["bins"], "pairs": cfg["pairs"],
                       "tile_n": cfg["tile_n"], "k_chunk": cfg["k_chunk"], "stages": cfg["stages"],
                       "l2": "inputs + slice planes (~870 MB) larger than L2 (126 MB); no flush needed",
                       "parallelism": "weak: one independent DGEMM per GPU" if ws > 1 else "single GPU"},
            "valid": bool(err["normwise_rel"] <= BOUND and (err_mpfr is None or err_mpfr["normwise_rel"] <= BOUND)),
            "accuracy_gate": {
                "bound": BOUND,
                "applies_to": "normwise relative error |C^ - C|_F / |C|_F on 1000 sampled entries, against the "
                              "exact products and against MPFR-106",
                "why_not_elementwise": "the largest elementwise relative error is set by entries that cancel to "
                                       "near zero: native FP64 DGEMM (cublas_dgemm_vs_exact.max_rel) misses 1e-15 by "
                                       "three orders of magnitude on these inputs; the elementwise form of the "
                                       "bound is reported under elementwise_mode"},
            "accuracy": {"vs_exact": err, "vs_mpfr106": err_mpfr, "cublas_dgemm_vs_exact": err_cublas},
            "elementwise_mode": elementwise_mode,
            "stage_ms": {k: statistics.median([t[k] for t in stage]) for k in stage[0]},
            "cublas_dgemm": {"value": flops / (cublas_ms * 1e-3) / 1e12, "unit": UNIT, "ms": cublas_ms},
            "cublas_fp64_emulated": cublas_emulated,
            "e2e": {"value": flops / (e2e_ms * 1e-3) / 1e12, "unit": UNIT, "ms_per_step": e2e_ms,
                    "host_memory": "pageable (plain numpy arrays)",
                    "h2d_bytes_per_step": 2 * M * K * 8, "d2h_bytes_per_step": M * N * 8,
                    "pinned": {"value": flops / (e2e_pinned_ms * 1e-3) / 1e12, "unit": UNIT,
                               "ms_per_step": e2e_pinned_ms}},
            "roofline": {"bound": "tensor", "kernel": "oz_gemm_kernel (slice-pair GEMM + exact drain + decode)",
                         "achieved": achieved, "peak": peaks["bf16_tflops"], "unit": "TFLOP/s",
                         "frac": achieved / peaks["bf16_tflops"], "traffic": traffic,
                         "peak_source": peaks["source"] + " bf16 burst (cuBLAS)",
                         "algorithmic": "2 * pairs * M * N * K bf16 MMA flops per launch"},
            "gpu_launches": gpu_launches,
            "batched": batched,
            "long_k": long_k,
            "adaptive_mix": mix,
            "sweep_4096": sweep,
            "autotuned": {s: {k: v for k, v in c.items() if k in ("tile_n", "k_chunk", "stages", "blocks", "block_lo",
                                                                 "block_nb", "issuers")} for s, c in tuned.items()}
            if tuned else None,
            "clocks": clk,
        }
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(A, B, cfg["slices"], cfg["bins"])
            line["cpu_blas_dgemm"] = cpu_blas_dgemm(A, B)
        print(json.dumps(line))
    h.close()
    if ws > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
