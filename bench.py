#!/usr/bin/env python
"""Benchmark of the GB300 sgemm_/dgemm_ path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME]

Metric: GEMM TFLOP/s (2*m*n*k per second) on one GB300 of the tensor-core
split form at equal error to the native FP32/FP64 kernel.  A step is one call
of the split form (split kernels + tcgen05 GEMM) over the workload's inputs,
already resident in HBM.  The default workload is SGEMM TN m=n=k=8192,
alpha=1, beta=0 (the configuration the metric is quoted on); the split form
(3xBF16, 6xBF16, scaled 3xFP16, or the autotuned layout of the shape class)
is the fastest of those whose max relative error on sampled entries does not
exceed the plain FP32 kernel's; --form pins one (e.g. fp16x3_c8_t256_pair).

Printed JSON line (rank 0): metric/value/unit, ms_per_step, e2e (the same
metric through the host-pointer C ABI with host<->device copies inside the
timed region), roofline of the dominant kernel (the tcgen05 GEMM), the plain
kernel's TFLOP/s and errors of both forms against exact sampled dot products,
clocks sampled during the timed region, gpu_launches, and a CPU baseline.

--impl reference times the reference's CPU implementation of the same
workload on all host cores (the reference library compiled from its sources
when this host can run it, else the oracle's C restatement of its algorithm).
Every step of that arm, and the GPU arm's cpu_baseline leg, compute the same
thing: the whole workload when its work is at most SGEMM 8192^3's, else a
fixed leading block of columns of C with that much work.

N > 1 (torchrun): every rank runs the same single-GPU workload (the path
shards by whole problems; replicas only), value = sum over ranks of the work /
max over ranks of the time.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # configs: SGEMM TN 8192^3 (the metric's configuration), DGEMM NN 2048^3,
    # DGEMM NT 16384^3 (phi = 0), rank-256 updates with padded ld.
    "sgemm_tn_8192": dict(prec="s", ta="T", tb="N", m=8192, n=8192, k=8192, lda=8192, ldb=8192,
                          ldc=8192, alpha=1.0, beta=0.0, seed=1),
    # the split forms at m = n = k = 16384, the size their speed-up targets are quoted at
    "sgemm_tn_16384": dict(prec="s", ta="T", tb="N", m=16384, n=16384, k=16384, lda=16384,
                           ldb=16384, ldc=16384, alpha=1.0, beta=0.0, seed=1),
    # a smaller case of the same kernels for ncu captures (split operands still > L2)
    "sgemm_tn_4096": dict(prec="s", ta="T", tb="N", m=4096, n=4096, k=4096, lda=4096, ldb=4096,
                          ldc=4096, alpha=1.0, beta=0.0, seed=1),
    "dgemm_nt_4096": dict(prec="d", ta="N", tb="T", m=4096, n=4096, k=4096, lda=4096, ldb=4096,
                          ldc=4096, alpha=1.0, beta=1.0, seed=2),
    "dgemm_nn_2048": dict(prec="d", ta="N", tb="N", m=2048, n=2048, k=2048, lda=2048, ldb=2048,
                          ldc=2048, alpha=1.0, beta=0.5, seed=0),
    "dgemm_nt_16384": dict(prec="d", ta="N", tb="T", m=16384, n=16384, k=16384, lda=16384,
                           ldb=16384, ldc=16384, alpha=1.0, beta=1.0, seed=2),
    "rank256_d": dict(prec="d", ta="N", tb="T", m=32768, n=32768, k=256, lda=32800, ldb=32800,
                      ldc=32832, alpha=-1.0, beta=1.0, seed=3),
    "rank256_s": dict(prec="s", ta="N", tb="T", m=32768, n=32768, k=256, lda=32800, ldb=32800,
                      ldc=32832, alpha=-1.0, beta=1.0, seed=3),
    # the rank-256 updates at a sixteenth of the output, for ncu captures (C still > L2)
    "rank256_d_8192": dict(prec="d", ta="N", tb="T", m=8192, n=8192, k=256, lda=8224, ldb=8224,
                           ldc=8256, alpha=-1.0, beta=1.0, seed=3),
    "rank256_s_8192": dict(prec="s", ta="N", tb="T", m=8192, n=8192, k=256, lda=8224, ldb=8224,
                           ldc=8256, alpha=-1.0, beta=1.0, seed=3),
}
# blocked TRSM (X = alpha inv(op(A)) B, left, lower, no transpose, non-unit
# diagonal) on the GEMM kernels: m^2 n flops per call
TRSM_WORKLOADS = {
    "dtrsm_lln_8192": dict(prec="d", m=8192, n=8192, alpha=1.0, seed=7),
    "strsm_lln_8192": dict(prec="s", m=8192, n=8192, alpha=1.0, seed=7),
    # triangular multiply B = op(A) B, the same shape
    "dtrmm_lln_8192": dict(prec="d", m=8192, n=8192, alpha=1.0, seed=7, routine="trmm"),
    "strmm_lln_8192": dict(prec="s", m=8192, n=8192, alpha=1.0, seed=7, routine="trmm"),
}
# complex GEMM (the reference's OpenBLAS-style c/z kernels): the split form on
# the embedded real problem, at equal error to the plain 4M method
CWORKLOADS = {
    "zgemm_nn_4096": dict(prec="z", ta="N", tb="N", m=4096, n=4096, k=4096, alpha=1.0, beta=1.0,
                          seed=5),
    "cgemm_nn_8192": dict(prec="c", ta="N", tb="N", m=8192, n=8192, k=8192, alpha=1.0, beta=1.0,
                          seed=6),
}
METRIC = "GEMM TFLOP/s on 1 GB300: tensor-core split vs native FP64/FP32, at equal error"
L2_BYTES = 129 * 2**20


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": d.get("hbm_gbs", 6800.0), "bf16_tflops": d.get("bf16_tflops", 1900.0),
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained", 1700.0),
                "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
            "source": "fallback"}


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return None
        sm = sorted(float(r[1]) for r in rows if r[1].replace(".", "").isdigit())
        mx = max((float(r[2]) for r in rows if r[2].replace(".", "").isdigit()), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx,
                "reasons": reasons, "samples": len(rows)}


# ----------------------------------------------------------------------------- exact samples
def _two_prod(a, b):
    """Dekker/Veltkamp TwoProduct without FMA: a*b = p + e exactly (numpy float64)."""
    import numpy as np

    p = a * b
    c = 134217729.0
    t = c * a
    ah = t - (t - a)
    al = a - ah
    t = c * b
    bh = t - (t - b)
    bl = b - bh
    e = ((ah * bh - p) + ah * bl + al * bh) + al * bl
    return p, np.asarray(e)


def exact_samples(A_rows, B_cols, alpha, beta, c0):
    """Correctly rounded alpha*dot + beta*c for each sampled (row of op(A), column of op(B))."""
    import numpy as np

    out = np.empty(A_rows.shape[0])
    for q in range(A_rows.shape[0]):
        p, e = _two_prod(A_rows[q].astype(np.float64), B_cols[q].astype(np.float64))
        dot = math.fsum(np.concatenate([p, e]).tolist())
        out[q] = math.fsum([alpha * dot, beta * float(c0[q])])
    return out


def rel_err(got, truth):
    import numpy as np

    d = np.abs(np.asarray(got, np.float64) - truth)
    mx = float(np.max(d / np.maximum(np.abs(truth), 1e-300)))
    fro = float(np.linalg.norm(d) / max(np.linalg.norm(truth), 1e-300))
    return mx, fro


# ----------------------------------------------------------------------------- workload
class Problem:
    """Device-resident operands of one workload (column-major, seeded U[-1,1))."""

    def __init__(self, torch, w):
        self.w = w
        dt = torch.float64 if w["prec"] == "d" else torch.float32
        gen = torch.Generator(device="cuda")
        gen.manual_seed(int(w["seed"]))
        ar, ac = (w["m"], w["k"]) if w["ta"] == "N" else (w["k"], w["m"])
        br, bc = (w["k"], w["n"]) if w["tb"] == "N" else (w["n"], w["k"])
        self.ar, self.ac, self.br, self.bc = ar, ac, br, bc
        # column-major ld x cols buffers are stored as row-major (cols, ld) tensors
        phi = float(w.get("phi", 0.0))
        if phi > 0.0:
            # exponent-spread inputs a = (u - 0.5) * exp(phi * g), u ~ U[0,1), g ~ N(0,1)
            def spread(shape):
                u = torch.rand(shape, generator=gen, device="cuda", dtype=torch.float64)
                gn = torch.randn(shape, generator=gen, device="cuda", dtype=torch.float64)
                return ((u - 0.5) * torch.exp(phi * gn)).to(dt)
            self.A = spread((ac, w["lda"]))
            self.B = spread((bc, w["ldb"]))
        else:
            self.A = torch.rand((ac, w["lda"]), generator=gen, device="cuda", dtype=dt) * 2 - 1
            self.B = torch.rand((bc, w["ldb"]), generator=gen, device="cuda", dtype=dt) * 2 - 1
        self.C0 = torch.rand((w["n"], w["ldc"]), generator=gen, device="cuda", dtype=dt) * 2 - 1
        if w["beta"] == 0.0:
            self.C0.zero_()
        self.C = self.C0.clone()
        self.flops = 2.0 * w["m"] * w["n"] * w["k"]

    def opA_rows(self, rows):
        A = self.A[:, :self.ar] if True else None  # (cols, ld) -> element (r, c) = A[c, r]
        if self.w["ta"] == "N":   # op(A)[i, :] = A[i, 0:k] -> tensor[0:k, i]
            return A[:, rows].T.cpu().numpy()
        return A[rows, :].cpu().numpy()  # op(A)[i, :] = A^T[i, :] = stored column i

    def opB_cols(self, cols):
        B = self.B[:, :self.br]
        if self.w["tb"] == "N":   # op(B)[:, j] = stored column j
            return B[cols, :].cpu().numpy()
        return B[:, cols].T.cpu().numpy()  # op(B)[:, j] = stored row j


def sample_truth(prob, n_samples=1024):
    import numpy as np

    w = prob.w
    rng = np.random.default_rng(99)
    rows = rng.integers(0, w["m"], n_samples)
    cols = rng.integers(0, w["n"], n_samples)
    Ar = prob.opA_rows(rows)
    Bc = prob.opB_cols(cols)
    c0 = prob.C0[cols, rows].cpu().numpy()
    return rows, cols, exact_samples(Ar, Bc, w["alpha"], w["beta"], c0)


# ----------------------------------------------------------------------------- our arm
def workload_config(name, w, world):
    """The `config` object of a workload's JSON line, the same in both arms:
    the workload and its call arguments (the split form the GPU arm chose is
    reported beside it, under "form")."""
    cplx = name in CWORKLOADS
    esz = {"d": 8, "s": 4, "z": 16, "c": 8}[w["prec"]]
    if cplx:
        a_bytes = w["m"] * w["k"] * esz
        cfg = {"workload": name, "transa": w["ta"], "transb": w["tb"], "m": w["m"], "n": w["n"],
               "k": w["k"], "alpha": w["alpha"], "beta": w["beta"], "flops_per_call": "8mnk"}
    else:
        a_bytes = w["lda"] * (w["k"] if w["ta"] == "N" else w["m"]) * esz
        cfg = {"workload": name, "transa": w["ta"], "transb": w["tb"], "m": w["m"], "n": w["n"],
               "k": w["k"], "lda": w["lda"], "ldb": w["ldb"], "ldc": w["ldc"],
               "alpha": w["alpha"], "beta": w["beta"], "phi": float(w.get("phi", 0.0))}
    if a_bytes > L2_BYTES:
        cfg["l2"] = "inputs larger than L2 (%d MB per operand > %d MB)" % (a_bytes // 2**20,
                                                                           L2_BYTES // 2**20)
    else:
        cfg["l2"] = "inputs fit in L2 (%d MB per operand <= %d MB): warm-L2 timing" % (
            a_bytes // 2**20, L2_BYTES // 2**20)
    cfg["parallelism"] = "replicas" if world > 1 else "single"
    return cfg


def run_ours(args, torch, rank, world):
    import numpy as np

    import gemm_avx2_gb300 as g

    w = dict(WORKLOADS[args.workload])
    if args.phi is not None:
        w["phi"] = args.phi
    prob = Problem(torch, w)
    stream = torch.cuda.current_stream().cuda_stream
    is_d = w["prec"] == "d"
    m, n, k = w["m"], w["n"], w["k"]

    def plain_call(C):
        return g.gemm_device(w["prec"], w["ta"], w["tb"], m, n, k, w["alpha"], prob.A.data_ptr(),
                             w["lda"], prob.B.data_ptr(), w["ldb"], w["beta"], C.data_ptr(),
                             w["ldc"], stream)

    # ---- accuracy of the plain kernel and of the split candidates (sampled, exact truth)
    rows, cols, truth = sample_truth(prob)
    prob.C.copy_(prob.C0)
    # the equal-error bar: the plain kernel's full-K accumulation (split-K
    # off), as the autotuner measures it; the throughput below is the plain
    # call as shipped (split along K where the shape asks for it)
    g.tune_param(g.TUNE_SPLIT_K, 1)
    try:
        assert plain_call(prob.C) == g.OK
    finally:
        g.tune_param(g.TUNE_SPLIT_K, 0)
    torch.cuda.synchronize()
    plain_err = rel_err(prob.C[cols, rows].cpu().numpy(), truth)
    # candidates: FP32: BF16xP products; FP64: the CRT form's moduli and the
    # slice form's slice counts.  Per scheme, the smallest one whose max and
    # Frobenius errors do not exceed the plain kernel's; for FP64 the faster
    # of the two qualifying schemes is timed below.
    schemes = [("crt", list(range(11, 25))), ("ozaki", list(range(6, 13)))] if is_d else \
        [("bf16x", [3, 6]), ("bf16x", [g.FP16X3])]
    # FP32: the autotuner's choice for this shape class on these operands
    # (form, chunk length, tile width, cluster mode), products = 0 below
    tuned = None
    if not is_d and not args.form:
        rc, chosen = g.autotune(g.TUNE_BF16X, w["ta"], w["tb"], m, n, k, prob.A.data_ptr(),
                                w["lda"], prob.B.data_ptr(), w["ldb"], stream)
        if rc == g.OK:
            _, tp, tc = g.tune_lookup(g.TUNE_BF16X, m, n, k)
            _, tile, mode = g.tune_layout(g.TUNE_BF16X, m, n, k)
            tuned = {"products": tp, "chunk": tc, "tile_n": tile,
                     "cluster": "pair MMAs" if mode == 1 else "one CTA per tile"}
            schemes.append(("bf16x", [0]))
    errs, qualified = {}, []
    ws = None

    def kind_of(f):
        return {"bf16x": 0, "ozaki": 1, "crt": 2}[f]

    def run_form(f, prm, need, C):
        assert g.split_prepare(f, w["ta"], w["tb"], m, n, k, prob.A.data_ptr(), w["lda"],
                               prob.B.data_ptr(), w["ldb"], prm, ws.data_ptr(), need,
                               stream) == g.OK
        assert g.split_run(f, m, n, k, w["alpha"], w["beta"], C.data_ptr(), w["ldc"], prm,
                           ws.data_ptr(), need, stream) == g.OK

    def name_of(f, prm):
        if f == "bf16x" and prm == 0 and tuned:
            base = "fp16x3" if tuned["products"] == g.FP16X3 else "bf16x%d" % tuned["products"]
            return "tuned:%s_c%d_t%d_%s" % (base, tuned["chunk"], tuned["tile_n"],
                                            "pair" if tuned["cluster"] == "pair MMAs" else "cta")
        if f == "bf16x" and prm == g.FP16X3:
            return "fp16x3"
        return {"bf16x": "bf16x%d", "ozaki": "ozaki_s%d", "crt": "crt_n%d"}[f] % prm

    for f, cands in schemes:
        for prm in cands:
            need = g.split_workspace_bytes(kind_of(f), m, n, k, prm)
            if need == 0:
                continue
            if ws is None or ws.numel() < need:
                ws = None
                torch.cuda.empty_cache()
                ws = torch.empty(need, dtype=torch.uint8, device="cuda")
            prob.C.copy_(prob.C0)
            run_form(f, prm, need, prob.C)
            torch.cuda.synchronize()
            e = rel_err(prob.C[cols, rows].cpu().numpy(), truth)
            errs[name_of(f, prm)] = e
            if e[0] <= plain_err[0] and e[1] <= plain_err[1]:
                qualified.append((f, prm))
                break
    if not qualified:
        f, cands = schemes[-1]
        qualified.append((f, cands[-1]))
    forced = parse_form(args.form) if args.form else None
    if forced:
        form, param = forced
    elif len(qualified) > 1:
        # time each qualifying form (one warm-up, two calls) and keep the faster
        best = None
        for f, prm in qualified:
            need = g.split_workspace_bytes(kind_of(f), m, n, k, prm)
            run_form(f, prm, need, prob.C)
            a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a0.record()
            for _ in range(2):
                run_form(f, prm, need, prob.C)
            a1.record()
            torch.cuda.synchronize()
            t_ = a0.elapsed_time(a1)
            if best is None or t_ < best[0]:
                best = (t_, f, prm)
        form, param = best[1], best[2]
    else:
        form, param = qualified[0]
    # a pinned layout keeps its full name (chunk, tile width, cluster mode)
    form_name = (args.form[len("tuned:"):] if args.form.startswith("tuned:") else args.form) \
        if forced else name_of(form, param)
    need = g.split_workspace_bytes(kind_of(form), m, n, k, param)
    if ws is None or ws.numel() < need:
        ws = None
        torch.cuda.empty_cache()
        ws = torch.empty(need, dtype=torch.uint8, device="cuda")

    # ---- timed region: W warm-up + K steps of prepare + run, inputs resident in HBM
    def step(ev0=None, ev1=None, ev2=None):
        if ev0 is not None:
            ev0.record()
        rc = g.split_prepare(form, w["ta"], w["tb"], m, n, k, prob.A.data_ptr(), w["lda"],
                             prob.B.data_ptr(), w["ldb"], param, ws.data_ptr(), need, stream)
        if ev1 is not None:
            ev1.record()
        rc |= g.split_run(form, m, n, k, w["alpha"], w["beta"], prob.C.data_ptr(), w["ldc"],
                          param, ws.data_ptr(), need, stream)
        if ev2 is not None:
            ev2.record()
        return rc

    for _ in range(args.warmup):
        assert step() == g.OK
    torch.cuda.synchronize()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    sampler = ClockSampler(torch.cuda.current_device()) if rank == 0 else None
    if sampler:
        sampler.start()
        time.sleep(0.3)
    barrier(torch, world)
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    for s in range(args.steps):
        assert step(*evs[s]) == g.OK
    t1.record()
    torch.cuda.synchronize()
    barrier(torch, world)
    clocks = sampler.stop() if sampler else None
    total_ms = t0.elapsed_time(t1)
    gemm_ms = sum(e[1].elapsed_time(e[2]) for e in evs) / args.steps
    prep_ms = sum(e[0].elapsed_time(e[1]) for e in evs) / args.steps
    # each timed step alone (prepare + run, CUDA events on the launching stream)
    step_times = sorted(e[0].elapsed_time(e[2]) for e in evs)
    max_ms = allreduce_max(torch, world, total_ms)
    value = prob.flops * args.steps * world / (max_ms / 1e3) / 1e12
    assert g.device_error() == 0

    # ---- plain kernel throughput (same workload)
    for _ in range(2):
        plain_call(prob.C)
    torch.cuda.synchronize()
    reps = 3 if not (is_d and m >= 16384) else 1
    a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a0.record()
    for _ in range(reps):
        plain_call(prob.C)
    a1.record()
    torch.cuda.synchronize()
    plain_ms = a0.elapsed_time(a1) / reps
    plain_tflops = prob.flops / (plain_ms / 1e3) / 1e12

    # ---- end to end through the host-pointer C ABI (pinned host buffers)
    e2e = None
    if args.no_e2e:
        e2e = {"value": None, "skipped": "--no-e2e"}
    try:
        if args.no_e2e:
            raise StopIteration
        hA = torch.empty(prob.A.shape, dtype=prob.A.dtype, pin_memory=True)
        hB = torch.empty(prob.B.shape, dtype=prob.B.dtype, pin_memory=True)
        hC = torch.empty(prob.C0.shape, dtype=prob.C0.dtype, pin_memory=True)
        hA.copy_(prob.A)
        hB.copy_(prob.B)
        hC.copy_(prob.C0)
        hC0 = hC.clone()   # the workload's C, restored before every step (C is in / out)
        ah, bh, ch = hA.numpy(), hB.numpy(), hC.numpy()
        c0h = hC0.numpy()
        # C is restored by one numpy copy outside the timed call: a torch copy
        # left its thread pool spinning on every core into the timed call
        for _ in range(2):
            np.copyto(ch, c0h)
            assert g.host_split_gemm(form, w["ta"], w["tb"], m, n, k, w["alpha"], ah, w["lda"],
                                     bh, w["ldb"], w["beta"], ch, w["ldc"], param) == g.OK
        # 3 calls per timed step, 10 to 30: one host-side hiccup (a 10-15 ms
        # call, seen about once in 40-60 calls on some boxes and never in 300
        # calls of a loop alone) weighs a third as much in the mean
        steps_e2e = max(10, min(3 * args.steps, 30))
        step_ms = []
        for _ in range(steps_e2e):
            np.copyto(ch, c0h)   # outside the timed call
            t = time.perf_counter()
            assert g.host_split_gemm(form, w["ta"], w["tb"], m, n, k, w["alpha"], ah, w["lda"],
                                     bh, w["ldb"], w["beta"], ch, w["ldc"], param) == g.OK
            step_ms.append((time.perf_counter() - t) * 1e3)
        dt = sum(step_ms) / steps_e2e / 1e3
        esz = 8 if is_d else 4
        # the pipelined host path (page-locked buffers, k >= 1024, m or n >= 4096;
        # 2048 for the FP64 CRT form)
        # leaves C in host memory when beta = 0 and every entry of C is finite and
        # non-negative (0 * C = +0): then only A and B cross the link
        c_moved = not (w["beta"] == 0.0 and k >= 1024 and
                       max(m, n) >= (2048 if form == "crt" else 4096) and
                       bool(torch.isfinite(hC0).all()) and not bool(torch.signbit(hC0).any()))
        h2d = (prob.ar * prob.ac + prob.br * prob.bc + (m * n if c_moved else 0)) * esz
        e2e = {"value": round(prob.flops / dt / 1e12, 3), "unit": "TFLOP/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": m * n * esz,
               "ms_per_step": round(dt * 1e3, 3),
               "step_ms": {"min": round(min(step_ms), 3), "median": round(sorted(step_ms)[len(step_ms) // 2], 3),
                           "max": round(max(step_ms), 3)},
               "api": "gb300_host_%s" %
               {"bf16x": "sgemm_bf16x", "ozaki": "dgemm_ozaki", "crt": "dgemm_ozaki2"}[form],
               "transfer": transfer_note(form)}
    except StopIteration:
        pass
    except Exception as ex:  # noqa: BLE001
        e2e = {"value": None, "error": repr(ex)}

    # ---- roofline of the dominant kernel (the tcgen05 GEMM of the split form)
    pk = peaks()
    eff = tuned["products"] if (form == "bf16x" and param == 0 and tuned) else param
    products = {"bf16x": 3 if eff == g.FP16X3 else eff,
                "ozaki": (param * (param + 1)) // 2, "crt": param}[form]
    pipe_flops = products * prob.flops
    achieved = pipe_flops / (gemm_ms / 1e3) / 1e12
    roof = {"bound": "tensor", "achieved": round(achieved, 2), "peak": pk["bf16_tflops"],
            "unit": "TFLOP/s", "frac": round(achieved / pk["bf16_tflops"], 4),
            "traffic": traffic_from_profile(args.workload, form_name),
            "kernel": {"bf16x": "bf16x_gemm_kernel", "ozaki": "ozaki_gemm_kernel",
                       "crt": "ozaki_gemm_kernel (CRT mode) + crt_reconstruct_kernel"}[form],
            "kernel_ms": round(gemm_ms, 4), "prepare_ms": round(prep_ms, 4),
            "peak_source": "%s bf16 burst (MEASURED_PEAKS.json)" % pk["source"],
            "algorithmic_flops_per_launch": pipe_flops}
    # the operands' and C's own bytes (A and B read once, C read and written)
    # over the same GEMM time: the HBM side of the roofline (skinny shapes)
    esz = 8 if is_d else 4
    io_bytes = esz * (m * k + k * n + 2 * m * n)
    roof["hbm"] = {"achieved": round(io_bytes / (gemm_ms / 1e3) / 1e9, 1), "unit": "GB/s",
                   "peak": pk["hbm_gbs"], "frac": round(io_bytes / (gemm_ms / 1e3) / 1e9 /
                                                        pk["hbm_gbs"], 4),
                   "algorithmic_bytes": io_bytes}
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "TFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(max_ms / args.steps, 4), "higher_is_better": True,
        "step_ms": {"best": round(step_times[0], 4),
                    "median": round(statistics.median(step_times), 4),
                    "samples": len(step_times), "rank": rank},
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if is_d else "f32",
        "data": "synthetic (seeded uniform[-1,1), generated on the device)",
        "config": workload_config(args.workload, w, world),
        "form": {"name": form_name, "autotuned": tuned,
                 "exponent_spread": exponent_spread(prob)},
        "e2e": e2e,
        "roofline": roof,
        "plain": {"kernel": "dgemm_plain (DMMA)" if is_d else "sgemm_plain (FFMA)",
                  "value": round(plain_tflops, 3), "unit": "TFLOP/s",
                  "ms": round(plain_ms, 3), "split_speedup": round(value / world / plain_tflops, 3)},
        "accuracy": {"samples": int(len(truth)), "truth": "exact sampled dot products",
                     "plain_max_rel": plain_err[0], "plain_fro_rel": plain_err[1],
                     "split": {p: {"max_rel": e[0], "fro_rel": e[1]} for p, e in errs.items()},
                     "chosen": form_name},
        "clocks": clocks,
        # per step: the split (both operands in one launch) and the GEMM; the
        # Ozaki form adds one max |.| launch (both operands, exponents by its
        # last CTA), the CRT form also the reconstruction; the scaled FP16
        # form's prepare as fp16x3_prepare_launches counts it
        "gpu_launches": args.steps * (
            1 + fp16x3_prepare_launches(w["ta"], w["tb"], k)
            if form == "bf16x" and eff == g.FP16X3
            else {"bf16x": 2, "ozaki": 3, "crt": 4}[form]),
    }
    if rank == 0:
        line["cpu_baseline"] = (cpu_baseline(w) if not args.no_cpu
                                else {"value": None, "skipped": "--no-cpu"})
        print(json.dumps(line), flush=True)


def parse_form(name):
    """'crt_n15' -> ('crt', 15), 'ozaki_s8' -> ('ozaki', 8), 'bf16x6' -> ('bf16x', 6),
    'fp16x3' -> ('bf16x', FP16X3) (the scaled FP16 form shares the BF16xP entry points).
    A tuned name such as 'tuned:fp16x3_c8_t256_pair' (or without 'tuned:') pins
    the layout the autotuner chose: hi*hi chunk length (_cN), tile width (_tN)
    and cluster mode (_pair: pair MMAs, _cta: one CTA per tile) are set as the library's tuning knobs."""
    import gemm_avx2_gb300 as g

    name = name[len("tuned:"):] if name.startswith("tuned:") else name
    parts = name.split("_")
    if name.startswith(("crt_n", "ozaki_s")):  # crt_nN / ozaki_sS, options after
        base, opts = "_".join(parts[:2]), parts[2:]
    else:
        base, opts = parts[0], parts[1:]
    for o in opts:
        if o[:1] == "c" and o[1:].isdigit():
            g.tune_param(g.TUNE_BF16X_CHUNK, int(o[1:]))
        elif o[:1] == "t" and o[1:].isdigit():
            assert g.tune_param(g.TUNE_TILE_N, int(o[1:])) == g.OK
        elif o in ("pair", "cta"):
            g.tune_param(g.TUNE_PAIR_MMA, 1 if o == "pair" else 2)
        else:
            raise SystemExit("--form: unknown option %r in %r" % (o, name))
    if base == "fp16x3":
        return "bf16x", g.FP16X3
    for prefix, form in (("crt_n", "crt"), ("ozaki_s", "ozaki"), ("bf16x", "bf16x")):
        if base.startswith(prefix) and base[len(prefix):].isdigit():
            return form, int(base[len(prefix):])
    raise SystemExit("--form: expected crt_nN, ozaki_sS, bf16xP or fp16x3 (optionally with "
                     "_cN, _tN, _pair or _cta), got %r" % name)


# ----------------------------------------------------------------------------- complex workloads
def exact_samples_complex(A_rows, B_cols, alpha, beta, c0):
    """Correctly rounded alpha*dot + beta*c (real alpha, beta) of complex dots."""
    import numpy as np

    out = np.empty(A_rows.shape[0], np.complex128)
    for q in range(A_rows.shape[0]):
        ar, ai = A_rows[q].real.astype(np.float64), A_rows[q].imag.astype(np.float64)
        br, bi = B_cols[q].real.astype(np.float64), B_cols[q].imag.astype(np.float64)
        terms_r, terms_i = [], []
        for x, y, sgn, dst in ((ar, br, 1, terms_r), (ai, bi, -1, terms_r), (ar, bi, 1, terms_i),
                               (ai, br, 1, terms_i)):
            p, e = _two_prod(sgn * x, y)
            dst.extend(p.tolist())
            dst.extend(e.tolist())
        re, im = math.fsum(terms_r), math.fsum(terms_i)
        out[q] = complex(math.fsum([alpha * re, beta * float(c0[q].real)]),
                         math.fsum([alpha * im, beta * float(c0[q].imag)]))
    return out


def rel_err_c(got, truth):
    import numpy as np

    d = np.abs(np.asarray(got, np.complex128) - truth)
    mx = float(np.max(d / np.maximum(np.abs(truth), 1e-300)))
    fro = float(np.linalg.norm(d) / max(np.linalg.norm(truth), 1e-300))
    return mx, fro


def run_complex(args, torch, rank, world):
    """ZGEMM / CGEMM NN: split form (Ozaki / BF16xP on the embedded 2m x n x 2k
    real problem) at equal error to the plain 4M method; 8mnk flops per call."""
    import numpy as np

    import gemm_avx2_gb300 as g

    w = CWORKLOADS[args.workload]
    p, m, n, k = w["prec"], w["m"], w["n"], w["k"]
    dt = torch.complex128 if p == "z" else torch.complex64
    rdt = torch.float64 if p == "z" else torch.float32
    gen = torch.Generator(device="cuda")
    gen.manual_seed(int(w["seed"]))

    def cu(rows, cols):  # column-major rows x cols, stored as a (cols, rows) tensor
        x = torch.rand((cols, rows, 2), generator=gen, device="cuda", dtype=rdt) * 2 - 1
        return torch.view_as_complex(x.contiguous())

    A, B, C0 = cu(m, k), cu(k, n), cu(m, n)
    C = C0.clone()
    stream = torch.cuda.current_stream().cuda_stream
    flops = 8.0 * m * n * k

    def call(method, param, Cbuf, ws=None, wsb=0):
        return g.complex_device(p, w["ta"], w["tb"], m, n, k, w["alpha"], A.data_ptr(), m,
                                B.data_ptr(), k, w["beta"], Cbuf.data_ptr(), m, method=method,
                                param=param, workspace=ws, workspace_bytes=wsb, stream=stream)

    rng = np.random.default_rng(99)
    rows, cols = rng.integers(0, m, 512), rng.integers(0, n, 512)
    Ar = A[:, rows].T.cpu().numpy()
    Bc = B[cols, :].cpu().numpy()
    truth = exact_samples_complex(Ar, Bc, w["alpha"], w["beta"], C0[cols, rows].cpu().numpy())

    def measure(method, param, reps):
        C.copy_(C0)
        assert call(method, param, C) == g.OK
        torch.cuda.synchronize()
        err = rel_err_c(C[cols, rows].cpu().numpy(), truth)
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record()
        for _ in range(reps):
            call(method, param, C)
        a1.record()
        torch.cuda.synchronize()
        return err, a0.elapsed_time(a1) / reps

    plain_err, plain_ms = measure(g.CPLX_4M, 0, 1 if p == "z" else 3)
    m3_err, m3_ms = measure(g.CPLX_3M, 0, 1 if p == "z" else 3)
    # ZGEMM: the CRT form's moduli and the slice form's slice counts; CGEMM:
    # BF16xP products.  Per scheme the smallest candidate at equal error to 4M;
    # of two qualifying schemes the faster one.
    schemes = [(g.CPLX_CRT, list(range(11, 25))), (g.CPLX_SPLIT, list(range(6, 13)))] \
        if p == "z" else [(g.CPLX_SPLIT, [3, 6]), (g.CPLX_SPLIT, [g.FP16X3])]

    def cname(meth, prm):
        if p == "c" and prm == g.FP16X3:
            return "fp16x3"
        return ("crt_n%d" if meth == g.CPLX_CRT else "ozaki_s%d" if p == "z" else "bf16x%d") % prm

    errs, qualified = {}, []
    for meth, cands in schemes:
        for prm in cands:
            C.copy_(C0)
            if call(meth, prm, C) != g.OK:
                continue
            torch.cuda.synchronize()
            e = rel_err_c(C[cols, rows].cpu().numpy(), truth)
            errs[cname(meth, prm)] = e
            if e[0] <= plain_err[0] and e[1] <= plain_err[1]:
                qualified.append((meth, prm))
                break
    if not qualified:
        qualified.append((schemes[-1][0], schemes[-1][1][-1]))
    best = None
    forced = parse_form(args.form) if args.form else None
    if forced:
        meth = g.CPLX_CRT if forced[0] == "crt" else g.CPLX_SPLIT
        qualified = [(meth, forced[1])]
    for meth, prm in qualified:
        call(meth, prm, C)
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record()
        for _ in range(2):
            call(meth, prm, C)
        a1.record()
        torch.cuda.synchronize()
        if best is None or a0.elapsed_time(a1) < best[0]:
            best = (a0.elapsed_time(a1), meth, prm)
    method, param = best[1], best[2]
    need = g.complex_workspace_bytes(p, method, w["tb"], m, n, k, param)
    ws = torch.empty(need, dtype=torch.uint8, device="cuda")

    for _ in range(args.warmup):
        assert call(method, param, C, ws.data_ptr(), need) == g.OK
    torch.cuda.synchronize()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(args.steps)]
    sampler = ClockSampler(torch.cuda.current_device()) if rank == 0 else None
    if sampler:
        sampler.start()
        time.sleep(0.3)
    barrier(torch, world)
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record()
    for s_ in range(args.steps):
        evs[s_][0].record()
        assert call(method, param, C, ws.data_ptr(), need) == g.OK
        evs[s_][1].record()
    t1.record()
    torch.cuda.synchronize()
    barrier(torch, world)
    clocks = sampler.stop() if sampler else None
    total_ms = t0.elapsed_time(t1)
    step_ms = sum(e[0].elapsed_time(e[1]) for e in evs) / args.steps
    max_ms = allreduce_max(torch, world, total_ms)
    value = flops * args.steps * world / (max_ms / 1e3) / 1e12
    assert g.device_error() == 0

    e2e = {"value": None, "skipped": "--no-e2e"}
    if not args.no_e2e:
        try:
            hA = torch.empty(A.shape, dtype=dt, pin_memory=True)
            hB = torch.empty(B.shape, dtype=dt, pin_memory=True)
            hC = torch.empty(C0.shape, dtype=dt, pin_memory=True)
            hA.copy_(A)
            hB.copy_(B)
            hC.copy_(C0)
            hC0 = hC.clone()   # the workload's C, restored before every step (C is in / out)
            ah, bh, ch = hA.numpy(), hB.numpy(), hC.numpy()
            c0h = hC0.numpy()
            for _ in range(2):
                np.copyto(ch, c0h)   # numpy: no torch thread pool left spinning
                assert g.host_complex(p, w["ta"], w["tb"], m, n, k, w["alpha"], ah, m, bh, k,
                                      w["beta"], ch, m, method=method, param=param) == g.OK
            steps_e2e = max(10, min(3 * args.steps, 30))
            dts = 0.0
            for _ in range(steps_e2e):
                np.copyto(ch, c0h)   # outside the timed call
                t = time.perf_counter()
                assert g.host_complex(p, w["ta"], w["tb"], m, n, k, w["alpha"], ah, m, bh, k,
                                      w["beta"], ch, m, method=method, param=param) == g.OK
                dts += time.perf_counter() - t
            dts /= steps_e2e
            esz = 16 if p == "z" else 8
            e2e = {"value": round(flops / dts / 1e12, 3), "unit": "TFLOP/s",
                   "h2d_bytes_per_step": (m * k + k * n + m * n) * esz,
                   "d2h_bytes_per_step": m * n * esz, "ms_per_step": round(dts * 1e3, 3),
                   "api": "gb300_host_%sgemm (%s)" % (
                       p, "GB300_CPLX_CRT" if method == g.CPLX_CRT else "GB300_CPLX_SPLIT"),
                   "transfer": "pinned host buffers read and written in place over the "
                               "coherent CPU-GPU link"}
        except Exception as ex:  # noqa: BLE001
            e2e = {"value": None, "error": repr(ex)}

    pk = peaks()
    products = (3 if param == g.FP16X3 else param) if (p == "c" or method == g.CPLX_CRT) \
        else (param * (param + 1)) // 2
    pipe_flops = products * flops
    achieved = pipe_flops / (step_ms / 1e3) / 1e12
    form_name = cname(method, param)
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "TFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(max_ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128" if p == "z" else "c64",
        "data": "synthetic (seeded uniform[-1,1) real and imaginary parts, on the device)",
        "config": workload_config(args.workload, w, world),
        "form": {"name": form_name},
        "e2e": e2e,
        "roofline": {"bound": "tensor", "achieved": round(achieved, 2),
                     "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                     "frac": round(achieved / pk["bf16_tflops"], 4), "traffic": None,
                     "kernel": ("ozaki_gemm_kernel (CRT mode)" if method == g.CPLX_CRT else
                                "ozaki_gemm_kernel" if p == "z" else "bf16x_gemm_kernel"),
                     "kernel_ms": round(step_ms, 4),
                     "timing": "whole step (operand embedding, split kernels and the tcgen05 "
                               "GEMM): a lower bound on the GEMM kernel's rate",
                     "peak_source": "%s bf16 burst (MEASURED_PEAKS.json)" % pk["source"],
                     "algorithmic_flops_per_launch": pipe_flops},
        "plain": {"kernel": "4M on the plain %s kernel" % ("DMMA" if p == "z" else "FFMA"),
                  "value": round(flops / (plain_ms / 1e3) / 1e12, 3), "unit": "TFLOP/s",
                  "ms": round(plain_ms, 3),
                  "split_speedup": round(value / world / (flops / (plain_ms / 1e3) / 1e12), 3)},
        "method_3m": {"value": round(flops / (m3_ms / 1e3) / 1e12, 3), "unit": "TFLOP/s (8mnk)",
                      "ms": round(m3_ms, 3), "max_rel": m3_err[0], "fro_rel": m3_err[1]},
        "accuracy": {"samples": int(len(truth)), "truth": "exact sampled complex dot products",
                     "plain_max_rel": plain_err[0], "plain_fro_rel": plain_err[1],
                     "split": {q: {"max_rel": e[0], "fro_rel": e[1]} for q, e in errs.items()},
                     "chosen": form_name},
        "clocks": clocks,
        # per step: the operand embedding, then the form's own kernels (the
        # embedded real problem is NN with 2k)
        "gpu_launches": args.steps * (1 + (4 if method == g.CPLX_CRT else 3 if p == "z" else
                                           1 + fp16x3_prepare_launches("N", "N", 2 * k)
                                           if param == g.FP16X3 else 2)),
    }
    if rank == 0:
        line["cpu_baseline"] = (cpu_baseline(w, cplx=True) if not args.no_cpu
                                else {"value": None, "skipped": "--no-cpu"})
        print(json.dumps(line), flush=True)


def exponent_spread(prob):
    """max - min of the binary exponent over the nonzero entries of op(A) and op(B)."""
    import torch

    out = {}
    for name, X, rows in (("A", prob.A, prob.ar), ("B", prob.B, prob.br)):
        x = X[:, :rows].abs()
        x = x[x > 0]
        e = torch.frexp(x.to(torch.float64))[1]
        out[name] = int(e.max().item() - e.min().item()) if e.numel() else 0
    return out


# ----------------------------------------------------------------------------- grouped workload
FP64_PEAK_TFLOPS = 1.05   # DFMA / DMMA m16n8k8, measured on GB300 by microbenchmark
FP32_PEAK_TFLOPS = 73.0   # FFMA, measured on GB300 by microbenchmark


# name -> (problems, largest dimension); grouped_256 is a reduced batch for
# multi-pass profiler captures (about 1 GB of workspaces against 13 GB)
GROUPED_WORKLOADS = {"grouped_1024": (1024, 2048), "grouped_256": (256, 1024)}


def run_grouped(args, torch, rank, world):
    """1024 independent GEMMs: m, n, k = round(exp(U[ln 16, ln 2048])), transa/transb
    N or T with p = 0.5, 60% FP64 / 40% FP32, alpha ~ U[0.5, 2], beta in {0, 1},
    entries U[-1,1), ld = rows of the stored matrix (seed 4); grouped_256: 256
    problems with dimensions up to 1024.  A step replays a
    captured CUDA graph: the split forms (per-problem operand preparation, one
    grouped GEMM launch per precision, per-problem FP64 reconstruction) for the
    headline, the plain forms (one persistent launch) for the comparison."""
    import numpy as np

    import gemm_avx2_gb300 as g

    rng = np.random.default_rng(4)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(4)
    count, max_dim = GROUPED_WORKLOADS[args.workload]
    probs, bufs, flops = [], [], 0.0
    fl_d = fl_s = 0.0
    for i in range(count):
        m, n, k = (int(round(math.exp(x)))
                   for x in rng.uniform(math.log(16), math.log(max_dim), 3))
        ta = "N" if rng.random() < 0.5 else "T"
        tb = "N" if rng.random() < 0.5 else "T"
        prec = "d" if rng.random() < 0.6 else "s"
        alpha = float(rng.uniform(0.5, 2.0))
        beta = float(rng.choice([0.0, 1.0]))
        dt = torch.float64 if prec == "d" else torch.float32
        ar, ac = (m, k) if ta == "N" else (k, m)
        br, bc = (k, n) if tb == "N" else (n, k)
        A = torch.rand((ac, ar), generator=gen, device="cuda", dtype=dt) * 2 - 1
        B = torch.rand((bc, br), generator=gen, device="cuda", dtype=dt) * 2 - 1
        C0 = torch.rand((n, m), generator=gen, device="cuda", dtype=dt) * 2 - 1
        C = C0.clone()
        bufs.append((A, B, C0, C))
        probs.append(dict(precision=prec, transa=ta, transb=tb, m=m, n=n, k=k, alpha=alpha,
                          beta=beta, A=A.data_ptr(), lda=ar, B=B.data_ptr(), ldb=br,
                          C=C.data_ptr(), ldc=m))
        f = 2.0 * m * n * k
        flops += f
        if prec == "d":
            fl_d += f
        else:
            fl_s += f
    stream = torch.cuda.current_stream().cuda_stream

    def reset():
        for (A, B, C0, C) in bufs:
            C.copy_(C0)

    def timed(graph, steps, warmup):
        for _ in range(warmup):
            reset()
            assert graph.launch(stream) == g.OK
        torch.cuda.synchronize()
        total = 0.0
        for _ in range(steps):
            reset()   # restore C outside the timed launch
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            assert graph.launch(stream) == g.OK
            e1.record()
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1)
        return total / steps

    gp = g.GroupedGraph(probs, form=0)
    gs = g.GroupedGraph(probs, form=1)
    kernels_split, gemm_launches_split = gs.stats()
    # accuracy of both forms on sampled entries of 48 problems (exact sampled dots)
    def sampled_errors(graph):
        reset()
        assert graph.launch(stream) == g.OK
        torch.cuda.synchronize()
        worst = [0.0, 0.0]
        for i in range(0, count, count // 48):
            p = probs[i]
            A, B, C0, C = bufs[i]
            r = rng.integers(0, p["m"], 8)
            c = rng.integers(0, p["n"], 8)
            Ah = A.cpu().numpy()
            Bh = B.cpu().numpy()
            Arows = Ah[:, r].T if p["transa"] == "N" else Ah[r, :]
            Bcols = Bh[c, :] if p["transb"] == "N" else Bh[:, c].T
            truth = exact_samples(Arows, Bcols, p["alpha"], p["beta"], C0[c, r].cpu().numpy())
            e = rel_err(C[c, r].cpu().numpy(), truth)
            tag = 0 if p["precision"] == "d" else 1
            worst[tag] = max(worst[tag], e[0])
        return {"fp64_max_rel": worst[0], "fp32_max_rel": worst[1]}

    err_plain = sampled_errors(gp)
    err_split = sampled_errors(gs)
    sampler = ClockSampler(torch.cuda.current_device()) if rank == 0 else None
    if sampler:
        sampler.start()
        time.sleep(0.3)
    barrier(torch, world)
    ms_split = timed(gs, args.steps, args.warmup)
    ms_plain = timed(gp, max(3, args.steps // 2), args.warmup)
    # per form: each precision's problems alone as a split-form graph
    # (tensor pipe work: 16 residue GEMMs per FP64 product, 6 BF16 products per FP32 one)
    per_form = {}
    pk = peaks()
    for tag, prec, fl, P in (("fp64_crt16", "d", fl_d, 16), ("fp32_bf16x6", "s", fl_s, 6)):
        sub = [p for p in probs if p["precision"] == prec]
        if not sub or fl == 0.0:
            continue
        gf = g.GroupedGraph(sub, form=1)
        ms = timed(gf, max(3, args.steps // 2), args.warmup)
        gf.destroy()
        per_form[tag] = {"problems": len(sub), "ms": round(ms, 4),
                         "tflops": round(fl / (ms / 1e3) / 1e12, 3),
                         "tensor_pipe_frac": round(P * fl / (ms / 1e3) / 1e12 / pk["bf16_tflops"], 4),
                         "peak": pk["bf16_tflops"], "peak_source": "%s bf16 burst" % pk["source"]}
    barrier(torch, world)
    clocks = sampler.stop() if sampler else None
    max_ms = allreduce_max(torch, world, ms_split)
    value = flops * world / (max_ms / 1e3) / 1e12
    plain_tflops = flops / (ms_plain / 1e3) / 1e12
    # roofline of the plain persistent kernel: FP64 tiles on the FP64 pipe, FP32 on FFMA
    t_lb = fl_d / (FP64_PEAK_TFLOPS * 1e12) + fl_s / (FP32_PEAK_TFLOPS * 1e12)
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "TFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(max_ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic (seeded uniform[-1,1), generated on the device)",
        "config": {"workload": args.workload, "problems": count, "max_dim": max_dim,
                   "fp64_share_of_flops":
                   round(fl_d / flops, 4), "total_gflop": round(flops / 1e9, 3),
                   "form": "split (FP32: bf16x6, FP64: CRT with 16 moduli), CUDA graph: "
                           "operand preparation in branches, one grouped GEMM launch per "
                           "precision, FP64 reconstruction in branches",
                   "l2": "%d MB of operands > %d MB" % (
                       sum(sum(t.numel() * t.element_size() for t in b[:3]) for b in bufs) // 2**20,
                       L2_BYTES // 2**20)},
        "plain": {"kernel": "grouped_plain_kernel (one persistent launch, CUDA graph)",
                  "value": round(plain_tflops, 3), "unit": "TFLOP/s", "ms": round(ms_plain, 3),
                  "split_speedup": round(value / world / plain_tflops, 3)},
        "roofline": {"bound": "fp64+fp32 pipes (plain grouped kernel)",
                     "achieved": round(plain_tflops, 3), "peak": round(flops / t_lb / 1e12, 3),
                     "unit": "TFLOP/s", "frac": round(t_lb / (ms_plain / 1e3), 4),
                     "traffic": None,
                     "peak_source": "FP64 1.05 and FP32 73 TFLOP/s measured by microbenchmark"},
        "per_form": per_form,
        "accuracy": {"plain": err_plain, "split": err_split, "samples": "8 entries x 48 problems"},
        "clocks": clocks,
        "gpu_launches": args.steps * kernels_split,
        "gemm_launches_per_step": gemm_launches_split,
        "e2e": {"value": None, "skipped": "device-pointer grouped API"},
    }
    gp.destroy()
    gs.destroy()
    if rank == 0:
        line["cpu_baseline"] = {"value": None, "skipped": "grouped workload"}
        print(json.dumps(line), flush=True)


def run_trsm(args, torch, rank, world):
    """TRSM (or TRMM) on the GEMM kernels: the diagonal blocks solved (or
    multiplied) by diag_left_kernel, the rest of B updated by GEMMs (plain
    form, or the split forms: Ozaki slices or the CRT form for FP64, 6xBF16 for
    FP32).  A is lower triangular with a raised diagonal (well conditioned); the
    accuracy is the sampled backward residual ||op(A) x - alpha b|| / (||A||
    ||x||) of the solve, or the relative error ||x - alpha op(A) b|| / (||A||
    ||b||) of the product, over 64 columns."""
    import numpy as np

    import gemm_avx2_gb300 as g

    w = TRSM_WORKLOADS[args.workload]
    p, m, n = w["prec"], w["m"], w["n"]
    trmm = w.get("routine") == "trmm"
    routine = g.trmm if trmm else g.trsm
    dt = torch.float64 if p == "d" else torch.float32
    gen = torch.Generator(device="cuda")
    gen.manual_seed(w["seed"])
    # column-major m x m stored as a (cols, rows) tensor: its upper triangle is
    # A's lower triangle
    A = (torch.rand((m, m), generator=gen, device="cuda", dtype=dt) * 2 - 1).triu()
    d = A.diagonal()
    d.add_(float(m) ** 0.5 * torch.where(d < 0, -1.0, 1.0).to(dt))
    B0 = torch.rand((n, m), generator=gen, device="cuda", dtype=dt) * 2 - 1
    B = B0.clone()
    stream = torch.cuda.current_stream().cuda_stream
    flops = float(m) * m * n

    def call(form):
        return routine(p, "L", "L", "N", "N", m, n, w["alpha"], A.data_ptr(), m, B.data_ptr(), m,
                      form=form, stream=stream)

    def timed(form, steps, warmup):
        for _ in range(warmup):
            B.copy_(B0)
            assert call(form) == g.OK
        total = 0.0
        for _ in range(steps):
            B.copy_(B0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            assert call(form) == g.OK
            e1.record()
            torch.cuda.synchronize()
            total += e0.elapsed_time(e1)
        return total / steps

    def residual(form):
        B.copy_(B0)
        assert call(form) == g.OK
        torch.cuda.synchronize()
        cols = np.random.default_rng(5).choice(n, 64, replace=False)
        Al = A.double().cpu().numpy().T          # A (lower triangular), row-major
        idx = torch.as_tensor(cols, device="cuda")
        X = B.index_select(0, idx).double().cpu().numpy().T          # m x 64
        Bc = B0.index_select(0, idx).double().cpu().numpy().T
        if trmm:
            R = X - w["alpha"] * (Al @ Bc)
            return float(np.linalg.norm(R) / (np.linalg.norm(Al) * np.linalg.norm(Bc)))
        R = Al @ X - w["alpha"] * Bc
        return float(np.linalg.norm(R) / (np.linalg.norm(Al) * np.linalg.norm(X)))

    # FP64 updates on the Ozaki slices (form 1) and on the CRT form (form 2),
    # the faster reported; FP32 on 6xBF16
    split_forms = [1, 2] if p == "d" else [1]
    form_names = {1: "Ozaki slices" if p == "d" else "6xBF16", 2: "CRT"}
    # --form plain | split | crt: that form alone (profiling runs)
    only = {"plain": 0, "split": 1, "crt": 2}.get(args.form) if args.form else None
    if args.form and only is None:
        raise SystemExit("--form for TRSM workloads: plain, split or crt")
    if only is not None:
        split_forms = [only]
        form_names[0] = "plain"
    res = {} if only is not None else {"plain": residual(0)}
    for f in split_forms:
        res[{0: "plain", 1: "split", 2: "crt"}[f]] = residual(f)
    sampler = ClockSampler(torch.cuda.current_device()) if rank == 0 else None
    if sampler:
        sampler.start()
        time.sleep(0.3)
    barrier(torch, world)
    ms_by_form = {f: timed(f, args.steps, args.warmup) for f in split_forms}
    best = min(ms_by_form, key=ms_by_form.get)
    ms_split = ms_by_form[best]
    ms_plain = timed(0, max(3, args.steps // 2), args.warmup) if only is None else None
    barrier(torch, world)
    clocks = sampler.stop() if sampler else None
    max_ms = allreduce_max(torch, world, ms_split)
    value = flops * world / (max_ms / 1e3) / 1e12
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "TFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(max_ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if p == "d" else "f32",
        "data": "synthetic (seeded uniform[-1,1), diagonal raised by sqrt(m), on the device)",
        "config": {"workload": args.workload, "routine": "trmm" if trmm else "trsm",
                   "side": "L", "uplo": "L", "transa": "N",
                   "diag": "N", "m": m, "n": n, "alpha": w["alpha"], "flops_per_call": "m^2 n",
                   "parallelism": "replicas" if world > 1 else "single"},
        "form": {"name": ("%s updates" if best == 0 else "split updates (%s)") % form_names[best],
                 "ms_by_form": {form_names[f]: round(v, 3) for f, v in ms_by_form.items()}},
        "plain": ({"value": round(flops / (ms_plain / 1e3) / 1e12, 3), "unit": "TFLOP/s",
                   "ms": round(ms_plain, 3)} if ms_plain is not None else None),
        "accuracy": {("relative_error" if trmm else "backward_residual"): res, "columns": 64},
        "clocks": clocks,
        "e2e": {"value": None, "skipped": "device-pointer TRSM API"},
    }
    if rank == 0:
        line["cpu_baseline"] = {"value": None, "skipped": "TRSM workload"}
        print(json.dumps(line), flush=True)


def fp16x3_prepare_launches(ta, tb, k):
    """Kernel launches of the scaled 3xFP16 prepare: k-contiguous operands (op(A)
    rows when A is transposed, op(B) columns when B is not) take the fused max
    pass and split when 1024 <= k and k rounded up to 64 is at most 16384; the
    others a max pass and a tile split.  Each kind is one launch for both
    operands."""
    fusable = k >= 1024 and (k + 63) // 64 * 64 <= 16384
    fa, fb = fusable and ta != "N", fusable and tb == "N"
    if fa and fb:
        return 1
    return 3 if (fa or fb) else 2


def transfer_note(form):
    """How the host-pointer call moves the step's bytes over the CPU-GPU link."""
    if form == "bf16x":
        return ("pinned host buffers; A, B and C are copied to HBM in row / column parts by the "
                "copy engines while earlier parts are split and their C blocks multiplied, and "
                "each C block is copied back as it finishes; with beta = 0 and C finite and "
                "non-negative (C = 0 here) C is zero-filled in HBM instead of copied (0 * C = +0); "
                "the workload's C is restored in host memory before every step, outside the "
                "timed call (bytes above cross the link once)")
    return ("pinned host buffers; A and B are copied to HBM, C is read and written in host memory "
            "by the epilogue or staged in HBM beside the prepare (bytes above cross the link once)")


def traffic_from_profile(workload, form_name):
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary
    (a tuned layout is looked up under its pinned name, without 'tuned:')."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        d = json.load(open(p))
        if form_name.startswith("tuned:"):
            form_name = form_name[len("tuned:"):]
        v = d.get("%s:%s" % (workload, form_name))
        if v is not None:
            return v
    return None


# ----------------------------------------------------------------------------- CPU side
# One CPU step computes the whole workload when its work is at most SGEMM
# 8192^3's (about 12 s with the port on 16 Grace cores), else the leading
# block of columns of C with that much work.  The block is fixed by the
# workload alone, so the CPU-baseline leg of the GPU arm and every step of the
# reference arm time the same computation.
CPU_STEP_FLOPS = 1.1e12


def cpu_columns(n, flops_per_column):
    if flops_per_column * n <= CPU_STEP_FLOPS:
        return n
    ns = int(CPU_STEP_FLOPS / flops_per_column)
    return max(16, ns - ns % 16)


class CpuWorkload:
    """The workload's CPU computation (the reference library where it runs on
    this host, else the oracle's restatement of its algorithm, on all host
    cores): `warmup()` runs a few columns (thread team start; it reads all of
    A, whose pages the generator already touched), `step()` times the step's
    columns of C and returns the seconds."""

    def __init__(self, w, cplx=False):
        import numpy as np

        import oracle

        if not os.path.exists(os.path.join(ROOT, "oracle", "liborc.so")):
            oracle.build()
        self.cores = os.cpu_count() or 1
        oracle.set_threads(self.cores)
        m, n, k = w["m"], w["n"], w["k"]
        self.w, self.cplx = w, cplx
        self.ns = cpu_columns(n, (8.0 if cplx else 2.0) * m * k)
        self.flops = (8.0 if cplx else 2.0) * m * self.ns * k
        if cplx:
            dt = np.complex128 if w["prec"] == "z" else np.complex64
            self.A = oracle.cuniform((m, k), dt, w["seed"], 0)
            self.B = oracle.cuniform((k, self.ns), dt, w["seed"], 1)
            self.C = oracle.cuniform((m, self.ns), dt, w["seed"], 2)
            ref = oracle.RefCplx() if oracle.RefCplx.available() else None
            self.kind = "reference" if ref else "port"

            def f(ns):  # NN: packs A once, then B's columns over the OpenMP team
                if ref:
                    ref.gemm_conj(0, 0, w["alpha"], self.A, self.B[:, :ns], self.C[:, :ns])
                else:
                    oracle.zgemm_port(0, 0, w["alpha"], self.A, self.B[:, :ns], self.C[:, :ns])
            self.f = f
            self.sample = "%sgemm NN m=%d n=%d (of %d) k=%d" % (w["prec"], m, self.ns, n, k)
        else:
            dt = np.float64 if w["prec"] == "d" else np.float32
            ar, ac = (m, k) if w["ta"] == "N" else (k, m)
            br, bc = (k, self.ns) if w["tb"] == "N" else (self.ns, k)
            phi = w.get("phi") or None  # exponent-spread inputs where the workload has them
            self.A = oracle.storage(ar, ac, w["lda"], dt, w["seed"], 0, phi)
            self.B = oracle.storage(br, bc, max(br, 1), dt, w["seed"], 1, phi)
            self.C = oracle.storage(m, self.ns, w["ldc"], dt, w["seed"], 2)
            ldb = max(br, 1)
            if oracle.RefLib.available():
                ref = oracle.RefLib()
                self.kind = "reference"
                g = ref.gemm
            else:
                self.kind = "port"
                g = lambda *a: oracle.refgemm(*a, self.cores)

            def f(ns):  # op(B)'s first ns columns: the leading columns (N) or rows (T) of B
                g(w["ta"], w["tb"], m, ns, k, w["alpha"], self.A, w["lda"], self.B, ldb,
                  w["beta"], self.C, w["ldc"])
            self.f = f
            self.sample = "%s%s m=%d n=%d (of %d) k=%d" % (w["ta"], w["tb"], m, self.ns, n, k)
        if self.ns == n:
            self.sample += ", the whole workload"
        else:
            self.sample += ", the first %d columns of C" % self.ns

    def warmup(self):
        self.f(min(self.ns, 16 * self.cores))

    def step(self):
        t = time.perf_counter()
        self.f(self.ns)
        return time.perf_counter() - t


def cpu_baseline(w, cplx=False):
    """One warm-up, then the step's computation timed once."""
    try:
        cw = CpuWorkload(w, cplx)
        cw.warmup()
        t = cw.step()
        return {"value": round(cw.flops / t / 1e12, 5), "unit": "TFLOP/s", "cores": cw.cores,
                "kind": cw.kind, "sample": cw.sample, "seconds": round(t, 2)}
    except Exception as ex:  # noqa: BLE001
        return {"value": None, "error": repr(ex)}


def run_reference(args, rank, world):
    if rank != 0:
        return
    if args.workload in GROUPED_WORKLOADS:
        print(json.dumps({"impl": "reference", "metric": METRIC,
                          "unavailable": "the reference has no grouped interface"}))
        return
    if args.workload in TRSM_WORKLOADS:
        print(json.dumps({"impl": "reference", "metric": METRIC,
                          "unavailable": "the reference's TRSM kernels are x86 AVX2 code "
                                         "without a driver; they serve as an oracle here"}))
        return
    cplx = args.workload in CWORKLOADS
    w = dict(CWORKLOADS[args.workload] if cplx else WORKLOADS[args.workload])
    if args.phi is not None and not cplx:
        w["phi"] = args.phi
    # every step is the same computation as the GPU arm's CPU-baseline leg:
    # the whole workload up to SGEMM 8192^3's work (else a fixed leading
    # column block); the warm-up steps start the thread team on a few columns
    cw = CpuWorkload(w, cplx)
    for _ in range(args.warmup):
        cw.warmup()
    times = [cw.step() for _ in range(args.steps)]
    tf = cw.flops * len(times) / sum(times) / 1e12
    line = {"metric": METRIC, "value": round(tf, 5), "unit": "TFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * sum(times) / len(times), 2),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"d": "f64", "s": "f32", "z": "c128", "c": "c64"}[w["prec"]],
            "data": "synthetic (the portable generator's seeded uniform[-1,1) inputs)",
            "config": workload_config(args.workload, w, world),
            "impl": "reference",
            "cpu_baseline": {"value": round(tf, 5), "unit": "TFLOP/s", "cores": cw.cores,
                             "kind": cw.kind, "sample": cw.sample},
            "e2e": {"value": round(tf, 5), "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- distributed
def barrier(torch, world):
    if world > 1:
        torch.distributed.barrier()


def allreduce_max(torch, world, v):
    if world <= 1:
        return v
    t = torch.tensor([v], dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + sorted(CWORKLOADS) +
                    sorted(TRSM_WORKLOADS) + sorted(GROUPED_WORKLOADS),
                    default="sgemm_tn_8192")
    ap.add_argument("--phi", type=float, default=None,
                    help="exponent spread of A and B: (u-0.5)*exp(phi*g) (DGEMM NT 16384 sweep)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-pointer leg (profiling runs)")
    ap.add_argument("--form", default=None,
                    help="use this split form instead of timing the qualifying ones "
                         "(crt_nN, ozaki_sS, bf16xP, fp16x3, optionally with _cN chunk, _tN "
                         "tile width, _pair / _cta cluster mode; TRSM workloads: plain, split or "
                         "crt; profiling runs)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus if args.gpus == 1 else 1)))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch

    torch.cuda.set_device(local)
    if world > 1:
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    if args.workload in GROUPED_WORKLOADS:
        run_grouped(args, torch, rank, world)
    elif args.workload in TRSM_WORKLOADS:
        run_trsm(args, torch, rank, world)
    elif args.workload in CWORKLOADS:
        run_complex(args, torch, rank, world)
    else:
        run_ours(args, torch, rank, world)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
