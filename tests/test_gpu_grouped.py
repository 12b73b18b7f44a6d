"""Grouped GEMMs on the GPU through the C ABI: one persistent launch over a
mixed batch (FP64/FP32, N/T, ragged and tiny sizes, odd and aligned leading
dimensions, alpha == 0, k == 0), CUDA-graph replay, and the split-form graph.
Each result is checked like a single call: against the bit-exact oracle
restatement of the reference, with the summation-order bound."""
import numpy as np
import pytest

import gemm_avx2_gb300 as g
from gpu_util import from_dev, sync, to_dev
from util import U32, U64, check_close, gemm_bound

pytestmark = pytest.mark.gpu


def make_batch(orc, count, seed, max_dim=300):
    rng = np.random.default_rng(seed)
    probs, host, dev = [], [], []
    for i in range(count):
        prec = "d" if rng.random() < 0.6 else "s"
        dt = np.float64 if prec == "d" else np.float32
        m, n, k = (int(x) for x in np.round(np.exp(rng.uniform(0, np.log(max_dim), 3))))
        if i == 3:
            k = 0
        ta, tb = ("N", "T")[rng.integers(2)], ("N", "T")[rng.integers(2)]
        alpha = 0.0 if i == 5 else float(rng.uniform(0.5, 2))
        beta = float(rng.choice([0.0, 1.0, 0.5]))
        ar, ac = (m, k) if ta == "N" else (k, m)
        br, bc = (k, n) if tb == "N" else (n, k)
        pad = int(rng.integers(0, 3)) if i % 2 else 0   # odd pads -> cp.async path
        lda, ldb, ldc = max(ar, 1) + pad, max(br, 1) + pad, max(m, 1) + pad
        A = orc.storage(ar, ac, lda, dt, seed * 1000 + i, 0)
        B = orc.storage(br, bc, ldb, dt, seed * 1000 + i, 1)
        C = orc.storage(m, n, ldc, dt, seed * 1000 + i, 2)
        dA, dB, dC = to_dev(A), to_dev(B), to_dev(C)
        probs.append(dict(precision=prec, transa=ta, transb=tb, m=m, n=n, k=k, alpha=alpha,
                          beta=beta, A=dA.data_ptr(), lda=lda, B=dB.data_ptr(), ldb=ldb,
                          C=dC.data_ptr(), ldc=ldc))
        host.append((A, B, C))
        dev.append((dA, dB, dC))
    return probs, host, dev


def check_batch(orc, probs, host, dev, C_inputs=None):
    for p, (A, B, C), (dA, dB, dC) in zip(probs, host, dev):
        C0 = C if C_inputs is None else C_inputs
        want = C0.copy(order="F")
        orc.refgemm(p["transa"], p["transb"], p["m"], p["n"], p["k"], p["alpha"], A, p["lda"], B,
                    p["ldb"], p["beta"], want, p["ldc"], 2)
        got = from_dev(dC, C0.shape[0])
        m, n = p["m"], p["n"]
        u = U64 if p["precision"] == "d" else U32
        check_close(got[:m, :n], want[:m, :n],
                    gemm_bound(A, B, C0, p["transa"], p["transb"], m, n, p["k"], p["alpha"],
                               p["beta"], u))
        assert np.array_equal(got[m:], C0[m:])


def test_grouped_one_launch_matches_oracle(orc):
    probs, host, dev = make_batch(orc, 48, 1)
    assert g.gemm_grouped(probs) == g.OK
    sync()
    check_batch(orc, probs, host, dev)
    assert g.device_error() == 0


def test_grouped_caller_workspace(orc):
    probs, host, dev = make_batch(orc, 9, 2, max_dim=200)
    import torch
    nb = g.grouped_workspace_bytes(len(probs))
    ws = torch.empty(nb, dtype=torch.uint8, device="cuda")
    assert g.gemm_grouped(probs, workspace=ws.data_ptr(), workspace_bytes=nb - 4096) == \
        g.ERR_WORKSPACE
    assert g.gemm_grouped(probs, workspace=ws.data_ptr(), workspace_bytes=nb) == g.OK
    sync()
    check_batch(orc, probs, host, dev)


def test_grouped_graph_replay(orc):
    """Capture once, replay twice; the second replay sees new A contents."""
    probs, host, dev = make_batch(orc, 24, 3)
    C_init = [h[2].copy(order="F") for h in host]
    graph = g.GroupedGraph(probs, form=0)
    assert graph.launch() == g.OK
    sync()
    check_batch(orc, probs, host, dev)
    # new operands in the same buffers; reset C; replay
    host2 = []
    for i, (p, (A, B, C), (dA, dB, dC)) in enumerate(zip(probs, host, dev)):
        A2 = (A * -0.5).astype(A.dtype, order="F")
        dA.copy_(to_dev(A2))
        dC.copy_(to_dev(C_init[i]))
        host2.append((A2, B, C_init[i]))
    assert graph.launch() == g.OK
    sync()
    check_batch(orc, probs, host2, dev)
    graph.destroy()
    assert g.device_error() == 0


def test_grouped_split_graph_branch_count_is_invisible(orc):
    """The same batch captured in 2 and in 64 branches gives identical results
    (each problem runs the same kernels; only their concurrency differs)."""
    probs, host, dev = make_batch(orc, 40, 5, max_dim=300)
    outs = []
    try:
        for nb in (2, 64):
            assert g.tune_param(g.TUNE_GRAPH_BRANCHES, nb) == g.OK
            for d, h in zip(dev, host):
                d[2].copy_(to_dev(h[2]))   # C back to its initial values
            graph = g.GroupedGraph(probs, form=1)
            assert graph.launch() == g.OK
            sync()
            outs.append([from_dev(d[2], h[2].shape[0]) for d, h in zip(dev, host)])
            graph.destroy()
    finally:
        g.tune_param(g.TUNE_GRAPH_BRANCHES, 0)
    for a, b in zip(*outs):
        assert np.array_equal(a, b)
    assert g.device_error() == 0


def test_grouped_split_graph(orc):
    """Split forms (6xBF16 for FP32, Ozaki for FP64) captured per problem."""
    probs, host, dev = make_batch(orc, 12, 4, max_dim=260)
    C_init = [h[2].copy(order="F") for h in host]
    graph = g.GroupedGraph(probs, form=1)
    assert graph.launch() == g.OK
    sync()
    for p, (A, B, C), (dA, dB, dC), C0 in zip(probs, host, dev, C_init):
        m, n = p["m"], p["n"]
        if m == 0 or n == 0:
            continue
        truth = orc.dot2gemm(p["transa"], p["transb"], m, n, p["k"], p["alpha"], A, p["lda"], B,
                             p["ldb"], p["beta"], C0, p["ldc"])
        got = from_dev(dC, C0.shape[0])[:m, :n].astype(np.float64)
        d = np.linalg.norm(got - truth) / max(np.linalg.norm(truth), 1e-300)
        assert d < (1e-13 if p["precision"] == "d" else 1e-6), (p, d)
    graph.destroy()
    assert g.device_error() == 0


def per_problem_split_calls(probs, dev, C_inputs):
    """Each problem's own split call (CRT form / 6xBF16) from C_inputs; the results."""
    for p, (dA, dB, dC), C0 in zip(probs, dev, C_inputs):
        dC.copy_(to_dev(C0))
        args = (p["transa"], p["transb"], p["m"], p["n"], p["k"], p["alpha"], dA.data_ptr(),
                p["lda"], dB.data_ptr(), p["ldb"], p["beta"], dC.data_ptr(), p["ldc"])
        rc = g.dgemm_ozaki2(*args) if p["precision"] == "d" else g.sgemm_bf16x(*args, products=6)
        assert rc == g.OK
    sync()
    return [from_dev(d[2], C0.shape[0]) for d, C0 in zip(dev, C_inputs)]


def test_grouped_split_graph_matches_per_problem_calls(orc):
    """The split-form graph runs the GEMMs of all FP64 problems in one grouped
    launch and those of all FP32 problems in another (128 x 128 tiles of many
    problems, each tile with its problem's tensor maps and parameters from a
    device table); every result is bit-identical to the problem's own
    gb300_dgemm_ozaki2 / gb300_sgemm_bf16x(products = 6) call, on the first
    replay and on a second one with new operand values.  Dimensions up to 700
    (several row and column tiles per problem), odd leading dimensions,
    alpha == 0 and k == 0 problems."""
    probs, host, dev = make_batch(orc, 40, 6, max_dim=700)
    C_init = [h[2].copy(order="F") for h in host]
    graph = g.GroupedGraph(probs, form=1)
    kernels, gemms = graph.stats()
    live = [p for p in probs if p["m"] and p["n"]]
    n_d = sum(1 for p in live if p["precision"] == "d" and p["k"] and p["alpha"] != 0)
    n_s = sum(1 for p in live if p["precision"] == "s" and p["k"] and p["alpha"] != 0)
    n_calls = sum(1 for p in live if not p["k"] or p["alpha"] == 0)
    assert gemms == (n_d > 0) + (n_s > 0) and gemms <= 2
    # per FP64 problem: exponents, residues, reconstruction; per FP32 problem: split
    assert gemms + 3 * n_d + n_s <= kernels <= gemms + 3 * n_d + n_s + n_calls
    for rnd in range(2):
        if rnd:   # new operand values (other magnitudes) in the same buffers, C reset
            for (A, B, C), (dA, dB, dC), C0 in zip(host, dev, C_init):
                dA.copy_(to_dev((A * -0.37).astype(A.dtype, order="F")))
                dC.copy_(to_dev(C0))
        assert graph.launch() == g.OK
        sync()
        grouped = [from_dev(d[2], h[2].shape[0]) for d, h in zip(dev, host)]
        single = per_problem_split_calls(probs, dev, C_init)
        for i in range(len(probs)):
            assert np.array_equal(grouped[i], single[i], equal_nan=True), \
                (rnd, i, probs[i]["precision"], probs[i]["m"], probs[i]["n"], probs[i]["k"])
    graph.destroy()
    assert g.device_error() == 0


def test_grouped_split_graph_long_k(orc):
    """FP64 problems with k > 1024 (the CRT epilogue's multi-chunk path) and
    FP32 ones with several chunk runs, one with an Inf and one with a NaN
    operand, in the grouped launches, against the per-problem calls bit for
    bit (NaN where they have NaN)."""
    rng = np.random.default_rng(8)
    probs, host, dev = [], [], []
    shapes = [("d", 300, 200, 1500), ("d", 129, 257, 2100), ("s", 260, 140, 1800),
              ("s", 90, 300, 1100), ("d", 40, 30, 1030), ("s", 128, 128, 64)]
    for i, (prec, m, n, k) in enumerate(shapes):
        dt = np.float64 if prec == "d" else np.float32
        A = orc.storage(m, k, m, dt, 800 + i, 0)
        B = orc.storage(n, k, n, dt, 800 + i, 1)
        if i == 0:
            A[3, 5] = np.inf     # a non-finite row of op(A): its row of C is NaN
        if i == 2:
            B[7, 2] = np.nan     # a non-finite column of op(B)
        C = orc.storage(m, n, m, dt, 800 + i, 2)
        dA, dB, dC = to_dev(A), to_dev(B), to_dev(C)
        probs.append(dict(precision=prec, transa="N", transb="T", m=m, n=n, k=k,
                          alpha=float(rng.uniform(0.5, 2)), beta=0.5, A=dA.data_ptr(), lda=m,
                          B=dB.data_ptr(), ldb=n, C=dC.data_ptr(), ldc=m))
        host.append((A, B, C))
        dev.append((dA, dB, dC))
    graph = g.GroupedGraph(probs, form=1)
    assert graph.stats()[1] == 2
    assert graph.launch() == g.OK
    sync()
    grouped = [from_dev(d[2], h[2].shape[0]) for d, h in zip(dev, host)]
    single = per_problem_split_calls(probs, dev, [h[2] for h in host])
    for i in range(len(probs)):
        assert np.array_equal(grouped[i], single[i], equal_nan=True), i
    assert np.isnan(grouped[0][3, :]).all() and np.isnan(grouped[2][:, 7]).all()
    graph.destroy()
    assert g.device_error() == 0
