"""Grouped calls (ozgb_dgemm_grouped) on the GPU: every problem of one grouped
call gives the bits of the single-problem device path with the same slice count,
and adaptive problems get the slice count of the host precision knob.

Bar: bit-identical results; identical slice choices.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _stats(A, B):
    f = lambda x: ((x.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int32)
    return (f(A).max(axis=1), (A * A).sum(axis=1), f(B).max(axis=0), (B * B).sum(axis=0), (A * A).sum(axis=0),
            (B * B).sum(axis=1))


def _problems(oracle, rng, n, bounds):
    import torch
    dev = torch.device("cuda", 0)
    probs, host = [], []
    for i in range(n):
        M, N, K = (int(x) for x in np.exp(rng.uniform(np.log(16), np.log(700), 3)))
        phi = float(rng.choice([0.5, 1.0, 2.0]))
        A = oracle.gen_phi((M, K), 100 + i, phi)
        B = oracle.gen_phi((K, N), 200 + i, phi)
        dA, dB = torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)
        dC = torch.full((M, N), float("nan"), dtype=torch.float64, device=dev)
        bound = bounds[i % len(bounds)]
        probs.append({"M": M, "N": N, "K": K, "A": dA.data_ptr(), "lda": K, "B": dB.data_ptr(), "ldb": N,
                      "C": dC.data_ptr(), "ldc": N, "error_bound": bound})
        host.append((A, B, dA, dB, dC, bound))
    return probs, host


@pytest.mark.parametrize("launch", [1, 0])
@pytest.mark.parametrize("graph", [0, 1])
def test_grouped_matches_single_problem_path(gpu_handle, oracle, ozlib, graph, launch):
    """launch 1: one persistent GEMM launch per plan class over all of its
    problems' tiles; launch 0: one launch per problem."""
    import torch
    rng = np.random.default_rng(7)
    bounds = [1e-15, 0.0, 1e-11, 1e-8, 1e-13]
    probs, host = _problems(oracle, rng, 23, bounds)
    gpu_handle.set_slices(8)  # problems without a bound use s = 8
    gpu_handle.set_bins(8)
    gpu_handle.set_graph(graph)
    gpu_handle.set_grouped_launch(launch)
    stream = torch.cuda.current_stream().cuda_stream
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    for _ in range(2):  # a second identical call (graph replay when enabled)
        rc, used = gpu_handle.dgemm_grouped(probs, stream, with_bins=True)
        assert rc == 0, gpu_handle.last_error()
        assert gpu_handle.sync() == 0, gpu_handle.last_error()
    torch.cuda.synchronize()
    for (A, B, dA, dB, dC, bound), p, (s, J) in zip(host, probs, used):
        M, N, K = p["M"], p["N"], p["K"]
        if bound > 0:
            er, ssr, ec, ssc, ca, rb = _stats(A, B)
            assert (s, J) == ozlib.choose_schedule(er, ssr, ec, ssc, K, 7, bound, ca, rb, sms=sms)[:2]
        else:
            assert (s, J) == (8, 8)
        h = ozlib.Handle()
        h.set_slices(s)
        h.set_bins(J)
        want = torch.full((M, N), float("nan"), dtype=torch.float64, device=dA.device)
        assert h.dgemm_device(M, N, K, dA.data_ptr(), K, dB.data_ptr(), N, want.data_ptr(), N, stream) == 0
        assert h.sync() == 0
        h.close()
        torch.cuda.synchronize()
        got = dC.cpu().numpy()
        assert np.array_equal(got.view(np.uint64), want.cpu().numpy().view(np.uint64)), (M, N, K, s)


def test_grouped_accuracy_against_exact(gpu_handle, oracle):
    import torch
    rng = np.random.default_rng(11)
    probs, host = _problems(oracle, rng, 9, [1e-15])
    rc, used = gpu_handle.dgemm_grouped(probs, torch.cuda.current_stream().cuda_stream)
    assert rc == 0, gpu_handle.last_error()
    assert gpu_handle.sync() == 0
    for (A, B, dA, dB, dC, bound), p in zip(host, probs):
        M, N = p["M"], p["N"]
        rows = np.repeat(np.arange(M, dtype=np.int32), N)
        cols = np.tile(np.arange(N, dtype=np.int32), M)
        exact = oracle.exact_entries(A, B, rows, cols)[0].reshape(M, N)
        C = dC.cpu().numpy()
        assert np.linalg.norm(C - exact) / np.linalg.norm(exact) <= 1e-15


def test_grouped_rejects_bad_problem(gpu_handle):
    rc, _ = gpu_handle.dgemm_grouped([{"M": 0, "N": 4, "K": 4, "A": 16, "lda": 4, "B": 16, "ldb": 4, "C": 16,
                                       "ldc": 4}])
    assert rc == 1


def test_grouped_e4m3_slices_match_single_problem_path(gpu_handle, oracle, ozlib):
    """With 4-bit slices the grouped call's split jobs write e4m3 slices: every
    problem keeps the bits of the single-problem path (and of the oracle)."""
    import torch
    rng = np.random.default_rng(17)
    probs, host = _problems(oracle, rng, 9, [0.0])
    gpu_handle.set_bits(4)
    gpu_handle.set_slices(12)
    gpu_handle.set_bins(12)
    stream = torch.cuda.current_stream().cuda_stream
    rc, used = gpu_handle.dgemm_grouped(probs, stream)
    assert rc == 0, gpu_handle.last_error()
    assert gpu_handle.sync() == 0, gpu_handle.last_error()
    assert gpu_handle.config()["slice_format"] == 1
    torch.cuda.synchronize()
    for (A, B, dA, dB, dC, bound), p in zip(host, probs):
        ref = oracle.dgemm(A, B, 4, 12, 12, 0)
        assert np.array_equal(dC.cpu().numpy().view(np.uint64), ref.view(np.uint64)), (p["M"], p["N"], p["K"])


def _check_against_oracle(oracle, host, probs, s):
    for (A, B, dA, dB, dC, bound), p in zip(host, probs):
        ref = oracle.dgemm(A, B, 7, s, s, 0)
        got = dC.cpu().numpy()
        assert np.array_equal(got.view(np.uint64), ref.view(np.uint64)), (p["M"], p["N"], p["K"])


def test_grouped_graph_not_replayed_after_a_call_without_graphs(gpu_handle, oracle):
    """Calls without graphs rewrite the tables that a captured graph reads: a
    graph call, a call without graphs on other problems, then the first problems
    again with graphs must give the oracle's bits each time (the captured graph
    is not replayed over the rewritten tables)."""
    import torch
    stream = torch.cuda.current_stream().cuda_stream
    gpu_handle.set_slices(7)
    gpu_handle.set_bins(7)
    first, host1 = _problems(oracle, np.random.default_rng(31), 6, [0.0])
    second, host2 = _problems(oracle, np.random.default_rng(32), 9, [0.0])
    for graph, probs, host in ((1, first, host1), (0, second, host2), (1, first, host1)):
        for _, _, _, _, dC, _ in host:
            dC.fill_(float("nan"))
        gpu_handle.set_graph(graph)
        rc, _ = gpu_handle.dgemm_grouped(probs, stream)
        assert rc == 0, gpu_handle.last_error()
        assert gpu_handle.sync() == 0, gpu_handle.last_error()
        torch.cuda.synchronize()
        _check_against_oracle(oracle, host, probs, 7)


def test_grouped_many_problems_one_launch_per_class(gpu_handle, oracle, ozlib):
    """120 problems of 1 to 300 rows and columns, K up to 600, s = 6: a few
    grouped launches cover every tile once (host walk of the launches), and every
    result has the oracle's bits."""
    import torch
    rng = np.random.default_rng(41)
    dev = torch.device("cuda", 0)
    probs, host, sizes = [], [], []
    for i in range(120):
        M, N = (int(x) for x in rng.integers(1, 301, 2))
        K = int(rng.integers(1, 601))
        A = oracle.gen_phi((M, K), 500 + i, 1.0)
        B = oracle.gen_phi((K, N), 700 + i, 1.0)
        dA, dB = torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)
        dC = torch.full((M, N), float("nan"), dtype=torch.float64, device=dev)
        probs.append({"M": M, "N": N, "K": K, "A": dA.data_ptr(), "lda": K, "B": dB.data_ptr(), "ldb": N,
                      "C": dC.data_ptr(), "ldc": N})
        host.append((A, B, dA, dB, dC, 0.0))
        sizes.append((M, N, K))
    rc, n_launch, units = ozlib.grouped_layout_check(sizes, 6, 6)
    assert rc == 0 and 1 <= n_launch <= 12
    gpu_handle.set_slices(6)
    gpu_handle.set_bins(6)
    before = gpu_handle.launch_count()
    rc, _ = gpu_handle.dgemm_grouped(probs, torch.cuda.current_stream().cuda_stream)
    assert rc == 0, gpu_handle.last_error()
    assert gpu_handle.sync() == 0, gpu_handle.last_error()
    assert gpu_handle.launch_count() - before == 1 + 1 + n_launch  # statistics, splits, GEMMs
    torch.cuda.synchronize()
    _check_against_oracle(oracle, host, probs, 6)
