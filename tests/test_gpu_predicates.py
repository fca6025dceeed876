"""Batched orient3d / insphere signs on the GPU against the reference's own signs
(tests/golden, made from the reference's predicates) and the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["orient3d", "insphere"])
@pytest.mark.parametrize("mode", ["compat", "exact"])
def test_stream_matches_reference_signs(cm, golden, kind, mode):
    g = golden("predicates")
    fn = cm.orient3d_stream if kind == "orient3d" else cm.insphere_stream
    m = cm.PRED_COMPAT if mode == "compat" else cm.PRED_EXACT
    got, st = fn(g[kind + "_soa"], m)
    assert np.array_equal(got, g[kind + "_" + mode])
    assert st["queries"] == g[kind + "_soa"].shape[1]


@pytest.mark.parametrize("kind", ["orient3d", "insphere"])
def test_stream_matches_oracle_large(cm, orc, kind):
    import oracle as O
    from cybermeshgenerator_gb300 import workloads as W
    S = W.predicate_stream(200_000, kind, degenerate=0.1, near=0.1, seed=31)
    fn = cm.orient3d_stream if kind == "orient3d" else cm.insphere_stream
    for mode in (cm.PRED_COMPAT, cm.PRED_EXACT):
        got, st = fn(S, mode)
        want = orc.stream(kind, S, O.COMPAT if mode == cm.PRED_COMPAT else O.EXACT)
        assert np.array_equal(got, want)
        # the FP32 filter certifies the generic queries; ties are resolved exactly,
        # the exactly degenerate ones by an FP64 evaluation in which nothing rounded
        assert st["fp64_queries"] < 0.5 * S.shape[1]
        assert st["exact_queries"] >= int(0.09 * S.shape[1])
        # every exactly degenerate query (10 %) is settled by the certificate; the
        # near ones whose rounded determinant is zero still need expansions
        assert st["exact_queries"] - st["expansion_queries"] >= int(0.09 * S.shape[1])


@pytest.mark.parametrize("kind", ["orient3d", "insphere"])
def test_stream_left_queries_beyond_compact_slots(cm, orc, kind):
    """The FP32 pass stores the coordinates of the queries it leaves at their list
    positions, up to a quarter of the stream (+256); the FP64 pass reads those and
    gathers the rest by index. With 60 % exactly degenerate and 20 % near queries both
    kinds of entries occur; signs equal the oracle's in both modes."""
    import oracle as O
    from cybermeshgenerator_gb300 import workloads as W
    n = 120_000
    S = W.predicate_stream(n, kind, degenerate=0.6, near=0.2, seed=34)
    fn = cm.orient3d_stream if kind == "orient3d" else cm.insphere_stream
    for mode in (cm.PRED_COMPAT, cm.PRED_EXACT):
        got, st = fn(S, mode)
        assert st["fp64_queries"] > n // 4 + 256
        want = orc.stream(kind, S, O.COMPAT if mode == cm.PRED_COMPAT else O.EXACT)
        assert np.array_equal(got, want)


@pytest.mark.parametrize("kind", ["orient3d", "insphere"])
def test_stream_wait_taken_as_run_out_reruns(cm, kind):
    """A wait of the TMA-staged FP32 pass taken as having run out (cmg_debug_fail_pred_wait,
    set on the host; no wait runs out for real): every warp of the CTA stops, the copies
    in flight are drained, and the host reruns the pass with per-thread loads. The signs
    equal a normal call's, the stats count the rerun, and the next call runs normally."""
    torch = pytest.importorskip("torch")
    from cybermeshgenerator_gb300 import _lib
    from cybermeshgenerator_gb300 import workloads as W
    L = _lib.load()
    S = W.predicate_stream(300_000, kind, degenerate=0.1, near=0.1, seed=35)
    fn = cm.orient3d_stream if kind == "orient3d" else cm.insphere_stream
    n = S.shape[1]
    d = torch.tensor(S, device="cuda")  # device columns: the TMA-staged pass takes them
    ptrs = [d[k].data_ptr() for k in range(S.shape[0])]
    stream = torch.cuda.current_stream().cuda_stream

    def run():
        out = torch.zeros(n, dtype=torch.int8, device="cuda")
        _, st = fn((ptrs, n, out.data_ptr()), cm.PRED_COMPAT, stream=stream)
        torch.cuda.synchronize()
        return out.cpu().numpy(), st

    want, st0 = run()
    assert st0["tma_reruns"] == 0
    try:
        assert L.cmg_debug_fail_pred_wait(2) == 0   # CTA 0's third tile
        got, st = run()
    finally:
        L.cmg_debug_fail_pred_wait(-1)
    assert st["tma_reruns"] == 1
    assert np.array_equal(got, want)
    for k in ("fp64_queries", "exact_queries", "expansion_queries"):
        assert st[k] == st0[k], k
    again, st2 = run()
    assert st2["tma_reruns"] == 0 and np.array_equal(again, want)
    host, _ = fn(S, cm.PRED_COMPAT)
    assert np.array_equal(host, want)


def test_stream_device_memory(cm):
    torch = pytest.importorskip("torch")
    from cybermeshgenerator_gb300 import workloads as W
    S = W.predicate_stream(50_000, "orient3d", degenerate=0.1, near=0.1, seed=32)
    host, _ = cm.orient3d_stream(S, cm.PRED_EXACT)
    d = torch.tensor(S, device="cuda")
    out = torch.zeros(S.shape[1], dtype=torch.int8, device="cuda")
    ptrs = [d[k].data_ptr() for k in range(12)]
    cm.orient3d_stream((ptrs, S.shape[1], out.data_ptr()), cm.PRED_EXACT,
                       stream=torch.cuda.current_stream().cuda_stream)
    assert np.array_equal(out.cpu().numpy(), host)


_STREAMS = {}


def _stream_case(kind, n):
    from cybermeshgenerator_gb300 import workloads as W
    if (kind, n) not in _STREAMS:
        _STREAMS.clear()
        _STREAMS[(kind, n)] = W.predicate_stream(n, kind, degenerate=0.1, near=0.1, seed=33)
    return _STREAMS[(kind, n)]


@pytest.mark.parametrize("path", ["pull", "copy"])
@pytest.mark.parametrize("kind,n", [("orient3d", (1 << 24) + 123_457), ("insphere", (1 << 22) + 1001)])
def test_host_stream_chunks_match_device_and_oracle(cm, orc, kind, n, path, monkeypatch):
    """Host arrays, both ways: read by the device through the host's page tables in
    chunks of 2^24 queries ("pull", where the device supports it), or copied in chunks
    of 2^22 with the next chunk's upload overlapping this one's certification
    ("copy"). Signs and counts equal those of one device-resident call; the chunk
    seams and the ragged tail equal the oracle."""
    torch = pytest.importorskip("torch")
    import oracle as O
    monkeypatch.setenv("CMG_HOST_STREAM", path)
    S = _stream_case(kind, n)
    fn = cm.orient3d_stream if kind == "orient3d" else cm.insphere_stream
    ncol = S.shape[0]
    d = torch.tensor(S, device="cuda")
    out = torch.zeros(n, dtype=torch.int8, device="cuda")
    ptrs = [d[k].data_ptr() for k in range(ncol)]
    seams = [k << 22 for k in range(1, (n >> 22) + 1)] + [n]
    idx = np.unique(np.concatenate([np.arange(max(0, b - 3000), min(n, b + 3000)) for b in seams]
                                   + [np.arange(0, 3000)]))
    for mode in (cm.PRED_COMPAT, cm.PRED_EXACT):
        host, st = fn(S, mode)
        _, dst = fn((ptrs, n, out.data_ptr()), mode, stream=torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), host)
        for k in ("queries", "fp64_queries", "exact_queries", "expansion_queries"):
            assert st[k] == dst[k], k
        want = orc.stream(kind, np.ascontiguousarray(S[:, idx]), O.COMPAT if mode == cm.PRED_COMPAT else O.EXACT)
        assert np.array_equal(host[idx], want)
    del d


def _lcg_cloud(n, s):
    # the point cloud of tests/test_backend.cpp:14-18 (LCG, 24-bit fractions)
    pts = []
    for _ in range(n):
        p = []
        for _ in range(3):
            s = (s * 1664525 + 1013904223) & 0xFFFFFFFF
            p.append((s >> 8) / float(1 << 24))
        pts.append(p)
    return np.array(pts), s


def test_orient3d_signs_replaces_cuda_backend(cm, orc):
    # tests/test_backend.cpp:37-54: 2000 points, 100k random candidate tetrahedra
    import oracle as O
    pts, _ = _lcg_cloud(2000, 9)
    s = 123
    tets = np.zeros((100_000, 4), dtype=np.int32)
    for i in range(100_000):
        for k in range(4):
            s = (s * 1664525 + 1013904223) & 0xFFFFFFFF
            tets[i, k] = (s >> 8) % 2000
    got = cm.orient3d_signs(pts, tets)
    soa = np.concatenate([pts[tets[:, k]].T for k in range(4)])
    want = orc.stream("orient3d", soa, O.COMPAT)
    assert np.array_equal(got, want.astype(np.int32))
