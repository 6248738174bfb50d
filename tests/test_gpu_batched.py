"""Batched build of many uneven sub-indexes (pg_build_batched_device) against building each
sub-index alone and against the oracle: ids must match bit for bit, evaluation counts must add up.
"""
import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOMB = 0xFFFFFFFF
SIZES = [1500, 700, 3000, 250, 2000, 40]  # uneven; the last one is smaller than the 32 seeds


@pytest.fixture(scope="module")
def pg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import paragraph_gb300
    paragraph_gb300.lib()
    return paragraph_gb300


@pytest.fixture(scope="module")
def subindexes():
    from paragraph_gb300 import datagen
    out = []
    for i, n in enumerate(SIZES):
        base, gt = datagen.make_dataset(n, 64, seed=100 + i)
        if gt.shape[1] < 128:
            gt = np.concatenate([gt, np.full((n, 128 - gt.shape[1]), TOMB, np.uint32)], 1)
        out.append((base, gt))
    return out


def _dev(a, dtype):
    a = np.ascontiguousarray(a)
    return torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).cuda()


@pytest.mark.parametrize("screen", [0, 1])
def test_batched_equals_one_by_one_and_oracle(pg, subindexes, screen):
    params = pg.default_params(32, 64, screen=screen)
    node_off = np.concatenate([[0], np.cumsum([b.shape[0] for b, _ in subindexes])])
    query_off = np.concatenate([[0], np.cumsum([g.shape[0] for _, g in subindexes])])
    base_all = np.concatenate([b for b, _ in subindexes])
    gt_all = np.concatenate([g for _, g in subindexes])
    n = base_all.shape[0]
    graph = torch.empty((n, 32), dtype=torch.int32, device="cuda")
    proj = torch.empty((n, 16), dtype=torch.int32, device="cuda")
    with pg.Handle(0) as h:
        st = h.build_batched(_dev(base_all, np.float32), _dev(gt_all, np.uint32), node_off,
                             query_off, graph, proj, params)
        g_all = graph.cpu().numpy().view(np.uint32)
        p_all = proj.cpu().numpy().view(np.uint32)
        total = 0
        for i, (b, g) in enumerate(subindexes):
            gi = torch.empty((b.shape[0], 32), dtype=torch.int32, device="cuda")
            pi = torch.empty((b.shape[0], 16), dtype=torch.int32, device="cuda")
            sti = h.build_device(_dev(b, np.float32), _dev(g, np.uint32), gi, pi, params)
            total += sti.evals_total
            lo, hi = node_off[i], node_off[i + 1]
            alone = gi.cpu().numpy().view(np.uint32)
            assert np.array_equal(g_all[lo:hi], alone), f"sub-index {i}: batched != alone"
            assert np.array_equal(p_all[lo:hi], pi.cpu().numpy().view(np.uint32))
            ref = oracle.build_graph(b, g, degree=32, beam=64)
            assert np.array_equal(alone, ref["graph"]), f"sub-index {i}: GPU != oracle"
    assert st.evals_total == total


def test_batched_rejects_bad_tables(pg, subindexes):
    b, g = subindexes[0]
    graph = torch.empty((b.shape[0], 32), dtype=torch.int32, device="cuda")
    with pg.Handle(0) as h:
        with pytest.raises(pg.PGError) as e:
            h.build_batched(_dev(b, np.float32), _dev(g, np.uint32), [0, 0, b.shape[0]],
                            [0, 10, b.shape[0]], graph)
        assert e.value.code == pg.PG_EINVAL
        bad = g.copy()
        bad[3, 5] = b.shape[0]  # a local id past its sub-index
        with pytest.raises(pg.PGError) as e:
            h.build_batched(_dev(b, np.float32), _dev(bad, np.uint32), [0, b.shape[0]],
                            [0, b.shape[0]], graph)
        assert e.value.code == pg.PG_EINVAL


def test_cuda_graph_replay_equals_eager(pg, subindexes):
    """PG_FLAG_CUDA_GRAPH: the captured build (batched table included) replays to the same
    graph as an eager build, and a changed table is re-captured."""
    node_off = np.concatenate([[0], np.cumsum([b.shape[0] for b, _ in subindexes])])
    query_off = np.concatenate([[0], np.cumsum([g.shape[0] for _, g in subindexes])])
    base_all = _dev(np.concatenate([b for b, _ in subindexes]), np.float32)
    gt_all = _dev(np.concatenate([g for _, g in subindexes]), np.uint32)
    n = int(node_off[-1])
    eager = torch.empty((n, 32), dtype=torch.int32, device="cuda")
    graph = torch.empty((n, 32), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    stream = torch.cuda.Stream()
    with pg.Handle(0, stream=stream) as h:
        st0 = h.build_batched(base_all, gt_all, node_off, query_off, eager, None,
                              pg.default_params(32, 64, screen=1))
        p = pg.default_params(32, 64, screen=1, flags=pg.FLAG_CUDA_GRAPH)
        for _ in range(3):  # capture, then replays
            graph.fill_(-1)
            torch.cuda.synchronize()
            st = h.build_batched(base_all, gt_all, node_off, query_off, graph, None, p)
            assert torch.equal(graph, eager)
            assert st.evals_total == st0.evals_total
        # a different sub-index table (first two merged into one) must not reuse the capture
        merged_off = np.concatenate([[0], node_off[2:]])
        merged_q = np.concatenate([[0], query_off[2:]])
        st2 = h.build_batched(base_all, gt_all, merged_off, merged_q, graph, None, p)
        assert st2.evals_total != st0.evals_total or not torch.equal(graph, eager)
