"""Full-size parity: the 1M x 200 inner-product build (M=32, L=64) and the 1M x 512 cosine build
(M=48, L=96) against the oracle.

The oracle builds the same 1M-point graph on the host cores in seconds, so the benchmark's own
workload is checked id for id (projection, final graph, evaluation counts), and two GPU builds
must agree exactly (no run-to-run variation: every race of the reference has a canonical
resolution here).
"""
import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

N, D = 1_000_000, 200


@pytest.fixture(scope="module")
def workload():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from paragraph_gb300 import datagen
    base, gt = datagen.make_dataset_cuda(N, D, gt_k=128, seed=1234, device="cuda")
    torch.cuda.synchronize()
    return base, gt


def test_full_size_build_matches_oracle(workload):
    import paragraph_gb300 as pg
    base, gt = workload
    params = pg.default_params(32, 64)
    graph = torch.empty((N, 32), dtype=torch.int32, device="cuda")
    proj = torch.empty((N, 16), dtype=torch.int32, device="cuda")
    with pg.Handle(0) as h:
        st = h.build_device(base, gt, graph, proj, params)
        g1 = graph.cpu().numpy().view(np.uint32).copy()
        p1 = proj.cpu().numpy().view(np.uint32).copy()
        st2 = h.build_device(base, gt, graph, proj, params)
        g2 = graph.cpu().numpy().view(np.uint32)
    assert np.array_equal(g1, g2), "two GPU builds differ"
    assert st.evals_total == st2.evals_total
    base_np = base.cpu().numpy()
    gt_np = gt.cpu().numpy().view(np.uint32)
    ref = oracle.build_graph(base_np, gt_np, degree=32, beam=64)
    assert np.array_equal(p1, ref["proj"]), f"{(p1 != ref['proj']).any(axis=1).sum()} proj rows differ"
    bad = (g1 != ref["graph"]).any(axis=1)
    assert not bad.any(), f"{bad.sum()} of {N} graph rows differ"
    assert st.evals_total == ref["stats"]["evals_total"]
    assert list(st.search_iters)[:2] == ref["stats"]["iters_search"][:2]
    # structural properties of the index
    valid = g1 != pg.TOMB
    assert (g1[valid] < N).all()
    assert not (g1 == np.arange(N, dtype=np.uint32)[:, None]).any()
    assert valid.sum(axis=1).max() <= 32


def test_full_size_screened_build_is_identical(workload):
    import paragraph_gb300 as pg
    base, gt = workload
    outs = []
    stats = []
    with pg.Handle(0) as h:
        for screen in (pg.SCREEN_NONE, pg.SCREEN_BF16):
            graph = torch.empty((N, 32), dtype=torch.int32, device="cuda")
            proj = torch.empty((N, 16), dtype=torch.int32, device="cuda")
            stats.append(h.build_device(base, gt, graph, proj, pg.default_params(32, 64, screen=screen)))
            outs.append((graph.cpu().numpy(), proj.cpu().numpy()))
    assert np.array_equal(outs[0][1], outs[1][1])
    bad = (outs[0][0] != outs[1][0]).any(axis=1)
    assert not bad.any(), f"{bad.sum()} rows differ between the plain and the screened build"
    assert stats[0].evals_total == stats[1].evals_total
    print("rescored", list(stats[1].rescored)[:2], "of", list(stats[1].evals_prune)[:2])


def test_full_size_index_matches_oracle(workload):
    """pg_build_index at 1M x 200 (the reference driver's whole index: GPU build, six MatchSup
    rounds, FusionNN, FusionFinal) against the oracle's pipeline, list for list."""
    import paragraph_gb300 as pg
    base, gt = workload
    params = pg.default_params(32, 64, screen=pg.SCREEN_BF16)
    out = torch.full((N, 150), -1, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(N, dtype=torch.int32, device="cuda")
    with pg.Handle(0) as h:
        st = h.build_index(base, gt, out, cnt, params)
    print(f"index 1M: {st.ms_total:.1f} ms (MatchSup {st.ms_match_sup:.1f}, FusionNN "
          f"{st.ms_fusion_nn:.1f}, FusionFinal {st.ms_fusion_final:.1f})")
    rows = out.cpu().numpy().view(np.uint32)
    k = cnt.cpu().numpy().view(np.uint32).astype(np.int64)
    base_np = base.cpu().numpy()
    gt_np = gt.cpu().numpy().view(np.uint32)
    g = oracle.build_graph(base_np, gt_np, degree=32, beam=64)
    rounds = [oracle.match_sup(base_np, gt_np, r) for r in range(1, 7)]
    fnn = oracle.fusion_nn(base_np, rounds)
    off, ids = oracle.fusion_final(base_np, g["proj"], fnn, g["graph"])
    ref_k = np.diff(off.astype(np.int64))
    assert np.array_equal(k, ref_k), f"{(k != ref_k).sum()} row lengths differ"
    mask = np.arange(rows.shape[1])[None, :] < k[:, None]
    assert np.array_equal(rows[mask], ids), "index ids differ"


def test_full_size_cosine_512_screened_equals_plain_and_oracle():
    """The precision configuration at full size: 1M x 512, base and queries L2-normalised
    (cosine), 128 centres, M = 48, L = 96 (Km = 64), ground truth top-128 from pg_ground_truth.
    The FP16-screened build, the plain FP32 build and the oracle give the same projection, graph
    and evaluation counts."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import paragraph_gb300 as pg
    from paragraph_gb300 import datagen
    n, d = 1_000_000, 512
    base, _, queries = datagen.make_dataset_cuda(n, d, cosine=True, centers=128, seed=4321,
                                                 device="cuda", with_gt=False)
    gt = torch.empty((n, 128), dtype=torch.int32, device="cuda")
    outs, stats = [], []
    with pg.Handle(0) as h:
        h.ground_truth(base, queries, gt)
        del queries
        torch.cuda.empty_cache()
        for screen in (pg.SCREEN_FP16, pg.SCREEN_NONE):
            graph = torch.empty((n, 48), dtype=torch.int32, device="cuda")
            proj = torch.empty((n, 16), dtype=torch.int32, device="cuda")
            stats.append(h.build_device(base, gt, graph, proj,
                                        pg.default_params(48, 96, screen=screen)))
            outs.append((graph.cpu().numpy().view(np.uint32), proj.cpu().numpy().view(np.uint32)))
    assert np.array_equal(outs[0][1], outs[1][1]), "projection: screened != plain"
    bad = (outs[0][0] != outs[1][0]).any(axis=1)
    assert not bad.any(), f"{bad.sum()} rows differ between the screened and the plain build"
    assert stats[0].evals_total == stats[1].evals_total
    base_np = base.cpu().numpy()
    gt_np = gt.cpu().numpy().view(np.uint32)
    del base, gt
    torch.cuda.empty_cache()
    ref = oracle.build_graph(base_np, gt_np, degree=48, beam=96)
    assert np.array_equal(outs[1][1], ref["proj"])
    bad = (outs[1][0] != ref["graph"]).any(axis=1)
    assert not bad.any(), f"{bad.sum()} of {n} graph rows differ from the oracle"
    assert stats[1].evals_total == ref["stats"]["evals_total"]
    print(f"cosine 1M x 512: screened {stats[0].ms_total:.1f} ms, plain {stats[1].ms_total:.1f} ms,"
          f" rescored {list(stats[0].rescored)[:2]}")
