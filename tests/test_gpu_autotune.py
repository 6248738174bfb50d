"""Autotuner (pg_autotune / pg_set_tuning): every launch shape it can choose builds the same graph
bit for bit; the beam it picks reaches the recall target or is the best of the three tried."""
import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

N, D = 20000, 200


@pytest.fixture(scope="module")
def pg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import paragraph_gb300
    paragraph_gb300.lib()
    return paragraph_gb300


@pytest.fixture(scope="module")
def data():
    from paragraph_gb300 import datagen
    base, queries = datagen.make_base_queries(N, D, seed=4242)
    gt = datagen.ground_truth(base, queries, 128)
    return base, queries, gt


def _dev(a):
    a = np.ascontiguousarray(a)
    return torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).cuda()


def _build(pg, h, base, gt, params):
    graph = torch.empty((base.shape[0], params.degree), dtype=torch.int32, device="cuda")
    h.build_device(base, gt, graph, None, params)
    return graph.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("field,value", [("search_rows", 16), ("search_warps_per_sm", 8),
                                         ("hash_factor", 4), ("screen_stages", 4)])
def test_every_launch_shape_builds_the_same_graph(pg, data, field, value):
    base, _, gt = data
    db, dg = _dev(base), _dev(gt)
    params = pg.default_params(32, 64, screen=1)
    with pg.Handle(0) as h:
        ref = _build(pg, h, db, dg, params)
        t = pg.Tuning()
        setattr(t, field, value)
        h.set_tuning(t)
        assert getattr(h.get_tuning(), field) == value
        assert np.array_equal(_build(pg, h, db, dg, params), ref)


def test_bad_tuning_is_rejected(pg):
    with pg.Handle(0) as h:
        for field, value in [("search_rows", 12), ("hash_factor", 3), ("screen_stages", 5)]:
            t = pg.Tuning()
            setattr(t, field, value)
            with pytest.raises(pg.PGError) as e:
                h.set_tuning(t)
            assert e.value.code == pg.PG_EINVAL


def test_autotune_keeps_results_and_picks_a_beam(pg, data):
    base, queries, gt = data
    db, dg, dq = _dev(base), _dev(gt), _dev(queries)
    params = pg.default_params(32, 64, screen=1)
    with pg.Handle(0) as h:
        p, t = h.autotune(db, dg, params, queries=dq, target_recall=0.95)
        print("tuning", t.as_dict(), "km", p.km)
        assert t.beam in (64, 96, 128) and p.km == t.beam - 32
        assert 0.0 <= t.recall <= 1.0
        assert t.ms_build <= t.ms_default
        assert t.search_rows in (8, 16) and t.hash_factor in (1, 2, 4)
        tuned = _build(pg, h, db, dg, p)
    with pg.Handle(0) as h2:  # default launch shapes, same params
        assert np.array_equal(_build(pg, h2, db, dg, p), tuned)
    ref = oracle.build_graph(base, gt, degree=32, beam=t.beam)["graph"]
    assert np.array_equal(tuned, ref)


def test_autotune_batched_table(pg):
    from paragraph_gb300 import datagen
    sizes = [3000, 700, 5000, 1200]
    subs = [datagen.make_dataset(n, 64, seed=900 + i) for i, n in enumerate(sizes)]
    node_off = np.concatenate([[0], np.cumsum(sizes)])
    base = _dev(np.concatenate([b for b, _ in subs]))
    gt = _dev(np.concatenate([g for _, g in subs]))
    params = pg.default_params(32, 64, screen=1)
    n = int(node_off[-1])
    with pg.Handle(0) as h:
        ref = torch.empty((n, 32), dtype=torch.int32, device="cuda")
        h.build_batched(base, gt, node_off, node_off, ref, None, params)
        p, t = h.autotune(base, gt, params, node_off=node_off, query_off=node_off)
        assert t.beam == 0 and p.km == params.km
        out = torch.empty_like(ref)
        h.build_batched(base, gt, node_off, node_off, out, None, p)
        assert torch.equal(out, ref)
