"""CUDA kernels against the oracle and the reference-generated golden fixtures (GPU).

Every comparison is bit-exact on ids (integer work).  The stage tests feed each kernel the exact
inputs the reference kernels received (tests/golden/ref_*.npz, produced by the reference's own
code) and compare every output; the search is compared with the reference's own search kernel
run under a warp emulator (tests/golden/ref_search_*.npz) and with the oracle; the whole-build
tests compare against the oracle.
"""
import os

import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOMB = 0xFFFFFFFF
CASES = ["mix", "edge"]


@pytest.fixture(scope="module")
def pg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import paragraph_gb300
    paragraph_gb300.lib()
    return paragraph_gb300


@pytest.fixture(scope="module")
def handle(pg):
    h = pg.Handle(0)
    yield h
    h.close()


def load(golden_dir, name):
    return dict(np.load(os.path.join(golden_dir, f"ref_{name}_1000x200.npz")))


def dev_u32(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint32).view(np.int32)).cuda()


def dev_f32(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


def host_u32(t):
    torch.cuda.synchronize()
    return t.cpu().numpy().view(np.uint32)


def empty_u32(*shape):
    return torch.full(shape, -1, dtype=torch.int32, device="cuda")


def masked(a, cnt):
    a = a.copy()
    c = np.minimum(cnt, a.shape[1])
    a[np.arange(a.shape[1])[None, :] >= c[:, None]] = TOMB
    return a


@pytest.mark.parametrize("case", CASES)
def test_match_top1_matches_reference(handle, golden_dir, case):
    f = load(golden_dir, case)
    out = empty_u32(1000, 128)
    handle.match_top1(dev_u32(f["gt"]), 1000, out)
    assert np.array_equal(host_u32(out), f["k0"])


def _prune(handle, base, graph, p, r, strict):
    n = base.shape[0]
    pr, pn = empty_u32(n, p), empty_u32(n)
    rv, rn = empty_u32(n, r), empty_u32(n)
    srt = empty_u32(n, graph.shape[1])
    ev = handle.prune_reverse(dev_f32(base), dev_u32(graph), pr, pn, rv, rn, strict, srt)
    return host_u32(pr), host_u32(pn), host_u32(rv), host_u32(rn), host_u32(srt), ev, (pr, pn, rv, rn)


@pytest.mark.parametrize("case", CASES)
def test_phase1_prune_reverse_merge_match_reference(handle, golden_dir, case):
    f = load(golden_dir, case)
    pr, pn, rv, rn, srt, ev, dev = _prune(handle, f["base"], f["k0"], 15, 111, False)
    assert np.array_equal(srt, f["p1_sorted"])
    assert np.array_equal(pn, f["p1_pnum"])
    assert np.array_equal(rn, f["p1_rnum"])
    assert np.array_equal(masked(pr, pn), f["p1_pruned"])
    assert np.array_equal(masked(rv, rn), f["p1_rev"])
    ref = oracle.prune_reverse(f["base"], f["k0"], 15, 111, strict=False)
    assert ev == ref.evals
    out = empty_u32(1000, 16)
    ev2 = handle.merge_prune(dev_f32(f["base"]), dev[0], dev[1], dev[2], dev[3], out, False)
    assert np.array_equal(host_u32(out), f["proj"])
    assert ev2 == oracle.merge_prune(f["base"], ref, 16, strict=False)[1]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("which,p,r", [("link32", 32, 94), ("link55", 55, 71)])
def test_link_prune_reverse_merge_match_reference(handle, golden_dir, case, which, p, r):
    f = load(golden_dir, case)
    pr, pn, rv, rn, srt, ev, dev = _prune(handle, f["base"], f["search_in"], p, r, True)
    assert np.array_equal(srt, f[f"{which}_sorted"])
    assert np.array_equal(pn, f[f"{which}_pnum"])
    assert np.array_equal(rn, f[f"{which}_rnum"])
    assert np.array_equal(masked(pr, pn), f[f"{which}_pruned"])
    assert np.array_equal(masked(rv, rn), f[f"{which}_rev"])
    out = empty_u32(1000, p)
    handle.merge_prune(dev_f32(f["base"]), dev[0], dev[1], dev[2], dev[3], out, True)
    assert np.array_equal(host_u32(out), f[f"{which}_graph"])


@pytest.mark.parametrize("case", CASES)
def test_search_matches_oracle(handle, golden_dir, case):
    f = load(golden_dir, case)
    out = empty_u32(1000, 64)
    ev, it = handle.search(dev_f32(f["base"]), dev_u32(f["proj"]), out)
    ref, rev, rit, hit = oracle.search(f["base"], f["proj"])
    got = host_u32(out)
    assert np.array_equal(got, ref), f"{(got != ref).any(axis=1).sum()} rows differ"
    assert (ev, it) == (rev, rit)
    assert np.array_equal(got, f["search_in"])


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("graph", ["proj", "link32_graph", "link55_graph"])
def test_search_matches_reference_search(handle, golden_dir, case, graph):
    """k_search_m32 against the reference's own link_process_v0_store_base_data
    (Gsearcher.cuh:890-1066), run under the warp emulator on the same inputs
    (tests/golden/ref_search_*.npz): the round-1 search over the projection and the round-2
    search over the reference-merged link graphs, id for id, with the evaluation and iteration
    counts."""
    f = load(golden_dir, case)
    r = np.load(os.path.join(golden_dir, f"ref_search_{case}_1000x200.npz"))
    out = empty_u32(1000, 64)
    ev, it = handle.search(dev_f32(f["base"]), dev_u32(f[graph]), out)
    got = host_u32(out)
    want = r[f"{graph}_ids"]
    assert np.array_equal(got, want), f"{(got != want).any(axis=1).sum()} rows differ"
    assert ev == int(r[f"{graph}_evals"].sum())
    assert it == int(r[f"{graph}_iters"].sum())


@pytest.mark.parametrize("km", [32, 64])
def test_search_beam_widths_match_oracle(handle, km):
    from paragraph_gb300 import datagen
    base, gt = datagen.make_dataset(3000, 128, seed=21)
    proj = oracle.build_graph(base, gt, link_rounds=0)["proj"]
    L = km + 32
    out = empty_u32(3000, L)
    ev, it = handle.search(dev_f32(base), dev_u32(proj), out, km=km)
    ref, rev, rit, _ = oracle.search(base, proj, km=km)
    assert np.array_equal(host_u32(out), ref)
    assert (ev, it) == (rev, rit)


def _build_both(pg, handle, base, gt, degree=32, beam=64, screen=0):
    n, d = base.shape
    graph = empty_u32(n, degree)
    proj = empty_u32(n, 16)
    st = handle.build_device(dev_f32(base), dev_u32(gt), graph, proj,
                             pg.default_params(degree, beam, screen=screen))
    ref = oracle.build_graph(base, gt, degree=degree, beam=beam)
    return host_u32(graph), host_u32(proj), st, ref


@pytest.mark.parametrize("case", CASES)
def test_full_build_fixture_matches_oracle(pg, handle, golden_dir, case):
    f = load(golden_dir, case)
    g, p, st, ref = _build_both(pg, handle, f["base"], f["gt"])
    assert np.array_equal(p, f["proj"])
    assert np.array_equal(p, ref["proj"])
    assert np.array_equal(g, ref["graph"])
    assert st.evals_total == ref["stats"]["evals_total"]


@pytest.mark.parametrize("n,d,degree,beam,seed", [
    (20000, 200, 32, 64, 1),   # the 1M x 200 configuration's shape at test size
    (8000, 512, 48, 96, 2),    # the cosine configuration's degree/beam (M=48, L=96)
    (5000, 64, 55, 64, 3),     # the reference's own degree 55 (R=71)
    (33, 8, 16, 64, 4),        # fewer points than search seeds: seeds wrap around
])
def test_full_build_matches_oracle(pg, handle, n, d, degree, beam, seed):
    from paragraph_gb300 import datagen
    base, gt = datagen.make_dataset(n, d, seed=seed, cosine=(d == 512))
    if gt.shape[1] < 128:  # fewer than 128 points: pad the ground truth with tombs
        gt = np.concatenate([gt, np.full((gt.shape[0], 128 - gt.shape[1]), TOMB, np.uint32)], 1)
    g, p, st, ref = _build_both(pg, handle, base, gt, degree, beam)
    assert np.array_equal(p, ref["proj"])
    assert np.array_equal(g, ref["graph"]), f"{(g != ref['graph']).any(axis=1).sum()} rows differ"
    assert st.evals_total == ref["stats"]["evals_total"]
    assert list(st.search_iters)[:2] == ref["stats"]["iters_search"][:2]


def test_build_host_equals_build_device(pg, handle, golden_dir):
    f = load(golden_dir, "mix")
    g_host, p_host, st = handle.build_host(f["base"], f["gt"], pg.default_params(32, 64))
    g_dev, p_dev, st2, _ = _build_both(pg, handle, f["base"], f["gt"])
    assert np.array_equal(g_host, g_dev) and np.array_equal(p_host, p_dev)
    assert st.h2d_bytes == f["base"].nbytes + f["gt"].nbytes
    assert st.evals_total == st2.evals_total


@pytest.mark.parametrize("n,d,seed", [(3001, 8, 21), (2999, 200, 22)])
def test_build_host_copy_split(pg, handle, n, d, seed):
    """pg_build_host splits the input bytes over two copy streams: D=8 puts all of base on the
    first and gt on the second (gt is the larger), D=200 splits base itself; odd n makes the
    split point fall inside a row.  Both equal the device-resident build and the oracle."""
    from paragraph_gb300 import datagen
    base, gt = datagen.make_dataset(n, d, seed=seed)
    g_host, p_host, st = handle.build_host(base, gt, pg.default_params(32, 64))
    g_dev, p_dev, _, ref = _build_both(pg, handle, base, gt)
    assert np.array_equal(g_host, g_dev) and np.array_equal(p_host, p_dev)
    assert np.array_equal(g_host, ref["graph"])
    assert st.h2d_bytes == base.nbytes + gt.nbytes


@pytest.mark.parametrize("n,d,seed", [(3001, 8, 23), (2999, 200, 24)])
def test_build_host_pinned_buffers(pg, handle, n, d, seed):
    """Pinned host buffers that the device can address are moved by the copy kernel (host to
    device and back) instead of the copy engines; results equal the device-resident build."""
    from paragraph_gb300 import datagen
    base, gt = datagen.make_dataset(n, d, seed=seed)
    params = pg.default_params(32, 64)
    base_h = torch.from_numpy(base).pin_memory()
    gt_h = torch.from_numpy(gt.view(np.int32)).pin_memory()
    graph_h = torch.empty((n, params.degree), dtype=torch.int32).pin_memory()
    proj_h = torch.empty((n, params.proj_degree), dtype=torch.int32).pin_memory()
    st = handle.build_host_ptr(base_h.data_ptr(), n, d, gt_h.data_ptr(), gt.shape[0],
                               graph_h.data_ptr(), proj_h.data_ptr(), params)
    g_dev, p_dev, _, ref = _build_both(pg, handle, base, gt)
    assert np.array_equal(graph_h.numpy().view(np.uint32), g_dev)
    assert np.array_equal(proj_h.numpy().view(np.uint32), p_dev)
    assert np.array_equal(g_dev, ref["graph"])
    assert st.h2d_bytes == base.nbytes + gt.nbytes


def test_builder_facade_and_savegraph(pg, golden_dir, tmp_path):
    f = load(golden_dir, "mix")
    b = pg.Builder(f["base"], f["gt"])
    graph = b.LaunchBuild(dim=200, gt_num=128)
    path = str(tmp_path / "index.bin")
    b.SaveGraph(path)
    ep, rows = pg.load_graph(path)
    assert ep == b.ep and len(rows) == 1000
    for i in (0, 17, 999):
        assert np.array_equal(rows[i], graph[i][graph[i] != TOMB])


def test_bad_ids_are_rejected(pg, handle):
    base = np.random.default_rng(0).standard_normal((100, 16)).astype(np.float32)
    gt = np.tile(np.arange(128, dtype=np.uint32) % 100, (100, 1))
    gt[5, 0] = 100  # out of range
    graph = empty_u32(100, 32)
    with pytest.raises(pg.PGError) as e:
        handle.build_device(dev_f32(base), dev_u32(gt), graph, None,
                            pg.default_params(32, 64, flags=pg.FLAG_VALIDATE_INPUT))
    assert e.value.code == pg.PG_EINVAL
    # the handle stays usable after the error
    gt[5, 0] = 7
    handle.build_device(dev_f32(base), dev_u32(gt), graph, None, pg.default_params(32, 64))


def test_iteration_cap_reports_timeout(pg, handle):
    base, gt = __import__("paragraph_gb300.datagen", fromlist=["x"]).make_dataset(500, 32, seed=9)
    graph = empty_u32(500, 32)
    with pytest.raises(pg.PGError) as e:
        handle.build_device(dev_f32(base), dev_u32(gt), graph, None,
                            pg.default_params(32, 64, max_search_iters=1))
    assert e.value.code == pg.PG_ETIMEOUT
    handle.build_device(dev_f32(base), dev_u32(gt), graph, None, pg.default_params(32, 64))


def test_unsupported_shapes_are_rejected(pg, handle):
    base = np.zeros((100, 10), dtype=np.float32)  # d % 4 != 0
    gt = np.zeros((100, 128), dtype=np.uint32)
    with pytest.raises(pg.PGError) as e:
        handle.build_device(dev_f32(base), dev_u32(gt), empty_u32(100, 32), None)
    assert e.value.code == pg.PG_EUNSUPPORTED


@pytest.mark.parametrize("case", CASES)
def test_screened_build_matches_plain_and_oracle_fixture(pg, handle, golden_dir, case):
    f = load(golden_dir, case)
    g, p, st, ref = _build_both(pg, handle, f["base"], f["gt"], screen=pg.SCREEN_BF16)
    assert np.array_equal(p, ref["proj"])
    assert np.array_equal(g, ref["graph"])
    assert st.evals_total == ref["stats"]["evals_total"]


@pytest.mark.parametrize("screen", [1, 3])  # BF16, FP16
@pytest.mark.parametrize("n,d,seed", [(20000, 200, 1), (6000, 64, 7), (3000, 8, 8),
                                      (4999, 100, 9)])
def test_screened_build_matches_oracle(pg, handle, n, d, seed, screen):
    """(4999, 100): an odd node count leaves the last two-node tile of the tensor-core prune half
    empty, and D = 100 ends in a chunk of 4 columns (one K = 16 MMA step on zero padding)."""
    from paragraph_gb300 import datagen
    base, gt = datagen.make_dataset(n, d, seed=seed)
    g, p, st, ref = _build_both(pg, handle, base, gt, screen=screen)
    assert np.array_equal(p, ref["proj"])
    bad = (g != ref["graph"]).any(axis=1)
    assert not bad.any(), f"{bad.sum()} rows differ"
    assert st.evals_total == ref["stats"]["evals_total"]
    # the screen decides most occlusion tests without the exact chain
    assert sum(st.rescored) < 0.5 * sum(st.evals_prune)


@pytest.mark.parametrize("beam", [64, 128])  # two nodes per tensor-core tile, one
@pytest.mark.parametrize("screen", [1, 3])  # BF16, FP16
def test_screened_build_extreme_scales(pg, handle, screen, beam):
    """Points scaled by 1e-6 .. 1e5: FP16 copies with subnormal coordinates (the norm bounds carry
    their norm, in case the tensor core flushes them) and coordinates beyond FP16's range (infinite
    norm bounds: every test of such a point goes to the exact chain).  Edges still equal the
    oracle's."""
    from paragraph_gb300 import datagen
    base, gt = datagen.make_dataset(3000, 64, seed=9)
    f = 10.0 ** np.random.default_rng(9).uniform(-6, 5, base.shape[0])
    base = np.ascontiguousarray(base * f[:, None].astype(np.float32), dtype=np.float32)
    assert np.isfinite(base).all() and (np.abs(base) > 65504).any()
    g, p, st, ref = _build_both(pg, handle, base, gt, beam=beam, screen=screen)
    assert np.array_equal(p, ref["proj"])
    bad = (g != ref["graph"]).any(axis=1)
    assert not bad.any(), f"{bad.sum()} rows differ"
    assert st.evals_total == ref["stats"]["evals_total"]


@pytest.mark.parametrize("screen", [1, 3])
def test_screened_build_with_hubs_and_duplicates(pg, handle, golden_dir, screen):
    """Exact duplicate vectors give exact ties and zero-width gaps: the screen must defer every
    such decision to the exact chain."""
    f = load(golden_dir, "edge")
    g, p, st, ref = _build_both(pg, handle, f["base"], f["gt"], screen=screen)
    assert np.array_equal(g, ref["graph"])


@pytest.mark.parametrize("screen", [1, 3])  # BF16, FP16
@pytest.mark.parametrize("n,d,degree,seed,cosine,beam", [(8000, 512, 48, 5, True, 96),
                                                         (6000, 200, 32, 6, False, 96),
                                                         (5000, 200, 32, 7, False, 128),
                                                         (4000, 36, 24, 8, True, 128)])
def test_screened_build_wide_beams(pg, handle, n, d, degree, seed, cosine, beam, screen):
    """L = 96 and 128: the screened prune's one-node tiles (more than 64 candidates per node
    fill a 128-row tensor-core tile on their own); D = 36 ends in a chunk of 4 columns."""
    from paragraph_gb300 import datagen
    base, q = datagen.make_base_queries(n, d, seed=seed, cosine=cosine)
    gt = datagen.ground_truth(base, q, 128)
    g, p, st, ref = _build_both(pg, handle, base, gt, degree=degree, beam=beam, screen=screen)
    assert np.array_equal(p, ref["proj"])
    bad = (g != ref["graph"]).any(axis=1)
    assert not bad.any(), f"{bad.sum()} rows differ"
    assert st.evals_total == ref["stats"]["evals_total"]
    assert sum(st.rescored) < 0.5 * sum(st.evals_prune)


@pytest.mark.parametrize("beam", [96, 128])
@pytest.mark.parametrize("screen", [1, 3])
def test_screened_wide_beams_with_hubs_and_duplicates(pg, handle, golden_dir, screen, beam):
    f = load(golden_dir, "edge")
    g, p, st, ref = _build_both(pg, handle, f["base"], f["gt"], degree=32, beam=beam,
                                screen=screen)
    assert np.array_equal(g, ref["graph"])
    assert st.evals_total == ref["stats"]["evals_total"]
