"""The oracle against the reference's own kernels (CPU, no GPU needed).

tests/golden/ref_*.npz hold the outputs of the reference's thread-per-node kernels
(include/Gbuilder.cuh) run on one thread by tests/golden/make_golden.py;
tests/golden/ref_search_*.npz and ref_qsearch_*.npz those of its warp-per-query beam searches
(include/Gsearcher.cuh) run under a 32-lane warp emulator by tests/golden/make_golden_search.py.
The oracle must reproduce every stage bit for bit: this pins oracle/pg_oracle.c to the
reference.
"""
import numpy as np
import pytest

import oracle

TOMB = oracle.TOMB
CASES = ["mix", "edge"]


def load(golden_dir, name):
    import os
    return dict(np.load(os.path.join(golden_dir, f"ref_{name}_1000x200.npz")))


def masked(a, cnt):
    a = a.copy()
    c = np.minimum(cnt, a.shape[1])
    a[np.arange(a.shape[1])[None, :] >= c[:, None]] = TOMB
    return a


@pytest.mark.parametrize("case", CASES)
def test_projection_rows(golden_dir, case):
    f = load(golden_dir, case)
    n = f["base"].shape[0]
    assert np.array_equal(oracle.match_top1(f["gt"], n), f["k0"])


@pytest.mark.parametrize("case", CASES)
def test_phase1_prune_reverse_and_merge(golden_dir, case):
    f = load(golden_dir, case)
    pr = oracle.prune_reverse(f["base"], f["k0"], 15, 111, strict=False)
    assert np.array_equal(pr.sorted_rows, f["p1_sorted"])
    assert np.array_equal(pr.pruned_num, f["p1_pnum"])
    assert np.array_equal(pr.reverse_num, f["p1_rnum"])
    assert np.array_equal(masked(pr.pruned, pr.pruned_num), f["p1_pruned"])
    assert np.array_equal(masked(pr.reverse, pr.reverse_num), f["p1_rev"])
    proj, ev = oracle.merge_prune(f["base"], pr, 16, strict=False)
    assert np.array_equal(proj, f["proj"])
    assert ev > 0


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("which,p,r", [("link32", 32, 94), ("link55", 55, 71)])
def test_link_round_prune_reverse_and_merge(golden_dir, case, which, p, r):
    f = load(golden_dir, case)
    pr = oracle.prune_reverse(f["base"], f["search_in"], p, r, strict=True)
    assert np.array_equal(pr.sorted_rows, f[f"{which}_sorted"])
    assert np.array_equal(pr.pruned_num, f[f"{which}_pnum"])
    assert np.array_equal(pr.reverse_num, f[f"{which}_rnum"])
    assert np.array_equal(masked(pr.pruned, pr.pruned_num), f[f"{which}_pruned"])
    assert np.array_equal(masked(pr.reverse, pr.reverse_num), f[f"{which}_rev"])
    g, _ = oracle.merge_prune(f["base"], pr, p, strict=True)
    assert np.array_equal(g, f[f"{which}_graph"])


def test_edge_case_exercises_reverse_cap(golden_dir):
    f = load(golden_dir, "edge")
    assert (f["link32_rnum"] == 94).sum() > 0, "hub case must overflow the reverse list"
    assert (f["gt"] == TOMB).any(), "padded ground truth rows present"


def test_visited_set_matches_reference_hashtable(golden_dir):
    import os
    h = np.load(os.path.join(golden_dir, "ref_hashtable.npz"))
    seen = set()
    flags = []
    for k, r in zip(h["keys"], h["reset"]):
        if r:
            seen.clear()
        new = int(k) not in seen
        seen.add(int(k))
        flags.append(1 if new else 0)
    assert np.array_equal(np.array(flags, dtype=np.uint8), h["flags"])


def test_reduction_orders():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((2, 200)).astype(np.float32)
    s = np.float32(0)
    for i in range(200):
        s = np.float32(np.float64(x[0, i]) * np.float64(x[1, i]) + np.float64(s))  # exact fma
    assert oracle.dist_seq(x, 0, 1) == -s
    lanes = np.zeros(32, dtype=np.float32)
    for i in range(200):
        l = i % 32
        lanes[l] = np.float32(np.float64(x[0, i]) * np.float64(x[1, i]) + np.float64(lanes[l]))
    for off in (16, 8, 4, 2, 1):
        lanes[:off] = lanes[:off] + lanes[off:2 * off]
    assert oracle.dist_lane(x[0], x[1]) == -lanes[0]


def test_full_build_runs_and_is_deterministic(golden_dir):
    f = load(golden_dir, "mix")
    a = oracle.build_graph(f["base"], f["gt"])
    b = oracle.build_graph(f["base"], f["gt"])
    assert np.array_equal(a["graph"], b["graph"]) and np.array_equal(a["proj"], b["proj"])
    assert np.array_equal(a["proj"], f["proj"])
    g = a["graph"]
    n = g.shape[0]
    valid = g != TOMB
    assert (g[valid] < n).all()
    assert not (g == np.arange(n, dtype=np.uint32)[:, None]).any(), "no self loops"
    assert a["stats"]["evals_total"] > 0 and not a["stats"]["cap_hit"]


SEARCH_GRAPHS = ["proj", "link32_graph", "link55_graph"]


@pytest.mark.parametrize("case", ["mix", "edge"])
@pytest.mark.parametrize("graph", SEARCH_GRAPHS)
def test_search_matches_reference_search(golden_dir, case, graph):
    """The oracle's beam search against the reference's own link_process_v0_store_base_data
    (Gsearcher.cuh:890-1066) run under the warp emulator (tests/golden/ref_search_*.npz): every
    id of every list, and the evaluation and iteration counts."""
    import os
    f = load(golden_dir, case)
    r = np.load(os.path.join(golden_dir, f"ref_search_{case}_1000x200.npz"))
    ids, ev, it, hit = oracle.search(f["base"], f[graph])
    assert not hit
    assert np.array_equal(ids, r[f"{graph}_ids"]), f"{(ids != r[graph + '_ids']).any(1).sum()} rows"
    assert ev == int(r[f"{graph}_evals"].sum())
    assert it == int(r[f"{graph}_iters"].sum())


def test_search_fixture_is_the_link_rounds_input(golden_dir):
    """The round-1 search input of the stage fixtures (search_in) is the reference search's own
    output over the reference-made projection."""
    import os
    for case in ("mix", "edge"):
        f = load(golden_dir, case)
        r = np.load(os.path.join(golden_dir, f"ref_search_{case}_1000x200.npz"))
        assert np.array_equal(f["search_in"], r["proj_ids"])


def test_query_search_matches_reference(golden_dir):
    """The oracle's query search against the reference's search_shared_hashtable
    (Gsearcher.cuh:108-296) under the warp emulator: 300 cross-modal queries, topk 10."""
    import os
    q = np.load(os.path.join(golden_dir, "ref_qsearch_2000x64.npz"))
    ids, ev, it = oracle.query_search(q["base"], q["graph"], q["queries"], topk=int(q["topk"]),
                                      reset_iter=int(q["reset_iter"]))
    assert np.array_equal(ids, q["ids"])
    assert (ev, it) == (int(q["evals"].sum()), int(q["iters"].sum()))
