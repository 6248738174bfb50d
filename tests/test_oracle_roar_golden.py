"""The oracle's restatement of the CPU RoarGraph path (oracle/pg_oracle_roar.c) against the
reference's own code (tests/golden/ref_cpu_*.npz, made by tests/golden/make_golden_cpu.py from
tests/test_t2iend.cu compiled with AVX-512): compare() bit for bit, MatchNN's entry point,
MatchSup rounds 1..6 as neighbour sets (the reference writes short merged lists in
std::unordered_set order; every consumer de-duplicates and re-sorts them), FusionNN and
FusionFinal list for list, in order."""
import os

import numpy as np
import pytest

import oracle
import paragraph_gb300 as pg

CASES = ["mix", "edge"]


def load(golden_dir, name):
    f = dict(np.load(os.path.join(golden_dir, f"ref_{name}_1000x200.npz")))
    c = dict(np.load(os.path.join(golden_dir, f"ref_cpu_{name}_1000x200.npz")))
    return f, c


def rows(off, ids):
    return [ids[off[i]:off[i + 1]] for i in range(len(off) - 1)]


@pytest.mark.parametrize("case", CASES)
def test_compare_order_bit_exact(golden_dir, case):
    f, c = load(golden_dir, case)
    base = f["base"]
    got = np.array([oracle.dist_avx(base[a], base[b]) for a, b in c["cmp_pairs"]], np.float32)
    assert np.array_equal(got.view(np.uint32), c["cmp_vals"].view(np.uint32))


@pytest.mark.parametrize("case", CASES)
def test_entry_point(golden_dir, case):
    f, c = load(golden_dir, case)
    assert pg.entry_point(f["gt"], f["base"].shape[0]) == int(c["ep"][0])


@pytest.mark.parametrize("case", CASES)
def test_match_sup_fusion_nn_fusion_final(golden_dir, case):
    f, c = load(golden_dir, case)
    base, gt = f["base"], f["gt"]
    rounds = []
    for r in range(1, 7):
        off, ids = oracle.match_sup(base, gt, r)
        ref = rows(c[f"sup{r}_off"], c[f"sup{r}_ids"])
        got = rows(off, ids)
        for i, (a, b) in enumerate(zip(got, ref)):
            assert np.array_equal(np.sort(a), np.sort(b)), f"MatchSup round {r}, base {i}"
        rounds.append((off, ids))
    off, ids = oracle.fusion_nn(base, rounds)
    assert np.array_equal(off, c["fnn_off"]) and np.array_equal(ids, c["fnn_ids"])
    off, ids = oracle.fusion_final(base, f["proj"], (c["fnn_off"], c["fnn_ids"]),
                                   f["link32_graph"])
    assert np.array_equal(off, c["ff_off"]) and np.array_equal(ids, c["ff_ids"])
    deg = np.diff(c["ff_off"].astype(np.int64))
    print(f"{case}: FusionFinal degree mean {deg.mean():.1f} max {deg.max()}, FusionNN max "
          f"{np.diff(c['fnn_off'].astype(np.int64)).max()}")


def test_fusion_final_long_bipartite_lists(golden_dir):
    """Bipartite lists longer than M_final (the reference's unsigned-wrap branch), repeats, the
    node itself and ids past n."""
    f = dict(np.load(os.path.join(golden_dir, "ref_mix_1000x200.npz")))
    w = dict(np.load(os.path.join(golden_dir, "ref_cpu_ffwrap_1000x200.npz")))
    off, ids = oracle.fusion_final(f["base"], f["proj"], (w["bip_off"], w["bip_ids"]),
                                   f["link32_graph"])
    assert np.array_equal(off, w["ff_off"]) and np.array_equal(ids, w["ff_ids"])
    assert np.diff(w["ff_off"].astype(np.int64)).max() > 70


def test_compare_tails_bit_exact(golden_dir):
    """compare()'s 8- and 4-wide tails (tests/test_t2iend.cu:44-64) at D = 4 .. 204."""
    t = dict(np.load(os.path.join(golden_dir, "ref_cpu_compare_tails.npz")))
    for d in (4, 12, 20, 36, 52, 204):
        got = np.array([oracle.dist_avx(a, b) for a, b in zip(t[f"a{d}"], t[f"b{d}"])],
                       np.float32)
        assert np.array_equal(got.view(np.uint32), t[f"v{d}"].view(np.uint32)), f"D={d}"
