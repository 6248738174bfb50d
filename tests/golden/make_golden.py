"""Generates the golden fixtures in tests/golden/ from the reference's own kernel code.

Run in a checkout where the reference tree is present (it is not shipped with this repository):

    oracle/build_ref.sh /path/to/ParaGraph 1000 200
    python tests/golden/make_golden.py

oracle/_ref/libref_harness_1000_200.so holds the reference's thread-per-node kernels
(include/Gbuilder.cuh: match_top1_kernel_v0, init_pr_lists, fusion_prune_reverse_kernel_v0,
fusion_merge_sort_prune_kernel) and its visited set (include/Ghashtable.cuh), compiled with g++
and launched with one thread, so every race resolves in ascending node order.  For each case this
script records the inputs and every stage output the reference produced:

  K0   projection rows (n x 128)                     tests/test_t2iend.cu:976
  K1+K2 phase-1 prune/reverse lists + sorted rows    tests/test_t2iend.cu:987-1001
  K3   phase-1 merge -> projection graph (n x 16)    tests/test_t2iend.cu:1010
  K5-K7 link-round prune/reverse + merge for M=32 (R=94) and the reference's M=55 (R=71),
       fed with a search result (the link rounds' input, tests/test_t2iend.cu:1062-1091)
  hash  new/seen flags of a key sequence with resets (Ghashtable.cuh:39-86)

The search result fed to the link-round kernels comes from the oracle (the reference's search
kernel is warp-synchronous and has no one-thread form); it is an input to those kernels here.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from paragraph_gb300 import datagen  # noqa: E402

N, D = 1000, 200
TOMB = 0xFFFFFFFF


def case_mix():
    base, gt = datagen.make_dataset(N, D, seed=7)
    return base, gt


def case_edge():
    """Hubs (large-norm points: reverse lists overflow R), exact duplicates (equal distances:
    tie order), a zero vector, and tomb-padded ground-truth rows."""
    base, queries = datagen.make_base_queries(N, D, seed=11, centers=16)
    rng = np.random.Generator(np.random.PCG64(99))
    hubs = rng.choice(N, 12, replace=False)
    base[hubs] *= np.float32(3.0)
    dup_src = rng.choice(N, 40, replace=False)
    dup_dst = rng.choice(np.setdiff1d(np.arange(N), np.concatenate([dup_src, hubs])), 40,
                         replace=False)
    base[dup_dst] = base[dup_src]
    base[dup_dst[0]] = 0.0
    gt = datagen.ground_truth(base, queries, 128)
    pad_rows = rng.choice(N, 25, replace=False)
    for i, q in enumerate(pad_rows):
        gt[q, 100 - i * 3:] = TOMB  # suffix padding as transform_gt_to_128.ipynb writes it
    return base, gt


def run_case(ref, base, gt):
    out = {"base": base, "gt": gt}
    k0 = ref.match_top1(gt)
    out["k0"] = k0
    srt, lists = ref.prune("phase1", base, k0)
    out["p1_sorted"] = srt
    rev, rnum, pru, pnum = oracle.split_lists(lists, 111, 15)
    out.update(p1_rev=rev, p1_rnum=rnum, p1_pruned=pru, p1_pnum=pnum)
    proj = ref.merge("phase1", base, lists, 16)
    out["proj"] = proj
    search, _, _, _ = oracle.search(base, proj)
    out["search_in"] = search
    for which, p, r in (("link32", 32, 94), ("link55", 55, 71)):
        srt, lists = ref.prune(which, base, search)
        rev, rnum, pru, pnum = oracle.split_lists(lists, r, p)
        out.update({f"{which}_sorted": srt, f"{which}_rev": rev, f"{which}_rnum": rnum,
                    f"{which}_pruned": pru, f"{which}_pnum": pnum})
        out[f"{which}_graph"] = ref.merge(which, base, lists, p)
    # mask unused list slots so that the fixture holds only what the reference defined
    for key, cnt in (("p1_rev", "p1_rnum"), ("p1_pruned", "p1_pnum"), ("link32_rev", "link32_rnum"),
                     ("link32_pruned", "link32_pnum"), ("link55_rev", "link55_rnum"),
                     ("link55_pruned", "link55_pnum")):
        a = out[key]
        c = np.minimum(out[cnt], a.shape[1])
        a[np.arange(a.shape[1])[None, :] >= c[:, None]] = TOMB
    return out


def hash_case(ref):
    rng = np.random.Generator(np.random.PCG64(5))
    keys = rng.integers(0, 3000, 5000).astype(np.uint32)
    keys[::7] = keys[::7] * 4096 % 100000  # colliding slots (same key & 4095)
    reset = np.zeros(5000, dtype=np.uint8)
    reset[::480] = 1
    return keys, reset, ref.hash_sequence(keys, reset)


def main():
    lib = os.path.join(ROOT, "oracle", "_ref", f"libref_harness_{N}_{D}.so")
    ref = oracle.RefHarness(lib)
    assert (ref.n, ref.d) == (N, D)
    for name, fn in (("mix", case_mix), ("edge", case_edge)):
        base, gt = fn()
        out = run_case(ref, base, gt)
        np.savez_compressed(os.path.join(HERE, f"ref_{name}_{N}x{D}.npz"), **out)
        print(name, {k: v.shape for k, v in out.items()})
    keys, reset, flags = hash_case(ref)
    np.savez_compressed(os.path.join(HERE, "ref_hashtable.npz"), keys=keys, reset=reset,
                        flags=flags)


if __name__ == "__main__":
    main()
