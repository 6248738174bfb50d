"""Generates tests/golden/ref_cpu_<case>_1000x200.npz from the reference's own CPU RoarGraph code.

Run where the reference tree is present, on an x86-64 host with AVX-512:

    oracle/build_ref_cpu.sh /path/to/ParaGraph
    python tests/golden/make_golden_cpu.py

oracle/_ref/libref_cpu.so holds the reference's compare, MatchNN, MatchSup, FusionNN and
FusionFinal (tests/test_t2iend.cu:31-613) run with one OpenMP thread.  For the two cases of
make_golden.py (same base and ground truth) this records:

  ep          MatchNN's entry point                                   :179-221
  sup<r>      MatchSup round r = 1..6 (M_nn = 40), CSR                :365-488, driver :912-921
  fnn         FusionNN over the six rounds (M_nn = 40), CSR           :490-537, driver :938-940
  ff          FusionFinal(M_supply = 16, M_link = 32, M_final = 70)   :539-613, driver :1226-1229
              of the case's projection and M=32 link graph, CSR
  cmp         compare() on 2000 seeded pairs                          :31-80

and ref_cpu_ffwrap_1000x200.npz: FusionFinal alone on crafted bipartite lists (see run_wrap);
ref_cpu_compare_tails.npz: compare() at dimensions that reach its 8- and 4-wide tails.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIB = os.path.join(ROOT, "oracle", "_ref", "libref_cpu.so")
ROUNDS = 6
M_NN = 40

VP, U32, U64 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64


def load():
    L = ctypes.CDLL(LIB)
    L.ref_cpu_compare.argtypes = [VP, VP, U32]
    L.ref_cpu_compare.restype = ctypes.c_float
    L.ref_cpu_match_nn_ep.argtypes = [U32, U32, VP, VP, U32]
    L.ref_cpu_match_nn_ep.restype = U32
    L.ref_cpu_match_sup.argtypes = [U32, U32, U32, U32, U32, VP, VP, U32, VP, VP, U64]
    L.ref_cpu_match_sup.restype = ctypes.c_longlong
    L.ref_cpu_fusion_nn.argtypes = [U32, U32, VP, U32, U32, VP, VP, VP, VP, VP, U64]
    L.ref_cpu_fusion_nn.restype = ctypes.c_longlong
    L.ref_cpu_fusion_final.argtypes = [U32, U32, U32, U32, VP, U32, VP, VP, VP, VP, VP, VP, U64]
    L.ref_cpu_fusion_final.restype = ctypes.c_longlong
    return L


def run_case(L, name: str):
    f = np.load(os.path.join(HERE, f"ref_{name}_1000x200.npz"))
    base = np.ascontiguousarray(f["base"], dtype=np.float32)
    gt = np.ascontiguousarray(f["gt"], dtype=np.uint32)
    proj = np.ascontiguousarray(f["proj"], dtype=np.uint32)
    link = np.ascontiguousarray(f["link32_graph"], dtype=np.uint32)
    n, d = base.shape
    q = gt.shape[0]
    out = {}
    out["ep"] = np.array([L.ref_cpu_match_nn_ep(n, q, gt.ctypes.data, base.ctypes.data, d)],
                         dtype=np.uint32)
    offs, idss = [], []
    for r in range(1, ROUNDS + 1):
        off = np.zeros(n + 1, np.uint64)
        ids = np.zeros(n * 128, np.uint32)
        k = L.ref_cpu_match_sup(n, q, r, gt.shape[1], M_NN, gt.ctypes.data, base.ctypes.data, d,
                                off.ctypes.data, ids.ctypes.data, ids.size)
        assert k >= 0
        out[f"sup{r}_off"], out[f"sup{r}_ids"] = off, ids[:k].copy()
        offs.append(off)
        idss.append(ids[:k].copy())
    sup_off = np.ascontiguousarray(np.concatenate(offs))
    sup_ids = np.ascontiguousarray(np.concatenate(idss))
    sup_base = np.ascontiguousarray(np.cumsum([0] + [len(i) for i in idss])[:-1], dtype=np.uint64)
    off = np.zeros(n + 1, np.uint64)
    ids = np.zeros(n * 2 * M_NN, np.uint32)
    k = L.ref_cpu_fusion_nn(n, M_NN, base.ctypes.data, d, ROUNDS, sup_off.ctypes.data,
                            sup_ids.ctypes.data, sup_base.ctypes.data, off.ctypes.data,
                            ids.ctypes.data, ids.size)
    assert k >= 0
    out["fnn_off"], out["fnn_ids"] = off, ids[:k].copy()
    fnn_off, fnn_ids = off, np.ascontiguousarray(ids[:k])
    off = np.zeros(n + 1, np.uint64)
    ids = np.zeros(n * (2 * M_NN + 70), np.uint32)
    k = L.ref_cpu_fusion_final(n, proj.shape[1], link.shape[1], 70, base.ctypes.data, d,
                               proj.ctypes.data, fnn_off.ctypes.data, fnn_ids.ctypes.data,
                               link.ctypes.data, off.ctypes.data, ids.ctypes.data, ids.size)
    assert k >= 0
    out["ff_off"], out["ff_ids"] = off, ids[:k].copy()
    rng = np.random.default_rng(5)
    pairs = rng.integers(0, n, (2000, 2)).astype(np.uint32)
    vals = np.array([L.ref_cpu_compare(base[a].ctypes.data, base[b].ctypes.data, d)
                     for a, b in pairs], dtype=np.float32)
    out["cmp_pairs"], out["cmp_vals"] = pairs, vals
    path = os.path.join(HERE, f"ref_cpu_{name}_1000x200.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, {k: v.shape for k, v in out.items() if k.endswith("ids")})


def run_wrap(L):
    """FusionFinal alone on crafted bipartite lists of 0..90 ids (repeats, the node itself, ids
    past n): lists longer than M_final = 70 take the reference's unsigned-wrap branch."""
    f = np.load(os.path.join(HERE, "ref_mix_1000x200.npz"))
    base = np.ascontiguousarray(f["base"], dtype=np.float32)
    proj = np.ascontiguousarray(f["proj"], dtype=np.uint32)
    link = np.ascontiguousarray(f["link32_graph"], dtype=np.uint32)
    n, d = base.shape
    rng = np.random.default_rng(17)
    lens = rng.integers(0, 91, n)
    lens[:50] = rng.integers(71, 91, 50)
    lists = []
    for i, k in enumerate(lens):
        row = rng.integers(0, n + 20, k).astype(np.uint32)  # ids >= n are skipped
        if k > 3:
            row[1] = row[0]  # a repeat
            row[2] = i  # the node itself
        lists.append(row)
    b_off = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    b_ids = np.ascontiguousarray(np.concatenate(lists), dtype=np.uint32)
    off = np.zeros(n + 1, np.uint64)
    ids = np.zeros(n * (90 + 70), np.uint32)
    k = L.ref_cpu_fusion_final(n, proj.shape[1], link.shape[1], 70, base.ctypes.data, d,
                               proj.ctypes.data, b_off.ctypes.data, b_ids.ctypes.data,
                               link.ctypes.data, off.ctypes.data, ids.ctypes.data, ids.size)
    assert k >= 0
    path = os.path.join(HERE, "ref_cpu_ffwrap_1000x200.npz")
    np.savez_compressed(path, bip_off=b_off, bip_ids=b_ids, ff_off=off, ff_ids=ids[:k].copy())
    print("wrote", path)


def run_compare_tails(L):
    """compare() at dimensions that reach its 8-wide and 4-wide tails (:44-64): D = 4, 12, 20, 36,
    52, 204 on seeded vectors."""
    rng = np.random.default_rng(23)
    out = {}
    for d in (4, 12, 20, 36, 52, 204):
        a = rng.standard_normal((300, d)).astype(np.float32) * 3
        b = rng.standard_normal((300, d)).astype(np.float32)
        out[f"a{d}"], out[f"b{d}"] = a, b
        out[f"v{d}"] = np.array([L.ref_cpu_compare(a[i].ctypes.data, b[i].ctypes.data, d)
                                 for i in range(300)], dtype=np.float32)
    path = os.path.join(HERE, "ref_cpu_compare_tails.npz")
    np.savez_compressed(path, **out)
    print("wrote", path)


def main():
    if not os.path.exists(LIB):
        sys.exit(f"{LIB} is missing: run oracle/build_ref_cpu.sh first")
    L = load()
    for name in ("mix", "edge"):
        run_case(L, name)
    run_wrap(L)
    run_compare_tails(L)


if __name__ == "__main__":
    main()
