"""Generates the beam-search fixtures in tests/golden/ from the reference's own search kernels.

Run in a checkout where the reference tree is present (it is not shipped with this repository),
on an x86-64 host:

    oracle/build_ref_search.sh /path/to/ParaGraph
    python tests/golden/make_golden_search.py

oracle/_ref/libref_search.so runs include/Gsearcher.cuh's kernels on the CPU under a 32-lane warp
emulator (oracle/ref_warp_emu.h, oracle/ref_search_harness.cpp), one warp per query:

  ref_search_<case>_1000x200.npz   link_process_v0_store_base_data (Gsearcher.cuh:890-1066;
      tests/test_t2iend.cu:1051,1096: Km=32, Kp=2, Kd=16, reset_iter=15, entry points
      (3030517 + i) % n) over the inputs of ref_<case>_1000x200.npz: the projection graph
      (`proj`, degree 16: the round-1 search) and the reference-merged link graphs
      (`link32_graph`, `link55_graph`: the round-2 search).  For each: ids (n x 64, parent bit
      cleared), evaluations and iterations per query.
  ref_qsearch_2000x64.npz   search_shared_hashtable (Gsearcher.cuh:108-296; Km=32, Kp=2, Kd=16,
      reset_iter=4, topk=10) of 300 held-out cross-modal queries over a 2000 x 64 base and a
      degree-32 graph (the oracle's build of that base: an input here).  D is a multiple of 32:
      the kernel's row-staging loop reads a list id once per 32 coordinates, and with D % 32 != 0
      its lanes would run that loop a different number of times.
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
GRAPHS = ("proj", "link32_graph", "link55_graph")


def main():
    ref = oracle.RefSearchHarness(os.path.join(ROOT, "oracle", "_ref", "libref_search.so"))
    assert (ref.n, ref.d) == (N, D)
    for case in ("mix", "edge"):
        f = np.load(os.path.join(HERE, f"ref_{case}_{N}x{D}.npz"))
        out = {}
        for g in GRAPHS:
            ids, ev, it = ref.link_search(f["base"], f[g])
            out[f"{g}_ids"] = ids
            out[f"{g}_evals"] = ev
            out[f"{g}_iters"] = it
        np.savez_compressed(os.path.join(HERE, f"ref_search_{case}_{N}x{D}.npz"), **out)
        print(case, {k: int(v.sum()) for k, v in out.items() if not k.endswith("_ids")})
    s = ref.query_shape
    base, queries = datagen.make_base_queries(s["n"], s["d"], s["n"] + s["nq"], seed=21)
    gt = datagen.ground_truth(base, queries[:s["n"]], 128)
    graph = oracle.build_graph(base, gt, degree=s["degree"], beam=64)["graph"]
    test_q = np.ascontiguousarray(queries[s["n"]:])
    ids, ev, it = ref.query_search(base, graph, test_q)
    np.savez_compressed(os.path.join(HERE, f"ref_qsearch_{s['n']}x{s['d']}.npz"), base=base,
                        graph=graph, queries=test_q, ids=ids, evals=ev, iters=it,
                        topk=np.uint32(s["topk"]), reset_iter=np.uint32(4))
    print("qsearch", s, int(ev.sum()), int(it.sum()))


if __name__ == "__main__":
    main()
