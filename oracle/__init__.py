"""CPU oracle for the ParaGraph GPU build path -- TEST INFRASTRUCTURE ONLY.

The restatement lives in ``pg_oracle.c`` (built to ``_build/libpg_oracle.so`` by
``build_oracle.sh``).  Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU legs
import this module; the ``paragraph_gb300`` package never does.

``RefHarness`` wraps ``_ref/libref_harness_<N>_<D>.so``: the reference's own thread-per-node
kernels (include/Gbuilder.cuh) compiled with g++ and run on one CPU thread.  ``RefSearchHarness``
wraps ``_ref/libref_search.so``: the reference's warp-per-query beam searches
(include/Gsearcher.cuh) under a 32-lane warp emulator.  Both exist only where the reference tree
was available at build time and are used to make the golden fixtures.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TOMB = 0xFFFFFFFF

_u32p = ctypes.POINTER(ctypes.c_uint32)
_f32p = ctypes.POINTER(ctypes.c_float)
_u64p = ctypes.POINTER(ctypes.c_uint64)


def build(force: bool = False) -> str:
    lib = os.path.join(HERE, "_build", "libpg_oracle.so")
    srcs = [os.path.join(HERE, f) for f in ("pg_oracle.c", "pg_oracle_roar.c")]
    if force or not os.path.exists(lib) or any(os.path.getmtime(lib) < os.path.getmtime(s)
                                               for s in srcs):
        subprocess.check_call([os.path.join(HERE, "build_oracle.sh")], stdout=subprocess.DEVNULL)
    return lib


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        L = ctypes.CDLL(build())
        L.pgo_match_top1.argtypes = [_u32p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64, _u32p]
        L.pgo_match_top1.restype = None
        L.pgo_prune_reverse.argtypes = [_f32p, ctypes.c_uint64, ctypes.c_uint32, _u32p,
                                        ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                        ctypes.c_int, _u32p, _u32p, _u32p, _u32p, _u32p]
        L.pgo_prune_reverse.restype = ctypes.c_uint64
        L.pgo_merge_prune.argtypes = [_f32p, ctypes.c_uint64, ctypes.c_uint32, _u32p, _u32p,
                                      ctypes.c_uint32, _u32p, _u32p, ctypes.c_uint32,
                                      ctypes.c_uint32, ctypes.c_int, _u32p]
        L.pgo_merge_prune.restype = ctypes.c_uint64
        L.pgo_search.argtypes = [_f32p, ctypes.c_uint64, ctypes.c_uint32, _u32p, ctypes.c_uint32,
                                 ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                 ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64,
                                 ctypes.c_uint64, ctypes.c_uint64, _u32p, _u64p, _u32p]
        L.pgo_search.restype = ctypes.c_uint64
        L.pgo_query_search.argtypes = [_f32p, ctypes.c_uint64, ctypes.c_uint32, _u32p,
                                       ctypes.c_uint32, _f32p, ctypes.c_uint64, ctypes.c_uint32,
                                       ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                       ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint32, _u32p,
                                       _u64p]
        L.pgo_query_search.restype = ctypes.c_uint64
        L.pgo_dist_seq.argtypes = [_f32p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32]
        L.pgo_dist_seq.restype = ctypes.c_float
        L.pgo_dist_lane.argtypes = [_f32p, _f32p, ctypes.c_uint64]
        L.pgo_dist_lane.restype = ctypes.c_float
        L.pgo_build.argtypes = [ctypes.c_void_p, _f32p, ctypes.c_uint64, ctypes.c_uint32, _u32p,
                                ctypes.c_uint64, _u32p, _u32p, _u32p, ctypes.c_void_p]
        L.pgo_build.restype = ctypes.c_int
        L.pgo_num_threads.restype = ctypes.c_int
        L.pgo_dist_avx.argtypes = [_f32p, _f32p, ctypes.c_uint64]
        L.pgo_dist_avx.restype = ctypes.c_float
        L.pgo_match_sup.argtypes = [_f32p, ctypes.c_uint64, ctypes.c_uint32, _u32p,
                                    ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32,
                                    ctypes.c_uint32, _u64p, _u32p, ctypes.c_uint64]
        L.pgo_match_sup.restype = ctypes.c_longlong
        L.pgo_fusion_nn.argtypes = [_f32p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32,
                                    ctypes.c_uint32, _u64p, _u32p, _u64p, _u64p, _u32p,
                                    ctypes.c_uint64]
        L.pgo_fusion_nn.restype = ctypes.c_longlong
        L.pgo_fusion_final.argtypes = [_f32p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32,
                                       ctypes.c_uint32, ctypes.c_uint32, _u32p, _u64p, _u32p,
                                       _u32p, _u64p, _u32p, ctypes.c_uint64]
        L.pgo_fusion_final.restype = ctypes.c_longlong
        L.pgo_ground_truth.argtypes = [_f32p, ctypes.c_uint64, ctypes.c_uint32, _f32p,
                                       ctypes.c_uint64, ctypes.c_uint32, _u32p]
        L.pgo_ground_truth.restype = None
        _LIB = L
    return _LIB


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(t)


def _u32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint32)


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def num_threads() -> int:
    return int(lib().pgo_num_threads())


def dist_seq(base, x: int, y: int) -> np.float32:
    base = _f32(base)
    return np.float32(lib().pgo_dist_seq(_p(base, _f32p), base.shape[1], x, y))


def dist_lane(q, x) -> np.float32:
    q = _f32(q)
    x = _f32(x)
    return np.float32(lib().pgo_dist_lane(_p(q, _f32p), _p(x, _f32p), q.shape[0]))


def match_top1(gt, n: int) -> np.ndarray:
    gt = _u32(gt)
    q, k = gt.shape
    out = np.empty((n, k), dtype=np.uint32)
    lib().pgo_match_top1(_p(gt, _u32p), q, k, n, _p(out, _u32p))
    return out


@dataclass
class PruneResult:
    pruned: np.ndarray       # n x P (valid up to pruned_num)
    pruned_num: np.ndarray   # n
    reverse: np.ndarray      # n x R (valid up to reverse_num)
    reverse_num: np.ndarray  # n (clamped to R)
    sorted_rows: np.ndarray  # n x C, rows after the in-place sort
    evals: int


def prune_reverse(base, graph, p: int, r: int, strict: bool) -> PruneResult:
    base = _f32(base)
    graph = _u32(graph)
    n, d = base.shape
    c = graph.shape[1]
    pruned = np.full((n, p), TOMB, dtype=np.uint32)
    pnum = np.zeros(n, dtype=np.uint32)
    rev = np.full((n, r), TOMB, dtype=np.uint32)
    rnum = np.zeros(n, dtype=np.uint32)
    srt = np.empty((n, c), dtype=np.uint32)
    ev = lib().pgo_prune_reverse(_p(base, _f32p), n, d, _p(graph, _u32p), c, p, r, int(strict),
                                 _p(pruned, _u32p), _p(pnum, _u32p), _p(rev, _u32p),
                                 _p(rnum, _u32p), _p(srt, _u32p))
    return PruneResult(pruned, pnum, rev, rnum, srt, int(ev))


def merge_prune(base, pr: PruneResult, deg: int, strict: bool):
    base = _f32(base)
    n, d = base.shape
    out = np.empty((n, deg), dtype=np.uint32)
    p = pr.pruned.shape[1]
    r = pr.reverse.shape[1]
    ev = lib().pgo_merge_prune(_p(base, _f32p), n, d, _p(_u32(pr.pruned), _u32p),
                               _p(_u32(pr.pruned_num), _u32p), p, _p(_u32(pr.reverse), _u32p),
                               _p(_u32(pr.reverse_num), _u32p), r, deg, int(strict),
                               _p(out, _u32p))
    return out, int(ev)


def search(base, graph, km: int = 32, kp: int = 2, kd: int = 16, reset_iter: int = 15,
           seed_base: int = 3030517, max_iters: int = 1 << 20, q_begin: int = 0,
           q_end: int | None = None):
    """Returns (ids n x L, evals, iterations, cap_hit)."""
    base = _f32(base)
    graph = _u32(graph)
    n, d = base.shape
    q_end = n if q_end is None else q_end
    L = km + kp * kd
    out = np.empty((q_end - q_begin, L), dtype=np.uint32)
    it = ctypes.c_uint64(0)
    hit = ctypes.c_uint32(0)
    ev = lib().pgo_search(_p(base, _f32p), n, d, _p(graph, _u32p), graph.shape[1], km, kp, kd,
                          reset_iter, seed_base, max_iters, q_begin, q_end, _p(out, _u32p),
                          ctypes.byref(it), ctypes.byref(hit))
    return out, int(ev), int(it.value), bool(hit.value)


def query_search(base, graph, queries, topk: int = 10, km: int = 32, kp: int = 2, kd: int = 16,
                 reset_iter: int = 4, seed_base: int = 3030517, max_iters: int = 1 << 20):
    """search_shared_hashtable (Gsearcher.cuh:108-296) with external queries: (ids nq x topk,
    evals, iterations)."""
    base = _f32(base)
    graph = _u32(graph)
    queries = _f32(queries)
    n, d = base.shape
    out = np.empty((queries.shape[0], topk), dtype=np.uint32)
    it = ctypes.c_uint64(0)
    ev = lib().pgo_query_search(_p(base, _f32p), n, d, _p(graph, _u32p), graph.shape[1],
                                _p(queries, _f32p), queries.shape[0], km, kp, kd, reset_iter,
                                seed_base, max_iters, topk, _p(out, _u32p), ctypes.byref(it))
    return out, int(ev), int(it.value)


class _Params(ctypes.Structure):
    _fields_ = [(f, ctypes.c_uint32) for f in (
        "gt_k", "proj_degree", "proj_pruned", "proj_reverse", "degree", "link_reverse",
        "link_rounds", "km", "kp", "kd", "reset_iter", "seed_base")] + [("max_iters", ctypes.c_uint64)]


class _Stats(ctypes.Structure):
    _fields_ = [("evals_proj_prune", ctypes.c_uint64), ("evals_proj_merge", ctypes.c_uint64),
                ("evals_search", ctypes.c_uint64 * 4), ("evals_prune", ctypes.c_uint64 * 4),
                ("evals_merge", ctypes.c_uint64 * 4), ("iters_search", ctypes.c_uint64 * 4),
                ("evals_total", ctypes.c_uint64), ("cap_hit", ctypes.c_uint32)]


def default_params(degree: int = 32, beam: int = 64) -> dict:
    """Parameter mapping of the ParaGraph driver (tests/test_t2iend.cu:671-727) onto (M, L):
    link-round pruned length = final degree = M, reverse length = 128 - 2 - M, Km = L - Kp*Kd."""
    kp, kd = 2, 16
    return dict(gt_k=128, proj_degree=16, proj_pruned=15, proj_reverse=111, degree=degree,
                link_reverse=128 - 2 - degree, link_rounds=2, km=beam - kp * kd, kp=kp, kd=kd,
                reset_iter=15, seed_base=3030517, max_iters=1 << 20)


def build_graph(base, gt, **params):
    """Full K0..K11 pipeline.  Returns dict(proj, graph, search, stats)."""
    P = default_params(params.pop("degree", 32), params.pop("beam", 64))
    P.update(params)
    base = _f32(base)
    gt = _u32(gt)
    n, d = base.shape
    q = gt.shape[0]
    assert gt.shape[1] == P["gt_k"]
    L = P["km"] + P["kp"] * P["kd"]
    proj = np.empty((n, P["proj_degree"]), dtype=np.uint32)
    graph = np.empty((n, P["degree"]), dtype=np.uint32)
    srch = np.empty((n, L), dtype=np.uint32)
    prm = _Params(**P)
    st = _Stats()
    rc = lib().pgo_build(ctypes.byref(prm), _p(base, _f32p), n, d, _p(gt, _u32p), q,
                         _p(proj, _u32p), _p(graph, _u32p), _p(srch, _u32p), ctypes.byref(st))
    if rc != 0:
        raise MemoryError("oracle build failed")
    stats = dict(evals_proj_prune=st.evals_proj_prune, evals_proj_merge=st.evals_proj_merge,
                 evals_search=list(st.evals_search), evals_prune=list(st.evals_prune),
                 evals_merge=list(st.evals_merge), iters_search=list(st.iters_search),
                 evals_total=st.evals_total, cap_hit=bool(st.cap_hit))
    return dict(proj=proj, graph=graph, search=srch, stats=stats)


class RefHarness:
    """The reference's own thread-per-node kernels, compiled with g++ (see ref_harness.cpp)."""

    def __init__(self, path: str):
        L = ctypes.CDLL(path)
        for f in ("ref_prune_phase1", "ref_prune_link32", "ref_prune_link55"):
            getattr(L, f).argtypes = [_f32p, _u32p, _u32p]
        for f in ("ref_merge_phase1", "ref_merge_link32", "ref_merge_link55"):
            getattr(L, f).argtypes = [_f32p, _u32p, _u32p]
        L.ref_match_top1.argtypes = [_u32p, _u32p]
        L.ref_n.restype = ctypes.c_uint32
        L.ref_d.restype = ctypes.c_uint32
        L.ref_hash_sequence.argtypes = [_u32p, ctypes.POINTER(ctypes.c_uint8), ctypes.c_uint32,
                                        ctypes.POINTER(ctypes.c_uint8)]
        self.L = L
        self.n = int(L.ref_n())
        self.d = int(L.ref_d())

    def match_top1(self, gt):
        gt = _u32(gt)
        out = np.empty((self.n, 128), dtype=np.uint32)
        self.L.ref_match_top1(_p(gt, _u32p), _p(out, _u32p))
        return out

    def prune(self, which: str, base, graph):
        """Returns (sorted graph, lists n x 128) after init_pr_lists + prune/reverse."""
        base = _f32(base)
        g = _u32(graph).copy()
        lists = np.zeros((self.n, 128), dtype=np.uint32)
        getattr(self.L, "ref_prune_" + which)(_p(base, _f32p), _p(g, _u32p), _p(lists, _u32p))
        return g, lists

    def merge(self, which: str, base, lists, deg: int):
        base = _f32(base)
        lists = _u32(lists).copy()
        out = np.empty((self.n, deg), dtype=np.uint32)
        getattr(self.L, "ref_merge_" + which)(_p(base, _f32p), _p(lists, _u32p), _p(out, _u32p))
        return out

    def hash_sequence(self, keys, reset_before):
        keys = _u32(keys)
        rb = np.ascontiguousarray(reset_before, dtype=np.uint8)
        out = np.zeros(len(keys), dtype=np.uint8)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        self.L.ref_hash_sequence(_p(keys, _u32p), rb.ctypes.data_as(u8p), len(keys),
                                 out.ctypes.data_as(u8p))
        return out


class RefSearchHarness:
    """The reference's own beam-search kernels under a 32-lane warp emulator (see
    ref_search_harness.cpp): link_process_v0_store_base_data (Gsearcher.cuh:890-1066) at the
    compiled size n x d, and search_shared_hashtable (Gsearcher.cuh:108-296) at its own compiled
    shape."""

    def __init__(self, path: str):
        L = ctypes.CDLL(path)
        L.ref_search_n.restype = ctypes.c_uint32
        L.ref_search_d.restype = ctypes.c_uint32
        L.ref_search_error.restype = ctypes.c_char_p
        L.ref_link_search.argtypes = [ctypes.c_uint32, _f32p, _u32p, _u32p, _u64p, _u64p]
        L.ref_query_shape.argtypes = [_u32p]
        L.ref_query_search.argtypes = [_f32p, _u32p, _f32p, _u32p, _u64p, _u64p]
        self.L = L
        self.n = int(L.ref_search_n())
        self.d = int(L.ref_search_d())
        shape = np.zeros(5, dtype=np.uint32)
        L.ref_query_shape(_p(shape, _u32p))
        self.query_shape = dict(zip(("n", "d", "nq", "degree", "topk"), map(int, shape)))

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(f"reference search failed ({rc}): "
                               f"{self.L.ref_search_error().decode()}")

    def link_search(self, base, graph):
        """Returns (ids n x 64, evals per query, iterations per query)."""
        base = _f32(base)
        graph = _u32(graph)
        assert base.shape == (self.n, self.d) and graph.shape[0] == self.n
        out = np.empty((self.n, 64), dtype=np.uint32)
        ev = np.zeros(self.n, dtype=np.uint64)
        it = np.zeros(self.n, dtype=np.uint64)
        self._check(self.L.ref_link_search(graph.shape[1], _p(base, _f32p), _p(graph, _u32p),
                                           _p(out, _u32p), _p(ev, _u64p), _p(it, _u64p)))
        return out, ev, it

    def query_search(self, base, graph, queries):
        """Returns (ids nq x topk, evals per query, iterations per query)."""
        s = self.query_shape
        base = _f32(base)
        graph = _u32(graph)
        queries = _f32(queries)
        assert base.shape == (s["n"], s["d"]) and graph.shape == (s["n"], s["degree"])
        assert queries.shape == (s["nq"], s["d"])
        out = np.empty((s["nq"], s["topk"]), dtype=np.uint32)
        ev = np.zeros(s["nq"], dtype=np.uint64)
        it = np.zeros(s["nq"], dtype=np.uint64)
        self._check(self.L.ref_query_search(_p(base, _f32p), _p(graph, _u32p),
                                            _p(queries, _f32p), _p(out, _u32p), _p(ev, _u64p),
                                            _p(it, _u64p)))
        return out, ev, it


def split_lists(lists: np.ndarray, r: int, p: int):
    """Split pr_neighbor_list records {rev_num, rev[R], pruned_num, pruned[P]}
    (Gbuilder.cuh:1009-1018) into (rev, rev_num, pruned, pruned_num)."""
    rev_num = lists[:, 0].copy()
    rev = lists[:, 1:1 + r].copy()
    pruned_num = lists[:, 1 + r].copy()
    pruned = lists[:, 2 + r:2 + r + p].copy()
    return rev, rev_num, pruned, pruned_num


# ---------------------------------------------------------------- CPU RoarGraph path (CSR graphs)
def dist_avx(a, b) -> np.float32:
    """compare (tests/test_t2iend.cu:31-80) in its AVX-512 FP32 order."""
    a = _f32(a)
    b = _f32(b)
    return np.float32(lib().pgo_dist_avx(_p(a, _f32p), _p(b, _f32p), a.shape[0]))


def _csr_out(cap: int, n: int):
    return np.zeros(n + 1, dtype=np.uint64), np.zeros(max(cap, 1), dtype=np.uint32)


def match_sup(base, gt, topn: int, m_nn: int = 40):
    """MatchSup (tests/test_t2iend.cu:365-488) round `topn`: CSR (off, ids)."""
    base = _f32(base)
    gt = _u32(gt)
    n, d = base.shape
    off, ids = _csr_out(n * 128, n)
    k = lib().pgo_match_sup(_p(base, _f32p), n, d, _p(gt, _u32p), gt.shape[0], gt.shape[1], topn,
                            m_nn, _p(off, _u64p), _p(ids, _u32p), ids.shape[0])
    assert k >= 0
    return off, ids[:k].copy()


def fusion_nn(base, rounds, m_nn: int = 40):
    """FusionNN (tests/test_t2iend.cu:490-537) over supply graphs [(off, ids), ...]: CSR."""
    base = _f32(base)
    n, d = base.shape
    sup_off = np.ascontiguousarray(np.concatenate([o for o, _ in rounds]), dtype=np.uint64)
    sup_ids = _u32(np.concatenate([i for _, i in rounds]) if rounds else np.zeros(1, np.uint32))
    sup_base = np.ascontiguousarray(np.cumsum([0] + [len(i) for _, i in rounds])[:-1],
                                    dtype=np.uint64)
    off, ids = _csr_out(n * 2 * m_nn, n)
    k = lib().pgo_fusion_nn(_p(base, _f32p), n, d, m_nn, len(rounds), _p(sup_off, _u64p),
                            _p(sup_ids, _u32p), _p(sup_base, _u64p), _p(off, _u64p),
                            _p(ids, _u32p), ids.shape[0])
    assert k >= 0
    return off, ids[:k].copy()


def fusion_final(base, supply, bip, link, m_final: int = 70):
    """FusionFinal (tests/test_t2iend.cu:539-613): supply n x m_supply (projection), bip CSR
    (FusionNN graph), link n x m_link (GPU graph): CSR."""
    base = _f32(base)
    supply = _u32(supply)
    link = _u32(link)
    n, d = base.shape
    b_off = np.ascontiguousarray(bip[0], dtype=np.uint64)
    b_ids = _u32(bip[1] if len(bip[1]) else np.zeros(1, np.uint32))
    bmax = int(np.diff(b_off).max()) if n else 0
    off, ids = _csr_out(n * (bmax + m_final), n)
    k = lib().pgo_fusion_final(_p(base, _f32p), n, d, supply.shape[1], link.shape[1], m_final,
                               _p(supply, _u32p), _p(b_off, _u64p), _p(b_ids, _u32p),
                               _p(link, _u32p), _p(off, _u64p), _p(ids, _u32p), ids.shape[0])
    assert k >= 0
    return off, ids[:k].copy()


def ground_truth(base, queries, k: int = 128) -> np.ndarray:
    """Exact inner-product top-k: FP64 sequential dot products, ties to the lower id."""
    base = _f32(base)
    queries = _f32(queries)
    out = np.empty((queries.shape[0], k), dtype=np.uint32)
    lib().pgo_ground_truth(_p(base, _f32p), base.shape[0], base.shape[1], _p(queries, _f32p),
                           queries.shape[0], k, _p(out, _u32p))
    return out
