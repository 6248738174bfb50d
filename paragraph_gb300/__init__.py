"""paragraph_gb300 -- GB300 (sm_103a) builder for ParaGraph / RoarGraph cross-modal graph indexes.

Python mirror of the C ABI in include/paragraph_gb300.h (libparagraph_gb300.so, built in-tree by
paragraph_gb300/build.py).  The compute path is the CUDA library only: if it cannot be loaded the
calls raise; there is no CPU fallback.

    from paragraph_gb300 import Builder
    b = Builder(base, gt)              # numpy float32 n x d, uint32 q x 128
    graph = b.LaunchBuild()            # n x M uint32, tomb (0xFFFFFFFF) padded
    b.SaveGraph("index.bin")           # the reference's SaveGraph layout

Stage functions (match_top1, prune_reverse, merge_prune, search) mirror the reference kernels of
include/Gbuilder.cuh and include/Gsearcher.cuh and take torch CUDA tensors.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TOMB = 0xFFFFFFFF

PG_OK, PG_EINVAL, PG_ECUDA, PG_ENOMEM, PG_ETIMEOUT, PG_EUNSUPPORTED, PG_EIO = range(7)
SCREEN_NONE, SCREEN_BF16, SCREEN_FP8, SCREEN_FP16 = 0, 1, 2, 3
FLAG_VALIDATE_INPUT = 1
FLAG_CUDA_GRAPH = 2

_ERRNAMES = {1: "PG_EINVAL", 2: "PG_ECUDA", 3: "PG_ENOMEM", 4: "PG_ETIMEOUT",
             5: "PG_EUNSUPPORTED", 6: "PG_EIO"}


class PGError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_ERRNAMES.get(code, code)}: {msg}")
        self.code = code


class Params(ctypes.Structure):
    _fields_ = [(f, ctypes.c_uint32) for f in (
        "gt_k", "proj_degree", "proj_pruned", "proj_reverse", "degree", "link_reverse",
        "link_rounds", "km", "kp", "kd", "reset_iter", "seed_base", "max_search_iters",
        "screen", "flags")] + [("reserved", ctypes.c_uint32 * 5)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


class Stats(ctypes.Structure):
    _fields_ = [("evals_total", ctypes.c_uint64), ("evals_proj_prune", ctypes.c_uint64),
                ("evals_proj_merge", ctypes.c_uint64), ("evals_search", ctypes.c_uint64 * 4),
                ("evals_prune", ctypes.c_uint64 * 4), ("evals_merge", ctypes.c_uint64 * 4),
                ("search_iters", ctypes.c_uint64 * 4), ("rescored", ctypes.c_uint64 * 4),
                ("ms_total", ctypes.c_float), ("ms_proj", ctypes.c_float),
                ("ms_search", ctypes.c_float * 4), ("ms_prune", ctypes.c_float * 4),
                ("ms_merge", ctypes.c_float * 4), ("ms_h2d", ctypes.c_float),
                ("ms_d2h", ctypes.c_float), ("h2d_bytes", ctypes.c_uint64),
                ("d2h_bytes", ctypes.c_uint64), ("ep", ctypes.c_uint32),
                ("ms_match_sup", ctypes.c_float), ("ms_fusion_nn", ctypes.c_float),
                ("ms_fusion_final", ctypes.c_float), ("reserved", ctypes.c_uint32 * 4)]

    def as_dict(self):
        out = {}
        for f, _ in self._fields_:
            if f == "reserved":
                continue
            v = getattr(self, f)
            out[f] = list(v) if hasattr(v, "__len__") else v
        return out


class Tuning(ctypes.Structure):
    """pg_tuning: launch shapes of a handle (results do not depend on them)."""
    _fields_ = [("search_rows", ctypes.c_uint32), ("search_warps_per_sm", ctypes.c_uint32),
                ("hash_factor", ctypes.c_uint32), ("screen_stages", ctypes.c_uint32),
                ("beam", ctypes.c_uint32), ("recall", ctypes.c_float),
                ("ms_build", ctypes.c_float), ("ms_default", ctypes.c_float),
                ("reserved", ctypes.c_uint32 * 8)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


_LIB = None
_VP = ctypes.c_void_p
_U64 = ctypes.c_uint64
_U32 = ctypes.c_uint32
_U64P = ctypes.POINTER(ctypes.c_uint64)
_U32P = ctypes.POINTER(ctypes.c_uint32)

# exported symbol -> (restype, argtypes)
SIGNATURES = {
    "pg_last_error": (ctypes.c_char_p, []),
    "pg_abi_version": (_U32, []),
    "pg_params_default": (ctypes.c_int, [ctypes.POINTER(Params), _U32, _U32]),
    "pg_create": (ctypes.c_int, [ctypes.POINTER(_VP), ctypes.c_int, _VP]),
    "pg_destroy": (ctypes.c_int, [_VP]),
    "pg_workspace_bytes": (ctypes.c_int, [ctypes.POINTER(Params), _U64, _U32, _U64, _U64P]),
    "pg_build_host": (ctypes.c_int, [_VP, ctypes.POINTER(Params), _VP, _U64, _U32, _VP, _U64,
                                     _VP, _VP, ctypes.POINTER(Stats)]),
    "pg_build_device": (ctypes.c_int, [_VP, ctypes.POINTER(Params), _VP, _U64, _U32, _VP, _U64,
                                       _VP, _VP, ctypes.POINTER(Stats)]),
    "pg_build_batched_device": (ctypes.c_int, [_VP, ctypes.POINTER(Params), _VP, _U32, _VP, _VP,
                                               _VP, _U32, _VP, _VP, ctypes.POINTER(Stats)]),
    "pg_match_top1": (ctypes.c_int, [_VP, _VP, _U64, _U32, _U64, _VP]),
    "pg_prune_reverse": (ctypes.c_int, [_VP, _VP, _U64, _U32, _VP, _U32, _U32, _U32, ctypes.c_int,
                                        _VP, _VP, _VP, _VP, _VP, _U64P]),
    "pg_merge_prune": (ctypes.c_int, [_VP, _VP, _U64, _U32, _VP, _VP, _U32, _VP, _VP, _U32, _U32,
                                      ctypes.c_int, _VP, _U64P]),
    "pg_search": (ctypes.c_int, [_VP, _VP, _U64, _U32, _VP, _U32, _U32, _U32, _U32, _U32, _U32,
                                 _U32, _VP, _U64P, _U64P]),
    "pg_prune_reverse_noalloc": (ctypes.c_int, [_VP, _VP, _U64, _U32, _VP, _U32, _U32, _U32,
                                                ctypes.c_int, _VP, _VP, _VP, _VP, _U64P]),
    "pg_query_search": (ctypes.c_int, [_VP, _VP, _U64, _U32, _VP, _U32, _VP, _U64, _U32, _U32,
                                       _U32, _U32, _U32, _U32, _U32, _VP, _U64P, _U64P]),
    "pg_match_sup": (ctypes.c_int, [_VP, _VP, _U64, _U32, _VP, _U64, _U32, _U32, _U32, _VP, _VP]),
    "pg_fusion_nn": (ctypes.c_int, [_VP, _VP, _U64, _U32, _U32, _VP, _VP, _U32, _VP, _VP]),
    "pg_fusion_final": (ctypes.c_int, [_VP, _VP, _U64, _U32, _VP, _VP, _VP, _U32, _VP, _U32, _VP,
                                       _U32, _U32, _U32, _VP, _VP]),
    "pg_build_index": (ctypes.c_int, [_VP, ctypes.POINTER(Params), _VP, _U64, _U32, _VP, _U64,
                                      _U32, _U32, _U32, _U32, _VP, _VP, ctypes.POINTER(Stats)]),
    "pg_build_index_host": (ctypes.c_int, [_VP, ctypes.POINTER(Params), _VP, _U64, _U32, _VP,
                                           _U64, _U32, _U32, _U32, _U32, _VP, _VP,
                                           ctypes.POINTER(Stats)]),
    "pg_ground_truth": (ctypes.c_int, [_VP, _VP, _U64, _U32, _VP, _U64, _U32, _VP]),
    "pg_screen_scores": (ctypes.c_int, [_VP, _VP, _U64, _VP, _U64, _U32, _VP]),
    "pg_set_tuning": (ctypes.c_int, [_VP, ctypes.POINTER(Tuning)]),
    "pg_get_tuning": (ctypes.c_int, [_VP, ctypes.POINTER(Tuning)]),
    "pg_autotune": (ctypes.c_int, [_VP, ctypes.POINTER(Params), _VP, _U32, _VP, _VP, _VP, _U32,
                                   _VP, ctypes.c_float, ctypes.POINTER(Tuning)]),
    "pg_read_file": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, _VP, _U64, _U32P, _U32P]),
    "pg_save_graph": (ctypes.c_int, [ctypes.c_char_p, _VP, _U64, _U32, _U32]),
    "pg_entry_point": (ctypes.c_int, [_VP, _U64, _U32, _U64, _U32P]),
}


def library_path() -> str:
    return os.path.join(HERE, "_lib", "libparagraph_gb300.so")


def lib(build_if_stale: bool = True):
    """Load libparagraph_gb300.so (compiling it first when nvcc is available and it is stale)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if build_if_stale:
        from . import build as _build
        try:
            path = _build.build()
        except RuntimeError as e:  # no nvcc: use an existing library or fail below
            if not os.path.exists(path):
                raise RuntimeError(f"libparagraph_gb300.so is missing and cannot be built: {e}")
    if not os.path.exists(path):
        raise RuntimeError(f"libparagraph_gb300.so not found at {path}; run "
                           "`python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = L
    return L


def _check(rc: int):
    if rc != PG_OK:
        raise PGError(rc, lib().pg_last_error().decode())


def default_params(degree: int = 32, beam: int = 64, **over) -> Params:
    """(M, L) -> the reference driver's constants (tests/test_t2iend.cu:671-727)."""
    p = Params()
    _check(lib().pg_params_default(ctypes.byref(p), degree, beam))
    for k, v in over.items():
        setattr(p, k, v)
    return p


def _ptr(t) -> int:
    """Device pointer of a torch tensor (or an int address)."""
    if isinstance(t, int):
        return t
    if t is None:
        return 0
    return t.data_ptr()


class Handle:
    """pg_handle: device workspace + stream.  `stream` is a torch.cuda.Stream, a raw
    cudaStream_t address, or None for torch's current stream."""

    def __init__(self, device: int = 0, stream=None):
        if stream is None:
            import torch
            stream = torch.cuda.current_stream(device)
        raw = stream if isinstance(stream, int) else getattr(stream, "cuda_stream", 0)
        self._h = _VP()
        _check(lib().pg_create(ctypes.byref(self._h), device, _VP(raw)))
        self.device = device

    def close(self):
        if self._h:
            lib().pg_destroy(self._h)
            self._h = _VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- whole build
    def build_host(self, base: np.ndarray, gt: np.ndarray, params: Params | None = None,
                   want_proj: bool = True):
        params = params or default_params()
        base = np.ascontiguousarray(base, dtype=np.float32)
        gt = np.ascontiguousarray(gt, dtype=np.uint32)
        n, d = base.shape
        q = gt.shape[0]
        graph = np.empty((n, params.degree), dtype=np.uint32)
        proj = np.empty((n, params.proj_degree), dtype=np.uint32) if want_proj else None
        st = Stats()
        _check(lib().pg_build_host(self._h, ctypes.byref(params), base.ctypes.data, n, d,
                                   gt.ctypes.data, q, graph.ctypes.data,
                                   proj.ctypes.data if proj is not None else None,
                                   ctypes.byref(st)))
        return graph, proj, st

    def build_host_ptr(self, base_ptr: int, n: int, d: int, gt_ptr: int, q: int, graph_ptr: int,
                       proj_ptr: int | None, params: Params) -> Stats:
        """pg_build_host on raw host addresses (pinned buffers owned by the caller)."""
        st = Stats()
        _check(lib().pg_build_host(self._h, ctypes.byref(params), base_ptr, n, d, gt_ptr, q,
                                   graph_ptr, proj_ptr, ctypes.byref(st)))
        return st

    def build_device(self, base, gt, graph, proj=None, params: Params | None = None) -> Stats:
        params = params or default_params()
        n, d = base.shape
        st = Stats()
        _check(lib().pg_build_device(self._h, ctypes.byref(params), _ptr(base), n, d, _ptr(gt),
                                     gt.shape[0], _ptr(graph), _ptr(proj), ctypes.byref(st)))
        return st

    def build_batched(self, base, gt, node_off, query_off, graph, proj=None,
                      params: Params | None = None) -> Stats:
        """pg_build_batched_device: base/gt/graph/proj are concatenated device tensors, the
        offsets host sequences (count + 1 entries)."""
        params = params or default_params()
        no = np.ascontiguousarray(node_off, dtype=np.uint64)
        qo = np.ascontiguousarray(query_off, dtype=np.uint64)
        st = Stats()
        _check(lib().pg_build_batched_device(self._h, ctypes.byref(params), _ptr(base),
                                             base.shape[1], _ptr(gt), no.ctypes.data,
                                             qo.ctypes.data, len(no) - 1, _ptr(graph), _ptr(proj),
                                             ctypes.byref(st)))
        return st

    # ---- stages (reference kernels)
    def match_top1(self, gt, n: int, out):
        """match_top1_kernel_v0 (Gbuilder.cuh:104-135)."""
        _check(lib().pg_match_top1(self._h, _ptr(gt), gt.shape[0], gt.shape[1], n, _ptr(out)))

    def prune_reverse(self, base, graph, pruned, pruned_num, reverse, reverse_num, strict: bool,
                      sorted_rows=None) -> int:
        """init_pr_lists + fusion_prune_reverse_kernel_v0 (Gbuilder.cuh:1066-1244)."""
        n, d = base.shape
        ev = ctypes.c_uint64(0)
        _check(lib().pg_prune_reverse(self._h, _ptr(base), n, d, _ptr(graph), graph.shape[1],
                                      pruned.shape[1], reverse.shape[1], int(strict),
                                      _ptr(pruned), _ptr(pruned_num), _ptr(reverse),
                                      _ptr(reverse_num), _ptr(sorted_rows), ctypes.byref(ev)))
        return int(ev.value)

    def merge_prune(self, base, pruned, pruned_num, reverse, reverse_num, out, strict: bool) -> int:
        """fusion_merge_sort_prune_kernel (Gbuilder.cuh:1467-1601)."""
        n, d = base.shape
        ev = ctypes.c_uint64(0)
        _check(lib().pg_merge_prune(self._h, _ptr(base), n, d, _ptr(pruned), _ptr(pruned_num),
                                    pruned.shape[1], _ptr(reverse), _ptr(reverse_num),
                                    reverse.shape[1], out.shape[1], int(strict), _ptr(out),
                                    ctypes.byref(ev)))
        return int(ev.value)

    def search(self, base, graph, out, km: int = 32, kp: int = 2, kd: int = 16,
               reset_iter: int = 15, seed_base: int = 3030517, max_iters: int = 1 << 20):
        """link_process_v0_store_base_data (Gsearcher.cuh:890-1066).  Returns (evals, iters)."""
        n, d = base.shape
        ev = ctypes.c_uint64(0)
        it = ctypes.c_uint64(0)
        _check(lib().pg_search(self._h, _ptr(base), n, d, _ptr(graph), graph.shape[1], km, kp, kd,
                               reset_iter, seed_base, max_iters, _ptr(out), ctypes.byref(ev),
                               ctypes.byref(it)))
        return int(ev.value), int(it.value)


    # ---- CPU RoarGraph path and final fusion (tests/test_t2iend.cu:365-613) on the GPU
    def match_sup(self, base, gt, topn: int, out, cnt, m_nn: int = 40):
        """pg_match_sup: MatchSup round `topn`; out n x m_nn, cnt n (device tensors)."""
        n, d = base.shape
        _check(lib().pg_match_sup(self._h, _ptr(base), n, d, _ptr(gt), gt.shape[0], gt.shape[1],
                                  topn, m_nn, _ptr(out), _ptr(cnt)))

    def fusion_nn(self, base, sup, sup_cnt, out, cnt, m_nn: int = 40):
        """pg_fusion_nn over rounds x n x m_nn lists (sup) and rounds x n counts."""
        n, d = base.shape
        _check(lib().pg_fusion_nn(self._h, _ptr(base), n, d, sup.shape[0], _ptr(sup),
                                  _ptr(sup_cnt), m_nn, _ptr(out), _ptr(cnt)))

    def fusion_final(self, base, supply, link, out, cnt, bip_off=None, bip_ids=None,
                     bip_rows=None, bip_cnt=None, m_final: int = 70):
        """pg_fusion_final; bipartite lists as CSR (bip_off, bip_ids) or rows (bip_rows,
        bip_cnt); out n x stride, cnt n."""
        n, d = base.shape
        if bip_off is not None:
            ids, stride = bip_ids, 0
        else:
            ids, stride = bip_rows, bip_rows.shape[1]
        _check(lib().pg_fusion_final(self._h, _ptr(base), n, d, _ptr(bip_off), _ptr(ids),
                                     _ptr(bip_cnt), stride, _ptr(supply), supply.shape[1],
                                     _ptr(link), link.shape[1], m_final, out.shape[1], _ptr(out),
                                     _ptr(cnt)))

    def build_index(self, base, gt, out, cnt, params: Params | None = None,
                    match_rounds: int = 6, m_nn: int = 40, m_final: int = 70) -> Stats:
        """pg_build_index: the reference driver's whole index (GPU build + MatchSup rounds +
        FusionNN + FusionFinal); out n x stride (>= 2*m_nn + m_final), cnt n."""
        params = params or default_params()
        n, d = base.shape
        st = Stats()
        _check(lib().pg_build_index(self._h, ctypes.byref(params), _ptr(base), n, d, _ptr(gt),
                                    gt.shape[0], match_rounds, m_nn, m_final, out.shape[1],
                                    _ptr(out), _ptr(cnt), ctypes.byref(st)))
        return st

    def build_index_host(self, base: np.ndarray, gt: np.ndarray, params: Params | None = None,
                         match_rounds: int = 6, m_nn: int = 40, m_final: int = 70):
        """pg_build_index_host: the whole index from host arrays.  Returns (rows n x
        (2*m_nn + m_final) tomb padded, counts n, Stats)."""
        params = params or default_params()
        base = np.ascontiguousarray(base, dtype=np.float32)
        gt = np.ascontiguousarray(gt, dtype=np.uint32)
        n, d = base.shape
        stride = 2 * m_nn + m_final
        out = np.empty((n, stride), dtype=np.uint32)
        cnt = np.empty(n, dtype=np.uint32)
        st = Stats()
        _check(lib().pg_build_index_host(self._h, ctypes.byref(params), base.ctypes.data, n, d,
                                         gt.ctypes.data, gt.shape[0], match_rounds, m_nn,
                                         m_final, stride, out.ctypes.data, cnt.ctypes.data,
                                         ctypes.byref(st)))
        out[np.arange(stride)[None, :] >= cnt[:, None].astype(np.int64)] = TOMB
        return out, cnt, st

    def ground_truth(self, base, queries, out):
        """pg_ground_truth: exact inner-product top-k (k = out.shape[1]) of every query."""
        n, d = base.shape
        _check(lib().pg_ground_truth(self._h, _ptr(base), n, d, _ptr(queries), queries.shape[0],
                                     out.shape[1], _ptr(out)))

    def screen_scores(self, a, b, out):
        """pg_screen_scores: out (len(a) x len(b)) = fp16(a) . fp16(b)^T, FP32 accumulation."""
        _check(lib().pg_screen_scores(self._h, _ptr(a), a.shape[0], _ptr(b), b.shape[0],
                                      a.shape[1], _ptr(out)))

    def set_tuning(self, tuning: Tuning):
        _check(lib().pg_set_tuning(self._h, ctypes.byref(tuning)))

    def get_tuning(self) -> Tuning:
        t = Tuning()
        _check(lib().pg_get_tuning(self._h, ctypes.byref(t)))
        return t

    def autotune(self, base, gt, params: Params | None = None, node_off=None, query_off=None,
                 queries=None, target_recall: float = 0.0) -> tuple[Params, Tuning]:
        """pg_autotune over device tensors (one index, or a batched table).  Returns the params
        (km updated when a recall target picked the beam) and the tuning now set on the handle."""
        params = params or default_params()
        p = Params.from_buffer_copy(params)
        if node_off is None:
            node_off, query_off = [0, base.shape[0]], [0, gt.shape[0]]
        no = np.ascontiguousarray(node_off, dtype=np.uint64)
        qo = np.ascontiguousarray(query_off, dtype=np.uint64)
        t = Tuning()
        _check(lib().pg_autotune(self._h, ctypes.byref(p), _ptr(base), base.shape[1], _ptr(gt),
                                 no.ctypes.data, qo.ctypes.data, len(no) - 1, _ptr(queries),
                                 float(target_recall), ctypes.byref(t)))
        return p, t

    def query_search(self, base, graph, queries, out, km: int = 32, kp: int = 2, kd: int = 16,
                     reset_iter: int = 4, seed_base: int = 3030517, max_iters: int = 1 << 20):
        """search_shared_hashtable (Gsearcher.cuh:108-296): top out.shape[1] ids per query."""
        n, d = base.shape
        ev = ctypes.c_uint64(0)
        it = ctypes.c_uint64(0)
        _check(lib().pg_query_search(self._h, _ptr(base), n, d, _ptr(graph), graph.shape[1],
                                     _ptr(queries), queries.shape[0], km, kp, kd, reset_iter,
                                     seed_base, max_iters, out.shape[1], _ptr(out),
                                     ctypes.byref(ev), ctypes.byref(it)))
        return int(ev.value), int(it.value)


# ---------------------------------------------------------------- file formats
def read_vectors(path: str, dtype, shape=None, headered: bool = False) -> np.ndarray:
    """read_vec_from_file (include/utils.hpp:17-35) for headerless files (give `shape`), or the
    Big-ANN [u32 n][u32 d] layout with headered=True."""
    dtype = np.dtype(dtype)
    rows = ctypes.c_uint32(0)
    cols = ctypes.c_uint32(0)
    if headered:
        _check(lib(False).pg_read_file(path.encode(), 1, None, 0, ctypes.byref(rows),
                                       ctypes.byref(cols)))
        shape = (rows.value, cols.value)
    out = np.empty(shape, dtype=dtype)
    _check(lib(False).pg_read_file(path.encode(), int(headered), out.ctypes.data, out.nbytes,
                                   ctypes.byref(rows), ctypes.byref(cols)))
    return out


def save_graph(path: str, graph: np.ndarray, ep: int):
    """SaveGraph (tests/test_t2iend.cu:615-633)."""
    graph = np.ascontiguousarray(graph, dtype=np.uint32)
    _check(lib(False).pg_save_graph(path.encode(), graph.ctypes.data, graph.shape[0],
                                    graph.shape[1], ep))


def load_graph(path: str):
    """Reads a SaveGraph file back: (ep, list of id arrays)."""
    raw = np.fromfile(path, dtype=np.uint32)
    ep, n = int(raw[0]), int(raw[1])
    rows, o = [], 2
    for _ in range(n):
        k = int(raw[o])
        rows.append(raw[o + 1:o + 1 + k].copy())
        o += 1 + k
    return ep, rows


def entry_point(gt: np.ndarray, n: int) -> int:
    """ep of MatchNN (tests/test_t2iend.cu:188-221)."""
    gt = np.ascontiguousarray(gt, dtype=np.uint32)
    ep = ctypes.c_uint32(0)
    _check(lib(False).pg_entry_point(gt.ctypes.data, gt.shape[0], gt.shape[1], n,
                                     ctypes.byref(ep)))
    return int(ep.value)


# ---------------------------------------------------------------- reference-shaped facade
class Builder:
    """Gbuilder::Builder<float> (include/Builder.hpp:15-35): Builder(base, gt), SetGt, LaunchBuild.

    LaunchBuild runs the K0..K11 pipeline and returns the n x degree graph; the projection,
    statistics and entry point are kept on the object.  grid/block arguments of the reference's
    template are accepted and ignored (launch shapes are chosen by the library)."""

    def __init__(self, base: np.ndarray, gt_ids: np.ndarray, degree: int = 32, beam: int = 64,
                 device: int = 0, **params):
        self.base_ = np.ascontiguousarray(base, dtype=np.float32)
        self.gt_ids_ = np.ascontiguousarray(gt_ids, dtype=np.uint32)
        self.params = default_params(degree, beam, **params)
        self.device = device
        self.graph = None
        self.projection = None
        self.index = None
        self.stats = None
        self.ep = None

    def SetGt(self, gt_ids: np.ndarray):
        self.gt_ids_ = np.ascontiguousarray(gt_ids, dtype=np.uint32)

    def LaunchBuild(self, grid_size: int | None = None, block_size: int | None = None,
                    gt_num: int | None = None, dim: int | None = None) -> np.ndarray:
        if gt_num is not None and gt_num != self.gt_ids_.shape[1]:
            raise PGError(PG_EINVAL, f"gt_num={gt_num} but gt has {self.gt_ids_.shape[1]} columns")
        if dim is not None and dim != self.base_.shape[1]:
            raise PGError(PG_EINVAL, f"dim={dim} but base has {self.base_.shape[1]} columns")
        with Handle(self.device, stream=0) as h:
            self.graph, self.projection, self.stats = h.build_host(self.base_, self.gt_ids_,
                                                                   self.params)
        self.index = None
        self.ep = entry_point(self.gt_ids_, self.base_.shape[0])
        return self.graph

    def LaunchIndex(self, match_rounds: int = 6, m_nn: int = 40, m_final: int = 70) -> np.ndarray:
        """The reference driver's whole index (tests/test_t2iend.cu:974-1258): the build, then
        MatchSup rounds, FusionNN and FusionFinal; returns the tomb-padded index rows, which
        SaveGraph then writes (the file the driver saves)."""
        with Handle(self.device, stream=0) as h:
            self.index, _, self.stats = h.build_index_host(self.base_, self.gt_ids_, self.params,
                                                           match_rounds, m_nn, m_final)
        self.ep = entry_point(self.gt_ids_, self.base_.shape[0])
        return self.index

    def SaveGraph(self, path: str):
        """SaveGraph (tests/test_t2iend.cu:615-633): the FusionFinal index after LaunchIndex, else
        the graph of LaunchBuild."""
        rows = self.index if self.index is not None else self.graph
        if rows is None:
            raise PGError(PG_EINVAL, "neither LaunchBuild nor LaunchIndex has run")
        save_graph(path, rows, self.ep)
