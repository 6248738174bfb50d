"""Seeded synthetic inputs with the shapes of ParaGraph's datasets (T2I / LAION / WebVid).

The reference builds from a base set and each training query's top-128 ground-truth base ids
(tests/test_t2iend.cu:735-760; the queries themselves are never read).  Those datasets are not
available here, so this module draws:

* base: N x D float32 from a mixture of ``centers`` isotropic Gaussians (centres ~ N(0, 1),
  sigma 0.3, uniform component choice);
* training queries (a different modality): q = 0.6 * R @ c + g + N(0, 0.2^2), with c a random
  centre, R a seeded Haar-random orthogonal matrix and g a fixed shift of norm 2;
* ground truth: exact float32 inner-product top-k base ids per query, ties to the lower id.

``cosine=True`` L2-normalises base and queries after generation (cosine == inner product).
Small sizes run on numpy; ``device="cuda"`` runs the same recipe on the GPU with torch for
million-point sets (the top-k there uses float32 matmul with TF32 disabled).
"""
from __future__ import annotations

import numpy as np


def _haar(rng: np.random.Generator, d: int) -> np.ndarray:
    a = rng.standard_normal((d, d))
    qm, r = np.linalg.qr(a)
    qm *= np.sign(np.diag(r))[None, :]
    return qm.astype(np.float32)


def make_base_queries(n: int, d: int, q: int | None = None, centers: int = 64, sigma: float = 0.3,
                      query_scale: float = 0.6, shift_norm: float = 2.0, noise: float = 0.2,
                      cosine: bool = False, seed: int = 1234):
    q = n if q is None else q
    rng = np.random.Generator(np.random.PCG64(seed))
    cent = rng.standard_normal((centers, d)).astype(np.float32)
    comp = rng.integers(0, centers, n)
    base = cent[comp] + np.float32(sigma) * rng.standard_normal((n, d)).astype(np.float32)
    rot = _haar(rng, d)
    g = rng.standard_normal(d).astype(np.float32)
    g *= np.float32(shift_norm) / np.linalg.norm(g)
    qcomp = rng.integers(0, centers, q)
    queries = (np.float32(query_scale) * (cent[qcomp] @ rot.T) + g[None, :]
               + np.float32(noise) * rng.standard_normal((q, d)).astype(np.float32))
    base = base.astype(np.float32)
    queries = queries.astype(np.float32)
    if cosine:
        base /= np.linalg.norm(base, axis=1, keepdims=True)
        queries /= np.linalg.norm(queries, axis=1, keepdims=True)
    return np.ascontiguousarray(base), np.ascontiguousarray(queries)


def ground_truth(base: np.ndarray, queries: np.ndarray, k: int = 128, chunk: int = 2048):
    """Exact float32 inner-product top-k ids, best first, ties to the lower id."""
    n = base.shape[0]
    k = min(k, n)
    out = np.empty((queries.shape[0], k), dtype=np.uint32)
    bt = np.ascontiguousarray(base.T)
    for s in range(0, queries.shape[0], chunk):
        sc = queries[s:s + chunk] @ bt  # float32
        part = np.argpartition(-sc, k - 1, axis=1)[:, :k]
        # resolve the k-th boundary exactly: take every id scoring >= the k-th best
        kth = np.take_along_axis(sc, part, axis=1).min(axis=1, keepdims=True)
        for i in range(sc.shape[0]):
            cand = np.nonzero(sc[i] >= kth[i])[0]
            order = np.lexsort((cand, -sc[i, cand]))
            out[s + i] = cand[order[:k]]
    return out


def make_dataset(n: int, d: int, q: int | None = None, gt_k: int = 128, seed: int = 1234, **kw):
    base, queries = make_base_queries(n, d, q, seed=seed, **kw)
    gt = ground_truth(base, queries, gt_k)
    return base, gt


def make_dataset_cuda(n: int, d: int, q: int | None = None, gt_k: int = 128, centers: int = 64,
                      sigma: float = 0.3, query_scale: float = 0.6, shift_norm: float = 2.0,
                      noise: float = 0.2, cosine: bool = False, seed: int = 1234,
                      chunk: int = 4096, device: str = "cuda", return_queries: bool = False,
                      with_gt: bool = True):
    """The same recipe on the GPU with torch (for N in the millions).  Returns device tensors
    (base float32 N x D, gt int32 viewed as uint32 Q x gt_k[, queries float32 Q x D])."""
    import torch

    q = n if q is None else q
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    f32 = torch.float32
    cent = torch.randn((centers, d), generator=gen, device=device, dtype=f32)
    comp = torch.randint(0, centers, (n,), generator=gen, device=device)
    base = cent[comp] + sigma * torch.randn((n, d), generator=gen, device=device, dtype=f32)
    # the D x D rotation is built on the host (numpy QR): small, and independent of the GPU's
    # linear-algebra libraries
    rot = torch.from_numpy(_haar(np.random.Generator(np.random.PCG64(seed + 1)), d)).to(device)
    g = torch.randn((d,), generator=gen, device=device, dtype=f32)
    g = g * (shift_norm / g.norm())
    qcomp = torch.randint(0, centers, (q,), generator=gen, device=device)
    queries = (query_scale * (cent[qcomp] @ rot.T) + g[None, :]
               + noise * torch.randn((q, d), generator=gen, device=device, dtype=f32))
    del qcomp, comp
    if cosine:
        base = base / base.norm(dim=1, keepdim=True)
        queries = queries / queries.norm(dim=1, keepdim=True)
    if not with_gt:  # the caller computes the ground truth (e.g. pg_ground_truth)
        return base.contiguous(), None, queries.contiguous()
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        gt = torch.empty((q, gt_k), dtype=torch.int32, device=device)
        bt = base.T.contiguous()
        for s in range(0, q, chunk):
            sc = queries[s:s + chunk] @ bt
            vals, idx = torch.topk(sc, gt_k, dim=1, largest=True, sorted=True)
            gt[s:s + chunk] = idx.to(torch.int32)
            del sc, vals, idx
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    if return_queries:
        return base.contiguous(), gt, queries.contiguous()
    del queries
    return base.contiguous(), gt
