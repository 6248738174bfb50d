"""Exact inner-product top-k ground truth (pg_ground_truth): the oracle's definition (FP64
inner products, ties to the lower id) checked against numpy on the CPU, and the GPU's FP16
tensor-core screening (a tcgen05 GEMM with a selecting epilogue) + FP64 re-scoring checked
against the oracle id for id -- over sizes that leave partial 128-row tiles, group sizes of the
threshold pass from 1 to 16 rows, dimensions that end inside a 64-element TMA box (36, 200) --
and the screening product
alone checked against exact products within its FP32 accumulation bound."""
import numpy as np
import pytest

import oracle
from paragraph_gb300 import datagen


def numpy_truth(base, queries, k):
    s = queries.astype(np.float64) @ base.astype(np.float64).T
    out = np.empty((len(queries), k), np.uint32)
    ids = np.arange(base.shape[0])
    for i in range(len(queries)):
        order = np.lexsort((ids, -s[i]))
        out[i, :min(k, len(order))] = order[:k]
        out[i, len(order):] = 0xFFFFFFFF
    return out


def test_oracle_definition():
    base, q = datagen.make_base_queries(3000, 40, 50, seed=9)
    a = oracle.ground_truth(base, q, 20)
    b = numpy_truth(base, q, 20)
    # FP64 sums in two orders may differ in the last bit: allow swaps of exact near-ties only
    s = q.astype(np.float64) @ base.astype(np.float64).T
    for i in range(len(q)):
        if not np.array_equal(a[i], b[i]):
            assert np.allclose(s[i, a[i]], s[i, b[i]], rtol=1e-12, atol=0)


GPU_CASES = [("ip", 20000, 200, 400, 128, False, False),
             ("cosine", 20000, 200, 300, 128, True, False),
             ("duplicates", 8000, 64, 200, 64, False, True),
             ("k_past_n", 100, 32, 20, 128, False, False),
             ("groups_of_8", 70000, 200, 300, 128, False, False),
             ("d512", 9000, 512, 300, 128, True, False),
             ("d36_k256", 5000, 36, 257, 256, False, False)]


@pytest.mark.gpu
@pytest.mark.parametrize("name,n,d,nq,k,cos,dup", GPU_CASES)
def test_gpu_ground_truth_equals_oracle(name, n, d, nq, k, cos, dup):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import paragraph_gb300 as pg
    base, q = datagen.make_base_queries(n, d, nq, seed=31, cosine=cos)
    if dup:  # exact duplicate rows: equal FP64 scores, the lower id first
        base[1::7] = base[0::7][:len(base[1::7])]
    ref = oracle.ground_truth(base, q, k)
    out = torch.full((nq, k), -1, dtype=torch.int32, device="cuda")
    with pg.Handle(0) as h:
        h.ground_truth(torch.from_numpy(base).cuda(), torch.from_numpy(q).cuda(), out)
    got = out.cpu().numpy().view(np.uint32)
    assert np.array_equal(got, ref), f"{(got != ref).any(axis=1).sum()} of {nq} rows differ"


SCORE_CASES = [(300, 1000, 200), (128, 128, 64), (257, 391, 512), (1, 5, 4), (700, 300, 36)]


@pytest.mark.gpu
@pytest.mark.parametrize("na,nb,d", SCORE_CASES)
def test_gpu_screen_scores_within_fp32_accumulation_bound(na, nb, d):
    """pg_screen_scores (the tcgen05 screening GEMM of pg_ground_truth, FP16 operands, FP32
    accumulation in TMEM) against the exact FP64 products of the same FP16-rounded operands:
    every score within the accumulation bound (d' * 2^-22) * sum |a_i b_i|, d' = d padded to a
    multiple of 16, plus 16."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import paragraph_gb300 as pg
    g = torch.Generator(device="cuda")
    g.manual_seed(na * 7 + nb)
    a = torch.randn((na, d), generator=g, device="cuda")
    b = torch.randn((nb, d), generator=g, device="cuda")
    out = torch.full((na, nb), float("nan"), device="cuda")
    with pg.Handle(0) as h:
        h.screen_scores(a, b, out)
    ah, bh = a.half().double(), b.half().double()
    exact = ah @ bh.T
    mag = ah.abs() @ bh.abs().T
    dp = (d + 15) // 16 * 16
    bound = (dp + 16) * 2.0 ** -22 * mag + 1e-30
    err = (out.double() - exact).abs()
    assert torch.isfinite(out).all()
    assert (err <= bound).all(), f"max err/bound {float((err / bound).max()):.3f}"
