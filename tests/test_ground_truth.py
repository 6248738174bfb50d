"""Exact inner-product top-k ground truth (pg_ground_truth): the oracle's definition (FP64
inner products, ties to the lower id) checked against numpy on the CPU, and the GPU's FP16
tensor-core screening + FP64 re-scoring checked against the oracle id for id."""
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
             ("k_past_n", 100, 32, 20, 128, False, False)]


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
