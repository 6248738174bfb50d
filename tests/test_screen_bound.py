"""Screening error of the BF16 Gram against FP64, and the bound the screened prune relies on.

The screened prune (paragraph_gb300/csrc/pg_screen.cu) decides an occlusion test from the BF16
score s^ = sum bf16(x) bf16(y) only when it lies farther than
    E = |e_x|(|y| + |e_y|) + |x||e_y| + c_acc (|x| + |e_x|)(|y| + |e_y|) + c_seq |x||y|
from the threshold (e = x - bf16(x)); otherwise it re-scores with the reference's FP32 chain.
Here BF16 rounding is emulated exactly (round to nearest even), s^ is accumulated in FP64 (the
tensor core's FP32 accumulation error is what c_acc covers), and every pair must satisfy
|s^ - chain| <= E.  The measured worst-case relative errors against FP64 are printed for the
record (BF16, and FP8 E4M3 with a per-vector scale, which is not built because its error sends
most tests to the exact path).
"""
import os

import numpy as np

import oracle


def bf16(x: np.ndarray) -> np.ndarray:
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def e4m3(x: np.ndarray) -> np.ndarray:
    """Round to FP8 E4M3 (3 mantissa bits, max 448, subnormals below 2^-6), per-vector scaled."""
    scale = np.abs(x).max(axis=1, keepdims=True) / 448.0
    y = x / scale
    ay = np.abs(y)
    exp = np.floor(np.log2(np.maximum(ay, 2.0 ** -9)))
    exp = np.maximum(exp, -6)
    step = 2.0 ** (exp - 3)
    q = np.sign(y) * np.round(ay / step) * step
    return (np.clip(q, -448, 448) * scale).astype(np.float64)


def fp16(x: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(x, dtype=np.float32).astype(np.float16).astype(np.float32)


def test_fp16_screen_bound_holds(golden_dir):
    """The same bound with FP16 rounding (the PG_SCREEN_FP16 path): e = x - fp16(x)."""
    f = np.load(os.path.join(golden_dir, "ref_edge_1000x200.npz"))
    x = f["base"].astype(np.float32)
    n, d = x.shape
    rng = np.random.default_rng(1)
    pairs = rng.integers(0, n, (6000, 2))
    xh = fp16(x).astype(np.float64)
    x64 = x.astype(np.float64)
    err = x64 - xh
    nrm = np.sqrt((x64 ** 2).sum(1)) * 1.0001
    enrm = np.sqrt((err ** 2).sum(1)) * 1.0001
    dp = (d + 15) // 16 * 16
    c_acc = (dp + 32) * 2.0 ** -21
    c_seq = (d + 2) * 2.0 ** -23
    i, j = pairs[:, 0], pairs[:, 1]
    s64 = (x64[i] * x64[j]).sum(1)
    shat = (xh[i] * xh[j]).sum(1)
    chain = np.array([-float(oracle.dist_seq(x, int(a), int(b))) for a, b in pairs])
    bound = (enrm[i] * (nrm[j] + enrm[j]) + nrm[i] * enrm[j]
             + c_acc * (nrm[i] + enrm[i]) * (nrm[j] + enrm[j]) + c_seq * nrm[i] * nrm[j])
    assert (np.abs(shat - chain) <= bound).all()
    nz = (nrm[i] > 0) & (nrm[j] > 0)
    rel = np.abs(shat - s64)[nz] / (nrm[i] * nrm[j])[nz]
    print(f"max |s-s64|/(|x||y|): fp16 {rel.max():.3e}")
    assert rel.max() < 2.0 ** -10


def test_bf16_screen_bound_holds_and_error_is_stated(golden_dir):
    f = np.load(os.path.join(golden_dir, "ref_edge_1000x200.npz"))  # includes hubs, duplicates
    x = f["base"].astype(np.float32)
    n, d = x.shape
    rng = np.random.default_rng(0)
    pairs = rng.integers(0, n, (6000, 2))
    xb = bf16(x).astype(np.float64)
    x64 = x.astype(np.float64)
    err = x64 - xb
    nrm = np.sqrt((x64 ** 2).sum(1)) * 1.0001
    enrm = np.sqrt((err ** 2).sum(1)) * 1.0001
    dp = (d + 15) // 16 * 16
    c_acc = (dp + 32) * 2.0 ** -21
    c_seq = (d + 2) * 2.0 ** -23
    i, j = pairs[:, 0], pairs[:, 1]
    s64 = (x64[i] * x64[j]).sum(1)
    shat = (xb[i] * xb[j]).sum(1)
    chain = np.array([-float(oracle.dist_seq(x, int(a), int(b))) for a, b in pairs])
    bound = (enrm[i] * (nrm[j] + enrm[j]) + nrm[i] * enrm[j]
             + c_acc * (nrm[i] + enrm[i]) * (nrm[j] + enrm[j]) + c_seq * nrm[i] * nrm[j])
    assert (np.abs(shat - chain) <= bound).all()
    nz = (nrm[i] > 0) & (nrm[j] > 0)  # the fixture holds a zero vector
    i, j, s64, shat, chain, bound = i[nz], j[nz], s64[nz], shat[nz], chain[nz], bound[nz]
    rel_bf16 = np.abs(shat - s64) / (nrm[i] * nrm[j])
    rel_chain = np.abs(chain - s64) / (nrm[i] * nrm[j])
    x8 = e4m3(np.where(nrm[:, None] > 0, x64, 1.0))
    s8 = (x8[i] * x8[j]).sum(1)
    rel_fp8 = np.abs(s8 - s64) / (nrm[i] * nrm[j])
    print(f"max |s-s64|/(|x||y|): bf16 {rel_bf16.max():.3e}  fp8-e4m3 {rel_fp8.max():.3e}  "
          f"fp32 chain {rel_chain.max():.3e}; mean bound/(|x||y|) "
          f"{(bound / (nrm[i] * nrm[j])).mean():.3e}")
    assert rel_bf16.max() < 2.0 ** -7          # the worst case for two BF16 roundings
    assert rel_chain.max() < (d + 2) * 2.0 ** -23
    assert rel_fp8.max() > 4 * rel_bf16.max()   # why FP8 screening is not built
