"""Screening error of the 16-bit Gram against FP64, and the bound the screened prune relies on.

The screened prune (paragraph_gb300/csrc/pg_screen.cu) decides an occlusion test from the
16-bit score s^ = sum x^ y^ (x^ = fp16(x) or bf16(x)) only when it lies farther than
    E = |e_x|(|y| + |e_y|) + |x||e_y| + c_acc (|x| + |e_x|)(|y| + |e_y|) + c_seq |x||y|
from the threshold (e = x - x^); otherwise it re-scores with the reference's FP32 chain.
Here the roundings are emulated exactly (round to nearest even), s^ is accumulated in FP64 (the
tensor core's FP32 accumulation error is what c_acc covers), and every pair must satisfy
|s^ - chain| <= E -- for FP16 also when subnormal inputs are flushed, with |e| carrying the norm
of the subnormal part as k_screen_norms computes it.  The measured worst-case relative errors
against FP64 are printed for the record (FP16, BF16, and FP8 E4M3 with a per-vector scale,
which is not built because its error sends most tests to the exact path).
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


def norm_bounds(x: np.ndarray, rnd, min_normal: float):
    """The per-point bounds k_screen_norms writes: (|x|, |x - x^| + |x^_sub|) with the kernel's
    1.0001 factor and 1e-21 underflow term, summed in FP32 as the kernel sums them."""
    x32 = np.ascontiguousarray(x, dtype=np.float32)
    xr = rnd(x32)
    e = x32 - xr
    sub = np.where(np.abs(xr) < min_normal, xr, np.float32(0))
    f = lambda v: np.sqrt((v.astype(np.float32) ** 2).sum(1, dtype=np.float32))
    return (f(x32) * np.float32(1.0001) + np.float32(1e-21),
            (f(e) + f(sub)) * np.float32(1.0001) + np.float32(1e-21))


def test_fp16_bound_holds_when_subnormal_inputs_are_flushed():
    """Points whose FP16 copies have many subnormal coordinates (|x^| < 2^-14): the screened
    score is modelled with those coordinates flushed to zero, as a tensor core that flushes
    subnormal inputs would compute it, and with them kept.  The bound with the subnormal part
    folded into |e| holds either way; without that part it fails under flushing."""
    rng = np.random.default_rng(5)
    n, d = 600, 64
    scale = 10.0 ** rng.uniform(-6, -2, (n, 1))
    x = (rng.standard_normal((n, d)) * scale).astype(np.float32)
    xh = fp16(x)
    assert (np.abs(xh[xh != 0]) < 2.0 ** -14).mean() > 0.2  # many subnormal FP16 values
    flushed = np.where(np.abs(xh) < 2.0 ** -14, 0.0, xh).astype(np.float64)
    kept = xh.astype(np.float64)
    nrm, err = norm_bounds(x, fp16, 2.0 ** -14)
    nrm = nrm.astype(np.float64)
    err = err.astype(np.float64)
    err_plain = np.sqrt(((x.astype(np.float64) - kept) ** 2).sum(1)) * 1.0001
    dp = (d + 15) // 16 * 16
    c_acc = (dp + 32) * 2.0 ** -21
    c_seq = (d + 2) * 2.0 ** -23
    i, j = rng.integers(0, n, (2, 4000))
    chain = np.array([-float(oracle.dist_seq(x, int(a), int(b))) for a, b in zip(i, j)])

    def bound(e):
        return (e[i] * (nrm[j] + e[j]) + nrm[i] * e[j]
                + c_acc * (nrm[i] + e[i]) * (nrm[j] + e[j]) + c_seq * nrm[i] * nrm[j] + 1e-30)

    for g in (flushed, kept):
        shat = (g[i] * g[j]).sum(1)
        assert (np.abs(shat - chain) <= bound(err)).all()
    # the subnormal term is what makes the flushed case hold
    shat = (flushed[i] * flushed[j]).sum(1)
    assert (np.abs(shat - chain) > bound(err_plain)).any()
