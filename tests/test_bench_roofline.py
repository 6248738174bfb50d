"""The roofline arithmetic that bench.py reports beside its headline (CPU only): the algorithmic
bytes of a search launch follow the stated formula, `frac` and `dram_frac` are those bytes and the
measured DRAM bytes over the launch time and the peak, and `bound` follows the DRAM fraction."""
import types

import pytest

import bench


def _stats(evals, iters, ms):
    return types.SimpleNamespace(evals_search=list(evals), search_iters=list(iters),
                                 ms_search=list(ms))


def _args(n=1_000_000, d=200, degree=32, beam=64, cosine=False):
    return types.SimpleNamespace(n=n, d=d, degree=degree, beam=beam, cosine=cosine)


def test_search_roofline_formula_and_fractions():
    n, d, L = 1_000_000, 200, 64
    st = _stats([300_000_000, 200_000_000], [40_000_000, 30_000_000], [28.0, 22.0])
    out = bench.search_roofline(st, _args(), 6772.2, "measured", 2)
    gathered = 200_000_000 - 32 * n
    by = gathered * (4 * d + 4) + 30_000_000 * 32 * 4 + n * (4 * d + 32 * 4 + 4 * L)
    assert out["algorithmic_bytes_per_launch"] == by
    assert out["achieved"] == pytest.approx(by / 0.022 / 1e9, rel=1e-6)
    assert out["frac"] == pytest.approx(by / 0.022 / 1e9 / 6772.2, abs=1e-4)
    traffic = bench.SEARCH_DRAM_BYTES[(n, d, 32, L, False)][1]
    assert out["traffic"] == traffic
    assert out["dram_frac"] == pytest.approx(traffic / 0.022 / 1e9 / 6772.2, abs=1e-4)
    assert out["bound"].startswith("latency")  # under 40% of the peak by DRAM counters
    r1 = out["round1_stage"]
    b0 = (300_000_000 - 32 * n) * (4 * d + 4) + 40_000_000 * 32 * 4 + \
        n * (4 * d + 32 * 4 + 4 * L) + n * (4 * d + 32 * 4)  # + the seed pre-pass
    assert r1["algorithmic_bytes"] == b0
    assert out["kernel"].startswith("k_search_m32")


def test_search_roofline_dram_bound_names_hbm():
    args = _args(d=512, degree=48, beam=96, cosine=True)
    traffic = bench.SEARCH_DRAM_BYTES[(1_000_000, 512, 48, 96, True)][1]
    ms = traffic / (0.5 * 6772.2e9) * 1e3  # half the peak rate
    st = _stats([900_000_000, 1_500_000_000], [50_000_000, 60_000_000], [160.0, ms])
    out = bench.search_roofline(st, args, 6772.2, "measured", 2)
    assert out["dram_frac"] == pytest.approx(0.5, abs=1e-3)
    assert out["bound"].startswith("hbm")
    assert out["kernel"].startswith("k_search_mk")


def test_search_roofline_without_a_dram_capture():
    st = _stats([10_000_000, 9_000_000], [1_000_000, 900_000], [2.0, 1.5])
    out = bench.search_roofline(st, _args(n=200_000), 6772.2, "measured", 2)
    assert out["traffic"] is None and "dram_frac" not in out
