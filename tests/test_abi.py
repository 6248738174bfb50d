"""C ABI and host logic without a GPU: the library loads, exports every symbol the header
declares, maps parameters like the reference driver, writes the reference's on-disk formats and
reports errors instead of exiting."""
import os
import re

import numpy as np
import pytest

import paragraph_gb300 as pg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "paragraph_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|uint32_t|const char\*)\s+(pg_\w+)\(", src, re.M)))


def test_library_exports_every_declared_symbol():
    L = pg.lib()
    names = declared_symbols()
    assert len(names) >= 14
    for name in names:
        assert hasattr(L, name), name
        assert name in pg.SIGNATURES, f"{name} has no ctypes signature"


def test_abi_version():
    assert pg.lib().pg_abi_version() == 1


@pytest.mark.parametrize("m,l,r,km", [(32, 64, 94, 32), (48, 96, 78, 64), (55, 64, 71, 32)])
def test_default_params_follow_reference_mapping(m, l, r, km):
    p = pg.default_params(m, l)
    assert (p.degree, p.link_reverse, p.km, p.kp, p.kd) == (m, r, km, 2, 16)
    assert (p.gt_k, p.proj_degree, p.proj_pruned, p.proj_reverse) == (128, 16, 15, 111)
    assert (p.reset_iter, p.seed_base, p.link_rounds) == (15, 3030517, 2)
    assert p.degree + p.link_reverse + 2 == 128  # the 512-byte pr list of the reference


def test_bad_params_report_errors():
    with pytest.raises(pg.PGError) as e:
        pg.default_params(0, 64)
    assert e.value.code == pg.PG_EINVAL
    with pytest.raises(pg.PGError):
        pg.default_params(32, 16)


def test_workspace_size_reported_without_gpu():
    import ctypes
    p = pg.default_params(32, 64)
    b = ctypes.c_uint64(0)
    assert pg.lib().pg_workspace_bytes(ctypes.byref(p), 1_000_000, 200, 1_000_000,
                                       ctypes.byref(b)) == 0
    assert 0.8e9 < b.value < 4e9
    assert pg.lib().pg_workspace_bytes(ctypes.byref(p), 1000, 10, 1000, ctypes.byref(b)) == \
        pg.PG_EUNSUPPORTED


def test_create_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import ctypes
    h = ctypes.c_void_p()
    rc = pg.lib().pg_create(ctypes.byref(h), 0, None)
    assert rc == pg.PG_ECUDA and not h.value
    assert pg.lib().pg_last_error()


def test_savegraph_layout(tmp_path):
    g = np.array([[3, 1, pg.TOMB], [pg.TOMB, pg.TOMB, pg.TOMB], [0, 2, 1]], dtype=np.uint32)
    path = str(tmp_path / "g.bin")
    pg.save_graph(path, g, ep=2)
    raw = np.fromfile(path, dtype=np.uint32)
    # SaveGraph (tests/test_t2iend.cu:615-633): [ep][n] then [deg][ids] per node
    assert raw.tolist() == [2, 3, 2, 3, 1, 0, 3, 0, 2, 1]
    ep, rows = pg.load_graph(path)
    assert ep == 2 and [r.tolist() for r in rows] == [[3, 1], [], [0, 2, 1]]


def test_savegraph_unwritable_path_is_an_error(tmp_path):
    with pytest.raises(pg.PGError) as e:
        pg.save_graph(str(tmp_path / "missing-dir" / "g.bin"), np.zeros((1, 1), np.uint32), 0)
    assert e.value.code == pg.PG_EIO


def test_read_headerless_and_headered(tmp_path):
    a = np.arange(12, dtype=np.float32).reshape(3, 4)
    p1 = str(tmp_path / "raw.fbin")
    a.tofile(p1)
    assert np.array_equal(pg.read_vectors(p1, np.float32, (3, 4)), a)
    p2 = str(tmp_path / "hdr.fbin")
    with open(p2, "wb") as f:
        np.array([3, 4], dtype=np.uint32).tofile(f)
        a.tofile(f)
    assert np.array_equal(pg.read_vectors(p2, np.float32, headered=True), a)
    with pytest.raises(pg.PGError) as e:
        pg.read_vectors(p1, np.float32, (4, 4))  # short file
    assert e.value.code == pg.PG_EIO
    with pytest.raises(pg.PGError):
        pg.read_vectors(str(tmp_path / "nope"), np.float32, (1, 1))


def matchnn_frequency(gt, n):
    """The counting loop of MatchNN (tests/test_t2iend.cu:188-205), restated."""
    freq = np.zeros(n, np.int64)
    vis = np.zeros(n, bool)
    for row in gt:
        for nn in row:
            if nn >= n:
                break
            freq[nn] += 1
            if not vis[nn]:
                vis[nn] = True
                break
    return freq


def test_entry_point_rule():
    rng = np.random.default_rng(4)
    n = 500
    gt = rng.integers(0, n, (800, 128)).astype(np.uint32)
    gt[:, 0] = rng.integers(0, 20, 800)  # concentrate the first columns: a clear maximum
    gt[:300, 0] = 7
    freq = matchnn_frequency(gt, n)
    ep = pg.entry_point(gt, n)
    assert freq[ep] == freq.max()
    assert ep == int(np.argmax(freq)) or freq[int(np.argmax(freq))] == freq[ep]
