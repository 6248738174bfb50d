"""The restored C++ class Gbuilder::Builder<float> (include/paragraph_gb300/Builder.hpp, the
reference's include/Builder.hpp:15-35) compiled against the C ABI: it compiles with g++ on any
host, and on a GPU its LaunchBuild + SaveGraph file equals the oracle's graph in the SaveGraph
layout (tests/test_t2iend.cu:615-633) with the MatchNN entry point (:188-221).
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "builder_demo.cpp")
TOMB = 0xFFFFFFFF


def _gxx():
    g = shutil.which("g++")
    if g is None:
        pytest.skip("g++ not available")
    return g


def test_builder_header_compiles(tmp_path):
    obj = tmp_path / "builder_demo.o"
    subprocess.run([_gxx(), "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    "-c", SRC, "-o", str(obj)], check=True)
    assert obj.exists()


def _demo(tmp_path):
    from paragraph_gb300 import build as pgb
    libpath = pgb.build()
    libdir = os.path.dirname(libpath)
    exe = tmp_path / "builder_demo"
    cuda_lib = "/usr/local/cuda/lib64"
    subprocess.run([_gxx(), "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC,
                    "-o", str(exe), f"-L{libdir}", "-lparagraph_gb300", f"-Wl,-rpath,{libdir}",
                    f"-L{cuda_lib}", "-lcudart", f"-Wl,-rpath,{cuda_lib}"], check=True)
    return exe


@pytest.mark.gpu
def test_builder_launch_and_save_graph_equal_oracle(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import paragraph_gb300 as pg
    from paragraph_gb300 import datagen
    exe = _demo(tmp_path)
    n, d = 3000, 64
    base, gt = datagen.make_dataset(n, d, seed=31)
    base.tofile(tmp_path / "base.fbin")
    gt.astype(np.uint32).tofile(tmp_path / "gt.ibin")
    out = tmp_path / "index.graph"
    r = subprocess.run([str(exe), str(tmp_path / "base.fbin"), str(tmp_path / "gt.ibin"), str(n),
                        str(d), "32", "64", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    ep, rows = pg.load_graph(str(out))
    ref = oracle.build_graph(base, gt, degree=32, beam=64)["graph"]
    assert len(rows) == n
    for i in range(n):
        assert np.array_equal(rows[i], ref[i][ref[i] != TOMB]), f"row {i}"
    assert ep == pg.entry_point(gt, n)


@pytest.mark.gpu
def test_builder_launch_index_saves_the_drivers_index(tmp_path):
    """LaunchIndex + SaveGraph write the FusionFinal index the reference driver saves
    (tests/test_t2iend.cu:1228-1258): equal to the oracle's pipeline (build, six MatchSup
    rounds, FusionNN, FusionFinal) list for list, with the MatchNN entry point."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import paragraph_gb300 as pg
    from paragraph_gb300 import datagen
    exe = _demo(tmp_path)
    n, d = 3000, 64
    base, gt = datagen.make_dataset(n, d, seed=33)
    base.tofile(tmp_path / "base.fbin")
    gt.astype(np.uint32).tofile(tmp_path / "gt.ibin")
    out = tmp_path / "index.graph"
    r = subprocess.run([str(exe), str(tmp_path / "base.fbin"), str(tmp_path / "gt.ibin"), str(n),
                        str(d), "32", "64", str(out), "index"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    ep, rows = pg.load_graph(str(out))
    ref = oracle.build_graph(base, gt, degree=32, beam=64)
    rounds = [oracle.match_sup(base, gt, t) for t in range(1, 7)]
    off, ids = oracle.fusion_final(base, ref["proj"], oracle.fusion_nn(base, rounds), ref["graph"])
    assert len(rows) == n
    for i in range(n):
        assert np.array_equal(rows[i], ids[off[i]:off[i + 1]]), f"row {i}"
    assert ep == pg.entry_point(gt, n)
    # the Python mirror of the class writes the same file
    b = pg.Builder(base, gt, degree=32, beam=64)
    b.LaunchIndex()
    b.SaveGraph(str(tmp_path / "index_py.graph"))
    assert (tmp_path / "index_py.graph").read_bytes() == out.read_bytes()
