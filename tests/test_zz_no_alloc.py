"""pg_prune_reverse_noalloc: the prune + reverse-edge stage for callers that cannot allocate
device memory (for example a host application that owns the GPU through its own pool and
forbids plugins to call cudaMalloc).  Its workspace is a fixed array inside the library, so it
needs no handle; it must give exactly the outputs of pg_prune_reverse, call after call.

This file is collected last on purpose: a failure here leaves every other test already run.
"""
import ctypes
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

P, R = 32, 94  # link-round lengths at M = 32


@pytest.fixture(scope="module")
def pg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import paragraph_gb300
    paragraph_gb300.lib()
    return paragraph_gb300


def _inputs(golden_dir):
    f = np.load(os.path.join(golden_dir, "ref_edge_1000x200.npz"))
    base = torch.from_numpy(np.ascontiguousarray(f["base"])).cuda()
    graph = torch.from_numpy(np.ascontiguousarray(f["search_in"]).view(np.int32)).cuda()
    return base, graph


def _outputs(n):
    return [torch.full(s, -1, dtype=torch.int32, device="cuda") for s in ((n, P), (n,), (n, R), (n,))]


def _noalloc(pg, base, graph, outs, stream, pruned=P):
    ev = ctypes.c_uint64(0)
    n, d = base.shape
    rc = pg.lib().pg_prune_reverse_noalloc(stream, base.data_ptr(), n, d, graph.data_ptr(),
                                           graph.shape[1], pruned, R, 1, outs[0].data_ptr(),
                                           outs[1].data_ptr(), outs[2].data_ptr(),
                                           outs[3].data_ptr(), ctypes.byref(ev))
    return rc, int(ev.value)


def _host(t):
    return t.cpu().numpy().view(np.uint32)


def _masked(a, cnt):
    a = a.copy()
    a[np.arange(a.shape[1])[None, :] >= np.minimum(cnt, a.shape[1])[:, None]] = 0xFFFFFFFF
    return a


def test_noalloc_matches_allocating_entry_point_twice(pg, golden_dir):
    base, graph = _inputs(golden_dir)
    n = base.shape[0]
    ref = _outputs(n)
    with pg.Handle(0) as h:
        ref_ev = h.prune_reverse(base, graph, *ref, strict=True)
    stream = torch.cuda.current_stream().cuda_stream
    results = []
    for _ in range(2):  # two calls in a row share (and must clear) the same workspace
        outs = _outputs(n)
        rc, ev = _noalloc(pg, base, graph, outs, stream)
        assert rc == pg.PG_OK, pg.lib().pg_last_error().decode()
        results.append((outs, ev))
    pr_num = _host(ref[1])
    rv_num = _host(ref[3])
    for outs, ev in results:
        assert ev == ref_ev
        assert np.array_equal(_host(outs[1]), pr_num)
        assert np.array_equal(_host(outs[3]), rv_num)
        assert np.array_equal(_masked(_host(outs[0]), pr_num), _masked(_host(ref[0]), pr_num))
        assert np.array_equal(_masked(_host(outs[2]), rv_num), _masked(_host(ref[2]), rv_num))


def test_noalloc_allocates_nothing_per_call(pg, golden_dir):
    base, graph = _inputs(golden_dir)
    outs = _outputs(base.shape[0])
    stream = torch.cuda.current_stream().cuda_stream
    assert _noalloc(pg, base, graph, outs, stream)[0] == pg.PG_OK  # first call: per-device set-up
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _noalloc(pg, base, graph, outs, stream)[0] == pg.PG_OK
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before


def test_noalloc_rejects_sizes_beyond_its_limit(pg):
    n = 32769
    base = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    graph = torch.full((n, 64), -1, dtype=torch.int32, device="cuda")
    outs = _outputs(n)
    rc, _ = _noalloc(pg, base, graph, outs, torch.cuda.current_stream().cuda_stream)
    assert rc == pg.PG_EINVAL
    assert b"32768" in pg.lib().pg_last_error()


def test_noalloc_rejects_edge_count_beyond_its_limit(pg):
    n, c, pruned = 32768, 64, 33  # n is allowed; n * pruned = 1081344 edges is not
    base = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    graph = torch.full((n, c), -1, dtype=torch.int32, device="cuda")
    outs = _outputs(n)
    rc, _ = _noalloc(pg, base, graph, outs, torch.cuda.current_stream().cuda_stream, pruned=pruned)
    assert rc == pg.PG_EINVAL
    assert b"1048576" in pg.lib().pg_last_error()


def test_noalloc_reports_out_of_range_id(pg, golden_dir):
    """An input id >= n that is not tomb: the prune kernel drops it without reading its row and
    flags it, and the call returns PG_EINVAL; the next call with good input succeeds."""
    f = np.load(os.path.join(golden_dir, "ref_edge_1000x200.npz"))
    bad = np.ascontiguousarray(f["search_in"]).copy()
    bad[3, 5] = 1000 + 7
    base = torch.from_numpy(np.ascontiguousarray(f["base"])).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    outs = _outputs(1000)
    rc, _ = _noalloc(pg, base, torch.from_numpy(bad.view(np.int32)).cuda(), outs, stream)
    assert rc == pg.PG_EINVAL
    assert b"id >= n" in pg.lib().pg_last_error()
    good = torch.from_numpy(np.ascontiguousarray(f["search_in"]).view(np.int32)).cuda()
    assert _noalloc(pg, base, good, outs, stream)[0] == pg.PG_OK
