"""The CPU RoarGraph path and final fusion on the GPU (pg_match_sup, pg_fusion_nn,
pg_fusion_final, pg_build_index) against the reference's own CPU code (tests/golden/ref_cpu_*,
made from tests/test_t2iend.cu) and against the oracle: ids equal list for list."""
import os

import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CASES = ["mix", "edge"]
M_NN = 40


@pytest.fixture(scope="module")
def pg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import paragraph_gb300
    paragraph_gb300.lib()
    return paragraph_gb300


def load(golden_dir, name):
    f = dict(np.load(os.path.join(golden_dir, f"ref_{name}_1000x200.npz")))
    c = dict(np.load(os.path.join(golden_dir, f"ref_cpu_{name}_1000x200.npz")))
    return f, c


def dev(a):
    a = np.ascontiguousarray(a)
    if a.dtype == np.uint32:
        a = a.view(np.int32)
    elif a.dtype == np.uint64:
        a = a.view(np.int64)
    return torch.from_numpy(a).cuda()


def host_rows(out, cnt):
    torch.cuda.synchronize()
    o = out.cpu().numpy().view(np.uint32)
    k = cnt.cpu().numpy().view(np.uint32)
    return [o[i, :k[i]].copy() for i in range(o.shape[0])]


def csr_rows(off, ids):
    return [ids[off[i]:off[i + 1]] for i in range(len(off) - 1)]


def u32(n, *shape):
    return torch.full((n, *shape) if shape else (n,), -1, dtype=torch.int32, device="cuda")


@pytest.mark.parametrize("case", CASES)
def test_match_sup_and_fusion_nn_equal_reference(pg, golden_dir, case):
    f, c = load(golden_dir, case)
    base, gt = f["base"], f["gt"]
    n = base.shape[0]
    db, dg = dev(base), dev(gt)
    sup = torch.full((6, n, M_NN), -1, dtype=torch.int32, device="cuda")
    supc = torch.zeros((6, n), dtype=torch.int32, device="cuda")
    with pg.Handle(0) as h:
        for r in range(1, 7):
            h.match_sup(db, dg, r, sup[r - 1], supc[r - 1])
            got = host_rows(sup[r - 1], supc[r - 1])
            ref = csr_rows(c[f"sup{r}_off"], c[f"sup{r}_ids"])
            o_off, o_ids = oracle.match_sup(base, gt, r)
            ora = csr_rows(o_off, o_ids)
            for i in range(n):
                assert np.array_equal(np.sort(got[i]), np.sort(ref[i])), f"round {r}, base {i}"
                assert np.array_equal(got[i], ora[i]), f"round {r}, base {i} (order)"
        out = u32(n, 2 * M_NN)
        cnt = u32(n)
        h.fusion_nn(db, sup, supc, out, cnt)
        got = host_rows(out, cnt)
    ref = csr_rows(c["fnn_off"], c["fnn_ids"])
    for i in range(n):
        assert np.array_equal(got[i], ref[i]), f"FusionNN base {i}"


@pytest.mark.parametrize("case", CASES + ["ffwrap"])
def test_fusion_final_equals_reference(pg, golden_dir, case):
    if case == "ffwrap":
        f = dict(np.load(os.path.join(golden_dir, "ref_mix_1000x200.npz")))
        c = dict(np.load(os.path.join(golden_dir, "ref_cpu_ffwrap_1000x200.npz")))
        b_off, b_ids = c["bip_off"], c["bip_ids"]
    else:
        f, c = load(golden_dir, case)
        b_off, b_ids = c["fnn_off"], c["fnn_ids"]
    base = f["base"]
    n = base.shape[0]
    stride = int(np.diff(b_off.astype(np.int64)).max()) + 70
    out = u32(n, stride)
    cnt = u32(n)
    with pg.Handle(0) as h:
        h.fusion_final(dev(base), dev(f["proj"]), dev(f["link32_graph"]), out, cnt,
                       bip_off=dev(b_off), bip_ids=dev(b_ids))
        got = host_rows(out, cnt)
    ref = csr_rows(c["ff_off"], c["ff_ids"])
    for i in range(n):
        assert np.array_equal(got[i], ref[i]), f"FusionFinal node {i}"


@pytest.mark.parametrize("n,d", [(3000, 64), (2500, 44)])  # 44 = 2*16 + 8 + 4: both tails
def test_build_index_equals_oracle_pipeline(pg, n, d):
    from paragraph_gb300 import datagen
    base, gt = datagen.make_dataset(n, d, seed=808)
    params = pg.default_params(32, 64)
    out = u32(n, 2 * M_NN + 70)
    cnt = u32(n)
    with pg.Handle(0) as h:
        st = h.build_index(dev(base), dev(gt), out, cnt, params)
        got = host_rows(out, cnt)
    print(f"index {n}x{d}: build {st.ms_total:.1f} ms (MatchSup {st.ms_match_sup:.1f}, "
          f"FusionNN {st.ms_fusion_nn:.1f}, FusionFinal {st.ms_fusion_final:.1f})")
    g = oracle.build_graph(base, gt, degree=32, beam=64)
    rounds = [oracle.match_sup(base, gt, r) for r in range(1, 7)]
    fnn = oracle.fusion_nn(base, rounds)
    off, ids = oracle.fusion_final(base, g["proj"], fnn, g["graph"])
    ref = csr_rows(off, ids)
    for i in range(n):
        assert np.array_equal(got[i], ref[i]), f"index node {i}"


def test_fusion_final_rejects_oversized_rows(pg, golden_dir):
    f, c = load(golden_dir, "mix")
    n = f["base"].shape[0]
    out = u32(n, 8)  # too narrow for most rows
    cnt = u32(n)
    with pg.Handle(0) as h:
        with pytest.raises(pg.PGError) as e:
            h.fusion_final(dev(f["base"]), dev(f["proj"]), dev(f["link32_graph"]), out, cnt,
                           bip_off=dev(c["fnn_off"]), bip_ids=dev(c["fnn_ids"]))
        assert e.value.code == pg.PG_EUNSUPPORTED
