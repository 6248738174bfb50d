"""Argument and capacity errors of the index, ground-truth and RoarGraph entry points: each is a
status code (never a crash), and the handle stays usable afterwards."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import paragraph_gb300
    paragraph_gb300.lib()
    return paragraph_gb300


def _i32(*shape):
    return torch.zeros(shape, dtype=torch.int32, device="cuda")


def test_errors_are_status_codes(pg):
    from paragraph_gb300 import datagen
    base, q = datagen.make_base_queries(500, 32, 600, seed=2)
    gt = datagen.ground_truth(base, q[:500], 128)
    tb = torch.from_numpy(base).cuda()
    tq = torch.from_numpy(np.ascontiguousarray(q[500:])).cuda()
    tg = torch.from_numpy(gt.view(np.int32)).cuda()
    with pg.Handle(0) as h:
        cases = [
            (lambda: h.ground_truth(tb, tq, _i32(100, 300)), pg.PG_EINVAL),  # k > 256
            (lambda: h.ground_truth(tb * 1e5, tq, _i32(100, 8)), pg.PG_EUNSUPPORTED),  # FP16 range
            (lambda: h.match_sup(tb, tg, 128, _i32(500, 40), _i32(500)), pg.PG_EINVAL),  # topn
            (lambda: h.match_sup(tb, tg, 1, _i32(500, 80), _i32(500), m_nn=80), pg.PG_EINVAL),
            (lambda: h.fusion_nn(tb, _i32(7, 500, 40), _i32(7, 500), _i32(500, 80), _i32(500)),
             pg.PG_EUNSUPPORTED),  # 7 rounds x 40 > 256 candidates
            (lambda: h.build_index(tb, tg, _i32(500, 100), _i32(500)), pg.PG_EINVAL),  # stride
            (lambda: h.build_index(tb, tg, _i32(500, 150), _i32(500), match_rounds=0),
             pg.PG_EINVAL),
        ]
        for i, (call, code) in enumerate(cases):
            with pytest.raises(pg.PGError) as e:
                call()
            assert e.value.code == code, (i, e.value)
        # still usable
        out = _i32(100, 16)
        h.ground_truth(tb, tq, out)
        rows, cnt = _i32(500, 150), _i32(500)
        h.build_index(tb, tg, rows, cnt)
        assert int(cnt.max()) > 0
