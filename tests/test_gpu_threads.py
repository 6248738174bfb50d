"""Threading contract of the C ABI: handles are independent, each runs on its own stream, and a
handle serialises its own calls.  Two handles driven from two host threads at once (each on its
own non-default stream, a different data set each, several builds in a row) must give exactly
the graphs that serial builds give; two threads sharing one handle must too (the handle's mutex
orders them).  The reference drives its builds from one host thread (tests/test_t2iend.cu:809-815).
"""
import threading

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


def _sets():
    from paragraph_gb300 import datagen
    return [datagen.make_dataset(12000, 64, seed=s) for s in (101, 202)]


def _serial(pg, sets, params):
    out = []
    with pg.Handle(0) as h:
        for base, gt in sets:
            g, p, st = h.build_host(base, gt, params)
            out.append((g, p, st.evals_total))
    return out


def _run_threads(fns):
    errors = []

    def wrap(f):
        try:
            f()
        except BaseException as e:  # surfaced in the main thread below
            errors.append(e)

    ts = [threading.Thread(target=wrap, args=(f,)) for f in fns]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=600)
    assert not any(t.is_alive() for t in ts), "a build thread did not finish"
    if errors:
        raise errors[0]


@pytest.mark.parametrize("screen", ["fp16", "none"])
def test_two_handles_two_threads_equal_serial(pg, screen):
    params = pg.default_params(32, 64, screen=pg.SCREEN_FP16 if screen == "fp16" else 0)
    sets = _sets()
    ref = _serial(pg, sets, params)
    results = [[], []]

    def worker(i):
        def run():
            stream = torch.cuda.Stream(0)
            with pg.Handle(0, stream=stream) as h:
                for _ in range(3):
                    g, p, st = h.build_host(*sets[i], params)
                    results[i].append((g, p, st.evals_total))
        return run

    _run_threads([worker(0), worker(1)])
    for i in range(2):
        assert len(results[i]) == 3
        for g, p, ev in results[i]:
            assert np.array_equal(g, ref[i][0]) and np.array_equal(p, ref[i][1])
            assert ev == ref[i][2]


def test_two_threads_one_handle_equal_serial(pg):
    params = pg.default_params(32, 64, screen=pg.SCREEN_FP16)
    sets = _sets()
    ref = _serial(pg, sets, params)
    results = [[], []]
    stream = torch.cuda.Stream(0)
    with pg.Handle(0, stream=stream) as h:
        def worker(i):
            def run():
                for _ in range(2):
                    g, p, st = h.build_host(*sets[i], params)
                    results[i].append((g, p, st.evals_total))
            return run

        _run_threads([worker(0), worker(1)])
    for i in range(2):
        for g, p, ev in results[i]:
            assert np.array_equal(g, ref[i][0]) and np.array_equal(p, ref[i][1])
            assert ev == ref[i][2]
