"""The request loop (hj_server): every plan of a mixed open-loop stream gives
the same result in the mix (concurrent slots, HBM admission, cached tables
over resident columns) as alone through Contest::execute; admission keeps to
its budget; a failing plan fails alone."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mix(engine):
    from hjgb300 import serve
    m = serve.c5_mix(engine, small_tables=4, small_lo=2_000, small_hi=40_000, medium_scale=0.01,
                     large_scale=0.004)
    yield m
    m.release(engine)


def _summaries(orc, engine, held):
    out = {}
    for i, res in held.items():
        r = engine.fetch(res)
        engine.free_result(res)
        out[i] = orc.summary(orc.Output(0, "", r.num_rows, [(c.type, c.pages) for c in r.columns]))
    return out


def test_results_same_alone_and_in_the_mix(engine, hj, orc, mix):
    from hjgb300 import serve
    sched = serve.schedule(mix, rate=3000, n=48, seed=3)
    assert {k for _, k, _ in sched} == set(serve.KINDS)
    alone, mixed = {}, {}
    serve.run_plain(engine, mix, sched, keep=lambda i, r: alone.__setitem__(i, r) or True)
    engine.set_option("table_cache", 1)
    try:
        rep = serve.run_served(engine, mix, sched, hbm_budget=8 << 30, slots=4,
                               keep=lambda i, r: mixed.__setitem__(i, r) or True)
    finally:
        engine.set_option("table_cache", 0)
    a, b = _summaries(orc, engine, alone), _summaries(orc, engine, mixed)
    for i in range(len(sched)):
        assert a[i][:3] == b[i][:3], (i, sched[i])
        assert np.array_equal(a[i][3], b[i][3]), (i, sched[i])
    assert rep["p99_ms"] >= rep["p50_ms"] > 0


def test_admission_keeps_to_the_budget(engine, hj, mix):
    from hjgb300 import serve
    sched = serve.schedule(mix, rate=5000, n=24, seed=4)
    rep = serve.run_served(engine, mix, sched, hbm_budget=1, slots=8)
    # a budget below every estimate admits one plan at a time
    with engine.server(1, 8) as srv:
        t = [srv.submit(mix.plans[k][i]) for _, k, i in sched[:4]]
        est = []
        for x in t:
            res, st = srv.wait(x)
            est.append(st["est_bytes"])
            engine.free_result(res)
        assert srv.info()["peak_bytes"] == max(est)
    assert rep["peak_admitted_bytes"] > 0


def test_failing_plan_fails_alone(engine, hj, mix):
    from hjgb300 import serve
    good = mix.plans["small"][0]
    p = hj.Plan()
    for t in mix.resident[:2]:  # the first small query's tables
        p.new_input(t)
    p.new_scan_node(0, [(7, hj.INT32)])  # no column 7
    p.root = 0
    with engine.server(8 << 30, 2) as srv:
        t1, t2, t3 = srv.submit(good), srv.submit(p), srv.submit(good)
        r1, _ = srv.wait(t1)
        with pytest.raises(hj.HjError):
            srv.wait(t2)
        r3, _ = srv.wait(t3)
        assert serve._summary(engine, r1) == serve._summary(engine, r3)
        engine.free_result(r1)
        engine.free_result(r3)
