"""Scan predicates (hj_filter): the reference's INT32 Comparison semantics
(NULL never compares true, IS [NOT] NULL on the bitmap, AND of several),
applied in place by compaction or fused into the probe's pass over raw rows;
every result equals the same plan over the pre-filtered table."""
from __future__ import annotations

import numpy as np
import pytest

import cases
from conftest import canon

pytestmark = pytest.mark.gpu


def gpu_out(orc, res):
    return orc.Output(0, "", res.num_rows, [(c.type, c.pages) for c in res.columns])


def _table(hj, vals, valid, extra=None):
    cols = [hj.Column.int32(vals, valid)]
    if extra is not None:
        cols.append(hj.Column.int32(extra))
    return hj.Table(len(vals), cols)


OPS = {"EQ": (0, lambda v, x: v == x), "NEQ": (1, lambda v, x: v != x), "LT": (2, lambda v, x: v < x),
       "GT": (3, lambda v, x: v > x), "LEQ": (4, lambda v, x: v <= x), "GEQ": (5, lambda v, x: v >= x)}


def test_filter_semantics_scan_root(engine, hj):
    r = np.random.default_rng(1)
    n = 5000
    v = r.integers(-50, 50, n).astype(np.int32)
    valid = (r.random(n) > 0.3).astype(np.uint8)
    pay = np.arange(n, dtype=np.int32)
    t = _table(hj, v, valid, pay)
    for name, (op, f) in OPS.items():
        for lit in (-50, 0, 7, 49, 2**31 + 3):  # the last is cast to int32 as the reference does
            p = hj.Plan()
            p.new_input(t)
            p.root = p.new_scan_node(0, [(1, hj.INT32)], filters=[(0, op, lit)])
            got = hj.decode_int32(engine.execute(p).columns[0])[0] if n else None
            x = np.int64(lit).astype(np.int32)
            want = pay[(valid == 1) & f(v, x)]
            assert np.array_equal(got, want), (name, lit)   # passing rows, in row order
    for op, want in ((8, pay[valid == 0]), (9, pay[valid == 1])):
        p = hj.Plan()
        p.new_input(t)
        p.root = p.new_scan_node(0, [(1, hj.INT32)], filters=[(0, op, 0)])
        assert np.array_equal(hj.decode_int32(engine.execute(p).columns[0])[0], want), op
    # AND of two filters; a filter column that is not an output column
    p = hj.Plan()
    p.new_input(t)
    p.root = p.new_scan_node(0, [(1, hj.INT32)], filters=[(0, 3, -10), (1, 2, 4000)])
    want = pay[(valid == 1) & (v > -10) & (pay < 4000)]
    assert np.array_equal(hj.decode_int32(engine.execute(p).columns[0])[0], want)


def test_filtered_join_sides_match_prefiltered(engine, hj, orc):
    r = np.random.default_rng(2)
    nb, npr = 3000, 20000
    bk = r.integers(0, 500, nb).astype(np.int32)
    bf = r.integers(0, 100, nb).astype(np.int32)
    pk = r.integers(0, 600, npr).astype(np.int32)
    pf = r.integers(0, 100, npr).astype(np.int32)
    pv = (r.random(npr) > 0.1).astype(np.uint8)
    B = hj.Table(nb, [hj.Column.int32(bk), hj.Column.int32(bf)])
    P = hj.Table(npr, [hj.Column.int32(pk), hj.Column.int32(pf, pv)])
    for build_left in (True, False):
        p = hj.Plan()
        p.new_input(B)
        p.new_input(P)
        p.new_scan_node(0, [(0, hj.INT32), (1, hj.INT32)], filters=[(1, 2, 60)])
        p.new_scan_node(1, [(0, hj.INT32), (1, hj.INT32)], filters=[(1, 5, 20)])
        p.root = p.new_join_node(build_left, 0, 1, 0, 0, [(0, hj.INT32), (1, hj.INT32), (3, hj.INT32)])
        kb, kp = bf < 60, (pv == 1) & (pf >= 20)
        q = hj.Plan()
        q.new_input(hj.Table(int(kb.sum()), [hj.Column.int32(bk[kb]), hj.Column.int32(bf[kb])]))
        q.new_input(hj.Table(int(kp.sum()), [hj.Column.int32(pk[kp]), hj.Column.int32(pf[kp])]))
        q.new_scan_node(0, [(0, hj.INT32), (1, hj.INT32)])
        q.new_scan_node(1, [(0, hj.INT32), (1, hj.INT32)])
        q.root = q.new_join_node(build_left, 0, 1, 0, 0, [(0, hj.INT32), (1, hj.INT32), (3, hj.INT32)])
        got = canon(orc.canonical_rows(gpu_out(orc, engine.execute(p))))
        assert got == canon(orc.canonical_rows(orc.run(orc.port(), q))), build_left
        assert len(got) > 1000


def test_fused_predicate_probe_equals_prefiltered_c2(engine, hj, orc):
    from hjgb300 import workloads
    w = workloads.c2raw(0.01)
    res = engine.execute(w.plan)
    assert res.num_rows == w.expected_rows
    got = orc.summary(gpu_out(orc, res))
    want = orc.summary(orc.run(orc.port(), w.meta["prefiltered_plan"]))
    assert got[:3] == want[:3] and np.array_equal(got[3], want[3])


def test_filter_errors(engine, hj):
    t = cases.table(hj, [["a"], ["b"]], [cases.V])
    for flt, status in (([(0, 2, 1)], hj.HJ_ERR_INVALID),       # VARCHAR filter column
                        ([(5, 2, 1)], hj.HJ_ERR_INVALID)):      # no such column
        p = hj.Plan()
        p.new_input(t)
        p.root = p.new_scan_node(0, [(0, cases.V)], filters=flt)
        with pytest.raises(hj.HjError) as e:
            engine.execute(p)
        assert e.value.status == status
    ti = _table(hj, np.arange(10, dtype=np.int32), None)
    for flt in ([(0, 6, 1)], [(0, 2, 1)] * 5):                 # LIKE; more than 4 filters
        p = hj.Plan()
        p.new_input(ti)
        p.root = p.new_scan_node(0, [(0, hj.INT32)], filters=flt)
        with pytest.raises(hj.HjError):
            engine.execute(p)
    p = hj.Plan()
    p.new_input(ti)
    p.root = p.new_scan_node(0, [(0, hj.INT32)], filters=[(0, 4, 3)])
    assert engine.execute(p).num_rows == 4
