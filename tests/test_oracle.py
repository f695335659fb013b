"""The oracle (CPU restatement of the reference join path) is pinned against
the reference's own known answers: the unit-test ground truths of
tests/unit_tests.cpp, fixtures recorded from the compiled reference, and --
where the reference checkout exists -- the compiled reference itself."""
from __future__ import annotations

import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import cases
from conftest import canon

GOLDEN = Path(__file__).resolve().parent / "golden"


def _golden(name):
    return json.loads((GOLDEN / name).read_text())


def _rows(orc, out):
    return canon(orc.canonical_rows(out))


@pytest.fixture(scope="module")
def unit_cases(hj):
    return cases.build_cases(hj)


def test_port_matches_unit_test_ground_truth(orc, unit_cases):
    for name, (plan, truth, types) in unit_cases.items():
        out = orc.run(orc.port(), plan)
        assert out.status == 0, (name, out.error)
        assert [t for t, _ in out.columns] == types, name
        if truth is not None:
            assert _rows(orc, out) == canon(truth), name
            assert out.num_rows == len(truth), name


def test_port_matches_recorded_reference_outputs(orc, unit_cases):
    gold = _golden("unit_cases.json")
    assert set(gold) == set(unit_cases)
    for name, (plan, _, _) in unit_cases.items():
        out = orc.run(orc.port(), plan)
        assert out.num_rows == gold[name]["num_rows"], name
        assert _rows(orc, out) == canon(gold[name]["rows"]), name


def test_recorded_reference_outputs_match_ground_truth(unit_cases):
    gold = _golden("unit_cases.json")
    for name, (_, truth, _) in unit_cases.items():
        if truth is not None:
            assert canon(gold[name]["rows"]) == canon(truth), name


def test_port_matches_reference_on_seeded_workloads(hj, orc):
    from hjgb300 import workloads
    gold = _golden("configs_small.json")
    for name, g in gold.items():
        w = getattr(workloads, name)(scale=g["scale"])
        out = orc.run(orc.port(), w.plan)
        n, counts, cks, _ = orc.summary(out)
        assert n == g["num_rows"], name
        assert counts == g["column_rows"], name
        assert str(cks) == g["checksum"], name
        if w.expected_rows >= 0:
            assert n == w.expected_rows, name


def test_port_vs_compiled_reference_more_seeds(hj, orc):
    ref = orc.ref()
    if ref is None:
        pytest.skip("compiled reference not available on this machine")
    from hjgb300 import workloads
    for seed in (1, 2):
        for w in (workloads.c1(0.003, seed), workloads.c2(0.001, seed), workloads.c3(0.005, seed)):
            a, b = orc.run(orc.port(), w.plan), orc.run(ref, w.plan)
            sa, sb = orc.summary(a), orc.summary(b)
            assert sa[:3] == sb[:3], (w.name, seed)
            assert np.array_equal(sa[3], sb[3]), (w.name, seed)


def test_port_error_classes_match_reference(hj, orc):
    # a VARCHAR join key with non-NULL values: runtime_error in both
    p = hj.Plan()
    t = cases.table(hj, [["a"], ["b"]], [cases.V])
    p.new_input(t)
    p.new_input(t)
    p.new_scan_node(0, [(0, cases.V)])
    p.new_scan_node(1, [(0, cases.V)])
    p.root = p.new_join_node(True, 0, 1, 0, 0, [(0, cases.V)])
    out = orc.run(orc.port(), p)
    assert out.status == hj.HJ_ERR_RUNTIME and "int32" in out.error
    # StrRef table-id overflow (> 1023): out_of_range in both
    p = hj.Plan()
    for _ in range(1025):
        p.new_input(cases.table(hj, [[1, "x"]], [cases.I, cases.V]))
    p.new_scan_node(1024, [(1, cases.V)])
    p.root = 0
    # (the compiled reference raises it inside a filter-pool thread, which ends
    # the process -- include/inner_column.h:13-107 -- so it is not run here)
    out = orc.run(orc.port(), p)
    assert out.status == hj.HJ_ERR_OUT_OF_RANGE and "table" in out.error


def _kat_keys(spec):
    import importlib.util
    spec_mod = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    m = importlib.util.module_from_spec(spec_mod)
    spec_mod.loader.exec_module(m)
    return m.kat_keys(spec)


def test_unchained_restatement_matches_reference_directory(orc):
    kat = _golden("unchained_kat.json")
    for name, e in kat.items():
        keys = _kat_keys(e["spec"])
        d = orc.unchained_directory(keys)
        assert d.size == e["dir_size"], name
        if "dir" in e:
            assert [int(x) for x in d] == e["dir"], name
        assert hashlib.sha256(d.astype("<u8").tobytes()).hexdigest() == e["sha256"], name


def test_unchained_restatement_counts(orc):
    r = np.random.default_rng(3)
    build = (r.zipf(1.2, 5000) % 300).astype(np.int32)
    probe = r.integers(-10, 400, 3000).astype(np.int32)
    got = orc.unchained_counts(build, probe)
    want = np.array([int((build == k).sum()) for k in probe])
    assert np.array_equal(got, want)
    ref = orc.ref()
    if ref is not None:
        assert np.array_equal(orc.unchained_counts(build, probe, lib=ref), want)
