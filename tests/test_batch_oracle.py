"""The batched-join oracle (oracle/batch_oracle.py) on the CPU: generator
properties, and chain results against the compiled reference's execute() and
the CPU restatement of it, run on the same relations as a left-deep plan."""
from __future__ import annotations

import numpy as np
import pytest

import batch_oracle as bo


def chain_plan(hj, rels):
    """Left-deep plan over [(keys, payload), ...]: output key, p0, ..., pm-1."""
    p = hj.Plan()
    for k, v in rels:
        p.new_input(hj.Table(k.size, [hj.Column.int32(k), hj.Column.int32(v)]))
    scans = [p.new_scan_node(j, [(0, hj.INT32), (1, hj.INT32)]) for j in range(len(rels))]
    cur, width = scans[0], 2
    for j in range(1, len(rels)):
        attrs = [(c, hj.INT32) for c in range(width)] + [(width + 1, hj.INT32)]
        cur = p.new_join_node(False, cur, scans[j], 0, 0, attrs)
        width += 1
    p.root = cur
    return p


def plan_result(orc, lib, plan, m):
    out = orc.run(lib, plan)
    assert out.status == 0, out.error
    dec = orc.decode(out.columns)
    if out.num_rows == 0:
        return 0, 0
    cols = [d[0] for _, d in dec]
    assert all(np.all(d[1]) for _, d in dec)  # no NULLs
    fp = bo.row_fingerprints(cols[0], np.array(cols[1:], dtype=np.int32).reshape(m, -1))
    return out.num_rows, int(fp.sum(dtype=np.uint64))


def test_generator_properties():
    seed, b, q = 42, 5000, int(0.3 * (1 << 24))
    keys1, _ = bo.relation(seed, 7, 1, b, q, b)
    assert np.unique(keys1).size == b and keys1.min() >= 0 and keys1.max() < 2 * b
    keys0, pay0 = bo.relation(seed, 7, 0, b, q, 10 * b)
    hit = np.isin(keys0, keys1)
    assert abs(hit.mean() - 0.3) < 0.02
    assert keys0.min() >= 0 and keys0.max() < 2 * b
    # payloads differ across relations and instances
    _, pay0b = bo.relation(seed, 8, 0, b, q, 10 * b)
    assert not np.array_equal(pay0, pay0b)
    # fewer build rows than build_rows: a prefix of the same keys
    k_short, _ = bo.relation(seed, 7, 1, b, q, 100)
    assert np.array_equal(k_short, keys1[:100])


def test_fold_known_values():
    """The fingerprint on fixed inputs (Python ints, independent of numpy)."""
    def fin(x):
        x &= bo.M64
        x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & bo.M64
        x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & bo.M64
        return x ^ (x >> 31)

    def add(st, v):
        return ((st ^ (v & 0xFFFFFFFF)) * bo.GOLD) & bo.M64

    key, p0, p1 = -5, 7, -(2**31)
    st = (((key & 0xFFFFFFFF) ^ 0x243F6A8885A308D3) * bo.GOLD) & bo.M64
    want = fin(add(add(st, p0), p1))
    got = bo.row_fingerprints(np.array([key], np.int32), np.array([[p0], [p1]], np.int32))
    assert int(got[0]) == want
    # a different pairing of the same values gives a different fingerprint
    other = bo.row_fingerprints(np.array([key], np.int32), np.array([[p1], [p0]], np.int32))
    assert int(other[0]) != want


@pytest.mark.parametrize("m,b,rate", [(2, 300, 0.5), (3, 800, 1.0), (4, 1500, 0.1), (2, 1, 1.0)])
def test_chain_result_matches_reference_execute(hj, orc, m, b, rate):
    q = int(round(rate * (1 << 24)))
    rels = bo.instance_relations(42, 11 + m, m, b, q, 10 * b)
    want = bo.chain_result(rels)
    plan = chain_plan(hj, rels)
    assert plan_result(orc, orc.port(), plan, m) == want
    ref = orc.ref()
    if ref is None:
        pytest.skip("reference build not available")
    assert plan_result(orc, ref, plan, m) == want


def test_chain_with_duplicate_keys(hj, orc):
    """Duplicate build keys give the cross product in the oracle as in the reference."""
    r = np.random.default_rng(3)
    rels = [(r.integers(0, 40, 500).astype(np.int32), r.integers(-9, 9, 500).astype(np.int32)),
            (r.integers(0, 60, 200).astype(np.int32), r.integers(-9, 9, 200).astype(np.int32)),
            (r.integers(20, 50, 100).astype(np.int32), r.integers(-9, 9, 100).astype(np.int32))]
    want = bo.chain_result(rels)
    assert want[0] > 500
    plan = chain_plan(hj, rels)
    assert plan_result(orc, orc.port(), plan, 3) == want
    ref = orc.ref()
    if ref is not None:
        assert plan_result(orc, ref, plan, 3) == want


def test_batch_waves_cover_every_instance(hj):
    from hjgb300 import batch, workloads
    w = workloads.c4(n=300, scale=0.01)
    ws = batch.waves(w, 200_000)
    flat = [i for g in ws for i in g]
    assert flat == list(range(len(w)))
    for g in ws:
        assert len(g) == 1 or sum(w.rows(i) for i in g) <= 200_000
    s = w.subset([3, 9])
    assert s.instance(1)[0] == 9 and s.instance(1)[1:] == w.instance(9)[1:]


def test_autotune_sample_and_radix_bits(hj):
    from hjgb300 import autotune, workloads
    w = workloads.c4(n=500, scale=1.0)
    s = autotune.sample(w, 64)
    assert len(s) == 64 and len(set(s.ids.tolist())) == 64
    # strata cover the size range
    assert s.build_rows.min() < 2_000 and s.build_rows.max() > 2_000_000
    assert autotune.radix_bits_for(4000, 12) == 0
    assert autotune.radix_bits_for(4_000_000, 12) == 10
    assert autotune.radix_bits_for(12_000_000, 9) == 11  # capped at 11 partition bits


def test_serving_schedule_is_a_seeded_poisson_mix(hj):
    from hjgb300 import serve
    mix = serve.Mix({"small": [0] * 16, "medium": [0], "large": [0]})
    a = serve.schedule(mix, rate=1000, n=20_000, seed=1)
    assert a == serve.schedule(mix, rate=1000, n=20_000, seed=1)
    t = np.array([x[0] for x in a])
    assert np.all(np.diff(t) > 0) and abs(t[-1] / 20_000 - 1e-3) < 5e-5       # mean gap 1/rate
    kinds = np.array([x[1] for x in a])
    for k, f in zip(serve.KINDS, mix.fractions):
        assert abs((kinds == k).mean() - f) < 0.015
    assert {x[2] for x in a if x[1] == "small"} == set(range(16))


def test_bench_c4_cpu_sample(hj, orc):
    """bench.py's c4 CPU baseline: every sampled instance runs as its left-deep
    plan through the restated execute(), and its row count is checked against
    the given (GPU) counts."""
    import importlib.util
    from pathlib import Path
    from hjgb300 import workloads
    spec = importlib.util.spec_from_file_location("bench", Path(__file__).resolve().parents[1] / "bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    w = workloads.c4(n=24, scale=0.004)
    rows = np.array([bo.chain_result(bo.instance_relations(w.seed, *w.instance(i)))[0] for i in range(len(w))])
    out = bench.c4_cpu_sample(hj, w, rows, 30.0, n=12)
    assert out["rows_equal_gpu"] and out["kind"] == "port" and out["value"] > 0
    assert out["sample"].startswith("12 of a seeded 12-instance sample")
    assert not bench.c4_cpu_sample(hj, w, rows + 1, 30.0, n=12)["rows_equal_gpu"]
