"""Batched independent joins on the GPU (hj_batch_execute, hj_batch_generate):
the device generator bit-for-bit against the oracle's restatement, and per
instance row counts and checksums of the persistent batch and of the plain
one-at-a-time path against the oracle, under every tunable."""
from __future__ import annotations

import numpy as np
import pytest

import batch_oracle as bo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small_c4():
    from hjgb300 import workloads
    return workloads.c4(n=96, scale=0.004)   # builds of 4 .. 16k rows


@pytest.fixture(scope="module")
def small_c4_truth(small_c4):
    w = small_c4
    out = []
    for i in range(len(w)):
        iid, m, b, q, p = w.instance(i)
        out.append(bo.chain_result(bo.instance_relations(w.seed, iid, m, b, q, p)))
    return np.array([r for r, _ in out], np.uint64), np.array([s for _, s in out], np.uint64)


def test_device_generator_matches_oracle(engine, hj):
    import torch
    for inst, rel, b, rate, rows in [(0, 0, 1000, 0.5, 10_000), (5, 1, 1000, 0.5, 1000), (77, 3, 123_457, 0.9, 50_000),
                                     (9, 0, 1, 1.0, 17), (4095, 2, 4_000_000, 0.1, 4_000_000)]:
        q = int(round(rate * (1 << 24)))
        k = torch.empty(rows, dtype=torch.int32, device="cuda")
        v = torch.empty(rows, dtype=torch.int32, device="cuda")
        engine.batch_generate(42, inst, rel, b, q, rows, k.data_ptr(), v.data_ptr())
        torch.cuda.ExternalStream(engine.stream).synchronize()
        wk, wv = bo.relation(42, inst, rel, b, q, rows)
        assert np.array_equal(k.cpu().numpy(), wk), (inst, rel)
        assert np.array_equal(v.cpu().numpy(), wv), (inst, rel)


def test_batched_and_plain_match_oracle(engine, hj, small_c4, small_c4_truth):
    from hjgb300 import batch
    want_rows, want_sums = small_c4_truth
    for mode in (hj.BATCH_PERSISTENT, hj.BATCH_PLAIN):
        rows, sums, redo, _ = batch.run(engine, small_c4, mode, max_rows=1 << 40)
        assert redo == 0
        assert np.array_equal(rows, want_rows), mode
        assert np.array_equal(sums, want_sums), mode


def test_batched_in_waves(engine, hj, small_c4, small_c4_truth):
    from hjgb300 import batch
    rows, sums, _, _ = batch.run(engine, small_c4, hj.BATCH_PERSISTENT, max_rows=300_000)
    assert len(batch.waves(small_c4, 300_000)) > 2
    assert np.array_equal(rows, small_c4_truth[0]) and np.array_equal(sums, small_c4_truth[1])


def test_batched_tunables_do_not_change_results(engine, hj, small_c4, small_c4_truth):
    from hjgb300 import batch
    sub = small_c4.subset(np.arange(0, len(small_c4), 3))
    want = small_c4_truth[0][::3], small_c4_truth[1][::3]
    opts = [{"batch_load_pct": p} for p in (90, 70, 200)] + \
           [{"batch_part_log2": b} for b in (8, 10, 13)] + [{"batch_graph": 0}]
    for opt in opts:
        saved = {k: engine.get_option(k) for k in opt}
        try:
            for k, v in opt.items():
                engine.set_option(k, v)
            rows, sums, redo, _ = batch.run(engine, sub, hj.BATCH_PERSISTENT, max_rows=1 << 40)
        finally:
            for k, v in saved.items():
                engine.set_option(k, v)
        assert np.array_equal(rows, want[0]) and np.array_equal(sums, want[1]), opt
        assert redo == 0


def test_plain_tunables_do_not_change_results(engine, hj, small_c4, small_c4_truth):
    from hjgb300 import batch
    sub = small_c4.subset(np.arange(1, len(small_c4), 7))
    want = small_c4_truth[0][1::7], small_c4_truth[1][1::7]
    for opt in ({"radix_bits": 0}, {"radix_bits": 12}, {"probe_group": 1}, {"probe_group": 32},
                {"dir_bits": 6}):
        saved = {k: engine.get_option(k) for k in opt}
        try:
            for k, v in opt.items():
                engine.set_option(k, v)
            rows, sums, _, _ = batch.run(engine, sub, hj.BATCH_PLAIN, max_rows=1 << 40)
        finally:
            for k, v in saved.items():
                engine.set_option(k, v)
        assert np.array_equal(rows, want[0]) and np.array_equal(sums, want[1]), opt


def test_batch_duplicates_empty_and_mixed_depths(engine, hj):
    """Hand-made relations: duplicate keys on both sides (cross products), an
    empty build relation, an empty probe relation, negative keys, 2- and 4-deep
    chains in one batch."""
    import torch
    r = np.random.default_rng(5)
    host = [
        [(r.integers(-30, 30, 4000), r.integers(-9, 9, 4000)), (r.integers(-20, 40, 900), r.integers(-9, 9, 900))],
        [(r.integers(0, 50, 3000), r.integers(0, 9, 3000)), (r.integers(0, 50, 300), r.integers(0, 9, 300)),
         (r.integers(10, 20, 40), r.integers(0, 9, 40)), (r.integers(0, 15, 7), r.integers(0, 9, 7))],
        [(r.integers(0, 5, 100), r.integers(0, 9, 100)), (np.zeros(0), np.zeros(0))],
        [(np.zeros(0), np.zeros(0)), (r.integers(0, 5, 10), r.integers(0, 9, 10)),
         (r.integers(0, 5, 10), r.integers(0, 9, 10))],
        [(np.array([2**31 - 1, -(2**31), 0]), np.array([1, 2, 3])),
         (np.array([-(2**31), -(2**31), 2**31 - 1]), np.array([4, 5, 6]))],
        # one key 3000 times: a partition larger than a shared-memory table
        [(np.concatenate([np.full(50, 7), r.integers(0, 100, 500)]), r.integers(0, 9, 550)),
         (np.concatenate([np.full(3000, 7), r.integers(0, 100, 100)]), r.integers(0, 9, 3100))],
    ]
    host = [[(k.astype(np.int32), v.astype(np.int32)) for k, v in inst] for inst in host]
    keep, insts = [], []
    for inst in host:
        rels = []
        for k, v in inst:
            tk = torch.from_numpy(k).cuda() if k.size else torch.empty(1, dtype=torch.int32, device="cuda")
            tv = torch.from_numpy(v).cuda() if v.size else torch.empty(1, dtype=torch.int32, device="cuda")
            keep += [tk, tv]
            rels.append((tk.data_ptr(), tv.data_ptr(), k.size))
        insts.append(rels)
    torch.cuda.synchronize()
    want = [bo.chain_result(inst) for inst in host]
    assert want[0][0] > 4000 and want[2][0] == 0 and want[3][0] == 0 and want[4][0] == 3
    assert want[5][0] > 150_000
    saved = engine.get_option("batch_part_log2")
    try:
        for mode, part in ((hj.BATCH_PERSISTENT, 12), (hj.BATCH_PERSISTENT, 8), (hj.BATCH_PLAIN, 12)):
            engine.set_option("batch_part_log2", part)
            rows, sums, redo = engine.batch_execute(insts, mode)
            assert [(int(a), int(b)) for a, b in zip(rows, sums)] == want, (mode, part)
            if mode == hj.BATCH_PERSISTENT:
                # 3000 equal build keys fit a 2^13-row table but not a 2^9-row one
                assert (redo >= 1) if part == 8 else (redo == 0), (part, redo)
    finally:
        engine.set_option("batch_part_log2", saved)


def test_batch_deep_chains_with_duplicates(engine, hj):
    """Chains of 3 to 8 relations with tens of thousands of probe rows: the
    rows that pass the first table are queued per warp for the later ones, so
    the queue fills, wraps and drains many times; duplicate keys in the first,
    a middle and the last table go through the odometer from each position."""
    import torch
    r = np.random.default_rng(17)
    dom = 4000

    def build(n, dup_frac):
        k = r.choice(dom, n, replace=False)
        d = r.choice(k, int(n * dup_frac), replace=False)
        k = np.concatenate([k, d, d[: d.size // 3]])
        return r.permutation(k), r.integers(-2**31, 2**31 - 1, k.size)

    host = []
    for m, dups in ((3, {1}), (3, set()), (4, {2}), (5, {4}), (6, {1, 3}), (8, set()), (8, {7})):
        rels = [(r.integers(0, dom, 40_000), r.integers(-2**31, 2**31 - 1, 40_000))]
        for j in range(1, m):
            rels.append(build(3000, 0.05 if j in dups else 0.0))
        host.append([(k.astype(np.int32), v.astype(np.int32)) for k, v in rels])
    keep, insts = [], []
    for inst in host:
        rels = []
        for k, v in inst:
            tk, tv = torch.from_numpy(k).cuda(), torch.from_numpy(v).cuda()
            keep += [tk, tv]
            rels.append((tk.data_ptr(), tv.data_ptr(), k.size))
        insts.append(rels)
    torch.cuda.synchronize()
    want = [bo.chain_result(inst) for inst in host]
    assert all(w[0] > 1000 for w in want)
    saved = engine.get_option("batch_part_log2")
    try:
        for mode, part in ((hj.BATCH_PERSISTENT, 12), (hj.BATCH_PERSISTENT, 9), (hj.BATCH_PLAIN, 12)):
            engine.set_option("batch_part_log2", part)
            rows, sums, redo = engine.batch_execute(insts, mode)
            assert [(int(a), int(b)) for a, b in zip(rows, sums)] == want, (mode, part)
            if mode == hj.BATCH_PERSISTENT:
                assert redo == 0
    finally:
        engine.set_option("batch_part_log2", saved)


def test_batch_rejects_bad_instances(engine, hj):
    import torch
    k = torch.zeros(4, dtype=torch.int32, device="cuda")
    with pytest.raises(hj.HjError) as e:
        engine.batch_execute([[(k.data_ptr(), k.data_ptr(), 4)]])
    assert e.value.status == hj.HJ_ERR_INVALID
    with pytest.raises(hj.HjError):
        engine.set_option("batch_part_log2", 3)
    with pytest.raises(hj.HjError):
        engine.batch_generate(1, 0, 1, 10, 0, 11, k.data_ptr(), k.data_ptr())  # build relation > build rows
    # the context stays usable
    rows, sums, _ = engine.batch_execute([[(k.data_ptr(), k.data_ptr(), 4), (k.data_ptr(), k.data_ptr(), 4)]])
    assert int(rows[0]) == 16


def test_autotuner_picks_options_without_changing_results(engine, hj, small_c4, small_c4_truth, tmp_path):
    from hjgb300 import autotune, batch
    cache = tmp_path / "tune.json"
    saved = {k: engine.get_option(k) for k in ("batch_part_log2", "batch_load_pct", "radix_bits", "probe_group")}
    try:
        t = autotune.tune(engine, small_c4, sample_instances=24, repeats=1, cache=cache)
        assert t["batched"]["batch_part_log2"] in autotune.BATCH_PART_LOG2
        assert t["plain"]["probe_group"] in autotune.PLAIN_PROBE_GROUP
        assert len(t["sweep"]["batched"]) == len(autotune.BATCH_PART_LOG2) * len(autotune.BATCH_LOAD_PCT)
        assert autotune.tune(engine, small_c4, cache=cache) == t  # served from the cache
        autotune.apply(engine, t)
        for mode in (hj.BATCH_PERSISTENT, hj.BATCH_PLAIN):
            rows, sums, _, _ = batch.run(engine, small_c4, mode, max_rows=1 << 40)
            assert np.array_equal(rows, small_c4_truth[0]) and np.array_equal(sums, small_c4_truth[1])
    finally:
        for k, v in saved.items():
            engine.set_option(k, v)
