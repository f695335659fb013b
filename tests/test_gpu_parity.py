"""GPU results through the C ABI against the oracle and the reference's
recorded answers.  Bit-exact: same row count, same multiset of rows (sorted
rows for small results, sorted 64-bit row fingerprints and their sum for
large ones); NULLs and string bytes included."""
from __future__ import annotations

import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import cases
from conftest import canon

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def gpu_out(orc, res):
    """engine Result -> oracle Output (so the oracle's reader checks it)."""
    return orc.Output(0, "", res.num_rows, [(c.type, c.pages) for c in res.columns])


def assert_same(orc, gpu_res, ref_out, what=""):
    g = orc.summary(gpu_out(orc, gpu_res))
    r = orc.summary(ref_out)
    assert g[0] == r[0], f"{what}: num_rows {g[0]} != {r[0]}"
    assert g[1] == r[1], f"{what}: column rows {g[1]} != {r[1]}"
    assert g[2] == r[2], f"{what}: checksum differs"
    assert np.array_equal(g[3], r[3]), f"{what}: row multisets differ"


@pytest.fixture(scope="module")
def unit_cases(hj):
    return cases.build_cases(hj)


def test_unit_cases_match_reference(engine, orc, unit_cases):
    gold = json.loads((GOLDEN / "unit_cases.json").read_text())
    for name, (plan, truth, types) in unit_cases.items():
        res = engine.execute(plan)
        out = gpu_out(orc, res)
        assert [c.type for c in res.columns] == types, name
        rows = canon(orc.canonical_rows(out))
        assert res.num_rows == gold[name]["num_rows"], name
        assert rows == canon(gold[name]["rows"]), name
        if truth is not None:
            assert rows == canon(truth), name


def test_seeded_small_workloads_match_reference_checksums(engine, orc):
    from hjgb300 import workloads
    gold = json.loads((GOLDEN / "configs_small.json").read_text())
    for name, g in gold.items():
        w = getattr(workloads, name)(scale=g["scale"])
        res = engine.execute(w.plan)
        n, counts, cks, _ = orc.summary(gpu_out(orc, res))
        assert (n, counts, str(cks)) == (g["num_rows"], g["column_rows"], g["checksum"]), name


@pytest.mark.parametrize("name,scale", [("c1", 1.0), ("c2", 1 / 16), ("c3", 0.1), ("c3", 1.0), ("c2", 0.01),
                                        ("c2", 1.0)])
def test_workloads_match_oracle(engine, orc, name, scale):
    from hjgb300 import workloads
    w = getattr(workloads, name)(scale=scale)
    res = engine.execute(w.plan)
    if w.expected_rows >= 0:
        assert res.num_rows == w.expected_rows
    assert_same(orc, res, orc.run(orc.port(), w.plan), f"{name}@{scale}")


def test_result_counters_describe_the_built_tables(engine, hj):
    """hj_result_counter: the c1 build side (1M unique keys) gives one table of
    1M tuples with UnchainedHash's next_pow2 directory, 2^20 + 1 words."""
    from hjgb300 import workloads
    w = workloads.c1(scale=1.0)
    r = engine.execute_raw(w.plan)
    try:
        cnt = engine.counters(r)
        b, p, o, _ = engine.stats(r)
    finally:
        engine.free_result(r)
    assert cnt["joins"] == 1 and cnt["table_tuples"] == 1_000_000
    assert cnt["dir_words"] == (1 << 20) + 1
    assert (b, p, o) == (1_000_000, 10_000_000, 10_000_000)
    assert cnt["launches"] > 0


def test_c2_full_size_properties(engine, orc):
    """16M x 256M (pre-filtered to ~25.6M): exact row count from the key
    histograms, every column the same length, and the oracle's checksum."""
    from hjgb300 import workloads
    w = workloads.c2(1.0)
    res = engine.execute(w.plan)
    assert res.num_rows == w.expected_rows
    out = gpu_out(orc, res)
    n, counts, cks, fp = orc.summary(out)
    assert n == w.expected_rows and all(c == n for c in counts)
    r = orc.summary(orc.run(orc.port(), w.plan))
    assert (n, counts, cks) == r[:3]
    assert np.array_equal(fp, r[3])


def test_results_independent_of_tunables(engine, orc):
    from hjgb300 import workloads
    w = workloads.c2(0.004)
    want = orc.summary(orc.run(orc.port(), w.plan))
    for opt in ({"probe_group": 1}, {"probe_group": 4}, {"probe_group": 32}, {"light_max": 1},
                {"light_max": 4}, {"dir_bits": 8}, {"dir_bits": 20}, {"radix_bits": 0}, {"radix_bits": 6},
                {"dir_cap_bits": 10}, {"dir_cap_bits": 32}):
        saved = {k: engine.get_option(k) for k in opt}
        try:
            for k, v in opt.items():
                engine.set_option(k, v)
            got = orc.summary(gpu_out(orc, engine.execute(w.plan)))
        finally:
            for k, v in saved.items():
                engine.set_option(k, v)
        assert got[:3] == want[:3], opt
        assert np.array_equal(got[3], want[3]), opt


def _irregular_int32(hj, vals, valid, rows_per_page):
    """An INT32 column written in chunks of `rows_per_page` rows, so that its
    pages are not the 1984-row dense pages read in place."""
    pages = [hj.Column.int32(vals[i:i + rows_per_page], None if valid is None else valid[i:i + rows_per_page]).pages
             for i in range(0, vals.size, rows_per_page)]
    return hj.Column(hj.INT32, np.concatenate(pages))


@pytest.mark.parametrize("form", ["pages", "plain", "tagged"])
def test_probe_key_forms(engine, orc, hj, form):
    """Probe keys staged in shared memory by bulk copies from each of their
    device forms: dense pages read in place, decoded int32 (irregular pages
    without NULLs) and value_t (with NULLs); tile ends at odd row counts and a
    Zipf-heavy key whose bucket length saturates the summary.  Checked against
    the join computed in numpy; for pages and value_t also against the oracle.
    (For irregular pages without NULLs the reference's direct mode reads row r
    at page r / 1984, past the rows those pages hold; the engine decodes such
    pages by their headers, a difference listed with the others.)"""
    r = np.random.default_rng(17)
    nb, npr = 120_001, 333_337
    bkey = (r.zipf(1.3, nb) % 30_000).astype(np.int32)
    bkey[:40_000] = 12345                     # a bucket far above the summary's length field
    pkey = r.integers(-5, 32_000, npr).astype(np.int32)
    pkey[::50_000] = 12345
    pval = None if form != "tagged" else (r.random(npr) > 0.1).astype(np.uint8)
    if form == "pages":
        pcol = hj.Column.int32(pkey)
    else:
        pcol = _irregular_int32(hj, pkey, pval, 1001)
    build = hj.Table(nb, [hj.Column.int32(bkey), hj.Column.int32(np.arange(nb, dtype=np.int32))])
    probe = hj.Table(npr, [pcol, hj.Column.int32(np.arange(npr, dtype=np.int32))])
    p = hj.Plan()
    p.new_input(build)
    p.new_input(probe)
    p.new_scan_node(0, [(0, hj.INT32), (1, hj.INT32)])
    p.new_scan_node(1, [(0, hj.INT32), (1, hj.INT32)])
    p.root = p.new_join_node(True, 0, 1, 0, 0, [(0, hj.INT32), (1, hj.INT32), (3, hj.INT32)])
    res = engine.execute(p)
    # the join in numpy: (key, build row, probe row) for every equal-key pair
    ok = np.ones(npr, bool) if pval is None else pval.astype(bool)
    order = np.argsort(bkey, kind="stable")
    sk = bkey[order]
    lo = np.searchsorted(sk, pkey, "left")
    hi = np.searchsorted(sk, pkey, "right")
    cnt = np.where(ok, hi - lo, 0)
    prow = np.repeat(np.arange(npr), cnt)
    start = np.repeat(lo, cnt)
    k = np.arange(prow.size) - np.repeat(np.cumsum(cnt) - cnt, cnt)
    brow = order[start + k]
    want = np.sort(pkey[prow].astype(np.int64) << 40 | brow.astype(np.int64) << 20 | prow)
    got_cols = [hj.decode_int32(c)[0].astype(np.int64) for c in res.columns]
    got = np.sort(got_cols[0] << 40 | got_cols[1] << 20 | got_cols[2])
    assert res.num_rows == want.size
    assert np.array_equal(got, want), form
    if form != "plain":
        assert_same(orc, res, orc.run(orc.port(), p), form)


def test_resident_tables_give_the_same_result(engine, orc, hj):
    from hjgb300 import workloads
    w = workloads.c2(0.01)
    host = engine.execute(w.plan)
    res_plan = hj.Plan(w.plan.nodes, [engine.upload(t) for t in w.plan.inputs], w.plan.root)
    try:
        a = engine.execute(res_plan)
        b = engine.execute(res_plan)
    finally:
        for t in res_plan.inputs:
            engine.release(t)
    sh = orc.summary(gpu_out(orc, host))
    for r in (a, b):
        s = orc.summary(gpu_out(orc, r))
        assert s[:3] == sh[:3] and np.array_equal(s[3], sh[3])


def test_host_transfer_paths_agree(engine, orc):
    """Pages moved by the GPU over host memory access and pages staged by host
    threads through pinned memory give the same result."""
    from hjgb300 import workloads
    w = workloads.c2(0.01)
    want = orc.summary(orc.run(orc.port(), w.plan))
    saved = engine.get_option("host_access")
    try:
        for v in (0, 1):
            engine.set_option("host_access", v)
            got = orc.summary(gpu_out(orc, engine.execute(w.plan)))
            assert got[:3] == want[:3] and np.array_equal(got[3], want[3]), v
    finally:
        engine.set_option("host_access", saved)


def test_probe_side_int32_outputs_and_type_mismatches(engine, orc, hj):
    """Probe-side INT32 columns with NULLs on pages of irregular row counts as
    output columns; the same INT32 column output as INT32 and as VARCHAR (all
    NULL through the matches: NULL strings), and a non-NULL value through the
    matches in a VARCHAR output (the reference's error)."""
    I, V = cases.I, cases.V
    r = np.random.default_rng(23)
    n = 100_000
    keys = r.integers(0, 20_000, n)
    pay = [None if x else int(v) for x, v in zip(r.random(n) < 0.3, r.integers(-2**31, 2**31 - 1, n))]
    pay2 = [None if x else int(v) for x, v in zip(r.random(n) < 0.05, r.integers(-5, 5, n))]
    build = cases.table(hj, [[k, f"s{k}"] for k in range(0, 20_000, 3)], [I, V])
    probe = cases.table(hj, [[int(k), a, b] for k, a, b in zip(keys, pay, pay2)], [I, I, I])
    p = hj.Plan()
    p.new_input(build)
    p.new_input(probe)
    p.new_scan_node(0, [(0, I), (1, V)])
    p.new_scan_node(1, [(0, I), (1, I), (2, I)])
    p.root = p.new_join_node(True, 0, 1, 0, 0, [(3, I), (0, I), (4, I), (1, V)])
    assert_same(orc, engine.execute(p), orc.run(orc.port(), p), "probe-side INT32 outputs")
    # the same INT32 column as INT32 and as VARCHAR output, all NULL through the matches
    b = cases.table(hj, [[1, "x"], [2, "y"], [5, "z"]], [I, V])
    pr = cases.table(hj, [[1, None], [2, None], [3, 7], [4, 8], [1, None], [5, None], [9, 11]], [I, I])
    p = hj.Plan()
    p.new_input(b)
    p.new_input(pr)
    p.new_scan_node(0, [(0, I), (1, V)])
    p.new_scan_node(1, [(0, I), (1, I)])
    p.root = p.new_join_node(True, 0, 1, 0, 0, [(3, I), (3, V), (1, V), (2, I)])
    want = orc.run(orc.port(), p)
    assert want.status == 0
    assert_same(orc, engine.execute(p), want, "INT32 column as VARCHAR output")
    # a non-NULL value through the matches: the reference's error
    pr = cases.table(hj, [[1, None], [2, 6], [5, None]], [I, I])
    p = hj.Plan()
    p.new_input(b)
    p.new_input(pr)
    p.new_scan_node(0, [(0, I), (1, V)])
    p.new_scan_node(1, [(0, I), (1, I)])
    p.root = p.new_join_node(True, 0, 1, 0, 0, [(3, I), (3, V)])
    assert orc.run(orc.port(), p).status != 0
    with pytest.raises(hj.HjError) as e:
        engine.execute(p)
    assert e.value.status == hj.HJ_ERR_RUNTIME and "not string or null" in str(e.value)


def test_error_classes(engine, hj):
    p = hj.Plan()
    t = cases.table(hj, [["a"], ["b"]], [cases.V])
    p.new_input(t)
    p.new_input(t)
    p.new_scan_node(0, [(0, cases.V)])
    p.new_scan_node(1, [(0, cases.V)])
    p.root = p.new_join_node(True, 0, 1, 0, 0, [(0, cases.V)])
    with pytest.raises(hj.HjError) as e:
        engine.execute(p)
    assert e.value.status == hj.HJ_ERR_RUNTIME and "int32" in str(e.value)
    p = hj.Plan()
    for _ in range(1025):
        p.new_input(cases.table(hj, [[1, "x"]], [cases.I, cases.V]))
    p.new_scan_node(1024, [(1, cases.V)])
    p.root = 0
    with pytest.raises(hj.HjError) as e:
        engine.execute(p)
    assert e.value.status == hj.HJ_ERR_OUT_OF_RANGE and "table" in str(e.value)
    # the context stays usable after an error
    plan, truth, _ = cases.build_cases(hj)["simple_join"]
    assert engine.execute(plan).num_rows == 3


# ---------------------------------------------------------- hash-table C ABI --

class _Dev:
    """Zero-copy view of device memory for torch (CUDA array interface)."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False),
                                         "version": 3}


def _kat_keys(spec):
    import importlib.util
    s = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    m = importlib.util.module_from_spec(s)
    s.loader.exec_module(m)
    return m.kat_keys(spec)


def test_table_directory_is_unchained_hash_directory(engine, hj):
    """hj_table_build gives the reference UnchainedHash's directory words."""
    import ctypes as C
    import torch
    L = hj.lib()
    kat = json.loads((GOLDEN / "unchained_kat.json").read_text())
    for name, e in kat.items():
        keys = torch.from_numpy(_kat_keys(e["spec"])).cuda()
        t = C.c_void_p()
        assert L.hj_table_build(engine.handle, keys.data_ptr(), None, keys.numel(), -1, C.byref(t)) == 0
        try:
            bits, nt, d = C.c_uint32(), C.c_uint64(), C.c_void_p()
            L.hj_table_info(t, C.byref(bits), C.byref(nt), C.byref(d), None, None)
            assert nt.value == keys.numel()
            n = (1 << bits.value) + 1
            assert n == e["dir_size"], name
            dev = torch.as_tensor(_Dev(d.value, n, "<u8"), device="cuda").cpu().numpy().astype("<u8")
            if "dir" in e:
                assert [int(x) for x in dev] == e["dir"], name
            assert hashlib.sha256(dev.tobytes()).hexdigest() == e["sha256"], name
        finally:
            L.hj_table_free(t)


def test_table_probe_pairs(engine, hj, orc):
    import ctypes as C
    import torch
    L = hj.lib()
    r = np.random.default_rng(9)
    build = (r.zipf(1.2, 200_000) % 50_000).astype(np.int32)
    build[:3] = [2**31 - 1, -(2**31), -7]
    probe = r.integers(-100, 60_000, 300_000).astype(np.int32)
    valid = (r.random(probe.size) > 0.1)
    bits = np.packbits(valid.astype(np.uint8), bitorder="little")
    bits = np.pad(bits, (0, (-bits.size) % 4)).view(np.uint32)
    want = orc.unchained_counts(build, probe) * valid
    kb, kp = torch.from_numpy(build).cuda(), torch.from_numpy(probe).cuda()
    vb = torch.from_numpy(bits.copy()).cuda()
    t = C.c_void_p()
    assert L.hj_table_build(engine.handle, kb.data_ptr(), None, kb.numel(), -1, C.byref(t)) == 0
    try:
        nm = C.c_uint64()
        rc = L.hj_table_probe(engine.handle, t, kp.data_ptr(), vb.data_ptr(), kp.numel(), None, None, 0,
                              C.byref(nm))
        assert rc == hj.HJ_ERR_CAPACITY and nm.value == int(want.sum())
        op = torch.empty(nm.value, dtype=torch.int32, device="cuda")
        ob = torch.empty(nm.value, dtype=torch.int32, device="cuda")
        assert L.hj_table_probe(engine.handle, t, kp.data_ptr(), vb.data_ptr(), kp.numel(), op.data_ptr(),
                                ob.data_ptr(), nm.value, C.byref(nm)) == 0
        pr, br = op.cpu().numpy(), ob.cpu().numpy()
        assert np.array_equal(probe[pr], build[br])          # every pair is a match
        assert np.array_equal(np.bincount(pr, minlength=probe.size), want)  # and all are there
        assert np.unique(pr.astype(np.int64) << 32 | br).size == pr.size   # no duplicates
        # keys at a 4-byte offset (no 16-byte alignment for the bulk copies):
        # read by direct loads, same matches
        ku = kp[1:]
        want_u = orc.unchained_counts(build, probe[1:])
        rc = L.hj_table_probe(engine.handle, t, ku.data_ptr(), None, ku.numel(), None, None, 0, C.byref(nm))
        assert rc == hj.HJ_ERR_CAPACITY and nm.value == int(want_u.sum())
        op = torch.empty(nm.value, dtype=torch.int32, device="cuda")
        ob = torch.empty(nm.value, dtype=torch.int32, device="cuda")
        assert L.hj_table_probe(engine.handle, t, ku.data_ptr(), None, ku.numel(), op.data_ptr(),
                                ob.data_ptr(), nm.value, C.byref(nm)) == 0
        pr, br = op.cpu().numpy(), ob.cpu().numpy()
        assert np.array_equal(probe[1:][pr], build[br])
        assert np.array_equal(np.bincount(pr, minlength=probe.size - 1), want_u)
    finally:
        L.hj_table_free(t)


def test_large_skewed_builds_match_unchained_hash(engine, hj, orc):
    """Builds of 2^21 keys whose partitions exceed one block's shared memory
    (Zipf-heavy keys, and 150 keys of 13,000 tuples, several sharing a
    partition): the same directory words as UnchainedHash, and every probe
    match found."""
    import ctypes as C
    import torch
    L = hj.lib()
    r = np.random.default_rng(11)
    n = 1 << 21
    zipf = r.permutation(np.arange(1 << 19, dtype=np.int64))[(r.zipf(1.15, n) - 1) % (1 << 19)].astype(np.int32)
    zipf[:4] = [2**31 - 1, -(2**31), -7, 0]
    heavy = r.choice(np.arange(-(1 << 29), 1 << 29, dtype=np.int64), 150, replace=False).astype(np.int32)
    flat = np.concatenate([np.repeat(heavy, 13_000),
                           r.integers(-(1 << 30), 1 << 30, n - 1_950_000).astype(np.int32)])
    flat = flat[r.permutation(n)]
    for build in (zipf, flat):
        # every distinct build key once (n matches in all), and keys that miss
        probe = np.concatenate([r.permutation(np.unique(build)),
                                r.integers(1 << 20, 1 << 21, 100_000).astype(np.int32) | (1 << 30)])
        want_dir = orc.unchained_directory(build)
        want = orc.unchained_counts(build, probe)
        kb, kp = torch.from_numpy(build).cuda(), torch.from_numpy(probe).cuda()
        t = C.c_void_p()
        assert L.hj_table_build(engine.handle, kb.data_ptr(), None, kb.numel(), -1, C.byref(t)) == 0
        try:
            bits, nt, d = C.c_uint32(), C.c_uint64(), C.c_void_p()
            L.hj_table_info(t, C.byref(bits), C.byref(nt), C.byref(d), None, None)
            assert nt.value == n
            dev = torch.as_tensor(_Dev(d.value, (1 << bits.value) + 1, "<u8"), device="cuda").cpu().numpy()
            assert np.array_equal(dev.astype(np.uint64), want_dir.astype(np.uint64))
            nm = C.c_uint64()
            rc = L.hj_table_probe(engine.handle, t, kp.data_ptr(), None, kp.numel(), None, None, 0, C.byref(nm))
            assert rc == hj.HJ_ERR_CAPACITY and nm.value == int(want.sum())
            op = torch.empty(nm.value, dtype=torch.int32, device="cuda")
            ob = torch.empty(nm.value, dtype=torch.int32, device="cuda")
            assert L.hj_table_probe(engine.handle, t, kp.data_ptr(), None, kp.numel(), op.data_ptr(),
                                    ob.data_ptr(), nm.value, C.byref(nm)) == 0
            pr, br = op.cpu().numpy(), ob.cpu().numpy()
            assert np.array_equal(probe[pr], build[br])
            assert np.array_equal(np.bincount(pr, minlength=probe.size), want)
            assert np.unique(pr.astype(np.int64) << 32 | br).size == pr.size
        finally:
            L.hj_table_free(t)


def _varchar_pages_fit(pages):
    """Every normal VARCHAR page fits (header, offsets, bytes, bitmap) with
    non-decreasing offsets; returns the number of normal pages."""
    normal = 0
    for pg in pages:
        h = pg[:4].view(np.uint16)
        rows, nn = int(h[0]), int(h[1])
        if rows in (0xFFFF, 0xFFFE):
            continue
        normal += 1
        offs = pg[4:4 + 2 * nn].view(np.uint16).astype(np.int64)
        assert nn <= rows and np.all(np.diff(offs) >= 0)
        end = int(offs[-1]) if nn else 0
        assert 4 + 2 * nn + end + (rows + 7) // 8 <= 8192
    return normal


def test_varchar_page_packing_both_rules(engine, orc, hj):
    """Output VARCHAR pages are packed per 4096-row tile by prefix sums (short
    strings) or by the greedy rule (a tile with a string over ~1 KB or a long
    string).  Both give the oracle's rows, every page fits, and the prefix-sum
    tiles use at most ~1% more pages than a greedy packing."""
    r = np.random.default_rng(5)
    n = 5 * 4096 + 77
    strs = [None if r.random() < 0.15 else "v" * int(r.integers(0, 65)) for _ in range(n)]
    strs[4096 + 10] = "K" * 2000          # tile 1: a row over kCap / 8 -> greedy
    strs[3 * 4096 + 5] = "L" * 9000       # tile 3: a long string -> greedy
    keys = list(range(n))
    build = cases.table(hj, [[k, s] for k, s in zip(keys, strs)], [cases.I, cases.V])
    probe = cases.table(hj, [[k] for k in keys], [cases.I])
    p = hj.Plan()
    cases._two_scans(hj, p, build, probe, [(0, cases.I), (1, cases.V)], [(0, cases.I)])
    p.root = p.new_join_node(True, 0, 1, 0, 0, [(1, cases.V), (2, cases.I)])
    res = engine.execute(p)
    assert_same(orc, res, orc.run(orc.port(), p), "varchar packing")
    normal = _varchar_pages_fit(res.columns[0].pages)
    bytes_ = sum(2 + len(s) for s in strs if s is not None and len(s) <= 8185) + n / 8
    assert normal <= bytes_ / 8000 + 6 * 2
