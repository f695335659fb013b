"""Host page writers and readers: the engine's Table::to_columnar packing is the
reference's, page by page (defined bytes), and round-trips through the
oracle's independent reader."""
from __future__ import annotations

import importlib.util
import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def _mg():
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_writer_matches_reference_layout(hj):
    mg = _mg()
    kat = json.loads((GOLDEN / "writer_kat.json").read_text())
    ints, valid, data, offs, svalid = mg.writer_inputs()
    got = {
        "int32_dense": mg.page_digest(hj.Column.int32(ints).pages, 0),
        "int32_nulls": mg.page_digest(hj.Column.int32(ints, valid).pages, 0),
        "varchar_nulls_long": mg.page_digest(hj.Column.varchar(data, offs, svalid).pages, 3),
    }
    for k in kat:
        assert got[k] == kat[k], k


def test_oracle_writer_matches_reference_layout(orc):
    """The oracle's own page writers (the reference arm builds its inputs with
    them, without the engine library) are pinned to the same golden digests."""
    mg = _mg()
    kat = json.loads((GOLDEN / "writer_kat.json").read_text())
    ints, valid, data, offs, svalid = mg.writer_inputs()
    w = orc.page_writer
    got = {
        "int32_dense": mg.page_digest(w("int32", np.ascontiguousarray(ints, np.int32), None), 0),
        "int32_nulls": mg.page_digest(w("int32", np.ascontiguousarray(ints, np.int32),
                                        np.ascontiguousarray(valid, np.uint8)), 0),
        "varchar_nulls_long": mg.page_digest(w("strings", np.ascontiguousarray(data, np.uint8),
                                               np.ascontiguousarray(offs, np.uint64),
                                               np.ascontiguousarray(svalid, np.uint8)), 3),
    }
    for k in kat:
        assert got[k] == kat[k], k


def test_oracle_writer_equals_library_writer(hj, orc):
    r = np.random.default_rng(11)
    for n in (0, 1, 1984, 1985, 30000):
        v = r.integers(-2**31, 2**31, n, dtype=np.int64).astype(np.int32)
        for m in (None, (r.random(n) > 0.2).astype(np.uint8)):
            assert np.array_equal(hj.Column.int32(v, m).pages, orc.page_writer("int32", v, m))
        lens = r.integers(0, 70, n)
        lens[::997] = 9000
        offs = np.zeros(n + 1, np.uint64)
        np.cumsum(lens, out=offs[1:])
        data = r.integers(0x20, 0x7f, int(offs[-1]), dtype=np.uint8)
        for m in (None, (r.random(n) > 0.2).astype(np.uint8)):
            assert np.array_equal(hj.Column.varchar(data, offs, m).pages, orc.page_writer("strings", data, offs, m))


def test_writer_round_trip_through_oracle_reader(hj, orc):
    r = np.random.default_rng(5)
    n = 20000
    vals = r.integers(-2**31, 2**31, n, dtype=np.int64).astype(np.int32)
    valid = (r.random(n) > 0.25).astype(np.uint8)
    col = hj.Column.int32(vals, valid)
    dv, dm = orc.decode_column(0, col.pages)
    assert np.array_equal(dm, valid)
    assert np.array_equal(dv[valid == 1], vals[valid == 1])
    lens = r.integers(0, 120, n)
    lens[[5, 6]] = [8185, 8186]
    offs = np.zeros(n + 1, np.uint64)
    np.cumsum(lens, out=offs[1:])
    data = r.integers(0, 256, int(offs[-1]), dtype=np.uint8)
    sv = (r.random(n) > 0.1).astype(np.uint8)
    col = hj.Column.varchar(data, offs, sv)
    b, o, m = orc.decode_column(3, col.pages)
    assert np.array_equal(m, sv)
    for i in np.flatnonzero(sv)[:2000]:
        assert bytes(b[o[i]:o[i + 1]]) == bytes(data[offs[i]:offs[i + 1]])
    # the package's own reader agrees
    strs = hj.decode_varchar(col)
    for i in range(0, n, 97):
        want = bytes(data[offs[i]:offs[i + 1]]) if sv[i] else None
        assert strs[i] == want


def test_dense_int32_pages_hold_1984_rows(hj):
    col = hj.Column.int32(np.arange(5000, dtype=np.int32))
    nr = [int(p[0]) | int(p[1]) << 8 for p in col.pages]
    assert nr == [1984, 1984, 1032]


def test_empty_and_all_null_columns(hj, orc):
    assert hj.Column.int32(np.zeros(0, np.int32)).num_pages == 0
    col = hj.Column.int32(np.zeros(70000, np.int32), np.zeros(70000, np.uint8))
    v, m = orc.decode_column(0, col.pages)
    assert m.size == 70000 and not m.any()
    col = hj.Column.varchar([None] * 100 + [""] * 3)
    b, o, m = orc.decode_column(3, col.pages)
    assert m.tolist() == [0] * 100 + [1] * 3


def test_prefix_sum_packing_rule_fits_and_stays_near_greedy():
    """The VARCHAR page rule of the GPU writer (k_pack_count): a row costs
    8 * (2 + len) + 1 eighths of a byte (NULL: 1), a page holds sum <= cap =
    65497 eighths, and row i of a 4096-row tile goes to page floor(S_i / T)
    with S_i the exclusive prefix and T = cap - (largest cost in the tile).
    Checked here on random tiles: every page fits, none is empty, and the page
    count is at most cap / T times the greedy rule's (the reference's) plus one:
    within 1% for strings of up to 64 bytes."""
    cap = 65536 - 32 - 7
    rng = np.random.default_rng(12)
    for trial in range(40):
        n = int(rng.integers(1, 4097))
        hi = [16, 64, 300, 1000][trial % 4]
        lens = rng.integers(0, hi + 1, n)
        null = rng.random(n) < 0.1
        cost = np.where(null, 1, 8 * (2 + lens) + 1).astype(np.int64)
        T = cap - int(cost.max())
        S = np.concatenate([[0], np.cumsum(cost)[:-1]])
        page = S // T
        npages = int(page[-1]) + 1
        assert np.array_equal(np.unique(page), np.arange(npages))  # no empty page
        for p in range(npages):
            c = cost[page == p]
            nn = int((~null[page == p]).sum())
            nbytes = int(lens[(page == p) & ~null].sum())
            rows = int(c.size)
            assert 4 + 2 * nn + nbytes + (rows + 7) // 8 <= 8192
        greedy, cur = 1, 0  # greedy: append while the page still fits
        for c in cost:
            if cur + c > cap:
                greedy, cur = greedy + 1, 0
            cur += c
        # pages are at least T / cap full: at most cap / T times greedy's count,
        # which is within 1% for strings of up to 64 bytes
        assert npages <= greedy * cap / T + 1
        if hi <= 64:
            assert npages <= greedy * 1.01 + 1
