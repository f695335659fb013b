"""Binary table files: the engine writes the reference's cache format byte
for byte (DumpTable) and reads files the reference writes (Table::from_cache
restated by hj_table_load); on the GPU a loaded table joins exactly like the
host table it came from."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest



def _table(hj):
    r = np.random.default_rng(11)
    n = 6000
    strs = [("x" * int(k)) if k < 40 else ("long" * 3000) for k in r.integers(0, 41, n)]
    data = "".join(strs).encode()
    offs = np.zeros(n + 1, np.uint64)
    np.cumsum([len(x) for x in strs], out=offs[1:])
    return hj.Table(n, [hj.Column.int32(r.integers(-99, 99, n).astype(np.int32), (r.random(n) > 0.2).astype(np.uint8)),
                        hj.Column.varchar(np.frombuffer(data, np.uint8), offs, (r.random(n) > 0.1).astype(np.uint8)),
                        hj.Column.int32(np.arange(n, dtype=np.int32))])


def test_dump_matches_reference_dump_and_from_cache(hj, orc, tmp_path):
    t = _table(hj)
    ours, theirs = tmp_path / "ours.tbl", tmp_path / "ref.tbl"
    hj.dump_table(t, ours)
    size = 8192 * (1 + sum(c.num_pages for c in t.columns))
    assert ours.stat().st_size == size
    head = np.fromfile(str(ours), np.uint8, count=208)
    assert tuple(head[:16].view(np.uint64)) == (t.num_rows, 3)
    ref = orc.ref()
    if ref is None:
        pytest.skip("reference build not available")
    td_cols = (hj.ColumnDesc * 3)()
    keep = []
    for j, col in enumerate(t.columns):
        td_cols[j].type, td_cols[j].num_pages, td_cols[j].pages = col.type, col.num_pages, hj._page_ptrs(col, keep)
    td = hj.TableDesc(t.num_rows, 3, td_cols, 0)
    ref.ref_dump_table.argtypes = [C.c_void_p, C.c_char_p]
    assert ref.ref_dump_table(C.addressof(td), str(theirs).encode()) == 0
    assert ours.read_bytes() == theirs.read_bytes()
    # the reference reads our file back to the same pages
    ref.ref_from_cache.argtypes = [C.c_char_p, C.POINTER(orc.OracleResult)]
    r = orc.OracleResult()
    assert ref.ref_from_cache(str(ours).encode(), C.byref(r)) == 0
    back = orc._collect(ref, r)
    assert back.num_rows == t.num_rows
    for (ty, pages), col in zip(back.columns, t.columns):
        assert ty == col.type and np.array_equal(pages, col.pages)


@pytest.mark.gpu
def test_loaded_table_joins_like_the_host_table(engine, hj, orc, tmp_path):
    from hjgb300 import workloads
    w = workloads.c1(scale=0.01)
    paths = []
    for i, t in enumerate(w.plan.inputs):
        paths.append(tmp_path / f"t{i}.tbl")
        hj.dump_table(t, paths[-1])
    loaded = [engine.load_table(p) for p in paths]
    try:
        assert [t.num_rows for t in loaded] == [t.num_rows for t in w.plan.inputs]
        a = engine.execute(hj.Plan(w.plan.nodes, loaded, w.plan.root))
        b = engine.execute(w.plan)
        sa = orc.summary(orc.Output(0, "", a.num_rows, [(c.type, c.pages) for c in a.columns]))
        sb = orc.summary(orc.Output(0, "", b.num_rows, [(c.type, c.pages) for c in b.columns]))
        assert sa[:3] == sb[:3] and np.array_equal(sa[3], sb[3])
    finally:
        for t in loaded:
            engine.release(t)
    bad = tmp_path / "bad.tbl"
    bad.write_bytes(paths[0].read_bytes()[:-100])  # truncated
    with pytest.raises(hj.HjError):
        engine.load_table(bad)
