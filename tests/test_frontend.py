"""Plan front-end (hash-join-optimizer_gb300/frontend.py): SQL subset parsing, SQL
three-valued predicate evaluation, and EXPLAIN JSON -> Plan by the rules of the
reference's load_join_pipeline (tests/read_sql.cpp:868-1192).  The query, the
EXPLAIN tree and the tables here are synthetic; the converted plan's result is
checked against a brute-force evaluation of the same query, through the oracle on
the CPU and through the engine on the GPU."""
from __future__ import annotations

import itertools

import numpy as np
import pytest

I, V = 0, 3

SQL = """
SELECT MIN(c.name) AS cname, MIN(m.title) AS title, MIN(r.score) AS score
FROM company AS c, movie AS m, rating AS r
WHERE c.id = m.company_id
  AND m.id = r.movie_id
  AND c.country IN ('de', 'fr')
  AND (m.title LIKE '%the%' OR m.year BETWEEN 1990 AND 1999)
  AND m.year IS NOT NULL
  AND r.score > 3
  AND NOT r.kind = 2;
"""

SCHEMA = {
    "company": [("id", I), ("name", V), ("country", V)],
    "movie": [("id", I), ("company_id", I), ("title", V), ("year", I)],
    "rating": [("movie_id", I), ("score", I), ("kind", I)],
}


def explain():
    """Aggregate -> Gather -> Hash Join(r, Hash(Hash Join(Hash(c), m)))."""
    scan = lambda rel, alias: {"Node Type": "Seq Scan", "Relation Name": rel, "Alias": alias}  # noqa: E731
    inner = {"Node Type": "Hash Join", "Hash Cond": "(c.id = m.company_id)",
             "Plans": [{"Node Type": "Hash", "Plans": [scan("company", "c")]}, scan("movie", "m")]}
    top = {"Node Type": "Hash Join", "Hash Cond": "(r.movie_id = m.id)",
           "Plans": [scan("rating", "r"), {"Node Type": "Hash", "Plans": [inner]}]}
    return {"Plan": {"Node Type": "Aggregate", "Plans": [{"Node Type": "Gather", "Plans": [top]}]}}


def data(seed=3):
    r = np.random.default_rng(seed)
    nc, nm, nr = 300, 2000, 6000
    words = ["the", "a", "night", "them", "other", "blue"]
    company = {
        "id": (np.arange(nc), None),
        "name": ([None if r.random() < 0.1 else f"co{i}" for i in range(nc)], None),
        "country": ([[None, "de", "fr", "us", "uk"][r.integers(0, 5)] for _ in range(nc)], None),
    }
    movie = {
        "id": (np.arange(nm), None),
        "company_id": (r.integers(0, nc + 20, nm), (r.random(nm) > 0.05).astype(np.uint8)),
        "title": ([" ".join(r.choice(words, 2)) for _ in range(nm)], None),
        "year": (r.integers(1970, 2020, nm), (r.random(nm) > 0.1).astype(np.uint8)),
    }
    rating = {
        "movie_id": (r.integers(0, nm, nr), None),
        "score": (r.integers(0, 10, nr), (r.random(nr) > 0.1).astype(np.uint8)),
        "kind": (r.integers(0, 4, nr), (r.random(nr) > 0.2).astype(np.uint8)),
    }
    return {"company": company, "movie": movie, "rating": rating}


def brute_force(d):
    """The query, row by row, with SQL NULL semantics written out by hand."""
    def rows(t):
        cols = d[t]
        n = len(cols[next(iter(cols))][0])
        out = []
        for i in range(n):
            row = {}
            for k, (vals, valid) in cols.items():
                v = vals[i]
                ok = v is not None if valid is None else bool(valid[i])
                row[k] = (v.item() if hasattr(v, "item") else v) if ok else None
            out.append(row)
        return out
    cs = [c for c in rows("company") if c["country"] in ("de", "fr")]

    def movie_ok(m):
        like = m["title"] is not None and "the" in m["title"]
        between = m["year"] is not None and 1990 <= m["year"] <= 1999
        return (like or between) and m["year"] is not None
    ms = [m for m in rows("movie") if movie_ok(m)]
    rs = [x for x in rows("rating") if x["score"] is not None and x["score"] > 3
          and x["kind"] is not None and not x["kind"] == 2]
    out = []
    for c, m in itertools.product(cs, ms):
        if c["id"] is None or m["company_id"] is None or c["id"] != m["company_id"]:
            continue
        for x in rs:
            if m["id"] is not None and x["movie_id"] == m["id"]:
                out.append((c["name"], m["title"], x["score"]))
    return sorted(out, key=lambda t: tuple((v is None, v) for v in t))


def test_parse_sql(hj):
    from hjgb300 import frontend as fe
    p = fe.parse_sql(SQL)
    assert p.tables == {"c": "company", "m": "movie", "r": "rating"}
    assert p.join_graph["c"]["m"] == ("id", "company_id") and p.join_graph["m"]["c"] == ("company_id", "id")
    assert p.join_graph["r"]["m"] == ("movie_id", "id")
    assert p.output_attrs == [("c", "name"), ("m", "title"), ("r", "score")]
    assert [a[0] for a in p.aggregates] == ["MIN", "MIN", "MIN"]
    assert set(p.filters) == {"c", "m", "r"}
    assert p.filters["m"].kind == "and" and len(p.filters["m"].args) == 2
    with pytest.raises(fe.FrontEndError):
        fe.parse_sql("SELECT a.x FROM t AS a, u AS b WHERE a.x = 1 OR b.y = 2")
    with pytest.raises(fe.FrontEndError):
        fe.parse_sql("SELECT a.x FROM t AS a, u AS b WHERE a.x < b.y")
    with pytest.raises(fe.FrontEndError):
        fe.parse_sql("SELECT a.x FROM t AS a WHERE a.x ~ 3")


def test_filter_mask_three_valued(hj):
    from hjgb300 import frontend as fe
    x = (np.array([1, 5, 7, 0]), np.array([True, True, True, False]))
    s = (np.array(["the end", "xthe", None, "abc"], dtype=object), np.array([True, True, False, True]))
    cols = {"x": x, "s": s}
    m = lambda q: list(fe.filter_mask(fe.parse_sql(f"SELECT a.x FROM t AS a WHERE {q}").filters["a"], cols, 4))  # noqa: E731
    assert m("a.x > 3") == [False, True, True, False]
    assert m("NOT a.x > 3") == [True, False, False, False]          # NULL stays out
    assert m("a.x > 3 OR a.x IS NULL") == [False, True, True, True]
    # unknown AND false is false, so its NOT is true; NOT unknown stays unknown
    assert m("NOT (a.x > 3 AND a.s LIKE '%the%')") == [True, False, False, True]
    assert m("a.s LIKE 'the%'") == [True, False, False, False]
    assert m("a.s NOT LIKE '%the%'") == [False, False, False, True]
    assert m("a.x IN (0, 7)") == [False, False, True, False]
    assert m("a.x NOT IN (0, 7)") == [True, True, False, False]
    assert m("a.x BETWEEN 1 AND 5") == [True, True, False, False]
    assert m("a.s IS NULL") == [False, False, True, False]
    with pytest.raises(fe.FrontEndError):
        m("a.s > 3")


def _convert(hj, d):
    from hjgb300 import frontend as fe
    parsed = fe.parse_sql(SQL)
    plan, cols = fe.load_join_pipeline(explain(), parsed, SCHEMA, fe.table_loader(hj, d, SCHEMA), hj)
    return plan, cols


def test_pipeline_shape_and_oracle_result(hj, orc):
    d = data()
    plan, cols = _convert(hj, d)
    assert [(a, c) for a, c, _ in cols] == [("c", "name"), ("m", "title"), ("r", "score")]
    kinds = [n["kind"] if isinstance(n, dict) else getattr(n, "kind", None) for n in plan.nodes]
    assert len(plan.inputs) == 3 and len(plan.nodes) == 5, kinds
    out = orc.run(orc.port(), plan)
    assert out.status == 0, out.error
    rows = sorted(orc.canonical_rows(out), key=lambda t: tuple((v is None, v) for v in t))
    assert rows == brute_force(d)


def test_pipeline_rejections(hj):
    from hjgb300 import frontend as fe
    parsed = fe.parse_sql(SQL)
    load = fe.table_loader(hj, data(), SCHEMA)
    nl = {"Node Type": "Nested Loop", "Plans": [{"Node Type": "Seq Scan", "Alias": "c"},
                                                {"Node Type": "Seq Scan", "Alias": "m"}]}
    with pytest.raises(fe.FrontEndError, match="Not Hash Join"):
        fe.load_join_pipeline(nl, parsed, SCHEMA, load, hj)
    two_hash = {"Node Type": "Hash Join", "Plans": [{"Node Type": "Hash", "Plans": [{"Node Type": "Seq Scan", "Alias": "c"}]},
                                                     {"Node Type": "Hash", "Plans": [{"Node Type": "Seq Scan", "Alias": "m"}]}]}
    with pytest.raises(fe.FrontEndError, match="one Hash child"):
        fe.load_join_pipeline(two_hash, parsed, SCHEMA, load, hj)
    with pytest.raises(fe.FrontEndError, match="Cannot find alias"):
        fe.load_join_pipeline({"Node Type": "Seq Scan", "Alias": "zz"}, parsed, SCHEMA, load, hj)
    with pytest.raises(fe.FrontEndError, match="Not supported node type"):
        fe.load_join_pipeline({"Node Type": "Sort", "Plans": []}, parsed, SCHEMA, load, hj)


@pytest.mark.gpu
def test_pipeline_on_the_gpu(engine, hj, orc):
    d = data(seed=8)
    plan, _ = _convert(hj, d)
    res = engine.execute(plan)
    got = orc.summary(orc.Output(0, "", res.num_rows, [(c.type, c.pages) for c in res.columns]))
    want = orc.summary(orc.run(orc.port(), plan))
    assert got[:3] == want[:3] and np.array_equal(got[3], want[3])


def test_read_plans_json(hj, tmp_path):
    import json
    from hjgb300 import frontend as fe
    f = tmp_path / "plans.json"
    f.write_text(json.dumps({"sql_directory": "q", "names": ["x1"], "plans": [explain()]}))
    d, plans = fe.read_plans_json(f)
    assert d == "q" and list(plans) == ["x1"]
    parsed = fe.parse_sql(SQL)
    plan, _ = fe.load_join_pipeline(plans["x1"], parsed, SCHEMA, fe.table_loader(hj, data(), SCHEMA), hj)
    assert len(plan.nodes) == 5


def test_parse_sql_forms(hj):
    """Aliases without AS, nested groups, NOT IN over strings, comments, no WHERE."""
    from hjgb300 import frontend as fe
    p = fe.parse_sql("""SELECT a.x, MIN(b.y) -- comment
                        FROM t a, u b
                        WHERE a.k = b.k AND ((a.s NOT IN ('p', 'q''s') AND a.x <> 3) OR a.x IS NULL)""")
    assert p.tables == {"a": "t", "b": "u"}
    assert p.aggregates == [("", "a", "x"), ("MIN", "b", "y")]
    f = p.filters["a"]
    assert f.kind == "or" and f.args[0].kind == "and"
    assert f.args[0].args[0].kind == "not" and f.args[0].args[0].args[0].value == ["p", "q's"]
    q = fe.parse_sql("SELECT a.x FROM t AS a;")
    assert q.filters == {} and q.join_graph == {"a": {}}
    with pytest.raises(fe.FrontEndError):
        fe.parse_sql("SELECT a.x FROM t AS a, t AS a")
    with pytest.raises(fe.FrontEndError):
        fe.parse_sql("SELECT z.x FROM t AS a")
