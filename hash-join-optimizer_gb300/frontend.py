"""Plan front-end: PostgreSQL EXPLAIN JSON plus the query's SQL -> a join Plan.

The reference turns the `plans.json` it ships (EXPLAIN (FORMAT JSON) output of
each query) and the query's SQL text into a `Plan` for `execute()`
(`load_join_pipeline`, tests/read_sql.cpp:868-1192).  This module does the same
for this engine, by the same rules:

* Aggregate and Gather nodes are looked through (their first child).
* Only Hash Join nodes join.  One child must be a Hash node; the side under the
  Hash is the build side (`build_left` when it is the first child).
* The join condition is the SQL's equi-join between an alias on the left and an
  alias on the right (the EXPLAIN `Hash Cond` is not parsed, as in the reference).
* Seq Scan / Index Only Scan nodes become scan nodes over an input table of their
  alias.  The input table comes from a caller-supplied loader, with the alias's
  predicates already applied.  The reference also filters while loading
  (Table::from_csv with the filter, src/build_table.cpp:321-370).
* Each node outputs exactly the attributes its parent needs: the join keys plus
  what is required above.  The root outputs the SELECT list's columns, in order.

The SQL parser covers the subset such join queries use:
- `SELECT MIN(a.x) AS n, ... | a.x, ...`
- `FROM table AS alias, ...`
- a WHERE clause that is an AND of:
  - equi-joins `a.x = b.y`;
  - single-alias predicates: `=, <>, !=, <, >, <=, >=` against literals,
    `[NOT] LIKE`, `[NOT] IN (...)`, `IS [NOT] NULL` and `[NOT] BETWEEN`;
  - parenthesised OR / AND groups of the single-alias predicates.

`filter_mask` evaluates a predicate on host columns with SQL semantics: a
comparison with NULL is not true, and NOT of unknown stays unknown.
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

INT32, INT64, FP64, VARCHAR = 0, 1, 2, 3


class FrontEndError(ValueError):
    """A plan or query outside what the front-end (and the reference's) accepts."""


# ------------------------------------------------------------------ SQL --------

_TOKEN = re.compile(r"""
    \s*(?:
      (?P<num>-?\d+(?:\.\d+)?)
    | (?P<str>'(?:[^']|'')*')
    | (?P<op><=|>=|<>|!=|=|<|>)
    | (?P<punct>[(),;*])
    | (?P<name>[A-Za-z_][A-Za-z_0-9]*(?:\.[A-Za-z_][A-Za-z_0-9]*)?)
    )""", re.X)


def _tokens(sql: str) -> List[Tuple[str, str]]:
    out, pos = [], 0
    sql = re.sub(r"--[^\n]*", " ", sql)
    while pos < len(sql):
        if sql[pos:].strip() == "":
            break
        m = _TOKEN.match(sql, pos)
        if not m:
            raise FrontEndError(f"cannot tokenize SQL at: {sql[pos:pos + 30]!r}")
        kind = m.lastgroup
        val = m.group(kind)
        if kind == "str":
            val = val[1:-1].replace("''", "'")
        out.append((kind, val))
        pos = m.end()
    return out


@dataclass
class Pred:
    """A predicate tree on one alias: kind is 'and' / 'or' / 'not' (args) or a leaf:
    'cmp' (op, value), 'like' (pattern), 'in' (values), 'null', 'between' (lo, hi)."""
    kind: str
    column: str = ""
    op: str = ""
    value: object = None
    args: List["Pred"] = field(default_factory=list)

    def aliases(self) -> set:
        if self.kind in ("and", "or", "not"):
            s = set()
            for a in self.args:
                s |= a.aliases()
            return s
        return {self.column.split(".")[0]}


@dataclass
class ParsedSQL:
    tables: Dict[str, str]                                  # alias -> table
    join_graph: Dict[str, Dict[str, Tuple[str, str]]]       # alias -> {alias: (own column, its column)}
    filters: Dict[str, Pred]                                # alias -> AND of its predicates
    output_attrs: List[Tuple[str, str]]                     # (alias, column), SELECT order
    aggregates: List[Tuple[str, str, str]]                  # (function or '', alias, column)


class _Parser:
    def __init__(self, toks):
        self.t, self.i = toks, 0

    def peek(self, k=0):
        return self.t[self.i + k] if self.i + k < len(self.t) else ("eof", "")

    def kw(self, word, k=0):
        kind, val = self.peek(k)
        return kind == "name" and val.upper() == word

    def take(self):
        tok = self.peek()
        self.i += 1
        return tok

    def expect(self, kind, val=None):
        k, v = self.take()
        if k != kind or (val is not None and v.upper() != val.upper()):
            raise FrontEndError(f"expected {val or kind}, got {v!r}")
        return v

    def literal(self):
        kind, val = self.take()
        if kind == "num":
            return float(val) if "." in val else int(val)
        if kind == "str":
            return val
        raise FrontEndError(f"expected a literal, got {val!r}")

    def column(self):
        kind, val = self.take()
        if kind != "name" or "." not in val:
            raise FrontEndError(f"expected alias.column, got {val!r}")
        return val

    # boolean expression: or_expr := and_expr (OR and_expr)*
    def or_expr(self):
        args = [self.and_expr()]
        while self.kw("OR"):
            self.take()
            args.append(self.and_expr())
        return args[0] if len(args) == 1 else Pred("or", args=args)

    def and_expr(self):
        args = [self.factor()]
        while self.kw("AND"):
            self.take()
            args.append(self.factor())
        return args[0] if len(args) == 1 else Pred("and", args=args)

    def factor(self):
        if self.peek() == ("punct", "("):
            self.take()
            e = self.or_expr()
            self.expect("punct", ")")
            return e
        if self.kw("NOT"):
            self.take()
            return Pred("not", args=[self.factor()])
        return self.predicate()

    def predicate(self):
        col = self.column()
        neg = False
        if self.kw("NOT"):
            self.take()
            neg = True
        kind, val = self.peek()
        if kind == "op":
            self.take()
            if neg:
                raise FrontEndError("NOT before a comparison operator")
            op = "<>" if val == "!=" else val
            nk, nv = self.peek()
            if nk == "name" and "." in nv:  # column = column: an equi-join
                self.take()
                if op != "=":
                    raise FrontEndError("only equi-joins between aliases")
                return Pred("join", column=col, value=nv)
            return Pred("cmp", column=col, op=op, value=self.literal())
        if self.kw("LIKE"):
            self.take()
            p = Pred("like", column=col, value=self.literal())
        elif self.kw("IN"):
            self.take()
            self.expect("punct", "(")
            vals = [self.literal()]
            while self.peek() == ("punct", ","):
                self.take()
                vals.append(self.literal())
            self.expect("punct", ")")
            p = Pred("in", column=col, value=vals)
        elif self.kw("BETWEEN"):
            self.take()
            lo = self.literal()
            self.expect("name", "AND")
            p = Pred("between", column=col, value=(lo, self.literal()))
        elif self.kw("IS"):
            self.take()
            isnot = False
            if self.kw("NOT"):
                self.take()
                isnot = True
            self.expect("name", "NULL")
            p = Pred("null", column=col)
            return Pred("not", args=[p]) if isnot != neg else p
        else:
            raise FrontEndError(f"unsupported predicate after {col}: {val!r}")
        return Pred("not", args=[p]) if neg else p


def parse_sql(sql: str) -> ParsedSQL:
    """Parses a `SELECT ... FROM ... WHERE ...` join query (see the module docstring)."""
    p = _Parser(_tokens(sql))
    p.expect("name", "SELECT")
    aggs = []
    while True:
        if p.peek(1) == ("punct", "("):
            fn = p.expect("name").upper()
            p.expect("punct", "(")
            col = p.column()
            p.expect("punct", ")")
        else:
            fn, col = "", p.column()
        if p.kw("AS"):
            p.take()
            p.expect("name")
        a, c = col.split(".")
        aggs.append((fn, a, c))
        if p.peek() != ("punct", ","):
            break
        p.take()
    p.expect("name", "FROM")
    tables = {}
    while True:
        name = p.expect("name")
        alias = name
        if p.kw("AS"):
            p.take()
            alias = p.expect("name")
        elif p.peek()[0] == "name" and not p.kw("WHERE"):
            alias = p.expect("name")
        if alias in tables:
            raise FrontEndError(f"alias {alias} used twice")
        tables[alias] = name
        if p.peek() != ("punct", ","):
            break
        p.take()
    conj: List[Pred] = []
    if p.kw("WHERE"):
        p.take()
        e = p.or_expr()
        conj = e.args if e.kind == "and" else [e]
    if p.peek() == ("punct", ";"):
        p.take()
    if p.peek()[0] != "eof":
        raise FrontEndError(f"unexpected {p.peek()[1]!r} after the WHERE clause")
    join_graph: Dict[str, Dict[str, Tuple[str, str]]] = {a: {} for a in tables}
    per_alias: Dict[str, List[Pred]] = {}
    for c in conj:
        if c.kind == "join":
            la, lc = c.column.split(".")
            ra, rc = str(c.value).split(".")
            for a in (la, ra):
                if a not in tables:
                    raise FrontEndError(f"unknown alias {a}")
            join_graph[la][ra] = (lc, rc)
            join_graph[ra][la] = (rc, lc)
            continue
        al = c.aliases()
        if len(al) != 1:
            raise FrontEndError("a predicate over several aliases that is not an equi-join")
        a = next(iter(al))
        if a not in tables:
            raise FrontEndError(f"unknown alias {a}")
        if _has_join(c):
            raise FrontEndError("a join condition inside an OR / NOT group")
        per_alias.setdefault(a, []).append(c)
    filters = {a: (ps[0] if len(ps) == 1 else Pred("and", args=ps)) for a, ps in per_alias.items()}
    for _, a, _c in aggs:
        if a not in tables:
            raise FrontEndError(f"unknown alias {a} in the SELECT list")
    return ParsedSQL(tables, join_graph, filters, [(a, c) for _, a, c in aggs], aggs)


def _has_join(p: Pred) -> bool:
    return p.kind == "join" or any(_has_join(a) for a in p.args)


# ------------------------------------------------------- predicate on host ----

def _like_regex(pattern: str) -> "re.Pattern":
    out = []
    for ch in pattern:
        out.append(".*" if ch == "%" else "." if ch == "_" else re.escape(ch))
    return re.compile("".join(out), re.S)


def _leaf(p: Pred, cols) -> Tuple[np.ndarray, np.ndarray]:
    """(true, unknown) masks of a leaf predicate."""
    col = p.column.split(".", 1)[1]
    if col not in cols:
        raise FrontEndError(f"unknown column {p.column}")
    vals, valid = cols[col]
    n = len(valid)
    unknown = ~valid
    if p.kind == "null":
        return ~valid, np.zeros(n, bool)
    is_str = vals.dtype == object
    if p.kind == "cmp":
        if is_str != isinstance(p.value, str):
            raise FrontEndError(f"comparison of {p.column} with a literal of another type")
        v = np.array(["" if x is None else x for x in vals], dtype=object) if is_str else vals
        res = {"=": v == p.value, "<>": v != p.value, "<": v < p.value, ">": v > p.value,
               "<=": v <= p.value, ">=": v >= p.value}[p.op]
        return np.asarray(res, bool) & valid, unknown
    if p.kind == "like":
        if not is_str:
            raise FrontEndError(f"LIKE on the non-string column {p.column}")
        rx = _like_regex(str(p.value))
        res = np.array([x is not None and rx.fullmatch(x) is not None for x in vals], bool)
        return res & valid, unknown
    if p.kind == "in":
        s = set(p.value)
        res = np.array([valid[i] and vals[i] in s for i in range(n)], bool)
        return res, unknown
    if p.kind == "between":
        lo, hi = p.value
        v = np.array(["" if x is None else x for x in vals], dtype=object) if is_str else vals
        return np.asarray((v >= lo) & (v <= hi), bool) & valid, unknown
    raise FrontEndError(f"unknown predicate kind {p.kind}")


def _eval(p: Pred, cols) -> Tuple[np.ndarray, np.ndarray]:
    if p.kind == "and":
        t, u = _eval(p.args[0], cols)
        f = ~t & ~u
        for a in p.args[1:]:
            t2, u2 = _eval(a, cols)
            f2 = ~t2 & ~u2
            t, f = t & t2, f | f2
            u = ~t & ~f
        return t, u
    if p.kind == "or":
        t, u = _eval(p.args[0], cols)
        for a in p.args[1:]:
            t2, u2 = _eval(a, cols)
            t = t | t2
            u = ~t & (u | u2)
        return t, u
    if p.kind == "not":
        t, u = _eval(p.args[0], cols)
        return ~t & ~u, u
    return _leaf(p, cols)


def filter_mask(pred: Optional[Pred], cols: Dict[str, Tuple[np.ndarray, np.ndarray]], n: int) -> np.ndarray:
    """Rows for which `pred` is true (SQL three-valued logic: unknown drops the row).
    cols: column -> (values, valid mask); VARCHAR values are an object array."""
    if pred is None:
        return np.ones(n, bool)
    return _eval(pred, cols)[0]


# ------------------------------------------------------------- the pipeline ----

_OTHER = ("Aggregate", "Gather")
_JOINS = ("Nested Loop", "Hash Join", "Merge Join")
_SCANS = ("Seq Scan", "Index Only Scan")


def _unwrap(plan: dict) -> dict:
    return plan["Plan"] if "Plan" in plan and "Node Type" not in plan else plan


def _join_children(node: dict) -> Tuple[bool, dict, dict]:
    """(build_left, left, right) of a Hash Join; the Hash node's child is its side."""
    if node["Node Type"] != "Hash Join":
        raise FrontEndError("Not Hash Join")
    a, b = node["Plans"][0], node["Plans"][1]
    if a["Node Type"] == "Hash" and b["Node Type"] != "Hash":
        return True, a["Plans"][0], b
    if a["Node Type"] != "Hash" and b["Node Type"] == "Hash":
        return False, a, b["Plans"][0]
    raise FrontEndError("Hash Join should have exactly one Hash child")


def _alias_of(node: dict, parsed: ParsedSQL) -> str:
    if "Alias" in node:
        a = node["Alias"]
        if a not in parsed.tables:
            raise FrontEndError(f"Cannot find alias: {a}")
        return a
    if "Relation Name" in node:
        rel = node["Relation Name"]
        hits = [a for a, t in parsed.tables.items() if t == rel]
        if len(hits) != 1:
            raise FrontEndError(f"Table {rel} is used {'at least twice' if hits else 'nowhere'}")
        return hits[0]
    raise FrontEndError('Neither "Alias" nor "Relation Name" exists in scan node')


def _entities(node: dict, parsed: ParsedSQL) -> List[str]:
    t = node["Node Type"]
    if t in _OTHER:
        return _entities(node["Plans"][0], parsed)
    if t in _JOINS:
        _, l, r = _join_children(node)
        return _entities(l, parsed) + _entities(r, parsed)
    if t in _SCANS:
        return [_alias_of(node, parsed)]
    raise FrontEndError(f"Not supported node type: {t}")


def load_join_pipeline(explain: dict, parsed: ParsedSQL, schema: Dict[str, Sequence[Tuple[str, int]]],
                       load_table: Callable[[str, str, Optional[Pred]], object], hj):
    """EXPLAIN JSON (one query's plan, with or without its {"Plan": ...} wrapper) and
    the parsed SQL -> (hj.Plan, [(alias, column, type)] of the root's outputs).

    schema[table]: the table's (column, type) in input-column order.
    load_table(alias, table, predicate) -> hj.Table of that relation, every schema
    column, with the alias's predicate already applied (None: no predicate)."""
    plan = hj.Plan()

    def rec(node: dict, required: List[Tuple[str, str]]):
        t = node["Node Type"]
        if t in _OTHER:
            return rec(node["Plans"][0], required)
        if t in _JOINS:
            build_left, lnode, rnode = _join_children(node)
            le, re_ = _entities(lnode, parsed), _entities(rnode, parsed)
            cond = None
            for a in le:  # the first equi-join between the two sides
                for b, (ca, cb) in parsed.join_graph.get(a, {}).items():
                    if b in re_ and cond is None:
                        cond = (a, ca, b, cb)
            if cond is None:
                raise FrontEndError("Cannot find join condition")
            la, lc, ra, rc = cond
            lreq, rreq = [], []
            for a, c in required:
                if a in le:
                    lreq.append((a, c))
                elif a in re_:
                    rreq.append((a, c))
                else:
                    raise FrontEndError("Required attributes cannot be found in either child")
            if (la, lc) not in lreq:
                lreq.append((la, lc))
            if (ra, rc) not in rreq:
                rreq.append((ra, rc))
            lid, lcols = rec(lnode, lreq)
            rid, rcols = rec(rnode, rreq)
            lattr = [i for i, (a, c, _) in enumerate(lcols) if (a, c) == (la, lc)][0]
            rattr = [i for i, (a, c, _) in enumerate(rcols) if (a, c) == (ra, rc)][0]
            both = lcols + rcols
            out_cols, out_attrs = [], []
            for a, c in required:
                idx = next((i for i, (x, y, _) in enumerate(both) if (x, y) == (a, c)), None)
                if idx is None:
                    raise FrontEndError(f"Cannot find the required attr: {a}.{c} in children's output")
                out_cols.append(both[idx])
                out_attrs.append((idx, both[idx][2]))
            return plan.new_join_node(build_left, lid, rid, lattr, rattr, out_attrs), out_cols
        if t in _SCANS:
            alias = _alias_of(node, parsed)
            table = parsed.tables[alias]
            if table not in schema:
                raise FrontEndError(f"Cannot find attributes for table: {table}")
            attrs = list(schema[table])
            inp = plan.new_input(load_table(alias, table, parsed.filters.get(alias)))
            out_cols, out_attrs = [], []
            for a, c in required:
                idx = next((i for i, (name, _) in enumerate(attrs) if a == alias and name == c), None)
                if idx is None:
                    raise FrontEndError(f"Cannot find the required attr: {a}.{c} in children's output")
                out_cols.append((alias, c, attrs[idx][1]))
                out_attrs.append((idx, attrs[idx][1]))
            return plan.new_scan_node(inp, out_attrs), out_cols
        raise FrontEndError(f"Not supported node type: {t}")

    root, cols = rec(_unwrap(explain), list(parsed.output_attrs))
    plan.root = root
    return plan, cols


def table_loader(hj, data: Dict[str, Dict[str, Tuple[Sequence, Optional[np.ndarray]]]],
                 schema: Dict[str, Sequence[Tuple[str, int]]]):
    """A load_table for host data: data[table][column] = (values, valid mask or None);
    INT32 values as integers, VARCHAR values as str (None = NULL).  The predicate is
    applied on the host before the pages are built, as the reference filters while
    loading."""
    def load(alias: str, table: str, pred: Optional[Pred]):
        cols = {}
        n = None
        for name, ty in schema[table]:
            vals, valid = data[table][name]
            if ty == VARCHAR:
                v = np.empty(len(vals), dtype=object)
                v[:] = list(vals)
                ok = np.array([x is not None for x in v], bool) if valid is None else np.asarray(valid, bool)
            else:
                v = np.asarray(vals, dtype=np.int64 if ty == INT64 else np.int32)
                ok = np.ones(len(v), bool) if valid is None else np.asarray(valid, bool)
            cols[name] = (v, ok)
            n = len(v) if n is None else n
            if len(v) != n:
                raise FrontEndError(f"columns of {table} differ in length")
        n = n or 0
        keep = filter_mask(pred, cols, n)
        out = []
        for name, ty in schema[table]:
            v, ok = cols[name]
            v, ok = v[keep], ok[keep]
            if ty == VARCHAR:
                out.append(hj.Column.varchar([x if o else None for x, o in zip(v, ok)]))
            elif ty == INT32:
                out.append(hj.Column.int32(v, ok.astype(np.uint8)))
            else:
                raise FrontEndError(f"column type {ty} of {table}.{name} is not loadable here")
        return hj.Table(int(keep.sum()), out)
    return load


def read_plans_json(path) -> Tuple[str, Dict[str, dict]]:
    """The reference's plans.json layout: {"sql_directory": dir, "names": [...],
    "plans": [EXPLAIN JSON per name]} -> (sql directory, {name: plan})."""
    import json
    from pathlib import Path
    d = json.loads(Path(path).read_text())
    names, plans = d.get("names", []), d.get("plans", [])
    if len(names) != len(plans):
        raise FrontEndError("plans.json: names and plans differ in length")
    return d.get("sql_directory", ""), dict(zip(names, plans))
