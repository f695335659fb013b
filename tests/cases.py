"""The reference's end-to-end join unit tests (tests/unit_tests.cpp:10-371 of
eleanalt/hash-join-optimizer) restated as data: each case builds the same Plan
and inputs and carries the reference test's ground truth (sorted rows, NULL as
None), plus a few edge cases of the same kind."""
from __future__ import annotations

import numpy as np

I, V = 0, 3  # INT32, VARCHAR


def table(hj, rows, types):
    """Rows (lists; None = NULL) -> engine Table built with Table::to_columnar packing."""
    cols = []
    for c, t in enumerate(types):
        vals = [r[c] for r in rows]
        if t == I:
            valid = np.array([v is not None for v in vals], np.uint8)
            cols.append(hj.Column.int32(np.array([0 if v is None else v for v in vals], np.int32), valid))
        else:
            cols.append(hj.Column.varchar(vals))
    return hj.Table(len(rows), cols)


def empty_table(hj, types):
    return hj.Table(0, [hj.Column(t, np.zeros((0, hj.PAGE_SIZE), np.uint8)) for t in types])


def _two_scans(hj, p, t1, t2, s1, s2):
    p.new_input(t1)
    p.new_input(t2)
    p.new_scan_node(0, s1)
    p.new_scan_node(1, s2)


def build_cases(hj):
    """name -> (Plan, expected sorted rows, expected column types)."""
    cases = {}

    # unit_tests.cpp:10-28 -- empty inputs
    p = hj.Plan()
    _two_scans(hj, p, empty_table(hj, [I]), empty_table(hj, [I]), [(0, I)], [(0, I)])
    p.root = p.new_join_node(True, 0, 1, 0, 0, [(0, I), (1, I)])
    cases["empty_join"] = (p, [], [I, I])

    # :30-57 -- one row each
    p = hj.Plan()
    _two_scans(hj, p, table(hj, [[1]], [I]), table(hj, [[1]], [I]), [(0, I)], [(0, I)])
    p.root = p.new_join_node(True, 0, 1, 0, 0, [(0, I), (1, I)])
    cases["one_line_join"] = (p, [(1, 1)], [I, I])

    # :59-91 -- 3-row self join
    d = [[1], [2], [3]]
    p = hj.Plan()
    _two_scans(hj, p, table(hj, d, [I]), table(hj, d, [I]), [(0, I)], [(0, I)])
    p.root = p.new_join_node(True, 0, 1, 0, 0, [(0, I), (1, I)])
    cases["simple_join"] = (p, [(1, 1), (2, 2), (3, 3)], [I, I])

    # :93-123 -- no matches
    p = hj.Plan()
    _two_scans(hj, p, table(hj, [[1], [2], [3]], [I]), table(hj, [[4], [5], [6]], [I]), [(0, I)], [(0, I)])
    p.root = p.new_join_node(True, 0, 1, 0, 0, [(0, I), (1, I)])
    cases["empty_result"] = (p, [], [I, I])

    # :125-161 -- duplicate keys: 2 x 2 for key 1
    d = [[1], [1], [2], [3]]
    p = hj.Plan()
    _two_scans(hj, p, table(hj, d, [I]), table(hj, d, [I]), [(0, I)], [(0, I)])
    p.root = p.new_join_node(True, 0, 1, 0, 0, [(0, I), (1, I)])
    cases["multiple_same_keys"] = (p, [(1, 1)] * 4 + [(2, 2), (3, 3)], [I, I])

    # :163-200 -- NULL keys never match
    d = [[1], [1], [None], [2], [3]]
    p = hj.Plan()
    _two_scans(hj, p, table(hj, d, [I]), table(hj, d, [I]), [(0, I)], [(0, I)])
    p.root = p.new_join_node(True, 0, 1, 0, 0, [(0, I), (1, I)])
    cases["null_keys"] = (p, [(1, 1)] * 4 + [(2, 2), (3, 3)], [I, I])

    # :202-241 -- VARCHAR payload, join on a non-first column
    d = [[1, "xxx"], [1, "yyy"], [None, "zzz"], [2, "uuu"], [3, "vvv"]]
    truth = [(1, 1, "xxx"), (1, 1, "xxx"), (1, 1, "yyy"), (1, 1, "yyy"), (2, 2, "uuu"), (3, 3, "vvv")]
    p = hj.Plan()
    _two_scans(hj, p, table(hj, d, [I, V]), table(hj, d, [I, V]), [(0, I)], [(1, V), (0, I)])
    p.root = p.new_join_node(True, 0, 1, 0, 1, [(0, I), (2, I), (1, V)])
    cases["multiple_columns"] = (p, truth, [I, I, V])

    # :243-282 -- build on the right
    p = hj.Plan()
    _two_scans(hj, p, table(hj, d, [I, V]), table(hj, d, [I, V]), [(0, I)], [(1, V), (0, I)])
    p.root = p.new_join_node(False, 0, 1, 0, 1, [(0, I), (2, I), (1, V)])
    cases["build_on_right"] = (p, truth, [I, I, V])

    # :284-321 -- left-deep 2-level join
    d = [[1], [2], [3]]
    p = hj.Plan()
    for _ in range(3):
        p.new_input(table(hj, d, [I]))
    p.new_scan_node(0, [(0, I)])
    p.new_scan_node(1, [(0, I)])
    p.new_scan_node(2, [(0, I)])
    p.new_join_node(True, 0, 1, 0, 0, [(0, I), (1, I)])
    p.root = p.new_join_node(False, 3, 2, 0, 0, [(0, I), (1, I), (2, I)])
    cases["leftdeep_2level"] = (p, [(1, 1, 1), (2, 2, 2), (3, 3, 3)], [I, I, I])

    # :323-371 -- 3-way join with VARCHAR on both sides
    p = hj.Plan()
    p.new_input(table(hj, [[1, "a"], [2, "b"], [3, "c"]], [I, V]))
    p.new_input(table(hj, [[1, "x"], [2, "y"]], [I, V]))
    p.new_input(table(hj, [[1, "u"], [2, "v"], [3, "w"]], [I, V]))
    for t in range(3):
        p.new_scan_node(t, [(0, I), (1, V)])
    p.new_join_node(False, 0, 1, 0, 0, [(0, I), (1, V)])
    p.root = p.new_join_node(False, 3, 2, 0, 0, [(0, I), (1, V), (3, V)])
    cases["three_way_join"] = (p, [(1, "a", "u"), (2, "b", "v")], [I, V, V])

    # --- further edge cases in the same style (no reference ground truth;
    # their expected rows come from the compiled reference / the restatement)
    # negative keys, keys at the INT32 limits, all-NULL payload
    d = [[-5, None], [2**31 - 1, 7], [-(2**31), 8], [0, None], [-5, 9]]
    p = hj.Plan()
    _two_scans(hj, p, table(hj, d, [I, I]), table(hj, d, [I, I]), [(0, I), (1, I)], [(0, I), (1, I)])
    p.root = p.new_join_node(False, 0, 1, 0, 0, [(1, I), (3, I), (0, I)])
    cases["extreme_keys"] = (p, None, [I, I, I])

    # scan as the root (copy_scan + table_to_columnar only)
    p = hj.Plan()
    p.new_input(table(hj, [[1, "a"], [None, None], [3, ""]], [I, V]))
    p.root = p.new_scan_node(0, [(1, V), (0, I)])
    cases["scan_root"] = (p, [("", 3), ("a", 1), (None, None)], [V, I])

    # long strings (> 8185 bytes: 0xffff/0xfffe pages) through a join
    big = "L" * 20000
    mid = "M" * 8186
    p = hj.Plan()
    _two_scans(hj, p, table(hj, [[1, big], [2, "s"], [3, mid]], [I, V]), table(hj, [[1], [3], [3]], [I]),
               [(0, I), (1, V)], [(0, I)])
    p.root = p.new_join_node(True, 0, 1, 0, 0, [(1, V), (2, I)])
    cases["long_strings"] = (p, [(big, 1), (mid, 3), (mid, 3)], [V, I])
    return cases
