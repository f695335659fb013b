"""Seeded synthetic join workloads with the shapes the join path is measured on.

The reference's own workload (JOB on IMDB) is not available offline, so these
generators stand in for it with the configured shapes, sizes and value
distributions.  Every table comes out in the reference page format (built with
the engine's host page writers, i.e. Table::to_columnar packing) and every
generator is deterministic in (seed, scale).

  c1  plain 2-table join: 1M-row build (unique permuted keys, 2 payloads),
      10M-row probe (foreign key uniform over the build keys, 1 payload);
      exactly 10M result rows.
  c2  skewed join: 16M-row build (keys Zipf(1.1) over 4M ranks, 2 INT32
      payloads with 20% NULLs, one ASCII VARCHAR of 8-64 bytes); 256M raw probe
      rows (keys Zipf(1.1) over 8M ranks, independent rank->key permutations)
      pre-filtered by an INT32 predicate `pred < 100` with pred ~ U[0, 1000)
      (10% kept), 2 INT32 payloads with 20% NULLs and one VARCHAR.
  c3  5-relation left-deep chain R1..R5 (36M, 15M, 4.2M, 2.5M, 134k rows):
      dense permuted PKs, FK fan-out per PK Zipf(1.0), per-relation pre-filter
      with log-uniform selectivity in [0.5%, 30%], 1-3 INT32 payloads with 5%
      NULLs and one VARCHAR of 4-40 bytes.

`scale` multiplies every row count and key domain (tests use small scales).
Pre-filters are applied here, before execute(), as the reference applies its
filters while loading tables (src/build_table.cpp:321-325).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Callable, Optional

import numpy as np

from . import CMP_LT, INT32, VARCHAR, Column, Plan, Table


@dataclass
class Workload:
    name: str
    plan: Plan
    probe_rows: int          # probe tuples of the (last) join the metric counts
    build_rows: int
    expected_rows: int = -1  # exact result size when known in closed form
    meta: dict = field(default_factory=dict)
    # sample(k): the same plan with only the first k probe rows (bounded CPU runs)
    sample: Optional[Callable[[int], Plan]] = None


def _rng(seed: int, *stream: int) -> np.random.Generator:
    return np.random.default_rng([seed, *stream])


def zipf_ranks(rng: np.random.Generator, n: int, k: int, s: float) -> np.ndarray:
    """n draws of a rank in [0, k) with P(rank = r) ~ (r + 1)^-s (inverse CDF)."""
    w = np.arange(1, k + 1, dtype=np.float64) ** (-s)
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    u = rng.random(n)
    return np.minimum(np.searchsorted(cdf, u, side="right"), k - 1).astype(np.int64)


def ascii_strings(rng: np.random.Generator, n: int, lo: int, hi: int):
    """n printable-ASCII strings with length uniform in [lo, hi]: (bytes, offsets)."""
    lens = rng.integers(lo, hi + 1, size=n, dtype=np.int64)
    offs = np.zeros(n + 1, dtype=np.uint64)
    np.cumsum(lens, out=offs[1:])
    data = rng.integers(0x20, 0x7F, size=int(offs[-1]), dtype=np.uint8)
    return data, offs


def nulls(rng: np.random.Generator, n: int, p: float) -> np.ndarray:
    """validity bytes: 0 with probability p."""
    return (rng.random(n) >= p).astype(np.uint8)


def c1(scale: float = 1.0, seed: int = 42) -> Workload:
    nb, npr = max(1, int(1_000_000 * scale)), max(1, int(10_000_000 * scale))
    r = _rng(seed, 1)
    key = r.permutation(nb).astype(np.int32)
    b1 = r.integers(0, 2**31, size=nb, dtype=np.int64).astype(np.int32)
    b2 = r.integers(0, 2**31, size=nb, dtype=np.int64).astype(np.int32)
    fk = key[r.integers(0, nb, size=npr)]
    p1 = r.integers(0, 2**31, size=npr, dtype=np.int64).astype(np.int32)
    build = Table(nb, [Column.int32(key), Column.int32(b1), Column.int32(b2)])

    def make_plan(k: int) -> Plan:
        plan = Plan()
        plan.new_input(build)
        plan.new_input(Table(k, [Column.int32(fk[:k]), Column.int32(p1[:k])]))
        plan.new_scan_node(0, [(0, INT32), (1, INT32), (2, INT32)])
        plan.new_scan_node(1, [(0, INT32), (1, INT32)])
        plan.root = plan.new_join_node(True, 0, 1, 0, 0, [(0, INT32), (1, INT32), (2, INT32), (4, INT32)])
        return plan

    return Workload("c1", make_plan(npr), npr, nb, expected_rows=npr,
                    meta={"build_rows": nb, "probe_rows": npr, "out_cols": "k,b1,b2,p1"},
                    sample=lambda k: make_plan(min(k, npr)))


def c2(scale: float = 1.0, seed: int = 42, raw_probe: int | None = None, raw: bool = False) -> Workload:
    """raw=True: the probe side is the raw table (all probe rows plus the
    predicate column `pred`, column 4) and the plan's probe scan carries the
    predicate pred < 100 instead of the table being pre-filtered.  Its passing
    rows hold exactly the pre-filtered table's values, so the result is the
    same; dropped rows get their own random keys and payloads and NULL strings."""
    nb = max(1, int(16_000_000 * scale))
    kb, kp = max(1, int(4_000_000 * scale)), max(1, int(8_000_000 * scale))
    nraw = raw_probe if raw_probe is not None else max(1, int(256_000_000 * scale))
    rb, rp = _rng(seed, 2, 0), _rng(seed, 2, 1)
    perm_b = rb.permutation(kb).astype(np.int32)
    key = perm_b[zipf_ranks(rb, nb, kb, 1.1)]
    b1 = rb.integers(0, 2**31, size=nb, dtype=np.int64).astype(np.int32)
    b2 = rb.integers(0, 2**31, size=nb, dtype=np.int64).astype(np.int32)
    v1, v2 = nulls(rb, nb, 0.2), nulls(rb, nb, 0.2)
    bs, bo = ascii_strings(rb, nb, 8, 64)
    # pre-filter: pred ~ U[0, 1000) over the raw probe rows, keep pred < 100
    pred = rp.integers(0, 1000, size=nraw, dtype=np.int16)
    keep = np.flatnonzero(pred < 100)
    npr = int(keep.size)
    perm_p = rp.permutation(kp).astype(np.int32)
    fk = perm_p[zipf_ranks(rp, npr, kp, 1.1)]
    p1 = rp.integers(0, 2**31, size=npr, dtype=np.int64).astype(np.int32)
    p2 = rp.integers(0, 2**31, size=npr, dtype=np.int64).astype(np.int32)
    w1, w2 = nulls(rp, npr, 0.2), nulls(rp, npr, 0.2)
    ps, po = ascii_strings(rp, npr, 8, 64)
    # exact result size: sum over keys of build count x probe count
    cb = np.bincount(key, minlength=kp)
    cp = np.bincount(fk, minlength=kp)
    expected = int(np.dot(cb[:kp].astype(np.int64), cp[: cb.size].astype(np.int64)))
    build = Table(nb, [Column.int32(key), Column.int32(b1, v1), Column.int32(b2, v2), Column.varchar(bs, bo)])

    def probe_table(k: int) -> Table:
        o = po[: k + 1]
        return Table(k, [Column.int32(fk[:k]), Column.int32(p1[:k], w1[:k]), Column.int32(p2[:k], w2[:k]),
                         Column.varchar(ps[: int(o[-1])], o, None)])

    def make_plan(probe: Table) -> Plan:
        plan = Plan()
        plan.new_input(build)
        plan.new_input(probe)
        plan.new_scan_node(0, [(0, INT32), (1, INT32), (2, INT32), (3, VARCHAR)])
        plan.new_scan_node(1, [(0, INT32), (1, INT32), (2, INT32), (3, VARCHAR)])
        plan.root = plan.new_join_node(True, 0, 1, 0, 0, [(1, INT32), (2, INT32), (3, VARCHAR),
                                                          (5, INT32), (6, INT32), (7, VARCHAR)])
        return plan

    if raw:
        rr = _rng(seed, 2, 2)
        drop = np.ones(nraw, dtype=bool)
        drop[keep] = False

        def spread(kept, fill):
            out = np.empty(nraw, dtype=kept.dtype)
            out[keep] = kept
            out[drop] = fill
            return out
        nd = int(drop.sum())
        fk_r = spread(fk, rr.integers(0, kp, size=nd, dtype=np.int64).astype(np.int32))
        p1_r = spread(p1, rr.integers(0, 2**31, size=nd, dtype=np.int64).astype(np.int32))
        p2_r = spread(p2, rr.integers(0, 2**31, size=nd, dtype=np.int64).astype(np.int32))
        w1_r, w2_r = spread(w1, nulls(rr, nd, 0.2)), spread(w2, nulls(rr, nd, 0.2))
        lens = np.zeros(nraw, dtype=np.int64)
        lens[keep] = np.diff(po.astype(np.int64))
        po_r = np.zeros(nraw + 1, dtype=np.uint64)
        np.cumsum(lens, out=po_r[1:])
        vs_r = (~drop).astype(np.uint8)
        raw_probe_t = Table(nraw, [Column.int32(fk_r), Column.int32(p1_r, w1_r), Column.int32(p2_r, w2_r),
                                   Column.varchar(ps, po_r, vs_r), Column.int32(pred.astype(np.int32))])
        plan = Plan()
        plan.new_input(build)
        plan.new_input(raw_probe_t)
        plan.new_scan_node(0, [(0, INT32), (1, INT32), (2, INT32), (3, VARCHAR)])
        plan.new_scan_node(1, [(0, INT32), (1, INT32), (2, INT32), (3, VARCHAR)], filters=[(4, CMP_LT, 100)])
        plan.root = plan.new_join_node(True, 0, 1, 0, 0, [(1, INT32), (2, INT32), (3, VARCHAR),
                                                          (5, INT32), (6, INT32), (7, VARCHAR)])
        return Workload("c2raw", plan, nraw, nb, expected_rows=expected,
                        meta={"build_rows": nb, "probe_rows_raw": nraw, "probe_rows": npr,
                              "prefiltered_plan": make_plan(probe_table(npr))})
    return Workload("c2", make_plan(probe_table(npr)), npr, nb, expected_rows=expected,
                    meta={"build_rows": nb, "probe_rows_raw": nraw, "probe_rows": npr,
                          "build_key_domain": kb, "probe_key_domain": kp,
                          "build_bytes_varchar": int(bo[-1]), "probe_bytes_varchar": int(po[-1])},
                    sample=lambda k: make_plan(probe_table(min(k, npr))))


C3_SIZES = (36_000_000, 15_000_000, 4_200_000, 2_500_000, 134_000)


def c2raw(scale: float = 1.0, seed: int = 42) -> Workload:
    """c2 with the predicate fused into the probe: the raw probe table and a scan filter."""
    return c2(scale, seed, raw=True)


def c3(scale: float = 1.0, seed: int = 42) -> Workload:
    """Left-deep chain ((((R1 x R2) x R3) x R4) x R5) on R_i.fk = R_{i+1}.pk.

    Each R_i keeps a log-uniform 0.5%-30% of its rows (its pre-filter) and its
    FKs reference R_{i+1}'s surviving PKs with Zipf(1.0) fan-out through a
    seeded rank permutation (a foreign-key constraint on the filtered tables:
    with FKs drawn over the unfiltered PK range, four independent filters leave
    the chain empty for almost every seed).  Every join builds on its smaller
    input.
    """
    sizes = [max(2, int(s * scale)) for s in C3_SIZES]
    k = len(sizes)
    rngs = [_rng(seed, 3, i) for i in range(k)]
    sel = [float(np.exp(r.uniform(np.log(0.005), np.log(0.30)))) for r in rngs]
    kept_rows = [np.sort(rngs[i].choice(sizes[i], size=max(1, int(round(sizes[i] * sel[i]))), replace=False))
                 for i in range(k)]
    pks = [rngs[i].permutation(sizes[i]).astype(np.int32)[kept_rows[i]] for i in range(k)]
    tables, ncols = [], []
    for i in range(k):
        r, m = rngs[i], kept_rows[i].size
        cols = [Column.int32(pks[i])]
        if i + 1 < k:
            targets = pks[i + 1][r.permutation(pks[i + 1].size)]
            cols.append(Column.int32(targets[zipf_ranks(r, m, targets.size, 1.0)]))
        for _ in range(int(r.integers(1, 4))):
            cols.append(Column.int32(r.integers(0, 2**31, size=m, dtype=np.int64).astype(np.int32),
                                     nulls(r, m, 0.05)))
        sb, so = ascii_strings(r, m, 4, 40)
        cols.append(Column.varchar(sb, so))
        tables.append(Table(m, cols))
        ncols.append(len(cols))
    plan = Plan()
    for t in tables:
        plan.new_input(t)
    typ = lambda rel, c: VARCHAR if c == ncols[rel] - 1 else INT32  # noqa: E731
    scans = [plan.new_scan_node(i, [(c, typ(i, c)) for c in range(ncols[i])]) for i in range(k)]
    layout = [(0, c) for c in range(ncols[0])]  # intermediate columns as (relation, column)
    cur, cur_rows = scans[0], kept_rows[0].size
    for i in range(1, k):
        out = layout + [(i, c) for c in range(ncols[i])]
        fk_idx = layout.index((i - 1, 1))
        # keep payloads and the next join's FK; drop keys already joined on
        keep = [j for j, (rel, c) in enumerate(out)
                if not ((c == 0 and rel < i) or (c == 1 and rel < i))]
        attrs = [(j, typ(*out[j])) for j in keep]
        cur = plan.new_join_node(cur_rows < kept_rows[i].size, cur, scans[i], fk_idx, 0, attrs)
        layout = [out[j] for j in keep]
    plan.root = cur
    meta = {"sizes": sizes, "kept": [int(x.size) for x in kept_rows], "selectivity": sel}
    # every R1 row reaches exactly one row of each later relation
    return Workload("c3", plan, int(kept_rows[0].size), int(sum(x.size for x in kept_rows[1:])),
                    expected_rows=int(kept_rows[0].size), meta=meta)


# ----------------------------------------------------------- batched (c4) --

@dataclass
class BatchWorkload:
    """Independent join chains R0 x R1 x ... on one INT32 key (hj_batch_execute).
    Instance i has relations[i] relations; R1.. hold build_rows[i] distinct keys,
    R0 probe_rows[i] keys of which a fraction match_q24[i] / 2^24 hit R1.  The
    relations themselves are generated on the device (hj_batch_generate),
    keyed by (seed, instance id)."""
    name: str
    seed: int
    relations: np.ndarray
    build_rows: np.ndarray
    probe_rows: np.ndarray
    match_q24: np.ndarray
    ids: Optional[np.ndarray] = None  # instance ids (default 0..n-1)

    def __len__(self) -> int:
        return int(self.relations.size)

    def instance_id(self, i: int) -> int:
        return int(self.ids[i]) if self.ids is not None else int(i)

    def instance(self, i: int):
        """(instance id, relations, build rows, match_q24, probe rows)."""
        return (self.instance_id(i), int(self.relations[i]), int(self.build_rows[i]), int(self.match_q24[i]),
                int(self.probe_rows[i]))

    def rows(self, i: int) -> int:
        """input rows of instance i (all relations)."""
        return int(self.probe_rows[i] + (self.relations[i] - 1) * self.build_rows[i])

    def subset(self, idx) -> "BatchWorkload":
        idx = np.asarray(idx, dtype=np.int64)
        ids = self.ids[idx] if self.ids is not None else idx
        return BatchWorkload(self.name, self.seed, self.relations[idx], self.build_rows[idx], self.probe_rows[idx],
                             self.match_q24[idx], ids)


def c4(n: int = 4096, seed: int = 42, scale: float = 1.0, lo: int = 1_000, hi: int = 4_000_000) -> BatchWorkload:
    """4,096 independent 2- to 4-way INT32 equi-joins: build sizes log-uniform in
    [1k, 4M] rows (times `scale`), every probe side 10x its build size, match
    rate uniform in [10%, 100%], one INT32 payload per relation."""
    r = _rng(seed, 4)
    b = np.exp(r.uniform(np.log(lo), np.log(hi), size=n))
    b = np.maximum(1, np.round(b * scale)).astype(np.int64)
    m = r.integers(2, 5, size=n).astype(np.int64)
    q = np.round(r.uniform(0.10, 1.00, size=n) * (1 << 24)).astype(np.int64)
    return BatchWorkload("c4", seed, m, b, 10 * b, q)
