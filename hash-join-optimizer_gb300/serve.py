"""The serving workload and its two runners: plans arriving as an open-loop
Poisson stream, run by the request loop (hj_server: concurrent slots, HBM
admission, tables built over resident columns kept for reuse) or one at a time
through Contest::execute (the plain path).

Mix (by arrival): 70% small -- a 2-way INT32 join, build side 10k..1M rows
(log-uniform), unique permuted keys and one payload, probe side 10x with a
foreign key uniform over the build keys and one payload; 25% medium -- the
5-relation chain at 1/10 scale; 5% large -- the 16M x 256M skewed join.  All
base tables are uploaded to HBM once and decoded there (hj_table_prepare); a
small query picks one of `small_tables` prepared table pairs.
"""
from __future__ import annotations

import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import INT32, Column, Engine, Plan, Table
from . import workloads as W

KINDS = ("small", "medium", "large")


@dataclass
class Mix:
    plans: dict                       # kind -> list of frozen Plans over resident tables
    resident: list = field(default_factory=list)
    fractions: tuple = (0.70, 0.25, 0.05)

    def release(self, engine: Engine) -> None:
        for t in self.resident:
            engine.release(t)
        self.resident.clear()


def _small_pair(rng: np.random.Generator, b: int):
    key = rng.permutation(b).astype(np.int32)
    bp = rng.integers(0, 2**31, size=b, dtype=np.int64).astype(np.int32)
    fk = key[rng.integers(0, b, size=10 * b)]
    pp = rng.integers(0, 2**31, size=10 * b, dtype=np.int64).astype(np.int32)
    return (Table(b, [Column.int32(key), Column.int32(bp)]),
            Table(10 * b, [Column.int32(fk), Column.int32(pp)]))


def small_plan(build: Table, probe: Table) -> Plan:
    p = Plan()
    p.new_input(build)
    p.new_input(probe)
    p.new_scan_node(0, [(0, INT32), (1, INT32)])
    p.new_scan_node(1, [(0, INT32), (1, INT32)])
    p.root = p.new_join_node(True, 0, 1, 0, 0, [(0, INT32), (1, INT32), (3, INT32)])
    return p


def c5_mix(engine: Engine, seed: int = 42, small_tables: int = 16, small_lo: int = 10_000,
           small_hi: int = 1_000_000, medium_scale: float = 0.1, large_scale: float = 1.0) -> Mix:
    """Uploads and prepares the base tables of the serving mix."""
    rng = np.random.default_rng([seed, 5])
    mix = Mix({k: [] for k in KINDS})

    def resident_plan(plan: Plan) -> Plan:
        ins = []
        for t in plan.inputs:
            r = engine.upload(t)
            engine.prepare(r)
            mix.resident.append(r)
            ins.append(r)
        return Plan(plan.nodes, ins, plan.root).frozen()

    sizes = np.exp(rng.uniform(np.log(small_lo), np.log(small_hi), size=small_tables)).astype(np.int64)
    for b in sizes:
        mix.plans["small"].append(resident_plan(small_plan(*_small_pair(rng, int(b)))))
    mix.plans["medium"].append(resident_plan(W.c3(scale=medium_scale, seed=seed).plan))
    mix.plans["large"].append(resident_plan(W.c2(scale=large_scale, seed=seed).plan))
    return mix


def schedule(mix: Mix, rate: float, n: int, seed: int = 1):
    """n arrivals of a Poisson stream at `rate` per second: [(seconds, kind, plan index)]."""
    rng = np.random.default_rng([seed, int(rate)])
    t = np.cumsum(rng.exponential(1.0 / rate, size=n))
    kinds = rng.choice(len(KINDS), size=n, p=np.array(mix.fractions) / sum(mix.fractions))
    out = []
    for ti, k in zip(t, kinds):
        kind = KINDS[int(k)]
        out.append((float(ti), kind, int(rng.integers(0, len(mix.plans[kind])))))
    return out


def _pct(lat):
    a = np.asarray(lat, dtype=np.float64)
    return {"p50_ms": float(np.percentile(a, 50)), "p95_ms": float(np.percentile(a, 95)),
            "p99_ms": float(np.percentile(a, 99)), "mean_ms": float(a.mean())}


def _summary(engine: Engine, res: int):
    """Row count and column count of a result handle (VARCHAR page counts follow
    the unspecified row order, so they are not part of it)."""
    import ctypes as C
    from . import lib
    nr, nc = C.c_uint64(), C.c_uint32()
    lib().hj_result_shape(res, C.byref(nr), C.byref(nc))
    return nr.value, nc.value


def run_served(engine: Engine, mix: Mix, sched, hbm_budget: int, slots: int, keep=None):
    """Open-loop run through hj_server.  keep(i, res) may take a result
    (returns True to keep it; the caller frees it); others are freed here."""
    srv = engine.server(hbm_budget, slots)
    tickets, lock, done = [], threading.Lock(), threading.Event()
    out = [None] * len(sched)

    def waiter():
        i = 0
        while i < len(sched):
            with lock:
                have = i < len(tickets)
            if not have:
                time.sleep(0.0002)
                continue
            res, st = srv.wait(tickets[i])
            out[i] = (st, _summary(engine, res))
            if not (keep and keep(i, res)):
                engine.free_result(res)
            i += 1
        done.set()

    th = threading.Thread(target=waiter, daemon=True)
    t0 = time.perf_counter()
    th.start()
    try:
        for at, kind, idx in sched:
            d = t0 + at - time.perf_counter()
            if d > 0:
                time.sleep(d)
            tk = srv.submit(mix.plans[kind][idx])
            with lock:
                tickets.append(tk)
        done.wait()
        t_end = time.perf_counter()
        info = srv.info()
    finally:
        th.join()
        srv.close()
    lat = [o[0]["latency_ms"] for o in out]
    by_kind = {k: _pct([o[0]["latency_ms"] for o, s in zip(out, sched) if s[1] == k])
               for k in KINDS if any(s[1] == k for s in sched)}
    return {"qps": len(sched) / (t_end - t0), "seconds": t_end - t0, **_pct(lat), "by_kind": by_kind,
            "peak_admitted_bytes": info["peak_bytes"], "results": [o[1] for o in out]}


def run_plain(engine: Engine, mix: Mix, sched, keep=None):
    """The same stream through Contest::execute, one plan at a time, in
    arrival order (a plan that arrives while another runs waits)."""
    t0 = time.perf_counter()
    lat, results = [], []
    for i, (at, kind, idx) in enumerate(sched):
        d = t0 + at - time.perf_counter()
        if d > 0:
            time.sleep(d)
        res = engine.execute_raw(mix.plans[kind][idx])
        lat.append(1e3 * (time.perf_counter() - (t0 + at)))
        results.append(_summary(engine, res))
        if not (keep and keep(i, res)):
            engine.free_result(res)
    t_end = time.perf_counter()
    by_kind = {k: _pct([l for l, s in zip(lat, sched) if s[1] == k]) for k in KINDS if any(s[1] == k for s in sched)}
    return {"qps": len(sched) / (t_end - t0), "seconds": t_end - t0, **_pct(lat), "by_kind": by_kind,
            "results": results}
