"""Batched independent joins on the device: waves of synthetic instances
generated in HBM (hj_batch_generate) and joined by hj_batch_execute, either as
one persistent, graph-launched batch or one instance at a time (the plain
path).

A batch workload can be larger than HBM (the 4,096-instance one holds about
2.4e10 input rows), so `waves()` cuts it into consecutive groups of instances
whose input rows fit a budget; each wave is generated, joined and freed before
the next.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import BATCH_PERSISTENT, Engine
from .workloads import BatchWorkload


def waves(w: BatchWorkload, max_rows: int) -> list:
    """Consecutive instance index groups with at most max_rows input rows each
    (an instance larger than the budget forms a wave of its own)."""
    out, cur, rows = [], [], 0
    for i in range(len(w)):
        r = w.rows(i)
        if cur and rows + r > max_rows:
            out.append(cur)
            cur, rows = [], 0
        cur.append(i)
        rows += r
    if cur:
        out.append(cur)
    return out


@dataclass
class DeviceWave:
    """The relations of a group of instances, generated in HBM."""
    instances: list                              # per instance: [(keys ptr, payload ptr, rows), ...]
    rows: int                                    # input rows of the wave
    keep: list = field(default_factory=list)     # device buffers


def generate(engine: Engine, w: BatchWorkload, idx, torch) -> DeviceWave:
    """Generates instances `idx` of w into one key and one payload buffer.  The
    generator runs on the engine's stream; hj_batch_execute on the same stream
    sees the data."""
    total = sum(w.rows(i) for i in idx)
    keys = torch.empty(max(1, total), dtype=torch.int32, device="cuda")
    pays = torch.empty(max(1, total), dtype=torch.int32, device="cuda")
    kb, pb = keys.data_ptr(), pays.data_ptr()
    insts, off = [], 0
    for i in idx:
        iid, m, b, q, p = w.instance(i)
        rels = []
        for j in range(m):
            n = p if j == 0 else b
            engine.batch_generate(w.seed, iid, j, b, q, n, kb + 4 * off, pb + 4 * off)
            rels.append((kb + 4 * off, pb + 4 * off, n))
            off += n
        insts.append(rels)
    torch.cuda.ExternalStream(engine.stream).synchronize()  # generation is not part of a timed join
    return DeviceWave(insts, total, [keys, pays])


def run(engine: Engine, w: BatchWorkload, mode: int = BATCH_PERSISTENT, max_rows: int = 1 << 31, torch=None,
        timer=None):
    """Joins every instance of w in waves.  Returns (rows, checksums, recomputed,
    seconds inside hj_batch_execute).  `timer(fn)` may wrap each call to time it
    on the device; by default the host wall clock is used."""
    import time
    if torch is None:
        import torch  # device buffers only
    rows = np.zeros(len(w), dtype=np.uint64)
    sums = np.zeros(len(w), dtype=np.uint64)
    redo, secs = 0, 0.0
    for idx in waves(w, max_rows):
        dw = generate(engine, w, idx, torch)
        call = lambda: engine.batch_execute(dw.instances, mode)  # noqa: E731
        if timer is None:
            t0 = time.perf_counter()
            r, s, k = call()
            secs += time.perf_counter() - t0
        else:
            (r, s, k), t = timer(call)
            secs += t
        rows[idx], sums[idx] = r, s
        redo += k
        del dw
    return rows, sums, redo, secs
