"""Autotuner for the batched and plain join paths.

Sweeps, on a seeded sample of a batch workload's instances (generated once on
the device, timed with CUDA events on the engine's stream, best of `repeats`):

  batched path (hj_batch_execute, HJ_BATCH_PERSISTENT)
    batch_part_log2  build rows per partition 2^8 .. 2^13 -- the radix fan-out:
                     an instance with b build rows gets ceil(log2(b / 2^x))
                     partition bits (0 .. 11), reported as `radix_bits`
    batch_load_pct   build rows per 100 buckets of a partition table (50 .. 90)
  plain path (HJ_BATCH_PLAIN, the engine's regular build / probe)
    radix_bits       MSD partition bits of the table build (0 .. 12, or -1 = automatic)
    probe_group      output rows per thread of the match writer (1, 4, 8, 32): a
                     probe key's matches spread over count / probe_group threads

The batched join gives each probe key one thread: its tables live in shared
memory and a bucket holds under one key on average, so wider groups only add
idle lanes.  Results are cached as JSON keyed by the GPU name and the
workload's shape; `apply()` sets the chosen options on an engine.
"""
from __future__ import annotations

import itertools
import json
import math
import os
from pathlib import Path

import numpy as np

from . import BATCH_PERSISTENT, BATCH_PLAIN, Engine
from . import batch as _batch
from .workloads import BatchWorkload

BATCH_PART_LOG2 = (9, 10, 11, 12, 13)
BATCH_LOAD_PCT = (50, 70, 90)
PLAIN_RADIX_BITS = (-1, 0, 4, 8, 12)
PLAIN_PROBE_GROUP = (1, 4, 8, 32)

DEFAULT_CACHE = Path(os.environ.get("HJ_TUNE_CACHE", Path(__file__).resolve().parent / "_tune" / "tune.json"))


def sample(w: BatchWorkload, k: int, seed: int = 7) -> BatchWorkload:
    """k instances of w, stratified over build size (sorted by size, one per stratum)."""
    if len(w) <= k:
        return w
    order = np.argsort(w.build_rows, kind="stable")
    rng = np.random.default_rng(seed)
    edges = np.linspace(0, len(w), k + 1).astype(int)
    pick = [order[rng.integers(a, b)] for a, b in zip(edges[:-1], edges[1:]) if b > a]
    return w.subset(np.sort(np.array(pick)))


def radix_bits_for(build_rows: int, part_log2: int) -> int:
    t = 1 << part_log2
    return 0 if build_rows <= t else min(11, math.ceil(math.log2(math.ceil(build_rows / t))))


def _timer(engine: Engine, torch):
    stream = torch.cuda.ExternalStream(engine.stream)

    def run(fn):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        out = fn()
        b.record(stream)
        b.synchronize()
        return out, a.elapsed_time(b) / 1e3
    return run


def _measure(engine: Engine, wave, mode: int, timer, repeats: int):
    best, res = float("inf"), None
    for _ in range(repeats):
        out, t = timer(lambda: engine.batch_execute(wave.instances, mode))
        if t < best:
            best, res = t, out
    return best, res


def _key(engine_name: str, w: BatchWorkload) -> str:
    sig = f"{w.name}:{len(w)}:{int(w.build_rows.sum())}:{int(w.probe_rows.sum())}:{int(w.relations.sum())}"
    return f"{engine_name}|{sig}"


def tune(engine: Engine, w: BatchWorkload, sample_instances: int = 256, repeats: int = 2,
         cache: Path | None = DEFAULT_CACHE, force: bool = False, torch=None) -> dict:
    """Best options for both paths on a sample of w; cached unless `force`."""
    if torch is None:
        import torch
    name = torch.cuda.get_device_name()
    key = _key(name, w)
    if cache is not None and cache.exists() and not force:
        try:
            got = json.loads(cache.read_text()).get(key)
            if got:
                return got
        except ValueError:
            pass
    s = sample(w, sample_instances)
    timer = _timer(engine, torch)
    saved = {k: engine.get_option(k) for k in ("batch_part_log2", "batch_load_pct", "radix_bits", "probe_group")}
    wave = _batch.generate(engine, s, list(range(len(s))), torch)
    try:
        ref = None
        batched = []
        for part, load in itertools.product(BATCH_PART_LOG2, BATCH_LOAD_PCT):
            engine.set_option("batch_part_log2", part)
            engine.set_option("batch_load_pct", load)
            t, (rows, sums, redo) = _measure(engine, wave, BATCH_PERSISTENT, timer, repeats)
            ref = (rows, sums) if ref is None else ref
            assert np.array_equal(rows, ref[0]) and np.array_equal(sums, ref[1]), "tuning changed a result"
            batched.append({"batch_part_log2": part, "batch_load_pct": load, "seconds": t, "recomputed": int(redo)})
        plain = []
        for rb, g in itertools.product(PLAIN_RADIX_BITS, PLAIN_PROBE_GROUP):
            engine.set_option("radix_bits", rb)
            engine.set_option("probe_group", g)
            t, (rows, sums, _) = _measure(engine, wave, BATCH_PLAIN, timer, 1)
            assert np.array_equal(rows, ref[0]) and np.array_equal(sums, ref[1]), "tuning changed a result"
            plain.append({"radix_bits": rb, "probe_group": g, "seconds": t})
    finally:
        for k, v in saved.items():
            engine.set_option(k, v)
        del wave
    bb = min(batched, key=lambda r: r["seconds"])
    bp = min(plain, key=lambda r: r["seconds"])
    big = int(s.build_rows.max() * (s.relations.max() - 1))
    out = {
        "device": name, "sample_instances": len(s),
        "batched": {"batch_part_log2": bb["batch_part_log2"], "batch_load_pct": bb["batch_load_pct"],
                    "radix_bits_largest_instance": radix_bits_for(big, bb["batch_part_log2"]),
                    "threads_per_key": 1, "seconds": bb["seconds"]},
        "plain": {"radix_bits": bp["radix_bits"], "probe_group": bp["probe_group"], "seconds": bp["seconds"]},
        "sweep": {"batched": batched, "plain": plain},
    }
    if cache is not None:
        cache.parent.mkdir(parents=True, exist_ok=True)
        try:
            allc = json.loads(cache.read_text()) if cache.exists() else {}
        except ValueError:
            allc = {}
        allc[key] = out
        cache.write_text(json.dumps(allc, indent=1))
    return out


def apply(engine: Engine, tuned: dict) -> None:
    """Sets the tuned options of both paths on `engine`."""
    engine.set_option("batch_part_log2", tuned["batched"]["batch_part_log2"])
    engine.set_option("batch_load_pct", tuned["batched"]["batch_load_pct"])
    engine.set_option("radix_bits", tuned["plain"]["radix_bits"])
    engine.set_option("probe_group", tuned["plain"]["probe_group"])
