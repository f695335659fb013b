"""Regenerates the golden fixtures in this directory from the reference itself.

Runs the UNMODIFIED reference sources of eleanalt/hash-join-optimizer,
compiled by oracle/Makefile into oracle/_ref/libhjref.so (needs the reference
checkout, so it runs only where that exists), and records:

  unit_cases.json     sorted result rows of the join unit cases (tests/cases.py:
                      the reference's tests/unit_tests.cpp cases + edge cases)
  unchained_kat.json  UnchainedHash<int32_t,...> directory words for key sets
                      (include/unchained.h, the class itself)
  writer_kat.json     Table::to_columnar page layout (header, packed data and
                      bitmap digests per page) for INT32 / VARCHAR columns
  configs_small.json  row count and order-independent checksum of the seeded
                      workloads at small scale (execute() of the reference)

Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "tests"))
sys.path.insert(0, str(ROOT / "oracle"))

from conftest import load_hj  # noqa: E402
import cases  # noqa: E402
import oracle  # noqa: E402

SMALL = {"c1": 0.01, "c2": 0.002, "c3": 0.01}

# UnchainedHash key sets: literal lists, or generated ("range", n) /
# ("random", seed, n) / ("zipf_mod", seed, n, a, mod)
KAT_SETS = {
    "single_7": [7],
    "dup_5x3": [5, 5, 5],
    "negatives": [-1, -2, -(2**31), 2**31 - 1, 0, 17, -17],
    "range_10000": ["range", 10000],  # unchained_tests.cpp:74-91
    "random_1000": ["random", 11, 1000],
    "zipf_dups_4096": ["zipf_mod", 12, 4096, 1.3, 700],
    **{f"pow2_boundary_{n}": ["range", n] for n in (1, 2, 3, 4, 5, 7, 8, 9, 15, 16, 17)},
}


def kat_keys(spec) -> np.ndarray:
    if spec and isinstance(spec[0], str):
        kind = spec[0]
        if kind == "range":
            return np.arange(spec[1], dtype=np.int32)
        if kind == "random":
            return np.random.default_rng(spec[1]).integers(-2**31, 2**31, size=spec[2], dtype=np.int64).astype(np.int32)
        if kind == "zipf_mod":
            return (np.random.default_rng(spec[1]).zipf(spec[3], size=spec[2]) % spec[4]).astype(np.int32)
        raise ValueError(spec)
    return np.array(spec, dtype=np.int32)


def page_digest(pages: np.ndarray, kind: int) -> list:
    """Per page: defined bytes only (the reference leaves the gap uninitialised)."""
    out = []
    for pg in pages:
        nr = int(pg[0]) | int(pg[1]) << 8
        cnt = int(pg[2]) | int(pg[3]) << 8
        if nr in (0xFFFF, 0xFFFE):
            body = pg[4:4 + cnt]
            bm = b""
        elif kind == oracle.INT32:
            body = pg[4:4 + 4 * cnt]
            bm = pg[8192 - (nr + 7) // 8:]
        else:
            offs = pg[4:4 + 2 * cnt].view(np.uint16)
            end = int(offs[-1]) if cnt else 0
            body = pg[4:4 + 2 * cnt + end]
            bm = pg[8192 - (nr + 7) // 8:]
        out.append([nr, cnt, hashlib.sha256(bytes(body)).hexdigest()[:16],
                    hashlib.sha256(bytes(bm)).hexdigest()[:16]])
    return out


def writer_inputs():
    r = np.random.default_rng(7)
    n = 5000
    ints = r.integers(-2**31, 2**31, size=n, dtype=np.int64).astype(np.int32)
    valid = (r.random(n) > 0.3).astype(np.uint8)
    lens = r.integers(0, 90, size=n)
    lens[[10, 11, 400]] = [9000, 8185, 20000]  # long strings and the 8185-byte limit
    offs = np.zeros(n + 1, np.uint64)
    np.cumsum(lens, out=offs[1:])
    data = r.integers(0x20, 0x7F, size=int(offs[-1]), dtype=np.uint8)
    svalid = (r.random(n) > 0.1).astype(np.uint8)
    return ints, valid, data, offs, svalid


def main() -> None:
    hj = load_hj()
    ref = oracle.ref()
    if ref is None:
        raise SystemExit("the compiled reference is not available here")

    # 1. unit cases
    unit = {}
    for name, (plan, truth, types) in cases.build_cases(hj).items():
        out = oracle.run(ref, plan)
        assert out.status == 0, (name, out.error)
        unit[name] = {"num_rows": out.num_rows, "types": [t for t, _ in out.columns],
                      "rows": [list(r) for r in oracle.canonical_rows(out)]}
    (HERE / "unit_cases.json").write_text(json.dumps(unit, indent=1) + "\n")

    # 2. UnchainedHash directory known-answer vectors (large sets by generator
    #    spec and digest of the little-endian directory words)
    kat = {}
    for name, spec in KAT_SETS.items():
        keys = kat_keys(spec)
        d = oracle.unchained_directory(keys, lib=ref)
        entry = {"spec": spec, "dir_size": int(d.size)}
        if d.size <= 64:
            entry["dir"] = [int(x) for x in d]
        entry["sha256"] = hashlib.sha256(d.astype("<u8").tobytes()).hexdigest()
        kat[name] = entry
    (HERE / "unchained_kat.json").write_text(json.dumps(kat, indent=1) + "\n")

    # 3. Table::to_columnar page layouts
    ints, valid, data, offs, svalid = writer_inputs()
    wk = {
        "int32_dense": page_digest(oracle.to_columnar_ref(oracle.INT32, ints), oracle.INT32),
        "int32_nulls": page_digest(oracle.to_columnar_ref(oracle.INT32, ints, valid), oracle.INT32),
        "varchar_nulls_long": page_digest(oracle.to_columnar_ref(oracle.VARCHAR, (data, offs), svalid),
                                          oracle.VARCHAR),
    }
    (HERE / "writer_kat.json").write_text(json.dumps(wk) + "\n")

    # 4. seeded workloads at small scale
    sys.path.insert(0, str(ROOT))
    from hjgb300 import workloads  # noqa: E402
    cfg = {}
    for name, scale in SMALL.items():
        w = getattr(workloads, name)(scale=scale)
        out = oracle.run(ref, w.plan)
        assert out.status == 0, out.error
        n, counts, cks, _ = oracle.summary(out)
        cfg[name] = {"scale": scale, "num_rows": n, "column_rows": counts, "checksum": str(cks)}
    (HERE / "configs_small.json").write_text(json.dumps(cfg, indent=1) + "\n")
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
