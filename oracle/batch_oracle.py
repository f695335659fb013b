"""Test infrastructure: CPU restatement of the batched-join instances and of
their results.  Not part of the product.

A batch instance is a chain R0 x R1 x ... x Rm-1 of INT32 inner equi-joins on
one key (R0 probes R1, the result probes R2, ...), each relation a (key,
payload) pair of INT32 columns without NULLs.  The join semantics are the
reference's JoinAlgorithm (src/execute.cpp:60-186 of eleanalt/hash-join-
optimizer): every (probe row, build row) pair with equal keys is a result row,
duplicates give the cross product, row order is unspecified.  The result is
summarised by its row count and the sum mod 2^64 of one 64-bit fingerprint per
row over (key, payload of R0, ..., payload of Rm-1):

    state0          = (uint32(key) ^ 0x243f6a8885a308d3) * 0x9e3779b97f4a7c15
    state'          = (state ^ uint32(v)) * 0x9e3779b97f4a7c15   for v = p0, p1, ...
    row fingerprint = splitmix64 output function of the last state

`relation()` restates the synthetic instance generator: key domain [0, 2b)
for build size b; perm_j(x) = (x * 2654435761 + c_j) mod 2b; build relation j
holds perm_j(0..rows-1); the probe relation draws perm_1(x) with x uniform in
[0, b) (a hit) with probability match_q24 / 2^24, else perm_1(b + x) (a miss).

Pinned by tests/test_batch_oracle.py against the compiled reference's
execute() on the same relations (as a left-deep plan), and by the GPU tests
bit-for-bit against the device generator and both device join paths.
"""
from __future__ import annotations

import numpy as np

M64 = (1 << 64) - 1
GOLD = 0x9E3779B97F4A7C15
PERM_MUL = 2654435761


def _fin(x):
    """splitmix64's output function, on Python ints or uint64 arrays."""
    if isinstance(x, int):
        x &= M64
        x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & M64
        x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & M64
        return x ^ (x >> 31)
    x = x.astype(np.uint64, copy=True)
    x ^= x >> np.uint64(30)
    x *= np.uint64(0xBF58476D1CE4E5B9)
    x ^= x >> np.uint64(27)
    x *= np.uint64(0x94D049BB133111EB)
    x ^= x >> np.uint64(31)
    return x


def gen_base(seed: int, inst: int, rel: int, which: int) -> int:
    a = _fin((seed + GOLD * (inst + 1)) & M64)
    return _fin((a + 0xD1B54A32D192ED03 * (rel * 4 + which + 1)) & M64)


def gen_val(base: int, rows: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        x = np.uint64(base) + np.uint64(GOLD) * (rows.astype(np.uint64) + np.uint64(1))
    return _fin(x)


def relation(seed: int, inst: int, rel: int, build_rows: int, match_q24: int, rows: int):
    """(keys int32[rows], payload int32[rows]) of relation `rel` of instance `inst`."""
    b = int(build_rows)
    D = 2 * b
    r = np.arange(rows, dtype=np.uint64)
    c = gen_base(seed, inst, 1 if rel == 0 else rel, 3) % D
    if rel == 0:
        hit = (gen_val(gen_base(seed, inst, 0, 0), r) >> np.uint64(40)) < np.uint64(match_q24)
        x = gen_val(gen_base(seed, inst, 0, 2), r) % np.uint64(b) + np.where(hit, np.uint64(0), np.uint64(b))
    else:
        x = r
    keys = ((x * np.uint64(PERM_MUL) + np.uint64(c)) % np.uint64(D)).astype(np.int64).astype(np.int32)
    pay = (gen_val(gen_base(seed, inst, rel, 1), r) & np.uint64(0xFFFFFFFF)).astype(np.uint32).view(np.int32)
    return keys, pay


def fp_add(st: np.ndarray, v: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        return (st.astype(np.uint64) ^ v.astype(np.int32).view(np.uint32).astype(np.uint64)) * np.uint64(GOLD)


def fp_start(key: np.ndarray, p0: np.ndarray) -> np.ndarray:
    k = key.astype(np.int32).view(np.uint32).astype(np.uint64)
    with np.errstate(over="ignore"):
        st = (k ^ np.uint64(0x243F6A8885A308D3)) * np.uint64(GOLD)
    return fp_add(st, p0)


def fp_final(st: np.ndarray) -> np.ndarray:
    return _fin(st)


def _join(pk: np.ndarray, bk: np.ndarray):
    """Every (probe row, build row) pair with equal keys (sort-merge)."""
    order = np.argsort(bk, kind="stable")
    sk = bk[order]
    lo = np.searchsorted(sk, pk, side="left")
    hi = np.searchsorted(sk, pk, side="right")
    cnt = (hi - lo).astype(np.int64)
    prow = np.repeat(np.arange(pk.size, dtype=np.int64), cnt)
    start = np.repeat(lo - np.concatenate(([0], np.cumsum(cnt)[:-1])), cnt)
    brow = order[start + np.arange(prow.size, dtype=np.int64)]
    return prow, brow


def chain_rows(rels):
    """Result rows of the chain: (key int32[n], payloads int32[m, n])."""
    key, pays = rels[0][0], [rels[0][1]]
    for bk, bp in rels[1:]:
        prow, brow = _join(key, bk)
        key = key[prow]
        pays = [p[prow] for p in pays] + [bp[brow]]
    return key, np.array(pays, dtype=np.int32).reshape(len(rels), -1)


def row_fingerprints(key: np.ndarray, pays: np.ndarray) -> np.ndarray:
    st = fp_start(key, pays[0])
    for p in pays[1:]:
        st = fp_add(st, p)
    return fp_final(st)


def chain_result(rels):
    """(row count, checksum) of the chain [(keys, payload), ...]."""
    key, pays = chain_rows(rels)
    fp = row_fingerprints(key, pays)
    return int(key.size), int(fp.sum(dtype=np.uint64)) if fp.size else 0


def instance_relations(seed: int, inst: int, num_relations: int, build_rows: int, match_q24: int,
                       probe_rows: int):
    return [relation(seed, inst, j, build_rows, match_q24, probe_rows if j == 0 else build_rows)
            for j in range(num_relations)]
