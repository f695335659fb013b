"""Test infrastructure: Python side of the oracle.  Not part of the product.

  port()  liboracle.so -- CPU restatement of the reference join path
          (ref_port.cpp) plus the result checker (checker.cpp)
  ref()   _ref/libhjref.so -- the reference's own sources compiled here
          (None where the reference checkout is absent, e.g. on GPU hosts)

`run(lib, plan)` executes a plan (the engine package's Plan, flattened to the
C ABI of include/hj_api.h) and returns its pages; `decode`, `fingerprints`,
`checksum` and `canonical_rows` check results independently of the GPU
library's own page decoder.  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg use this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass
from pathlib import Path
from typing import Optional

import numpy as np

HERE = Path(__file__).resolve().parent
PAGE = 8192
INT32, VARCHAR = 0, 3


class OracleResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("error", C.c_char * 256), ("num_rows", C.c_uint64),
                ("num_columns", C.c_uint32), ("types", C.POINTER(C.c_int32)),
                ("num_pages", C.POINTER(C.c_uint64)), ("pages", C.POINTER(C.POINTER(C.c_uint8)))]


@dataclass
class Output:
    status: int
    error: str
    num_rows: int
    columns: list  # [(type, pages ndarray (n, 8192) uint8)]


_port: Optional[C.CDLL] = None
_ref: Optional[C.CDLL] = None


def build(with_ref: bool = True) -> None:
    """Builds liboracle.so (and _ref when the reference sources exist)."""
    targets = ["port"] + (["ref"] if with_ref else [])
    subprocess.run(["make", "-s", "-C", str(HERE), *targets], check=True)


def _setup(L: C.CDLL, execute_name: str) -> C.CDLL:
    fn = getattr(L, execute_name)
    fn.argtypes = [C.c_void_p, C.POINTER(OracleResult)]
    fn.restype = C.c_int
    L.oracle_result_free.argtypes = [C.POINTER(OracleResult)]
    L.oracle_result_free.restype = None
    return L


def port() -> C.CDLL:
    global _port
    if _port is None:
        so = HERE / "liboracle.so"
        build(with_ref=False)  # make: rebuilds when a source or include/hj_api.h changed
        L = _setup(C.CDLL(str(so)), "oracle_execute")
        vp, u64 = C.c_void_p, C.c_uint64
        L.oracle_decode_int32.argtypes = [vp, u64, vp, vp, u64, C.POINTER(u64)]
        L.oracle_decode_strings.argtypes = [vp, u64, vp, u64, vp, vp, u64, C.POINTER(u64), C.POINTER(u64)]
        L.oracle_row_hashes.argtypes = [vp, u64, C.c_uint32, C.c_int32, vp, vp, vp, vp]
        L.oracle_checksum.argtypes = [vp, u64]
        L.oracle_checksum.restype = u64
        L.oracle_unchained_directory.argtypes = [vp, u64, vp, u64, C.POINTER(u64)]
        L.oracle_unchained_counts.argtypes = [vp, u64, vp, u64, vp]
        L.oracle_last_stats.argtypes = [C.POINTER(u64), C.POINTER(u64), C.POINTER(C.c_double)]
        L.oracle_last_stats.restype = None
        L.oracle_pages_from_int32.argtypes = [vp, vp, u64, vp, u64, C.POINTER(u64)]
        L.oracle_pages_from_strings.argtypes = [vp, vp, vp, u64, vp, u64, C.POINTER(u64)]
        _port = L
    return _port


def ref() -> Optional[C.CDLL]:
    """The compiled reference, or None when it cannot exist on this machine."""
    global _ref
    if _ref is None:
        so = HERE / "_ref" / "libhjref.so"
        if Path(os.environ.get("HJ_REFERENCE", "/root/reference"), "src").is_dir():
            build(with_ref=True)  # make: rebuilds when a source or include/hj_api.h changed
        elif not so.exists():
            return None
        try:
            L = _setup(C.CDLL(str(so)), "ref_execute")
        except OSError:  # built for another architecture
            return None
        vp, u64 = C.c_void_p, C.c_uint64
        L.ref_to_columnar_int32.argtypes = [vp, vp, u64, C.POINTER(OracleResult)]
        L.ref_to_columnar_strings.argtypes = [vp, vp, vp, u64, C.POINTER(OracleResult)]
        L.ref_unchained_directory.argtypes = [vp, u64, vp, u64, C.POINTER(u64)]
        L.ref_unchained_counts.argtypes = [vp, u64, vp, u64, vp]
        L.ref_pdh_directory.argtypes = [vp, u64, u64, C.c_uint32, vp]
        _ref = L
    return _ref


def _collect(L: C.CDLL, r: OracleResult) -> Output:
    cols = []
    for c in range(r.num_columns):
        n = int(r.num_pages[c])
        buf = np.ctypeslib.as_array(r.pages[c], shape=(max(1, n) * PAGE,))[: n * PAGE]
        cols.append((int(r.types[c]), buf.copy().reshape(n, PAGE)))
    out = Output(int(r.status), r.error.decode(errors="replace"), int(r.num_rows), cols)
    L.oracle_result_free(C.byref(r))
    return out


def run(L: C.CDLL, plan) -> Output:
    """Runs plan (engine Plan object) through oracle_execute or ref_execute."""
    d, keep = plan.desc()
    r = OracleResult()
    fn = L.oracle_execute if hasattr(L, "oracle_execute") else L.ref_execute
    fn(C.addressof(d), C.byref(r))
    return _collect(L, r)


def timed_execute(plan) -> dict:
    """One restated execute() of `plan` for timing: its result pages are freed
    uncopied.  Returns rows, build / probe tuples (summed over the joins) and
    the seconds from the call to the finished result pages."""
    L = port()
    d, keep = plan.desc()
    r = OracleResult()
    L.oracle_execute(C.addressof(d), C.byref(r))
    if r.status != 0:
        err = r.error.decode(errors="replace")
        L.oracle_result_free(C.byref(r))
        raise RuntimeError(err)
    b, p, sec = C.c_uint64(), C.c_uint64(), C.c_double()
    L.oracle_last_stats(C.byref(b), C.byref(p), C.byref(sec))
    rows = int(r.num_rows)
    L.oracle_result_free(C.byref(r))
    return {"rows": rows, "build_tuples": b.value, "probe_tuples": p.value, "seconds": sec.value}


def to_columnar_ref(kind: int, values, valid=None):
    """Pages the reference's Table::to_columnar writes for one column."""
    L = ref()
    r = OracleResult()
    m = None if valid is None else np.ascontiguousarray(valid, np.uint8)
    if kind == INT32:
        v = np.ascontiguousarray(values, np.int32)
        L.ref_to_columnar_int32(v.ctypes.data, None if m is None else m.ctypes.data, v.size, C.byref(r))
    else:
        data, offs = values
        b = np.ascontiguousarray(data, np.uint8)
        o = np.ascontiguousarray(offs, np.uint64)
        L.ref_to_columnar_strings(b.ctypes.data if b.size else None, o.ctypes.data,
                                  None if m is None else m.ctypes.data, o.size - 1, C.byref(r))
    return _collect(L, r).columns[0][1]


def page_writer(kind: str, *arrays) -> np.ndarray:
    """Reference-format pages of one column written by the oracle's own writers
    (pages.cpp): kind "int32" with (values, valid) or "strings" with (bytes,
    offsets, valid).  The engine package calls this instead of its library's
    writers once hooked in with `use_page_writer(oracle.page_writer)`."""
    L = port()
    n = C.c_uint64()
    if kind == "int32":
        v, m = arrays
        args = (v.ctypes.data, None if m is None else m.ctypes.data, v.size)
        fn = L.oracle_pages_from_int32
    else:
        b, o, m = arrays
        args = (b.ctypes.data if b.size else None, o.ctypes.data, None if m is None else m.ctypes.data, o.size - 1)
        fn = L.oracle_pages_from_strings
    fn(*args, None, 0, C.byref(n))
    pages = np.zeros((n.value, PAGE), dtype=np.uint8)
    rc = fn(*args, pages.ctypes.data if n.value else None, n.value, C.byref(n))
    assert rc == 0
    return pages


# ------------------------------------------------------------------ checker --

def decode_column(kind: int, pages: np.ndarray):
    """INT32 -> (vals, valid); VARCHAR -> (bytes, offsets, valid)."""
    L = port()
    n_pages = pages.shape[0]
    pages = np.ascontiguousarray(pages)
    n = C.c_uint64()
    if kind == INT32:
        L.oracle_decode_int32(pages.ctypes.data, n_pages, None, None, 0, C.byref(n))
        vals = np.zeros(max(1, n.value), np.int32)
        valid = np.zeros(max(1, n.value), np.uint8)
        rc = L.oracle_decode_int32(pages.ctypes.data, n_pages, vals.ctypes.data, valid.ctypes.data,
                                   n.value, C.byref(n))
        assert rc == 0
        return vals[: n.value], valid[: n.value]
    nb = C.c_uint64()
    L.oracle_decode_strings(pages.ctypes.data, n_pages, None, 0, None, None, 0, C.byref(n), C.byref(nb))
    data = np.zeros(max(1, nb.value), np.uint8)
    offs = np.zeros(n.value + 1, np.uint64)
    valid = np.zeros(max(1, n.value), np.uint8)
    rc = L.oracle_decode_strings(pages.ctypes.data, n_pages, data.ctypes.data, nb.value, offs.ctypes.data,
                                 valid.ctypes.data, n.value, C.byref(n), C.byref(nb))
    assert rc == 0
    return data[: nb.value], offs, valid[: n.value]


def decode(out_columns) -> list:
    return [(kind, decode_column(kind, pages)) for kind, pages in out_columns]


def column_rows(dec) -> int:
    kind, d = dec
    return int(d[1].size if kind == INT32 else d[2].size)


def fingerprints(decoded: list, n: int) -> np.ndarray:
    """Per-row 64-bit fingerprints over all columns (in column order)."""
    L = port()
    h = np.zeros(max(1, n), np.uint64)
    for ci, (kind, d) in enumerate(decoded):
        if kind == INT32:
            vals, valid = d
            L.oracle_row_hashes(h.ctypes.data, n, ci, kind, vals.ctypes.data, None, None, valid.ctypes.data)
        else:
            data, offs, valid = d
            L.oracle_row_hashes(h.ctypes.data, n, ci, kind, None, data.ctypes.data, offs.ctypes.data,
                                valid.ctypes.data)
    return h[:n]


def checksum(fp: np.ndarray) -> int:
    return int(port().oracle_checksum(np.ascontiguousarray(fp).ctypes.data, fp.size))


def summary(out: Output):
    """(num_rows, per-column row counts, checksum, sorted fingerprints)."""
    dec = decode(out.columns)
    counts = [column_rows(d) for d in dec]
    n = counts[0] if counts else 0
    fp = fingerprints(dec, n) if dec and all(c == n for c in counts) else np.zeros(0, np.uint64)
    return out.num_rows, counts, checksum(fp), np.sort(fp)


def canonical_rows(out: Output) -> list:
    """Decoded rows as sorted Python tuples (small results only); None = NULL."""
    dec = decode(out.columns)
    cols = []
    for kind, d in dec:
        if kind == INT32:
            vals, valid = d
            cols.append([int(v) if ok else None for v, ok in zip(vals, valid)])
        else:
            data, offs, valid = d
            cols.append([bytes(data[offs[i]:offs[i + 1]]).decode("latin-1") if valid[i] else None
                         for i in range(valid.size)])
    rows = list(zip(*cols)) if cols else []
    return sorted(rows, key=lambda r: tuple((True, 0) if x is None else (False, x) for x in r))


def unchained_directory(keys: np.ndarray, lib: C.CDLL | None = None) -> np.ndarray:
    """UnchainedHash directory words for int32 keys (restatement, or the
    reference's own class when lib is ref())."""
    k = np.ascontiguousarray(keys, np.int32)
    cap = 2 * max(1, k.size) + 2
    out = np.zeros(cap, np.uint64)
    ds = C.c_uint64()
    if lib is None:
        port().oracle_unchained_directory(k.ctypes.data, k.size, out.ctypes.data, cap, C.byref(ds))
    else:
        lib.ref_unchained_directory(k.ctypes.data, k.size, out.ctypes.data, cap, C.byref(ds))
    return out[: ds.value + 1] if ds.value else out[:0]


def unchained_counts(build: np.ndarray, probe: np.ndarray, lib: C.CDLL | None = None) -> np.ndarray:
    b = np.ascontiguousarray(build, np.int32)
    p = np.ascontiguousarray(probe, np.int32)
    out = np.zeros(max(1, p.size), np.uint64)
    L = lib if lib is not None else port()
    fn = L.ref_unchained_counts if lib is not None else L.oracle_unchained_counts
    fn(b.ctypes.data, b.size, p.ctypes.data, p.size, out.ctypes.data)
    return out[: p.size]
