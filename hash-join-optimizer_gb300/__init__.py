"""Python binding of the GB300 hash-join engine (C ABI in include/hj_api.h).

Mirrors the contest API of eleanalt/hash-join-optimizer (include/plan.h):
`Plan.new_scan_node / new_join_node / new_input`, tables of 8 KiB pages in the
reference format, and `Engine.execute(plan)` returning the root's columns as
pages.  The engine runs on the GPU only: importing works anywhere, but
creating an `Engine` needs the built library and a CUDA device and raises
otherwise -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

PAGE_SIZE = 8192
INT32, INT64, FP64, VARCHAR = 0, 1, 2, 3
NODE_JOIN, NODE_SCAN = 0, 1
# scan filter operators (Comparison::Op numbering)
CMP_EQ, CMP_NEQ, CMP_LT, CMP_GT, CMP_LEQ, CMP_GEQ, CMP_IS_NULL, CMP_IS_NOT_NULL = 0, 1, 2, 3, 4, 5, 8, 9

HJ_OK, HJ_ERR_INVALID, HJ_ERR_RUNTIME, HJ_ERR_OUT_OF_RANGE = 0, 1, 2, 3
HJ_ERR_CUDA, HJ_ERR_NO_DEVICE, HJ_ERR_CAPACITY, HJ_ERR_DEVICE_STATUS, HJ_ERR_NOMEM = 4, 5, 6, 7, 8

LIB_PATH = Path(__file__).resolve().parent / "libhjgb300.so"

# every symbol include/hj_api.h declares
EXPORTS = [
    "hj_context_create", "hj_context_destroy", "hj_last_error", "hj_version", "hj_context_stream",
    "hj_set_option", "hj_get_option", "hj_table_upload", "hj_table_release",
    "hj_execute", "hj_result_shape", "hj_result_column", "hj_result_copy_pages",
    "hj_result_copy_contiguous", "hj_result_stats", "hj_result_phase_ms", "hj_result_counter", "hj_result_free",
    "hj_table_build", "hj_table_info", "hj_table_probe", "hj_table_free",
    "hj_pages_from_int32", "hj_pages_from_strings", "hj_table_probe_noalloc",
    "hj_batch_execute", "hj_batch_generate", "hj_table_prepare",
    "hj_server_create", "hj_server_submit", "hj_server_wait", "hj_server_info", "hj_server_destroy",
    "hj_table_dump", "hj_table_load", "hj_host_register", "hj_host_unregister",
]
BATCH_PERSISTENT, BATCH_PLAIN = 0, 1
NOALLOC_MAX_PROBE_ROWS = 65536  # HJ_NOALLOC_MAX_PROBE_ROWS


class HjError(RuntimeError):
    """An engine call failed; `status` is the HJ_* code."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


# ---------------------------------------------------------------- C structs --

class ColumnDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("num_pages", C.c_uint64), ("pages", C.POINTER(C.c_void_p))]


class TableDesc(C.Structure):
    _fields_ = [("num_rows", C.c_uint64), ("num_columns", C.c_uint32),
                ("columns", C.POINTER(ColumnDesc)), ("resident", C.c_uint64)]


class Attr(C.Structure):
    _fields_ = [("index", C.c_uint64), ("type", C.c_int32)]


class FilterDesc(C.Structure):
    _fields_ = [("column", C.c_uint64), ("op", C.c_int32), ("pad", C.c_int32), ("value", C.c_int64)]


class NodeDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("build_left", C.c_int32), ("base_table_id", C.c_uint64),
                ("left", C.c_uint64), ("right", C.c_uint64), ("left_attr", C.c_uint64),
                ("right_attr", C.c_uint64), ("num_attrs", C.c_uint32), ("attrs", C.POINTER(Attr)),
                ("num_filters", C.c_uint32), ("filters", C.POINTER(FilterDesc))]


class PlanDesc(C.Structure):
    _fields_ = [("num_nodes", C.c_uint32), ("nodes", C.POINTER(NodeDesc)),
                ("num_inputs", C.c_uint32), ("inputs", C.POINTER(TableDesc)), ("root", C.c_uint64)]


class BatchRelation(C.Structure):
    _fields_ = [("keys", C.c_void_p), ("payload", C.c_void_p), ("rows", C.c_uint64)]


class BatchInstance(C.Structure):
    _fields_ = [("num_relations", C.c_uint32), ("relations", C.POINTER(BatchRelation))]


class ServerOptions(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("slots", C.c_uint32)]


class RequestStats(C.Structure):
    _fields_ = [("queue_ms", C.c_double), ("service_ms", C.c_double), ("latency_ms", C.c_double),
                ("est_bytes", C.c_uint64)]


_lib: Optional[C.CDLL] = None


def lib() -> C.CDLL:
    """Loads libhjgb300.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise HjError(HJ_ERR_NO_DEVICE, f"{LIB_PATH.name} is not built; run build.py")
    L = C.CDLL(str(LIB_PATH))
    vp, u64, i32, i64, u32 = C.c_void_p, C.c_uint64, C.c_int32, C.c_int64, C.c_uint32
    P = C.POINTER
    L.hj_context_create.restype = vp
    L.hj_context_create.argtypes = [C.c_int]
    L.hj_context_destroy.argtypes = [vp]
    L.hj_last_error.restype = C.c_char_p
    L.hj_last_error.argtypes = [vp]
    L.hj_version.restype = C.c_char_p
    L.hj_context_stream.restype = vp
    L.hj_context_stream.argtypes = [vp]
    L.hj_result_phase_ms.argtypes = [vp, C.c_char_p, P(C.c_double)]
    L.hj_set_option.argtypes = [vp, C.c_char_p, i64]
    L.hj_get_option.argtypes = [vp, C.c_char_p, P(i64)]
    L.hj_table_upload.argtypes = [vp, P(TableDesc), P(u64)]
    L.hj_table_release.argtypes = [vp, u64]
    L.hj_execute.argtypes = [vp, P(PlanDesc), P(vp)]
    L.hj_result_shape.argtypes = [vp, P(u64), P(u32)]
    L.hj_result_column.argtypes = [vp, u32, P(i32), P(u64)]
    L.hj_result_copy_pages.argtypes = [vp, vp, u32, P(vp)]
    L.hj_result_copy_contiguous.argtypes = [vp, vp, u32, vp]
    L.hj_host_register.argtypes = [vp, u64]
    L.hj_host_unregister.argtypes = [vp]
    L.hj_result_stats.argtypes = [vp, P(u64), P(u64), P(u64)]
    L.hj_result_counter.argtypes = [vp, C.c_char_p, P(u64)]
    L.hj_result_free.argtypes = [vp]
    L.hj_table_build.argtypes = [vp, vp, vp, u64, i32, P(vp)]
    L.hj_table_info.argtypes = [vp, P(u32), P(u64), P(vp), P(vp), P(vp)]
    L.hj_table_probe.argtypes = [vp, vp, vp, vp, u64, vp, vp, u64, P(u64)]
    L.hj_table_free.argtypes = [vp]
    L.hj_table_probe_noalloc.argtypes = [vp, vp, vp, vp, u64, vp, vp, u64, P(u64)]
    L.hj_pages_from_int32.argtypes = [vp, vp, u64, vp, u64, P(u64)]
    L.hj_pages_from_strings.argtypes = [vp, vp, vp, u64, vp, u64, P(u64)]
    L.hj_batch_execute.argtypes = [vp, P(BatchInstance), u32, i32, P(u64), P(u64), P(u32)]
    L.hj_batch_generate.argtypes = [vp, u64, u32, u32, u64, u32, u64, vp, vp]
    L.hj_table_prepare.argtypes = [vp, u64]
    L.hj_table_dump.argtypes = [P(TableDesc), C.c_char_p]
    L.hj_table_load.argtypes = [vp, C.c_char_p, P(u64)]
    L.hj_server_create.restype = vp
    L.hj_server_create.argtypes = [vp, P(ServerOptions)]
    L.hj_server_submit.argtypes = [vp, P(PlanDesc), P(u64)]
    L.hj_server_wait.argtypes = [vp, u64, P(vp), P(RequestStats), C.c_char_p, u32]
    L.hj_server_info.argtypes = [vp, P(u64), P(u64), P(u64), P(u64)]
    L.hj_server_destroy.argtypes = [vp]
    L.hj_server_destroy.restype = None
    L.hj_context_destroy.restype = None
    L.hj_result_free.restype = None
    L.hj_table_free.restype = None
    _lib = L
    return L


def _ptr(a: Optional[np.ndarray]) -> Optional[int]:
    return None if a is None else a.ctypes.data


# Writer of host pages for Column.int32 / Column.varchar: None = the library's
# hj_pages_from_int32 / hj_pages_from_strings.
_page_writer = None


def use_page_writer(fn) -> None:
    """Builds host tables with `fn(kind, *arrays) -> (n, 8192) uint8 pages`
    (kind "int32": (values, valid); "strings": (bytes, offsets, valid)) instead
    of the library's writers, so that a process that only prepares
    reference-format tables need not load the GPU library.  None restores the
    library's writers."""
    global _page_writer
    _page_writer = fn


# --------------------------------------------------------------- host tables --

@dataclass
class Column:
    """One column as reference-format pages: `pages` is (num_pages, 8192) uint8."""
    type: int
    pages: np.ndarray

    @property
    def num_pages(self) -> int:
        return int(self.pages.shape[0])

    @staticmethod
    def int32(values, valid=None) -> "Column":
        """Packs like Table::to_columnar (src/build_table.cpp:666-700)."""
        v = np.ascontiguousarray(values, dtype=np.int32)
        m = None if valid is None else np.ascontiguousarray(valid, dtype=np.uint8)
        if _page_writer is not None:
            return Column(INT32, _page_writer("int32", v, m))
        n = C.c_uint64()
        L = lib()
        _check(None, L.hj_pages_from_int32(_ptr(v), _ptr(m), v.size, None, 0, C.byref(n)))
        pages = np.zeros((n.value, PAGE_SIZE), dtype=np.uint8)
        _check(None, L.hj_pages_from_int32(_ptr(v), _ptr(m), v.size, _ptr(pages), n.value, C.byref(n)))
        return Column(INT32, pages)

    @staticmethod
    def varchar(data, offsets=None, valid=None) -> "Column":
        """Strings as (bytes, offsets[n+1], valid) or a list of bytes/str/None."""
        if offsets is None:
            items = list(data)
            valid = np.array([x is not None for x in items], dtype=np.uint8)
            enc = [b"" if x is None else (x.encode() if isinstance(x, str) else bytes(x)) for x in items]
            offsets = np.zeros(len(enc) + 1, dtype=np.uint64)
            offsets[1:] = np.cumsum([len(x) for x in enc]) if enc else []
            data = np.frombuffer(b"".join(enc), dtype=np.uint8) if enc else np.zeros(0, np.uint8)
        b = np.ascontiguousarray(data, dtype=np.uint8)
        o = np.ascontiguousarray(offsets, dtype=np.uint64)
        m = None if valid is None else np.ascontiguousarray(valid, dtype=np.uint8)
        nrows = o.size - 1
        if _page_writer is not None:
            return Column(VARCHAR, _page_writer("strings", b, o, m))
        n = C.c_uint64()
        L = lib()
        bp = _ptr(b) if b.size else None
        _check(None, L.hj_pages_from_strings(bp, _ptr(o), _ptr(m), nrows, None, 0, C.byref(n)))
        pages = np.zeros((n.value, PAGE_SIZE), dtype=np.uint8)
        _check(None, L.hj_pages_from_strings(bp, _ptr(o), _ptr(m), nrows, _ptr(pages), n.value, C.byref(n)))
        return Column(VARCHAR, pages)


@dataclass
class Table:
    """ColumnarTable: num_rows + columns of pages."""
    num_rows: int
    columns: list = field(default_factory=list)
    resident: int = 0  # handle from Engine.upload(); 0 = host pages


@dataclass
class Plan:
    """The contest Plan (include/plan.h:173-210)."""
    nodes: list = field(default_factory=list)
    inputs: list = field(default_factory=list)
    root: int = 0

    def new_scan_node(self, base_table_id: int, output_attrs: Sequence[tuple],
                      filters: Sequence[tuple] = ()) -> int:
        """filters: (column, CMP_* operator, int literal) triples, AND-combined, on INT32
        columns of the table (the reference applies them while loading the table)."""
        node = ("scan", int(base_table_id), [(int(i), int(t)) for i, t in output_attrs])
        if filters:
            node = node + ([(int(c), int(o), int(v)) for c, o, v in filters],)
        self.nodes.append(node)
        return len(self.nodes) - 1

    def new_join_node(self, build_left: bool, left: int, right: int, left_attr: int, right_attr: int,
                      output_attrs: Sequence[tuple]) -> int:
        self.nodes.append(("join", (bool(build_left), int(left), int(right), int(left_attr),
                                    int(right_attr)), [(int(i), int(t)) for i, t in output_attrs]))
        return len(self.nodes) - 1

    def new_input(self, table: Table) -> int:
        self.inputs.append(table)
        return len(self.inputs) - 1

    def desc(self):
        """(PlanDesc, keepalive) for the C ABI; keepalive must outlive the call."""
        keep = []
        nodes = (NodeDesc * max(1, len(self.nodes)))()
        for i, node in enumerate(self.nodes):
            kind, data, attrs = node[:3]
            arr = (Attr * max(1, len(attrs)))(*[Attr(a, t) for a, t in attrs])
            keep.append(arr)
            nd = nodes[i]
            nd.num_attrs, nd.attrs = len(attrs), arr
            if kind == "scan":
                nd.kind, nd.base_table_id = NODE_SCAN, data
                if len(node) > 3:
                    fl = (FilterDesc * len(node[3]))(*[FilterDesc(c, o, 0, v) for c, o, v in node[3]])
                    keep.append(fl)
                    nd.num_filters, nd.filters = len(node[3]), fl
            else:
                nd.kind = NODE_JOIN
                nd.build_left, nd.left, nd.right, nd.left_attr, nd.right_attr = int(data[0]), *data[1:]
        tables = (TableDesc * max(1, len(self.inputs)))()
        for i, t in enumerate(self.inputs):
            cols = (ColumnDesc * max(1, len(t.columns)))()
            for j, col in enumerate(t.columns):
                cols[j].type, cols[j].num_pages, cols[j].pages = col.type, col.num_pages, _page_ptrs(col, keep)
            keep.append(cols)
            tables[i].num_rows, tables[i].num_columns = t.num_rows, len(t.columns)
            tables[i].columns, tables[i].resident = cols, t.resident
        keep += [nodes, tables]
        d = PlanDesc(len(self.nodes), nodes, len(self.inputs), tables, self.root)
        return d, keep

    def frozen(self) -> "FrozenPlan":
        """The descriptor built once, for plans submitted many times unchanged."""
        return FrozenPlan(*self.desc())


@dataclass
class FrozenPlan:
    """A Plan's C-ABI descriptor, built once (Plan.frozen)."""
    d: object
    keep: list

    def desc(self):
        return self.d, self.keep


def _page_ptrs(col: "Column", keep: list):
    """Array of the column's page addresses (kept alive through `keep`)."""
    arr = np.arange(max(1, col.num_pages), dtype=np.uint64) * np.uint64(PAGE_SIZE) + np.uint64(col.pages.ctypes.data)
    keep.append(arr)
    return arr.ctypes.data_as(C.POINTER(C.c_void_p))


def host_register(a: np.ndarray) -> None:
    """Page-locks the memory of a contiguous array (hj_host_register): input
    pages and result buffers there move through the copy engines."""
    if not a.flags.c_contiguous or a.nbytes == 0:
        raise ValueError("host_register needs a non-empty contiguous array")
    _check(None, lib().hj_host_register(a.ctypes.data, a.nbytes))


def host_unregister(a: np.ndarray) -> None:
    _check(None, lib().hj_host_unregister(a.ctypes.data))


def _check(ctx, rc: int) -> None:
    if rc != HJ_OK:
        msg = lib().hj_last_error(ctx)
        raise HjError(rc, msg.decode() if msg else "error")


@dataclass
class Result:
    num_rows: int
    columns: list  # list[Column]
    build_tuples: int = 0
    probe_tuples: int = 0
    output_rows: int = 0
    phases: dict = field(default_factory=dict)  # device ms per phase (option "timing")

PHASES = ("upload", "decode", "build", "probe", "probe_sync", "probe_write", "materialize", "mat_varchar_plan",
          "mat_sync", "mat_varchar_write", "total", "launches")


class Engine:
    """A context on one GPU (Contest::build_context / destroy_context)."""

    def __init__(self, device: int = -1):
        L = lib()
        self._ctx = L.hj_context_create(device)
        if not self._ctx:
            msg = L.hj_last_error(None)
            raise HjError(HJ_ERR_NO_DEVICE, msg.decode() if msg else "no CUDA device")

    def close(self) -> None:
        if self._ctx:
            lib().hj_context_destroy(self._ctx)
            self._ctx = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> int:
        return self._ctx

    @property
    def stream(self) -> int:
        """cudaStream_t of the engine (for torch.cuda.ExternalStream)."""
        return lib().hj_context_stream(self._ctx)

    def set_option(self, name: str, value: int) -> None:
        _check(self._ctx, lib().hj_set_option(self._ctx, name.encode(), int(value)))

    def get_option(self, name: str) -> int:
        v = C.c_int64()
        _check(self._ctx, lib().hj_get_option(self._ctx, name.encode(), C.byref(v)))
        return v.value

    def upload(self, table: Table) -> Table:
        """Uploads a host table to HBM; returns a Table that refers to it."""
        cols = (ColumnDesc * max(1, len(table.columns)))()
        keep = []
        for j, col in enumerate(table.columns):
            cols[j].type, cols[j].num_pages, cols[j].pages = col.type, col.num_pages, _page_ptrs(col, keep)
        td = TableDesc(table.num_rows, len(table.columns), cols, 0)
        h = C.c_uint64()
        _check(self._ctx, lib().hj_table_upload(self._ctx, C.byref(td), C.byref(h)))
        return Table(table.num_rows, [Column(c.type, np.zeros((0, PAGE_SIZE), np.uint8)) for c in table.columns],
                     resident=h.value)

    def release(self, table: Table) -> None:
        _check(self._ctx, lib().hj_table_release(self._ctx, table.resident))

    def load_table(self, path) -> Table:
        """A table file (the reference's cache format) uploaded as a resident table."""
        h = C.c_uint64()
        _check(self._ctx, lib().hj_table_load(self._ctx, str(path).encode(), C.byref(h)))
        head = np.fromfile(str(path), dtype=np.uint8, count=208)
        num_rows, ncols = (int(x) for x in head[:16].view(np.uint64))
        types = head[16:80].view(np.int32)[:ncols]
        return Table(num_rows, [Column(int(t), np.zeros((0, PAGE_SIZE), np.uint8)) for t in types],
                     resident=h.value)

    def prepare(self, table: Table) -> None:
        """Decodes a resident table's columns once and keeps them decoded in HBM."""
        _check(self._ctx, lib().hj_table_prepare(self._ctx, table.resident))

    def server(self, hbm_budget_bytes: int, slots: int) -> "Server":
        return Server(self, hbm_budget_bytes, slots)

    def execute_raw(self, plan: Plan) -> int:
        """Runs the plan and returns the opaque hj_result pointer (pages stay in HBM)."""
        d, keep = plan.desc()
        res = C.c_void_p()
        _check(self._ctx, lib().hj_execute(self._ctx, C.byref(d), C.byref(res)))
        return res.value

    def fetch(self, res: int) -> Result:
        L = lib()
        nrows, ncols = C.c_uint64(), C.c_uint32()
        L.hj_result_shape(res, C.byref(nrows), C.byref(ncols))
        cols = []
        for i in range(ncols.value):
            ty, np_ = C.c_int32(), C.c_uint64()
            L.hj_result_column(res, i, C.byref(ty), C.byref(np_))
            pages = np.empty((np_.value, PAGE_SIZE), dtype=np.uint8)
            if np_.value:
                _check(self._ctx, L.hj_result_copy_contiguous(self._ctx, res, i, pages.ctypes.data))
            cols.append(Column(ty.value, pages))
        return Result(nrows.value, cols, *self.stats(res))

    def stats(self, res: int):
        """(build tuples, probe tuples, output rows, {phase: device ms})."""
        L = lib()
        b, p, o = C.c_uint64(), C.c_uint64(), C.c_uint64()
        L.hj_result_stats(res, C.byref(b), C.byref(p), C.byref(o))
        ph = {}
        for name in PHASES:
            ms = C.c_double()
            L.hj_result_phase_ms(res, name.encode(), C.byref(ms))
            ph[name] = ms.value
        return b.value, p.value, o.value, ph

    def counters(self, res: int) -> dict:
        """hj_result_counter: directory words, table tuples, joins and kernel launches of a result."""
        out = {}
        for name in ("dir_words", "table_tuples", "joins", "launches"):
            v = C.c_uint64()
            _check(self._ctx, lib().hj_result_counter(res, name.encode(), C.byref(v)))
            out[name] = v.value
        return out

    def free_result(self, res: int) -> None:
        lib().hj_result_free(res)

    def batch_generate(self, seed: int, instance: int, relation: int, build_rows: int, match_q24: int,
                       rows: int, keys: int, payload: int) -> None:
        """hj_batch_generate: one synthetic relation into device buffers (enqueued on `stream`)."""
        _check(self._ctx, lib().hj_batch_generate(self._ctx, seed, instance, relation, build_rows, match_q24,
                                                  rows, keys, payload))

    def batch_execute(self, instances: Sequence[Sequence[tuple]], mode: int = BATCH_PERSISTENT):
        """hj_batch_execute over instances given as [(keys ptr, payload ptr, rows), ...]
        per relation (device pointers).  Returns (rows uint64[n], checksums uint64[n],
        instances recomputed on the plain path)."""
        n = len(instances)
        rels = [(BatchRelation * len(inst))(*[BatchRelation(k, p, r) for k, p, r in inst]) for inst in instances]
        arr = (BatchInstance * max(1, n))()
        for i, r in enumerate(rels):
            arr[i].num_relations, arr[i].relations = len(r), r
        rows = np.zeros(max(1, n), dtype=np.uint64)
        sums = np.zeros(max(1, n), dtype=np.uint64)
        redo = C.c_uint32()
        _check(self._ctx, lib().hj_batch_execute(self._ctx, arr, n, mode,
                                                 rows.ctypes.data_as(C.POINTER(C.c_uint64)),
                                                 sums.ctypes.data_as(C.POINTER(C.c_uint64)), C.byref(redo)))
        return rows[:n], sums[:n], redo.value

    def execute(self, plan: Plan) -> Result:
        """Contest::execute: runs the plan and returns the root's pages on the host."""
        res = self.execute_raw(plan)
        try:
            return self.fetch(res)
        finally:
            self.free_result(res)


class Server:
    """hj_server: a request loop running plans concurrently on the engine's GPU
    against an HBM budget.  submit() returns a ticket; wait() blocks until that
    plan ran and returns (result handle, stats dict); free results with
    Engine.free_result, fetch them with Engine.fetch."""

    def __init__(self, engine: Engine, hbm_budget_bytes: int, slots: int):
        self.engine = engine
        opt = ServerOptions(int(hbm_budget_bytes), int(slots))
        self._s = lib().hj_server_create(engine.handle, C.byref(opt))
        if not self._s:
            msg = lib().hj_last_error(engine.handle)
            raise HjError(HJ_ERR_INVALID, msg.decode() if msg else "hj_server_create failed")
        self._keep = {}

    def submit(self, plan: Plan) -> int:
        d, keep = plan.desc()
        t = C.c_uint64()
        _check(self.engine.handle, lib().hj_server_submit(self._s, C.byref(d), C.byref(t)))
        self._keep[t.value] = (d, keep)  # host pages of non-resident inputs stay alive until wait
        return t.value

    def wait(self, ticket: int):
        res = C.c_void_p()
        st = RequestStats()
        err = C.create_string_buffer(512)
        rc = lib().hj_server_wait(self._s, ticket, C.byref(res), C.byref(st), err, 512)
        self._keep.pop(ticket, None)
        if rc != HJ_OK:
            raise HjError(rc, err.value.decode(errors="replace"))
        return res.value, {"queue_ms": st.queue_ms, "service_ms": st.service_ms, "latency_ms": st.latency_ms,
                           "est_bytes": st.est_bytes}

    def info(self) -> dict:
        q, r, rb, pb = C.c_uint64(), C.c_uint64(), C.c_uint64(), C.c_uint64()
        lib().hj_server_info(self._s, C.byref(q), C.byref(r), C.byref(rb), C.byref(pb))
        return {"queued": q.value, "running": r.value, "running_bytes": rb.value, "peak_bytes": pb.value}

    def close(self) -> None:
        if self._s:
            lib().hj_server_destroy(self._s)
            self._s = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def dump_table(table: Table, path) -> None:
    """Writes a host table in the reference's binary cache format (DumpTable)."""
    cols = (ColumnDesc * max(1, len(table.columns)))()
    keep = []
    for j, col in enumerate(table.columns):
        cols[j].type, cols[j].num_pages, cols[j].pages = col.type, col.num_pages, _page_ptrs(col, keep)
    td = TableDesc(table.num_rows, len(table.columns), cols, 0)
    rc = lib().hj_table_dump(C.byref(td), str(path).encode())
    if rc != HJ_OK:
        raise HjError(rc, f"hj_table_dump({path}) failed")


# ------------------------------------------------------------ page decoding --

def decode_int32(col: Column):
    """INT32 pages -> (values int32[n], valid bool[n]) (reader of the reference
    page format, src/build_table.cpp:527-540)."""
    vals, valid = [], []
    for pg in col.pages:
        nr = int(pg[0]) | (int(pg[1]) << 8)
        data = pg[4:4 + 4 * 2047].view(np.int32)
        bm = np.unpackbits(pg[PAGE_SIZE - (nr + 7) // 8:], bitorder="little")[:nr].astype(bool)
        v = np.zeros(nr, dtype=np.int32)
        v[bm] = data[: int(bm.sum())]
        vals.append(v)
        valid.append(bm)
    if not vals:
        return np.zeros(0, np.int32), np.zeros(0, bool)
    return np.concatenate(vals), np.concatenate(valid)


def decode_varchar(col: Column) -> list:
    """VARCHAR pages -> list of bytes / None."""
    out: list = []
    for pg in col.pages:
        nr = int(pg[0]) | (int(pg[1]) << 8)
        cnt = int(pg[2]) | (int(pg[3]) << 8)
        if nr == 0xFFFF:
            out.append(bytes(pg[4:4 + cnt]))
            continue
        if nr == 0xFFFE:
            out[-1] = out[-1] + bytes(pg[4:4 + cnt])
            continue
        offs = pg[4:4 + 2 * cnt].view(np.uint16)
        data = pg[4 + 2 * cnt:]
        bm = np.unpackbits(pg[PAGE_SIZE - (nr + 7) // 8:], bitorder="little")[:nr]
        k, start = 0, 0
        for i in range(nr):
            if bm[i]:
                end = int(offs[k])
                out.append(bytes(data[start:end]))
                start, k = end, k + 1
            else:
                out.append(None)
    return out
