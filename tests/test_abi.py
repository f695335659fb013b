"""The C-ABI library loads and exports every entry point include/*.h declares
(no compute calls: these run without a GPU)."""
from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions() -> set[str]:
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        # strip comments
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b(hj_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(hj):
    lib = hj.lib()
    declared = declared_functions()
    assert declared, "no C entry points found in include/"
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"
    assert set(hj.EXPORTS) <= declared


def test_symbols_are_plain_c(hj):
    out = subprocess.run(["nm", "-D", "--defined-only", str(hj.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    for name in declared_functions():
        assert name in exported, f"{name} is not an unmangled C symbol"
    # the C++ drop-in entry points (Contest::build_context/destroy_context/execute)
    assert any("7Contest7execute" in s for s in exported)
    assert any("7Contest13build_context" in s for s in exported)
    assert any("7Contest15destroy_context" in s for s in exported)


def test_version_string(hj):
    v = hj.lib().hj_version()
    assert b"sm_103a" in v


def test_host_page_writer_runs_without_gpu(hj):
    col = hj.Column.int32([1, 2, 3], [1, 0, 1])
    assert col.num_pages == 1
    vals, valid = hj.decode_int32(col)
    assert valid.tolist() == [True, False, True]
    assert vals[valid].tolist() == [1, 3]


def test_context_create_without_device_fails_cleanly(hj):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = hj.lib()
    assert not lib.hj_context_create(0)
    assert b"device" in lib.hj_last_error(None)
    with pytest.raises(hj.HjError):
        hj.Engine()


def test_invalid_arguments_are_rejected_without_gpu(hj):
    lib = hj.lib()
    assert lib.hj_execute(None, None, None) == hj.HJ_ERR_INVALID
    assert lib.hj_set_option(None, b"dir_bits", 3) == hj.HJ_ERR_INVALID
    n = C.c_uint64()
    assert lib.hj_pages_from_int32(None, None, 5, None, 0, C.byref(n)) == hj.HJ_ERR_INVALID


def test_scan_filters_reach_the_c_abi_and_the_oracle_refuses_them(hj, orc):
    import ctypes as C
    p = hj.Plan()
    p.new_input(hj.Table(3, [hj.Column.int32(np.array([1, 2, 3], np.int32))]))
    p.root = p.new_scan_node(0, [(0, hj.INT32)], filters=[(0, hj.CMP_GEQ, 2), (0, hj.CMP_IS_NOT_NULL, 0)])
    d, keep = p.desc()
    n = d.nodes[0]
    assert n.num_filters == 2 and n.filters[0].op == hj.CMP_GEQ and n.filters[0].value == 2
    assert C.sizeof(hj.FilterDesc) == 24
    out = orc.run(orc.port(), p)
    assert out.status != 0 and "filter" in out.error
