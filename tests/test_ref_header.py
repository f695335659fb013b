"""The reference's own include/plan.h against libhjgb300.so (CPU only).

A caller that keeps the reference's header, as the drop-in instructions say,
must (1) compile and link against the library's Contest:: exports and (2) lay
out every type crossing the boundary exactly as the library does.  Both are
checked here by compiling against a reference checkout (HJ_REFERENCE, default
below); skipped where there is none, as on hosts that only run the GPU tests."""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
REF_INC = Path(os.environ.get("HJ_REFERENCE", "/root/reference")) / "include"

pytestmark = pytest.mark.skipif(not (REF_INC / "plan.h").exists(), reason="reference checkout not present")


def _ref_flags() -> list[str]:
    import torch  # fmt ships header-only inside torch's include tree

    torch_inc = Path(torch.__file__).parent / "include"
    return ["-std=c++23", "-w", "-DFMT_HEADER_ONLY", "-I", str(ROOT / "oracle" / "shim"), "-I", str(REF_INC),
            "-I", str(torch_inc)]


def _run(cmd: list[str]) -> str:
    out = subprocess.run(cmd, capture_output=True, text=True)
    assert out.returncode == 0, " ".join(cmd) + "\n" + out.stdout + out.stderr
    return out.stdout


def test_boundary_types_have_the_reference_layout(tmp_path):
    ours, ref = tmp_path / "lp_ours", tmp_path / "lp_ref"
    _run(["g++", "-std=c++17", "-I", str(ROOT / "include"), str(ROOT / "tests" / "layout_probe.cpp"), "-o", str(ours)])
    _run(["g++", *_ref_flags(), str(ROOT / "tests" / "layout_probe.cpp"), "-o", str(ref)])
    a, b = _run([str(ours)]), _run([str(ref)])
    assert a == b
    assert "Page size 8192 align 8" in a


def test_harness_links_with_the_reference_header(hj, tmp_path):
    """The unit-test harness compiled against the reference's plan.h resolves
    Contest::build_context / execute / destroy_context in libhjgb300.so."""
    exe = tmp_path / "harness_ref"
    lib_dir = hj.LIB_PATH.parent
    _run(["g++", *_ref_flags(), "-O1", str(ROOT / "tests" / "contest_harness.cpp"), "-L", str(lib_dir), "-lhjgb300",
          f"-Wl,-rpath,{lib_dir}", "-Wl,--no-undefined", "-o", str(exe)])
    syms = _run(["nm", "-C", "-u", str(exe)])
    for name in ("Contest::build_context()", "Contest::destroy_context(void*)", "Contest::execute(Plan const&, void*)"):
        assert name in syms
    # and the library defines each of them
    defined = _run(["nm", "-C", "-D", "--defined-only", str(hj.LIB_PATH)])
    for name in ("Contest::build_context()", "Contest::destroy_context(void*)", "Contest::execute(Plan const&, void*)"):
        assert name in defined
