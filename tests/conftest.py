"""Shared fixtures.  The engine package (directory hash-join-optimizer_gb300)
is imported as module `hjgb300`; the oracle (test infrastructure) from oracle/."""
from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG_DIR = ROOT / "hash-join-optimizer_gb300"
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "tests"))


def load_hj():
    if "hjgb300" in sys.modules:
        return sys.modules["hjgb300"]
    spec = importlib.util.spec_from_file_location("hjgb300", PKG_DIR / "__init__.py",
                                                  submodule_search_locations=[str(PKG_DIR)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["hjgb300"] = mod
    spec.loader.exec_module(mod)
    if not mod.LIB_PATH.exists():
        build_spec = importlib.util.spec_from_file_location("hjgb300_build", PKG_DIR / "build.py")
        b = importlib.util.module_from_spec(build_spec)
        build_spec.loader.exec_module(b)
        b.build()
    return mod


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 host)")


@pytest.fixture(scope="session")
def hj():
    return load_hj()


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.port()
    return oracle


@pytest.fixture(scope="session")
def engine(hj):
    e = hj.Engine()
    yield e
    e.close()


def sort_key(row):
    return tuple((True, 0) if x is None else (False, x) for x in row)


def canon(rows):
    return sorted([tuple(r) for r in rows], key=sort_key)
