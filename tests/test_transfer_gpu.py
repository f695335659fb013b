"""Host <-> HBM transfers from page-locked memory (hj_host_register): input
pages and result buffers there move with one copy-engine transfer per run of
consecutive pages.  The results must be the same as from pageable memory (GPU
gather / scatter or staged) and as the oracle's, for plain executes, for both
result copy entry points and through the server with plans in flight."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest


def _summary(orc, res):
    return orc.summary(orc.Output(0, "", res.num_rows, [(c.type, c.pages) for c in res.columns]))


def _same(a, b):
    assert a[:3] == b[:3] and np.array_equal(a[3], b[3])


def _locked_inputs(hj, plan):
    arrays = [c.pages for t in plan.inputs for c in t.columns if c.num_pages]
    for a in arrays:
        hj.host_register(a)
    return arrays


def test_register_rejects_bad_ranges(hj):
    with pytest.raises(ValueError):
        hj.host_register(np.zeros(0, np.uint8))
    with pytest.raises(ValueError):
        hj.host_register(np.zeros((4, 4), np.uint8)[:, ::2])


@pytest.mark.gpu
@pytest.mark.parametrize("host_access", [1, 0])
def test_locked_inputs_and_outputs_match_pageable_and_oracle(engine, hj, orc, host_access):
    from hjgb300 import workloads
    w = workloads.c2(scale=0.004)
    engine.set_option("host_access", host_access)
    try:
        want = orc.summary(orc.run(orc.port(), w.plan))
        pageable = engine.execute(w.plan)
        _same(_summary(orc, pageable), want)
        locked = _locked_inputs(hj, w.plan)
        try:
            # copy_contiguous into a page-locked buffer (copy engine)
            res = engine.execute_raw(w.plan)
            L = hj.lib()
            cols = []
            try:
                nrows, ncols = C.c_uint64(), C.c_uint32()
                L.hj_result_shape(res, C.byref(nrows), C.byref(ncols))
                for i in range(ncols.value):
                    ty, npg = C.c_int32(), C.c_uint64()
                    L.hj_result_column(res, i, C.byref(ty), C.byref(npg))
                    buf = np.zeros((max(1, npg.value), hj.PAGE_SIZE), np.uint8)
                    hj.host_register(buf)
                    try:
                        if npg.value:
                            assert L.hj_result_copy_contiguous(engine.handle, res, i, buf.ctypes.data) == 0
                        # and copy_pages into page-locked pages, in two runs
                        pages = np.zeros((max(1, npg.value) + 1, hj.PAGE_SIZE), np.uint8)
                        hj.host_register(pages)
                        try:
                            idx = [p + (1 if p >= npg.value // 2 else 0) for p in range(npg.value)]
                            ptrs = (C.c_void_p * max(1, npg.value))(*[pages.ctypes.data + q * hj.PAGE_SIZE for q in idx])
                            if npg.value:
                                assert L.hj_result_copy_pages(engine.handle, res, i, ptrs) == 0
                            assert np.array_equal(pages[idx], buf[: npg.value])
                        finally:
                            hj.host_unregister(pages)
                    finally:
                        hj.host_unregister(buf)
                    cols.append(hj.Column(ty.value, buf[: npg.value].copy()))
                got = hj.Result(nrows.value, cols, *engine.stats(res))
            finally:
                engine.free_result(res)
            _same(_summary(orc, got), want)
        finally:
            for a in locked:
                hj.host_unregister(a)
    finally:
        engine.set_option("host_access", 1)


@pytest.mark.gpu
def test_locked_inputs_through_the_server_in_flight(engine, hj, orc):
    from hjgb300 import workloads
    w = workloads.c2(scale=0.004)
    want = orc.summary(orc.run(orc.port(), w.plan))
    locked = _locked_inputs(hj, w.plan)
    try:
        with hj.Server(engine, hbm_budget_bytes=8 << 30, slots=2) as srv:
            tickets = [srv.submit(w.plan) for _ in range(4)]
            for t in tickets:
                r, _ = srv.wait(t)
                try:
                    _same(_summary(orc, engine.fetch(r)), want)
                finally:
                    engine.free_result(r)
    finally:
        for a in locked:
            hj.host_unregister(a)
