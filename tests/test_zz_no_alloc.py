"""hj_table_probe_noalloc: the probe for callers that cannot allocate device
memory during the call (engines with their own fixed-budget sub-allocator,
embedders whose memory pool must not grow after start-up, latency-critical
paths).  Its temporaries live in a fixed array inside the library instead of
per-call allocations; its matches must be those of hj_table_probe.

Collected last (file name) so that a run stopping at the first failure has run
every other test first; it creates its own engine and passes alone as well."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pairs(op, ob, n):
    p = op[:n].cpu().numpy().astype(np.int64)
    b = ob[:n].cpu().numpy().astype(np.int64)
    return np.sort(p << 32 | b)


def test_noalloc_probe_matches_allocating_probe(hj):
    import torch
    L = hj.lib()
    r = np.random.default_rng(21)
    build = (r.zipf(1.2, 300_000) % 40_000).astype(np.int32)          # skewed duplicates
    build[:3] = [2**31 - 1, -(2**31), -9]
    probe = r.integers(-50, 45_000, hj.NOALLOC_MAX_PROBE_ROWS).astype(np.int32)
    probe[:2] = [2**31 - 1, -9]
    valid = r.random(probe.size) > 0.05
    bits = np.packbits(valid.astype(np.uint8), bitorder="little")
    bits = np.pad(bits, (0, (-bits.size) % 4)).view(np.uint32)
    with hj.Engine() as eng:
        kb, kp = torch.from_numpy(build).cuda(), torch.from_numpy(probe).cuda()
        vb = torch.from_numpy(bits.copy()).cuda()
        t = C.c_void_p()
        assert L.hj_table_build(eng.handle, kb.data_ptr(), None, kb.numel(), -1, C.byref(t)) == 0
        try:
            for call in range(2):  # two calls in a row share the static scratch
                n1, n2 = C.c_uint64(), C.c_uint64()
                assert L.hj_table_probe(eng.handle, t, kp.data_ptr(), vb.data_ptr(), kp.numel(), None, None, 0,
                                        C.byref(n1)) == hj.HJ_ERR_CAPACITY
                cap = n1.value
                assert cap > 0
                ap = torch.empty(cap, dtype=torch.int32, device="cuda")
                ab = torch.empty(cap, dtype=torch.int32, device="cuda")
                assert L.hj_table_probe(eng.handle, t, kp.data_ptr(), vb.data_ptr(), kp.numel(), ap.data_ptr(),
                                        ab.data_ptr(), cap, C.byref(n1)) == 0
                bp = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
                bb = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
                rc = L.hj_table_probe_noalloc(eng.handle, t, kp.data_ptr(), vb.data_ptr(), kp.numel(),
                                              bp.data_ptr(), bb.data_ptr(), cap, C.byref(n2))
                assert rc == 0, L.hj_last_error(eng.handle)
                assert n2.value == n1.value, call
                # integer row ids: identical match multisets (order is unspecified)
                assert np.array_equal(_pairs(bp, bb, cap), _pairs(ap, ab, cap)), call
                assert np.array_equal(probe[bp.cpu().numpy()], build[bb.cpu().numpy()])
            # too small an output buffer: the count, nothing written
            small = C.c_uint64()
            assert L.hj_table_probe_noalloc(eng.handle, t, kp.data_ptr(), vb.data_ptr(), kp.numel(), None, None, 0,
                                            C.byref(small)) == hj.HJ_ERR_CAPACITY
            assert small.value == n1.value
            # more probe rows than the static scratch holds: rejected with a clear error
            big = torch.zeros(hj.NOALLOC_MAX_PROBE_ROWS + 1, dtype=torch.int32, device="cuda")
            rc = L.hj_table_probe_noalloc(eng.handle, t, big.data_ptr(), None, big.numel(), None, None, 0,
                                          C.byref(small))
            assert rc == hj.HJ_ERR_INVALID
            assert b"limit" in L.hj_last_error(eng.handle)
        finally:
            L.hj_table_free(t)
