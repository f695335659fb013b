"""The multi-GPU form is replicas only: one process per GPU, a barrier and a
max over ranks around the timed region, no data-path collective.  Its host
side runs here as world_size-2 gloo ranks on the CPU."""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    d = bench.Dist()
    d.barrier()
    got = d.max(1.5 + rank)           # each rank's step time; the job's is the slowest
    low = -d.max(-(1.5 + rank))       # the lowest over ranks (the e2e link probe)
    q.put((rank, d.world, got, low))
    d.close()


def test_barrier_and_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2, 2.5, 1.5), (1, 2, 2.5, 1.5)]


def test_reference_arm_under_torchrun_prints_one_line_from_rank_0():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py",
           "--impl", "reference", "--gpus", "2", "--scale", "0.001", "--steps", "2", "--warmup", "1"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0


_NO_LIB = r"""
import json, sys
sys.path.insert(0, ".")
import bench
class A: pass
a = A()
a.workload, a.scale, a.steps, a.warmup, a.ref_budget_s = "c2", 0.001, 2, 1, 60.0
line = bench.run_reference(a, bench.Dist())
maps = open("/proc/self/maps").read()
print(json.dumps({"line": line, "lib_mapped": "libhjgb300" in maps,
                  "lib_loaded": sys.modules["hjgb300"]._lib is not None}))
"""


def test_reference_arm_never_loads_the_engine_library():
    """The reference arm builds its input pages with the oracle's writers and
    times the oracle: the engine library stays unloaded, and its config is the
    one the GPU arm prints for the same workload."""
    r = subprocess.run([sys.executable, "-c", _NO_LIB], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert not out["lib_mapped"] and not out["lib_loaded"]
    line = out["line"]
    assert line["unit"] == line["e2e"]["unit"] == line["cpu_baseline"]["unit"] == "probe tuples/s"
    assert line["config"]["workload"].startswith("c2: 16000 build")
    assert line["config"]["probe_tuples"] > 0 and line["config"]["output_rows"] > 0
    assert "whole workload" in line["cpu_baseline"]["sample"]
