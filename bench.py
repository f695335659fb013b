#!/usr/bin/env python3
"""Probe throughput of the GB300 hash-join engine on the 16M x 256M skewed join.

Workload (default c2): 16M-row build side (INT32 keys Zipf(1.1) over 4M ranks,
2 INT32 payloads with 20% NULLs, ASCII VARCHAR 8-64 B), 256M raw probe rows
pre-filtered to ~25.6M by `pred < 100` (keys Zipf(1.1) over 8M ranks, 2 INT32
payloads with 20% NULLs, VARCHAR), all payloads of both sides in the output.
A step is one Contest::execute of that plan: page decode, unchained-table
build, probe, and the output written as reference-format pages.

  value  probe tuples/s with the input pages already resident in HBM
         (device time of whole steps, CUDA events on the engine's stream)
  e2e    the same through the C ABI with HOST input pages: upload, execute and
         the copy of every result page back to host memory in the timed region
  roofline  the probe phase (count + write kernels) against measured HBM
         bandwidth, algorithmic bytes 4*N_probe + 8*D + 8*N_build + 8*N_out
  cpu_baseline  the oracle restatement of the reference's execute() on the
         same inputs, all host threads (the whole workload when it takes at
         most about 30 s of CPU time, else a stated probe-side prefix)

The default c2 line also carries `workloads` (c1 and c3 at full size, device
time, probe roofline and CPU baseline of each) and `systems` (the batched and
served forms at reduced size, each against the plain path).  `--workload c4`
adds a CPU baseline on a seeded 64-instance sample.

The inputs (>2 GB of pages) exceed the 126 MB L2, so no flush is needed
between steps.  `--impl reference` times the CPU restatement alone, one
execute() of the same workload per step, with input pages built by the
oracle's own page writers (the engine library is never loaded).
Multi-GPU (torchrun): independent replicas, one per GPU (the path has no
exchange step); value = all ranks' probe tuples / max step time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["c1", "c2", "c2raw", "c3", "c4", "c5"], default="c2")
    ap.add_argument("--rates", default="50,100,200,500,1000,2000,5000", help="c5: offered queries/s")
    ap.add_argument("--requests", type=int, default=200, help="c5: requests per rate")
    ap.add_argument("--slots", type=int, default=8, help="c5: plans running at once")
    ap.add_argument("--budget-gb", type=float, default=150.0, help="c5: HBM admission budget")
    ap.add_argument("--instances", type=int, default=4096, help="c4: batch instances")
    ap.add_argument("--wave-rows", type=int, default=1 << 32, help="c4: input rows per wave")
    ap.add_argument("--retune", action="store_true", help="c4: ignore the autotuner cache")
    ap.add_argument("--plain-instances", type=int, default=-1,
                    help="c4: instances timed on the plain path (-1 = all)")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--cpu-budget-s", type=float, default=30.0,
                    help="CPU seconds the cpu_baseline leg may spend; a prefix of the probe side is timed "
                         "when one execute() of the whole workload would exceed it")
    ap.add_argument("--ref-budget-s", type=float, default=240.0,
                    help="--impl reference: seconds for all steps; a probe-side prefix per step when the "
                         "whole workload would exceed it")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--opt", action="append", default=[], metavar="NAME=VALUE",
                    help="engine option for the timed runs (hj_set_option), repeatable")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-systems", action="store_true",
                    help="c2: leave out the batched and served summaries (c4 / c5 at reduced size)")
    ap.add_argument("--no-workloads", action="store_true",
                    help="c2: leave out the c1 and c3 summaries (full size, 100 steps each)")
    ap.add_argument("--e2e-depth", type=int, default=3,
                    help="plans in flight in the pipelined end-to-end mode (1 = serial only)")
    ap.add_argument("--e2e-pageable", action="store_true",
                    help="end to end from pageable host memory (GPU gather / scatter) instead of page-locked")
    return ap.parse_args()


# ------------------------------------------------------------- distributed --

class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ------------------------------------------------------------------ clocks --

class Clocks:
    """nvidia-smi samples (200 ms) of one GPU during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.p = None
        return self

    def __exit__(self, *exc):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self) -> dict:
        self.f.flush()
        rows = []
        for line in Path(self.f.name).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1])]
        mx = [num(r[2]) for r in rows if num(r[2])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# --------------------------------------------------------------- workloads --

def make_workload(hj, name: str, scale: float):
    from hjgb300 import workloads
    return getattr(workloads, name)(scale=scale)


def peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(workload: str):
    """DRAM bytes per launch of the probe kernels from a committed ncu summary."""
    p = ROOT / "profiles" / f"probe_traffic_{workload}.json"
    if p.exists():
        try:
            return json.loads(p.read_text()).get("bytes_per_step")
        except (ValueError, KeyError):
            return None
    return None


def oracle_mod():
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    return oracle


def workload_config(w, args, world: int, build_tuples: int, probe_tuples: int, output_rows: int) -> dict:
    """The `config` of a plain-path line; both arms print the same one."""
    raw = w.meta.get("probe_rows_raw")
    desc = {"c1": "c1: 1,000,000 build x 10,000,000 probe rows, unique permuted keys",
            "c2": f"c2: {w.build_rows} build x {raw} raw probe rows ({w.probe_rows} after the pre-filter)",
            "c2raw": f"c2raw: {w.build_rows} build x {raw} raw probe rows, predicate pred < 100 in the plan",
            "c3": "c3: 5-relation left-deep chain, " + " / ".join(str(k) for k in w.meta.get("kept", []))
                  + " rows after the pre-filters (of " + " / ".join(str(k) for k in w.meta.get("sizes", [])) + ")"}
    return {"workload": desc.get(w.name, w.name), "scale": args.scale, "build_tuples": build_tuples,
            "probe_tuples": probe_tuples, "output_rows": output_rows, "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2"}


def cpu_reference_steps(w, oracle, steps: int, warmup: int, budget_s: float):
    """Times `steps` restated execute() calls after `warmup` untimed ones, all
    host threads.  The whole workload per call when (steps + warmup) calls fit
    in budget_s (judged from the first call), else the plan's probe-side
    prefix sized to fit.  Returns (seconds per step, probe tuples per step,
    stats of the last call, sample description)."""
    threads = os.cpu_count() or 1
    os.environ["SIGMOD_THREADS"] = str(threads)
    first = oracle.timed_execute(w.plan)
    plan, k = w.plan, None
    per_call = first["seconds"]
    if (steps + max(0, warmup - 1)) * per_call > budget_s and w.sample is not None:
        frac = budget_s / ((steps + warmup) * per_call)
        k = max(1, int(w.probe_rows * frac))
        plan = w.sample(k)
    for _ in range(max(0, warmup - 1)):
        oracle.timed_execute(plan)
    times, st = [], first
    for _ in range(steps):
        st = oracle.timed_execute(plan)
        times.append(st["seconds"])
    if k is None:
        sample = (f"the whole workload per step ({st['build_tuples']} build and {st['probe_tuples']} probe tuples, "
                  f"{st['rows']} result rows); execute() to finished result pages, {threads} threads")
    else:
        sample = (f"first {k} of {w.probe_rows} probe rows against the whole build side per step (the whole "
                  f"workload took {per_call:.1f} s per execute()); {threads} threads")
    return statistics.median(times), st["probe_tuples"], st, sample


# --------------------------------------------------------- end to end ---

def run_e2e(args, d: Dist, hj, eng, w, npr: int, out_pages: list, stream) -> dict:
    """The metric through the C ABI with HOST buffers: every step uploads its
    input pages from page-locked host memory (hj_host_register; copy engines)
    and copies every result column back into page-locked host buffers.

    serial:    one hj_execute + result copy at a time.
    pipelined: the same steps through hj_server with --e2e-depth plans in
               flight, so that the upload of one plan, the kernels of another
               and the result download of a third overlap (the link carries
               both directions at once for page-locked memory).
    Both modes are reported (`modes`); `value` is the faster one, named in
    `mode`.  Each mode's time is a median over timed blocks, leaving out blocks
    that a busy host link slowed (see `timed`)."""
    import ctypes as C
    import collections
    import numpy as np
    import torch

    L = hj.lib()
    inputs = [c.pages for t in w.plan.inputs for c in t.columns if c.num_pages]
    # VARCHAR page counts follow the (unspecified) output row order, so each
    # result is sized on its own; buffers get 10% slack, touched up front so
    # that first-touch page faults stay out of the timed region
    host_bufs = []
    for n in out_pages:
        b = np.empty((int(n * 1.1) + 1, hj.PAGE_SIZE), np.uint8)
        b.fill(0)
        host_bufs.append(b)
    locked = []
    if not args.e2e_pageable:
        for a in inputs + host_bufs:
            hj.host_register(a)
            locked.append(a)
    h2d = sum(a.nbytes for a in inputs)
    d2h_seen = []
    step_parts = []  # per serial step: upload, execute and fetch ms

    def fetch(r):
        total = 0
        for i in range(len(host_bufs)):
            ty, npg = C.c_int32(), C.c_uint64()
            L.hj_result_column(r, i, C.byref(ty), C.byref(npg))
            if host_bufs[i].shape[0] < npg.value:
                raise RuntimeError("result column larger than its host buffer")
            if npg.value:
                assert L.hj_result_copy_contiguous(eng.handle, r, i, host_bufs[i].ctypes.data) == 0
            total += npg.value
        d2h_seen.append(total * hj.PAGE_SIZE)

    host_plan = w.plan.frozen()  # descriptor built once; the pages are read every step

    def serial_step():
        t0 = time.perf_counter()
        r = eng.execute_raw(host_plan)
        t1 = time.perf_counter()
        up = eng.stats(r)[3].get("upload", 0.0)
        fetch(r)
        step_parts.append((up, 1e3 * (t1 - t0) - up, 1e3 * (time.perf_counter() - t1)))
        eng.free_result(r)

    # the host link's bandwidth right before each timed block: a 512 MiB
    # copy each way between page-locked host memory and HBM (copy engines)
    probe_h = torch.empty(256 << 20, dtype=torch.int16, pin_memory=True)
    probe_d = torch.empty(256 << 20, dtype=torch.int16, device=f"cuda:{d.local}")

    def link_gbs():
        out = []
        for dst, src in ((probe_d, probe_h), (probe_h, probe_d)):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                a.record(stream)
                dst.copy_(src, non_blocking=True)
                b.record(stream)
            b.synchronize()
            out.append(round(src.numel() * 2 / (a.elapsed_time(b) * 1e6), 1))
        return out

    all_links = []  # every link probe of the run, both modes

    def timed(fn, k, blocks=9, links=None):
        """Median over `blocks` timed blocks of k steps.  The host link is
        shared with the machine's other GPUs, whose traffic shows up as slow
        blocks; `links` collects the link probe taken before each block (the
        lowest over ranks).  Blocks whose probe found either direction below
        80% of the best probe so far in this run (either mode) are left out of
        the median when at least three blocks remain; otherwise every block
        counts.  Returns the median,
        every block's time and the indices of the blocks in the median."""
        per = []
        for _ in range(blocks):
            d.barrier()
            torch.cuda.synchronize()
            if links is not None:
                links.append([-d.max(-x) for x in link_gbs()])
                all_links.append(links[-1])
            s2, e2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s2.record(stream)
            fn(k)
            e2.record(stream)
            torch.cuda.synchronize()
            per.append(d.max(s2.elapsed_time(e2) / k))
        used = list(range(len(per)))
        if links:
            best = [max(x[i] for x in all_links) for i in (0, 1)]
            quiet = [b for b, x in enumerate(links) if all(x[i] >= 0.8 * best[i] for i in (0, 1))]
            if len(quiet) >= 3:
                used = quiet
        sel = sorted(per[b] for b in used)
        return sel[len(sel) // 2], per, used

    k2 = max(1, min(args.steps, 5))
    try:
        serial_step()
        step_parts.clear()
        d2h_seen.clear()
        serial_links = []
        serial_ms, serial_blocks, serial_used = timed(lambda k: [serial_step() for _ in range(k)], k2,
                                                      links=serial_links)
        # steps of the blocks in the median (block b holds steps b*k2 .. b*k2+k2-1)
        kept = [p for i, p in enumerate(step_parts) if i // k2 in serial_used]
        modes = {"serial": {"ms_per_step": serial_ms, "blocks_ms_per_step": [round(x, 3) for x in serial_blocks],
                            "link_gbs_h2d_d2h_before_block": serial_links, "blocks_in_median": serial_used,
                            "parts_ms": {key: round(sum(p[i] for p in kept) / max(1, len(kept)), 3)
                                         for i, key in enumerate(("upload_ms", "execute_ms", "fetch_ms"))}}}
        out = {"value": npr * d.world / (serial_ms / 1e3), "unit": "probe tuples/s", "ms_per_step": serial_ms,
               "mode": "serial", "host_memory": "pageable" if args.e2e_pageable else "page-locked",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": int(sum(d2h_seen) / max(1, len(d2h_seen))),
               "modes": modes}
        depth = args.e2e_depth
        if depth > 1:
            srv = hj.Server(eng, hbm_budget_bytes=int(args.budget_gb * 2**30), slots=depth)
            try:
                # per plan, to see where overlap is lost: its upload (device time),
                # its time in a slot (upload + execute) and the client's fetch
                seen = {"upload_ms": [], "service_ms": [], "fetch_ms": []}

                def finish(ticket):
                    r, st = srv.wait(ticket)
                    seen["upload_ms"].append(eng.stats(r)[3].get("upload", 0.0))
                    seen["service_ms"].append(st["service_ms"])
                    t0 = time.perf_counter()
                    fetch(r)
                    seen["fetch_ms"].append(1e3 * (time.perf_counter() - t0))
                    eng.free_result(r)

                def pipelined(k):
                    q = collections.deque()
                    for _ in range(k):
                        q.append(srv.submit(w.plan))
                        if len(q) >= depth:
                            finish(q.popleft())
                    while q:
                        finish(q.popleft())
                kp = max(k2, 3 * depth)
                # warm the slots: each slot's first plans set up its stream's pools
                for _ in range(2):
                    pipelined(kp)
                for v in seen.values():
                    v.clear()
                pipe_links = []
                pipe_ms, pipe_blocks, pipe_used = timed(pipelined, kp, links=pipe_links)
            finally:
                srv.close()
            modes["pipelined"] = {"ms_per_step": pipe_ms, "plans_in_flight": depth,
                                  "blocks_ms_per_step": [round(x, 3) for x in pipe_blocks],
                                  "link_gbs_h2d_d2h_before_block": pipe_links, "blocks_in_median": pipe_used,
                                  "median_per_plan_ms": {k: round(sorted(v)[len(v) // 2], 3)
                                                         for k, v in seen.items() if v}}
            if pipe_ms < serial_ms:
                out.update({"value": npr * d.world / (pipe_ms / 1e3), "ms_per_step": pipe_ms,
                            "mode": f"pipelined through hj_server, {depth} plans in flight"})
        return out
    finally:
        for a in locked:
            hj.host_unregister(a)


# ------------------------------------------------------------------- ours ---

def run_ours(args, d: Dist) -> dict:
    import numpy as np
    import torch
    from __graft_entry__ import load

    hj = load()
    torch.cuda.set_device(d.local)
    eng = hj.Engine(d.local)
    eng.set_option("timing", 1)
    for o in args.opt:
        k, v = o.split("=", 1)
        eng.set_option(k, int(v))
    w = make_workload(hj, args.workload, args.scale)
    stream = torch.cuda.ExternalStream(eng.stream)

    # ---- device-resident inputs; the plan's C-ABI descriptor is built once,
    # as a caller that submits the same plan repeatedly holds it
    resident_plan = hj.Plan(w.plan.nodes, [eng.upload(t) for t in w.plan.inputs], w.plan.root)
    resident = resident_plan.frozen()
    first = eng.execute_raw(resident)
    nb, npr, nout, _ = eng.stats(first)
    out_pages = []
    L = hj.lib()
    import ctypes as C
    nrows, ncols = C.c_uint64(), C.c_uint32()
    L.hj_result_shape(first, C.byref(nrows), C.byref(ncols))
    for i in range(ncols.value):
        ty, np_ = C.c_int32(), C.c_uint64()
        L.hj_result_column(first, i, C.byref(ty), C.byref(np_))
        out_pages.append(np_.value)
    eng.free_result(first)
    for _ in range(max(0, args.warmup - 1)):
        eng.free_result(eng.execute_raw(resident))

    # ---- timed steps: whole executes, no per-phase events (option timing off)
    L_counter = hj.lib().hj_result_counter
    launches = 0
    nlaunch = C.c_uint64()
    eng.set_option("timing", 0)
    with Clocks(d.local) as clk:
        d.barrier()
        torch.cuda.synchronize()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for _ in range(args.steps):
            r = eng.execute_raw(resident)
            L_counter(r, b"launches", C.byref(nlaunch))
            launches += nlaunch.value
            eng.free_result(r)
        end.record(stream)
        torch.cuda.synchronize()
        d.barrier()
    ms = d.max(start.elapsed_time(end) / args.steps)
    clocks = clk.summary()
    # ---- phase times from a second pass with per-phase CUDA events (which
    # add about 35 us of host work per execute, so they stay out of `value`)
    eng.set_option("timing", 1)
    # (per phase the median over the steps: one step that the host stalls
    # between two events must not move a phase's figure)
    phase_steps = min(args.steps, 50)
    phase_seen = {}
    for _ in range(phase_steps):
        r = eng.execute_raw(resident)
        for k, v in eng.stats(r)[3].items():
            phase_seen.setdefault(k, []).append(v)
        last = r
        if _ < phase_steps - 1:
            eng.free_result(r)
    last_counters = eng.counters(last)
    eng.free_result(last)
    phases = {k: round(statistics.median(v), 4) for k, v in phase_seen.items() if k != "launches"}

    # ---- roofline of the probe phase: directory words and table tuples of
    # the tables this execute built (summed over its joins)
    cnt = last_counters
    D, nt = cnt["dir_words"], cnt["table_tuples"]
    a_probe = 4 * npr + 8 * D + 8 * nt + 8 * nout
    # the probe kernels: count + write, without the host readback between them
    t_probe = (phases.get("probe", 0.0) + phases.get("probe_write", 0.0)) / 1e3
    peak, peak_kind = peaks()
    achieved = a_probe / t_probe / 1e9 if t_probe > 0 else None
    roofline = {"bound": "hbm", "kernel": "probe (count + write kernels)", "achieved": achieved,
                "peak": peak, "unit": "GB/s", "frac": achieved / peak if achieved else None,
                "traffic": ncu_traffic(args.workload), "algorithmic_bytes": a_probe,
                "bytes_formula": f"4*N_probe + 8*D + 8*N_table + 8*N_out = 4*{npr} + 8*{D} + 8*{nt} + 8*{nout}",
                "probe_ms": t_probe * 1e3,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind}

    # ---- end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, d, hj, eng, w, npr, out_pages, stream)

    # ---- CPU baseline (rank 0): the oracle restatement on the same inputs
    cpu = None
    if d.rank == 0 and not args.no_cpu_baseline:
        sec, ptup, _st, sample = cpu_reference_steps(w, oracle_mod(), 1, 1, args.cpu_budget_s)
        cpu = {"value": ptup / sec, "unit": "probe tuples/s", "cores": os.cpu_count() or 1, "kind": "port",
               "sample": sample + f"; {sec:.2f} s per execute()"}

    for t in resident_plan.inputs:
        eng.release(t)
    eng.close()
    return {
        "metric": "probe tuples/s", "value": npr * d.world / (ms / 1e3), "unit": "probe tuples/s",
        "n_gpus": d.world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded generator with the configured shapes; inputs > L2, no flush needed)",
        "config": workload_config(w, args, d.world, nb, npr, nout),
        "build_tuples_per_s": nb * d.world / (ms / 1e3),
        "phases_ms": phases, "phases_from": f"median of {phase_steps} further steps with per-phase CUDA events",
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": launches, "clocks": clocks,
    }


def chain_plan(hj, rels):
    """A c4 instance [(keys, payload), ...] as the left-deep plan the
    reference would run: R0 joins R1 on the key, the result joins R2, ...;
    output key, p0, ..., pm-1 (INT32)."""
    p = hj.Plan()
    for k, v in rels:
        p.new_input(hj.Table(k.size, [hj.Column.int32(k), hj.Column.int32(v)]))
    scans = [p.new_scan_node(j, [(0, hj.INT32), (1, hj.INT32)]) for j in range(len(rels))]
    cur, width = scans[0], 2
    for j in range(1, len(rels)):
        attrs = [(c, hj.INT32) for c in range(width)] + [(width + 1, hj.INT32)]
        cur = p.new_join_node(False, cur, scans[j], 0, 0, attrs)
        width += 1
    p.root = cur
    return p


def c4_cpu_sample(hj, w, gpu_rows, budget_s: float, n: int = 64) -> dict:
    """CPU baseline of c4: a seeded sample of n instances, each one run as its
    left-deep plan through the oracle's restatement of execute() with all host
    threads (relations from the oracle's generator, paged untimed), in sample
    order until the sample is done or budget_s of execute() time is spent.
    Each instance's row count is checked against the GPU's."""
    import numpy as np
    sys.path.insert(0, str(ROOT / "oracle"))
    import batch_oracle as bo
    oracle = oracle_mod()
    threads = os.cpu_count() or 1
    os.environ["SIGMOD_THREADS"] = str(threads)
    pick = np.random.default_rng(4096).choice(len(w), min(n, len(w)), replace=False)
    secs, done, probe, same = 0.0, 0, 0, True
    for i in pick:
        iid, m, b, q, pr = w.instance(int(i))
        plan = chain_plan(hj, bo.instance_relations(w.seed, iid, m, b, q, pr))
        st = oracle.timed_execute(plan)
        secs += st["seconds"]
        done += 1
        probe += pr
        same &= st["rows"] == int(gpu_rows[int(i)])
        if secs > budget_s:
            break
    return {"value": done / secs, "unit": "queries/s", "cores": threads, "kind": "port",
            "sample": f"{done} of a seeded {len(pick)}-instance sample ({probe} probe rows), each a left-deep plan "
                      f"through the restated execute() to finished result pages; {secs:.1f} s of execute()",
            "rows_equal_gpu": bool(same)}


def run_batch(args, d: Dist) -> dict:
    """c4: the batched form against the plain one-query-at-a-time path."""
    import numpy as np
    import torch
    from __graft_entry__ import load

    hj = load()
    from hjgb300 import batch, workloads
    torch.cuda.set_device(d.local)
    eng = hj.Engine(d.local)
    stream = torch.cuda.ExternalStream(eng.stream)
    w = workloads.c4(n=args.instances, scale=args.scale)

    def timer(fn):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        out = fn()
        b.record(stream)
        b.synchronize()
        return out, a.elapsed_time(b) / 1e3

    # options of both paths from the autotuner (sweeps a stratified sample)
    from hjgb300 import autotune
    tuned = autotune.tune(eng, w, torch=torch, cache=None if args.retune else autotune.DEFAULT_CACHE,
                          force=args.retune)
    autotune.apply(eng, tuned)
    # warm-up: whole passes (the memory pools grow to the largest wave here)
    for _ in range(args.warmup):
        batch.run(eng, w, hj.BATCH_PERSISTENT, args.wave_rows, torch, timer)
    npl = len(w) if args.plain_instances < 0 else min(len(w), args.plain_instances)
    wp = w.subset(np.arange(npl))
    batch.run(eng, wp, hj.BATCH_PLAIN, args.wave_rows, torch, timer)
    with Clocks(d.local) as clk:
        d.barrier()
        secs, redo = 0.0, 0
        for _ in range(args.steps):
            rows, sums, k, t = batch.run(eng, w, hj.BATCH_PERSISTENT, args.wave_rows, torch, timer)
            secs += t
            redo += k
        d.barrier()
    clocks = clk.summary()
    t_batch = d.max(secs / args.steps)
    # plain path: every instance (or a prefix) once, compared instance by instance
    prow, psum, _, t_plain = batch.run(eng, wp, hj.BATCH_PLAIN, args.wave_rows, torch, timer)
    t_plain = d.max(t_plain)
    same = bool(np.array_equal(prow, rows[:npl]) and np.array_equal(psum, sums[:npl]))
    eng.close()
    cpu = None
    if d.rank == 0 and not args.no_cpu_baseline:
        cpu = c4_cpu_sample(hj, w, rows, args.cpu_budget_s)
    q_batch = len(w) * d.world / t_batch
    q_plain = npl * d.world / t_plain
    probe_rows = int(w.probe_rows.sum())
    return {
        "metric": "batched queries/s", "value": q_batch, "unit": "queries/s", "n_gpus": d.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_batch * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (instances generated on the device per (seed, id), in waves; generation untimed)",
        "config": {"workload": f"c4: {len(w)} independent 2-4-way INT32 join chains, builds log-uniform "
                               f"{int(w.build_rows.min())}-{int(w.build_rows.max())} rows, probe 10x build",
                   "instances": len(w), "build_rows": int(w.build_rows.sum()), "probe_rows": probe_rows,
                   "waves": len(batch.waves(w, args.wave_rows)), "wave_rows": args.wave_rows,
                   "l2": "inputs larger than L2",
                   "tuned": {"batched": {k: v for k, v in tuned["batched"].items() if k != "seconds"},
                             "plain": {k: v for k, v in tuned["plain"].items() if k != "seconds"}}},
        "plain": {"value": q_plain, "unit": "queries/s", "instances": npl, "seconds": t_plain},
        "speedup_vs_plain": q_batch / q_plain, "results_equal_plain": same, "recomputed": redo,
        "probe_tuples_per_s": probe_rows / t_batch, "cpu_baseline": cpu, "clocks": clocks,
    }


def run_serve(args, d: Dist) -> dict:
    """c5: the request loop against the plain one-plan-at-a-time path."""
    import torch
    from __graft_entry__ import load

    hj = load()
    from hjgb300 import serve
    torch.cuda.set_device(d.local)
    eng = hj.Engine(d.local)
    mix = serve.c5_mix(eng, large_scale=args.scale)
    rates = [float(x) for x in args.rates.split(",")]
    budget = int(args.budget_gb * (1 << 30))
    # warm-up: every plan once on each path (pools grow, cached tables get built)
    for kind in serve.KINDS:
        for p in mix.plans[kind]:
            eng.free_result(eng.execute_raw(p))
    eng.set_option("table_cache", 1)
    for _ in range(max(1, args.warmup)):
        serve.run_served(eng, mix, serve.schedule(mix, rates[-1], 64, seed=99), budget, args.slots)
    lines, equal = [], True
    with Clocks(d.local) as clk:
        for r in rates:
            sched = serve.schedule(mix, r, args.requests, seed=int(r))
            eng.set_option("table_cache", 1)
            sv = serve.run_served(eng, mix, sched, budget, args.slots)
            eng.set_option("table_cache", 0)
            pl = serve.run_plain(eng, mix, sched)
            same = sv.pop("results") == pl.pop("results")
            equal &= same
            lines.append({"offered_qps": r, "served": sv, "plain": pl, "results_equal": same})
    clocks = clk.summary()
    mix.release(eng)
    eng.close()
    top = lines[-1]
    return {
        "metric": "served queries/s", "value": top["served"]["qps"], "unit": "queries/s", "n_gpus": d.world,
        "steps": len(rates), "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded generators; base tables resident and decoded in HBM)",
        "config": {"workload": "c5: open-loop Poisson stream, 70% small 2-way (build 10k-1M, probe 10x), "
                               "25% c3 at 1/10, 5% c2 (16M x 256M)",
                   "requests_per_rate": args.requests, "slots": args.slots, "hbm_budget_gb": args.budget_gb,
                   "large_scale": args.scale},
        "plain_qps_at_top_rate": top["plain"]["qps"], "speedup_vs_plain": top["served"]["qps"] / top["plain"]["qps"],
        "p99_ms_at_top_rate": top["served"]["p99_ms"], "results_equal_plain": equal, "rates": lines,
        "clocks": clocks,
    }


def run_reference(args, d: Dist):
    """The reference's CPU path (the oracle restatement of Contest::execute,
    all host threads) on the same workload and config as the GPU arm: one
    execute() per step, input pages built by the oracle's own writers, so the
    engine library is never loaded.  Rank 0 alone runs under torchrun."""
    if d.rank != 0:
        return None
    if args.workload in ("c4", "c5"):
        return {"impl": "reference", "unavailable": f"{args.workload} is compared against the plain GPU path; "
                                                      "the CPU reference arm covers c1, c2, c2raw and c3"}
    oracle = oracle_mod()
    from __graft_entry__ import load
    hj = load()  # Plan / Table types only; the page writers below are the oracle's
    hj.use_page_writer(oracle.page_writer)
    w = make_workload(hj, args.workload, args.scale)
    if w.name == "c2raw":  # the oracle takes pre-filtered tables, as the reference's execute() does
        w.plan = w.meta["prefiltered_plan"]
    sec, ptup, st, sample = cpu_reference_steps(w, oracle, args.steps, args.warmup, args.ref_budget_s)
    v = ptup / sec
    threads = os.cpu_count() or 1
    return {"impl": "reference", "metric": "probe tuples/s", "value": v, "unit": "probe tuples/s",
            "n_gpus": d.world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded generator with the configured shapes)",
            "config": workload_config(w, args, d.world, st["build_tuples"], st["probe_tuples"], st["rows"]),
            "cpu_baseline": {"value": v, "unit": "probe tuples/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "probe tuples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def systems_summary(args, d: Dist) -> dict:
    """The two systems forms at a reduced size, attached to the default c2 line
    (one GPU) so that a plain `python bench.py` records them too: the batched
    executor on the first 1,024 of the 4,096 c4 instances, and the serving loop
    at 1,000 and 5,000 offered queries/s (200 requests each), both against the
    plain one-query-at-a-time path on the same inputs.  `--workload c4|c5` runs
    the full configurations."""
    import copy
    a = copy.copy(args)
    a.instances, a.steps, a.warmup, a.scale = 1024, 3, 3, 1.0
    b = run_batch(a, d)
    a = copy.copy(args)
    a.rates, a.requests, a.warmup, a.scale = "1000,5000", 200, 3, 1.0
    v = run_serve(a, d)
    top = v["rates"][-1]
    return {
        "batched": {"metric": b["metric"], "value": b["value"], "unit": b["unit"],
                    "plain_value": b["plain"]["value"], "speedup_vs_plain": b["speedup_vs_plain"],
                    "results_equal_plain": b["results_equal_plain"], "workload": b["config"]["workload"],
                    "size": "1,024 of the 4,096 c4 instances", "steps": b["steps"]},
        "served": {"metric": v["metric"], "value": v["value"], "unit": v["unit"],
                   "offered_qps": top["offered_qps"], "plain_value": v["plain_qps_at_top_rate"],
                   "speedup_vs_plain": v["speedup_vs_plain"], "p50_ms": top["served"]["p50_ms"],
                   "p95_ms": top["served"]["p95_ms"], "p99_ms": top["served"]["p99_ms"],
                   "plain_p99_ms": top["plain"]["p99_ms"], "results_equal": v["results_equal_plain"],
                   "workload": v["config"]["workload"], "size": "200 requests per rate, rates 1,000 and 5,000 q/s"},
    }


def workloads_summary(args, d: Dist) -> dict:
    """The two other plain-path configurations at full size, attached to the
    default c2 line (one GPU) so that a plain `python bench.py` records them
    too: c1 (1M x 10M unique keys) and c3 (the 5-relation chain), each with
    device-resident inputs, 100 timed steps, its phase times, the probe
    roofline and (unless --no-cpu-baseline) the oracle's restatement of
    execute() on the same inputs with all host threads, at most 20 s each.
    `--workload c1|c3` runs either with every leg (e2e too)."""
    import copy
    out = {}
    for name in ("c1", "c3"):
        a = copy.copy(args)
        a.workload, a.scale, a.steps, a.warmup = name, 1.0, 100, 3
        a.no_e2e, a.cpu_budget_s = True, min(args.cpu_budget_s, 20.0)
        r = run_ours(a, d)
        out[name] = {"workload": r["config"]["workload"], "steps": r["steps"], "ms_per_step": r["ms_per_step"],
                     "probe_tuples_per_s": r["value"], "build_tuples_per_s": r["build_tuples_per_s"],
                     "output_rows": r["config"]["output_rows"], "phases_ms": r["phases_ms"],
                     "probe_roofline_frac": r["roofline"]["frac"], "probe_achieved_gbs": r["roofline"]["achieved"],
                     "algorithmic_bytes": r["roofline"]["algorithmic_bytes"], "gpu_launches": r["gpu_launches"],
                     "cpu_baseline": r["cpu_baseline"]}
    return out


def main():
    args = parse()
    d = Dist()
    if args.impl == "reference":
        line = run_reference(args, d)
    elif args.workload == "c4":
        line = run_batch(args, d)
    elif args.workload == "c5":
        line = run_serve(args, d)
    else:
        line = run_ours(args, d)
        if (line is not None and args.workload == "c2" and args.scale == 1.0 and d.world == 1
                and not args.no_workloads):
            line["workloads"] = workloads_summary(args, d)
        if (line is not None and args.workload == "c2" and args.scale == 1.0 and d.world == 1
                and not args.no_systems):
            line["systems"] = systems_summary(args, d)
    if d.rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    d.close()


if __name__ == "__main__":
    main()
