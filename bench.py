#!/usr/bin/env python
"""Benchmark of the GB300 stable LSD radix sort (one JSON line on stdout, rank 0).

Workload (one step): the mode/dtype sweep at 2^28 keys, one array each --
  * float32 N(0, 1e3) with 1% -0.0, 0.5% +-inf, 0.1% NaN, sorted descending with the
    absolute filter (rsbd8::radixsortcopy<dscfwdorder, nativeabs>);
  * int64 uniform over the full signed range, ascending;
  * uint32 with only the low 12 bits random (the pass-skip test drops two digits), ascending.
Synthetic seeded data of exactly those shapes (no dataset exists for this benchmark).

value      device-resident throughput: keys sorted per second over the K timed steps
           (inputs already in HBM, radixsortcopynoalloc with preallocated buffers; every input
           is larger than the 129 MB L2, so no flush is needed between steps);
e2e        the same sorts through the C ABI from pinned HOST buffers: each step copies the
           inputs host->device, sorts, and copies the sorted arrays back (one stream per array,
           so the copy engines move one array while another is sorted; the plain serial
           sequence is reported beside it);
roofline   the dominant kernel (the onesweep scatter pass on 64-bit keys): algorithmic bytes per
           launch (2 x 8 B x 2^28: read + write of one pass) / its average launch time, measured
           with CUDA events on the launch stream inside the timed region, against the measured
           HBM copy bandwidth;
cpu_baseline  the oracle's multithreaded C port of the reference's LSD sort on a bounded sample,
           on the host cores of the same machine.
`--impl reference` times that CPU implementation as the reference arm.
With --gpus N (launched under torchrun) every rank sorts its own copy of the workload
(replicas: the sort has no exchange step) and value is the sum over ranks.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from radixsortbidi8_gb300.synth import SWEEP_SEEDS as SEEDS  # noqa: E402
CLOCK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--log2n", type=int, default=28, help="keys per array (2^log2n)")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-configs", action="store_true",
                   help="skip the other benchmark configurations (2^20 plain sort, records, batches, serving)")
    p.add_argument("--case", default=None, choices=["u32", "i64", "f32abs", "u32low12", "f64ind", "u128", "x87",
                                                    "merge_u32", "merge_i64"],
                   help="profiling aid: sort only this one array --steps times and print its timings")
    p.add_argument("--config", default="sweep", choices=["sweep", "batched", "serving"],
                   help="sweep: the default line; batched: segmented batches vs a per-array loop; "
                        "serving: Poisson request stream through the serving loop")
    p.add_argument("--duration", type=float, default=10.0, help="serving: seconds of arrivals")
    p.add_argument("--rate", type=float, default=2000.0, help="serving: requests per second")
    p.add_argument("--batch-scale", type=float, default=1.0, help="batched: fraction of the segment counts")
    p.add_argument("--batches", default="A_2p28,A,B", help="batched: which batches to run (comma-separated)")
    p.add_argument("--calibrate-cpu", action="store_true",
                   help="where the reference was compiled (oracle/_ref): time its sort beside the oracle's port "
                        "on the same host cores and inputs, and print the ratio")
    return p.parse_args()


def workload_config(log2n: int) -> dict:
    return {"workload": f"mode/dtype sweep, 3 arrays x 2^{log2n} keys: float32 N(0,1e3)+specials "
                        f"dscfwdorder nativeabs; int64 uniform ascfwdorder; uint32 low-12-bit ascfwdorder",
            "keys_per_step": 3 * (1 << log2n), "api": "radixsortcopynoalloc (C ABI)",
            "l2": "inputs larger than L2 (>= 1 GiB per array), no flush",
            "parallelism": "replicas (no exchange step)"}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic():
    """dram bytes per launch of the dominant kernel from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "onesweep_u64_int64_2p28_traffic.txt")
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch_full_size:"):
                    return float(line.split(":", 1)[1])
    except Exception:
        pass
    return None


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons while the timed region runs."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={CLOCK_FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# ---- the workload ------------------------------------------------------------------------

def make_arrays(log2n: int, device):
    """Device-resident inputs of the sweep: (name, bits tensor, key dtype, direction, mode)."""
    from radixsortbidi8_gb300 import synth as S
    return S.sweep_arrays_torch(1 << log2n, device=device)


def active_passes(bits, name: str) -> int:
    """Digits the pass-skip test keeps: bytes of the filtered key that are not constant."""
    import torch
    x = bits
    if name.startswith("float32_abs"):
        x = x & 0x7FFFFFFF                      # the absolute filter drops the sign bit
    kb = x.element_size()
    cnt = 0
    for p in range(kb):
        d = (x >> (8 * p)) & 0xFF
        if int(d.min()) != int(d.max()):
            cnt += 1
    del torch
    return cnt


def max_over_ranks(x: float, world: int, device=None) -> float:
    """The largest per-step time over all ranks (every rank sorts its own replica of the workload)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_gkeys(keys_per_rank_step: int, world: int, ms_step: float) -> float:
    """Whole-job throughput: the keys all ranks sorted in one step over the slowest rank's step time."""
    return world * keys_per_rank_step / (ms_step * 1e-3) / 1e9


def gb300_arm(args, rank: int, world: int):
    import numpy as np
    import torch
    import radixsortbidi8_gb300 as rs

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    rs.lib()
    n = 1 << args.log2n
    arrays = make_arrays(args.log2n, dev)
    stream = torch.cuda.Stream(device=dev)
    bufs = []
    for name, bits, kdt, d, m in arrays:
        nb = rs.scratch_bytes(kdt, n, d, m)
        bufs.append((torch.empty_like(bits), torch.empty_like(bits),
                     torch.empty(nb, dtype=torch.uint8, device=dev)))
    act = [active_passes(b, nm) for nm, b, *_ in arrays]
    torch.cuda.synchronize()

    def step():
        for (name, bits, kdt, d, m), (out, buf, scr) in zip(arrays, bufs):
            rs.radixsortcopynoalloc(bits, out, buf, scr, d, m, key_dtype=kdt, stream=stream)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    torch.cuda.synchronize()
    for (out, buf, scr) in bufs:
        assert rs.scratch_status(scr, stream) == 0

    clocks = ClockSampler(dev.index)
    clocks.start()
    time.sleep(0.3)
    barrier()
    torch.cuda.synchronize()
    rs.api.profile_enable(True)
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(args.steps):
        step()
    t1.record(stream)
    torch.cuda.synchronize()
    rs.api.profile_enable(False)
    barrier()
    clk = clocks.stop()
    ms_total = t0.elapsed_time(t1)
    recs = rs.api.profile_collect()
    for (out, buf, scr) in bufs:
        assert rs.scratch_status(scr, stream) == 0

    # end to end first: large host-side work (the oracle's arrays) makes the next host<->device
    # copies of pinned buffers slow for a while (measured: 12-25 GB/s against 190-210 GB/s)
    e2e = None if args.no_e2e else e2e_arm(args, rs, arrays, stream)
    # the serving run next, for the same reason: its tail latency suffers from host-side work
    serving = None
    if rank == 0 and world == 1 and not args.no_configs:
        serving = serving_run(args, 2000.0, 5.0, 2000, 0 if args.no_cpu else 32)
        # near the server's capacity (about 36 GKeys/s offered): requests queue, and the waiting
        # ones are coalesced into shared launches
        serving["near_capacity"] = serving_run(args, 6000.0, 2.0, 0, 0 if args.no_cpu else 8)
    # correctness of the timed outputs: byte comparison with the oracle, outside the timed region
    check = "not checked (--no-cpu)" if args.no_cpu else verify_outputs(arrays, bufs)

    ms_step = max_over_ranks(ms_total / args.steps, world, dev)
    keys_step = 3 * n
    value = whole_job_gkeys(keys_step, world, ms_step)

    peak, peak_kind = measured_peak()
    # per-sort and per-kernel breakdown from the launch records (launch order is fixed per step)
    per_sort = {nm: {"ms": 0.0, "sweep_ms": [], "launches": 0} for nm, *_ in arrays}
    ours = [r for r in recs if r["kernel"] != "memset"]
    # every sort's launches start with its memset; the sorts of a step run in the arrays' order
    names = [nm for nm, *_ in arrays]
    sort_i = -1
    for r in recs:
        if r["kernel"] == "memset":
            sort_i += 1
        nm = names[max(sort_i, 0) % len(names)]
        per_sort[nm]["ms"] += r["ms"]
        if r["kernel"] != "memset":
            per_sort[nm]["launches"] += 1
        if r["kernel"] == "onesweep":
            per_sort[nm]["sweep_ms"].append((r["pass_"], r["ms"]))
    per_dtype = {}
    for (nm, bits, kdt, d, m), a in zip(arrays, act):
        kb = bits.element_size()
        t = per_sort[nm]["ms"] / args.steps
        algo = a * 2 * kb * n
        per_dtype[nm] = {"gkeys_s": round(n / (t * 1e-3) / 1e9, 3), "ms": round(t, 4), "active_passes": a,
                         "algorithmic_bytes": algo,
                         "roofline_frac": round(algo / (t * 1e-3) / 1e9 / peak, 4)}
    # dominant kernel: onesweep on the 64-bit keys (every pass active)
    sw = [ms for p, ms in per_sort["int64_ascfwdorder"]["sweep_ms"]]
    avg_ms = sum(sw) / len(sw)
    bytes_launch = 2 * 8 * n
    achieved = bytes_launch / (avg_ms * 1e-3) / 1e9
    share = {k: 0.0 for k in ("memset", "histogram", "plan", "onesweep", "copy")}
    for r in recs:
        share[r["kernel"]] = share.get(r["kernel"], 0.0) + r["ms"]
    tot = sum(share.values())
    roofline = {"bound": "hbm", "kernel": "k_onesweep_pipe<uint64, 512 x 16> (int64 sort, 8 active passes)",
                "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": f"of {peak_kind}",
                "traffic": profiled_traffic(), "bytes_per_launch": bytes_launch,
                "avg_launch_ms": round(avg_ms, 4),
                "time_share": {k: round(v / tot, 4) for k, v in share.items() if tot}}

    extra = uniform_u32(args, rs, dev, stream, peak)
    f32_rev = float32_abs_reverse(args, rs, arrays, stream)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(arrays, min(args.log2n, 24))
    # the other benchmark configurations, each timed on its own and checked against the oracle
    configs = None
    if rank == 0 and world == 1 and not args.no_configs:
        del bufs
        torch.cuda.empty_cache()
        do_check = not args.no_cpu
        configs = {"1_plain_u32_2p20": config1_small(args, rs, dev, stream),
                   "3_records_2p26": config3_records(args, rs, dev, stream, peak),
                   "4_batched": {w: batched_run(args, w, max(3, min(args.steps, 10)), do_check)
                                 for w in ("A_2p28", "B")},
                   "5_serving": serving}
    line = {
        "metric": "GKeys/s", "value": round(value, 3), "unit": "GKeys/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/i64/u32 keys (integer ops)",
        "data": "synthetic (seeded splitmix64; shapes and distributions of the benchmark configuration)",
        "config": workload_config(args.log2n),
        "roofline": roofline, "per_dtype": per_dtype, "uint32_uniform_2p28": extra,
        "float32_abs_dscrevorder_2p28": f32_rev,
        "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
        "gpu_launches": len(ours), "checked": check, "configs": configs,
    }
    return line


def verify_outputs(arrays, bufs) -> str:
    """Verification of the timed outputs: each one copied to the host and compared byte for
    byte with the oracle's sort (the C restatement, all host threads) of the host copy of its input.
    Runs after the timed region."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    for (nm, bits, kdt, d, m), (out, buf, scr) in zip(arrays, bufs):
        a = bits.cpu().numpy().view(kdt)
        got = out.cpu().numpy().view(kdt)
        want = O.sortcopy(a, m, d, threads=threads)
        if not np_bytes_equal(got, want):
            return f"FAILED {nm}: differs from the oracle"
    return "bit-exact vs oracle"


def np_bytes_equal(a, b) -> bool:
    import numpy as np
    return a.shape == b.shape and bool(np.array_equal(a.view(np.uint8), b.view(np.uint8)))


def uniform_u32(args, rs, dev, stream, peak) -> dict:
    """2^28 uniform uint32 keys (4 active passes): the 70%-of-roofline target, measured alone."""
    import numpy as np
    import torch
    from radixsortbidi8_gb300 import synth as S
    n = 1 << args.log2n
    bits = S.uniform_bits_torch(SEEDS["u32"], n, 4, device=dev)
    out, buf = torch.empty_like(bits), torch.empty_like(bits)
    scr = torch.empty(rs.scratch_bytes(np.uint32, n), dtype=torch.uint8, device=dev)
    # the input was made, and these arrays allocated, on the default stream; the sorts run on `stream`
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for _ in range(max(3, args.warmup)):
            rs.radixsortcopynoalloc(bits, out, buf, scr, key_dtype=np.uint32, stream=stream)
    torch.cuda.synchronize()
    rs.api.profile_enable(True)
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(args.steps):
        rs.radixsortcopynoalloc(bits, out, buf, scr, key_dtype=np.uint32, stream=stream)
    t1.record(stream)
    torch.cuda.synchronize()
    rs.api.profile_enable(False)
    recs = rs.api.profile_collect()
    ms = t0.elapsed_time(t1) / args.steps
    sw = [r["ms"] for r in recs if r["kernel"] == "onesweep"]
    hist = [r["ms"] for r in recs if r["kernel"] == "histogram"]
    algo = 4 * 2 * 4 * n
    k = out.to(torch.int64) & 0xFFFFFFFF
    ok = bool((k[:-1] <= k[1:]).all())
    del bits, out, buf, scr
    return {"gkeys_s": round(n / (ms * 1e-3) / 1e9, 3), "ms": round(ms, 4),
            "roofline_frac": round(algo / (ms * 1e-3) / 1e9 / peak, 4),
            "onesweep_avg_ms": round(sum(sw) / len(sw), 4),
            "onesweep_GBps": round(2 * 4 * n / (sum(sw) / len(sw) * 1e-3) / 1e9, 1),
            "histogram_ms": round(sum(hist) / len(hist), 4), "sorted": ok}


def float32_abs_reverse(args, rs, arrays, stream) -> dict:
    """The float32 array of the sweep sorted dscrevorder (descending by absolute value, ties in
    reverse input order: the first surviving pass reads back to front), timed alone."""
    import numpy as np
    import torch
    bits = arrays[0][1]
    n = bits.numel()
    out, buf = torch.empty_like(bits), torch.empty_like(bits)
    scr = torch.empty(rs.scratch_bytes(np.float32, n, "dscrevorder", "nativeabs"), dtype=torch.uint8,
                      device=bits.device)
    run = lambda: rs.radixsortcopynoalloc(bits, out, buf, scr, "dscrevorder", "nativeabs", key_dtype=np.float32,
                                          stream=stream)
    torch.cuda.synchronize()                  # allocated on the default stream, used on `stream`
    for _ in range(max(3, args.warmup)):
        run()
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(args.steps):
        run()
    t1.record(stream)
    torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / args.steps
    k = out.to(torch.int64) & 0x7FFFFFFF          # |x| bits: the key of the absolute float modes
    ok = bool((k[:-1] >= k[1:]).all())
    del out, buf, scr
    return {"gkeys_s": round(n / (ms * 1e-3) / 1e9, 3), "ms": round(ms, 4), "sorted": ok}


E2E_SLOTS = 2   # buffer sets of the end-to-end pipeline (three measured slower: 26.8 against 29.7 GKeys/s)


def e2e_arm(args, rs, arrays, stream) -> dict:
    """Host buffers in, host buffers out, through the C ABI: every step copies each array's keys
    from pinned host memory, sorts them (radixsortcopynoalloc) and copies the result back.

    Pipelined (the headline): one stream per stage -- host-to-device copies, sorts, device-to-host
    copies -- ordered by events per array, with E2E_SLOTS sets of device buffers used in turn by the steps,
    so the copy engines move one array while the SMs sort another.  The NVLink-C2C link to the host
    (about 0.2 TB/s each way, 0.34 TB/s both ways at once) bounds this path.  Serial: the same calls
    one after another on one stream."""
    import torch
    steps = max(1, min(args.steps, 10))
    dev = arrays[0][1].device
    host_in = [b.cpu().pin_memory() for _, b, *_ in arrays]
    n = arrays[0][1].numel()
    h2d = sum(h.numel() * h.element_size() for h in host_in)
    slots = []
    for _ in range(E2E_SLOTS):
        slots.append({
            "in": [torch.empty_like(b) for _, b, *_ in arrays],
            "out": [torch.empty_like(b) for _, b, *_ in arrays],
            "buf": [torch.empty_like(b) for _, b, *_ in arrays],
            "scr": [torch.empty(rs.scratch_bytes(kdt, n, d, m), dtype=torch.uint8, device=dev)
                    for _, b, kdt, d, m in arrays],
            "host_out": [torch.empty_like(h).pin_memory() for h in host_in],
        })
    torch.cuda.synchronize()                  # the buffers are used on the stage streams below
    # pipeline: one stream per stage; events order each array's H2D -> sort -> D2H and keep a
    # buffer set from being refilled before the step two back has finished with it
    s_h2d, s_sort, s_d2h = (torch.cuda.Stream(device=dev) for _ in range(3))
    ev = {key: [[None] * len(arrays) for _ in range(E2E_SLOTS)] for key in ("h2d", "sort", "d2h")}

    def record(key, slot_i, i, st):
        e = torch.cuda.Event()
        e.record(st)
        ev[key][slot_i][i] = e

    def one(k: int, serial: bool):
        slot_i = k % E2E_SLOTS
        slot = slots[slot_i]
        for i, (nm, b, kdt, d, m) in enumerate(arrays):
            if serial:
                with torch.cuda.stream(stream):
                    slot["in"][i].copy_(host_in[i], non_blocking=True)
                    rs.radixsortcopynoalloc(slot["in"][i], slot["out"][i], slot["buf"][i], slot["scr"][i], d, m,
                                            key_dtype=kdt, stream=stream)
                    slot["host_out"][i].copy_(slot["out"][i], non_blocking=True)
                continue
            if ev["sort"][slot_i][i] is not None:
                s_h2d.wait_event(ev["sort"][slot_i][i])       # the sort two steps back read this input
            with torch.cuda.stream(s_h2d):
                slot["in"][i].copy_(host_in[i], non_blocking=True)
            record("h2d", slot_i, i, s_h2d)
            s_sort.wait_event(ev["h2d"][slot_i][i])
            if ev["d2h"][slot_i][i] is not None:
                s_sort.wait_event(ev["d2h"][slot_i][i])       # its output was copied out
            rs.radixsortcopynoalloc(slot["in"][i], slot["out"][i], slot["buf"][i], slot["scr"][i], d, m,
                                    key_dtype=kdt, stream=s_sort)
            record("sort", slot_i, i, s_sort)
            s_d2h.wait_event(ev["sort"][slot_i][i])
            with torch.cuda.stream(s_d2h):
                slot["host_out"][i].copy_(slot["out"][i], non_blocking=True)
            record("d2h", slot_i, i, s_d2h)

    def timed(pipelined: bool) -> float:
        one(0, not pipelined)
        torch.cuda.synchronize()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for st in (s_h2d, s_sort, s_d2h):
            st.wait_stream(stream)
        for k in range(steps):
            one(k, not pipelined)
        for st in (s_h2d, s_sort, s_d2h):
            stream.wait_stream(st)
        t1.record(stream)
        torch.cuda.synchronize()
        return t0.elapsed_time(t1) / steps

    ms_serial = timed(False)

    def stages() -> dict:
        """One serial step with CUDA events between its stages: where an end-to-end step spends its time."""
        slot = slots[0]
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3 * len(arrays) + 1)]
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            ev[0].record(stream)
            for i, (nm, b, kdt, d, m) in enumerate(arrays):
                slot["in"][i].copy_(host_in[i], non_blocking=True)
                ev[3 * i + 1].record(stream)
                rs.radixsortcopynoalloc(slot["in"][i], slot["out"][i], slot["buf"][i], slot["scr"][i], d, m,
                                        key_dtype=kdt, stream=stream)
                ev[3 * i + 2].record(stream)
                slot["host_out"][i].copy_(slot["out"][i], non_blocking=True)
                ev[3 * i + 3].record(stream)
        torch.cuda.synchronize()
        out = {}
        for i, (nm, *_) in enumerate(arrays):
            out[nm] = {"h2d_ms": round(ev[3 * i].elapsed_time(ev[3 * i + 1]), 3),
                       "sort_ms": round(ev[3 * i + 1].elapsed_time(ev[3 * i + 2]), 3),
                       "d2h_ms": round(ev[3 * i + 2].elapsed_time(ev[3 * i + 3]), 3)}
        return out

    stage_ms = stages()
    # the host link is shared with the machine's other GPUs: three pipelined runs, the median kept
    runs = sorted(timed(True) for _ in range(3))
    ms = runs[1]

    def copy_gbps(h2d_on: bool, d2h_on: bool) -> float:
        """Copy-engine bandwidth alone (same buffers, one stream per direction), GB/s."""
        sa, sb = torch.cuda.Stream(device=dev), torch.cuda.Stream(device=dev)
        torch.cuda.synchronize()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        sa.wait_stream(stream)
        sb.wait_stream(stream)
        for i in range(len(arrays)):
            if h2d_on:
                with torch.cuda.stream(sa):
                    slots[0]["in"][i].copy_(host_in[i], non_blocking=True)
            if d2h_on:
                with torch.cuda.stream(sb):
                    slots[1]["host_out"][i].copy_(slots[1]["out"][i], non_blocking=True)
        stream.wait_stream(sa)
        stream.wait_stream(sb)
        t1.record(stream)
        torch.cuda.synchronize()
        return round((h2d * (int(h2d_on) + int(d2h_on))) / (t0.elapsed_time(t1) * 1e-3) / 1e9, 1)

    copies = {"h2d_alone_GBps": copy_gbps(True, False), "d2h_alone_GBps": copy_gbps(False, True),
              "both_directions_GBps": copy_gbps(True, True)}
    last = slots[(steps - 1) % E2E_SLOTS]
    same = all(torch.equal(last["host_out"][i], last["out"][i].cpu()) for i in range(len(arrays)))
    return {"value": round(3 * n / (ms * 1e-3) / 1e9, 3), "unit": "GKeys/s", "ms_per_step": round(ms, 3),
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d, "steps": steps,
            "path": "pinned host -> cudaMemcpyAsync -> radixsortcopynoalloc -> cudaMemcpyAsync -> pinned host; "
                    f"one stream per stage (H2D, sort, D2H) ordered by events, {E2E_SLOTS} buffer sets used in turn by the "
                    "steps, so the copy engines move one array while another is sorted",
            "serial": {"value": round(3 * n / (ms_serial * 1e-3) / 1e9, 3), "ms_per_step": round(ms_serial, 3),
                       "path": "the same calls in order on one stream"},
            "runs_ms_per_step": [round(r, 3) for r in runs], "host_results_match_device": bool(same),
            "serial_stage_ms": stage_ms,
            "copy_bandwidth": copies}


def cpu_sample_arrays(log2n_sample: int):
    """Host copies of the first 2^k keys of each array (numpy, same generators, filled in parallel)."""
    import numpy as np
    from radixsortbidi8_gb300 import synth as S
    n = 1 << log2n_sample
    return [
        (S.host_parallel(S.float_specials, n, np.float32, SEEDS["f32"], dtype=np.float32), "nativeabs", "dscfwdorder"),
        (S.host_parallel(S.uniform_bits, n, np.int64, SEEDS["i64"], dtype=np.int64), "native", "ascfwdorder"),
        (S.host_parallel(S.low_bits_u32, n, np.uint32, SEEDS["u32low12"]), "native", "ascfwdorder"),
    ]


# the port against the reference's own rsbd8::radixsortcopy on the same cores and inputs (8 x86-64
# cores, `bench.py --calibrate-cpu`; the float32 absolute-value array by its native-float stand-in)
PORT_VS_REFERENCE = "the port sorts this mix about 1.2x faster than the reference's own code (1.25x at 2^24, 1.18x at 2^26)"


def cpu_baseline(arrays, log2n_sample: int, reps: int = 3) -> dict:
    """The oracle's multithreaded C port of the reference LSD sort on a bounded sample."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    samples = cpu_sample_arrays(log2n_sample)
    best = float("inf")
    for _ in range(reps):
        t = time.perf_counter()
        for a, m, d in samples:
            O.sortcopy(a, m, d, threads=threads)
        best = min(best, time.perf_counter() - t)
    keys = sum(a.size for a, *_ in samples)
    return {"value": round(keys / best / 1e9, 4), "unit": "GKeys/s", "cores": threads, "kind": "port",
            "sample": f"first 2^{log2n_sample} keys of each of the 3 arrays (same generators), best of {reps}",
            "port_vs_reference": PORT_VS_REFERENCE}


REFERENCE_ARM_BUDGET_S = 150.0   # the reference arm's timed sorts stay within this on the host


def reference_arm(args, rank: int, world: int) -> dict | None:
    """The reference's algorithm (the oracle's multithreaded C port) on the host cores, on the GPU
    arm's own arrays (3 x 2^log2n keys) when steps + warm-up at that size fit REFERENCE_ARM_BUDGET_S
    (one sort of each array, timed first, decides), else on the first 2^24 keys of each array."""
    if rank != 0:
        return None
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    k = args.log2n
    samples = cpu_sample_arrays(k)
    t = time.perf_counter()
    for a, m, d in samples:
        O.sortcopy(a, m, d, threads=threads)
    one = time.perf_counter() - t
    if k > 24 and one * (args.steps + args.warmup) > REFERENCE_ARM_BUDGET_S:
        k = 24
        samples = cpu_sample_arrays(k)
    for _ in range(max(0, args.warmup - 1)):
        for a, m, d in samples:
            O.sortcopy(a, m, d, threads=threads)
    t = time.perf_counter()
    for _ in range(args.steps):
        for a, m, d in samples:
            O.sortcopy(a, m, d, threads=threads)
    el = time.perf_counter() - t
    keys = args.steps * sum(a.size for a, *_ in samples)
    v = keys / el / 1e9
    return {"metric": "GKeys/s", "value": round(v, 4), "unit": "GKeys/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(el / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32/i64/u32 keys (integer ops)",
            "data": "synthetic (seeded splitmix64)", "config": workload_config(args.log2n), "impl": "reference",
            "cpu_baseline": {"value": round(v, 4), "unit": "GKeys/s", "cores": threads, "kind": "port",
                             "sample": (f"each step sorts the 3 arrays of 2^{k} keys the GPU arm sorts" if k == args.log2n
                                        else f"each step sorts the first 2^{k} keys of each of the 3 arrays (the GPU "
                                             f"arm sorts 2^{args.log2n})"), "port_vs_reference": PORT_VS_REFERENCE},
            "e2e": {"value": round(v, 4), "unit": "GKeys/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference's CPU algorithm as the oracle's multithreaded C port (the reference's own "
                    "compiled code does not travel to this host)"}


def calibrate_cpu(args) -> dict:
    """The CPU baseline's calibration: the oracle's C port of the reference's LSD sort (what bench
    times as the reference arm where the reference's own code cannot run) against the reference's own
    rsbd8::radixsortcopy compiled from its header (oracle/_ref), on the same inputs and host cores.
    float32 by absolute value has no reference timing (the reference's absolute modes write out of
    bounds at this snapshot); the native-float descending sort of the same array stands in."""
    import numpy as np
    from oracle import oracle as O
    from radixsortbidi8_gb300 import synth as S
    if not O.ref_available():
        return {"calibrate_cpu": "unavailable: oracle/_ref (the reference compiled from its header) is not built here"}
    threads = os.cpu_count() or 1

    def best(fn, reps=3):
        t = float("inf")
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            t = min(t, time.perf_counter() - t0)
        return t

    rows = {}
    for k in (24, 26):
        n = 1 << k
        cases = [("uint32_uniform", S.uniform_bits(SEEDS["u32"], n, np.uint32), "native", "ascfwdorder", True),
                 ("uint32_low12", S.low_bits_u32(SEEDS["u32low12"], n), "native", "ascfwdorder", True),
                 ("int64_uniform", S.uniform_bits(SEEDS["i64"], n, np.int64), "native", "ascfwdorder", True),
                 ("float32_native_dscfwdorder", S.float_specials(SEEDS["f32"], n, np.float32), "native", "dscfwdorder", True),
                 ("float32_abs_dscfwdorder", S.float_specials(SEEDS["f32"], n, np.float32), "nativeabs", "dscfwdorder", False)]
        for name, a, m, d, ref_ok in cases:
            O.sortcopy(a, m, d, threads=threads)                     # warm
            tp = best(lambda: O.sortcopy(a, m, d, threads=threads))
            row = {"port_gkeys_s": round(n / tp / 1e9, 4)}
            if ref_ok:
                O.ref_sortcopy(a, m, d)
                tr = best(lambda: O.ref_sortcopy(a, m, d))
                row["reference_gkeys_s"] = round(n / tr / 1e9, 4)
                row["port_over_reference"] = round(tr / tp, 3)
            rows[f"{name}_2p{k}"] = row
    return {"calibrate_cpu": rows, "threads": threads, "host": os.uname().machine,
            "note": "best of 3 after a warm-up; the reference with its default thread count "
                    "(std::thread::hardware_concurrency), the port with the same number of threads"}


def single_case(args) -> dict:
    """One workload alone (for ncu captures of a small case): uniform uint32, int64, the float32
    absolute descending array, the low-12-bit uint32 array, the 24-byte record indirection, or
    16-byte keys (128-bit integers ascending, x87 extended precision descending)."""
    import numpy as np
    import torch
    import radixsortbidi8_gb300 as rs
    from radixsortbidi8_gb300 import synth as S
    dev = torch.device("cuda", 0)
    n = 1 << args.log2n
    stream = torch.cuda.current_stream()
    if args.case in ("merge_u32", "merge_i64"):
        # the two halves of a uniform array, each sorted, merged into one (the reference's mergehalves*)
        kb = 4 if args.case == "merge_u32" else 8
        kdt = np.uint32 if kb == 4 else np.int64
        bits = S.uniform_bits_torch(SEEDS["u32"] if kb == 4 else SEEDS["i64"], n, kb, device=dev)
        runs = torch.empty_like(bits)
        h = rs.api.halves(n)
        rs.radixsortcopy(bits[:h[0]], runs[:h[0]], key_dtype=kdt)
        rs.radixsortcopy(bits[h[0]:], runs[h[0]:], key_dtype=kdt)
        out = torch.empty_like(bits)
        run = lambda: rs.api.merge_runs(runs, out, h, key_dtype=kdt, stream=stream)
    elif args.case == "f64ind":
        rec = torch.empty(n * 24, dtype=torch.uint8, device=dev)
        keys = S.float_specials_torch(SEEDS["f32"], n, 8, device=dev)
        rec.view(torch.int64).view(n, 3)[:, 1] = keys
        ptrs = torch.arange(n, dtype=torch.int64, device=dev) * 24 + rec.data_ptr()
        out = torch.empty_like(ptrs)
        run = lambda: rs.radixsortcopy_member(ptrs, out, np.float64, 8)
    else:
        kb, kdt, d, m, gen = {"u32": (4, np.uint32, "ascfwdorder", "native", lambda: S.uniform_bits_torch(SEEDS["u32"], n, 4, device=dev)),
                              "i64": (8, np.int64, "ascfwdorder", "native", lambda: S.uniform_bits_torch(SEEDS["i64"], n, 8, device=dev)),
                              "f32abs": (4, np.float32, "dscfwdorder", "nativeabs", lambda: S.float_specials_torch(SEEDS["f32"], n, 4, device=dev)),
                              "u32low12": (4, np.uint32, "ascfwdorder", "native", lambda: S.low_bits_u32_torch(SEEDS["u32low12"], n, device=dev)),
                              # 16-byte keys: n keys of two uniform 64-bit words each
                              "u128": (16, "u128", "ascfwdorder", "native", lambda: S.uniform_bits_torch(SEEDS["i64"], 2 * n, 8, device=dev)),
                              "x87": (16, "x87", "dscfwdorder", "native", lambda: S.uniform_bits_torch(SEEDS["f32"], 2 * n, 8, device=dev))}[args.case]
        bits = gen()
        out, buf = torch.empty_like(bits), torch.empty_like(bits)
        scr = torch.empty(rs.scratch_bytes(kdt, n, d, m), dtype=torch.uint8, device=dev)
        run = lambda: rs.radixsortcopynoalloc(bits, out, buf, scr, d, m, key_dtype=kdt, stream=stream)
    for _ in range(args.warmup):
        run()
    torch.cuda.synchronize()
    rs.api.profile_enable(True)
    for _ in range(args.steps):
        run()
    torch.cuda.synchronize()
    rs.api.profile_enable(False)
    recs = rs.api.profile_collect()
    agg, by_pass = {}, {}
    for r in recs:
        agg.setdefault(r["kernel"], []).append(r["ms"])
        if r["kernel"] == "onesweep":
            by_pass.setdefault(r["pass_"], []).append(r["ms"])
    res = {}
    if args.case.startswith("merge"):
        ms = sum(r["ms"] for r in recs) / args.steps
        byts = 2 * n * (4 if args.case == "merge_u32" else 8)
        res = {"merge_GBps": round(byts / (ms * 1e-3) / 1e9, 1)}
    return {"case": args.case, "n": n, "steps": args.steps, **res,
            "ms_per_sort": round(sum(r["ms"] for r in recs) / args.steps, 4),
            "kernels": {k: {"launches": len(v), "avg_ms": round(sum(v) / len(v), 4)} for k, v in agg.items()},
            "onesweep_ms_by_pass": {p: round(sum(v) / len(v), 4) for p, v in sorted(by_pass.items())}}


def oracle_threads() -> int:
    return os.cpu_count() or 1


def config1_small(args, rs, dev, stream) -> dict:
    """2^20 uniform uint32 keys (seed 0x5EED0001), ascending, radixsortcopynoalloc: each sort timed alone
    with CUDA events after the L2 was flushed (the array fits in L2); checked against the oracle."""
    import numpy as np
    import torch
    from radixsortbidi8_gb300 import synth as S
    n = 1 << 20
    a = S.uniform_bits(0x5EED0001, n, np.uint32)
    bits = torch.from_numpy(a.view(np.int32).copy()).to(dev)
    out, buf = torch.empty_like(bits), torch.empty_like(bits)
    scr = torch.empty(rs.scratch_bytes(np.uint32, n), dtype=torch.uint8, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()                  # made on the default stream, used on `stream`
    times = []
    with torch.cuda.stream(stream):
        for i in range(max(3, args.warmup) + max(10, args.steps)):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            rs.radixsortcopynoalloc(bits, out, buf, scr, key_dtype=np.uint32, stream=stream)
            e1.record(stream)
            e1.synchronize()
            if i >= max(3, args.warmup):
                times.append(e0.elapsed_time(e1))
    ms = statistics.median(times)
    from oracle import oracle as O          # verifies the results, outside the timed region
    want = O.sortcopy(a, threads=oracle_threads())
    ok = np_bytes_equal(out.cpu().numpy().view(np.uint32), want)
    # the same sort captured once as a CUDA graph and replayed (the launch sequence has no host
    # synchronisation, so a latency-sensitive caller can issue it as one graph launch)
    out.zero_()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        with torch.cuda.graph(g, stream=stream):
            rs.radixsortcopynoalloc(bits, out, buf, scr, key_dtype=np.uint32, stream=stream)
    gtimes = []
    with torch.cuda.stream(stream):
        for i in range(max(3, args.warmup) + max(10, args.steps)):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            g.replay()
            e1.record(stream)
            e1.synchronize()
            if i >= max(3, args.warmup):
                gtimes.append(e0.elapsed_time(e1))
    gms = statistics.median(gtimes)
    gok = np_bytes_equal(out.cpu().numpy().view(np.uint32), want)
    del flush, g
    return {"keys": n, "ms": round(ms, 4), "gkeys_s": round(n / (ms * 1e-3) / 1e9, 3),
            "timing": "median of single sorts, L2 flushed before each (256 MiB write)",
            "graph_replay": {"ms": round(gms, 4), "gkeys_s": round(n / (gms * 1e-3) / 1e9, 3),
                             "checked": "bit-exact vs oracle" if gok else "FAILED vs oracle"},
            "checked": "bit-exact vs oracle" if ok else "FAILED vs oracle"}


def config3_records(args, rs, dev, stream, peak) -> dict:
    """2^26 records of 24 bytes {u64 id, f64 key, u32 tag, pad}, key lognormal(0, 2) x random sign with
    10% duplicated keys; the pointer array sorted by the key at byte 8, ascending
    (radixsortcopynoalloc, member indirection); exact pointer order checked against the oracle."""
    import numpy as np
    import torch
    from radixsortbidi8_gb300 import api, synth as S
    n = 1 << 26
    rec = S.records24_torch(S.RECORDS_SEED, n, device=dev)
    base = rec.data_ptr()
    ptrs = torch.arange(n, dtype=torch.int64, device=dev) * 24 + base
    out, buf = torch.empty_like(ptrs), torch.empty_like(ptrs)
    scr = torch.empty(rs.scratch_bytes(np.float64, n, indirection=api.MEMBER, offset1=8), dtype=torch.uint8,
                      device=dev)
    run = lambda: rs.radixsortcopynoalloc_member(ptrs, out, buf, scr, np.float64, 8, stream=stream)
    torch.cuda.synchronize()                  # records and pointers made on the default stream
    with torch.cuda.stream(stream):
        for _ in range(max(3, args.warmup)):
            run()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            run()
        e1.record(stream)
    torch.cuda.synchronize()
    assert rs.scratch_status(scr, stream) == 0
    ms = e0.elapsed_time(e1) / args.steps
    algo = 8 * 2 * 16 * n                     # 8 digit passes x read + write of key and pointer
    got = (out.cpu().numpy() - base) // 24
    rec_h = np.ascontiguousarray(rec.cpu().numpy())
    del rec, ptrs, out, buf, scr
    torch.cuda.empty_cache()
    from oracle import oracle as O          # verifies the results, outside the timed region
    hb = rec_h.ctypes.data
    hp = np.uint64(hb) + np.arange(n, dtype=np.uint64) * np.uint64(24)
    want = (O.sortcopy_indirect(hp, np.float64, 8, "native", "ascfwdorder", threads=oracle_threads())
            - np.uint64(hb)) // np.uint64(24)
    ok = bool(np.array_equal(got, want.astype(np.int64)))
    return {"keys": n, "ms": round(ms, 4), "gkeys_s": round(n / (ms * 1e-3) / 1e9, 3),
            "algorithmic_bytes": algo, "roofline_frac": round(algo / (ms * 1e-3) / 1e9 / peak, 4),
            "checked": "bit-exact pointer order vs oracle" if ok else "FAILED vs oracle"}


def batched_run(args, which: str, steps: int, check: bool) -> dict:
    """One batch of the batched configuration: one captured CUDA graph of the segmented sort, replayed
    `steps` times, against the per-array loop of plain noalloc sorts on the same GPU; every segment
    compared with the oracle (check) and the loop's output with the batched output."""
    import numpy as np
    import torch
    from radixsortbidi8_gb300 import batched as B, synth as S
    dev = torch.device("cuda", torch.cuda.current_device())
    lens = S.batch_lengths(which, args.batch_scale)
    offs = np.zeros(lens.size + 1, dtype=np.int64)
    np.cumsum(lens, out=offs[1:])
    total = int(offs[-1])
    kdt = np.uint32 if which.startswith("A") else np.float64
    keys = S.batch_keys_torch(which, total, device=dev)
    off_t = torch.from_numpy(offs).to(dev)
    torch.cuda.synchronize()
    sorter = B.SegmentedSorter(keys, off_t, key_dtype=kdt).capture()
    for _ in range(max(1, args.warmup)):
        sorter.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(sorter.stream)
    for _ in range(steps):
        sorter.replay()
    e1.record(sorter.stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    assert sorter.status() == 0
    loop_out = torch.empty_like(keys)
    ls = torch.cuda.Stream(device=dev)
    B.sort_each(keys, loop_out, offs, key_dtype=kdt, stream=ls)      # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    B.sort_each(keys, loop_out, offs, key_dtype=kdt, stream=ls)
    torch.cuda.synchronize()
    loop_ms = (time.perf_counter() - t0) * 1e3
    same = bool(torch.equal(loop_out, sorter.output))
    res = {"arrays": int(lens.size), "keys": total, "batched_ms": round(ms, 3),
           "batched_gkeys_s": round(total / (ms * 1e-3) / 1e9, 3), "loop_ms": round(loop_ms, 2),
           "loop_gkeys_s": round(total / (loop_ms * 1e-3) / 1e9, 3),
           "speedup_vs_loop": round(loop_ms / ms, 2), "identical_to_loop": same,
           "tuning": {"small_variant": sorter.tuning.small_variant, "small_cutoff": sorter.tuning.small_cutoff,
                      "large_variant": sorter.tuning.large_variant}}
    if check:
        got = sorter.output.cpu().numpy().view(kdt)
        a = keys.cpu().numpy().view(kdt)
        from oracle import oracle as O          # verifies the results, outside the timed region
        want = O.sortcopy_segments(a, offs, "native", "ascfwdorder", threads=oracle_threads())
        res["checked"] = "every segment bit-exact vs oracle" if np_bytes_equal(got, want) else "FAILED vs oracle"
    del keys, off_t, sorter, loop_out
    torch.cuda.empty_cache()
    return res


def batched_config(args) -> dict:
    """Batch A: 100,000 uint32 arrays, lengths log-uniform [16, 2^20] (seed 0x5EED0005), also truncated
    at a cumulative 2^28 keys; batch B: 20,000 float64 arrays, log-uniform [64, 2^18] (seed 0x5EED0006)."""
    which = [w for w in args.batches.split(",") if w]
    if not which or any(w not in ("A_2p28", "A", "B") for w in which):
        raise SystemExit(f"--batches: a comma-separated subset of A_2p28, A, B, not {args.batches!r}")
    res = {w: batched_run(args, w, args.steps, check=not args.no_cpu) for w in which}
    return {"config": "batched segmented sort (one captured CUDA graph per batch) vs per-array loop",
            "steps": args.steps, "results": res}


def serving_run(args, rate: float, duration: float, closed: int, checks: int) -> dict:
    """Poisson arrivals at `rate` req/s for `duration` s; length log-uniform [2^10, 2^26]; key type
    uniform over {uint16, int32, float32, float64}; direction asc/desc (forward order); absolute filter
    with probability 0.5; 64 GB device budget.  Inputs are slices of device-resident pools (the loop
    measures sort service, not host transfers).  Then (unless `closed` is 0) the first `closed`
    requests, closed-loop: all queued at once through the server vs a loop of plain allocating
    sorts.  `checks` served results
    (spread over the run, the largest request included) are compared with the oracle."""
    import numpy as np
    import torch
    from radixsortbidi8_gb300 import serving, synth as S
    import radixsortbidi8_gb300 as rs
    dev = torch.device("cuda", torch.cuda.current_device())
    arr, lens, kind, desc, absf = S.serving_requests(rate, duration)
    nreq = arr.size
    kinds = [(np.uint16, torch.int16), (np.int32, torch.int32), (np.float32, torch.int32), (np.float64, torch.int64)]
    pool_n = 1 << 27
    pools = []
    for kd, td in kinds:
        kb = np.dtype(kd).itemsize
        bits = S.float_specials_torch(7, pool_n, kb, device=dev) if kd in (np.float32, np.float64) else \
            S.uniform_bits_torch(7, pool_n, kb, device=dev)
        pools.append(bits.view(td) if bits.dtype != td else bits)
    ring_n = 1 << 30
    rings = [torch.empty(ring_n, dtype=td, device=dev) for _, td in kinds]
    ring_pos = [0, 0, 0, 0]
    ring_owner = [[], [], [], []]           # (start, end, request id) still possibly in flight
    starts = (S.splitmix64(S.SERVING_SEED, nreq, stream=44) % np.uint64(pool_n - (1 << 26))).astype(np.int64)
    torch.cuda.synchronize()                  # the pools are read, and the rings written, on the server's streams
    srv = serving.Server(budget_bytes=64 << 30, max_inflight=4)
    ids, metas = [], []

    def dm(i):
        return ("dscfwdorder" if desc[i] else "ascfwdorder"), ("nativeabs" if absf[i] else "native")

    def out_region(k, n):
        p = ring_pos[k] if ring_pos[k] + n <= ring_n else 0
        keep = []
        for (a, b, rid) in ring_owner[k]:
            if a < p + n and p < b:
                srv.wait(rid)             # the region is about to be reused
            else:
                keep.append((a, b, rid))
        ring_owner[k] = keep
        ring_pos[k] = p + n
        return p

    t_begin = time.perf_counter()
    for i in range(nreq):
        delay = t_begin + arr[i] - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        k = kind[i]
        n = int(lens[i])
        p = out_region(k, n)
        d, m = dm(i)
        rid = srv.submit(pools[k][starts[i]:starts[i] + n], rings[k][p:p + n], d, m, key_dtype=kinds[k][0])
        ring_owner[k].append((p, p + n, rid))
        ids.append(rid)
        metas.append((k, n, d, m, int(starts[i]), p))
    srv.drain()
    infos = [srv.wait(r) for r in ids]
    st = srv.stats()
    t_first = min(i.submit_s for i in infos)
    t_last = max(i.done_s for i in infos)
    keys = int(sum(i.count for i in infos))
    lat = serving.latency_summary(infos)
    # checks: results whose output region no later request of the same key type overwrote, against
    # the oracle
    from oracle import oracle as O          # verifies the results, outside the timed region
    kk = np.array([m[0] for m in metas])
    pp = np.array([m[5] for m in metas], dtype=np.int64)
    nn = np.array([m[1] for m in metas], dtype=np.int64)
    cand = []
    for j in range(nreq):
        later = np.nonzero(kk[j + 1:] == kk[j])[0] + j + 1
        if not np.any((pp[later] < pp[j] + nn[j]) & (pp[j] < pp[later] + nn[later])):
            cand.append(j)
    pick = sorted(set(cand[::max(1, len(cand) // max(1, checks - 1))][:max(0, checks - 1)] +
                      ([max(cand, key=lambda j: metas[j][1])] if cand else []))) if checks > 0 else []
    items, gots = [], []
    for j in pick:
        k, n, d, m, s0, p = metas[j]
        kd = kinds[k][0]
        items.append((pools[k][s0:s0 + n].cpu().numpy().view(kd), m, d))
        gots.append(rings[k][p:p + n].cpu().numpy().view(kd))
    wants = O.sortcopy_batch(items, threads=oracle_threads()) if items else []
    bad = sum(not np_bytes_equal(g, w) for g, w in zip(gots, wants))
    srv.close()
    del rings
    torch.cuda.empty_cache()
    open_loop = {"config": f"serving: Poisson {rate:g} req/s for {duration:g} s, lengths log-uniform "
                           f"[2^10, 2^26], {{u16, i32, f32, f64}}, asc/desc, abs p=0.5, 64 GB budget",
                 "requests": nreq, "offered_gkeys_s": round(float(lens.sum()) / duration / 1e9, 3),
                 "served_gkeys_s": round(keys / (t_last - t_first) / 1e9, 3), "latency": lat,
                 "batches": st["batches"], "launches_per_request": round(st["batches"] / max(1, nreq), 3),
                 "max_coalesced": st["max_coalesced"], "max_inflight_batches": st["max_inflight_batches"],
                 "checked": f"{len(pick) - bad} of {len(pick)} served results bit-exact vs oracle"}
    if closed <= 0:
        return open_loop
    # closed loop: a prefix of the same requests, queued at once vs a plain allocating-sort loop
    m_req = min(nreq, closed)
    outs = [torch.empty(int(lens[i]), dtype=kinds[kind[i]][1], device=dev) for i in range(m_req)]
    torch.cuda.synchronize()
    srv2 = serving.Server(budget_bytes=64 << 30, max_inflight=4)
    for i in range(min(m_req, 64)):          # warm-up of kernels and module loading
        d, m = dm(i)
        srv2.submit(pools[kind[i]][starts[i]:starts[i] + int(lens[i])], outs[i], d, m, key_dtype=kinds[kind[i]][0])
    srv2.drain()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ids2 = []
    for i in range(m_req):
        d, m = dm(i)
        ids2.append(srv2.submit(pools[kind[i]][starts[i]:starts[i] + int(lens[i])], outs[i], d, m,
                                key_dtype=kinds[kind[i]][0]))
    srv2.drain()
    served_s = time.perf_counter() - t0
    st2 = srv2.stats()
    srv2.close()
    # the closed loop's results, the largest requests included, against the oracle
    cpick = sorted(set(list(range(0, m_req, max(1, m_req // max(1, checks - 1))))[:max(0, checks - 1)] +
                       [int(np.argmax(lens[:m_req]))])) if checks > 0 and m_req > 0 else []
    citems, cgots = [], []
    for i in cpick:
        d, m = dm(i)
        kd = kinds[kind[i]][0]
        citems.append((pools[kind[i]][starts[i]:starts[i] + int(lens[i])].cpu().numpy().view(kd), m, d))
        cgots.append(outs[i].cpu().numpy().view(kd))
    cwants = O.sortcopy_batch(citems, threads=oracle_threads()) if citems else []
    cbad = sum(not np_bytes_equal(g, w) for g, w in zip(cgots, cwants))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(m_req):
        d, m = dm(i)
        rs.radixsortcopy(pools[kind[i]][starts[i]:starts[i] + int(lens[i])], outs[i], d, m,
                         key_dtype=kinds[kind[i]][0])
    torch.cuda.synchronize()
    loop_s = time.perf_counter() - t0
    keys2 = int(lens[:m_req].sum())
    del outs
    torch.cuda.empty_cache()
    return {**open_loop,
            "closed_loop": {"requests": m_req, "keys": keys2,
                            "served_gkeys_s": round(keys2 / served_s / 1e9, 3),
                            "plain_loop_gkeys_s": round(keys2 / loop_s / 1e9, 3),
                            "speedup": round(loop_s / served_s, 2), "batches": st2["batches"],
                            "checked": f"{len(cpick) - cbad} of {len(cpick)} results bit-exact vs oracle"}}


def serving_config(args) -> dict:
    return serving_run(args, args.rate, args.duration, 2000, 64)


def main():
    args = parse_args()
    if args.calibrate_cpu:
        print(json.dumps(calibrate_cpu(args)), flush=True)
        return
    if args.case:
        print(json.dumps(single_case(args)), flush=True)
        return
    if args.config == "batched":
        print(json.dumps(batched_config(args)), flush=True)
        return
    if args.config == "serving":
        print(json.dumps(serving_config(args)), flush=True)
        return
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if world > 1 and args.impl == "gb300":
        import torch
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    if args.impl == "reference":
        line = reference_arm(args, rank, world)
    else:
        line = gb300_arm(args, rank, world)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if world > 1 and args.impl == "gb300":
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
