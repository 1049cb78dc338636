"""Batched (segmented) sort: many independent arrays of uneven sizes in one stream-ordered call.

``segmented_sortcopy`` sorts every segment ``[offsets[s], offsets[s+1])`` of a concatenated
device array on its own (the semantics of ``radixsortcopy``); small segments are sorted whole in
shared memory by a block-local radix sort, large ones run the onesweep passes, all in the same
launches (C ABI ``rsbd8g_segmented_sortcopy``).  ``SegmentedSorter`` owns the buffers of one
batch shape and can capture the whole call into a CUDA graph (one graph launch per batch).

The small-segment block-sort shape (threads x items), the small/large cutoff and the tile of the
large segments' onesweep passes (keys per thread) are picked per key size by ``autotune`` and kept
in ``tuning.json`` beside this file; ``tuning_for`` reads it.
"""
from __future__ import annotations

import ctypes
import json
import os
import time

import numpy as np

from . import api

TUNING_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning.json")
SMALL_SHAPES = {  # variant -> (threads, items) per key size, as compiled in the library
    1: [(256, 8), (256, 16), (512, 16)], 2: [(256, 8), (256, 16), (512, 16)],
    4: [(256, 8), (256, 16), (512, 16)], 8: [(256, 8), (256, 12), (512, 12)],
}
LARGE_SHAPES = {  # large_variant -> (threads, items) of the large segments' onesweep tiles
    1: [(512, 28), (512, 20)], 2: [(512, 28), (512, 20)], 4: [(512, 28), (512, 20)], 8: [(512, 12), (512, 16)],
}


class SegTuning(ctypes.Structure):
    """rsbd8g_segtuning of include/rsbd8g.h"""
    _fields_ = [("small_variant", ctypes.c_uint32), ("small_cutoff", ctypes.c_uint32),
                ("large_variant", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


def _lib():
    L = api.lib()
    if not getattr(L, "_seg_sigs", False):
        P, S, VP = ctypes.POINTER(api.Desc), ctypes.c_size_t, ctypes.c_void_p
        L.rsbd8g_segmented_scratch_bytes.argtypes = [P, S, S, ctypes.POINTER(SegTuning), ctypes.POINTER(S)]
        L.rsbd8g_segmented_scratch_bytes.restype = ctypes.c_int
        L.rsbd8g_segmented_sortcopy.argtypes = [P, S, S, VP, VP, S, VP, VP, VP, ctypes.POINTER(SegTuning), VP]
        L.rsbd8g_segmented_sortcopy.restype = ctypes.c_int
        L.rsbd8g_segmented_sortcopy_ptrs.argtypes = [P, S, S, VP, VP, VP, VP, VP, S, ctypes.POINTER(SegTuning), VP]
        L.rsbd8g_segmented_sortcopy_ptrs.restype = ctypes.c_int
        L.rsbd8g_segmented_sortcopy_ptrs_dirs.argtypes = [P, S, S, VP, VP, VP, VP, VP, VP, S, ctypes.POINTER(SegTuning),
                                                          VP]
        L.rsbd8g_segmented_sortcopy_ptrs_dirs.restype = ctypes.c_int
        L._seg_sigs = True
    return L


def tuning_for(key_bytes: int) -> SegTuning:
    """The tuned small-segment shape, cutoff and large-segment tile for a key size (library defaults
    if untuned)."""
    try:
        with open(TUNING_PATH) as f:
            t = json.load(f)["segmented"][str(key_bytes)]
        return SegTuning(int(t["small_variant"]), int(t["small_cutoff"]), int(t.get("large_variant", 0)))
    except (OSError, KeyError, ValueError):
        return SegTuning(1, 0)


def segmented_scratch_bytes(key_dtype, total: int, nsegs: int, direction="ascfwdorder", mode="native",
                            tuning: SegTuning | None = None) -> int:
    d = api.make_desc(key_dtype, direction, mode)
    t = tuning if tuning is not None else tuning_for(d.key_bytes)
    out = ctypes.c_size_t(0)
    api._check(_lib().rsbd8g_segmented_scratch_bytes(ctypes.byref(d), total, nsegs, ctypes.byref(t),
                                                     ctypes.byref(out)), "rsbd8g_segmented_scratch_bytes")
    return out.value


def segmented_sortcopy_ptrs(inputs, outputs, buffers, scratch, direction="ascfwdorder", mode="native",
                            key_dtype=None, tuning: SegTuning | None = None, stream=None, flags: int = 0,
                            directions=None):
    """Sort every device tensor of `inputs` into the tensor of `outputs` at the same place, using the
    tensor of `buffers` there (rsbd8g_segmented_sortcopy_ptrs: one segment per array, in one call).
    Stream-ordered; read device errors with api.scratch_status.  flags may carry
    api.FLAG_DEVICE_ARRAYS when every array is device memory (tiles are then prefetched into L2).
    With `directions` (one sortingdirection name or value per array) every array is sorted in its
    own direction (rsbd8g_segmented_sortcopy_ptrs_dirs) and `direction` is not used.
    Returns the device pointer tables and offsets: keep them until the call's work is done."""
    import torch
    dev = inputs[0].device
    kb = api.key_kind(key_dtype if key_dtype is not None else inputs[0].dtype)[1]
    lens = [int(x.numel() * x.element_size() // kb) for x in inputs]
    offs = torch.zeros(len(lens) + 1, dtype=torch.int64)
    offs[1:] = torch.cumsum(torch.tensor(lens, dtype=torch.int64), 0)
    tabs = [torch.tensor([api._ptr(x) if x.numel() else 0 for x in arrs], dtype=torch.int64).to(dev)
            for arrs in (inputs, outputs, buffers)]
    offs = offs.to(dev)
    d = api.make_desc(key_dtype if key_dtype is not None else inputs[0].dtype, direction, mode, flags=flags)
    t = tuning if tuning is not None else tuning_for(d.key_bytes)
    if directions is not None:
        dirs = torch.tensor([api._direction(x) for x in directions], dtype=torch.uint8).to(dev)
        tabs.append(dirs)
        api._check(_lib().rsbd8g_segmented_sortcopy_ptrs_dirs(
            ctypes.byref(d), int(offs[-1]), len(lens), api._ptr(offs), api._ptr(tabs[0]), api._ptr(tabs[1]),
            api._ptr(tabs[2]), dirs.data_ptr(), api._ptr(scratch), scratch.numel() * scratch.element_size(),
            ctypes.byref(t), api._stream(stream)), "rsbd8g_segmented_sortcopy_ptrs_dirs")
        return tabs, offs
    api._check(_lib().rsbd8g_segmented_sortcopy_ptrs(
        ctypes.byref(d), int(offs[-1]), len(lens), api._ptr(offs), api._ptr(tabs[0]), api._ptr(tabs[1]),
        api._ptr(tabs[2]), api._ptr(scratch), scratch.numel() * scratch.element_size(), ctypes.byref(t),
        api._stream(stream)), "rsbd8g_segmented_sortcopy_ptrs")
    return tabs, offs


def segmented_sortcopy(input, output, buffer, offsets, scratch, direction="ascfwdorder", mode="native",
                       key_dtype=None, tuning: SegTuning | None = None, stream=None, flags: int = 0) -> None:
    """Sort every segment of `input` into `output` (device tensors; `offsets` an int64/uint64 CUDA
    tensor of nsegs + 1 offsets).  Stream-ordered; read device errors with api.scratch_status."""
    d = api.make_desc(key_dtype if key_dtype is not None else input.dtype, direction, mode, flags=flags)
    t = tuning if tuning is not None else tuning_for(d.key_bytes)
    nsegs = int(offsets.numel()) - 1
    api._check(_lib().rsbd8g_segmented_sortcopy(
        ctypes.byref(d), api._count(input, None, d), nsegs, api._ptr(offsets), api._ptr(scratch),
        scratch.numel() * scratch.element_size(), api._ptr(input), api._ptr(output), api._ptr(buffer),
        ctypes.byref(t), api._stream(stream)), "rsbd8g_segmented_sortcopy")


class SegmentedSorter:
    """Buffers for one batch shape; ``run`` sorts, ``capture`` records one CUDA graph of the call
    and ``replay`` launches it (one graph launch per batch).

    The sort runs on the sorter's own stream, ordered after the work already queued on the
    caller's current stream (which made the input and allocated the buffers) and before the work
    the caller queues after the call, as a call on the current stream would be."""

    def __init__(self, input, offsets, direction="ascfwdorder", mode="native", key_dtype=None,
                 tuning: SegTuning | None = None, stream=None):
        import torch
        self.input, self.offsets = input, offsets
        self.direction, self.mode = direction, mode
        self.key_dtype = key_dtype if key_dtype is not None else input.dtype
        self.tuning = tuning if tuning is not None else tuning_for(api.key_kind(self.key_dtype)[1])
        self.output = torch.empty_like(input)
        self.buffer = torch.empty_like(input)
        total = int(input.numel() * input.element_size() // api.key_kind(self.key_dtype)[1])
        nb = segmented_scratch_bytes(self.key_dtype, total, int(offsets.numel()) - 1,
                                     direction, mode, self.tuning)
        self.scratch = torch.empty(nb, dtype=torch.uint8, device=input.device)
        self.stream = stream if stream is not None else torch.cuda.Stream(device=input.device)
        self.graph = None

    def _after_caller(self):
        """the sorter's stream waits for the caller's queued work; returns the caller's stream"""
        import torch
        cur = torch.cuda.current_stream(self.input.device)
        if cur != self.stream:
            self.stream.wait_stream(cur)
        return cur

    def _before_caller(self, cur) -> None:
        """the caller's later work waits for the sort"""
        if cur != self.stream:
            cur.wait_stream(self.stream)

    def _sort(self):
        segmented_sortcopy(self.input, self.output, self.buffer, self.offsets, self.scratch, self.direction,
                           self.mode, self.key_dtype, self.tuning, self.stream)

    def run(self):
        cur = self._after_caller()
        self._sort()
        self._before_caller(cur)
        return self.output

    def capture(self):
        import torch
        cur = self._after_caller()
        with torch.cuda.stream(self.stream):
            self._sort()               # first call outside capture: kernel attributes, module loading
            self.stream.synchronize()
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph, stream=self.stream):
                self._sort()
        self._before_caller(cur)
        return self

    def replay(self):
        import torch
        cur = self._after_caller()
        with torch.cuda.stream(self.stream):       # a graph launches on the current stream
            self.graph.replay()
        self._before_caller(cur)
        return self.output

    def status(self) -> int:
        return api.scratch_status(self.scratch, self.stream)


def sort_each(input, output, offsets_host: np.ndarray, direction="ascfwdorder", mode="native", key_dtype=None,
              stream=None) -> None:
    """The per-array loop the batched call replaces: one plain noalloc sort per segment."""
    import torch
    kd = key_dtype if key_dtype is not None else input.dtype
    lens = np.diff(offsets_host)
    big = int(lens.max()) if lens.size else 0
    scratch = torch.empty(api.scratch_bytes(kd, max(big, 2), direction, mode), dtype=torch.uint8,
                          device=input.device)
    buf = torch.empty(max(big, 1), dtype=input.dtype, device=input.device)
    es = input.element_size()
    ip, op, bp = input.data_ptr(), output.data_ptr(), buf.data_ptr()
    L = api.lib()
    d = api.make_desc(kd, direction, mode)
    cur = torch.cuda.current_stream(input.device)
    if isinstance(stream, torch.cuda.Stream) and stream != cur:
        stream.wait_stream(cur)                 # the buffers above were allocated on the caller's stream
    elif stream is not None and not isinstance(stream, torch.cuda.Stream):
        cur.synchronize()                       # a raw stream handle: wait on the host instead
    st = api._stream(stream)
    nb = scratch.numel()
    sp = scratch.data_ptr()
    for s in range(lens.size):
        n = int(lens[s])
        if n == 0:
            continue
        o = int(offsets_host[s]) * es
        rc = L.rsbd8g_radixsortcopynoalloc(ctypes.byref(d), n, sp, nb, ip + o, op + o, bp, st)
        if rc != 0:
            raise api.RSBD8GError(rc, "radixsortcopynoalloc")


# ---- autotuner -------------------------------------------------------------------------------

def _synthetic_batch(key_bytes: int, nsegs: int, lo: int, hi: int, seed: int, device="cuda"):
    import torch
    from . import synth
    lens = synth.log_uniform_lengths(seed, nsegs, lo, hi)
    offs = np.zeros(nsegs + 1, dtype=np.int64)
    np.cumsum(lens, out=offs[1:])
    keys = synth.uniform_bits_torch(seed, int(offs[-1]), key_bytes, device=device)
    return keys, torch.from_numpy(offs).to(device), offs


def _time_sorter(keys, offs, kd, t: SegTuning, reps: int) -> float:
    """ms per sort of the batch with tuning t"""
    import torch
    s = SegmentedSorter(keys, offs, key_dtype=kd, tuning=t)
    torch.cuda.current_stream().synchronize()    # keys made, buffers allocated on this stream
    with torch.cuda.stream(s.stream):
        s.run()
        s.stream.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            s.run()
        s.stream.synchronize()
    ms = (time.perf_counter() - t0) / reps * 1e3
    del s
    return ms


# the batch each key size is tuned on: (segments, shortest, longest), lengths log-uniform; keys up to
# 4 bytes: the 2^28-key batch of uniform arrays of 16 to 2^20 keys, 8-byte keys: arrays of 64 to 2^18
TUNE_BATCHES = {1: (3000, 16, 1 << 20), 2: (3000, 16, 1 << 20), 4: (3000, 16, 1 << 20), 8: (20000, 64, 1 << 18)}


def autotune(key_bytes_list=(2, 4, 8), reps: int = 3, batches: dict | None = None, write: bool = True) -> dict:
    """Per key size: time every compiled small-segment shape (threads x items) with a few cutoffs,
    each with every compiled tile of the large segments' onesweep passes (keys per thread), on a
    synthetic batch of log-uniform lengths (TUNE_BATCHES); the fastest settings go to tuning.json."""
    import torch
    kd = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}
    shapes = batches if batches is not None else TUNE_BATCHES
    best = {}
    report = {}
    for kb in key_bytes_list:
        nsegs, lo, hi = shapes[kb]
        keys, offs, _ = _synthetic_batch(kb, nsegs, lo, hi, seed=1234 + kb)
        results = []
        for v, (th, it) in enumerate(SMALL_SHAPES[kb]):
            cap = th * it
            for cutoff in sorted({cap // 4, cap // 2, cap}):
                for lv in range(len(LARGE_SHAPES[kb])):
                    results.append((_time_sorter(keys, offs, kd[kb], SegTuning(v, cutoff, lv), reps), v, cutoff, lv))
        results.sort()
        ms, v, cutoff, lv = results[0]
        del keys, offs
        torch.cuda.empty_cache()
        best[str(kb)] = {"small_variant": v, "small_cutoff": cutoff, "threads_items": SMALL_SHAPES[kb][v],
                         "large_variant": lv, "large_threads_items": LARGE_SHAPES[kb][lv], "ms": round(ms, 3),
                         "batch": {"segments": nsegs, "lengths": f"log-uniform [{lo}, {hi}]"}}
        report[str(kb)] = [{"ms": round(m, 3), "small_variant": a, "small_cutoff": c, "large_variant": x}
                           for m, a, c, x in results]
    if write:
        data = {}
        try:
            with open(TUNING_PATH) as f:
                data = json.load(f)
        except (OSError, ValueError):
            pass
        data.setdefault("segmented", {}).update(best)
        data["segmented_workload"] = {"reps": reps, "batches": {str(k): list(v) for k, v in shapes.items()}}
        with open(TUNING_PATH, "w") as f:
            json.dump(data, f, indent=1)
    return {"best": best, "all": report}
