"""Seeded synthetic workloads of the benchmark configurations (deterministic, counter-based).

Every value is a function of (seed, index) through splitmix64, and the numpy generators use
only correctly rounded basic arithmetic (no log/exp/cos from the platform's maths library), so
the same call gives the same bits on any host -- the reference-generated fixtures depend on it.
The torch variants compute the identical integer stream on the GPU for the large benchmark
inputs; their floating-point shaping uses device maths functions and is not bit-identical to
the numpy one, which nothing relies on.

Workloads (the reference benchmarks random bit patterns only; these stand in for the
configurations it is measured on):
  * uniform bits of any 1/2/4/8-byte key type;
  * uint32 with only the low 12 bits random (exercises the pass-skip test);
  * float32/float64 N(0, sigma) with 1% -0.0, 0.5% +-inf and 0.1% NaN (half 0x7FC00000-style
    positive quiet NaN, half negative);
  * int64 uniform over the full signed range;
  * 24-byte records {u64 id, f64 key, u32 tag, u32 pad}, key = lognormal(0, 2) x random sign,
    10% of the records copy the key of an earlier random record;
  * log-uniform segment lengths; Poisson arrival times.
"""
from __future__ import annotations

import os

import numpy as np

GOLDEN = np.uint64(0x9E3779B97F4A7C15)
M1 = np.uint64(0xBF58476D1CE4E5B9)
M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, n: int, offset: int = 0, stream: int = 0) -> np.ndarray:
    """n uint64 values: splitmix64 of the counters offset..offset+n-1 (stream selects a sub-sequence)."""
    with np.errstate(over="ignore"):
        base = np.uint64((seed * 0x632BE59BD9B4E019 + stream * 0x8CB92BA72F3D8DD7) & 0xFFFFFFFFFFFFFFFF)
        z = (np.arange(offset, offset + n, dtype=np.uint64) + np.uint64(1)) * GOLDEN + base
        z = (z ^ (z >> np.uint64(30))) * M1
        z = (z ^ (z >> np.uint64(27))) * M2
        return z ^ (z >> np.uint64(31))


def unit_interval(bits: np.ndarray) -> np.ndarray:
    """uint64 -> float64 in (0, 1]."""
    return ((bits >> np.uint64(11)).astype(np.float64) + 1.0) * (1.0 / 9007199254740992.0)


# Every generator below is a function of the element index (counter-based), so `offset` gives
# elements offset..offset+n-1 of the same sequence: host_parallel fills one array from chunks.

def uniform_bits(seed: int, n: int, dtype, offset: int = 0) -> np.ndarray:
    dt = np.dtype(dtype)
    ut = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[dt.itemsize]
    return splitmix64(seed, n, offset).astype(ut).view(dt)


def low_bits_u32(seed: int, n: int, bits: int = 12, offset: int = 0) -> np.ndarray:
    return (splitmix64(seed, n, offset) & np.uint64((1 << bits) - 1)).astype(np.uint32)


def normal(seed: int, n: int, stream: int = 0, offset: int = 0) -> np.ndarray:
    """Approximately N(0, 1): the Irwin-Hall sum of 12 uniforms minus 6 (summed in a fixed order,
    so every platform rounds identically)."""
    acc = np.zeros(n, dtype=np.float64)
    for k in range(12):
        acc += unit_interval(splitmix64(seed, n, offset, stream=100 * stream + k + 1))
    return acc - 6.0


def exp2_det(t: np.ndarray) -> np.ndarray:
    """2**t from basic arithmetic only: ldexp of a fixed-order Taylor polynomial of 2**f, f in [0, 1)."""
    i = np.floor(t)
    x = (t - i) * 0.6931471805599453
    p = np.ones_like(x)
    term = np.ones_like(x)
    for k in range(1, 12):
        term = term * x / float(k)
        p = p + term
    return np.ldexp(p, i.astype(np.int64))


def float_specials(seed: int, n: int, dtype=np.float32, sigma: float = 1e3, offset: int = 0) -> np.ndarray:
    """N(0, sigma) with 1% -0.0, 0.5% +-inf (half each sign), 0.1% NaN (half each sign)."""
    dt = np.dtype(dtype)
    x = (normal(seed, n, offset=offset) * sigma).astype(dt)
    r = unit_interval(splitmix64(seed, n, offset, stream=7))
    x[r <= 0.01] = -0.0
    inf = (r > 0.01) & (r <= 0.015)
    x[inf & (r <= 0.0125)] = np.inf
    x[inf & (r > 0.0125)] = -np.inf
    nan = (r > 0.015) & (r <= 0.016)
    ut = {4: np.uint32, 8: np.uint64}[dt.itemsize]
    qnan = {4: 0x7FC00000, 8: 0x7FF8000000000000}[dt.itemsize]
    sbit = {4: 0x80000000, 8: 0x8000000000000000}[dt.itemsize]
    bits = x.view(ut)
    bits[nan & (r <= 0.0155)] = ut(qnan)
    bits[nan & (r > 0.0155)] = ut(qnan | sbit)
    return x


def host_parallel(gen, n: int, out_dtype, *args, chunk: int = 1 << 22, threads: int | None = None,
                  **kw) -> np.ndarray:
    """gen(*args, m, ..., offset=o) for chunks of m elements, filled into one array by a thread pool
    (the numpy operations release the interpreter lock); equal to one call of gen over n elements.
    `args` are the arguments before the count (the seed), `kw` those after it."""
    import concurrent.futures as cf
    out = np.empty(n, dtype=out_dtype)

    def fill(o):
        m = min(chunk, n - o)
        out[o:o + m] = gen(*args, m, offset=o, **kw)

    with cf.ThreadPoolExecutor(max_workers=threads or os.cpu_count() or 1) as ex:
        list(ex.map(fill, range(0, n, chunk)))
    return out


def records24(seed: int, n: int) -> np.ndarray:
    """24-byte records {u64 id, f64 key, u32 tag, u32 pad}; key = lognormal(0, 2) x random sign,
    10% duplicate the key of an earlier random record."""
    rec = np.zeros(n, dtype=[("id", "<u8"), ("key", "<f8"), ("tag", "<u4"), ("pad", "<u4")])
    rec["id"] = np.arange(n, dtype=np.uint64)
    key = exp2_det(normal(seed, n) * (2.0 / 0.6931471805599453))      # lognormal(0, 2)
    sgn = (splitmix64(seed, n, stream=11) & np.uint64(1)).astype(bool)
    key = np.where(sgn, -key, key)
    dup = unit_interval(splitmix64(seed, n, stream=12)) <= 0.1
    dup[0] = False
    src = (unit_interval(splitmix64(seed, n, stream=13)) * np.arange(n)).astype(np.int64)
    src = np.minimum(src, np.maximum(np.arange(n) - 1, 0))
    # a duplicate copies the final key of its source, which may itself be a duplicate
    root = np.where(dup, src, np.arange(n))
    while True:
        chain = dup[root]
        if not chain.any():
            break
        root[chain] = src[root[chain]]
    rec["key"] = key[root]
    rec["tag"] = (splitmix64(seed, n, stream=14) & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    return rec


def log_uniform_lengths(seed: int, count: int, lo: int, hi: int) -> np.ndarray:
    u = unit_interval(splitmix64(seed, count, stream=21))
    return np.minimum(np.floor(np.exp(u * np.log(hi / lo)) * lo), hi).astype(np.int64)


def poisson_arrivals(seed: int, rate: float, duration: float) -> np.ndarray:
    """Arrival times (s) of a Poisson process of `rate` per second over `duration` seconds."""
    est = int(rate * duration * 1.2 + 100)
    gaps = -np.log(unit_interval(splitmix64(seed, est, stream=31))) / rate
    t = np.cumsum(gaps)
    return t[t < duration]


# ---- GPU (torch) versions of the integer stream, for the large configurations -------------

def splitmix64_torch(seed: int, n: int, device="cuda", offset: int = 0, stream: int = 0):
    """The splitmix64 stream of splitmix64(), computed on the device as int64 (same bits)."""
    import torch

    def s64(v):
        v &= 0xFFFFFFFFFFFFFFFF
        return v - (1 << 64) if v >= (1 << 63) else v

    base = s64(seed * 0x632BE59BD9B4E019 + stream * 0x8CB92BA72F3D8DD7)
    z = torch.arange(offset + 1, offset + n + 1, dtype=torch.int64, device=device)
    z.mul_(s64(0x9E3779B97F4A7C15)).add_(base)

    def lsr(x, k):
        return (x >> k) & ((1 << (64 - k)) - 1)

    z = (z ^ lsr(z, 30)) * s64(0xBF58476D1CE4E5B9)
    z = (z ^ lsr(z, 27)) * s64(0x94D049BB133111EB)
    return z ^ lsr(z, 31)


def uniform_bits_torch(seed: int, n: int, key_bytes: int, device="cuda"):
    """Uniform random key bits as a signed torch tensor of key_bytes width."""
    import torch
    z = splitmix64_torch(seed, n, device)
    if key_bytes == 8:
        return z
    t = {1: torch.int8, 2: torch.int16, 4: torch.int32}[key_bytes]
    mask = (1 << (8 * key_bytes)) - 1
    half = 1 << (8 * key_bytes - 1)
    v = z & mask
    return torch.where(v >= half, v - (1 << (8 * key_bytes)), v).to(t)


def low_bits_u32_torch(seed: int, n: int, bits: int = 12, device="cuda"):
    import torch
    return (splitmix64_torch(seed, n, device) & ((1 << bits) - 1)).to(torch.int32)


def float_specials_torch(seed: int, n: int, key_bytes: int = 4, sigma: float = 1e3, device="cuda"):
    """float_specials() computed on the device; returns the key bits as int32/int64."""
    import torch

    def unit(z):
        return (((z >> 11) & ((1 << 53) - 1)).to(torch.float64) + 1.0) * (1.0 / 9007199254740992.0)

    u1 = unit(splitmix64_torch(seed, n, device, stream=1))
    u2 = unit(splitmix64_torch(seed, n, device, stream=2))
    x = torch.sqrt(-2.0 * torch.log(u1)) * torch.cos(2.0 * np.pi * u2) * sigma
    del u1, u2
    r = unit(splitmix64_torch(seed, n, device, stream=7))
    if key_bytes == 4:
        x = x.to(torch.float32)
    x[r <= 0.01] = -0.0
    x[(r > 0.01) & (r <= 0.0125)] = float("inf")
    x[(r > 0.0125) & (r <= 0.015)] = float("-inf")
    bits = x.view(torch.int32 if key_bytes == 4 else torch.int64)
    qnan = 0x7FC00000 if key_bytes == 4 else 0x7FF8000000000000
    nqnan = (0x7FC00000 | 0x80000000) - (1 << 32) if key_bytes == 4 else (0x7FF8000000000000 | (1 << 63)) - (1 << 64)
    bits[(r > 0.015) & (r <= 0.0155)] = qnan
    bits[(r > 0.0155) & (r <= 0.016)] = nqnan
    return bits


def unit_interval_torch(z):
    """unit_interval() of a splitmix64_torch stream: float64 in (0, 1], the same values."""
    import torch
    return (((z >> 11) & ((1 << 53) - 1)).to(torch.float64) + 1.0) * (1.0 / 9007199254740992.0)


def normal_torch(seed: int, n: int, stream: int = 0, device="cuda"):
    """normal() on the device: the same Irwin-Hall sum in the same order, so the same bits."""
    import torch
    acc = torch.zeros(n, dtype=torch.float64, device=device)
    for k in range(12):
        acc += unit_interval_torch(splitmix64_torch(seed, n, device, stream=100 * stream + k + 1))
    return acc - 6.0


def exp2_det_torch(t):
    """exp2_det() on the device: the same Taylor polynomial, and 2**i built from its exponent bits
    (exact), so the same bits."""
    import torch
    i = torch.floor(t)
    x = (t - i) * 0.6931471805599453
    p = torch.ones_like(x)
    term = torch.ones_like(x)
    for k in range(1, 12):
        term = term * x / float(k)
        p = p + term
    scale = ((i.to(torch.int64) + 1023) << 52).view(torch.float64)
    return p * scale


def records24_torch(seed: int, n: int, device="cuda"):
    """records24() built on the device, bit for bit: an (n, 3) int64 tensor holding the n 24-byte
    records {u64 id, f64 key, u32 tag, u32 pad = 0}, row i at byte 24 * i."""
    import torch
    ar = torch.arange(n, dtype=torch.int64, device=device)
    key = exp2_det_torch(normal_torch(seed, n, device=device) * (2.0 / 0.6931471805599453))
    sgn = (splitmix64_torch(seed, n, device, stream=11) & 1).bool()
    key = torch.where(sgn, -key, key)
    dup = unit_interval_torch(splitmix64_torch(seed, n, device, stream=12)) <= 0.1
    dup[0] = False
    src = (unit_interval_torch(splitmix64_torch(seed, n, device, stream=13)) * ar.to(torch.float64)).to(torch.int64)
    src = torch.minimum(src, torch.clamp(ar - 1, min=0))
    root = torch.where(dup, src, ar)
    while True:
        chain = dup[root]
        if not bool(chain.any()):
            break
        root[chain] = src[root[chain]]
    rec = torch.empty((n, 3), dtype=torch.int64, device=device)
    rec[:, 0] = ar
    rec[:, 1] = key[root].view(torch.int64)
    rec[:, 2] = splitmix64_torch(seed, n, device, stream=14) & 0xFFFFFFFF
    return rec


# ---- the benchmark configurations' inputs ------------------------------------------------

# seeds of the mode/dtype sweep (three arrays of one size) and of the uniform uint32 array
SWEEP_SEEDS = {"f32": 0x5EED0002, "i64": 0x5EED0003, "u32low12": 0x5EED0004, "u32": 0x5EED0005}
RECORDS_SEED = 0x5EED0003
BATCH_A_SEED, BATCH_B_SEED, SERVING_SEED = 0x5EED0005, 0x5EED0006, 0x5EED0007


def sweep_arrays_torch(n: int, device="cuda"):
    """The mode/dtype sweep, one array each of n keys, on the device:
    (name, key bits tensor, key dtype, direction, mode) for float32 N(0, 1e3) with specials sorted
    descending with the absolute filter, int64 uniform ascending, and uint32 with only the low 12
    bits random ascending."""
    return [
        ("float32_abs_dscfwdorder", float_specials_torch(SWEEP_SEEDS["f32"], n, 4, device=device), np.float32,
         "dscfwdorder", "nativeabs"),
        ("int64_ascfwdorder", uniform_bits_torch(SWEEP_SEEDS["i64"], n, 8, device=device), np.int64,
         "ascfwdorder", "native"),
        ("uint32_low12_ascfwdorder", low_bits_u32_torch(SWEEP_SEEDS["u32low12"], n, device=device), np.uint32,
         "ascfwdorder", "native"),
    ]


def batch_lengths(which: str, scale: float = 1.0) -> np.ndarray:
    """Segment lengths of the batched configuration: "A" 100,000 uint32 arrays log-uniform in
    [16, 2^20]; "A_2p28" the same list cut where the running total reaches 2^28 keys; "B" 20,000
    float64 arrays log-uniform in [64, 2^18]."""
    if which in ("A", "A_2p28"):
        lens = log_uniform_lengths(BATCH_A_SEED, max(1, int(100000 * scale)), 16, 1 << 20)
        if which == "A_2p28":
            cut = int(np.searchsorted(np.cumsum(lens), 1 << 28))
            lens = lens[:max(1, cut)]
        return lens
    if which == "B":
        return log_uniform_lengths(BATCH_B_SEED, max(1, int(20000 * scale)), 64, 1 << 18)
    raise ValueError(which)


def batch_keys_torch(which: str, total: int, device="cuda"):
    """Concatenated keys of a batch (uint32 uniform bits for A, float64 with specials for B), built
    in chunks of 2^27 keys on the device."""
    import torch
    key_bytes = 4 if which.startswith("A") else 8
    seed = BATCH_A_SEED if key_bytes == 4 else BATCH_B_SEED
    t = torch.int32 if key_bytes == 4 else torch.int64
    keys = torch.empty(total, dtype=t, device=device)
    chunk = 1 << 27
    for o in range(0, total, chunk):
        m = min(chunk, total - o)
        keys[o:o + m] = uniform_bits_torch(seed + o, m, 4, device=device) if key_bytes == 4 else \
            float_specials_torch(seed + o, m, 8, device=device)
    return keys


SERVING_KINDS = (np.uint16, np.int32, np.float32, np.float64)


def serving_requests(rate: float, duration: float, lo: int = 1 << 10, hi: int = 1 << 26):
    """The serving configuration's request stream: arrival times (Poisson at `rate` per second for
    `duration` seconds), lengths log-uniform in [lo, hi], key type uniform over SERVING_KINDS,
    direction ascending/descending (forward order) and the absolute filter each with
    probability 1/2.  Returns (arrivals, lengths, kind index, descending flag, abs flag)."""
    arr = poisson_arrivals(SERVING_SEED, rate, duration)
    nreq = arr.size
    lens = log_uniform_lengths(SERVING_SEED, nreq, lo, hi)
    kind = (splitmix64(SERVING_SEED, nreq, stream=41) % np.uint64(len(SERVING_KINDS))).astype(int)
    desc = (splitmix64(SERVING_SEED, nreq, stream=42) & np.uint64(1)).astype(int)
    absf = (splitmix64(SERVING_SEED, nreq, stream=43) & np.uint64(1)).astype(int)
    return arr, lens, kind, desc, absf
