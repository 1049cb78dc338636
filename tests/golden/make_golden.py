"""Generate tests/golden/ref_golden.json: outputs of the reference's own sort (oracle/_ref,
compiled from Radixsortbidi8.hpp by `make -C oracle ref`) on seeded inputs.

Run where the reference tree exists:   python tests/golden/make_golden.py
Each case runs three times, each time in a fresh subprocess, because the reference snapshot
has multithreading races: at some sizes it crashes or returns different orders from
run to run.  A case is recorded as
  "ok"        three runs agree and the output is a permutation of the input (a check that
              needs no sorting semantics; the sha256 of the output bytes is stored),
  "corrupt"   a run returned something that is not a permutation of the input,
  "crash"     a run died (signal / non-zero exit),
  "unstable"  the runs disagree,
  "hang"      a run did not finish within 60 s (the reference spins forever at some sizes).
Inputs are regenerated from (generator, seed, n) with radixsortbidi8_gb300.synth, so the
fixture stays small; outputs of n <= 64 are stored in full.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "ref_golden.json")

DIRS = ["ascfwdorder", "dscfwdorder", "ascrevorder", "dscrevorder"]
TYPES = ["uint8", "int8", "uint16", "int16", "uint32", "int32", "float32", "uint64", "int64", "float64"]


def make_input(gen: str, dtype: str, n: int, seed: int):
    """The input array of a case (also used by the tests)."""
    import numpy as np
    from radixsortbidi8_gb300 import synth as S
    dt = np.dtype(dtype)
    if gen == "mixed":
        a = S.float_specials(seed, n, dt) if dt.kind == "f" else S.uniform_bits(seed, n, dt)
        if n > 8:
            a[::7] = a[3]
        return a
    if gen == "uniform":
        return S.uniform_bits(seed, n, dt)
    if gen == "low12":
        return S.low_bits_u32(seed, n)
    if gen == "specials":
        return S.float_specials(seed, n, dt)
    raise ValueError(gen)


def cases() -> list[dict]:
    cs = []
    for t in TYPES:
        for d in DIRS:
            for n in (1000, (1 << 18) + 3):
                cs.append(dict(form="copy", dtype=t, mode="native", direction=d, n=n, gen="mixed", seed=1000 + n))
    for t, modes in (("uint16", (0, 1, 2, 6)), ("uint32", (1, 2, 6)), ("uint64", (1, 2, 6)),
                     ("int32", ("nativetieredabs",)), ("int64", ("nativetieredabs",))):
        for m in modes:
            for d in DIRS:
                cs.append(dict(form="copy", dtype=t, mode=m, direction=d, n=50021, gen="mixed", seed=7))
    for t in ("uint16", "uint32", "uint64"):          # inside-out float: sound at small sizes only
        for d in DIRS:
            cs.append(dict(form="copy", dtype=t, mode=4, direction=d, n=3001, gen="mixed", seed=8))
    for t in ("uint32", "float32", "int64", "float64", "uint16"):
        for d in DIRS:
            cs.append(dict(form="indirect8", dtype=t, mode="native", direction=d, n=100003, gen="mixed", seed=9))
    for d in DIRS:
        cs.append(dict(form="member", dtype="float64", mode="native", direction=d, n=100003, gen="records", seed=3))
    for t in ("uint32", "float32", "int64", "float64", "int16"):
        for d in DIRS:
            cs.append(dict(form="inplace", dtype=t, mode="native", direction=d, n=100003, gen="mixed", seed=11))
    cs.append(dict(form="copy", dtype="uint32", mode="native", direction="ascfwdorder", n=1 << 20,
                   gen="uniform", seed=0x5EED0001))
    cs.append(dict(form="copy", dtype="uint32", mode="native", direction="ascfwdorder", n=1 << 20,
                   gen="low12", seed=0x5EED0004))
    cs.append(dict(form="copy", dtype="float32", mode="native", direction="dscfwdorder", n=1 << 20,
                   gen="specials", seed=0x5EED0002))
    cs.append(dict(form="copy", dtype="int64", mode="native", direction="ascfwdorder", n=1 << 20,
                   gen="uniform", seed=0x5EED0003))
    for i, c in enumerate(cs):
        c["id"] = i
    return cs


def run_case(c: dict) -> bytes:
    """Worker: run one case through the reference; returns the output bytes (indices for indirection)."""
    import numpy as np
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    from radixsortbidi8_gb300 import synth as S
    if c["form"] in ("indirect8", "member"):
        n = c["n"]
        if c["gen"] == "records":
            rec = S.records24(c["seed"], n)
            buf = rec.view(np.uint8).reshape(n, 24).copy()
        else:
            keys = make_input("mixed", c["dtype"], n, c["seed"])
            buf = np.zeros((n, 24), np.uint8)
            kb = keys.dtype.itemsize
            buf[:, 8:8 + kb] = keys.view(np.uint8).reshape(n, kb)
        base = np.uint64(buf.ctypes.data)
        ptrs = base + np.arange(n, dtype=np.uint64) * np.uint64(24)
        out = O.ref_indirect(ptrs, c["dtype"], c["mode"], c["direction"], member=c["form"] == "member")
        idx = ((out - base) // np.uint64(24)).astype(np.uint64)
        perm = np.array_equal(np.sort(idx), np.arange(n, dtype=np.uint64))
        return idx.tobytes(), perm
    a = make_input(c["gen"], c["dtype"], c["n"], c["seed"])
    if c["form"] == "inplace":
        out = O.ref_inplace(a, c["mode"], c["direction"])
    else:
        out = O.ref_sortcopy(a, c["mode"], c["direction"])
    ut = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[a.dtype.itemsize]
    perm = np.array_equal(np.sort(out.view(ut)), np.sort(a.view(ut)))
    return out.tobytes(), perm


def _spawn(c: dict) -> tuple[str, str | None, str | None]:
    try:
        r = subprocess.run([sys.executable, os.path.abspath(__file__), "--case", json.dumps(c)],
                           capture_output=True, text=True, timeout=60, cwd=ROOT)
    except subprocess.TimeoutExpired:
        return "hang", None, None
    if r.returncode != 0:
        return "crash", None, None
    line = r.stdout.strip().splitlines()[-1]
    sha, perm, small = line.split(" ", 2)
    if perm != "1":
        return "corrupt", None, None
    return "ok", sha, (small if small != "-" else None)


def main() -> None:
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    if not O.ref_available():
        O.build(ref=True)
    cs = cases()

    def both(c):
        runs = []
        for _ in range(3):
            r = _spawn(c)
            if r[0] != "ok":
                return dict(c, status=r[0])
            runs.append(r)
        if len({r[1] for r in runs}) != 1:
            return dict(c, status="unstable")
        d = dict(c, status="ok", sha256=runs[0][1])
        if runs[0][2]:
            d["output_hex"] = runs[0][2]
        return d

    with cf.ThreadPoolExecutor(max_workers=4) as ex:
        res = list(ex.map(both, cs))
    # the reference races more under load: retry the failed cases one at a time
    for i, r in enumerate(res):
        if r["status"] != "ok":
            res[i] = both(cs[i])
    with open(OUT, "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "reference": "Radixsortbidi8.hpp (rsbd8)",
                   "cases": res}, f, indent=0)
    bad = [r for r in res if r["status"] != "ok"]
    print(f"{len(res)} cases, {len(bad)} not ok: " + ", ".join(f"{r['id']}:{r['status']}" for r in bad))


if __name__ == "__main__":
    if len(sys.argv) > 2 and sys.argv[1] == "--case":
        b, perm = run_case(json.loads(sys.argv[2]))
        print(hashlib.sha256(b).hexdigest(), int(bool(perm)), b.hex() if len(b) <= 64 * 8 else "-")
    else:
        main()
