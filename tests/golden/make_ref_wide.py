"""Generate tests/golden/ref_wide.json: outputs of the reference's own sort (oracle/_ref, compiled
from Radixsortbidi8.hpp by `make -C oracle ref`) on seeded 16-byte keys.

Run where the reference tree exists:   python tests/golden/make_ref_wide.py
The keys are (n, 2) arrays of little-endian 64-bit words.  Kinds:
  x87   long double on x86-64 (x87 extended precision in 16 bytes, the upper 48 bits padding),
        through rsbd8::radixsortcopy<direction, native>(count, long double const*, long double*);
  w128  a 16-byte class under a forced mode (the reference's test128 with the mode bits of the
        call: forceunsigned, forcetieredabssigned, forcesigned, specialfloatingp, forcefloatingp).
Each case runs in fresh subprocesses.  The reference's 16-byte paths crash at random at every size
(a segmentation fault in roughly one run of six at n = 1000, most runs above 16k keys), so a case is
run up to eight times and is "ok" when at least two runs finished, every finished run returned the
same output, and that output is a permutation of the input; the sha256 of the output is stored
with the counts of finished and crashed runs.  "corrupt": a finished run returned something that
is not a permutation; "unstable": finished runs disagree; "crash": fewer than two runs finished.
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
OUT = os.path.join(HERE, "ref_wide.json")
DIRS = ["ascfwdorder", "dscfwdorder", "ascrevorder", "dscrevorder"]

# multiplatform/main.cpp:83-89: the seven longdoubletest128 values (garbage in the padding)
MAIN_X87 = [(0, 0xBBBBAAAAABABFFFF), (0, 0x22221111D0017FFF), (0x8000000000000000, 0x44443333EEEEFFFF),
            (0xFFFFFFFFFFFFFFFF, 0x6666555501017FFE), (0, 0x88887777FFF80001),
            (0xFFFFFFFFFFFFFFFF, 0xCCCC9999C7C80000), (1, 0xFFFFDDDDB3710000)]


def wide_input(gen: str, n: int, seed: int):
    """The (n, 2) uint64 input of a case (also used by the tests)."""
    import numpy as np
    from radixsortbidi8_gb300 import synth as S
    if gen == "main_x87":
        return np.array(MAIN_X87, dtype=np.uint64)
    lo = S.splitmix64(seed, n, stream=0)
    hi = S.splitmix64(seed, n, stream=1)
    cls = S.splitmix64(seed, n, stream=2) % np.uint64(100)
    if gen == "x87":
        pad = hi & np.uint64(0xFFFFFFFFFFFF0000)                    # random padding
        sign = (S.splitmix64(seed, n, stream=3) & np.uint64(1)) << np.uint64(15)
        exp = (hi & np.uint64(0x7FFF)) % np.uint64(0x7FFE) + np.uint64(1)
        exp = np.where(cls < 3, np.uint64(0), exp)                  # zeros and subnormals
        exp = np.where((cls >= 3) & (cls < 5), np.uint64(0x7FFF), exp)   # infinities and NaNs
        lo = np.where(cls == 0, np.uint64(0), lo)                   # +-0
        lo = np.where(cls == 3, np.uint64(0x8000000000000000), lo)  # +-inf
        hi = pad | sign | exp
    elif gen == "w128":
        hi = np.where(cls == 0, hi & np.uint64(0x8000000000000000), hi)   # +-0 in float modes
        lo = np.where(cls == 0, np.uint64(0), lo)
    else:
        raise ValueError(gen)
    a = np.stack([lo, hi], axis=1).astype(np.uint64)
    if n > 8:
        a[::7] = a[3]                                               # ties
    return a


def cases() -> list[dict]:
    cs = []
    for d in DIRS:
        cs.append(dict(kind="x87", mode="native", direction=d, n=7, gen="main_x87", seed=0))
        for n in (1000, 4097, 100003):
            cs.append(dict(kind="x87", mode="native", direction=d, n=n, gen="x87", seed=500 + n))
    for m in ("forceunsigned", "forcetieredabssigned", "forcesigned", "forcefloatingp"):
        for d in DIRS:
            for n in (1000, 50021):
                cs.append(dict(kind="w128", mode=m, direction=d, n=n, gen="w128", seed=700 + n))
    for d in DIRS:                      # inside-out float: sound at small sizes only
        cs.append(dict(kind="w128", mode="specialfloatingp", direction=d, n=3001, gen="w128", seed=9))
    for i, c in enumerate(cs):
        c["id"] = i
    return cs


def run_case(c: dict):
    import numpy as np
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    a = wide_input(c["gen"], c["n"], c["seed"])
    out = O.ref_sortcopy_wide(a, "x87" if c["kind"] == "x87" else "f128", c["mode"], c["direction"])
    key = lambda x: x[np.lexsort((x[:, 0], x[:, 1]))]
    return out.tobytes(), np.array_equal(key(out), key(a))


def _spawn(c: dict):
    try:
        r = subprocess.run([sys.executable, os.path.abspath(__file__), "--case", json.dumps(c)],
                           capture_output=True, text=True, timeout=60, cwd=ROOT)
    except subprocess.TimeoutExpired:
        return "hang", None
    if r.returncode != 0:
        return "crash", None
    sha, perm = r.stdout.strip().splitlines()[-1].split()
    return ("ok", sha) if perm == "1" else ("corrupt", None)


def main() -> None:
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    if not O.ref_available():
        O.build(ref=True)

    def attempt(c):
        shas, crashes = [], 0
        for _ in range(8):
            st, sha = _spawn(c)
            if st == "corrupt":
                return dict(c, status="corrupt")
            if st == "ok":
                shas.append(sha)
            else:
                crashes += 1
            if len(shas) >= 3:
                break
        if len(shas) < 2:
            return dict(c, status="crash", finished=len(shas), crashed=crashes)
        if len(set(shas)) != 1:
            return dict(c, status="unstable", finished=len(shas), crashed=crashes)
        return dict(c, status="ok", sha256=shas[0], finished=len(shas), crashed=crashes)

    cs = cases()
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        res = list(ex.map(attempt, cs))
    with open(OUT, "w") as f:
        json.dump({"generator": "tests/golden/make_ref_wide.py", "reference": "Radixsortbidi8.hpp (rsbd8)",
                   "cases": res}, f, indent=0)
    bad = [r for r in res if r["status"] != "ok"]
    print(f"{len(res)} cases, {len(bad)} not ok: " + ", ".join(f"{r['id']}:{r['status']}" for r in bad))


if __name__ == "__main__":
    if len(sys.argv) > 2 and sys.argv[1] == "--case":
        b, perm = run_case(json.loads(sys.argv[2]))
        print(hashlib.sha256(b).hexdigest(), int(bool(perm)))
    else:
        main()
