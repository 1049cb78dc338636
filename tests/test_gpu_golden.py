"""The GPU sort against the reference itself: every reference-generated golden case
(tests/golden/ref_golden.json, outputs of Radixsortbidi8.hpp's own radixsortcopy / radixsort on
seeded inputs) is recomputed on the GPU through the C ABI and compared by SHA-256."""
import hashlib
import json
import os
import sys

import numpy as np
import pytest

from conftest import empty_dev, from_dev, to_dev

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
pytestmark = pytest.mark.gpu


def _cases():
    p = os.path.join(HERE, "golden", "ref_golden.json")
    if not os.path.exists(p):
        return []
    with open(p) as f:
        return [c for c in json.load(f)["cases"] if c["status"] == "ok"]


@pytest.mark.parametrize("case", _cases(), ids=lambda c: f'{c["id"]}-{c["form"]}-{c["dtype"]}-{c["direction"]}')
def test_gpu_matches_reference_golden(case):
    import torch
    import radixsortbidi8_gb300 as rs
    from make_golden import make_input
    from radixsortbidi8_gb300 import synth as S
    c = case
    if c["form"] in ("indirect8", "member"):
        n = c["n"]
        if c["gen"] == "records":
            buf = S.records24(c["seed"], n).view(np.uint8).reshape(n, 24).copy()
        else:
            keys = make_input("mixed", c["dtype"], n, c["seed"])
            buf = np.zeros((n, 24), np.uint8)
            kb = keys.dtype.itemsize
            buf[:, 8:8 + kb] = keys.view(np.uint8).reshape(n, kb)
        raw = torch.from_numpy(buf.reshape(-1).copy()).cuda()
        base = raw.data_ptr()
        ptrs = torch.arange(n, dtype=torch.int64, device="cuda") * 24 + base
        out = torch.empty_like(ptrs)
        assert rs.radixsortcopy_member(ptrs, out, np.dtype(c["dtype"]), 8, c["direction"], c["mode"])
        got = ((out.cpu().numpy() - base) // 24).astype(np.uint64).tobytes()
    else:
        a = make_input(c["gen"], c["dtype"], c["n"], c["seed"])
        if c["form"] == "inplace":
            t = to_dev(a)
            assert rs.radixsort(t, c["direction"], c["mode"], key_dtype=a.dtype)
            got = from_dev(t, a.dtype).tobytes()
        else:
            inp, out = to_dev(a), empty_dev(a.size, a.dtype)
            assert rs.radixsortcopy(inp, out, c["direction"], c["mode"], key_dtype=a.dtype)
            got = from_dev(out, a.dtype).tobytes()
    assert hashlib.sha256(got).hexdigest() == c["sha256"]
