"""16-byte keys on the GPU: the reference-generated fixtures (tests/golden/ref_wide.json: x87 long
double in 16-byte storage and a 16-byte class under forced modes), every filter combination
against the oracle, tile edges, in place, through member indirection, and the argument checks."""
import hashlib
import json
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
pytestmark = pytest.mark.gpu
DIRS = ["ascfwdorder", "dscfwdorder", "ascrevorder", "dscrevorder"]


def _cases():
    with open(os.path.join(HERE, "golden", "ref_wide.json")) as f:
        return [c for c in json.load(f)["cases"] if c["status"] == "ok"]


def _dev(words):
    import torch
    return torch.from_numpy(np.ascontiguousarray(words).view(np.int64).reshape(-1)).cuda()


def _host(t):
    return t.cpu().numpy().view(np.uint64).reshape(-1, 2)


def _gpu_copy(words, kind, mode, direction):
    import torch
    import radixsortbidi8_gb300 as rs
    x = _dev(words)
    y = torch.empty_like(x)
    assert rs.radixsortcopy(x, y, direction, mode, key_dtype=kind)
    return _host(y)


@pytest.mark.parametrize("case", _cases(), ids=lambda c: f'{c["id"]}-{c["kind"]}-{c["mode"]}-{c["direction"]}-{c["n"]}')
def test_gpu_matches_reference_wide_golden(case):
    from make_ref_wide import wide_input
    a = wide_input(case["gen"], case["n"], case["seed"])
    got = _gpu_copy(a, "x87" if case["kind"] == "x87" else "f128", case["mode"], case["direction"])
    assert hashlib.sha256(got.tobytes()).hexdigest() == case["sha256"]


@pytest.mark.parametrize("kind", ["u128", "i128", "f128", "x87"])
@pytest.mark.parametrize("mode", ["native", "nativeabs", "nativetieredabs", 0, 1, 2, 3, 4, 5, 6, 7])
def test_gpu_wide_every_mode_matches_oracle(kind, mode):
    from make_ref_wide import wide_input
    a = wide_input("x87" if kind == "x87" else "w128", 30011, 17)
    for d in DIRS:
        assert np.array_equal(_gpu_copy(a, kind, mode, d), O.sortcopy_wide(a, kind, mode, d)), d


@pytest.mark.parametrize("n", [2, 3, 33, 4095, 4096, 4097, 8193, 65543])
def test_gpu_wide_tile_edges(n):
    from make_ref_wide import wide_input
    for kind, gen in (("x87", "x87"), ("f128", "w128")):
        a = wide_input(gen, n, n)
        assert np.array_equal(_gpu_copy(a, kind, "native", "dscrevorder"), O.sortcopy_wide(a, kind, "native", "dscrevorder"))


def test_gpu_wide_pass_skip_and_inplace():
    import torch
    import radixsortbidi8_gb300 as rs
    from make_ref_wide import wide_input
    # only the low 12 bits vary: 14 of the 16 digit passes are skipped
    a = np.zeros((100000, 2), np.uint64)
    a[:, 0] = wide_input("w128", 100000, 3)[:, 0] & np.uint64(0xFFF)
    assert np.array_equal(_gpu_copy(a, "u128", "native", "ascfwdorder"), O.sortcopy_wide(a, "u128"))
    b = wide_input("x87", 70001, 4)
    for d in DIRS:
        x = _dev(b)
        assert rs.radixsort(x, d, "native", key_dtype="x87")
        assert np.array_equal(_host(x), O.sortcopy_wide(b, "x87", "native", d)), d


@pytest.mark.parametrize("n", [50021, 1_900_003])
def test_gpu_wide_member_indirection(n):
    """32-byte records {u64 id; u64 pad; 16-byte key at byte 16}, sorted through object pointers
    (1.9 M records: enough 3072-pointer tiles for the pipelined pass)."""
    import torch
    import radixsortbidi8_gb300 as rs
    from make_ref_wide import wide_input
    keys = wide_input("x87", n, 8)
    rec = np.zeros((n, 4), np.uint64)
    rec[:, 0] = np.arange(n, dtype=np.uint64)
    rec[:, 2:] = keys
    raw = torch.from_numpy(rec.reshape(-1).view(np.int64).copy()).cuda()
    base = raw.data_ptr()
    ptrs = torch.arange(n, dtype=torch.int64, device="cuda") * 32 + base
    for d in DIRS:
        out = torch.empty_like(ptrs)
        assert rs.radixsortcopy_member(ptrs, out, "x87", 16, d)
        idx = (out.cpu().numpy() - base) // 32
        assert np.array_equal(idx, O.sort_indices_wide(keys, "x87", "native", d)), d


def test_gpu_wide_argument_checks():
    import torch
    import radixsortbidi8_gb300 as rs
    from radixsortbidi8_gb300 import api, batched
    x = torch.zeros(2 * 1001, dtype=torch.int64, device="cuda")
    y = torch.empty_like(x)
    with pytest.raises(api.RSBD8GError) as e:             # 8-byte aligned, not 16: refused
        rs.radixsortcopy(x[1:2001], y[1:2001], key_dtype="u128", count=1000)
    assert e.value.status == api.ERR_BAD_ARG
    offs = torch.tensor([0, 500, 1000], dtype=torch.int64, device="cuda")
    with pytest.raises(api.RSBD8GError):                   # x87 keys have no segmented form
        batched.segmented_scratch_bytes("x87", 1000, 2)
    nb = batched.segmented_scratch_bytes("u128", 1000, 2)  # 128-bit integers do
    scr = torch.empty(nb, dtype=torch.uint8, device="cuda")
    with pytest.raises(api.RSBD8GError) as e:             # but their arrays must be 16-byte aligned
        batched.segmented_sortcopy(x[1:2001], y[1:2001], torch.empty_like(y)[1:2001], offs, scr, key_dtype="u128")
    assert e.value.status == api.ERR_BAD_ARG


def test_gpu_wide_crowded_pass():
    """128-bit keys whose digit 1 is one value for ~70 % of them (warp ranking units under a crowded
    pass), at a size that runs the pipelined pass."""
    from make_ref_wide import wide_input
    from radixsortbidi8_gb300 import synth as S
    n = (1 << 21) + 13
    a = wide_input("w128", n, 31)
    pick = (S.splitmix64(17, n) % np.uint64(10)) < np.uint64(7)
    a[pick, 0] = (a[pick, 0] & ~np.uint64(0xFF00)) | np.uint64(0x5A00)
    for d in ("ascfwdorder", "dscrevorder"):
        assert np.array_equal(_gpu_copy(a, "i128", "native", d), O.sortcopy_wide(a, "i128", "native", d)), d
