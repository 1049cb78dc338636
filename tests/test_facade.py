"""The C++ facade include/rsbd8.hpp: it compiles with the reference's call forms (CPU), and the
facade program runs the reference's known-answer cases on the GPU and writes random cases
that are compared with the oracle here."""
import json
import os
import sys
import shutil
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "facade_test.cpp")


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(nvcc))


def test_facade_compiles_with_reference_call_forms():
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    r = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-Wall", "-I", os.path.join(ROOT, "include"),
                        "-I", os.path.join(_cuda_home(), "include"), SRC], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


@pytest.mark.gpu
def test_facade_program_on_gpu(tmp_path):
    import radixsortbidi8_gb300 as rs
    lib = rs.api.library_path()
    rs.lib()
    exe = str(tmp_path / "facade_test")
    nvcc = os.path.join(_cuda_home(), "bin", "nvcc")
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
                        lib, f"-Xlinker=-rpath={os.path.dirname(lib)}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([exe, str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "PASS" in r.stdout, r.stdout + r.stderr
    f = np.fromfile(out / "f32_in.bin", dtype=np.float32)
    got = np.fromfile(out / "f32_nativeabs_dscrevorder.bin", dtype=np.float32)
    assert np.array_equal(got.view(np.uint32), O.sortcopy(f, "nativeabs", "dscrevorder").view(np.uint32))
    got = np.fromfile(out / "f32_native_ascrevorder_movetobuffer.bin", dtype=np.float32)
    assert np.array_equal(got.view(np.uint32), O.sortcopy(f, "native", "ascrevorder").view(np.uint32))
    keys = np.fromfile(out / "rec_keys.bin", dtype=np.float64)
    idx = np.fromfile(out / "rec_member_dscfwdorder_idx.bin", dtype=np.uint64)
    assert np.array_equal(idx.astype(np.int64), O.numpy_sort_indices(keys, "native", "dscfwdorder"))
    # the indexed / offset indirection forms give the reference's own orders
    with open(os.path.join(ROOT, "tests", "golden", "ref_forms.json")) as f:
        want = json.load(f)["forms"]
    got = {}
    for line in (out / "forms.txt").read_text().splitlines():
        name, _, rest = line.partition(":")
        got[name] = [int(x) for x in rest.split()]
    assert got == want


def test_ref_forms_fixture_matches_reference_binary():
    """tests/golden/ref_forms.json is what the reference itself prints (where it was built here)."""
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_forms")
    if not os.path.exists(exe):
        pytest.skip("oracle/_ref/ref_forms not built (the reference tree is absent)")
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from make_ref_forms import parse
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    with open(os.path.join(ROOT, "tests", "golden", "ref_forms.json")) as f:
        assert parse(out) == json.load(f)["forms"]
    assert "all calls returned true: 1" in out
