"""rsbd8g_prepare: every kernel a descriptor's sorts can launch is loaded ahead of the first sort.

Every key type and mode prepares without error (direct keys, member indirection, 16-byte and x87
keys), sorts after it equal the oracle, and a server (which prepares every key type and mode it
accepts when it is created) is created within a bound."""
import time

import numpy as np
import pytest

from conftest import empty_dev, from_dev, same_bits, to_dev
from oracle import oracle as O
from radixsortbidi8_gb300 import synth as S

pytestmark = pytest.mark.gpu

MODES = ["native", "nativeabs", "nativetieredabs", "forceunsigned", "forcesigned", "forceabssigned",
         "forcefloatingp", "forceabsfloatingp", "specialfloatingp", "forcetieredabsfloatingp", "forcetieredabssigned"]


def test_prepare_every_key_type_and_mode():
    from radixsortbidi8_gb300 import api
    for dt in (np.uint8, np.int16, np.uint32, np.float32, np.int64, np.float64, "u128", "i128", "f128", "x87"):
        for m in MODES:
            api.prepare(dt, "dscrevorder", m)
    for dt in (np.float32, np.int64):
        api.prepare(dt, "ascfwdorder", "native", indirection=api.MEMBER, offset1=8)


@pytest.mark.parametrize("dt,mode,direction", [(np.uint32, "native", "ascfwdorder"), (np.float64, "nativeabs", "dscrevorder"),
                                               (np.int16, "nativetieredabs", "dscfwdorder")],
                         ids=lambda x: str(getattr(x, "__name__", x)))
def test_sorts_after_prepare_match_oracle(dt, mode, direction):
    import radixsortbidi8_gb300 as rs
    from radixsortbidi8_gb300 import api
    api.prepare(dt, direction, mode)
    for n in (1000, (1 << 20) + 7):
        a = S.float_specials(n, n, dt) if np.dtype(dt).kind == "f" else S.uniform_bits(n, n, dt)
        x, y = to_dev(a), empty_dev(n, dt)
        assert rs.radixsortcopy(x, y, direction, mode, key_dtype=dt)
        assert same_bits(from_dev(y, dt), O.sortcopy(a, mode, direction))


def test_server_creation_prepares_within_a_bound():
    from radixsortbidi8_gb300 import serving
    t0 = time.perf_counter()
    with serving.Server(budget_bytes=256 << 20, max_inflight=2) as srv:
        created = time.perf_counter() - t0
        a = S.uniform_bits(3, 5000, np.uint16)
        x, y = to_dev(a), empty_dev(a.size, np.uint16)
        rid = srv.submit(x, y, "dscfwdorder", key_dtype=np.uint16)
        assert srv.wait(rid).status == 0
    assert same_bits(from_dev(y, np.uint16), O.sortcopy(a, "native", "dscfwdorder"))
    assert created < 30.0, created
