"""Serving loop on the GPU: requests of mixed sizes, key types and modes submitted while others run
are admitted, coalesced and overlapped; every result is byte-identical to the same request
sorted alone (and to the oracle); a tight budget queues requests instead of failing them."""
import threading
import time

import numpy as np
import pytest

from conftest import empty_dev, from_dev, same_bits, to_dev
from oracle import oracle as O
from radixsortbidi8_gb300 import synth as S

pytestmark = [pytest.mark.gpu, pytest.mark.timeout(240)]

KINDS = [(np.uint16, "native", "ascfwdorder"), (np.int32, "nativeabs", "dscfwdorder"),
         (np.float32, "native", "dscfwdorder"), (np.float64, "nativeabs", "ascfwdorder"),
         (np.float32, "nativeabs", "ascfwdorder"), (np.int32, "native", "ascfwdorder")]


def _requests(n_req, seed, lo=1 << 4, hi=1 << 18):
    lens = S.log_uniform_lengths(seed, n_req, lo, hi)
    pick = (S.splitmix64(seed, n_req, stream=5) % np.uint64(len(KINDS))).astype(int)
    reqs = []
    for i in range(n_req):
        dt, mode, d = KINDS[pick[i]]
        dt = np.dtype(dt)
        a = S.float_specials(seed + i, int(lens[i]), dt) if dt.kind == "f" else S.uniform_bits(seed + i, int(lens[i]), dt)
        reqs.append((a, dt, mode, d))
    return reqs


def test_served_results_equal_alone_and_oracle():
    from radixsortbidi8_gb300 import serving, api
    reqs = _requests(300, 101)
    dev_in = [to_dev(a) for a, *_ in reqs]
    dev_out = [empty_dev(a.size, dt) for a, dt, *_ in reqs]
    with serving.Server(budget_bytes=2 << 30, max_inflight=4) as srv:
        # two submitting threads, so requests arrive while earlier batches are on the GPU
        ids = [None] * len(reqs)

        def submitter(k):
            for i in range(k, len(reqs), 2):
                a, dt, mode, d = reqs[i]
                ids[i] = srv.submit(dev_in[i], dev_out[i], d, mode, key_dtype=dt)
                if i % 16 == 0:
                    time.sleep(0.001)

        th = [threading.Thread(target=submitter, args=(k,)) for k in range(2)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        infos = [srv.wait(r) for r in ids]
        st = srv.stats()
    assert all(i.status == 0 for i in infos)
    assert st["completed"] == len(reqs)
    assert st["batches"] < len(reqs)            # requests were coalesced into shared launches
    assert st["max_coalesced"] > 1
    for i, (a, dt, mode, d) in enumerate(reqs):
        got = from_dev(dev_out[i], dt)
        alone = empty_dev(a.size, dt)
        import radixsortbidi8_gb300 as rs
        rs.radixsortcopy(dev_in[i], alone, d, mode, key_dtype=dt)
        assert same_bits(got, from_dev(alone, dt)), i
        assert same_bits(got, O.sortcopy(a, mode, d)), i
    del api


def test_tight_budget_queues_requests():
    from radixsortbidi8_gb300 import serving
    reqs = _requests(60, 202, lo=1 << 16, hi=1 << 19)
    dev_in = [to_dev(a) for a, *_ in reqs]
    dev_out = [empty_dev(a.size, dt) for a, dt, *_ in reqs]
    with serving.Server(budget_bytes=24 << 20, max_inflight=2) as srv:   # a few requests at a time
        ids = [srv.submit(dev_in[i], dev_out[i], d, mode, key_dtype=dt) for i, (a, dt, mode, d) in enumerate(reqs)]
        srv.drain()
        infos = [srv.wait(r) for r in ids]
        st = srv.stats()
    assert all(i.status == 0 for i in infos)
    assert st["arena_used"] == 0
    for i, (a, dt, mode, d) in enumerate(reqs):
        assert same_bits(from_dev(dev_out[i], dt), O.sortcopy(a, mode, d)), i


def test_request_larger_than_budget_refused():
    from radixsortbidi8_gb300 import serving, api
    a = S.uniform_bits(1, 1 << 22, np.uint32)
    x, y = to_dev(a), empty_dev(a.size, np.uint32)
    with serving.Server(budget_bytes=4 << 20, max_inflight=1) as srv:
        with pytest.raises(api.RSBD8GError) as e:
            srv.submit(x, y, key_dtype=np.uint32)
        assert e.value.status == api.ERR_BUSY


def test_sixteen_byte_keys_served_beside_other_requests():
    """128-bit integer and binary128-float keys (held as pairs of 64-bit words) submitted among
    4-byte requests: every result equals the oracle's sort of its input."""
    import torch
    from radixsortbidi8_gb300 import serving
    lens = S.log_uniform_lengths(303, 40, 1 << 4, 1 << 17)
    wide = [("u128", "native", "ascfwdorder"), ("i128", "native", "dscfwdorder"), ("f128", "nativeabs", "ascfwdorder")]
    reqs = []
    for i, m in enumerate(int(x) for x in lens):
        if i % 2:
            words = S.uniform_bits(400 + i, 2 * m, np.uint64)
            words[2::10] = words[0]
            words[3::10] = words[1]                  # repeated 128-bit keys
            reqs.append(("wide", words) + wide[i % 3])
        else:
            reqs.append(("narrow", S.uniform_bits(400 + i, m, np.uint32), np.uint32, "native", "dscfwdorder"))
    ins = [torch.from_numpy(r[1].view(np.int64 if r[0] == "wide" else np.int32).copy()).cuda() for r in reqs]
    outs = [torch.empty_like(x) for x in ins]
    with serving.Server(budget_bytes=1 << 30, max_inflight=4) as srv:
        ids = [srv.submit(ins[i], outs[i], r[4], r[3], key_dtype=r[2]) for i, r in enumerate(reqs)]
        srv.drain()
        infos = [srv.wait(q) for q in ids]
    assert all(x.status == 0 for x in infos)
    for i, r in enumerate(reqs):
        if r[0] == "wide":
            got = outs[i].cpu().numpy().view(np.uint64)
            assert same_bits(got, O.sortcopy_wide(r[1], r[2], r[3], r[4]).reshape(-1)), (i, r[2])
        else:
            assert same_bits(from_dev(outs[i], np.uint32), O.sortcopy(r[1], r[3], r[4])), i
