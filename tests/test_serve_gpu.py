"""The continuous-batching server: every request's result is the same
whether it runs alone or in a mix with others admitted while it runs, and
equals the oracle; admission waits for pool memory instead of failing."""
import threading
import time

import numpy as np
import pytest

from batch_oracle import reference_outputs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def serve(edpp):
    from edpp import serve as s
    return s


def _requests(edpp, serve, sizes, seed):
    from edpp import batch as B
    ops = [i % 3 for i in range(len(sizes))]
    segs = B.layout(sizes, ops, buckets=64)
    in0, in1 = B.gen_inputs(segs, seed=seed)
    reqs = []
    for s in segs:
        o, L, op = int(s["offset"]), int(s["length"]), int(s["op"])
        a0 = serve.pinned_empty(L)
        a1 = serve.pinned_empty(L)
        a0[:] = in0[o:o + L]
        a1[:] = in1[o:o + L]
        reqs.append((op, a0, a1))
    return segs, in0, in1, reqs


def _run(srv, serve, reqs, concurrent):
    outs = [(serve.pinned_empty(len(a0)), serve.pinned_empty(len(a0))) for _, a0, _ in reqs]
    for o0, o1 in outs:
        o0[:] = 0
        o1[:] = 0
    timings = []
    if not concurrent:
        for (op, a0, a1), (o0, o1) in zip(reqs, outs):
            rid = srv.submit(op, a0, a1, o0, o1, buckets=64)
            st, t = srv.wait(rid)
            assert st == 0
            timings.append(t.latency_ms)
        return outs, timings
    # two client threads submitting with small random gaps
    ids = [None] * len(reqs)

    def client(k):
        rng = np.random.default_rng(k)
        for i in range(k, len(reqs), 2):
            op, a0, a1 = reqs[i]
            ids[i] = srv.submit(op, a0, a1, outs[i][0], outs[i][1], buckets=64)
            time.sleep(float(rng.exponential(0.0005)))

    ts = [threading.Thread(target=client, args=(k,)) for k in range(2)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    for rid in ids:
        st, t = srv.wait(rid)
        assert st == 0
        timings.append(t.latency_ms)
    return outs, timings


@pytest.mark.parametrize("schedule", [0, 1])  # batches as KINDS launches / one QUEUE launch
def test_alone_equals_mix_equals_oracle(cuda, edpp, serve, schedule):
    sizes = [4096, 1, 777, 100003, 1 << 20, 3 << 18, 65536, 4097, 250000, 12345] * 4
    segs, in0, in1, reqs = _requests(edpp, serve, sizes, seed=21)
    e0, e1 = reference_outputs(segs, in0, in1)
    tu = serve.Tuning(3, 1, 1, schedule)
    with serve.Server(pool_bytes=256 << 20, slots=3, tuning=tu) as srv:
        alone, _ = _run(srv, serve, reqs, concurrent=False)
        mix3, _ = _run(srv, serve, reqs, concurrent=True)
        assert srv.stats()["completed"] == 2 * len(reqs)
    # one slot: requests arriving while a batch runs queue up and are
    # admitted together into the next batch
    with serve.Server(pool_bytes=256 << 20, slots=1, tuning=tu) as srv:
        mix, lat = _run(srv, serve, reqs, concurrent=True)
        stats = srv.stats()
    for i in range(len(reqs)):
        np.testing.assert_array_equal(mix3[i][0], mix[i][0])
        np.testing.assert_array_equal(mix3[i][1], mix[i][1])
    for i, s in enumerate(segs):
        o, L, op = int(s["offset"]), int(s["length"]), int(s["op"])
        np.testing.assert_array_equal(alone[i][0], mix[i][0])
        np.testing.assert_array_equal(alone[i][0], e0[o:o + L])
        if op == 1:
            np.testing.assert_array_equal(alone[i][1], mix[i][1])
            np.testing.assert_array_equal(alone[i][1], e1[o:o + L])
    assert all(x > 0 for x in lat)
    assert stats["completed"] == len(reqs)
    assert stats["max_requests_per_batch"] > 1  # requests were batched together


def test_admission_waits_for_memory(cuda, edpp, serve):
    # a pool that holds about two of these requests at once: the rest wait
    sizes = [1 << 20] * 12
    segs, in0, in1, reqs = _requests(edpp, serve, sizes, seed=22)
    e0, e1 = reference_outputs(segs, in0, in1)
    with serve.Server(pool_bytes=2 * 16 * (1 << 20) + (1 << 20), slots=4) as srv:
        mix, _ = _run(srv, serve, reqs, concurrent=True)
        stats = srv.stats()
        assert stats["max_pool_bytes_used"] <= 2 * 16 * (1 << 20) + (1 << 20)
        # a request larger than the whole pool is refused up front
        big = serve.pinned_empty(64 << 20)
        with pytest.raises(edpp.EdppError):
            srv.submit(0, big, None, big)
    for i, s in enumerate(segs):
        o, L = int(s["offset"]), int(s["length"])
        np.testing.assert_array_equal(mix[i][0], e0[o:o + L])


def test_batches_overlap_in_flight(cuda, edpp, serve):
    """With one request per batch and four slots, requests submitted together
    run as several batches on separate streams at once (their copies and
    kernels can overlap on the device), and each result still equals the
    oracle."""
    sizes = [1 << 22] * 8
    segs, in0, in1, reqs = _requests(edpp, serve, sizes, seed=23)
    e0, e1 = reference_outputs(segs, in0, in1)
    with serve.Server(pool_bytes=1 << 30, slots=4, max_batch_requests=1) as srv:
        outs = [(serve.pinned_empty(len(a0)), serve.pinned_empty(len(a0))) for _, a0, _ in reqs]
        ids = [srv.submit(op, a0, a1, o0, o1, buckets=64)
               for (op, a0, a1), (o0, o1) in zip(reqs, outs)]
        for rid in ids:
            st, _ = srv.wait(rid)
            assert st == 0
        stats = srv.stats()
    assert stats["batches"] == len(reqs)
    assert stats["max_batches_in_flight"] > 1, stats
    for i, s in enumerate(segs):
        o, L, op = int(s["offset"]), int(s["length"]), int(s["op"])
        np.testing.assert_array_equal(outs[i][0], e0[o:o + L])
        if op == 1:
            np.testing.assert_array_equal(outs[i][1], e1[o:o + L])
