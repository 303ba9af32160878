"""The batched form against the oracle (bit-exact) and against the plain
per-segment C-ABI calls, including the 4096-segment workload and CUDA-graph
replay, under both schedules: KINDS (one launch per tile kind) and QUEUE (one
persistent work-queue launch)."""
import numpy as np
import pytest

from batch_oracle import reference_outputs
from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch(edpp):
    from edpp import batch as b
    return b


def _run_batch(batch, cuda, segs, in0, in1, tuning=None):
    n = len(in0)
    d0, d1 = to_dev(in0), to_dev(in1)
    o0 = cuda.zeros(n, dtype=cuda.int32, device="cuda")
    o1 = cuda.zeros(n, dtype=cuda.int32, device="cuda")
    plan = batch.Plan(segs, tuning)
    ws = plan.workspace("cuda")
    plan.upload(ws)
    plan.launch(d0, d1, o0, o1, ws)
    return o0, o1, (plan, ws, d0, d1)


def _mask_unused(segs, a0, a1):
    """Zero the alignment gaps and out1 of non-split segments (not written)."""
    m0 = np.zeros(len(a0), bool)
    m1 = np.zeros(len(a0), bool)
    for s in segs:
        o, L = int(s["offset"]), int(s["length"])
        m0[o:o + L] = True
        if int(s["op"]) == 1:
            m1[o:o + L] = True
    return np.where(m0, a0, 0), np.where(m1, a1, 0)


SIZES = [1, 2, 31, 4095, 4096, 4097, 8192, 12289, 100003, 1 << 18]


@pytest.mark.parametrize("tuning", [None, (0, 0, 0, 0), (2, 0, 0, 1), (8, 4, 1, 1)])
def test_mixed_small_batch_vs_oracle(cuda, edpp, batch, tuning):
    sizes = SIZES * 3
    ops = [i % 3 for i in range(len(sizes))]
    segs = batch.layout(sizes, ops, buckets=64)
    in0, in1 = batch.gen_inputs(segs, seed=11)
    tu = batch.Tuning(*tuning) if tuning else None
    o0, o1, _ = _run_batch(batch, cuda, segs, in0, in1, tu)
    assert edpp.sync_status() == edpp.EDPP_OK
    e0, e1 = reference_outputs(segs, in0, in1)
    g0, g1 = _mask_unused(segs, to_host(o0), to_host(o1))
    np.testing.assert_array_equal(g0, e0)
    np.testing.assert_array_equal(g1, e1)


@pytest.mark.parametrize("schedule", [0, 1])
@pytest.mark.parametrize("buckets", [1, 2, 16, 64, 256])
def test_split_bucket_counts(cuda, edpp, batch, buckets, schedule):
    segs = batch.layout([70001, 4096, 9000], [1, 1, 1], buckets=buckets)
    in0, in1 = batch.gen_inputs(segs, seed=12)
    o0, o1, _ = _run_batch(batch, cuda, segs, in0, in1, batch.Tuning(3, 1, 1, schedule))
    e0, e1 = reference_outputs(segs, in0, in1)
    g0, g1 = _mask_unused(segs, to_host(o0), to_host(o1))
    np.testing.assert_array_equal(g0, e0)
    np.testing.assert_array_equal(g1, e1)


@pytest.mark.parametrize("schedule", [0, 1])
def test_unaligned_segment_offsets(cuda, edpp, batch, schedule):
    # offsets that are not multiples of 4 elements: the bulk-copy path is off
    segs = batch.layout([5000, 7001, 9003], [0, 1, 2])
    segs["offset"] += np.array([1, 3, 2])
    in0, in1 = batch.gen_inputs(segs, seed=13)
    o0, o1, _ = _run_batch(batch, cuda, segs, in0, in1, batch.Tuning(3, 1, 1, schedule))
    e0, e1 = reference_outputs(segs, in0, in1)
    g0, g1 = _mask_unused(segs, to_host(o0), to_host(o1))
    np.testing.assert_array_equal(g0, e0)
    np.testing.assert_array_equal(g1, e1)


def test_config5_batch_equals_plain_and_graph_replay(cuda, edpp, batch):
    segs = batch.config5_segments()
    in0, in1 = batch.gen_inputs(segs, seed=4)
    o0, o1, (plan, ws, d0, d1) = _run_batch(batch, cuda, segs, in0, in1)
    assert edpp.sync_status() == edpp.EDPP_OK
    n = len(in0)
    p0 = cuda.zeros(n, dtype=cuda.int32, device="cuda")
    p1 = cuda.zeros(n, dtype=cuda.int32, device="cuda")
    pws = batch.plain_workspace(segs, "cuda")
    batch.run_plain(segs, d0, d1, p0, p1, pws)
    assert edpp.sync_status() == edpp.EDPP_OK
    assert cuda.equal(o0, p0) and cuda.equal(o1, p1)
    # the work-queue schedule gives the same arrays
    r0, r1, _ = _run_batch(batch, cuda, segs, in0, in1, batch.Tuning(3, 4, 1, 1))
    assert edpp.sync_status() == edpp.EDPP_OK
    assert cuda.equal(r0, p0) and cuda.equal(r1, p1)
    del r0, r1
    # spot-check some segments of every op against the oracle
    pick = [i for op in (0, 1, 2) for i in np.nonzero(segs["op"] == op)[0][:3]]
    sub = segs[pick]
    e0, e1 = reference_outputs(sub, in0, in1)
    h0, h1 = to_host(o0), to_host(o1)
    for s in sub:
        o, L = int(s["offset"]), int(s["length"])
        np.testing.assert_array_equal(h0[o:o + L], e0[o:o + L])
        if int(s["op"]) == 1:
            np.testing.assert_array_equal(h1[o:o + L], e1[o:o + L])
    # CUDA graph: capture one launch, replay twice, same results
    g = cuda.cuda.CUDAGraph()
    q0 = cuda.zeros_like(o0)
    q1 = cuda.zeros_like(o1)
    s = cuda.cuda.Stream()
    s.wait_stream(cuda.cuda.current_stream())
    with cuda.cuda.stream(s):
        with cuda.cuda.graph(g):
            plan.launch(d0, d1, q0, q1, ws)
    cuda.cuda.current_stream().wait_stream(s)
    for _ in range(2):
        q0.zero_()
        q1.zero_()
        g.replay()
        cuda.cuda.synchronize()
        assert cuda.equal(q0, o0) and cuda.equal(q1, o1)
    assert edpp.sync_status() == edpp.EDPP_OK


@pytest.mark.parametrize("seed", [101, 102, 103])
def test_random_segment_tables_every_schedule(cuda, edpp, batch, seed):
    # 300 segments of 0..131072 elements, random ops and split bucket counts,
    # random gaps between segments (so some start off a 16-byte boundary);
    # every schedule gives the oracle's arrays
    rng = np.random.default_rng(seed)
    num = 300
    lengths = (2.0 ** rng.uniform(0, 17, num)).astype(np.int64)
    lengths[rng.random(num) < 0.05] = 0
    ops = rng.integers(0, 3, num)
    segs = np.zeros(num, batch.SEG_DTYPE)
    off = 0
    for i in range(num):
        off += int(rng.integers(0, 6))
        b = int(2 ** rng.integers(0, 9)) if ops[i] == 1 else 0
        segs[i] = (off, int(lengths[i]), int(ops[i]), b, 0)
        off += int(lengths[i])
    in0, in1 = batch.gen_inputs(segs, seed=seed)
    e0, e1 = reference_outputs(segs, in0, in1)
    for tu in (None, batch.Tuning(0, 0, 0, 0), batch.Tuning(2, 0, 1, 1), batch.Tuning(3, 2, 0, 1)):
        o0, o1, _ = _run_batch(batch, cuda, segs, in0, in1, tu)
        assert edpp.sync_status() == edpp.EDPP_OK
        g0, g1 = _mask_unused(segs, to_host(o0), to_host(o1))
        np.testing.assert_array_equal(g0, e0)
        np.testing.assert_array_equal(g1, e1)


@pytest.mark.parametrize("buckets", [4, 16, 64, 256])
def test_split_segments_with_one_bucket(cuda, edpp, batch, buckets):
    # every key of every split segment falls in the last bucket (the
    # ranking's same-address case): each segment keeps its input order
    sizes = [1, 33, 4096, 4097, 20000, 70001]
    segs = batch.layout(sizes, [1] * len(sizes), buckets=buckets)
    in0, in1 = batch.gen_inputs(segs, seed=21)
    in0 = (in0 * buckets + (buckets - 1)).astype(np.int32)
    e0, e1 = reference_outputs(segs, in0, in1)
    for s in segs:
        o, L = int(s["offset"]), int(s["length"])
        np.testing.assert_array_equal(e0[o:o + L], in0[o:o + L])
    for tu in (None, batch.Tuning(3, 4, 1, 1)):
        o0, o1, _ = _run_batch(batch, cuda, segs, in0, in1, tu)
        assert edpp.sync_status() == edpp.EDPP_OK
        g0, g1 = _mask_unused(segs, to_host(o0), to_host(o1))
        np.testing.assert_array_equal(g0, _mask_unused(segs, e0, e1)[0])
        np.testing.assert_array_equal(g1, _mask_unused(segs, e0, e1)[1])
