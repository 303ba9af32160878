"""Host side of the batched form: the config-5 segment table, the planner,
and its argument checks (no GPU)."""
import ctypes

import numpy as np
import pytest


@pytest.fixture(scope="module")
def batch(edpp):
    from edpp import batch as b
    return b


def test_config5_segments(batch):
    segs = batch.config5_segments()
    assert len(segs) == 4096
    L = segs["length"].astype(np.int64)
    assert L.min() >= 1024 and L.sum() <= 1 << 30
    assert L.sum() > 0.99 * (1 << 30) - 4096 * 1024  # the cap is used
    assert set(np.unique(segs["op"])) == {0, 1, 2}
    assert np.all(segs["offset"] % 64 == 0)
    assert np.all(np.diff(segs["offset"]) >= L[:-1])  # no overlap
    assert np.all(segs["buckets"][segs["op"] == 1] == 64)
    # log-uniform before scaling: sizes span ~ 4 decades
    assert L.max() / L.min() > 1000
    np.testing.assert_array_equal(segs, batch.config5_segments())  # deterministic


def test_plan_tasks_and_workspace(batch):
    segs = batch.layout([1, 4096, 4097, 100000, 0, 5000], [0, 1, 2, 1, 0, 2])
    plan = batch.Plan(segs)
    tiles = [1, 1, 2, 25, 0, 2]
    # split segments have a HIST and a SPLIT task per tile
    expect = sum(t * (2 if op == 1 else 1) for t, op in zip(tiles, [0, 1, 2, 1, 0, 2]))
    assert plan.num_tasks == expect
    assert plan.workspace_bytes > 0
    for tu in (batch.Tuning(2, 0, 0, 0), batch.Tuning(8, 4, 1, 0), batch.Tuning(2, 0, 0, 1),
               batch.Tuning(8, 4, 1, 1)):
        p2 = batch.Plan(segs, tu)
        assert p2.num_tasks == expect and p2.workspace_bytes == plan.workspace_bytes


def test_plan_rejects_bad_schedule(batch, edpp):
    segs = batch.layout([4096], [0])
    h = ctypes.c_void_p()
    tu = batch.Tuning(2, 0, 0, 7)
    assert edpp.lib().edpp_batch_plan_create(ctypes.c_void_p(segs.ctypes.data), 1, ctypes.byref(tu),
                                             ctypes.byref(h)) == edpp.EDPP_EINVAL
    assert batch.Tuning.from_dict({"blocks_per_sm": 3, "split_defer_segments": 4,
                                   "largest_first": 1}).schedule == batch.SCHEDULE_KINDS
    assert batch.Tuning.from_dict(batch.Tuning(3, 4, 1, 1).as_dict()).schedule == batch.SCHEDULE_QUEUE


def test_plan_rejects_bad_segments(batch, edpp):
    lib = edpp.lib()
    for bad in ([(0, 10, 7, 0, 0)], [(0, 10, 1, 3, 0)], [(0, 10, 1, 512, 0)], [(0, -1, 0, 0, 0)]):
        segs = np.array(bad, batch.SEG_DTYPE)
        h = ctypes.c_void_p()
        assert lib.edpp_batch_plan_create(ctypes.c_void_p(segs.ctypes.data), 1, None,
                                          ctypes.byref(h)) == edpp.EDPP_EINVAL


def test_inputs_deterministic(batch):
    segs = batch.layout([3000, 5000, 7000], [0, 1, 2])
    a0, a1 = batch.gen_inputs(segs, seed=4)
    b0, b1 = batch.gen_inputs(segs, seed=4)
    np.testing.assert_array_equal(a0, b0)
    np.testing.assert_array_equal(a1, b1)
    g = segs[2]
    idx = a1[g["offset"]:g["offset"] + g["length"]]
    assert np.array_equal(np.sort(idx), np.arange(g["length"], dtype=np.int32))
    sc = a0[:3000]
    assert sc.min() >= 0 and sc.max() <= 100


def test_launch_rejects_missing_value_arrays(batch, edpp):
    """Gather tiles read in1 and split tiles read in1 and write out1: a NULL
    for either is an argument error, returned before any device work (the
    pointers below are never dereferenced)."""
    lib = edpp.lib()
    fake = ctypes.c_void_p(256)
    nul = ctypes.c_void_p(0)
    for ops, need_in1, need_out1 in (([0], False, False), ([2], True, False),
                                     ([1], True, True), ([0, 2, 1], True, True)):
        segs = batch.layout([5000] * len(ops), ops)
        plan = batch.Plan(segs)
        wsb = plan.workspace_bytes
        tu = batch.Tuning()
        best_ms = ctypes.c_float()
        sp = ctypes.c_void_p(segs.ctypes.data)
        for in1, out1 in ((nul, fake), (fake, nul)):
            expect_bad = (in1.value is None and need_in1) or (out1.value is None and need_out1)
            if not expect_bad:
                continue
            assert lib.edpp_batch_launch(plan.h, fake, in1, fake, out1, fake, wsb,
                                         nul) == edpp.EDPP_EINVAL
            assert lib.edpp_batch_run_plain(sp, len(segs), fake, in1, fake, out1, fake, 1 << 30,
                                            nul) == edpp.EDPP_EINVAL
            assert lib.edpp_batch_autotune(sp, len(segs), fake, in1, fake, out1, fake, wsb, nul,
                                           1, ctypes.byref(tu),
                                           ctypes.byref(best_ms)) == edpp.EDPP_EINVAL
    # scan-only batches need neither
    segs = batch.layout([5000], [0])
    assert lib.edpp_batch_run_plain(ctypes.c_void_p(segs.ctypes.data), 1, nul, nul, nul, nul,
                                    fake, 1 << 30, nul) == edpp.EDPP_EINVAL  # in0/out0 missing
