"""Batched segments: Python harness over the batch C ABI (include/edpp.h).

    segs = config5_segments()                    # 4096 uneven segments
    in0, in1 = gen_inputs(segs, seed=4)          # numpy, seeded
    plan = Plan(segs, tuning)                    # host planner (C++)
    ws = plan.workspace(device); plan.upload(ws)
    plan.launch(d_in0, d_in1, d_out0, d_out1, ws)   # one launch per tile kind
    run_plain(segs, ...)                         # one C-ABI call per segment

Segment table rows follow edpp_segment: offset, length, op, buckets.
"""
from __future__ import annotations

import ctypes
import json
import math
from pathlib import Path

import numpy as np

from . import _p, _torch, check, current_stream_handle, lib, workspace

SEG_DTYPE = np.dtype([("offset", "<i8"), ("length", "<i4"), ("op", "<i4"), ("buckets", "<i4"),
                      ("reserved", "<i4")])
assert SEG_DTYPE.itemsize == 24
OP_SCAN, OP_SPLIT, OP_GATHER = 0, 1, 2
OP_NAMES = {OP_SCAN: "scan", OP_SPLIT: "split", OP_GATHER: "gather"}
OP_BYTES = {OP_SCAN: 8, OP_SPLIT: 16, OP_GATHER: 12}  # algorithmic bytes per element
ALIGN = 64  # segment offsets in elements (256 bytes)
TUNING_TABLE = Path(__file__).resolve().parent.parent / "tuning" / "batch_gb300.json"


SCHEDULE_KINDS, SCHEDULE_QUEUE = 0, 1
SCHEDULE_NAMES = {SCHEDULE_KINDS: "kinds", SCHEDULE_QUEUE: "queue"}


class Tuning(ctypes.Structure):
    """edpp_batch_tuning: `schedule` KINDS (one launch per tile kind, the
    default) or QUEUE (one persistent work-queue launch, which the other
    three knobs tune)."""
    _fields_ = [("blocks_per_sm", ctypes.c_int32), ("split_defer_segments", ctypes.c_int32),
                ("largest_first", ctypes.c_int32), ("schedule", ctypes.c_int32)]

    def as_dict(self):
        return {"blocks_per_sm": self.blocks_per_sm,
                "split_defer_segments": self.split_defer_segments,
                "largest_first": self.largest_first,
                "schedule": SCHEDULE_NAMES.get(self.schedule, str(self.schedule))}

    @classmethod
    def from_dict(cls, d):
        sched = d.get("schedule", "kinds")
        sched = {v: k for k, v in SCHEDULE_NAMES.items()}.get(sched, sched)
        return cls(int(d["blocks_per_sm"]), int(d["split_defer_segments"]),
                   int(d["largest_first"]), int(sched))


def _draw(seed: int, i: int) -> int:
    return lib().edpp_gen_draw(seed, i)


def layout(lengths, ops, buckets=64) -> np.ndarray:
    """Segment table with offsets packed in order, each aligned to 64 elements."""
    segs = np.zeros(len(lengths), SEG_DTYPE)
    off = 0
    for i, (n, op) in enumerate(zip(lengths, ops)):
        segs[i] = (off, int(n), int(op), buckets if op == OP_SPLIT else 0, 0)
        off += (int(n) + ALIGN - 1) // ALIGN * ALIGN
    return segs


def config5_segments(num=4096, seed=4, lo_log2=10, hi_log2=24, cap=1 << 30, buckets=64):
    """4096 segments, sizes log-uniform in [2^10, 2^24] (draws of seed 4), op
    uniform over {scan, 64-bucket split, permutation gather} (seed 4 ^ 0xA5).

    Size rule: the raw sizes sum to about 7e9 > 2^30, so all sizes are
    multiplied by s = (cap - num * 1024) / sum, floored, and clamped to
    >= 1024; the total then stays <= cap (each clamp adds < 1024)."""
    raw = []
    for i in range(num):
        u = (_draw(seed, i) >> 11) * (1.0 / 9007199254740992.0)
        raw.append(int(2.0 ** (lo_log2 + (hi_log2 - lo_log2) * u)))
    total = sum(raw)
    if total > cap:
        s = (cap - num * 1024) / total
        sizes = [max(1024, int(math.floor(r * s))) for r in raw]
    else:
        sizes = raw
    ops = [_draw(seed ^ 0xA5, i) % 3 for i in range(num)]
    return layout(sizes, ops, buckets)


def array_length(segs) -> int:
    return int(segs["offset"].max() + segs["length"][segs["offset"].argmax()]) if len(segs) else 0


def algorithmic_bytes(segs) -> int:
    return int(sum(int(n) * OP_BYTES[int(op)] for n, op in zip(segs["length"], segs["op"])))


def gen_inputs(segs, seed=4):
    n = array_length(segs)
    in0 = np.zeros(n, np.int32)
    in1 = np.zeros(n, np.int32)
    segs = np.ascontiguousarray(segs)
    lib().edpp_gen_batch_inputs(ctypes.c_void_p(segs.ctypes.data), len(segs), seed,
                                ctypes.c_void_p(in0.ctypes.data), ctypes.c_void_p(in1.ctypes.data))
    return in0, in1


def size_class(segs) -> str:
    """Key of the tuning table: log2 of the total elements and of the mean."""
    tot = max(1, int(segs["length"].sum()))
    mean = max(1, tot // max(1, len(segs)))
    return f"total2^{tot.bit_length() - 1}_mean2^{mean.bit_length() - 1}"


def tuned(segs) -> Tuning | None:
    """The autotuner's choice for this size class, if the table has one."""
    if not TUNING_TABLE.exists():
        return None
    table = json.loads(TUNING_TABLE.read_text())
    e = table.get("classes", {}).get(size_class(segs))
    return Tuning.from_dict(e["tuning"]) if e else None


class Plan:
    def __init__(self, segs, tuning: Tuning | None = None):
        self.segs = np.ascontiguousarray(segs, dtype=SEG_DTYPE)
        self.tuning = tuning
        h = ctypes.c_void_p()
        tp = ctypes.byref(tuning) if tuning is not None else None
        check(lib().edpp_batch_plan_create(ctypes.c_void_p(self.segs.ctypes.data), len(self.segs),
                                           tp, ctypes.byref(h)), "batch_plan_create")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib().edpp_batch_plan_destroy(self.h)
            self.h = None

    @property
    def workspace_bytes(self) -> int:
        return lib().edpp_batch_plan_workspace_size(self.h)

    @property
    def num_tasks(self) -> int:
        return lib().edpp_batch_plan_num_tasks(self.h)

    def workspace(self, device=None):
        return workspace(self.workspace_bytes, device)

    def upload(self, ws):
        check(lib().edpp_batch_plan_upload(self.h, _p(ws), ws.numel(), current_stream_handle()),
              "batch_plan_upload")

    def launch(self, in0, in1, out0, out1, ws):
        check(lib().edpp_batch_launch(self.h, _p(in0), _p(in1), _p(out0), _p(out1), _p(ws),
                                      ws.numel(), current_stream_handle()), "batch_launch")


def plain_workspace(segs, device=None):
    segs = np.ascontiguousarray(segs, dtype=SEG_DTYPE)
    return workspace(lib().edpp_batch_plain_workspace_size(ctypes.c_void_p(segs.ctypes.data),
                                                           len(segs)), device)


def run_plain(segs, in0, in1, out0, out1, ws):
    segs = np.ascontiguousarray(segs, dtype=SEG_DTYPE)
    check(lib().edpp_batch_run_plain(ctypes.c_void_p(segs.ctypes.data), len(segs), _p(in0),
                                     _p(in1), _p(out0), _p(out1), _p(ws), ws.numel(),
                                     current_stream_handle()), "batch_run_plain")


def autotune(segs, in0, in1, out0, out1, ws, reps=3):
    """Run the native autotuner; returns (Tuning, ms)."""
    segs = np.ascontiguousarray(segs, dtype=SEG_DTYPE)
    best = Tuning()
    ms = ctypes.c_float()
    check(lib().edpp_batch_autotune(ctypes.c_void_p(segs.ctypes.data), len(segs), _p(in0), _p(in1),
                                    _p(out0), _p(out1), _p(ws), ws.numel(),
                                    current_stream_handle(), reps, ctypes.byref(best),
                                    ctypes.byref(ms)), "batch_autotune")
    return best, ms.value


def record_tuning(segs, tuning: Tuning, ms: float, extra=None):
    """Store the autotuner's choice for this size class in the tuning table."""
    TUNING_TABLE.parent.mkdir(parents=True, exist_ok=True)
    table = json.loads(TUNING_TABLE.read_text()) if TUNING_TABLE.exists() else {"classes": {}}
    table["classes"][size_class(segs)] = {"tuning": tuning.as_dict(), "ms": round(ms, 4),
                                          **(extra or {})}
    TUNING_TABLE.write_text(json.dumps(table, indent=1, sort_keys=True) + "\n")
