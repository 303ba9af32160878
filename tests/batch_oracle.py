"""Expected outputs of a batch, segment by segment, from the oracle."""
import numpy as np

from oracle import oracle as orc

OP_SCAN, OP_SPLIT, OP_GATHER = 0, 1, 2


def reference_outputs(segs, in0, in1):
    n = len(in0)
    out0 = np.zeros(n, np.int32)
    out1 = np.zeros(n, np.int32)
    for s in segs:
        o, L, op = int(s["offset"]), int(s["length"]), int(s["op"])
        if L == 0:
            continue
        if op == OP_SCAN:
            out0[o:o + L] = orc.scan(in0[o:o + L])
        elif op == OP_SPLIT:
            k, v, _ = orc.split(in0[o:o + L], int(s["buckets"]), in1[o:o + L])
            out0[o:o + L], out1[o:o + L] = k, v
        else:
            out0[o:o + L] = orc.gather(in0[o:o + L], in1[o:o + L])
    return out0, out1
