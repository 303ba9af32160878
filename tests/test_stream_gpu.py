"""GPU STREAM copy/scale/add/triad: f32 and int32 against the oracle
(bit-exact: each output is one IEEE operation or wrapping int op of its
inputs), and int32 against the reference's own CUDA kernels."""
import numpy as np
import pytest

from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("op", ["copy", "scale", "add", "triad"])
@pytest.mark.parametrize("n", [1, 3, 4, 5, 1023, 65536 + 7, (1 << 22) + 1])
def test_f32(cuda, edpp, orc, op, n):
    a = np.arange(n, dtype=np.float32)           # a[i] = i  (cuda/test_bandwidth.cu:59-62)
    b = (np.arange(n) + 10).astype(np.float32)   # b[i] = i + 10
    c = to_host(edpp.stream(op, to_dev(a), to_dev(b), 3.0))
    e, _ = orc.stream(op, a, b, 3.0)
    np.testing.assert_array_equal(c, e)


@pytest.mark.parametrize("op", ["copy", "scale", "add", "triad"])
def test_i32_wrapping_and_unaligned(cuda, edpp, orc, op):
    n = 100001
    a = edpp.gen_uniform_i32(n, 1, -2**31, 2**31 - 1)
    b = edpp.gen_uniform_i32(n, 2, -2**31, 2**31 - 1)
    c = to_host(edpp.stream(op, to_dev(a), to_dev(b), 3))
    e, _ = orc.stream(op, a, b, 3)
    np.testing.assert_array_equal(c, e)
    buf = cuda.zeros(n + 2, dtype=cuda.int32, device="cuda")
    buf[1:n + 1] = to_dev(a)
    c2 = to_host(edpp.stream(op, buf[1:n + 1], to_dev(b), 3))
    np.testing.assert_array_equal(c2, e)


@pytest.mark.parametrize("op", [0, 1, 2, 3])
def test_against_reference_cuda_kernels(cuda, edpp, orc, op):
    rc = orc.ref_cuda()
    if rc is None:
        pytest.skip("reference CUDA cubins not available on this machine")
    import ctypes
    n = 1 << 20
    a = edpp.gen_uniform_i32(n, 1, -2**31, 2**31 - 1)
    b = edpp.gen_uniform_i32(n, 2, -2**31, 2**31 - 1)
    ref = np.zeros(n, np.int32)
    P = lambda x: ctypes.c_void_p(x.ctypes.data)
    assert rc.refcu_stream_i32(op, P(a), P(b), P(ref), n) == 0
    name = ["copy", "scale", "add", "triad"][op]
    np.testing.assert_array_equal(to_host(edpp.stream(name, to_dev(a), to_dev(b), 3)), ref)


@pytest.mark.parametrize("op", ["copy", "scale", "add", "triad"])
def test_large_arrays_one_vector_per_thread(cuda, edpp, op):
    # 2^26 elements and more take the one-vector-per-thread kernel; a ragged
    # tail of 3 elements.  f32 copy/scale/add are single IEEE operations;
    # triad a + 3b is one fused multiply-add (as nvcc compiles the
    # reference's kernels), i.e. the exact value rounded once
    torch = cuda
    n = (1 << 26) + 3
    a = torch.arange(n, dtype=torch.float32, device="cuda")
    b = a + 10
    c = edpp.stream(op, a, b, 3.0)
    fused = (a.double() + b.double() * 3.0).float()
    want = {"copy": a, "scale": a * 3.0, "add": a + b, "triad": fused}[op]
    assert torch.equal(c, want)
    ai = torch.arange(n, dtype=torch.int32, device="cuda") * 7919
    bi = ai + 10
    ci = edpp.stream(op, ai, bi, 3)
    wi = {"copy": ai, "scale": ai * 3, "add": ai + bi, "triad": ai + bi * 3}[op]
    assert torch.equal(ci, wi)
