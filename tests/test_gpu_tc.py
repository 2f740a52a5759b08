"""cs_tc_update: the tensor-core block update C -= A B^T (tcgen05.mma, TMEM
accumulators) of the reduced-precision condensation, against numpy on the
same rounded operands (TF32: round to nearest, ties away, 10 mantissa bits;
BF16: round to nearest even, 7 bits).  The tensor core accumulates in FP32
in its own order: tolerance 4 K 2^-24 of sum |a| |b| per entry."""
import ctypes

import numpy as np
import pytest

from conftest import pkg

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def round_tf32(x):
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    return ((b + 0x1000) & 0xFFFFE000).astype(np.uint32).view(np.float32)


def round_bf16(x):
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    return ((b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000).astype(np.uint32).view(np.float32)


@pytest.mark.parametrize("prec", [1, 2])
@pytest.mark.parametrize("M,N,K", [(128, 16, 16), (1, 1, 1), (77, 257, 24), (200, 300, 64), (256, 512, 40),
                                   (129, 33, 7)])
def test_tensor_core_update_matches_numpy(prec, M, N, K):
    cs = pkg()
    lib = cs._lib.load()
    rng = np.random.default_rng(M * 1000 + N * 10 + K)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    C = rng.standard_normal((M, N)).astype(np.float32)
    dA, dB, dC = (torch.from_numpy(x).cuda() for x in (A, B, C))
    torch.cuda.synchronize()
    rc = lib.cs_tc_update(prec, M, N, K, ctypes.c_void_p(dA.data_ptr()), K, ctypes.c_void_p(dB.data_ptr()), K,
                          ctypes.c_void_p(dC.data_ptr()), N, None)
    assert rc == 0, cs._lib.last_error()
    got = dC.cpu().numpy().astype(np.float64)
    rnd = round_tf32 if prec == 1 else round_bf16
    Ar, Br = rnd(A).astype(np.float64), rnd(B).astype(np.float64)
    ref = C.astype(np.float64) - Ar @ Br.T
    bound = 4 * K * 2.0 ** -24 * (np.abs(Ar) @ np.abs(Br).T) + 2.0 ** -23 * np.abs(C)
    assert np.all(np.abs(got - ref) <= bound + 1e-30), np.abs(got - ref).max()


def test_tensor_core_update_rejects_bad_sizes():
    cs = pkg()
    lib = cs._lib.load()
    assert lib.cs_tc_update(3, 4, 4, 4, None, 4, None, 4, None, 4, None) == 1
    assert lib.cs_tc_update(2, 300, 4, 4, None, 4, None, 4, None, 4, None) == 1
    assert "M <= 256" in cs._lib.last_error()
