"""The learned preconditioner's node update on the tcgen05 tensor cores
(mba_gnn_gemm: Z = A W^T + A2 W2^T + bias, H = bf16(relu(Z))) against an
FP32 product of the same BF16 operands in numpy.  Bars: Z within the FP32
accumulation error (1e-5 relative to the sum of |products| of the row);
H equal to numpy's round-to-nearest-even BF16 of relu(Z) from the device Z.
Sizes cover a partial last tile, a single row and several tiles."""
import ctypes

import numpy as np
import pytest

from maplab_gb300 import _native as N
from maplab_gb300 import ba

pytestmark = pytest.mark.gpu


def to_bf16(x):
    """float32 -> bf16 bit patterns, round to nearest even."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((u >> 16) & 1) + 0x7FFF
    return ((u + r) >> 16).astype(np.uint16)


def from_bf16(b):
    return (b.astype(np.uint32) << 16).view(np.float32)


def _ptr16(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16))


@pytest.mark.parametrize("k", [32, 64])
@pytest.mark.parametrize("n, two, with_bias", [(1, True, True), (127, True, True), (128, False, True),
                                               (1000, True, False), (20011, True, True)])
def test_tensor_core_node_update_matches_fp32(k, n, two, with_bias):
    rng = np.random.default_rng(n * 7 + k)
    A = to_bf16(rng.normal(size=(n, k)))
    W = to_bf16(rng.normal(scale=0.2, size=(64, k)))
    A2 = to_bf16(rng.normal(size=(n, k))) if two else None
    W2 = to_bf16(rng.normal(scale=0.2, size=(64, k))) if two else None
    bias = rng.normal(size=64).astype(np.float32) if with_bias else None
    Z = np.zeros((n, 64), dtype=np.float32)
    H = np.zeros((n, 64), dtype=np.uint16)
    st = ba.lib().mba_gnn_gemm(0, n, k, _ptr16(A), _ptr16(W), _ptr16(A2), _ptr16(W2),
                               None if bias is None else bias.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                               Z.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), _ptr16(H))
    assert st == N.MBA_OK, st
    a, w = from_bf16(A).astype(np.float64), from_bf16(W).astype(np.float64)
    ref = a @ w.T
    mag = np.abs(a) @ np.abs(w).T
    if two:
        a2, w2 = from_bf16(A2).astype(np.float64), from_bf16(W2).astype(np.float64)
        ref += a2 @ w2.T
        mag += np.abs(a2) @ np.abs(w2).T
    if bias is not None:
        ref += bias
        mag += np.abs(bias)
    err = np.abs(Z - ref) / np.maximum(mag, 1e-30)
    assert err.max() <= 1e-5, (err.max(), np.unravel_index(err.argmax(), err.shape))
    np.testing.assert_array_equal(H, to_bf16(np.maximum(Z, 0.0)))


def test_invalid_arguments_are_refused():
    A = np.zeros((4, 48), dtype=np.uint16)
    Z = np.zeros((4, 64), dtype=np.float32)
    st = ba.lib().mba_gnn_gemm(0, 4, 48, _ptr16(A), _ptr16(A), None, None, None,
                               Z.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), None)
    assert st == N.MBA_ERR_INVALID_ARG


def test_bounded_wait_reports_a_timeout_and_the_device_stays_usable():
    """Failure detection without a fault: a barrier nothing signals (the
    operand copies left out) makes the kernel's bounded wait run out; the
    kernel raises its error flag and returns, the host reads MBA_ERR_TIMEOUT,
    and a normal launch right after gives correct results."""
    assert ba.lib().mba_gnn_gemm_wait_check(0) == N.MBA_ERR_TIMEOUT
    test_tensor_core_node_update_matches_fp32(64, 300, True, True)
