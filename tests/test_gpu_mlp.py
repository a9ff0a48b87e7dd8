"""Tensor-core path of the learned part: the BF16 GEMM with an FP32
accumulator in tensor memory (tcgen05) against a float64 product of the same
BF16 operands."""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from vct_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def bf16_bits(x: np.ndarray) -> np.ndarray:
    """float32 -> bfloat16 bit patterns, round to nearest even."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def bf16_value(b: np.ndarray) -> np.ndarray:
    return (b.astype(np.uint32) << 16).view(np.float32)


def _gemm(k, n, variant, seed=0):
    import torch

    rng = np.random.default_rng(seed)
    a = bf16_bits(rng.standard_normal((128, k)).astype(np.float32))
    b = bf16_bits(rng.standard_normal((n, k)).astype(np.float32))
    da = torch.from_numpy(a.view(np.int16)).cuda()
    db = torch.from_numpy(b.view(np.int16)).cuda()
    dd = torch.zeros(128 * n, dtype=torch.float32, device="cuda")
    L.call("vct_tensor_core_check", da.data_ptr(), db.data_ptr(), k, n, variant, dd.data_ptr(),
           torch.cuda.current_stream().cuda_stream)
    ref = bf16_value(a).astype(np.float64) @ bf16_value(b).astype(np.float64).T
    return dd.cpu().numpy().reshape(128, n), ref


@pytest.mark.parametrize("k,n", [(16, 16), (48, 64), (64, 64), (64, 16), (32, 48)])
def test_tensor_core_gemm(k, n):
    d, ref = _gemm(k, n, 0)
    err = np.abs(d - ref).max() / np.abs(ref).max()
    assert err < 1e-5, err


def test_descriptor_strides_matter():
    d, ref = _gemm(64, 64, 1)
    assert not np.allclose(d, ref, rtol=1e-3, atol=1e-3)
