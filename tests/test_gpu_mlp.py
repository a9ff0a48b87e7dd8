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


def test_bounded_wait_times_out_and_device_stays_usable():
    """The timeout path of the tensor-core kernels' bounded waits: a wait on an
    mbarrier that nothing arrives on gives up after 2 ms and the call reports
    VCT_ERR_TIMEOUT instead of hanging; the tensor-core path then still gives
    the right product."""
    import time

    import torch

    t0 = time.perf_counter()
    with pytest.raises(L.VctError) as e:
        L.call("vct_timeout_probe", 2_000_000, torch.cuda.current_stream().cuda_stream)
    assert e.value.status == L.VCT_ERR_TIMEOUT
    assert time.perf_counter() - t0 < 5.0
    with pytest.raises(L.VctError) as e:
        L.call("vct_timeout_probe", 10, None)
    assert e.value.status == L.VCT_ERR_INVALID_ARGUMENT
    d, ref = _gemm(64, 64, 0, seed=3)
    assert np.abs(d - ref).max() / np.abs(ref).max() < 1e-5


@pytest.mark.parametrize("k,n", [(16, 16), (48, 64), (64, 64), (64, 16), (32, 48)])
def test_tensor_core_gemm(k, n):
    d, ref = _gemm(k, n, 0)
    err = np.abs(d - ref).max() / np.abs(ref).max()
    assert err < 1e-5, err


def test_descriptor_strides_matter():
    d, ref = _gemm(64, 64, 1)
    assert not np.allclose(d, ref, rtol=1e-3, atol=1e-3)


# ----------------------------------------------------------------- the MLP
from oracle import mlp as OM  # noqa: E402
from vct_gb300 import api  # noqa: E402


def _net(seed=3):
    m = api.Mlp(seed=seed)
    p = m.params().astype(np.float64)
    rng = np.random.default_rng(seed)
    # non-zero biases exercise the bias paths
    for name, (o, n) in {"b1": (2688, 64), "b2": (6848, 64), "b3": (11008, 64), "b4": (11328, 4)}.items():
        p[o:o + n] = rng.uniform(-0.2, 0.2, n)
    m.set_params(p.astype(np.float32))
    return m, m.params().astype(np.float64)


def _rows(n, seed=0):
    import torch

    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, (n, OM.IN)).astype(np.float32)
    y = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    return x, y, torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_mlp_params_roundtrip_and_init():
    m, p = _net(7)
    w = OM.unpack(p)
    bound = np.sqrt(6.0 / 42)
    # He-uniform: U(-bound, bound), standard deviation bound / sqrt(3)
    assert np.abs(w["W1"]).max() <= bound and abs(w["W1"].std() - bound / np.sqrt(3)) < 0.05 * bound
    m2 = api.Mlp(seed=7)
    assert np.array_equal(api.Mlp(seed=7).params(), m2.params())
    assert not np.array_equal(api.Mlp(seed=8).params(), m2.params())


@pytest.mark.parametrize("n", [1, 127, 128, 1000, 40000])
def test_mlp_forward_matches_oracle(n):
    import torch

    m, p = _net()
    x, _, dx, _ = _rows(n)
    out = torch.empty(n, 4, device="cuda")
    m.forward(dx, out)
    got = out.cpu().numpy()
    emu = OM.forward_backward(p, x, emulate_bf16=True)[0]
    f64 = OM.forward_backward(p, x)[0]
    assert _rel(got, emu) < 2e-3, _rel(got, emu)
    assert _rel(got, f64) < 2e-2, _rel(got, f64)


@pytest.mark.parametrize("n", [100, 1000, 5000])
def test_mlp_gradients_match_oracle(n):
    import torch

    m, p = _net()
    x, y, dx, dy = _rows(n, seed=1)
    grad = torch.empty(OM.NPARAMS, device="cuda")
    loss = torch.empty(1, device="cuda")
    m.gradients(dx, dy, grad, loss)
    g = grad.cpu().numpy().astype(np.float64)
    _, l_emu, g_emu = OM.forward_backward(p, x, y, emulate_bf16=True)
    _, l64, g64 = OM.forward_backward(p, x, y)
    assert abs(float(loss.item()) - l_emu) <= 1e-3 * l_emu
    assert _rel(g, g_emu) < 1e-2, _rel(g, g_emu)
    assert _rel(g, g64) < 5e-2, _rel(g, g64)
    cos = float(g @ g64 / (np.linalg.norm(g) * np.linalg.norm(g64)))
    assert cos > 0.998, cos
    # every parameter block carries gradient
    for name, (o, k) in {"W1": (0, 2688), "b1": (2688, 64), "W4": (11072, 256), "b4": (11328, 4),
                         "W4 error row": (11072 + 192, 64), "b4 error": (11331, 1)}.items():
        assert _rel(g[o:o + k], g_emu[o:o + k]) < 2e-2, name


def test_adam_step_matches_oracle():
    import torch

    m, p = _net(5)
    x, y, dx, dy = _rows(3000, seed=2)
    grad = torch.empty(OM.NPARAMS, device="cuda")
    m.gradients(dx, dy, grad)
    g = grad.cpu().numpy().astype(np.float64)
    m.train_step(dx, dy, None, 3000, 1e-3)
    after = m.params().astype(np.float64)
    ref, _, _ = OM.adam(p, g, np.zeros_like(p), np.zeros_like(p), 1, 1e-3)
    assert np.abs(after - ref).max() < 1e-6


def test_training_fits_a_teacher_network():
    import torch

    teacher, tp = _net(11)
    x, _, dx, _ = _rows(65536, seed=4)
    out = torch.empty(65536, 4, device="cuda")
    teacher.forward(dx, out)
    dy = out[:, :3].contiguous()
    m = api.Mlp(seed=12)
    loss = torch.zeros(1, device="cuda")
    first = None
    gen = torch.Generator(device="cuda")
    gen.manual_seed(0)
    for step in range(400):
        idx = torch.randint(0, 65536, (8192,), device="cuda", dtype=torch.int32, generator=gen)
        m.train_step(dx, dy, idx, 8192, 2e-3, loss)
        if step == 0:
            first = float(loss.item())
    torch.cuda.synchronize()
    last = float(loss.item())
    assert last < 0.1 * first, (first, last)
