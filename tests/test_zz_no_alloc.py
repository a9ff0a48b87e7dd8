"""vct_voxelize_static: voxelisation for callers that cannot allocate device
memory (an application that reserves all of it up front for its own
allocator, a plugin in a process whose memory pool is owned elsewhere, a
frame loop that must not allocate).  It keeps its scratch in a fixed device
array inside the library and writes into volumes the caller owns.

The test calls it twice in a row through the C ABI and compares each call's
colour, normal and radiance volumes and counters, bit for bit (the bar of
every integer/binary16 stage in these tests), with the context path
vct_voxelize on the same inputs.  The second call shows that the shared
array is cleared between calls, and that it allocates nothing: the device's
free memory and torch's reserved bytes are the same before and after it.  A
second case runs with the temporal filter on, where the caller's radiance
volume holds the previous frame and is read before it is overwritten.  This
file is collected last so that a run stopping at the first failure has
already run every other test.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from vct_gb300 import _lib as L
from vct_gb300 import api, scenes

pytestmark = pytest.mark.gpu


def _inputs(sc):
    import torch

    dev = "cuda:0"
    pos, nrm, alb = (torch.from_numpy(a).to(dev) for a in (sc.positions, sc.normals, sc.albedo))
    tris = api.triangles(pos, nrm, alb)
    W, H = sc.shadow_size
    sm = torch.empty(W * H, dtype=torch.float32, device=dev)
    api.render_shadowmap(tris, sc, sm)
    return (pos, nrm, alb, sm), tris, api.shadow_desc(sc, sm), api.light_array(sc.lights)


VOLUMES = (L.VCT_VOLUME_COLOR, L.VCT_VOLUME_NORMAL, L.VCT_VOLUME_RADIANCE)


def _prior_radiance(seed):
    """A radiance level 0 of another scene: the 'previous frame' that the
    temporal filter mixes with (int16 binary16 bit patterns)."""
    import torch

    sc = scenes.cornell(seed=seed)
    keep, tris, shadow, lights = _inputs(sc)
    with api.Context(api.config_for(sc)) as ctx:
        ctx.set_params(api.scene_params(sc))
        ctx.voxelize(tris, lights, shadow, sc.eye)
        torch.cuda.synchronize()
        prior = ctx.read_volume(L.VCT_VOLUME_RADIANCE, 0)
    del keep
    return prior


@pytest.mark.parametrize("temporal", [0, 1])
def test_static_scratch_matches_context_path(temporal):
    import torch

    torch.cuda.set_device(0)
    sc = scenes.cornell(seed=5)
    keep, tris, shadow, (lights, n) = _inputs(sc)
    params = api.scene_params(sc, temporal_filter=temporal, temporal_decay=0.75)
    cfg = api.config_for(sc)
    nv = sc.dim ** 3
    prior = _prior_radiance(seed=6) if temporal else None

    with api.Context(cfg) as ctx:
        ctx.set_params(params)
        if temporal:  # the context's radiance level 0 holds the previous frame
            ptr, d = ctx.volume_ptr(L.VCT_VOLUME_RADIANCE, 0)
            api.device_view(ptr, (d * d * d * 4,), "<i2").copy_(prior)
            torch.cuda.synchronize()
        ctx.voxelize(tris, (lights, n), shadow, sc.eye)
        torch.cuda.synchronize()
        want = [ctx.read_volume(v, 0).cpu().numpy() for v in VOLUMES]
        want_stats = ctx.stats()

    lib = L.load()
    stream = api._stream(None)
    # Outputs are allocated by the caller, before the calls.
    outs = [torch.full((nv * 4,), -1, dtype=torch.int16, device="cuda:0") for _ in range(3)]
    for call in range(2):
        if temporal:
            outs[2].copy_(prior)
        torch.cuda.synchronize()
        free0, reserved0 = torch.cuda.mem_get_info(0)[0], torch.cuda.memory_reserved(0)
        st = L.vct_stats()
        rc = lib.vct_voxelize_static(C.byref(cfg), C.byref(params), C.byref(tris), lights, n, C.byref(shadow),
                                     outs[0].data_ptr(), outs[1].data_ptr(), outs[2].data_ptr(), C.byref(st), stream)
        L.check(rc, "vct_voxelize_static")
        torch.cuda.synchronize()
        if call == 1:  # the first call on a device may load the array's module; later calls allocate nothing
            assert torch.cuda.mem_get_info(0)[0] == free0, "device free memory changed across the call"
            assert torch.cuda.memory_reserved(0) == reserved0, "torch's reserved bytes changed across the call"
        for got, ref in zip(outs, want):
            assert np.array_equal(got.cpu().numpy(), ref), f"call {call}"
        assert st.total_voxel_fragments == want_stats["total_voxel_fragments"]
        assert st.unique_voxels == want_stats["unique_voxels"]
        assert st.max_fragments_per_voxel == want_stats["max_fragments_per_voxel"]
        assert st.error_flags == 0
    if temporal:  # the mix is not a no-op: the previous frame shows in the result
        with api.Context(cfg) as ctx:
            ctx.set_params(api.scene_params(sc))
            ctx.voxelize(tris, (lights, n), shadow, sc.eye)
            torch.cuda.synchronize()
            plain = ctx.read_volume(L.VCT_VOLUME_RADIANCE, 0).cpu().numpy()
        assert not np.array_equal(outs[2].cpu().numpy(), plain)
    del keep


def test_static_scratch_rejects_oversize():
    import torch

    torch.cuda.set_device(0)
    sc = scenes.tiny(seed=1)
    keep, tris, shadow, (lights, n) = _inputs(sc)
    params = api.scene_params(sc)
    lib = L.load()
    big = api.config_for(sc, dim=128)
    out = torch.zeros(4, dtype=torch.int16, device="cuda:0")
    rc = lib.vct_voxelize_static(C.byref(big), C.byref(params), C.byref(tris), lights, n, C.byref(shadow),
                                 out.data_ptr(), out.data_ptr(), out.data_ptr(), None, api._stream(None))
    assert rc == L.VCT_ERR_INVALID_ARGUMENT
    assert b"VCT_STATIC_MAX_DIM" in lib.vct_last_error()
    many = api.triangles(keep[0], keep[1], keep[2])
    # Rejected by the size check before any device work (the arrays behind
    # this descriptor are never read).
    many.count = 16384 + 1
    rc = lib.vct_voxelize_static(C.byref(api.config_for(sc)), C.byref(params), C.byref(many), lights, n,
                                 C.byref(shadow), out.data_ptr(), out.data_ptr(), out.data_ptr(), None,
                                 api._stream(None))
    assert rc == L.VCT_ERR_INVALID_ARGUMENT
    assert b"VCT_STATIC_MAX_TRIANGLES" in lib.vct_last_error()
    # Output volumes must be 32-byte aligned (checked before any device work).
    vol = torch.zeros(sc.dim ** 3 * 4 + 16, dtype=torch.int16, device="cuda:0")
    rc = lib.vct_voxelize_static(C.byref(api.config_for(sc)), C.byref(params), C.byref(tris), lights, n,
                                 C.byref(shadow), vol.data_ptr() + 16, vol.data_ptr(), vol.data_ptr(), None,
                                 api._stream(None))
    assert rc == L.VCT_ERR_INVALID_ARGUMENT
    assert b"32-byte aligned" in lib.vct_last_error()


def test_static_scratch_stats_rejected_under_capture():
    """The counters' read-back synchronises the stream, which a stream
    capture forbids: with stats given, a call on a capturing stream is
    refused before it enqueues anything, and the capture stays valid."""
    import torch

    torch.cuda.set_device(0)
    sc = scenes.tiny(seed=2)
    keep, tris, shadow, (lights, n) = _inputs(sc)
    params = api.scene_params(sc)
    cfg = api.config_for(sc)
    nv = sc.dim ** 3
    outs = [torch.zeros(nv * 4, dtype=torch.int16, device="cuda:0") for _ in range(3)]
    lib = L.load()
    # first call on this device outside any capture (it looks up the array's address)
    L.check(lib.vct_voxelize_static(C.byref(cfg), C.byref(params), C.byref(tris), lights, n, C.byref(shadow),
                                    outs[0].data_ptr(), outs[1].data_ptr(), outs[2].data_ptr(), None,
                                    api._stream(None)), "vct_voxelize_static")
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    st = L.vct_stats()
    with torch.cuda.graph(g, stream=side):
        rc = lib.vct_voxelize_static(C.byref(cfg), C.byref(params), C.byref(tris), lights, n, C.byref(shadow),
                                     outs[0].data_ptr(), outs[1].data_ptr(), outs[2].data_ptr(), C.byref(st),
                                     side.cuda_stream)
    assert rc == L.VCT_ERR_INVALID_ARGUMENT
    assert b"captured" in lib.vct_last_error()
    torch.cuda.synchronize()
    del keep
