// Voxel warping (common.glsl:11-64, voxelize.frag:100-106, phong.frag:150-157):
// positions in [0,1]^3 volume coordinates are remapped before they index or
// sample the grid.  Compiled with --fmad=false everywhere it is used; the
// operation order follows the GLSL expressions.
#pragma once

#include "vct_internal.h"

namespace vct {

constexpr int kWarpDim = VCT_WARP_DIM;

// voxelWarpFn (common.glsl:11-18) with alpha = 0.25:
// alpha x + (3 - 3 alpha) x^2 + (2 alpha - 2) x^3, clamped to [0,1].
__device__ __forceinline__ float warp_fn(float x) {
    const float y = (0.25f * x + 2.25f * x * x) + -1.5f * x * x * x;
    return fminf(fmaxf(y, 0.0f), 1.0f);
}

// voxelWarp (common.glsl:20-27): the offset from the eye, mapped to [0,1],
// warped, mapped back.
__device__ __forceinline__ f3 voxel_warp(f3 p, f3 c) {
    f3 r;
    const float pc[3] = {p.x, p.y, p.z}, cc[3] = {c.x, c.y, c.z};
    float o[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float off = pc[k] - cc[k];
        off = 0.5f * off + 0.5f;
        off = warp_fn(off);
        off = 2.0f * off - 1.0f;
        o[k] = cc[k] + off;
    }
    r.x = o[0];
    r.y = o[1];
    r.z = o[2];
    return r;
}

// texture(warpmap, p).xyz: GL_LINEAR with clamp-to-edge over the 32^3 RGBA16
// unorm map, read through its fp32 copy (texel value c / 65535), lerped
// along x, then y, then z.
__device__ __forceinline__ f3 warp_lookup(const float4* __restrict__ mapf, f3 p) {
    const float u = p.x * (float)kWarpDim - 0.5f, v = p.y * (float)kWarpDim - 0.5f, w = p.z * (float)kWarpDim - 0.5f;
    const float fu = floorf(u), fv = floorf(v), fw = floorf(w);
    const float a = u - fu, b = v - fv, c = w - fw;
    const int i0 = (int)fu, j0 = (int)fv, k0 = (int)fw;
    const int ix[2] = {min(max(i0, 0), kWarpDim - 1), min(max(i0 + 1, 0), kWarpDim - 1)};
    const int iy[2] = {min(max(j0, 0), kWarpDim - 1), min(max(j0 + 1, 0), kWarpDim - 1)};
    const int iz[2] = {min(max(k0, 0), kWarpDim - 1), min(max(k0 + 1, 0), kWarpDim - 1)};
    float t[8][3];
#pragma unroll
    for (int n = 0; n < 8; ++n) {
        const float4 q = __ldg(mapf + ((iz[n >> 2] * kWarpDim + iy[(n >> 1) & 1]) * kWarpDim + ix[n & 1]));
        t[n][0] = q.x;
        t[n][1] = q.y;
        t[n][2] = q.z;
    }
    float o[3];
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        const float x00 = t[0][ch] * (1.0f - a) + t[1][ch] * a;
        const float x10 = t[2][ch] * (1.0f - a) + t[3][ch] * a;
        const float x01 = t[4][ch] * (1.0f - a) + t[5][ch] * a;
        const float x11 = t[6][ch] * (1.0f - a) + t[7][ch] * a;
        const float y0 = x00 * (1.0f - b) + x10 * b;
        const float y1 = x01 * (1.0f - b) + x11 * b;
        o[ch] = y0 * (1.0f - c) + y1 * c;
    }
    f3 r;
    r.x = o[0];
    r.y = o[1];
    r.z = o[2];
    return r;
}

// voxelTesselationWarpedPosition (common.glsl:37-42): pv * (p, 1), divided
// by w, mapped from [-1,1] to [0,1].  Every consumer drops (voxeliser,
// injection) or reads as border (cone tracer) a coordinate outside [-1, 2],
// so such results, infinities and NaN (points on or behind the camera plane)
// are replaced by -1, which keeps the float-to-int truncations defined.
__device__ __forceinline__ f3 perspective_tc(const WarpDev& W, f3 p) {
    const float* m = W.pv;
    float c[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) c[r] = ((m[r] * p.x + m[4 + r] * p.y) + m[8 + r] * p.z) + m[12 + r] * 1.0f;
    f3 q;
    q.x = __fdiv_rn(c[0], c[3]) * 0.5f + 0.5f;
    q.y = __fdiv_rn(c[1], c[3]) * 0.5f + 0.5f;
    q.z = __fdiv_rn(c[2], c[3]) * 0.5f + 0.5f;
    if (!(q.x >= -1.0f && q.x <= 2.0f && q.y >= -1.0f && q.y <= 2.0f && q.z >= -1.0f && q.z <= 2.0f))
        q.x = q.y = q.z = -1.0f;
    return q;
}

// Volume coordinate -> world (phong.frag:159: p * (max - min) + center + min)
// -> perspective coordinate.
__device__ __forceinline__ f3 perspective_from_tc(const WarpDev& W, f3 t) {
    f3 w;
    w.x = (t.x * W.ext.x + W.vcenter.x) + W.vmin.x;
    w.y = (t.y * W.ext.y + W.vcenter.y) + W.vmin.y;
    w.z = (t.z * W.ext.z + W.vcenter.z) + W.vmin.z;
    return perspective_tc(W, w);
}

// Warps that can move a position off [0,1]^3 (the samplers check the footprint).
__device__ __forceinline__ bool warp_leaves_volume(int mode) {
    return mode == VCT_WARP_ANALYTIC || mode == VCT_WARP_PERSPECTIVE;
}

__device__ __forceinline__ f3 apply_warp(const WarpDev& W, f3 p) {
    if (W.mode == VCT_WARP_ANALYTIC) return voxel_warp(p, W.eye_tc);
    if (W.mode == VCT_WARP_TEXTURE) return warp_lookup(W.mapf, p);
    if (W.mode == VCT_WARP_PERSPECTIVE) return perspective_from_tc(W, p);
    return p;
}

}  // namespace vct
