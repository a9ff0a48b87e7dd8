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

// The fp32 copy of the map read by the lookups is bordered: (D+2)^3 texels,
// texel (i, j, k) at (i+1, j+1, k+1) and the border repeating the edge
// texels, which is what clamp-to-edge reads there.
constexpr int kWarpPad = kWarpDim + 2;

// texture(warpmap, p).xyz: GL_LINEAR with clamp-to-edge over the 32^3 RGBA16
// unorm map, read through its bordered fp32 copy (texel value c / 65535),
// lerped along x, then y, then z.  The footprint's lower corner is clamped to
// the border, so the eight loads are constant offsets from one address and
// read the texels the clamped indices would; x and y are interpolated as
// packed fp32 pairs (each element rounds as the scalar product and sum do).
__device__ __forceinline__ f3 warp_lookup(const float4* __restrict__ mapf, f3 p) {
    const float u = p.x * (float)kWarpDim - 0.5f, v = p.y * (float)kWarpDim - 0.5f, w = p.z * (float)kWarpDim - 0.5f;
    const float fu = floorf(u), fv = floorf(v), fw = floorf(w);
    const float a = u - fu, b = v - fv, c = w - fw;
    const int i = min(max((int)fu + 1, 0), kWarpDim), j = min(max((int)fv + 1, 0), kWarpDim),
              k = min(max((int)fw + 1, 0), kWarpDim);
    const float4* q = mapf + ((k * kWarpPad + j) * kWarpPad + i);
    constexpr int sy = kWarpPad, sz = kWarpPad * kWarpPad;
    const float4 t0 = __ldg(q), t1 = __ldg(q + 1), t2 = __ldg(q + sy), t3 = __ldg(q + sy + 1);
    const float4 t4 = __ldg(q + sz), t5 = __ldg(q + sz + 1), t6 = __ldg(q + sz + sy), t7 = __ldg(q + sz + sy + 1);
    // p * (1 - s) + q * s on the (x, y) pair and on z
    auto lerp_xy = [](float2 p, float2 q, float s) {
        return __fadd2_rn(__fmul2_rn(p, make_float2(1.0f - s, 1.0f - s)), __fmul2_rn(q, make_float2(s, s)));
    };
    auto lerp_z = [](float p, float q, float s) { return p * (1.0f - s) + q * s; };
    auto xy = [](float4 t) { return make_float2(t.x, t.y); };
    const float2 x00 = lerp_xy(xy(t0), xy(t1), a), x10 = lerp_xy(xy(t2), xy(t3), a);
    const float2 x01 = lerp_xy(xy(t4), xy(t5), a), x11 = lerp_xy(xy(t6), xy(t7), a);
    const float2 o = lerp_xy(lerp_xy(x00, x10, b), lerp_xy(x01, x11, b), c);
    const float z00 = lerp_z(t0.z, t1.z, a), z10 = lerp_z(t2.z, t3.z, a);
    const float z01 = lerp_z(t4.z, t5.z, a), z11 = lerp_z(t6.z, t7.z, a);
    f3 r;
    r.x = o.x;
    r.y = o.y;
    r.z = lerp_z(lerp_z(z00, z10, b), lerp_z(z01, z11, b), c);
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
