// Cone marching shared by the cone tracer (trace.cu) and the learned path
// (learned.cu): textureLod with GL_LINEAR_MIPMAP_LINEAR semantics over the
// radiance chain (shaders/phong.frag:135-180; sampler of
// src/Application.cpp:1088-1116) and the front-to-back cone march.
//
// Every fused multiply-add is written out (fmaf, __ffma2_rn); the including
// translation units are compiled without FMA contraction, so every
// instantiation rounds the same way.
#pragma once

#include "vct_device.cuh"

namespace vct {
namespace cone {

__device__ __forceinline__ f3 fnormalize(f3 v) { return mul(v, rsqrtf(dot(v, v))); }

// Texel (i, j, k) of level 0 from the bordered chain (0 outside the level).
__device__ __forceinline__ float4 texel0(const float4* __restrict__ pchain, int S, int i, int j, int k) {
    if ((unsigned)i >= (unsigned)S || (unsigned)j >= (unsigned)S || (unsigned)k >= (unsigned)S)
        return make_float4(0.f, 0.f, 0.f, 0.f);
    const int Pd = S + 2;
    return __ldg(pchain + (((k + 1) * Pd + (j + 1)) * Pd + (i + 1)));
}

__device__ __forceinline__ float4 lerp4(float4 p, float4 q, float t) {
    return make_float4(fmaf(t, q.x, fmaf(-t, p.x, p.x)), fmaf(t, q.y, fmaf(-t, p.y, p.y)),
                       fmaf(t, q.z, fmaf(-t, p.z, p.z)), fmaf(t, q.w, fmaf(-t, p.w, p.w)));
}

// RGBA as two packed fp32 pairs: Blackwell issues one FFMA2/FMUL2 per pair.
struct rgba2 {
    float2 rg, ba;
};

// The bordered chain holds each binary16 texel widened to fp32 (exactly), so
// a texel is one 16-byte read-only load with no conversion.
__device__ __forceinline__ rgba2 ld_texel(const float4* __restrict__ p) {
    const float4 v = __ldg(p);
    return {make_float2(v.x, v.y), make_float2(v.z, v.w)};
}

// t*q + (p - t*p) on both pairs: two FFMA2 per pair.
__device__ __forceinline__ rgba2 lerp2(rgba2 p, rgba2 q, float t) {
    const float2 tt = make_float2(t, t), nt = make_float2(-t, -t);
    return {__ffma2_rn(tt, q.rg, __ffma2_rn(nt, p.rg, p.rg)), __ffma2_rn(tt, q.ba, __ffma2_rn(nt, p.ba, p.ba))};
}

__device__ __forceinline__ float4 to_float4(rgba2 v) { return make_float4(v.rg.x, v.rg.y, v.ba.x, v.ba.y); }

// GL_LINEAR within level l with a (0,0,0,0) border, read from the bordered
// chain: for a position in [0,1]^3 the footprint's lower corner is in
// [-1, S-1]^3, i.e. [0, S]^3 of the (S+2)^3 bordered level, so the eight
// texels are plain loads at constant offsets with no bounds tests.
//
// With `guard` (positions warped about an eye outside the volume, or
// projected by the perspective warp, can leave [0,1]^3) the footprint is
// checked first: the bordered level holds texel
// indices -1..S, i.e. u = p S - 1/2 in [-1, S); outside that every texel of
// the footprint is border and the sample is (0,0,0,0).
__device__ __forceinline__ rgba2 trilinear2(const TraceParams& P, const int* __restrict__ off, int l, f3 p,
                                            bool guard = false) {
    const int S = P.dim >> l, Pd = S + 2;
    const float4* base = P.pchain + off[l];
    const float u = fmaf(p.x, (float)S, -0.5f), v = fmaf(p.y, (float)S, -0.5f), w = fmaf(p.z, (float)S, -0.5f);
    if (guard && !(u >= -1.0f && v >= -1.0f && w >= -1.0f && u < (float)S && v < (float)S && w < (float)S))
        return {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    const float fu = floorf(u), fv = floorf(v), fw = floorf(w);
    const float a = u - fu, b = v - fv, c = w - fw;
    const int i = (int)fu + 1, j = (int)fv + 1, k = (int)fw + 1;
    const float4* q = base + ((k * Pd + j) * Pd + i);
    const int sy = Pd, sz = Pd * Pd;
    const rgba2 t0 = ld_texel(q), t1 = ld_texel(q + 1), t2 = ld_texel(q + sy), t3 = ld_texel(q + sy + 1);
    const rgba2 t4 = ld_texel(q + sz), t5 = ld_texel(q + sz + 1), t6 = ld_texel(q + sz + sy),
                t7 = ld_texel(q + sz + sy + 1);
    const rgba2 x00 = lerp2(t0, t1, a), x10 = lerp2(t2, t3, a);
    const rgba2 x01 = lerp2(t4, t5, a), x11 = lerp2(t6, t7, a);
    return lerp2(lerp2(x00, x10, b), lerp2(x01, x11, b), c);
}

__device__ __forceinline__ float4 trilinear(const TraceParams& P, const int* off, int l, f3 p, bool guard = false) {
    return to_float4(trilinear2(P, off, l, p, guard));
}

template <int MODE>
__device__ __forceinline__ float4 sample_lod(const TraceParams& P, const int* off, f3 p, float lambda) {
    if (MODE == VCT_FILTER_HARDWARE) return tex3DLod<float4>(P.tex, p.x, p.y, p.z, lambda);
    const int q = P.levels - 1;
    if (MODE == VCT_FILTER_HARDWARE_LEVELS) {
        // Texture units filter within each level; the two levels are blended
        // with the exact fp32 fraction (GL_LINEAR_MIPMAP_LINEAR level choice).
        if (lambda <= 0.0f) return tex3DLod<float4>(P.tex, p.x, p.y, p.z, 0.0f);
        if (lambda >= (float)q) return tex3DLod<float4>(P.tex, p.x, p.y, p.z, (float)q);
        const float fl = floorf(lambda);
        return lerp4(tex3DLod<float4>(P.tex, p.x, p.y, p.z, fl), tex3DLod<float4>(P.tex, p.x, p.y, p.z, fl + 1.0f),
                     lambda - fl);
    }
    if (MODE == VCT_FILTER_HYBRID && lambda > 0.0f && lambda < (float)q) {
        // The level with the larger weight exactly, the other one by the
        // texture units at its integral level: the texture units' fixed-point
        // filter weights then enter the sample scaled by at most 1/2.  (The
        // step's level is the same in every lane, so the branch is uniform.)
        const float fl = floorf(lambda);
        const int d1 = (int)fl;
        const float f = lambda - fl;
        const bool guard = warp_leaves_volume(P.warp.mode);
        if (f <= 0.5f) {
            const rgba2 fine = trilinear2(P, off, d1, p, guard);
            const float4 c = tex3DLod<float4>(P.tex, p.x, p.y, p.z, fl + 1.0f);
            return to_float4(lerp2(fine, {make_float2(c.x, c.y), make_float2(c.z, c.w)}, f));
        }
        const float4 c = tex3DLod<float4>(P.tex, p.x, p.y, p.z, fl);
        const rgba2 coarse = trilinear2(P, off, d1 + 1, p, guard);
        return to_float4(lerp2({make_float2(c.x, c.y), make_float2(c.z, c.w)}, coarse, f));
    }
    if (lambda <= 0.0f) {  // magnification: GL_NEAREST on level 0 (index S = border)
        const int S = P.dim;
        return texel0(P.pchain + off[0], S, (int)floorf(p.x * S), (int)floorf(p.y * S), (int)floorf(p.z * S));
    }
    const bool guard = warp_leaves_volume(P.warp.mode);
    if (lambda >= (float)q) return trilinear(P, off, q, p, guard);
    float fl = floorf(lambda);
    int d1 = (int)fl;
    float f = lambda - fl;
    if (guard) return to_float4(lerp2(trilinear2(P, off, d1, p, true), trilinear2(P, off, d1 + 1, p, true), f));
    return to_float4(lerp2(trilinear2(P, off, d1, p), trilinear2(P, off, d1 + 1, p), f));
}

// `tanh` is tanf(c.cone_angle * 0.5f), which callers with many cones of one
// setting compute once.
template <int MODE>
__device__ __forceinline__ float4 trace_cone(const TraceParams& P, const int* off, f3 pos, f3 n, f3 dir,
                                             const vct_cone_settings c, float maxd, unsigned& ns, float tanh) {
    dir = fnormalize(dir);
    const float scale = 1.0f / (float)P.dim;
    const f3 start = add(pos, mul(mul(n, c.bias), scale));
    float h = c.cone_initial_height;
    float alpha = 0.0f;
    f3 col = mk(0.f, 0.f, 0.f);
    for (int i = 0; i < c.steps && alpha < 0.95f; ++i) {
        float r = h * tanh;
        float lod = __log2f(fmaxf(1.0f, 2.0f * r));
        const f3 dh = mul(dir, h);
        const f3 sp = mk(fmaf(dh.x, scale, start.x), fmaf(dh.y, scale, start.y), fmaf(dh.z, scale, start.z));
        // any(notEqual(p, clamp(p, 0, 1))): outside, or NaN
        if (!(sp.x >= 0.f && sp.y >= 0.f && sp.z >= 0.f && sp.x <= 1.f && sp.y <= 1.f && sp.z <= 1.f)) break;
        if (h * scale > maxd) break;
        float4 s = sample_lod<MODE>(P, off, P.warp.mode ? apply_warp(P.warp, sp) : sp, lod + c.lod_offset);
        ++ns;
        float a = 1.0f - alpha;
        col = mk(fmaf(s.x, a, col.x), fmaf(s.y, a, col.y), fmaf(s.z, a, col.z));
        alpha = fmaf(a, s.w, alpha);
        h += r;
    }
    return make_float4(col.x, col.y, col.z, alpha);
}

template <int MODE>
__device__ __forceinline__ float4 trace_cone(const TraceParams& P, const int* off, f3 pos, f3 n, f3 dir,
                                             const vct_cone_settings c, float maxd, unsigned& ns) {
    return trace_cone<MODE>(P, off, pos, n, dir, c, maxd, ns, tanf(c.cone_angle * 0.5f));
}

}  // namespace cone
}  // namespace vct
