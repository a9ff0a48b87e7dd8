// Device-side helpers shared by the VCT kernels.
//
// The voxelisation, normalisation, injection and mip kernels are compiled
// with --fmad=false: every a*b+c below is two IEEE-rounded operations and
// every division and square root is IEEE-rounded, so their results are
// reproducible bit for bit by any CPU that evaluates the same expressions in
// the same order.  The operation order used here is fixed: it follows the
// GLSL expression order of the reference shaders (left to right).
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

#include "vct_internal.h"
#include "warp.cuh"

namespace vct {

// ---- the carry table of exact accumulation (vct_internal.h, kCarrySlots)
__device__ __forceinline__ uint32_t carry_slot(uint32_t v, int probe) {
    return (((v * 2654435761u) >> (32 - kCarrySlotsLog2)) + (uint32_t)probe) & (uint32_t)(kCarrySlots - 1);
}
// Adds the crossings ev[] of voxel v to its entry (claimed on first use).
__device__ __forceinline__ void carry_add(uint32_t* table, uint32_t v, const uint32_t (&ev)[kCarryEvents],
                                          StatsDev* stats) {
    const uint32_t key = v + 1u;
    for (int i = 0; i < kCarryProbes; ++i) {
        uint32_t* e = table + 8 * carry_slot(v, i);
        const uint32_t k = atomicCAS(e, 0u, key);
        if (k == 0u || k == key) {
#pragma unroll
            for (int f = 0; f < kCarryEvents; ++f)
                if (ev[f]) atomicAdd(e + 1 + f, ev[f]);
            return;
        }
    }
    atomicOr(&stats->error_flags, VCT_STATS_COUNT_OVERFLOW);
}
// Whether adding `a` to the 64-bit word whose value was `o` carried out of
// the low 32-bit field, and whether the high field (with that carry) wrapped.
__device__ __forceinline__ uint32_t carry_lo(unsigned long long o, unsigned long long a) {
    return (uint32_t)(((o & 0xffffffffull) + (a & 0xffffffffull)) >> 32);
}
__device__ __forceinline__ uint32_t wrap_hi(unsigned long long o, unsigned long long a) {
    return (uint32_t)(((o >> 32) + (a >> 32) + carry_lo(o, a)) >> 32);
}

__device__ __forceinline__ f3 mk(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ f3 add(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 sub(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 mul(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ f3 mulv(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 ld3(const float* p) { return {p[0], p[1], p[2]}; }
// normalize(v) = v * (1 / sqrt(dot(v, v))), both operations IEEE-rounded.
__device__ __forceinline__ f3 normalize(f3 v) {
    float inv = __fdiv_rn(1.0f, __fsqrt_rn(dot(v, v)));
    return mul(v, inv);
}
__device__ __forceinline__ float length(f3 v) { return __fsqrt_rn(dot(v, v)); }
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float smoothstep(float e0, float e1, float x) {
    float t = clampf(__fdiv_rn(x - e0, e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

// glm mat4 (column-major) * vec4, columns summed in order.
__device__ __forceinline__ void mat_vec(const float* m, float x, float y, float z, float w, float out[4]) {
#pragma unroll
    for (int r = 0; r < 4; ++r) out[r] = m[0 + r] * x + m[4 + r] * y + m[8 + r] * z + m[12 + r] * w;
}

// ---------------------------------------------------------------- binary16
__device__ __forceinline__ uint16_t f2h(float f) { return __half_as_ushort(__float2half_rn(f)); }
__device__ __forceinline__ float h2f(uint16_t h) { return __half2float(__ushort_as_half(h)); }
__device__ __forceinline__ uint2 pack_h4(float a, float b, float c, float d) {
    uint2 r;
    r.x = (uint32_t)f2h(a) | ((uint32_t)f2h(b) << 16);
    r.y = (uint32_t)f2h(c) | ((uint32_t)f2h(d) << 16);
    return r;
}
__device__ __forceinline__ float4 unpack_h4(uint2 v) {
    float2 lo = __half22float2(*reinterpret_cast<const __half2*>(&v.x));
    float2 hi = __half22float2(*reinterpret_cast<const __half2*>(&v.y));
    return make_float4(lo.x, lo.y, hi.x, hi.y);
}

// ------------------------------------------------------- rasterisation core
// Pixel-centre coverage on a 1/256 sub-pixel grid with a top-left tie rule,
// identical to the CPU oracle: window coordinates are snapped with
// rint(w * 256) after clamping to +-2^20 pixels, edge functions are exact
// 64-bit integers, and interpolation weights are e_k * (1 / area) in fp32.
constexpr long long kSub = 256;

__device__ __forceinline__ long long snap(float w) {
    w = clampf(w, -1048576.0f, 1048576.0f);
    return (long long)rintf(w * 256.0f);
}
__device__ __forceinline__ long long floordiv(long long a, long long b) {
    long long q = a / b;
    if ((a % b != 0) && ((a < 0) != (b < 0))) --q;
    return q;
}
__device__ __forceinline__ long long edge(long long ax, long long ay, long long bx, long long by, long long px,
                                          long long py) {
    return (bx - ax) * (py - ay) - (by - ay) * (px - ax);
}

struct RasterTri {
    long long X[3], Y[3];
    long long area;
    long long bias[3];
    int px0, px1, py0, py1;
    int perm1;  // 1: vertices 1 and 2 were swapped to make the triangle CCW
};

__device__ __forceinline__ bool raster_setup(const float wx[3], const float wy[3], int W, int H, RasterTri& t) {
    long long X[3], Y[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        X[k] = snap(wx[k]);
        Y[k] = snap(wy[k]);
    }
    long long area = edge(X[0], Y[0], X[1], Y[1], X[2], Y[2]);
    if (area == 0) return false;
    t.perm1 = area < 0;
    if (t.perm1) {
        area = -area;
        long long tx = X[1], ty = Y[1];
        X[1] = X[2];
        Y[1] = Y[2];
        X[2] = tx;
        Y[2] = ty;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        t.X[k] = X[k];
        t.Y[k] = Y[k];
    }
    t.area = area;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        int a = (k + 1) % 3, b = (k + 2) % 3;
        long long dx = X[b] - X[a], dy = Y[b] - Y[a];
        bool tl = (dy < 0) || (dy == 0 && dx < 0);
        t.bias[k] = tl ? 0 : -1;
    }
    long long minx = min(X[0], min(X[1], X[2])), maxx = max(X[0], max(X[1], X[2]));
    long long miny = min(Y[0], min(Y[1], Y[2])), maxy = max(Y[0], max(Y[1], Y[2]));
    long long x0 = -floordiv(-(minx - kSub / 2), kSub);
    long long x1 = floordiv(maxx - kSub / 2, kSub);
    long long y0 = -floordiv(-(miny - kSub / 2), kSub);
    long long y1 = floordiv(maxy - kSub / 2, kSub);
    x0 = max(x0, 0LL);
    y0 = max(y0, 0LL);
    x1 = min(x1, (long long)W - 1);
    y1 = min(y1, (long long)H - 1);
    if (x0 > x1 || y0 > y1) return false;
    t.px0 = (int)x0;
    t.px1 = (int)x1;
    t.py0 = (int)y0;
    t.py1 = (int)y1;
    return true;
}

__device__ __forceinline__ bool raster_cover(const RasterTri& t, int px, int py, long long e[3]) {
    long long sx = (long long)px * kSub + kSub / 2, sy = (long long)py * kSub + kSub / 2;
    bool in = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        int a = (k + 1) % 3, b = (k + 2) % 3;
        e[k] = edge(t.X[a], t.Y[a], t.X[b], t.Y[b], sx, sy);
        in = in && (e[k] + t.bias[k] >= 0);
    }
    return in;
}

// Weights in the caller's original vertex order.
__device__ __forceinline__ void raster_weights(const RasterTri& t, const long long e[3], float l[3]) {
    float inv = __fdiv_rn(1.0f, __ll2float_rn(t.area));
    float l0 = __ll2float_rn(e[0]) * inv, l1 = __ll2float_rn(e[1]) * inv, l2 = __ll2float_rn(e[2]) * inv;
    l[0] = l0;
    l[1] = t.perm1 ? l2 : l1;
    l[2] = t.perm1 ? l1 : l2;
}

__device__ __forceinline__ float interp(const float l[3], float a, float b, float c) {
    return l[0] * a + l[1] * b + l[2] * c;
}

// ------------------------------------------- bilinear fetch, border 1.0
__device__ __forceinline__ float shadow_fetch(const float* __restrict__ sm, int W, int H, int i, int j) {
    if (i < 0 || j < 0 || i >= W || j >= H) return 1.0f;
    return __ldg(sm + (long long)j * W + i);
}
__device__ __forceinline__ float shadow_bilinear(const float* __restrict__ sm, int W, int H, float u, float v, int ox,
                                                 int oy) {
    float x = (u * (float)W + (float)ox) - 0.5f;
    float y = (v * (float)H + (float)oy) - 0.5f;
    float fx = floorf(x), fy = floorf(y);
    float a = x - fx, b = y - fy;
    int i = (int)fx, j = (int)fy;
    float t00 = shadow_fetch(sm, W, H, i, j), t10 = shadow_fetch(sm, W, H, i + 1, j);
    float t01 = shadow_fetch(sm, W, H, i, j + 1), t11 = shadow_fetch(sm, W, H, i + 1, j + 1);
    float bot = t00 * (1.0f - a) + t10 * a;
    float top = t01 * (1.0f - a) + t11 * a;
    return bot * (1.0f - b) + top * b;
}

// calcShadowFactor (voxelize.frag:160-184 = phong.frag:183-207): 5-tap PCF of
// the bilinear light-space depth with bias 0.01; 0 beyond the far plane.
__device__ __forceinline__ float pcf5(const float* __restrict__ sm, int sw, int sh, const float* ls, f3 wp) {
    float c[4];
    mat_vec(ls, wp.x, wp.y, wp.z, 1.0f, c);
    // x / 1 == x exactly: skip the divide for an orthographic light.
    if (c[3] != 1.0f) {
        c[0] = __fdiv_rn(c[0], c[3]);
        c[1] = __fdiv_rn(c[1], c[3]);
        c[2] = __fdiv_rn(c[2], c[3]);
    }
    float sx = (c[0] + 1.0f) * 0.5f;
    float sy = (c[1] + 1.0f) * 0.5f;
    float sz = (c[2] + 1.0f) * 0.5f;
    float frag = sz - 0.01f;
    if (frag > 1.0f) return 0.0f;
    const int ox[5] = {0, 1, 0, -1, 0};
    const int oy[5] = {0, 0, 1, 0, -1};
    float f = 0.0f;
#pragma unroll
    for (int s = 0; s < 5; ++s)
        if (frag > shadow_bilinear(sm, sw, sh, sx, sy, ox[s], oy[s])) f += 1.0f;
    return __fdiv_rn(f, 5.0f);
}

__device__ __forceinline__ uint32_t quant16(float x) { return __float2uint_rn(clampf(x, 0.0f, 1.0f) * 65535.0f); }

// ------------------------------------------------------------ scene sets
// Kernels are templated on a scene set: OneScene keeps the parameters in
// kernel-parameter space (the single-frame path), ManyScenes reads them from
// device memory and maps a global work index to (scene, local index).
template <class Params>
struct OneScene {
    Params p;
    __device__ __forceinline__ int count() const { return 1; }
    __device__ __forceinline__ const Params& get(int) const { return p; }
    __device__ __forceinline__ int find(long long w, long long& local) const {
        local = w;
        return 0;
    }
};

template <class Params>
struct ManyScenes {
    SceneBatch<Params> b;
    __device__ __forceinline__ int count() const { return b.n; }
    __device__ __forceinline__ const Params& get(int s) const { return b.p[s]; }
    __device__ __forceinline__ int find(long long w, long long& local) const {
        int lo = 0, hi = b.n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(b.off + mid) <= w)
                lo = mid;
            else
                hi = mid - 1;
        }
        local = w - __ldg(b.off + lo);
        return lo;
    }
};

// The viewpoints of a ViewSet (at most kMaxViews): found by a linear scan.
struct FewScenes {
    ViewSet v;
    __device__ __forceinline__ int count() const { return v.n; }
    __device__ __forceinline__ const TraceParams& get(int s) const { return v.p[s]; }
    __device__ __forceinline__ int find(long long w, long long& local) const {
        int s = 0;
        while (s + 1 < v.n && v.off[s + 1] <= w) ++s;
        local = w - v.off[s];
        return s;
    }
};

}  // namespace vct
