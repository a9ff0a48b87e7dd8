// Voxel cone tracing: shaders/phong.frag:135-180 (traceCone) and the
// indirect / specular / composite code of phong.frag:455-520.
//
// One thread per pixel; a CTA shades a 16x16 tile and each warp an 8x4
// sub-tile, so the 32 lanes of a warp march neighbouring cones through
// neighbouring voxels at the same time (the cone step sequence depends only on
// the cone parameters, so every lane is at the same mip level each step).
// A lane leaves its cone at alpha >= 0.95 or on leaving the volume; the warp
// moves to the next cone once all lanes are done.
//
// Two samplers implement textureLod with GL_LINEAR_MIPMAP_LINEAR, LOD clamped
// to [0, levels-1] and a (0,0,0,0) border (src/Application.cpp:1088-1116):
//  - software: fp32 trilinear over 8 texels of two levels, read with 16-byte
//    read-only loads from a bordered fp32 copy of the chain (no bounds tests);
//  - hardware: tex3DLod on a mip-mapped CUDA array (texture units, with
//    their fixed-point filter weights).
//
// The file is compiled without FMA contraction: every fused multiply-add is
// written out (fmaf, __ffma2_rn), so the single-scene and the batched
// instantiations of the kernel give bit-identical results.
#include "vct_device.cuh"

namespace vct {

namespace {

__constant__ float kConeDir[6][3] = {{0.f, 1.f, 0.f},
                                     {0.f, 0.5f, 0.866025f},
                                     {0.823639f, 0.5f, 0.267617f},
                                     {0.509037f, 0.5f, -0.700629f},
                                     {-0.5909037f, 0.5f, -0.700629f},  // sic, phong.frag:475
                                     {-0.823639f, 0.5f, 0.267617f}};
__constant__ float kConeWeight[6] = {0.25f, 0.15f, 0.15f, 0.15f, 0.15f, 0.15f};

__device__ __forceinline__ f3 fnormalize(f3 v) { return mul(v, rsqrtf(dot(v, v))); }

__device__ __forceinline__ float4 texel(const uint2* __restrict__ base, int S, int i, int j, int k) {
    if ((unsigned)i >= (unsigned)S || (unsigned)j >= (unsigned)S || (unsigned)k >= (unsigned)S)
        return make_float4(0.f, 0.f, 0.f, 0.f);
    return unpack_h4(__ldg(base + ((k * S + j) * S + i)));
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
__device__ __forceinline__ rgba2 trilinear2(const TraceParams& P, const int* __restrict__ off, int l, f3 p) {
    const int S = P.dim >> l, Pd = S + 2;
    const float4* base = P.pchain + off[l];
    const float u = fmaf(p.x, (float)S, -0.5f), v = fmaf(p.y, (float)S, -0.5f), w = fmaf(p.z, (float)S, -0.5f);
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

__device__ __forceinline__ float4 trilinear(const TraceParams& P, const int* off, int l, f3 p) {
    return to_float4(trilinear2(P, off, l, p));
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
    if (lambda <= 0.0f) {  // magnification: GL_NEAREST on level 0 (index S = border)
        const int S = P.dim;
        return texel(P.chain, S, (int)floorf(p.x * S), (int)floorf(p.y * S), (int)floorf(p.z * S));
    }
    if (lambda >= (float)q) return trilinear(P, off, q, p);
    float fl = floorf(lambda);
    int d1 = (int)fl;
    float f = lambda - fl;
    return to_float4(lerp2(trilinear2(P, off, d1, p), trilinear2(P, off, d1 + 1, p), f));
}

template <int MODE>
__device__ __forceinline__ float4 trace_cone(const TraceParams& P, const int* off, f3 pos, f3 n, f3 dir,
                                             const vct_cone_settings c,
                             float maxd, unsigned& ns) {
    dir = fnormalize(dir);
    const float scale = 1.0f / (float)P.dim;
    const f3 start = add(pos, mul(mul(n, c.bias), scale));
    const float tanh = tanf(c.cone_angle * 0.5f);
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
        float4 s = sample_lod<MODE>(P, off, sp, lod + c.lod_offset);
        ++ns;
        float a = 1.0f - alpha;
        col = mk(fmaf(s.x, a, col.x), fmaf(s.y, a, col.y), fmaf(s.z, a, col.z));
        alpha = fmaf(a, s.w, alpha);
        h += r;
    }
    return make_float4(col.x, col.y, col.z, alpha);
}

template <int MODE, class Scenes>
__global__ void __launch_bounds__(256) trace_kernel(const Scenes S) {
    // One CTA per tile of 2^tile_w_log2 x 2^tile_h_log2 = 256 pixels (a
    // tuning setting; tiles of every scene of the launch in a row), one warp
    // per 2^warp_w_log2 x 32/2^warp_w_log2 sub-tile.
    long long tile;
    const TraceParams& P = S.get(S.find(blockIdx.x, tile));
    const int twl = P.tile_w_log2, thl = P.tile_h_log2, wwl = P.warp_w_log2;
    const int tiles_x = (P.width + (1 << twl) - 1) >> twl;
    const int tx = (int)(tile % tiles_x), ty = (int)(tile / tiles_x);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int wxl = twl - wwl;  // log2 of warps per tile row
    const int x = (tx << twl) + ((wid & ((1 << wxl) - 1)) << wwl) + (lane & ((1 << wwl) - 1));
    const int y = (ty << thl) + ((wid >> wxl) << (5 - wwl)) + (lane >> wwl);
    // Offsets of the bordered levels (32-bit: the chain holds < 2^31 voxels).
    __shared__ int s_off[VCT_MAX_LEVELS];
    if (threadIdx.x < VCT_MAX_LEVELS)
        s_off[threadIdx.x] = threadIdx.x < P.levels ? (int)padded_level_offset(P.dim, threadIdx.x) : 0;
    __syncthreads();
    unsigned ns = 0;
    if (x < P.width && y < P.height) {
        const long long pix = (long long)y * P.width + x;
        float4 irr = make_float4(0.f, 0.f, 0.f, 0.f), spc = irr, out = irr;
        const float4 gp = __ldg(P.gpos + pix);
        if (gp.w != 0.0f) {
            const float4 gn = __ldg(P.gnrm + pix);
            const float4 ga = __ldg(P.galb + pix);
            const f3 N = fnormalize(mk(gn.x, gn.y, gn.z));
            f3 rgb;
            if (P.enable_indirect) {
                const f3 ext = sub(P.vmax, P.vmin);
                const f3 vp = mk(((gp.x - P.vcenter.x) - P.vmin.x) / ext.x, ((gp.y - P.vcenter.y) - P.vmin.y) / ext.y,
                                 ((gp.z - P.vcenter.z) - P.vmin.z) / ext.z);
                // Orthonormal basis from N: Duff et al. 2017, "Building an
                // Orthonormal Basis, Revisited" (JCGT 6(1)).
                const float sgn = N.z >= 0.0f ? 1.0f : -1.0f;
                const float ca = -1.0f / (sgn + N.z);
                const float cb = N.x * N.y * ca;
                const f3 T = mk(1.0f + sgn * N.x * N.x * ca, sgn * cb, -sgn * N.x);
                const f3 B = mk(cb, sgn + N.y * N.y * ca, -N.y);
                float4 ind = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 1
                for (int c = 0; c < 6; ++c) {
                    const float dx = kConeDir[c][0], dy = kConeDir[c][1], dz = kConeDir[c][2];
                    f3 d = P.ref_tbn_quirk ? add(add(mul(T, dx), mul(B, dy)), mul(N, dz))
                                           : sub(add(mul(T, dx), mul(N, dy)), mul(B, dz));
                    float4 cr = trace_cone<MODE>(P, s_off, vp, N, d, P.diffuse, P.max_distance, ns);
                    const float w = kConeWeight[c];
                    ind = make_float4(fmaf(w, cr.x, ind.x), fmaf(w, cr.y, ind.y), fmaf(w, cr.z, ind.z),
                                      fmaf(w, cr.w, ind.w));
                }
                irr = ind;
                const float occ = 1.0f - clampf(ind.w, 0.0f, 1.0f);
                rgb = mk(ind.x, ind.y, ind.z);
                if (P.enable_reflections) {
                    const f3 I = sub(mk(gp.x, gp.y, gp.z), P.eye);
                    const f3 R = sub(I, mul(N, 2.0f * dot(N, I)));
                    spc = trace_cone<MODE>(P, s_off, vp, N, R, P.specular_cone, P.max_distance, ns);
                    rgb = add(rgb, mul(mk(spc.x, spc.y, spc.z), P.reflect_scale));
                }
                const float as = P.ambient_scale;
                rgb = mk(rgb.x * (as * ga.x), rgb.y * (as * ga.y), rgb.z * (as * ga.z));
                if (P.draw_occlusion) rgb = mul(rgb, occ);
            } else {
                rgb = mk(P.ambient_scale * ga.x, P.ambient_scale * ga.y, P.ambient_scale * ga.z);
            }
            if (P.enable_postprocess) {
                const float g = 1.0f / 2.2f;
                rgb = mk(powf(rgb.x / (rgb.x + 1.0f), g), powf(rgb.y / (rgb.y + 1.0f), g),
                         powf(rgb.z / (rgb.z + 1.0f), g));
            }
            out = make_float4(rgb.x, rgb.y, rgb.z, 1.0f);
        }
        if (P.irradiance) P.irradiance[pix] = irr;
        if (P.specular) P.specular[pix] = spc;
        if (P.color) P.color[pix] = out;
    }
    if (P.samples) {
        unsigned tot = __reduce_add_sync(0xffffffffu, ns);
        if (lane == 0 && tot) atomicAdd(P.samples, (unsigned long long)tot);
    }
}

}  // namespace

template <class Scenes>
void launch_trace_set(const Scenes& S, int filter, long long tiles, cudaStream_t s) {
    if (tiles <= 0) return;
    if (filter == VCT_FILTER_HARDWARE)
        trace_kernel<VCT_FILTER_HARDWARE><<<(unsigned)tiles, 256, 0, s>>>(S);
    else if (filter == VCT_FILTER_HARDWARE_LEVELS)
        trace_kernel<VCT_FILTER_HARDWARE_LEVELS><<<(unsigned)tiles, 256, 0, s>>>(S);
    else
        trace_kernel<VCT_FILTER_SOFTWARE><<<(unsigned)tiles, 256, 0, s>>>(S);
    note_launches(1);
}

long long trace_tiles(int width, int height, int tile_w_log2, int tile_h_log2) {
    const long long tw = 1LL << tile_w_log2, th = 1LL << tile_h_log2;
    return ((width + tw - 1) / tw) * ((height + th - 1) / th);
}

void launch_trace(const TraceParams& P, cudaStream_t s) {
    launch_trace_set(OneScene<TraceParams>{P}, P.filter, trace_tiles(P.width, P.height, P.tile_w_log2, P.tile_h_log2),
                     s);
}

void launch_trace_batch(const SceneBatch<TraceParams>& B, int filter, long long tiles, cudaStream_t s) {
    launch_trace_set(ManyScenes<TraceParams>{B}, filter, tiles, s);
}

}  // namespace vct
