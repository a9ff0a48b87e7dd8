// Voxel cone tracing: shaders/phong.frag:135-180 (traceCone) and the
// indirect / specular / composite code of phong.frag:455-520.
//
// One thread per pixel; a 256-thread CTA shades a pixel tile (16x16 by
// default; the shape is a tuning setting) and each warp a sub-tile (8x4 by
// default), so the 32 lanes of a warp march neighbouring cones through
// neighbouring voxels at the same time (the cone step sequence depends only on
// the cone parameters, so every lane is at the same mip level each step).
// A lane leaves its cone at alpha >= 0.95 or on leaving the volume; the warp
// moves to the next cone once all lanes are done.
//
// Two samplers implement textureLod (cone.cuh): the software fp32 trilinear
// over a bordered fp32 copy of the chain (exact GL arithmetic), and the
// texture units (tex3DLod on a mip-mapped CUDA array, with their fixed-point
// filter weights).
//
// The file is compiled without FMA contraction: every fused multiply-add is
// written out (fmaf, __ffma2_rn), so the single-scene and the batched
// instantiations of the kernel give bit-identical results.
#include "cone.cuh"

namespace vct {

namespace {

using namespace cone;

__constant__ float kConeDir[6][3] = {{0.f, 1.f, 0.f},
                                     {0.f, 0.5f, 0.866025f},
                                     {0.823639f, 0.5f, 0.267617f},
                                     {0.509037f, 0.5f, -0.700629f},
                                     {-0.5909037f, 0.5f, -0.700629f},  // sic, phong.frag:475
                                     {-0.823639f, 0.5f, 0.267617f}};
__constant__ float kConeWeight[6] = {0.25f, 0.15f, 0.15f, 0.15f, 0.15f, 0.15f};

// Four resident CTAs per SM (64 registers): the cone march keeps the L1
// data pipe busy with its 16-byte texel loads (which mostly hit L1) and
// issues at about 60% of peak, and the extra warps hide the load latency.
template <int MODE, class Scenes>
__global__ void __launch_bounds__(256, 4) trace_kernel(const Scenes S) {
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
    __shared__ float s_tan[2];  // tanf of the diffuse and specular half-apertures
    if (threadIdx.x < VCT_MAX_LEVELS)
        s_off[threadIdx.x] = threadIdx.x < P.levels ? (int)padded_level_offset(P.dim, threadIdx.x) : 0;
    if (threadIdx.x == 32) s_tan[0] = tanf(P.diffuse.cone_angle * 0.5f);
    if (threadIdx.x == 64) s_tan[1] = tanf(P.specular_cone.cone_angle * 0.5f);
    __syncthreads();
    unsigned ns = 0;
    if (x < P.width && y < P.height) {
        const long long pix = (long long)y * P.width + x;
        float4 irr = make_float4(0.f, 0.f, 0.f, 0.f), spc = irr, out = irr;
        const float4 gp = __ldg(P.gpos + pix);
        if (gp.w != 0.0f) {
            const float4 gn = __ldg(P.gnrm + pix);
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
                    float4 cr = trace_cone<MODE>(P, s_off, vp, N, d, P.diffuse, P.max_distance, ns, s_tan[0]);
                    const float w = kConeWeight[c];
                    ind = make_float4(fmaf(w, cr.x, ind.x), fmaf(w, cr.y, ind.y), fmaf(w, cr.z, ind.z),
                                      fmaf(w, cr.w, ind.w));
                }
                irr = ind;
                const float occ = 1.0f - clampf(ind.w, 0.0f, 1.0f);
                rgb = mk(ind.x, ind.y, ind.z);
                if (P.enable_reflections) {
                    // the position is read again rather than kept live across the diffuse cones
                    const float4 gq = __ldg(P.gpos + pix);
                    const f3 I = sub(mk(gq.x, gq.y, gq.z), P.eye);
                    const f3 R = sub(I, mul(N, 2.0f * dot(N, I)));
                    spc = trace_cone<MODE>(P, s_off, vp, N, R, P.specular_cone, P.max_distance, ns, s_tan[1]);
                    rgb = add(rgb, mul(mk(spc.x, spc.y, spc.z), P.reflect_scale));
                }
                // the albedo is loaded after the cones: it is not live across them
                const float4 ga = __ldg(P.galb + pix);
                const float as = P.ambient_scale;
                rgb = mk(rgb.x * (as * ga.x), rgb.y * (as * ga.y), rgb.z * (as * ga.z));
                if (P.draw_occlusion) rgb = mul(rgb, occ);
            } else {
                const float4 ga = __ldg(P.galb + pix);
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

// Peak rate of textureLod samples (the denominator of the cone tracer's
// roofline): every thread takes `iters` samples with the tracer's sampler at
// positions inside one 8-voxel-wide region near the volume's centre, at the
// levels and fractions cone steps use, so the texels stay in L1 and nothing
// but sampling is timed.  The sum goes to `sink` so the work is kept.
template <int MODE>
__global__ void __launch_bounds__(256, 4) sampler_rate_kernel(const TraceParams P, int iters, float* sink) {
    __shared__ int s_off[VCT_MAX_LEVELS];
    if (threadIdx.x < VCT_MAX_LEVELS)
        s_off[threadIdx.x] = threadIdx.x < P.levels ? (int)padded_level_offset(P.dim, threadIdx.x) : 0;
    __syncthreads();
    const float span = 8.0f / (float)P.dim;
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    f3 p = mk(0.5f + span * (float)(t & 7) * 0.125f, 0.5f + span * (float)((t >> 3) & 7) * 0.125f,
              0.5f + span * (float)((t >> 6) & 7) * 0.125f);
    const f3 step = mk(span * 0.031f, span * 0.017f, span * 0.023f);
    const float top = (float)(P.levels - 1);
    float acc = 0.0f;
    for (int i = 0; i < iters; ++i) {
        const float lambda = fminf(0.1f + 0.37f * (float)(i & 7), top - 0.05f);
        const float4 v = sample_lod<MODE>(P, s_off, p, lambda);
        acc += v.x + v.y + v.z + v.w;
        p = add(p, step);
        if (p.x > 0.5f + span) p.x -= span;
        if (p.y > 0.5f + span) p.y -= span;
        if (p.z > 0.5f + span) p.z -= span;
    }
    sink[t] = acc;
}

}  // namespace

void launch_sampler_rate(const TraceParams& P, int filter, int blocks, int iters, float* sink, cudaStream_t s) {
    if (filter == VCT_FILTER_HARDWARE)
        sampler_rate_kernel<VCT_FILTER_HARDWARE><<<blocks, 256, 0, s>>>(P, iters, sink);
    else if (filter == VCT_FILTER_HARDWARE_LEVELS)
        sampler_rate_kernel<VCT_FILTER_HARDWARE_LEVELS><<<blocks, 256, 0, s>>>(P, iters, sink);
    else if (filter == VCT_FILTER_HYBRID)
        sampler_rate_kernel<VCT_FILTER_HYBRID><<<blocks, 256, 0, s>>>(P, iters, sink);
    else
        sampler_rate_kernel<VCT_FILTER_SOFTWARE><<<blocks, 256, 0, s>>>(P, iters, sink);
    note_launches(1);
}

template <class Scenes>
void launch_trace_set(const Scenes& S, int filter, long long tiles, cudaStream_t s) {
    if (tiles <= 0) return;
    if (filter == VCT_FILTER_HARDWARE)
        trace_kernel<VCT_FILTER_HARDWARE><<<(unsigned)tiles, 256, 0, s>>>(S);
    else if (filter == VCT_FILTER_HARDWARE_LEVELS)
        trace_kernel<VCT_FILTER_HARDWARE_LEVELS><<<(unsigned)tiles, 256, 0, s>>>(S);
    else if (filter == VCT_FILTER_HYBRID)
        trace_kernel<VCT_FILTER_HYBRID><<<(unsigned)tiles, 256, 0, s>>>(S);
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

void launch_trace_views(const ViewSet& V, int filter, cudaStream_t s) {
    launch_trace_set(FewScenes{V}, filter, V.off[V.n], s);
}

}  // namespace vct
