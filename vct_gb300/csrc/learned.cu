// Learned indirect light (the "learned" configuration): a cheap two-cone
// quarter-resolution trace plus G-buffer features feed a small BF16 MLP
// (42-64-64-64-4, FP32 accumulation) that predicts the 16-cone full-resolution
// irradiance and an estimate of its own error there.  Inference and training run on the fifth-generation tensor
// cores (tcgen05.mma, accumulators in TMEM; umma.cuh).
//
// Compiled with --fmad=false: the cone marching (cone.cuh) writes its fused
// multiply-adds out.
#include <cuda_bf16.h>

#include <cmath>

#include "cone.cuh"
#include "umma.cuh"

namespace vct {

namespace {

using namespace umma;

// ------------------------------------------------------------ GEMM check
// One 128 x N x K BF16 GEMM through the tensor core: A (128 x K) and B (N x K)
// row-major in global memory, D = A B^T (128 x N, FP32) back to global.
// `swap` exchanges the two descriptor strides (a diagnostic of the layout
// convention; both variants stay inside the zero-filled operand regions).
constexpr int kCheckSmemA = 32768, kCheckSmemB = 16384;

__global__ void __launch_bounds__(128) umma_check_kernel(const uint16_t* __restrict__ A,
                                                          const uint16_t* __restrict__ B, int K, int N, int swap,
                                                          float* __restrict__ D, uint32_t* __restrict__ status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint8_t* sa = smem;
    uint8_t* sb = smem + kCheckSmemA;
    for (int i = threadIdx.x; i < (kCheckSmemA + kCheckSmemB) / 16; i += blockDim.x)
        reinterpret_cast<uint4*>(smem)[i] = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    for (int i = threadIdx.x; i < 128 * K; i += blockDim.x)
        *reinterpret_cast<uint16_t*>(sa + tile_offset(i / K, i % K, 128)) = A[i];
    for (int i = threadIdx.x; i < N * K; i += blockDim.x)
        *reinterpret_cast<uint16_t*>(sb + tile_offset(i / K, i % K, N)) = B[i];
    fence_async_smem();
    if (threadIdx.x == 0) {
        mbar_init(smem_u32(&mbar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        tmem_alloc(smem_u32(&tmem_base), 64);
        tmem_relinquish();
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tbase = tmem_base;
    if (threadIdx.x == 0) {
        const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
        const uint32_t idesc = idesc_bf16_f32(128, N);
        for (int j = 0; j < K / 16; ++j) {
            const uint64_t da = swap ? smem_desc(a0 + j * 2 * 128 * 16, 128, 128 * 16) : tile_desc(a0, 128, j);
            const uint64_t db = swap ? smem_desc(b0 + j * 2 * N * 16, 128, N * 16) : tile_desc(b0, N, j);
            mma_bf16(tbase, da, db, idesc, j > 0 ? 1u : 0u);
        }
        commit(smem_u32(&mbar));
    }
    const int ok = __syncthreads_and(mbar_wait(smem_u32(&mbar), 0) ? 1 : 0);
    fence_after_sync();
    if (ok) {
        for (int c = 0; c < N; c += 16) {
            float v[16];
            tmem_ld16(tmem_addr(tbase, warp, c), v);
#pragma unroll
            for (int i = 0; i < 16; ++i) D[(32 * warp + lane) * N + c + i] = v[i];
        }
    } else if (threadIdx.x == 0) {
        atomicOr(status, 1u);
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tbase, 64);
}

// -------------------------------------------------------------- helpers
__device__ __forceinline__ uint32_t bf16x2(float a, float b) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&v);
}
// max(a, 0) and max(b, 0) rounded to BF16 and packed (a low): one
// conversion with ReLU, which commutes with round-to-nearest.
__device__ __forceinline__ uint32_t bf16x2_relu(float a, float b) {
    uint32_t r;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(b), "f"(a));
    return r;
}
__device__ __forceinline__ uint16_t bf16(float a) { return __bfloat16_as_ushort(__float2bfloat16_rn(a)); }
__device__ __forceinline__ float bf16f(uint32_t bits16) { return __uint_as_float(bits16 << 16); }

__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// Barrier that also orders tcgen05 operations across it.
__device__ __forceinline__ void tc_sync() {
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
}

// Orthonormal basis (T, B) around unit N: Duff et al. 2017, "Building an
// Orthonormal Basis, Revisited" (JCGT 6(1)), as the cone tracer uses it.
__device__ __forceinline__ void onb(f3 N, f3& T, f3& B) {
    const float sgn = N.z >= 0.0f ? 1.0f : -1.0f;
    const float ca = -1.0f / (sgn + N.z);
    const float cb = N.x * N.y * ca;
    T = mk(1.0f + sgn * N.x * N.x * ca, sgn * cb, -sgn * N.x);
    B = mk(cb, sgn + N.y * N.y * ca, -N.y);
}

// Position in [0,1]^3 volume texture coordinates (voxelLinearPosition).
__device__ __forceinline__ f3 volume_coord(const TraceParams& P, float4 gp) {
    const f3 ext = sub(P.vmax, P.vmin);
    return mk(((gp.x - P.vcenter.x) - P.vmin.x) / ext.x, ((gp.y - P.vcenter.y) - P.vmin.y) / ext.y,
              ((gp.z - P.vcenter.z) - P.vmin.z) / ext.z);
}

__device__ __forceinline__ void level_offsets(const TraceParams& P, int* s_off) {
    if (threadIdx.x < VCT_MAX_LEVELS)
        s_off[threadIdx.x] = (int)threadIdx.x < P.levels ? (int)padded_level_offset(P.dim, threadIdx.x) : 0;
}

// ------------------------------------------------------- cheap trace
// Quarter-resolution features: for each 4x4 pixel block, at its first
// covered pixel (centre pixels first), two 90-degree cones along
// normalize(N + T) and normalize(N - T).  With a 90-degree aperture a cone's
// diameter doubles every step, so step s (distance 2^s voxels past the
// one-voxel normal bias) is one trilinear sample of mip level s + 1.  Each
// cone marches 8 steps (levels 1..8, clamped to the chain), compositing front
// to back as traceCone does; its accumulated RGBA after the samples of levels
// 2, 4, 6 and 8 are the cone's 4 x 4 features.  A cone that leaves the volume
// keeps its accumulated value.
__constant__ unsigned char kRepOrder[16] = {5, 10, 6, 9, 0, 1, 2, 3, 4, 7, 8, 11, 12, 13, 14, 15};

__global__ void __launch_bounds__(256) learned_features_kernel(const LearnedParams P) {
    __shared__ int s_off[VCT_MAX_LEVELS];
    level_offsets(P.T, s_off);
    __syncthreads();
    const int qx = blockIdx.x * 16 + (threadIdx.x & 15), qy = blockIdx.y * 16 + (threadIdx.x >> 4);
    if (qx >= P.wq || qy >= P.hq) return;
    const TraceParams& T = P.T;
    float4 gp = make_float4(0.f, 0.f, 0.f, 0.f);
    long long pix = -1;
    for (int k = 0; k < 16 && pix < 0; ++k) {
        const int x = 4 * qx + (kRepOrder[k] & 3), y = 4 * qy + (kRepOrder[k] >> 2);
        if (x < T.width && y < T.height) {
            const long long p = (long long)y * T.width + x;
            gp = __ldg(T.gpos + p);
            if (gp.w != 0.0f) pix = p;
        }
    }
    uint32_t f[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) f[i] = 0u;
    if (pix >= 0) {
        const float4 gn = __ldg(T.gnrm + pix);
        const f3 N = cone::fnormalize(mk(gn.x, gn.y, gn.z));
        f3 Tg, Bg;
        onb(N, Tg, Bg);
        const f3 vp = volume_coord(T, gp);
        const float scale = 1.0f / (float)T.dim;
        const f3 start = add(vp, mul(N, scale));
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const f3 d = cone::fnormalize(c == 0 ? add(N, Tg) : sub(N, Tg));
            float h = 1.0f, alpha = 0.0f;
            f3 col = mk(0.f, 0.f, 0.f);
            bool inside = true;
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const f3 sp = mk(fmaf(d.x, h * scale, start.x), fmaf(d.y, h * scale, start.y),
                                 fmaf(d.z, h * scale, start.z));
                inside = inside && sp.x >= 0.f && sp.y >= 0.f && sp.z >= 0.f && sp.x <= 1.f && sp.y <= 1.f &&
                         sp.z <= 1.f;
                if (inside) {
                    const f3 wp = T.warp.mode ? apply_warp(T.warp, sp) : sp;
                    const float4 smp =
                        cone::trilinear(T, s_off, min(i + 1, T.levels - 1), wp, warp_leaves_volume(T.warp.mode));
                    const float a = 1.0f - alpha;
                    col = mk(fmaf(smp.x, a, col.x), fmaf(smp.y, a, col.y), fmaf(smp.z, a, col.z));
                    alpha = fmaf(a, smp.w, alpha);
                }
                if (i & 1) {
                    const int k = c * 8 + (i >> 1) * 2;
                    f[k] = bf16x2(col.x, col.y);
                    f[k + 1] = bf16x2(col.z, alpha);
                }
                h *= 2.0f;
            }
        }
    }
    uint4* dst = reinterpret_cast<uint4*>(const_cast<uint16_t*>(P.qfeat) + ((long long)qy * P.wq + qx) * kCheapFeatures);
#pragma unroll
    for (int i = 0; i < 4; ++i) dst[i] = make_uint4(f[4 * i], f[4 * i + 1], f[4 * i + 2], f[4 * i + 3]);
}

// The 42 features of pixel `pix` (covered: gp.w != 0) as 24 packed BF16
// pairs (48 features, the last 6 zero): the quarter-resolution cone features
// of its 4x4 block, the unit normal N, the eye distance times depth_scale,
// the albedo, and the near-field radiance RGB: one trilinear sample of mip
// level 1 where the diffuse cones take their first sample along N (two
// voxels above the surface), zero outside the volume.
__device__ __forceinline__ void pixel_features(const LearnedParams& P, long long pix, float4 gp, uint32_t (&f)[24]) {
    const TraceParams& T = P.T;
    const int x = (int)(pix % T.width), y = (int)(pix / T.width);
    const uint4* q =
        reinterpret_cast<const uint4*>(P.qfeat + ((long long)(y >> 2) * P.wq + (x >> 2)) * kCheapFeatures);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const uint4 v = __ldg(q + i);
        f[4 * i] = v.x;
        f[4 * i + 1] = v.y;
        f[4 * i + 2] = v.z;
        f[4 * i + 3] = v.w;
    }
    const float4 gn = __ldg(T.gnrm + pix);
    const float4 ga = __ldg(T.galb + pix);
    const f3 N = cone::fnormalize(mk(gn.x, gn.y, gn.z));
    const f3 d = sub(mk(gp.x, gp.y, gp.z), T.eye);
    const float dist = sqrtf(dot(d, d));
    const f3 vp = volume_coord(T, gp);
    const float step = 2.0f / (float)T.dim;
    const f3 sp = mk(fmaf(N.x, step, vp.x), fmaf(N.y, step, vp.y), fmaf(N.z, step, vp.z));
    float4 near = make_float4(0.f, 0.f, 0.f, 0.f);
    if (sp.x >= 0.f && sp.y >= 0.f && sp.z >= 0.f && sp.x <= 1.f && sp.y <= 1.f && sp.z <= 1.f) {
        const int off[2] = {(int)padded_level_offset(T.dim, 0), (int)padded_level_offset(T.dim, 1)};
        near = cone::trilinear(T, off, 1, T.warp.mode ? apply_warp(T.warp, sp) : sp, warp_leaves_volume(T.warp.mode));
    }
    f[16] = bf16x2(N.x, N.y);
    f[17] = bf16x2(N.z, dist * P.depth_scale);
    f[18] = bf16x2(ga.x, ga.y);
    f[19] = bf16x2(ga.z, near.x);
    f[20] = bf16x2(near.y, near.z);
    f[21] = f[22] = f[23] = 0u;
}

// Training rows: the 42 features of listed pixels as fp32 (exactly the BF16
// values the inference kernel feeds the network).
__global__ void __launch_bounds__(256) learned_rows_kernel(const LearnedParams P) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const long long pix = P.pixels[i];
    const float4 gp = __ldg(P.T.gpos + pix);
    float* row = P.rows_out + i * kMlpIn;
    if (gp.w == 0.0f) {
        for (int k = 0; k < kMlpIn; ++k) row[k] = 0.0f;
        return;
    }
    uint32_t f[24];
    pixel_features(P, pix, gp, f);
    for (int k = 0; k < kMlpIn; ++k) row[k] = bf16f((f[k >> 1] >> ((k & 1) * 16)) & 0xFFFFu);
}

// ------------------------------------------------------- 16-cone trace
// Irradiance of the 16-cone reference set: cones of the Fibonacci hemisphere
// set in the (T, B, N) frame, each weighted by its cosine, summed.
__device__ __forceinline__ float4 irradiance16(const LearnedParams& P, const int* off, const float (*dirs)[4],
                                               float4 gp, float4 gn, unsigned& ns) {
    const TraceParams& T = P.T;
    const f3 N = cone::fnormalize(mk(gn.x, gn.y, gn.z));
    f3 Tg, Bg;
    onb(N, Tg, Bg);
    const f3 vp = volume_coord(T, gp);
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 1
    for (int c = 0; c < 16; ++c) {
        const f3 d = add(add(mul(Tg, dirs[c][0]), mul(Bg, dirs[c][1])), mul(N, dirs[c][2]));
        const float4 cr = cone::trace_cone<VCT_FILTER_SOFTWARE>(T, off, vp, N, d, P.ref_cone, T.max_distance, ns);
        const float w = dirs[c][3];
        acc = make_float4(fmaf(w, cr.x, acc.x), fmaf(w, cr.y, acc.y), fmaf(w, cr.z, acc.z), fmaf(w, cr.w, acc.w));
    }
    return acc;
}

__device__ __forceinline__ void load_dirs(const LearnedParams& P, float (*s_dirs)[4]) {
    if (threadIdx.x < 64) s_dirs[threadIdx.x >> 2][threadIdx.x & 3] = P.dirs16[threadIdx.x >> 2][threadIdx.x & 3];
}

// 16-cone irradiance of whole 16x16 tiles (every tile, or the listed ones).
__global__ void __launch_bounds__(256) trace16_kernel(const LearnedParams P, int listed) {
    __shared__ int s_off[VCT_MAX_LEVELS];
    __shared__ float s_dirs[16][4];
    level_offsets(P.T, s_off);
    load_dirs(P, s_dirs);
    __syncthreads();
    const TraceParams& T = P.T;
    const int tiles_x = (T.width + kLearnTile - 1) / kLearnTile;
    const long long total = listed ? (long long)*P.count : (long long)tiles_x * ((T.height + kLearnTile - 1) / kLearnTile);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned ns = 0;
    for (long long t = blockIdx.x; t < total; t += gridDim.x) {
        const long long tile = listed ? (long long)P.list[t] : t;
        const int x = (int)(tile % tiles_x) * kLearnTile + (wid & 1) * 8 + (lane & 7);
        const int y = (int)(tile / tiles_x) * kLearnTile + (wid >> 1) * 4 + (lane >> 3);
        if (x >= T.width || y >= T.height) continue;
        const long long pix = (long long)y * T.width + x;
        const float4 gp = __ldg(T.gpos + pix);
        float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gp.w != 0.0f) r = irradiance16(P, s_off, s_dirs, gp, __ldg(T.gnrm + pix), ns);
        P.out[pix] = make_float4(r.x, r.y, r.z, 0.0f);
    }
}

// The per-pixel fallback's list: every covered pixel whose error estimate
// exceeds threshold x the frame's root-mean-square network irradiance over
// covered pixels.  A CTA scans a 16 x 16 pixel tile, each warp an 8 x 4
// part of it, and appends the tile's flagged pixels with one atomic, in
// warp order: the list holds them in 2D clusters whose cones march through
// neighbouring voxels when the fallback traces them.
__global__ void __launch_bounds__(256) learned_flag_kernel(const LearnedParams P) {
    const int W = P.T.width, H = P.T.height, tiles_x = (W + 15) / 16;
    const int tile = blockIdx.x, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int x = (tile % tiles_x) * 16 + (warp & 1) * 8 + (lane & 7);
    const int y = (tile / tiles_x) * 16 + (warp >> 1) * 4 + (lane >> 3);
    const long long i = (long long)y * W + x;
    const float n = P.frame_sums[1];
    const float bound = P.threshold * sqrtf(n > 0.0f ? P.frame_sums[0] / n : 0.0f);
    const bool fb = x < W && y < H && P.est[i] >= 0.0f && P.est[i] > bound;
    const unsigned m = __ballot_sync(0xffffffffu, fb);
    __shared__ uint32_t s_off[8], s_base;
    if (lane == 0) s_off[warp] = (uint32_t)__popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t tot = 0;
        for (int w = 0; w < 8; ++w) {
            const uint32_t c = s_off[w];
            s_off[w] = tot;
            tot += c;
        }
        s_base = tot ? atomicAdd(P.count, tot) : 0u;
    }
    __syncthreads();
    if (fb) P.list[s_base + s_off[warp] + __popc(m & ((1u << lane) - 1u))] = (uint32_t)i;
}

// 16-cone irradiance of the listed pixels (the per-pixel fallback), one
// thread per list entry; the grid covers the longest possible list and
// threads past the list's length return at once.
__global__ void __launch_bounds__(256, 4) trace16_pixels_kernel(const LearnedParams P) {
    __shared__ int s_off[VCT_MAX_LEVELS];
    __shared__ float s_dirs[16][4];
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if ((long long)blockIdx.x * blockDim.x >= (long long)*P.count) return;  // the whole CTA is past the list
    level_offsets(P.T, s_off);
    load_dirs(P, s_dirs);
    __syncthreads();
    if (i >= (long long)*P.count) return;
    const long long pix = (long long)P.list[i];
    unsigned ns = 0;
    const float4 r = irradiance16(P, s_off, s_dirs, __ldg(P.T.gpos + pix), __ldg(P.T.gnrm + pix), ns);
    P.out[pix] = make_float4(r.x, r.y, r.z, 0.0f);
}

// Per-tile error estimate of the network's output: the 16-cone irradiance at
// four probe pixels of each 16x16 tile (offsets 4 and 12 on each axis) against
// the network, relative L2 over the covered probes.  Tiles above the bound
// are listed for the 16-cone fallback.  One thread per (tile, probe, cone):
// a warp holds two probes' 16 cones, two warps a tile.
constexpr int kProbeThreads = 256;  // 4 tiles per CTA

__global__ void __launch_bounds__(kProbeThreads) learned_probe_kernel(const LearnedParams P) {
    __shared__ int s_off[VCT_MAX_LEVELS];
    __shared__ float s_dirs[16][4];
    __shared__ float s_part[kProbeThreads / 32][2];
    level_offsets(P.T, s_off);
    load_dirs(P, s_dirs);
    __syncthreads();
    const TraceParams& T = P.T;
    const int tiles_x = (T.width + kLearnTile - 1) / kLearnTile;
    const long long ntiles = (long long)tiles_x * ((T.height + kLearnTile - 1) / kLearnTile);
    const long long tile = (long long)blockIdx.x * (kProbeThreads / 64) + (threadIdx.x >> 6);
    const int pr = (threadIdx.x >> 4) & 3, c = threadIdx.x & 15;
    float4 rc = make_float4(0.f, 0.f, 0.f, 0.f);
    long long pix = -1;
    unsigned ns = 0;
    if (tile < ntiles) {
        const int x = (int)(tile % tiles_x) * kLearnTile + ((pr & 1) ? 12 : 4);
        const int y = (int)(tile / tiles_x) * kLearnTile + ((pr & 2) ? 12 : 4);
        if (x < T.width && y < T.height) {
            const long long p = (long long)y * T.width + x;
            const float4 gp = __ldg(T.gpos + p);
            if (gp.w != 0.0f) {
                pix = p;
                const float4 gn = __ldg(T.gnrm + p);
                const f3 N = cone::fnormalize(mk(gn.x, gn.y, gn.z));
                f3 Tg, Bg;
                onb(N, Tg, Bg);
                const f3 vp = volume_coord(T, gp);
                const f3 d = add(add(mul(Tg, s_dirs[c][0]), mul(Bg, s_dirs[c][1])), mul(N, s_dirs[c][2]));
                const float4 cr = cone::trace_cone<VCT_FILTER_SOFTWARE>(T, s_off, vp, N, d, P.ref_cone, T.max_distance, ns);
                const float w = s_dirs[c][3];
                rc = make_float4(w * cr.x, w * cr.y, w * cr.z, 0.0f);
            }
        }
    }
    // irradiance of the probe: the sum over its 16 lanes (an estimate: the
    // order differs from the 16-cone trace's sequential accumulation)
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) {
        rc.x += __shfl_xor_sync(0xffffffffu, rc.x, o);
        rc.y += __shfl_xor_sync(0xffffffffu, rc.y, o);
        rc.z += __shfl_xor_sync(0xffffffffu, rc.z, o);
    }
    float se = 0.0f, st = 0.0f;
    if (c == 0 && pix >= 0) {
        const float4 o = P.out[pix];
        const float dx = o.x - rc.x, dy = o.y - rc.y, dz = o.z - rc.z;
        se = dx * dx + dy * dy + dz * dz;
        st = rc.x * rc.x + rc.y * rc.y + rc.z * rc.z;
    }
    se += __shfl_xor_sync(0xffffffffu, se, 16);
    st += __shfl_xor_sync(0xffffffffu, st, 16);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_part[w][0] = se;
        s_part[w][1] = st;
    }
    __syncthreads();
    if ((threadIdx.x & 63) == 0 && tile < ntiles) {
        se = s_part[w][0] + s_part[w + 1][0];
        st = s_part[w][1] + s_part[w + 1][1];
        const float err = st > 0.0f ? sqrtf(se / st) : (se > 0.0f ? 1.0e30f : 0.0f);
        P.tile_err[tile] = err;
        if (err > P.threshold) P.list[atomicAdd(P.count, 1u)] = (uint32_t)tile;
    }
}

// ------------------------------------------------------- MLP inference
// A CTA holds the forward weights once in shared memory and runs kInferGroups
// independent groups of four warps; a group owns kInferTiles 128-pixel tiles
// at a time (one pixel of each per thread and per TMEM lane), 64 TMEM columns
// and an A-operand tile per tile, an mbarrier, and its own named barrier, so
// the groups' MMA chains and epilogues interleave on the SM.  Per layer the
// group's elected thread issues the K/16 MMAs of every tile (A = the tile's
// BF16 activations, B = the layer's weights) into the tiles' FP32
// accumulators and commits once to the group's mbarrier; every thread then
// loads its rows, adds the bias, applies ReLU and writes the BF16 rows back as
// the next layer's A operands.  Each wait and barrier thus serves kInferTiles
// tiles: the chain of MMA, commit, wait, barrier, TMEM load and epilogue is
// mostly latency, and one group's tiles share it.  The features of the
// group's next tiles are gathered while its first MMAs run.
constexpr int kInferGroups = 2;
constexpr int kInferTiles = 2;
constexpr int kInferThreads = 128 * kInferGroups;
constexpr int kInferTile = 128 * kMlpHidden * 2;
constexpr int kInferSmem = kImgFwd + kInferGroups * kInferTiles * kInferTile;
constexpr int kInferCols = 64 * kInferTiles * kInferGroups;  // TMEM columns per CTA
constexpr int kInferBlocksPerSM = 2;                        // 2 x 88 KB of shared memory, 2 x 256 TMEM columns

template <bool ROWS>
__device__ __forceinline__ bool gather_features(const LearnedParams& P, long long idx, uint32_t (&f)[24]) {
#pragma unroll
    for (int i = 0; i < 24; ++i) f[i] = 0u;
    if (idx >= P.n) return false;
    if (ROWS) {
        const float2* r = reinterpret_cast<const float2*>(P.rows + idx * kMlpIn);
#pragma unroll
        for (int i = 0; i < kMlpIn / 2; ++i) {
            const float2 v = __ldg(r + i);
            f[i] = bf16x2(v.x, v.y);
        }
        return true;
    }
    const float4 gp = __ldg(P.T.gpos + idx);
    if (gp.w == 0.0f) return false;
    pixel_features(P, idx, gp, f);
    return true;
}

template <bool ROWS>
__global__ void __launch_bounds__(kInferThreads, kInferBlocksPerSM) mlp_infer_kernel(const LearnedParams P) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(16) float s_bias[kBiasPad];
    __shared__ __align__(8) uint64_t mbar[kInferGroups];
    __shared__ uint32_t s_tmem;
    __shared__ int s_done[kInferGroups];
    const int tid = threadIdx.x, warp = tid >> 5, grp = warp >> 2, row = tid & 127;
    for (int i = tid; i < kImgFwd / 16; i += kInferThreads)
        reinterpret_cast<uint4*>(smem)[i] = __ldg(reinterpret_cast<const uint4*>(P.img) + i);
    for (int i = tid; i < kBiasPad; i += kInferThreads) s_bias[i] = P.bias[i];
    if (tid < kInferGroups) mbar_init(smem_u32(&mbar[tid]), 1);
    if (tid == 0) fence_mbar_init();
    if (warp == 0) {
        tmem_alloc(smem_u32(&s_tmem), kInferCols);
        tmem_relinquish();  // lets the SM's other CTAs allocate
    }
    fence_async_smem();
    tc_sync();
    // tile k of the group: A operand at sa[k], accumulator at TMEM columns tm[k]
    uint8_t* sa[kInferTiles];
    uint32_t tm[kInferTiles], a0[kInferTiles];
#pragma unroll
    for (int k = 0; k < kInferTiles; ++k) {
        sa[k] = smem + kImgFwd + (grp * kInferTiles + k) * kInferTile;
        a0[k] = smem_u32(sa[k]);
        tm[k] = s_tmem + 64u * (uint32_t)(grp * kInferTiles + k);
    }
    const uint32_t w0 = smem_u32(smem), mb = smem_u32(&mbar[grp]);
    const int bar = 1 + grp;
    const bool leader = row == 0;
    auto group_sync = [&]() {
        fence_before_sync();
        named_sync(bar, 128);
        fence_after_sync();
    };
    const long long ntiles = (P.n + 127) / 128;
    // the group's tiles: kInferTiles consecutive ones per step
    const long long stride = (long long)gridDim.x * kInferGroups * kInferTiles;
    uint32_t phase = 0;
    int ok = 1;
    long long t = ((long long)blockIdx.x * kInferGroups + grp) * kInferTiles;
    uint32_t f[kInferTiles][24];
    bool covered[kInferTiles];
#pragma unroll
    for (int k = 0; k < kInferTiles; ++k) covered[k] = gather_features<ROWS>(P, (t + k) * 128 + row, f[k]);
    float sum_sq = 0.0f, n_cov = 0.0f;
    for (; t < ntiles && ok; t += stride) {
        bool cov[kInferTiles];
#pragma unroll
        for (int k = 0; k < kInferTiles; ++k) {
            cov[k] = covered[k];
#pragma unroll
            for (int c = 0; c < 6; ++c)
                *reinterpret_cast<uint4*>(sa[k] + tile_offset(row, 8 * c, 128)) =
                    make_uint4(f[k][4 * c], f[k][4 * c + 1], f[k][4 * c + 2], f[k][4 * c + 3]);
        }
        fence_async_smem();
        group_sync();
        float o[kInferTiles][4];
#pragma unroll 1
        for (int layer = 0; layer < 4; ++layer) {
            const int K = layer == 0 ? kMlpInPad : kMlpHidden;
            const int N = layer == 3 ? kMlpOutPad : kMlpHidden;
            const uint32_t b = w0 + (layer == 0 ? kImgW1 : layer == 1 ? kImgW2 : layer == 2 ? kImgW3 : kImgW4);
            if (leader) {
                const uint32_t id = idesc_bf16_f32(128, N);
#pragma unroll
                for (int k = 0; k < kInferTiles; ++k)
                    for (int j = 0; j < K / 16; ++j)
                        mma_bf16(tm[k], tile_desc(a0[k], 128, j), tile_desc(b, N, j), id, j > 0);
                commit(mb);
            }
            // the next tiles' features load while the first layer runs
            if (layer == 0) {
#pragma unroll
                for (int k = 0; k < kInferTiles; ++k)
                    covered[k] = gather_features<ROWS>(P, (t + stride + k) * 128 + row, f[k]);
            }
            if (leader) s_done[grp] = mbar_wait(mb, phase) ? 1 : 0;
            phase ^= 1u;
            group_sync();
            ok = s_done[grp];
            if (!ok) break;
            if (layer < 3) {
                const float4* bb = reinterpret_cast<const float4*>(s_bias + kMlpHidden * layer);
#pragma unroll
                for (int k = 0; k < kInferTiles; ++k) {
#pragma unroll
                    for (int c = 0; c < kMlpHidden; c += 32) {
                        float v[32];
                        tmem_ld32(tmem_addr(tm[k], warp, c), v);
                        uint32_t pk[16];
                        // bias in packed FP32 pairs, then ReLU and rounding in one conversion
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            const float4 b4 = bb[c / 4 + i];
                            const float2 z0 = __fadd2_rn(make_float2(v[4 * i], v[4 * i + 1]), make_float2(b4.x, b4.y));
                            const float2 z1 = __fadd2_rn(make_float2(v[4 * i + 2], v[4 * i + 3]), make_float2(b4.z, b4.w));
                            pk[2 * i] = bf16x2_relu(z0.x, z0.y);
                            pk[2 * i + 1] = bf16x2_relu(z1.x, z1.y);
                        }
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            *reinterpret_cast<uint4*>(sa[k] + tile_offset(row, c + 8 * q, 128)) =
                                make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
                    }
                }
                fence_async_smem();
                group_sync();
            } else {
#pragma unroll
                for (int k = 0; k < kInferTiles; ++k) {
                    float v[16];
                    tmem_ld16(tmem_addr(tm[k], warp, 0), v);
#pragma unroll
                    for (int q = 0; q < 4; ++q) o[k][q] = v[q] + s_bias[3 * kMlpHidden + q];
                }
            }
        }
        if (!ok) break;
#pragma unroll
        for (int k = 0; k < kInferTiles; ++k) {
            const long long idx = (t + k) * 128 + row;
            if (idx >= P.n) continue;
            if (ROWS) {
                *reinterpret_cast<float4*>(P.out_rows + idx * 4) = make_float4(o[k][0], o[k][1], o[k][2], o[k][3]);
            } else {
                P.out[idx] = cov[k] ? make_float4(o[k][0], o[k][1], o[k][2], 0.0f) : make_float4(0.f, 0.f, 0.f, 0.f);
                if (P.est) {
                    // the per-pixel fallback's inputs: the error estimate (-1 for
                    // background) and the frame's sum of squared irradiance
                    P.est[idx] = cov[k] ? o[k][3] : -1.0f;
                    if (cov[k]) {
                        sum_sq += o[k][0] * o[k][0] + o[k][1] * o[k][1] + o[k][2] * o[k][2];
                        n_cov += 1.0f;
                    }
                }
            }
        }
    }
    if (P.est) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sum_sq += __shfl_xor_sync(0xffffffffu, sum_sq, o);
            n_cov += __shfl_xor_sync(0xffffffffu, n_cov, o);
        }
        if ((tid & 31) == 0 && n_cov > 0.0f) {
            atomicAdd(P.frame_sums, sum_sq);
            atomicAdd(P.frame_sums + 1, n_cov);
        }
    }
    if (!ok && leader) atomicOr(P.status, 1u);
    tc_sync();
    if (warp == 0) tmem_dealloc(s_tmem, kInferCols);
}

// ------------------------------------------------------- MLP training
// One CTA per SM (210 KB of shared memory, all 512 TMEM columns), 128
// samples per tile.  Forward as in inference, keeping each hidden layer's
// ReLU mask in registers and its BF16 activations transposed (features x
// samples) for the weight gradients.  Backward, per layer l:
//   dZ_l = (dZ_{l+1} W_{l+1}) * mask_l           (MMA into the 64 scratch columns)
//   dW_l^T += H_{l-1}^T dZ_l                     (MMA, accumulated in TMEM over the CTA's tiles)
// The transposed activation tiles are padded to 128 rows (M = 128) with one
// row of ones below the features, so the same MMA also accumulates the bias
// gradient.  At the end each CTA adds its TMEM gradients to the global fp32
// gradient with fire-and-forget atomics.  Loss: mean squared error over the
// n x 3 irradiance outputs, plus kMlpConfidenceWeight times the mean over the
// n samples of (e - |y - t|)^2, where e is the fourth output (the error
// estimate) and |y - t| the Euclidean error of the sample's irradiance, held
// constant (no gradient flows from this term into the irradiance outputs).
constexpr int kTrW = 0;
constexpr int kTrA = kImgAll;                      // 128 x 64 A operand
constexpr int kTrT = kTrA + 128 * 64 * 2;          // 4 transposed activation tiles, 128 x 128 each
constexpr int kTrTile = 128 * 128 * 2;
constexpr int kTrDZT = kTrT + 4 * kTrTile;         // 64 x 128
constexpr int kTrDYT = kTrDZT + 64 * 128 * 2;      // 16 x 128
constexpr int kTrDY = kTrDYT + 16 * 128 * 2;       // 128 x 16
constexpr int kTrSmem = kTrDY + 128 * 16 * 2;
static_assert(kTrSmem <= 227 * 1024 - 2048, "training tiles exceed shared memory");
// TMEM columns: scratch, dW1^T, dW2^T, dW3^T, dW4^T.
constexpr uint32_t kColFb = 0, kColW1 = 64, kColW2 = 128, kColW3 = 192, kColW4 = 256;
constexpr uint16_t kBf16One = 0x3F80u;

// Element (row, col) of an R-row operand tile.
__device__ __forceinline__ void st_t(uint8_t* base, int row, int col, uint16_t v, int R = 128) {
    *reinterpret_cast<uint16_t*>(base + tile_offset(row, col, R)) = v;
}

__global__ void __launch_bounds__(128, 1) mlp_train_kernel(const TrainParams P) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ float s_bias[kBiasPad];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t s_tmem;
    __shared__ float s_loss[4], s_closs[4];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int i = tid; i < kImgAll / 16; i += 128)
        reinterpret_cast<uint4*>(smem + kTrW)[i] = __ldg(reinterpret_cast<const uint4*>(P.mlp.img) + i);
    for (int i = tid; i < kBiasPad; i += 128) s_bias[i] = P.mlp.bias[i];
    for (int i = tid; i < (kTrSmem - kTrT) / 16; i += 128)
        reinterpret_cast<uint4*>(smem + kTrT)[i] = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    uint8_t* sa = smem + kTrA;
    uint8_t* T0 = smem + kTrT;
    uint8_t* Th[3] = {smem + kTrT + kTrTile, smem + kTrT + 2 * kTrTile, smem + kTrT + 3 * kTrTile};
    uint8_t* dzt = smem + kTrDZT;
    uint8_t* dyt = smem + kTrDYT;
    uint8_t* dy = smem + kTrDY;
    // rows of ones: bias gradients
    st_t(T0, kMlpInPad, tid, kBf16One);
    for (int l = 0; l < 3; ++l) st_t(Th[l], kMlpHidden, tid, kBf16One);
    if (tid == 0) {
        mbar_init(smem_u32(&mbar), 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc(smem_u32(&s_tmem), 512);
        tmem_relinquish();
    }
    fence_async_smem();
    tc_sync();
    const uint32_t tm = s_tmem, mb = smem_u32(&mbar), w0 = smem_u32(smem + kTrW);
    const uint32_t a0 = smem_u32(sa), t0 = smem_u32(T0), dzt0 = smem_u32(dzt), dyt0 = smem_u32(dyt), dy0 = smem_u32(dy);
    const uint32_t th0[3] = {smem_u32(Th[0]), smem_u32(Th[1]), smem_u32(Th[2])};
    const uint32_t id64 = idesc_bf16_f32(128, 64), id16 = idesc_bf16_f32(128, 16);
    const long long ntiles = (P.n + 127) / 128;
    uint32_t phase = 0;
    int ok = 1;
    bool first = true;
    float loss = 0.0f, closs = 0.0f;

    // Issues nothing itself: waits for the MMAs committed by thread 0.
    auto wait_mma = [&]() -> int {
        int done = 1;
        if (tid == 0) {
            commit(mb);
            done = mbar_wait(mb, phase) ? 1 : 0;
        }
        phase ^= 1u;
        const int r = __syncthreads_and(done);
        fence_after_sync();
        return r;
    };

    for (long long t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const long long idx = t * 128 + tid;
        const bool valid = idx < P.n;
        const long long row = valid ? (P.index ? (long long)P.index[idx] : idx) : 0;
        // ---- input
        uint32_t f[24];
#pragma unroll
        for (int i = 0; i < 24; ++i) f[i] = 0u;
        if (valid) {
            const float2* r = reinterpret_cast<const float2*>(P.rows + row * kMlpIn);
#pragma unroll
            for (int i = 0; i < kMlpIn / 2; ++i) {
                const float2 v = __ldg(r + i);
                f[i] = bf16x2(v.x, v.y);
            }
        }
#pragma unroll
        for (int c = 0; c < 6; ++c)
            *reinterpret_cast<uint4*>(sa + tile_offset(tid, 8 * c, 128)) =
                make_uint4(f[4 * c], f[4 * c + 1], f[4 * c + 2], f[4 * c + 3]);
#pragma unroll
        for (int k = 0; k < kMlpIn; ++k) st_t(T0, k, tid, (uint16_t)((f[k >> 1] >> ((k & 1) * 16)) & 0xFFFFu));
        fence_async_smem();
        tc_sync();
        // ---- forward, hidden layers
        uint64_t mask[3] = {0, 0, 0};
#pragma unroll 1
        for (int layer = 0; layer < 3 && ok; ++layer) {
            const int K = layer == 0 ? kMlpInPad : kMlpHidden;
            const uint32_t b = w0 + (layer == 0 ? kImgW1 : layer == 1 ? kImgW2 : kImgW3);
            if (tid == 0)
                for (int j = 0; j < K / 16; ++j) mma_bf16(tm + kColFb, tile_desc(a0, 128, j), tile_desc(b, 64, j), id64, j > 0);
            if (!(ok = wait_mma())) break;
            const float* bb = s_bias + kMlpHidden * layer;
            uint64_t m = 0;
#pragma unroll
            for (int c = 0; c < kMlpHidden; c += 16) {
                float v[16];
                tmem_ld16(tmem_addr(tm + kColFb, warp, c), v);
                uint32_t pk[8];
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    v[i] = fmaxf(v[i] + bb[c + i], 0.0f);
                    if (v[i] > 0.0f) m |= 1ull << (c + i);
                }
#pragma unroll
                for (int i = 0; i < 8; ++i) pk[i] = bf16x2(v[2 * i], v[2 * i + 1]);
                *reinterpret_cast<uint4*>(sa + tile_offset(tid, c, 128)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                *reinterpret_cast<uint4*>(sa + tile_offset(tid, c + 8, 128)) = make_uint4(pk[4], pk[5], pk[6], pk[7]);
#pragma unroll
                for (int i = 0; i < 16; ++i) st_t(Th[layer], c + i, tid, (uint16_t)((pk[i >> 1] >> ((i & 1) * 16)) & 0xFFFFu));
            }
            mask[layer] = m;
            fence_async_smem();
            tc_sync();
        }
        if (!ok) break;
        // ---- output layer, loss and dY
        if (tid == 0)
            for (int j = 0; j < 4; ++j) mma_bf16(tm + kColFb, tile_desc(a0, 128, j), tile_desc(w0 + kImgW4, 16, j), id16, j > 0);
        if (!(ok = wait_mma())) break;
        {
            float v[16];
            tmem_ld16(tmem_addr(tm + kColFb, warp, 0), v);
            float d[4] = {0.f, 0.f, 0.f, 0.f};
            if (valid) {
                float e2 = 0.0f;
#pragma unroll
                for (int o = 0; o < 3; ++o) {
                    const float diff = (v[o] + s_bias[3 * kMlpHidden + o]) - __ldg(P.targets + row * 3 + o);
                    loss += diff * diff;
                    e2 += diff * diff;
                    d[o] = P.scale * diff;
                }
                // the error estimate's target |output - target| is a constant of the step
                const float dc = (v[3] + s_bias[3 * kMlpHidden + 3]) - sqrtf(e2);
                closs += dc * dc;
                d[3] = P.conf_scale * dc;
            }
            const uint32_t p01 = bf16x2(d[0], d[1]), p23 = bf16x2(d[2], d[3]);
            *reinterpret_cast<uint4*>(dy + tile_offset(tid, 0, 128)) = make_uint4(p01, p23, 0u, 0u);
            st_t(dyt, 0, tid, (uint16_t)(p01 & 0xFFFFu), 16);
            st_t(dyt, 1, tid, (uint16_t)(p01 >> 16), 16);
            st_t(dyt, 2, tid, (uint16_t)(p23 & 0xFFFFu), 16);
            st_t(dyt, 3, tid, (uint16_t)(p23 >> 16), 16);
        }
        fence_async_smem();
        tc_sync();
        // ---- backward
        // dW4^T += H3^T dY ; dH3 = dY W4
        if (tid == 0) {
            for (int j = 0; j < 8; ++j)
                mma_bf16(tm + kColW4, tile_desc(th0[2], 128, j), tile_desc(dyt0, 16, j), id16, (!first || j > 0) ? 1u : 0u);
            mma_bf16(tm + kColFb, tile_desc(dy0, 128, 0), tile_desc(w0 + kImgW4t, 64, 0), id64, 0u);
        }
        if (!(ok = wait_mma())) break;
#pragma unroll 1
        for (int layer = 2; layer >= 0; --layer) {
            // dZ_layer = dH * mask -> A operand (for dH of the layer below) and transposed (for dW)
#pragma unroll
            for (int c = 0; c < kMlpHidden; c += 16) {
                float v[16];
                tmem_ld16(tmem_addr(tm + kColFb, warp, c), v);
                uint32_t pk[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const float a = (mask[layer] >> (c + 2 * i)) & 1ull ? v[2 * i] : 0.0f;
                    const float b = (mask[layer] >> (c + 2 * i + 1)) & 1ull ? v[2 * i + 1] : 0.0f;
                    pk[i] = bf16x2(a, b);
                }
                if (layer > 0) {
                    *reinterpret_cast<uint4*>(sa + tile_offset(tid, c, 128)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                    *reinterpret_cast<uint4*>(sa + tile_offset(tid, c + 8, 128)) = make_uint4(pk[4], pk[5], pk[6], pk[7]);
                }
#pragma unroll
                for (int i = 0; i < 16; ++i)
                    *reinterpret_cast<uint16_t*>(dzt + tile_offset(c + i, tid, 64)) =
                        (uint16_t)((pk[i >> 1] >> ((i & 1) * 16)) & 0xFFFFu);
            }
            fence_async_smem();
            tc_sync();
            if (tid == 0) {
                // dW_layer^T += H_{layer-1}^T dZ_layer   (H_{-1} = X)
                const uint32_t hT = layer == 0 ? t0 : th0[layer - 1];
                const uint32_t col = layer == 0 ? kColW1 : layer == 1 ? kColW2 : kColW3;
                for (int j = 0; j < 8; ++j)
                    mma_bf16(tm + col, tile_desc(hT, 128, j), tile_desc(dzt0, 64, j), id64, (!first || j > 0) ? 1u : 0u);
                if (layer > 0) {
                    // dH_{layer-1} = dZ_layer W_layer
                    const uint32_t wt = w0 + (layer == 2 ? kImgW3t : kImgW2t);
                    for (int j = 0; j < 4; ++j)
                        mma_bf16(tm + kColFb, tile_desc(a0, 128, j), tile_desc(wt, 64, j), id64, j > 0);
                }
            }
            if (!(ok = wait_mma())) break;
        }
        first = false;
    }
    // ---- gradients out
    if (ok && !first) {
        float* g = P.mlp.grad;
        const int r = tid;  // TMEM lane = row of dW^T = input feature (or the bias row)
#pragma unroll 1
        for (int layer = 0; layer < 4; ++layer) {
            const int in = layer == 0 ? kMlpIn : kMlpHidden;
            const int bias_row = layer == 0 ? kMlpInPad : kMlpHidden;
            const int nout = layer == 3 ? kMlpOut : kMlpHidden;
            const uint32_t col = layer == 0 ? kColW1 : layer == 1 ? kColW2 : layer == 2 ? kColW3 : kColW4;
            const int offw = layer == 0 ? kOffW1 : layer == 1 ? kOffW2 : layer == 2 ? kOffW3 : kOffW4;
            const int offb = layer == 0 ? kOffB1 : layer == 1 ? kOffB2 : layer == 2 ? kOffB3 : kOffB4;
            for (int c = 0; c < (layer == 3 ? 16 : 64); c += 16) {
                float v[16];
                tmem_ld16(tmem_addr(tm + col, warp, c), v);
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const int o = c + i;
                    if (o >= nout) continue;
                    if (r < in) atomicAdd(g + offw + o * in + r, v[i]);
                    else if (r == bias_row) atomicAdd(g + offb + o, v[i]);
                }
            }
        }
    }
    // ---- loss
    for (int o = 16; o > 0; o >>= 1) {
        loss += __shfl_xor_sync(0xffffffffu, loss, o);
        closs += __shfl_xor_sync(0xffffffffu, closs, o);
    }
    if (lane == 0) {
        s_loss[warp] = loss;
        s_closs[warp] = closs;
    }
    if (!ok && tid == 0) atomicOr(P.status, 1u);
    tc_sync();
    if (tid == 0)
        atomicAdd(P.mlp.loss, (s_loss[0] + s_loss[1] + s_loss[2] + s_loss[3]) * (0.5f * P.scale) +
                                  (s_closs[0] + s_closs[1] + s_closs[2] + s_closs[3]) * (0.5f * P.conf_scale));
    if (warp == 0) tmem_dealloc(tm, 512);
}

// ------------------------------------------------------- optimiser
// Adam on the fp32 master parameters (optional), then the BF16 operand
// images and the padded bias vector the kernels read.
__global__ void mlp_update_kernel(const MlpDev M, float lr, float beta1, float beta2, float eps, float c1, float c2,
                                  int update) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kMlpParams) return;
    float w = M.params[i];
    if (update) {
        const float g = M.grad[i];
        const float m = beta1 * M.m[i] + (1.0f - beta1) * g;
        const float v = beta2 * M.v[i] + (1.0f - beta2) * g * g;
        M.m[i] = m;
        M.v[i] = v;
        w = w - lr * (m * c1) / (sqrtf(v * c2) + eps);
        M.params[i] = w;
    }
    const uint16_t h = bf16(w);
    uint8_t* img = M.img;
    if (i < kOffB1) {
        const int o = i / kMlpIn, f = i % kMlpIn;
        *reinterpret_cast<uint16_t*>(img + kImgW1 + tile_offset(o, f, 64)) = h;
    } else if (i < kOffW2) {
        M.bias[i - kOffB1] = w;
    } else if (i < kOffB2) {
        const int o = (i - kOffW2) / kMlpHidden, f = (i - kOffW2) % kMlpHidden;
        *reinterpret_cast<uint16_t*>(img + kImgW2 + tile_offset(o, f, 64)) = h;
        *reinterpret_cast<uint16_t*>(img + kImgW2t + tile_offset(f, o, 64)) = h;
    } else if (i < kOffW3) {
        M.bias[kMlpHidden + i - kOffB2] = w;
    } else if (i < kOffB3) {
        const int o = (i - kOffW3) / kMlpHidden, f = (i - kOffW3) % kMlpHidden;
        *reinterpret_cast<uint16_t*>(img + kImgW3 + tile_offset(o, f, 64)) = h;
        *reinterpret_cast<uint16_t*>(img + kImgW3t + tile_offset(f, o, 64)) = h;
    } else if (i < kOffW4) {
        M.bias[2 * kMlpHidden + i - kOffB3] = w;
    } else if (i < kOffB4) {
        const int o = (i - kOffW4) / kMlpHidden, f = (i - kOffW4) % kMlpHidden;
        *reinterpret_cast<uint16_t*>(img + kImgW4 + tile_offset(o, f, 16)) = h;
        *reinterpret_cast<uint16_t*>(img + kImgW4t + tile_offset(f, o, 64)) = h;
    } else {
        M.bias[3 * kMlpHidden + i - kOffB4] = w;
    }
}

}  // namespace

// The timeout path of the bounded waits: one thread waits on an mbarrier that
// nothing arrives on, gives up after `limit_ns` and records it in `status`,
// exactly as the MLP kernels do when an MMA never completes.
__global__ void wait_probe_kernel(uint32_t* status, unsigned long long limit_ns) {
    __shared__ __align__(8) uint64_t mbar;
    if (threadIdx.x == 0) {
        mbar_init(smem_u32(&mbar), 1);
        fence_mbar_init();
        if (!mbar_wait_for(smem_u32(&mbar), 0u, limit_ns)) atomicOr(status, 1u);
    }
}

void launch_wait_probe(uint32_t* status, unsigned long long limit_ns, cudaStream_t s) {
    wait_probe_kernel<<<1, 32, 0, s>>>(status, limit_ns);
    note_launches(1);
}

void launch_umma_check(const uint16_t* A, const uint16_t* B, int K, int N, int swap, float* D, uint32_t* status,
                       cudaStream_t s) {
    cudaFuncSetAttribute(umma_check_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kCheckSmemA + kCheckSmemB);
    umma_check_kernel<<<1, 128, kCheckSmemA + kCheckSmemB, s>>>(A, B, K, N, swap, D, status);
    note_launches(1);
}

void launch_learned_features(const LearnedParams& P, cudaStream_t s) {
    const dim3 grid((P.wq + 15) / 16, (P.hq + 15) / 16);
    learned_features_kernel<<<grid, 256, 0, s>>>(P);
    note_launches(1);
}

void launch_learned_rows(const LearnedParams& P, cudaStream_t s) {
    if (P.n <= 0) return;
    learned_rows_kernel<<<(unsigned)((P.n + 255) / 256), 256, 0, s>>>(P);
    note_launches(1);
}

void launch_mlp_infer(const LearnedParams& P, int num_sms, cudaStream_t s) {
    if (P.n <= 0) return;
    const long long tiles = (P.n + 127) / 128;
    // kInferBlocksPerSM resident CTAs per SM, each taking kInferGroups x kInferTiles tiles a step.
    const long long per_cta = (long long)kInferGroups * kInferTiles;
    const long long slots = (long long)num_sms * kInferBlocksPerSM * per_cta;
    const long long grid = (tiles < slots ? tiles + per_cta - 1 : slots) / per_cta;
    if (P.rows) {
        cudaFuncSetAttribute(mlp_infer_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kInferSmem);
        mlp_infer_kernel<true><<<(unsigned)grid, kInferThreads, kInferSmem, s>>>(P);
    } else {
        cudaFuncSetAttribute(mlp_infer_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kInferSmem);
        mlp_infer_kernel<false><<<(unsigned)grid, kInferThreads, kInferSmem, s>>>(P);
    }
    note_launches(1);
}

void launch_learned_probe(const LearnedParams& P, cudaStream_t s) {
    const long long tiles = (long long)((P.T.width + kLearnTile - 1) / kLearnTile) *
                            ((P.T.height + kLearnTile - 1) / kLearnTile);
    learned_probe_kernel<<<(unsigned)((tiles + kProbeThreads / 64 - 1) / (kProbeThreads / 64)), kProbeThreads, 0, s>>>(P);
    note_launches(1);
}

void launch_trace16(const LearnedParams& P, bool listed, int num_sms, cudaStream_t s) {
    const long long tiles = (long long)((P.T.width + kLearnTile - 1) / kLearnTile) *
                            ((P.T.height + kLearnTile - 1) / kLearnTile);
    // Persistent over the listed tiles: as many CTAs as fit (8 per SM).
    const long long cap = (long long)num_sms * 8;
    const long long grid = listed ? cap : (tiles < cap * 4 ? tiles : cap * 4);
    trace16_kernel<<<(unsigned)(grid > 0 ? grid : 1), 256, 0, s>>>(P, listed ? 1 : 0);
    note_launches(1);
}

void launch_trace16_pixels(const LearnedParams& P, cudaStream_t s) {
    const long long n = (long long)P.T.width * P.T.height;
    const long long tiles = (long long)((P.T.width + 15) / 16) * ((P.T.height + 15) / 16);  // one CTA each
    learned_flag_kernel<<<(unsigned)tiles, 256, 0, s>>>(P);
    trace16_pixels_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(P);
    note_launches(2);
}

void launch_mlp_train(const TrainParams& P, int num_sms, cudaStream_t s) {
    if (P.n <= 0) return;
    const long long tiles = (P.n + 127) / 128;
    const long long grid = tiles < num_sms ? tiles : num_sms;
    cudaFuncSetAttribute(mlp_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrSmem);
    mlp_train_kernel<<<(unsigned)grid, 128, kTrSmem, s>>>(P);
    note_launches(1);
}

void launch_mlp_update(const MlpDev& M, int step, float lr, float beta1, float beta2, float eps, int update,
                       cudaStream_t s) {
    const double c1 = update ? 1.0 / (1.0 - std::pow((double)beta1, (double)step)) : 1.0;
    const double c2 = update ? 1.0 / (1.0 - std::pow((double)beta2, (double)step)) : 1.0;
    mlp_update_kernel<<<(kMlpParams + 255) / 256, 256, 0, s>>>(M, lr, beta1, beta2, eps, (float)c1, (float)c2, update);
    note_launches(1);
}

}  // namespace vct
