// Volume passes: normalisation (transferVoxels.comp), radiance injection
// (injectRadiance.comp), the 2x2x2 box mip chain (filterRadiance.comp) and
// the fused resolve used by vct_frame.  Compiled with --fmad=false.
//
// Layout: RGBA16F voxels (8 bytes, handled as uint2), x fastest.  The dense
// passes walk 16^3 bricks, one CTA per brick, each thread owning runs of 4
// voxels along x: the occupancy and lit masks are read as 4-bit fields, only
// occupied voxels touch their 32-byte accumulator record, and the colour,
// normal and radiance outputs leave as 32-byte vector stores.  The fused
// resolve also reduces the brick's first four mip levels in shared memory.
#include "vct_device.cuh"

namespace vct {

namespace {

constexpr int kBrick = 16;
constexpr int kBrickVox = kBrick * kBrick * kBrick;  // 4096
constexpr int kThreads = 256;

__device__ __forceinline__ void block_stats(StatsDev* stats, uint32_t uniq, uint32_t mx, uint32_t flags) {
    uniq = __reduce_add_sync(0xffffffffu, uniq);
    mx = __reduce_max_sync(0xffffffffu, mx);
    flags = __reduce_or_sync(0xffffffffu, flags);
    __shared__ uint32_t s_u, s_m, s_f;
    if (threadIdx.x == 0) {
        s_u = 0;
        s_m = 0;
        s_f = 0;
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&s_u, uniq);
        atomicMax(&s_m, mx);
        atomicOr(&s_f, flags);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_u) atomicAdd(&stats->unique_voxels, s_u);
        if (s_m) atomicMax(&stats->max_fragments_per_voxel, s_m);
        if (s_f) atomicOr(&stats->error_flags, s_f);
    }
}

// Four consecutive binary16 RGBA voxels (32 bytes, 32-byte aligned: the
// first voxel's index is a multiple of 4) in one 256-bit store, so that every
// lane writes a whole sector.  Two 16-byte stores per lane left each warp
// instruction writing half of 32 sectors.
__device__ __forceinline__ void store4(uint2* dst, const uint2 v[4]) {
    asm volatile("st.global.v8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(dst), "r"(v[0].x), "r"(v[0].y),
                 "r"(v[1].x), "r"(v[1].y), "r"(v[2].x), "r"(v[2].y), "r"(v[3].x), "r"(v[3].y)
                 : "memory");
}

__device__ __forceinline__ bool in_grid(int x, int y, int z, int N) {
    return x >= 0 && y >= 0 && z >= 0 && x < N && y < N && z < N;
}

// radianceLighting branch (injectRadiance.comp:74-98).  With the temporal
// filter the relit colour mixes with `prev`, the radiance transferVoxels
// seeded this frame: rgb = (1 - decay) rgb + decay prev.rgb, alpha = prev.a.
// (The shader's stores race when several shadow texels reach one voxel; here
// every store reads the seeded value, which makes the result deterministic.)
__device__ __forceinline__ uint2 light_voxel(f3 light_vox, f3 light_int, uint2 color, uint2 normal, int x, int y,
                                             int z, bool temporal = false, float decay = 0.0f,
                                             uint2 prev = make_uint2(0u, 0u)) {
    float4 c = unpack_h4(color);
    float4 nn = unpack_h4(normal);
    f3 n = mk(2.0f * nn.x - 1.0f, 2.0f * nn.y - 1.0f, 2.0f * nn.z - 1.0f);
    f3 L = normalize(sub(light_vox, mk((float)x, (float)y, (float)z)));
    float diff = fmaxf(dot(n, L), 0.0f);
    float r = (diff * light_int.x) * c.x, g = (diff * light_int.y) * c.y, b = (diff * light_int.z) * c.z, a = c.w;
    if (temporal) {
        const float4 p = unpack_h4(prev);
        r = (1.0f - decay) * r + decay * p.x;
        g = (1.0f - decay) * g + decay * p.y;
        b = (1.0f - decay) * b + decay * p.z;
        a = p.w;
    }
    return pack_h4(r, g, b, a);
}

// voxelIndex(lightPos) (injectRadiance.comp:80): computed on the host without
// warping, on the device with it (the warp map lives on the device).
__device__ __forceinline__ f3 light_voxel_index(const WarpDev& W, f3 light_vox, f3 light_tc, f3 light_pos, int N) {
    if (W.mode == VCT_WARP_NONE) return light_vox;
    const f3 t = W.mode == VCT_WARP_PERSPECTIVE ? perspective_tc(W, light_pos) : apply_warp(W, light_tc);
    return mk((float)N * t.x, (float)N * t.y, (float)N * t.z);
}

// -------------------------------------------------------------------- mips
// filterRadiance.comp BOX2: fp32 sum over the children in the shader's order
// (z fastest, then y, then x), times 0.125, rounded to binary16.
__device__ __forceinline__ uint2 box8(const uint2 c[8]) {
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        float4 t = unpack_h4(c[i]);
        acc.x += t.x;
        acc.y += t.y;
        acc.z += t.z;
        acc.w += t.w;
    }
    return pack_h4(acc.x * 0.125f, acc.y * 0.125f, acc.z * 0.125f, acc.w * 0.125f);
}

// Interior voxel (x,y,z) of a bordered level of side S.
__device__ __forceinline__ long long pad_index(int x, int y, int z, int S) {
    const long long P = S + 2;
    return ((long long)(z + 1) * P + (y + 1)) * P + (x + 1);
}

// Reduces a cube of side S (in shared memory, x fastest) into side S/2 with
// threads [0, nthr), writing the result to shared memory, to the linear level
// and, when given, to the texture-unit copy (`surf`) and the bordered fp32
// copy (`pdst`).
__device__ __forceinline__ void reduce_level(const uint2* src, uint2* dst, int S, uint2* gdst, cudaSurfaceObject_t surf,
                                             float4* pdst, int gS, int gx0, int gy0, int gz0, int nthr) {
    const int D = S / 2;
    const int n = D * D * D;
    for (int t = threadIdx.x; t < n; t += nthr) {
        int x = t % D, y = (t / D) % D, z = t / (D * D);
        uint2 c[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            int ox = i >> 2, oy = (i >> 1) & 1, oz = i & 1;
            c[i] = src[((2 * z + oz) * S + (2 * y + oy)) * S + (2 * x + ox)];
        }
        uint2 r = box8(c);
        dst[t] = r;
        if (gdst) gdst[((long long)(gz0 + z) * gS + (gy0 + y)) * gS + (gx0 + x)] = r;
        if (surf) surf3Dwrite(r, surf, (gx0 + x) * (int)sizeof(uint2), gy0 + y, gz0 + z);
        if (pdst) pdst[pad_index(gx0 + x, gy0 + y, gz0 + z, gS)] = unpack_h4(r);
    }
}

// Levels 1..nlev of a 16^3 brick held in s0 (shared).  Threads retire as the
// levels shrink (512, 64, 8, 1 outputs): after the first level only two warps
// continue (synchronised by a 64-thread named barrier), after the second one.
// Threads that are no longer needed return, so call this last.
__device__ __forceinline__ void brick_mips(uint2* s0, uint2* s1, int nlev, uint2* const* gdst,
                                           const cudaSurfaceObject_t* surf, float4* const* pdst, int S0, int bx, int by,
                                           int bz) {
    uint2* a = s0;
    uint2* b = s1;
    int side = kBrick;
    for (int l = 1; l <= nlev; ++l) {
        const int sub = side / 2;
        const int nout = sub * sub * sub;
        const int nthr = nout >= kThreads ? kThreads : (nout >= 64 ? 64 : 32);
        if ((int)threadIdx.x >= nthr) return;
        reduce_level(a, b, side, gdst[l], surf[l], pdst[l], S0 >> l, bx * sub, by * sub, bz * sub, nthr);
        if (nthr == kThreads)
            __syncthreads();
        else if (nthr == 64)
            asm volatile("bar.sync 1, 64;" ::: "memory");
        else
            __syncwarp();
        uint2* t = a;
        a = b;
        b = t;
        side = sub;
    }
}

// ----------------------------------------------------------- brick resolve
// FUSED = false: transferVoxels.comp (radiance level 0 = (0,0,0,alpha)).
// FUSED = true : additionally applies injectRadiance's stores (voxels marked
//                in the lit mask take their colour, or the relit colour) and
//                builds radiance levels 1..mip_levels of the brick.  The
//                result equals normalise; inject; filter because the value
//                injectRadiance stores into a voxel depends only on that
//                voxel (its stores are idempotent).
//
// EXACT = false: every brick the carry pass did not flag (all of them for
// the rasterising voxeliser).  EXACT = true: only the flagged bricks, whose
// rewritten records hold their sums' float values (bit 31 of the count);
// a separate instantiation so that the common path keeps its registers.
template <bool FUSED, bool EXACT, class Scenes>
__global__ void __launch_bounds__(kThreads, 3) resolve_kernel(const Scenes S) {
    __shared__ uint2 s0[FUSED ? kBrickVox : 1];
    __shared__ uint2 s1[FUSED ? kBrickVox / 8 : 1];
    long long brick;
    const ResolveParams& R = S.get(S.find(blockIdx.x, brick));
    const NormalizeParams& P = R.norm;
    if ((P.brick_exact ? P.brick_exact[brick] != 0u : false) != EXACT) return;  // the other pass's brick
    const int N = P.dim;
    const int bpa = N / kBrick;
    const int bx = (int)(brick % bpa), by = (int)((brick / bpa) % bpa), bz = (int)(brick / (bpa * bpa));
    const f3 lvox = FUSED ? light_voxel_index(R.warp, R.light_vox, R.light_tc, R.light_pos, N) : R.light_vox;
    uint32_t uniq = 0, mx = 0, flags = 0;
#pragma unroll 1
    for (int it = 0; it < kBrickVox / 4 / kThreads; ++it) {
        const int q = threadIdx.x + it * kThreads;
        const int lx = (q & 3) * 4, ly = (q >> 2) & 15, lz = q >> 6;
        const int x = bx * kBrick + lx, y = by * kBrick + ly, z = bz * kBrick + lz;
        const long long v0 = ((long long)z * N + y) * N + x;
        const uint32_t ob = (__ldg(P.occ + (v0 >> 5)) >> (v0 & 31)) & 15u;
        uint32_t lb = 0;
        if (FUSED) lb = (__ldg(R.lit + (v0 >> 5)) >> (v0 & 31)) & 15u;
        uint4 rec[4][2];
        // x is a multiple of 4: voxel x + j's record is (j & 1) + (j >> 1) N slots on
        uint4* recp = reinterpret_cast<uint4*>(P.acc + kAccWords * record_slot(v0, N));
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if ((ob >> j) & 1u) {  // the whole 32-byte record in one streaming load
                asm volatile("ld.global.cs.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                             : "=r"(rec[j][0].x), "=r"(rec[j][0].y), "=r"(rec[j][0].z), "=r"(rec[j][0].w),
                               "=r"(rec[j][1].x), "=r"(rec[j][1].y), "=r"(rec[j][1].z), "=r"(rec[j][1].w)
                             : "l"(recp + 2 * ((j & 1) + (j >> 1) * (long long)N)));
            } else {
                rec[j][0] = rec[j][1] = make_uint4(0u, 0u, 0u, 0u);
            }
        }
        uint4 prev[2] = {make_uint4(0u, 0u, 0u, 0u), make_uint4(0u, 0u, 0u, 0u)};
        if (P.temporal) {
            const uint4* rp = reinterpret_cast<const uint4*>(P.radiance + v0);
            prev[0] = rp[0];
            prev[1] = rp[1];
        }
        uint2 col[4], nrm[4], rad[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            // EXACT: bit 31 of the count says the six sums hold the float values
            // of their 64-bit sums (records the carry pass rewrote)
            const bool fbits = EXACT && (rec[j][0].x >> 31) != 0u;
            const uint32_t c = EXACT ? rec[j][0].x & 0x7fffffffu : rec[j][0].x;
            float alpha = 0.0f;
            col[j] = make_uint2(0u, 0u);
            nrm[j] = make_uint2(0u, 0u);
            if ((ob >> j) & 1u) {
                // zeroed for the next frame's accumulation, in one streaming store
                asm volatile("st.global.cs.v8.b32 [%0], {%1, %1, %1, %1, %1, %1, %1, %1};"
                             ::"l"(recp + 2 * ((j & 1) + (j >> 1) * (long long)N)), "r"(0u)
                             : "memory");
                ++uniq;
                mx = max(mx, c);
                // transferVoxels.comp:37-51: colour / count, opacity override.
                const float denom = 65535.0f * __uint2float_rn(c);
                alpha = P.opacity > 0.0f ? P.opacity : 1.0f;
                if (c >= VCT_MAX_EXACT_FRAGMENTS && !P.brick_exact) flags |= VCT_STATS_COUNT_OVERFLOW;
                if (EXACT) {
                    auto sum = [fbits](uint32_t f) { return fbits ? __uint_as_float(f) : __uint2float_rn(f); };
                    col[j] = pack_h4(__fdiv_rn(sum(rec[j][0].y), denom), __fdiv_rn(sum(rec[j][0].z), denom),
                                     __fdiv_rn(sum(rec[j][0].w), denom), alpha);
                    nrm[j] = pack_h4(__fdiv_rn(sum(rec[j][1].x), denom), __fdiv_rn(sum(rec[j][1].y), denom),
                                     __fdiv_rn(sum(rec[j][1].z), denom), 1.0f);
                } else {
                    col[j] = pack_h4(__fdiv_rn(__uint2float_rn(rec[j][0].y), denom),
                                     __fdiv_rn(__uint2float_rn(rec[j][0].z), denom),
                                     __fdiv_rn(__uint2float_rn(rec[j][0].w), denom), alpha);
                    nrm[j] = pack_h4(__fdiv_rn(__uint2float_rn(rec[j][1].x), denom),
                                     __fdiv_rn(__uint2float_rn(rec[j][1].y), denom),
                                     __fdiv_rn(__uint2float_rn(rec[j][1].z), denom), 1.0f);
                }
            }
            // transferVoxels.comp:53-62: radiance seed.
            if (P.temporal) {
                const float w = 1.0f - P.decay;
                const uint2 pv = (j & 1) ? make_uint2(prev[j >> 1].z, prev[j >> 1].w)
                                         : make_uint2(prev[j >> 1].x, prev[j >> 1].y);
                const float4 p4 = unpack_h4(pv);
                rad[j] = pack_h4(p4.x * (1.0f - w) + 0.0f * w, p4.y * (1.0f - w) + 0.0f * w,
                                 p4.z * (1.0f - w) + 0.0f * w, p4.w * (1.0f - w) + alpha * w);
            } else {
                rad[j] = ((ob >> j) & 1u) ? pack_h4(0.0f, 0.0f, 0.0f, alpha) : make_uint2(0u, 0u);
            }
            if (FUSED && ((lb >> j) & 1u))
                rad[j] = (R.lighting && !R.dilate) ? light_voxel(lvox, R.light_int, col[j], nrm[j], x + j, y, z,
                                                                 P.temporal != 0, P.decay, rad[j])
                                                   : col[j];
        }
        store4(P.color + v0, col);
        store4(P.normal + v0, nrm);
        // the fused frame may leave the linear copy of level 0 to the texture array
        if (!FUSED || R.radiance_levels[0]) store4((FUSED ? R.radiance_levels[0] : P.radiance) + v0, rad);
        if (FUSED) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                s0[(lz * kBrick + ly) * kBrick + lx + j] = rad[j];
                if (R.surf[0]) surf3Dwrite(rad[j], R.surf[0], (x + j) * (int)sizeof(uint2), y, z);
            }
        }
    }
    if (FUSED) __syncthreads();
    if (FUSED && R.pad_levels[0]) {
        // The sampler's bordered copy of level 0 from the brick in shared
        // memory: each half-warp writes one row of 16 texels (256 bytes).
        for (int t = threadIdx.x; t < kBrickVox; t += kThreads)
            R.pad_levels[0][pad_index(bx * kBrick + (t & 15), by * kBrick + ((t >> 4) & 15), bz * kBrick + (t >> 8), N)] =
                unpack_h4(s0[t]);
    }
    block_stats(P.stats, uniq, mx, flags);
    if (FUSED) {
        brick_mips(s0, s1, R.mip_levels, R.radiance_levels, R.surf, R.pad_levels, N, bx, by, bz);
    }
}

// ------------------------------------------------------------- injection
// injectRadiance.comp:40-56: texel -> voxel.  Returns false when the shader
// would return early.
__device__ __forceinline__ bool inject_voxel(const InjectParams& P, int x, int y, int& ix, int& iy, int& iz) {
    float u = __fdiv_rn((float)x, (float)P.sw), v = __fdiv_rn((float)y, (float)P.sh);
    float depth = shadow_bilinear(P.shadowmap, P.sw, P.sh, u, v, 0, 0);
    float ndx = u * 2.0f - 1.0f, ndy = v * 2.0f - 1.0f, ndz = depth * 2.0f - 1.0f;
    float w[4];
    mat_vec(P.ls_inverse, ndx, ndy, ndz, 1.0f, w);
    f3 ext = sub(P.vmax, P.vmin);
    float N = (float)P.dim;
    float tx = __fdiv_rn((w[0] - P.vcenter.x) - P.vmin.x, ext.x);
    float ty = __fdiv_rn((w[1] - P.vcenter.y) - P.vmin.y, ext.y);
    float tz = __fdiv_rn((w[2] - P.vcenter.z) - P.vmin.z, ext.z);
    if (P.warp.mode != VCT_WARP_NONE) {  // getVoxelPosition (common.glsl:44-60)
        const f3 t = P.warp.mode == VCT_WARP_PERSPECTIVE ? perspective_tc(P.warp, mk(w[0], w[1], w[2]))
                                                         : apply_warp(P.warp, mk(tx, ty, tz));
        tx = t.x;
        ty = t.y;
        tz = t.z;
    }
    ix = __float2int_rz(tx * N);
    iy = __float2int_rz(ty * N);
    iz = __float2int_rz(tz * N);
    return !(ix >= P.dim || iy >= P.dim || iz >= P.dim || ix < 0 || iy < 0 || iz < 0);
}

// injectRadiance.comp:58-72, sic: (-1,0,0) twice and no (0,0,-1).
__constant__ int kDilate[7][3] = {{0, 0, 0}, {0, 0, 1}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {1, 0, 0}, {-1, 0, 0}};

__global__ void __launch_bounds__(kThreads) inject_kernel(const InjectParams P) {
    int x = blockIdx.x * 16 + (threadIdx.x & 15);
    int y = blockIdx.y * 16 + (threadIdx.x >> 4);
    if (x >= P.nx || y >= P.ny) return;
    int ix, iy, iz;
    if (!inject_voxel(P, x, y, ix, iy, iz)) return;
    const int N = P.dim;
    if (P.dilate) {
        for (int k = 0; k < 7; ++k) {
            int a = ix + kDilate[k][0], b = iy + kDilate[k][1], c = iz + kDilate[k][2];
            if (!in_grid(a, b, c, N)) continue;
            long long v = ((long long)c * N + b) * N + a;
            P.radiance[v] = P.color[v];
        }
        return;
    }
    long long v = ((long long)iz * N + iy) * N + ix;
    if (P.lighting)
        P.radiance[v] = light_voxel(light_voxel_index(P.warp, P.light_vox, P.light_tc, P.light_pos, N), P.light_int, P.color[v],
                                    P.normal[v], ix, iy, iz);
    else
        P.radiance[v] = P.color[v];
}

// Fused path: mark the voxels injectRadiance would store to.  One thread per
// shadow texel over the texels of every scene of the launch.
template <class Scenes>
__global__ void __launch_bounds__(kThreads) inject_mark_kernel(const Scenes S, long long ntexels) {
    const long long g = (long long)blockIdx.x * kThreads + threadIdx.x;
    if (g >= ntexels) return;
    long long local;
    const InjectParams& P = S.get(S.find(g, local));
    const int y = (int)(local / P.nx), x = (int)(local - (long long)y * P.nx);
    int ix, iy, iz;
    if (!inject_voxel(P, x, y, ix, iy, iz)) return;
    const int N = P.dim;
    const int nk = P.dilate ? 7 : 1;
    for (int k = 0; k < nk; ++k) {
        int a = ix + kDilate[k][0], b = iy + kDilate[k][1], c = iz + kDilate[k][2];
        if (!in_grid(a, b, c, N)) continue;
        long long v = ((long long)c * N + b) * N + a;
        // Many texels land in one voxel (with a warp map, distant surfaces
        // compress into few voxels), and their ORs on one word serialise in
        // L2.  The mask only gains bits during the pass, so a texel that
        // already sees its bit set skips the atomic; a stale read only costs
        // a redundant OR.
        uint32_t* w = P.lit + (v >> 5);
        const uint32_t bit = 1u << (v & 31);
        if (!(__ldcg(w) & bit)) atomicOr(w, bit);
    }
}

// One 16^3 brick of level `first` -> up to 4 coarser levels.
__global__ void __launch_bounds__(kThreads) mip_brick_kernel(const MipLevels M, int first, int nlev) {
    __shared__ uint2 s0[kBrickVox];
    __shared__ uint2 s1[kBrickVox / 8];
    const int S = M.dim >> first;
    const int bpa = S / kBrick;
    const int bx = blockIdx.x % bpa, by = (blockIdx.x / bpa) % bpa, bz = blockIdx.x / (bpa * bpa);
    const uint2* src = M.level[first];
    for (int t = threadIdx.x; t < kBrickVox; t += kThreads) {
        int x = t & 15, y = (t >> 4) & 15, z = t >> 8;
        s0[t] = src[((long long)(bz * kBrick + z) * S + (by * kBrick + y)) * S + (bx * kBrick + x)];
    }
    __syncthreads();
    brick_mips(s0, s1, nlev, M.level + first, M.surf + first, M.pad + first, S, bx, by, bz);
}

// Small levels (side <= 16): one CTA per scene builds every level after
// M.first.
template <class Scenes>
__global__ void __launch_bounds__(kThreads) mip_tail_kernel(const Scenes SS) {
    __shared__ uint2 s0[kBrickVox];
    __shared__ uint2 s1[kBrickVox / 8];
    const MipLevels& M = SS.get(blockIdx.x);
    const int first = M.first;
    // Chains of at most five levels are complete after the resolve; the tail
    // (side of level `first` <= 16) only exists for longer ones.
    if (first + 1 >= M.levels) return;
    const int S = M.dim >> first;
    const uint2* src = M.level[first];
    for (int t = threadIdx.x; t < S * S * S; t += kThreads) s0[t] = src[t];
    __syncthreads();
    uint2* a = s0;
    uint2* b = s1;
    int side = S;
    for (int l = first + 1; l < M.levels; ++l) {
        reduce_level(a, b, side, M.level[l], M.surf[l], M.pad[l], side / 2, 0, 0, 0, kThreads);
        __syncthreads();
        uint2* t = a;
        a = b;
        b = t;
        side /= 2;
    }
}

// Linear level -> interior of the bordered level (borders stay zero).
__global__ void pad_copy_kernel(const uint2* __restrict__ src, float4* __restrict__ dst, int S) {
    const long long n = (long long)S * S * S;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(v % S), y = (int)((v / S) % S), z = (int)(v / ((long long)S * S));
        dst[pad_index(x, y, z, S)] = unpack_h4(src[v]);
    }
}

__global__ void fill_u32_kernel(uint32_t* p, uint32_t v, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        p[i] = v;
}

// Stage-path injection through the lit mask: one thread per 4 voxels along x.
__global__ void __launch_bounds__(kThreads) inject_apply_kernel(const InjectParams P) {
    const int N = P.dim;
    const long long nq = (long long)N * N * N / 4;
    const f3 lvox = light_voxel_index(P.warp, P.light_vox, P.light_tc, P.light_pos, N);
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += (long long)gridDim.x * blockDim.x) {
        const long long v0 = q * 4;
        const uint32_t lb = (__ldg(P.lit + (v0 >> 5)) >> (v0 & 31)) & 15u;
        if (!lb) continue;
        const int x = (int)(v0 % N), y = (int)((v0 / N) % N), z = (int)(v0 / ((long long)N * N));
        for (int j = 0; j < 4; ++j) {
            if (!((lb >> j) & 1u)) continue;
            const long long v = v0 + j;
            P.radiance[v] = (P.lighting && !P.dilate) ? light_voxel(lvox, P.light_int, P.color[v], P.normal[v], x + j,
                                                                     y, z, P.temporal != 0, P.decay, P.radiance[v])
                                                      : P.color[v];
        }
    }
}

__global__ void decay_kernel(uint2* radiance, long long nv, float decay) {
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += (long long)gridDim.x * blockDim.x) {
        const float4 c = unpack_h4(radiance[v]);
        radiance[v] = pack_h4(c.x * decay, c.y * decay, c.z * decay, c.w * decay);
    }
}

// voxelize.vert:15-22 for rigid actors: one thread per triangle.
__global__ void transform_actors_kernel(const ActorsDev A) {
    const long long t0 = A.start[0], t1 = A.end[A.n - 1];
    for (long long t = t0 + (long long)blockIdx.x * blockDim.x + threadIdx.x; t < t1;
         t += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = A.n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (A.start[mid] <= t)
                lo = mid;
            else
                hi = mid - 1;
        }
        if (t >= A.end[lo]) continue;  // between two actors' ranges
        const float* M = A.model[lo];
        const float* Nm = A.normal[lo];
        for (int k = 0; k < 3; ++k) {
            const float* p = A.src_pos + t * 9 + 3 * k;
            const float* n = A.src_nrm + t * 9 + 3 * k;
            float o[4];
            mat_vec(M, p[0], p[1], p[2], 1.0f, o);
            float* dp = A.dst_pos + t * 9 + 3 * k;
            dp[0] = o[0];
            dp[1] = o[1];
            dp[2] = o[2];
            float* dn = A.dst_nrm + t * 9 + 3 * k;
            for (int r = 0; r < 3; ++r) dn[r] = Nm[0 + r] * n[0] + Nm[3 + r] * n[1] + Nm[6 + r] * n[2];
        }
    }
}

// ------------------------------------------------------------- warp map
// Application.cpp:300-371 + generateWarpmapWeights.frag + generateWarpmap.frag
// for the 32^3 warp map: per-axis inclusive prefix counts of the occupancy,
// the per-row resolution weights (high for occupied cells, low for empty
// ones, keeping each row's total of 32; stored as binary16 by the weight
// textures), and per texel the warped coordinate of its cell centre, stored
// RGBA16 unorm.  One CTA per z slice, one thread per cell: a row of the
// occupancy is one 32-bit word, so the x counts are population counts, and
// the y and z counts walk the 4 KB mask, held in shared memory by every CTA.
__device__ __forceinline__ void warpmap_slice(const WarpmapArgs& A, int z) {
    constexpr int D = kWarpDim;
    static_assert(D == 32, "a warp-map row is one 32-bit occupancy word");
    __shared__ uint32_t occ[D * D];   // word (z * D + y): row (y, z), bit x
    __shared__ float wts[2][D + 1];  // binary16-rounded low / high weights per occupied count
    const int t = threadIdx.x;
    occ[t] = A.occ[t];
    if (t <= D) {
        float l = 1.0f, h = 1.0f;
        if (t != 0 && t != D) {
            const int occupied = t, empty = D - t, total = D;
            h = A.high;
            l = ((float)total - h * (float)occupied) / (float)empty;
            if (l < A.low) {
                l = A.low;
                h = ((float)total - l * (float)empty) / (float)occupied;
            }
        }
        wts[0][t] = __half2float(__float2half_rn(l));
        wts[1][t] = __half2float(__float2half_rn(h));
    }
    __syncthreads();
    const int x = t & (D - 1), y = t >> 5;
    const uint32_t row = occ[z * D + y];
    const bool o = ((row >> x) & 1u) != 0u;
    // inclusive prefix counts along x, y, z and each line's total
    int ps[3], tot[3];
    ps[0] = __popc(row & (0xffffffffu >> (31 - x)));
    tot[0] = __popc(row);
    int cy = 0, cz = 0;
    ps[1] = ps[2] = 0;
#pragma unroll 8
    for (int k = 0; k < D; ++k) {
        cy += (occ[z * D + k] >> x) & 1u;
        cz += (occ[k * D + y] >> x) & 1u;
        if (k == y) ps[1] = cy;
        if (k == z) ps[2] = cz;
    }
    tot[1] = cy;
    tot[2] = cz;
    const int idx[3] = {x, y, z};
    uint16_t out[4];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float lo = wts[0][tot[k]], hi = wts[1][tot[k]];
        const float res = o ? hi : lo;
        const float prev = (float)(o ? ps[k] - 1 : ps[k]);
        const float offset = lo * ((float)idx[k] - prev) + hi * prev;
        const float inner = 0.5f * res;
        const float w = (offset + inner) / (float)D;
        out[k] = (uint16_t)__float2uint_rn(fminf(fmaxf(w, 0.0f), 1.0f) * 65535.0f);
    }
    // packCellInfo: totals (5 bits each) and the cell's occupancy
    out[3] = (uint16_t)((tot[0] & 0x1F) | ((tot[1] & 0x1F) << 5) | ((tot[2] & 0x1F) << 10) | ((o ? 1 : 0) << 15));
    const int i = (z * D + y) * D + x;
    reinterpret_cast<uint2*>(A.map)[i] =
        make_uint2((uint32_t)out[0] | ((uint32_t)out[1] << 16), (uint32_t)out[2] | ((uint32_t)out[3] << 16));
    const float4 f = make_float4(__fdiv_rn((float)out[0], 65535.0f), __fdiv_rn((float)out[1], 65535.0f),
                                 __fdiv_rn((float)out[2], 65535.0f), __fdiv_rn((float)out[3], 65535.0f));
    // the fp32 copy at (x+1, y+1, z+1), and on the border beside an edge
    // texel (clamp-to-edge): up to 8 places for a corner texel
    const int xs[2] = {x + 1, x == 0 ? 0 : x == D - 1 ? D + 1 : -1};
    const int ys[2] = {y + 1, y == 0 ? 0 : y == D - 1 ? D + 1 : -1};
    const int zs[2] = {z + 1, z == 0 ? 0 : z == D - 1 ? D + 1 : -1};
#pragma unroll
    for (int n = 0; n < 8; ++n) {
        const int bx = xs[n & 1], by = ys[(n >> 1) & 1], bz = zs[n >> 2];
        if (bx >= 0 && by >= 0 && bz >= 0) A.mapf[(bz * kWarpPad + by) * kWarpPad + bx] = f;
    }
}

__global__ void __launch_bounds__(kWarpDim * kWarpDim) warpmap_kernel(const WarpmapArgs A) {
    warpmap_slice(A, blockIdx.x);
}

// blockIdx.y: the scene of a batch; scenes without a texture warp have no map.
__global__ void __launch_bounds__(kWarpDim * kWarpDim) warpmap_batch_kernel(const WarpmapArgs* __restrict__ args) {
    const WarpmapArgs A = args[blockIdx.y];
    if (!A.map) return;
    warpmap_slice(A, blockIdx.x);
}

}  // namespace

void launch_warpmap(const uint32_t* occ32, float high, float low, uint16_t* map, float4* mapf, cudaStream_t s) {
    warpmap_kernel<<<kWarpDim, kWarpDim * kWarpDim, 0, s>>>(WarpmapArgs{occ32, high, low, map, mapf});
    note_launches(1);
}

void launch_warpmap_batch(const WarpmapArgs* args, int n, cudaStream_t s) {
    if (n <= 0) return;
    warpmap_batch_kernel<<<dim3(kWarpDim, n), kWarpDim * kWarpDim, 0, s>>>(args);
    note_launches(1);
}

void launch_normalize(const NormalizeParams& P, cudaStream_t s) {
    ResolveParams R;
    memset(&R, 0, sizeof R);
    R.norm = P;
    const int bpa = P.dim / kBrick;
    resolve_kernel<false, false><<<bpa * bpa * bpa, kThreads, 0, s>>>(OneScene<ResolveParams>{R});
    if (P.brick_exact) {
        resolve_kernel<false, true><<<bpa * bpa * bpa, kThreads, 0, s>>>(OneScene<ResolveParams>{R});
        note_launches(1);
    }
    note_launches(1);
}

void launch_inject(const InjectParams& P, cudaStream_t s) {
    dim3 grid((P.nx + 15) / 16, (P.ny + 15) / 16);
    inject_kernel<<<grid, kThreads, 0, s>>>(P);
    note_launches(1);
}

void launch_inject_apply(const InjectParams& P, cudaStream_t s) {
    const long long nq = (long long)P.dim * P.dim * P.dim / 4;
    long long blocks = (nq + kThreads - 1) / kThreads;
    if (blocks > 8192) blocks = 8192;
    inject_apply_kernel<<<(unsigned)blocks, kThreads, 0, s>>>(P);
    note_launches(1);
}

void launch_decay(uint2* radiance, long long nv, float decay, cudaStream_t s) {
    long long blocks = (nv + 255) / 256;
    if (blocks > 8192) blocks = 8192;
    decay_kernel<<<(unsigned)blocks, 256, 0, s>>>(radiance, nv, decay);
    note_launches(1);
}

void launch_transform_actors(const ActorsDev& A, cudaStream_t s) {
    if (A.n <= 0) return;
    const long long total = A.end[A.n - 1] - A.start[0];
    if (total <= 0) return;
    long long blocks = (total + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    transform_actors_kernel<<<(unsigned)blocks, 256, 0, s>>>(A);
    note_launches(1);
}

void launch_inject_mark(const InjectParams& P, cudaStream_t s) {
    const long long n = (long long)P.nx * P.ny;
    inject_mark_kernel<<<(unsigned)((n + kThreads - 1) / kThreads), kThreads, 0, s>>>(OneScene<InjectParams>{P}, n);
    note_launches(1);
}

void launch_resolve(const ResolveParams& R, cudaStream_t s) {
    const int bpa = R.norm.dim / kBrick;
    resolve_kernel<true, false><<<bpa * bpa * bpa, kThreads, 0, s>>>(OneScene<ResolveParams>{R});
    if (R.norm.brick_exact) {
        resolve_kernel<true, true><<<bpa * bpa * bpa, kThreads, 0, s>>>(OneScene<ResolveParams>{R});
        note_launches(1);
    }
    note_launches(1);
}

void launch_mips(const MipLevels& M, int first, cudaStream_t s) {
    int l = first;
    while (l + 1 < M.levels) {
        int S = M.dim >> l;
        if (S > kBrick) {
            int nlev = M.levels - 1 - l;
            if (nlev > 4) nlev = 4;
            int bpa = S / kBrick;
            mip_brick_kernel<<<bpa * bpa * bpa, kThreads, 0, s>>>(M, l, nlev);
            note_launches(1);
            l += nlev;
        } else {
            MipLevels T = M;
            T.first = l;
            mip_tail_kernel<<<1, kThreads, 0, s>>>(OneScene<MipLevels>{T});
            note_launches(1);
            break;
        }
    }
}

void launch_inject_mark_batch(const SceneBatch<InjectParams>& B, long long ntexels, cudaStream_t s) {
    if (ntexels <= 0) return;
    inject_mark_kernel<<<(unsigned)((ntexels + kThreads - 1) / kThreads), kThreads, 0, s>>>(
        ManyScenes<InjectParams>{B}, ntexels);
    note_launches(1);
}

void launch_resolve_batch(const SceneBatch<ResolveParams>& B, long long nbricks, bool exact, cudaStream_t s) {
    resolve_kernel<true, false><<<(unsigned)nbricks, kThreads, 0, s>>>(ManyScenes<ResolveParams>{B});
    if (exact) {
        resolve_kernel<true, true><<<(unsigned)nbricks, kThreads, 0, s>>>(ManyScenes<ResolveParams>{B});
        note_launches(1);
    }
    note_launches(1);
}

void launch_mip_tail_batch(const SceneBatch<MipLevels>& B, cudaStream_t s) {
    mip_tail_kernel<<<B.n, kThreads, 0, s>>>(ManyScenes<MipLevels>{B});
    note_launches(1);
}

namespace {
// The per-scene clears of a batched frame (statistics, masks, carry tables)
// in one launch instead of a memset per buffer: range blockIdx.y, 16-byte
// stores and word stores for a ragged end.
__global__ void __launch_bounds__(kThreads) clear_ranges_kernel(const ClearRange* __restrict__ R) {
    const ClearRange r = R[blockIdx.y];
    const long long stride = (long long)gridDim.x * kThreads * 4;
    for (long long i = ((long long)blockIdx.x * kThreads + threadIdx.x) * 4; i < r.words; i += stride) {
        if (i + 4 <= r.words)
            *reinterpret_cast<uint4*>(r.p + i) = make_uint4(0u, 0u, 0u, 0u);
        else
            for (long long k = i; k < r.words; ++k) r.p[k] = 0u;
    }
}
}  // namespace

void launch_clear_ranges(const ClearRange* ranges, int n, long long max_words, cudaStream_t s) {
    if (n <= 0 || max_words <= 0) return;
    const long long per_cta = (long long)kThreads * 4 * 4;  // four 16-byte stores per thread
    const unsigned gx = (unsigned)std::min<long long>((max_words + per_cta - 1) / per_cta, 1024);
    clear_ranges_kernel<<<dim3(gx, (unsigned)n), kThreads, 0, s>>>(ranges);
    note_launches(1);
}

void launch_pad_copy(const uint2* chain, float4* pchain, int dim, int levels, cudaStream_t s) {
    long long off = 0;
    for (int l = 0; l < levels; ++l) {
        const int S = dim >> l;
        const long long n = (long long)S * S * S;
        long long blocks = (n + 255) / 256;
        if (blocks > 8192) blocks = 8192;
        pad_copy_kernel<<<(unsigned)blocks, 256, 0, s>>>(chain + off, pchain + padded_level_offset(dim, l), S);
        note_launches(1);
        off += n;
    }
}

void launch_fill_u32(uint32_t* p, uint32_t v, long long n, cudaStream_t s) {
    if (n <= 0) return;
    long long blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    fill_u32_kernel<<<(unsigned)blocks, 256, 0, s>>>(p, v, n);
    note_launches(1);
}

}  // namespace vct
