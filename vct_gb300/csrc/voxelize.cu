// Triangle voxelisation: shaders/voxelize.geom:25-73 + voxelize.frag:75-280.
//
// Three launches, balanced at fragment granularity (triangle sizes vary by
// more than three orders of magnitude in one scene), for one scene or for the
// concatenated triangles of a batch of scenes:
//  1. voxelize_setup_kernel, one thread per triangle: the geometry-shader
//     part (dominant axis from the summed vertex normals, per-axis ortho
//     projection, snapping to the 1/256 sub-pixel grid, bounding box) into a
//     48-byte record, and the triangle's share of work: its bounding box's
//     rows in units of about 2^unit_log2 candidate pixels (a tuning
//     setting), with a block-local exclusive scan;
//  2. voxelize_scan_kernel, one CTA: exclusive scan of the per-block totals;
//  3. voxelize_raster_kernel, persistent: warps take work units from a
//     shared counter, narrow each row to the triangle's span, test 32 pixel
//     centres at a time for coverage, compact
//     covered fragments (clipped to the depth range) with a ballot into a
//     per-warp ring queue in shared memory, and whenever 32 are queued each
//     lane lights one fragment (all enabled lights, 5-tap PCF for shadow
//     casters) and adds it into the voxel's 32-byte accumulator record with
//     fire-and-forget 64-bit reductions.
//
// Integer sums make the result independent of fragment order: it is
// bit-exact against the CPU oracle.  Compiled with --fmad=false (see
// vct_device.cuh).
#include "vct_device.cuh"

namespace vct {

namespace {

constexpr int kWarps = 8;
constexpr int kQueue = 64;
constexpr int kRasterBlocksPerSM = 3;  // register budget: up to 3 raster CTAs per SM
constexpr int kMaxBatchScenes = 256;  // scene id travels in 8 bits of a queue entry
constexpr int kGrabUnits = 2;          // work units a warp takes from the shared counter at a time
constexpr int kStagedBlocks = 4096;    // setup-block offsets copied to shared memory when they fit

// The raster warps' shared work counter: 8 bytes after block_off[nblocks]
// (zeroed by the setup kernel).
__device__ __forceinline__ unsigned long long* grab_counter(const VoxWork& W, int nblocks) {
    return reinterpret_cast<unsigned long long*>(W.block_off + (((long long)nblocks + 2) & ~1LL));
}

struct FragQueue {
    int tri[kQueue];       // triangle index within its scene
    uint32_t pix[kQueue];  // px | py << 11 | axis << 22 | scene << 24
    float l0[kQueue], l1[kQueue], l2[kQueue], z[kQueue];
};

__device__ __forceinline__ float shadow_factor(const AccumParams& P, f3 wp) {
    return pcf5(P.shadowmap, P.sw, P.sh, P.ls, wp);
}

// Block-local exclusive scan of the per-triangle unit counts of one setup
// block into tri_scan, and the block's total into block_off[blockIdx.x].
__device__ __forceinline__ void block_scan_units(const VoxWork& W, long long g, uint32_t units) {
    __shared__ uint32_t warp_tot[kSetupThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t incl = units;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    uint32_t before = 0, total = 0;
#pragma unroll
    for (int w = 0; w < kSetupThreads / 32; ++w) {
        before += (w < wid) ? warp_tot[w] : 0u;
        total += warp_tot[w];
    }
    if (g < W.ntri) W.tri_scan[g] = before + incl - units;
    if (threadIdx.x == 0) W.block_off[blockIdx.x] = total;
}

// ------------------------------------------------------------- 1. setup
// voxelize.geom:25-73 for triangle t of P: the dominant axis of the summed
// normals (strict >, ties to z, or the override), the projection through
// that axis' orthographic matrix into the N x N viewport, and the snapped
// raster set-up.  False when the triangle covers no pixel centre's bounding
// box (zero snapped area, or outside the viewport).
__device__ __forceinline__ bool project_triangle(const AccumParams& P, long long t, RasterTri& rt, float z[3],
                                                 int& axis) {
    const float* Pp = P.pos + t * 9;
    const float* Pn = P.nrm + t * 9;
    f3 n0 = ld3(Pn), n1 = ld3(Pn + 3), n2 = ld3(Pn + 6);
    f3 fn = normalize(add(add(n0, n1), n2));
    float ax = fabsf(fn.x), ay = fabsf(fn.y), az = fabsf(fn.z);
    axis = 2;
    if (ax > ay && ax > az)
        axis = 0;
    else if (ay > ax && ay > az)
        axis = 1;
    if (P.axis_override >= 0 && P.axis_override <= 2) axis = P.axis_override;
    const float* M = P.mvp + 16 * axis;
    const int N = P.dim;
    float wx[3], wy[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float c[4];
        mat_vec(M, Pp[3 * k], Pp[3 * k + 1], Pp[3 * k + 2], 1.0f, c);
        float nx = __fdiv_rn(c[0], c[3]), ny = __fdiv_rn(c[1], c[3]);
        z[k] = __fdiv_rn(c[2], c[3]);
        wx[k] = (nx + 1.0f) * 0.5f * (float)N;
        wy[k] = (ny + 1.0f) * 0.5f * (float)N;
    }
    return raster_setup(wx, wy, N, N, rt);
}

template <class Scenes>
__global__ void __launch_bounds__(kSetupThreads) voxelize_setup_kernel(const Scenes S, const VoxWork W) {
    const long long g = (long long)blockIdx.x * kSetupThreads + threadIdx.x;
    uint32_t units = 0;
    if (g < W.ntri) {
        long long t;
        const AccumParams& P = S.get(S.find(g, t));
        RasterTri rt;
        float z[3];
        int axis;
        if (project_triangle(P, t, rt, z, axis)) {
            const uint32_t bw = rt.px1 - rt.px0 + 1, bh = rt.py1 - rt.py0 + 1;
            const uint32_t bias = (rt.bias[0] ? 1u : 0u) | (rt.bias[1] ? 2u : 0u) | (rt.bias[2] ? 4u : 0u);
            const float inv = __fdiv_rn(1.0f, __ll2float_rn(rt.area));
            uint4* rec = W.tri_rec + 3 * g;
            rec[0] = make_uint4((uint32_t)rt.X[0], (uint32_t)rt.Y[0], (uint32_t)rt.X[1], (uint32_t)rt.Y[1]);
            rec[1] = make_uint4((uint32_t)rt.X[2], (uint32_t)rt.Y[2], __float_as_uint(z[0]), __float_as_uint(z[1]));
            // A work unit is R whole rows of the bounding box, R chosen so that
            // the unit holds about 2^unit_log2 candidate pixels: a row's span
            // of the triangle (the area over the rows, on average) and a
            // pixel each side.  A sliver's rows are short, so its units take
            // many rows.
            const float row_px = (float)rt.area * (0.5f / (float)(kSub * kSub)) / (float)bh + 2.0f;
            const uint32_t R = (uint32_t)fminf(fmaxf((float)(1u << W.unit_log2) / row_px, 1.0f), 1023.0f);
            rec[2] = make_uint4(__float_as_uint(z[2]), __float_as_uint(inv),
                                (uint32_t)rt.px0 | ((uint32_t)rt.py0 << 11) | ((uint32_t)axis << 22) |
                                    ((uint32_t)rt.perm1 << 24) | (bias << 25),
                                bw | (bh << 11) | (R << 22));
            units = (bh + R - 1) / R;
        }
        W.tri_units[g] = units;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *grab_counter(W, gridDim.x) = 0ull;
    block_scan_units(W, g, units);
}

// --------------------------------------------------------------- 2. scan
__global__ void __launch_bounds__(1024) voxelize_scan_kernel(uint32_t* block_off, int nblocks) {
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int base = 0; base < nblocks; base += 1024) {
        const int i = base + threadIdx.x;
        const uint32_t v = i < nblocks ? block_off[i] : 0u;
        uint32_t incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t s = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += s;
        }
        if (lane == 31) warp_tot[wid] = incl;
        __syncthreads();
        uint32_t before = carry, total = 0;
        for (int w = 0; w < 32; ++w) {
            before += (w < wid) ? warp_tot[w] : 0u;
            total += warp_tot[w];
        }
        if (i < nblocks) block_off[i] = before + incl - v;
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) block_off[nblocks] = carry;
}

// ------------------------------------------------------------- 3. raster
// Voxel of a fragment: voxelize.frag:79-108.  Without warping the axis
// swizzle resolves to integers: the projected coordinates are the pixel
// indices and the depth axis is trunc(N * (1 - u.z)).  With warping the
// fragment's volume coordinate (pixel centre (p + 0.5) / N, depth
// (z + 1) / 2, swizzled, z flipped) is warped and scaled, as the shader does.
__device__ __forceinline__ bool fragment_voxel(const AccumParams& P, int px, int py, int axis, float zf, int& vx,
                                               int& vy, int& vz) {
    const int N = P.dim;
    const float uz = (zf + 1.0f) * 0.5f;
    // voxelize.frag reads warpVoxels and warpTexture only: the perspective
    // warp (voxelizeTesselationWarp) leaves the rasterised grid linear.
    if (P.warp.mode == VCT_WARP_NONE || P.warp.mode == VCT_WARP_PERSPECTIVE) {
        const int iz = __float2int_rz((float)N * (1.0f - uz));
        if (axis == 0) {
            vx = iz;
            vy = py;
            vz = N - 1 - px;
        } else if (axis == 1) {
            vx = px;
            vy = iz;
            vz = N - 1 - py;
        } else {
            vx = px;
            vy = py;
            vz = iz;
        }
    } else {
        const float fN = (float)N;
        const float ux = __fdiv_rn((float)px + 0.5f, fN), uy = __fdiv_rn((float)py + 0.5f, fN);
        f3 u = axis == 0 ? mk(1.0f - uz, uy, ux) : axis == 1 ? mk(ux, 1.0f - uz, uy) : mk(ux, uy, uz);
        u.z = 1.0f - u.z;
        u = apply_warp(P.warp, u);
        vx = __float2int_rz(fN * u.x);
        vy = __float2int_rz(fN * u.y);
        vz = __float2int_rz(fN * u.z);
    }
    return !(vx < 0 || vy < 0 || vz < 0 || vx >= N || vy >= N || vz >= N);
}

// voxelize.frag:186-280 for one queued fragment.
__device__ __forceinline__ void shade_fragment(const AccumParams& P, const FragQueue& q, int e) {
    const long long t = q.tri[e];
    const uint32_t pix = q.pix[e];
    const int px = (int)(pix & 0x7ffu), py = (int)((pix >> 11) & 0x7ffu), axis = (int)((pix >> 22) & 3u);
    int vx, vy, vz;
    if (!fragment_voxel(P, px, py, axis, q.z[e], vx, vy, vz)) return;
    const int N = P.dim;
    const long long v = ((long long)vz * N + vy) * N + vx;
    const float l[3] = {q.l0[e], q.l1[e], q.l2[e]};
    const float* Pp = P.pos + t * 9;
    const float* Pn = P.nrm + t * 9;
    const f3 p0 = ld3(Pp), p1 = ld3(Pp + 3), p2 = ld3(Pp + 6);
    const f3 n0 = ld3(Pn), n1 = ld3(Pn + 3), n2 = ld3(Pn + 6);
    const f3 wp = mk(interp(l, p0.x, p1.x, p2.x), interp(l, p0.y, p1.y, p2.y), interp(l, p0.z, p1.z, p2.z));
    const f3 ni = mk(interp(l, n0.x, n1.x, n2.x), interp(l, n0.y, n1.y, n2.y), interp(l, n0.z, n1.z, n2.z));
    const f3 Nf = normalize(ni);
    f3 color = ld3(P.albedo + t * 3);
    if (P.lighting) {
        f3 fin = mk(0.0f, 0.0f, 0.0f);
        for (int li = 0; li < P.nlights; ++li) {
            const LightDev& L = P.lights[li];
            if (!L.enabled) continue;
            f3 lit = mk(0.0f, 0.0f, 0.0f);
            if (L.type == 0u) {
                f3 d = sub(L.position, wp);
                float ndl = fmaxf(0.0f, dot(Nf, normalize(d)));
                lit = mul(mulv(mul(color, L.intensity), L.color), ndl);
                float att = 1.0f - smoothstep(L.range075, L.range, length(d));
                lit = mul(lit, att);
            } else if (L.type == 1u) {
                float ndl = fmaxf(0.0f, dot(Nf, L.neg_dir_n));
                lit = mul(mul(mulv(color, L.color), L.intensity), ndl);
            }
            // lit *= 1 - shadow: when lit is exactly zero (the surface faces away, or the
            // light is out of range) the product is +-0 and adding it leaves `fin`
            // unchanged (1 - shadow is finite), so the PCF is not evaluated.
            if (L.shadow_caster && (lit.x != 0.0f || lit.y != 0.0f || lit.z != 0.0f))
                lit = mul(lit, 1.0f - shadow_factor(P, wp));
            fin = add(fin, lit);
        }
        color = mk(clampf(fin.x, 0.0f, 1.0f), clampf(fin.y, 0.0f, 1.0f), clampf(fin.z, 0.0f, 1.0f));
    }
    const f3 n01 = mk((Nf.x + 1.0f) * 0.5f, (Nf.y + 1.0f) * 0.5f, (Nf.z + 1.0f) * 0.5f);
    unsigned long long* rec = reinterpret_cast<unsigned long long*>(P.acc + kAccWords * record_slot(v, P.dim));
    const unsigned long long qr = quant16(color.x), qg = quant16(color.y), qb = quant16(color.z);
    const unsigned long long qx = quant16(n01.x), qy = quant16(n01.y), qz = quant16(n01.z);
    // Fire-and-forget reductions: no result is waited for.  (Setting the
    // occupancy bit only for the fragment that finds the count at 0 waits
    // for the first add's result and is slower.)
    atomicAdd(rec + 0, 1ull | (qr << 32));
    atomicAdd(rec + 1, qg | (qb << 32));
    atomicAdd(rec + 2, qx | (qy << 32));
    atomicAdd(rec + 3, qz);
    atomicOr(P.occ + (v >> 5), 1u << (v & 31));
}

// Coverage of pixel (px, py) by a set-up triangle (snapped vertices X, Y; edge
// k runs from vertex a = k+1 to b = k+2 with deltas dX, dY; bit k of `bias`
// set for an edge that is not top-left) and the fragment's barycentrics and
// depth.  The edge function at the pixel centre is dX (sy - Ya) - dY (sx - Xa),
// every factor within 32 bits (|snapped coordinates| <= 2^28), each product
// exact in 64.  False outside the triangle or outside GL's depth clip.
__device__ __forceinline__ bool pixel_fragment(const int X[3], const int Y[3], const int dX[3], const int dY[3],
                                               int bias, int perm1, float inv, const float z[3], int px, int py,
                                               float l[3], float& zf) {
    const int sx = px * (int)kSub + (int)kSub / 2, sy = py * (int)kSub + (int)kSub / 2;
    long long e[3];
    bool cov = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int a = (k + 1) % 3;
        e[k] = (long long)dX[k] * (long long)(sy - Y[a]) - (long long)dY[k] * (long long)(sx - X[a]);
        cov = cov && (e[k] - ((bias >> k) & 1) >= 0);
    }
    if (!cov) return false;
    const float w0 = __ll2float_rn(e[0]) * inv, w1 = __ll2float_rn(e[1]) * inv, w2 = __ll2float_rn(e[2]) * inv;
    l[0] = w0;
    l[1] = perm1 ? w2 : w1;
    l[2] = perm1 ? w1 : w2;
    zf = interp(l, z[0], z[1], z[2]);
    return zf >= -1.0f && zf <= 1.0f;  // GL clipping
}

template <class Scenes>
__device__ __forceinline__ long long unit_start(const VoxWork& W, long long g) {
    return (long long)W.block_off[g / kSetupThreads] + W.tri_scan[g];
}

template <class Scenes>
__global__ void __launch_bounds__(kWarps * 32, kRasterBlocksPerSM)
    voxelize_raster_kernel(const Scenes S, const VoxWork W, int nblocks) {
    __shared__ FragQueue queues[kWarps];
    __shared__ unsigned frag_count[kMaxBatchScenes];  // VoxelizeInfo.totalVoxelFragments per scene
    __shared__ uint32_t s_boff[kStagedBlocks + 1];
    const int lane = threadIdx.x & 31;
    FragQueue& q = queues[threadIdx.x >> 5];
    const unsigned FULL = 0xffffffffu;
    const int nscenes = S.count();
    for (int i = threadIdx.x; i < nscenes; i += blockDim.x) frag_count[i] = 0;
    const bool staged = nblocks <= kStagedBlocks;
    if (staged)
        for (int i = threadIdx.x; i <= nblocks; i += blockDim.x) s_boff[i] = W.block_off[i];
    __syncthreads();
    auto boff = [&](long long b) -> long long { return staged ? s_boff[b] : W.block_off[b]; };
    const long long total = boff(nblocks);
    unsigned long long* grab = grab_counter(W, nblocks);
    // The queue is a ring of kQueue entries: fragments [head, head + qn).
    int qn = 0, head = 0;  // warp-uniform

    // Shades the 32 oldest queued fragments (or `nact`), one per lane.
    auto shade32 = [&](int nact) {
        __syncwarp();
        if (lane < nact) {
            const int e = (head + lane) & (kQueue - 1);
            shade_fragment(S.get((int)(q.pix[e] >> 24)), q, e);
        }
        __syncwarp();
    };
    // VoxelizeInfo.totalVoxelFragments: covered fragments are counted where
    // they are queued, for the unit's scene, and added to the CTA's
    // per-scene counter when the scene changes.
    int cur_scene = 0;
    unsigned pending = 0;
    auto flush_count = [&]() {
        if (lane == 0 && pending) atomicAdd(&frag_count[cur_scene], pending);
        pending = 0;
    };

    // Warps take kGrabUnits work units at a time from a shared counter until
    // none are left, so that every warp ends at about the same time whatever
    // the units cost (their pixel counts and coverage vary by orders of
    // magnitude).  Fragments are summed as integers, so the order in which
    // warps take the units does not change the result.
    for (;;) {
        unsigned long long gu = 0;
        if (lane == 0) gu = atomicAdd(grab, (unsigned long long)kGrabUnits);
        gu = __shfl_sync(FULL, gu, 0);
        if ((long long)gu >= total) break;
        const long long u0 = (long long)gu, u1 = min(u0 + (long long)kGrabUnits, total);
        // Triangle owning unit u0: binary search over the block offsets, then
        // the block-local scan, 8 entries per lane: the number of entries <=
        // u0 is one past the last triangle starting at or before u0.
        int lo = 0, hi = nblocks - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (boff(mid) <= u0)
                lo = mid;
            else
                hi = mid - 1;
        }
        const long long gbase = (long long)lo * kSetupThreads;
        const int in_block = (int)min((long long)kSetupThreads, W.ntri - gbase);
        const uint32_t rel = (uint32_t)(u0 - boff(lo));
        int below = 0;
#pragma unroll
        for (int j = 0; j < kSetupThreads / 32; ++j) {
            const int k = lane * (kSetupThreads / 32) + j;
            below += (k < in_block && __ldg(W.tri_scan + gbase + k) <= rel) ? 1 : 0;
        }
        below = __reduce_add_sync(FULL, below);
        long long g = gbase + max(below - 1, 0);
        long long start = boff(lo) + W.tri_scan[g];
        uint32_t nunits = W.tri_units[g];
        for (long long u = u0; u < u1; ++u) {
            while (u >= start + nunits) {
                ++g;
                start = boff(g / kSetupThreads) + W.tri_scan[g];
                nunits = W.tri_units[g];
            }
            long long tl;
            const int scene = S.find(g, tl);
            if (scene != cur_scene) {
                flush_count();
                cur_scene = scene;
            }
            const uint4* rp = W.tri_rec + 3 * g;
            const uint4 r0 = __ldg(rp), r1 = __ldg(rp + 1), r2 = __ldg(rp + 2);
            const int X[3] = {(int)r0.x, (int)r0.z, (int)r1.x};
            const int Y[3] = {(int)r0.y, (int)r0.w, (int)r1.y};
            const float z[3] = {__uint_as_float(r1.z), __uint_as_float(r1.w), __uint_as_float(r2.x)};
            const float inv = __uint_as_float(r2.y);
            const int px0 = (int)(r2.z & 0x7ffu), py0 = (int)((r2.z >> 11) & 0x7ffu);
            const int axis = (int)((r2.z >> 22) & 3u), perm1 = (int)((r2.z >> 24) & 1u), bias = (int)(r2.z >> 25);
            const int bw = (int)(r2.w & 0x7ffu), bh = (int)((r2.w >> 11) & 0x7ffu), R = (int)(r2.w >> 22);
            int dX[3], dY[3];  // edge k: vertex k+2 minus vertex k+1
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                dX[k] = X[(k + 2) % 3] - X[(k + 1) % 3];
                dY[k] = Y[(k + 2) % 3] - Y[(k + 1) % 3];
            }
            // The unit's rows of the bounding box, 32 at a time: each lane takes
            // one row and narrows it to the pixels between the triangle's
            // crossings of the row's centre line (widened by one pixel each
            // side, so that float rounding never drops a covered pixel); the
            // warp then tests the rows' candidates 32 at a time.
            const int r_a = (int)(u - start) * R, r_b = min(r_a + R, bh) - 1;
            float slope[3];  // x per unit y along edge k
#pragma unroll
            for (int k = 0; k < 3; ++k) slope[k] = dY[k] != 0 ? __fdividef((float)dX[k], (float)dY[k]) : 0.0f;
            for (int rb = r_a; rb <= r_b; rb += 32) {
                const int r = rb + lane;
                int lo = 0, cnt = 0;
                if (r <= r_b) {
                    const int sy = (py0 + r) * (int)kSub + (int)kSub / 2;
                    float xmin = 3.0e38f, xmax = -3.0e38f;
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        const int a = (k + 1) % 3, bb = (k + 2) % 3;
                        if (min(Y[a], Y[bb]) <= sy && sy <= max(Y[a], Y[bb])) {
                            const float x0 = dY[k] != 0 ? fmaf((float)(sy - Y[a]), slope[k], (float)X[a]) : (float)X[a];
                            const float x1 = dY[k] != 0 ? x0 : (float)X[bb];
                            xmin = fminf(xmin, fminf(x0, x1));
                            xmax = fmaxf(xmax, fmaxf(x0, x1));
                        }
                    }
                    if (xmin <= xmax) {
                        const float rs = 1.0f / (float)kSub, hs = 0.5f * (float)kSub;
                        const int s0 = (int)ceilf((xmin - hs) * rs) - 1 - px0;
                        const int s1 = (int)floorf((xmax - hs) * rs) + 1 - px0;
                        lo = max(0, s0);
                        cnt = max(min(bw - 1, s1) - lo + 1, 0);
                    }
                }
                int excl = cnt;  // exclusive prefix of the rows' candidate counts
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int v = __shfl_up_sync(FULL, excl, o);
                    if (lane >= o) excl += v;
                }
                const int ncand = __shfl_sync(FULL, excl, 31);
                excl -= cnt;
                for (int k0 = 0; k0 < ncand; k0 += 32) {
                    const int kc = k0 + lane;
                    int j = 0;  // the last row whose candidates start at or before kc
#pragma unroll
                    for (int st = 16; st > 0; st >>= 1)
                        if (__shfl_sync(FULL, excl, j + st) <= kc) j += st;
                    const int lo_j = __shfl_sync(FULL, lo, j), ex_j = __shfl_sync(FULL, excl, j);
                    bool cov = false;
                    float l[3] = {0.f, 0.f, 0.f}, zf = 0.f;
                    const int py = py0 + rb + j, px = px0 + lo_j + (kc - ex_j);
                    if (kc < ncand) cov = pixel_fragment(X, Y, dX, dY, bias, perm1, inv, z, px, py, l, zf);
                    const unsigned m = __ballot_sync(FULL, cov);
                    if (cov) {
                        const int slot = (head + qn + __popc(m & ((1u << lane) - 1u))) & (kQueue - 1);
                        q.tri[slot] = (int)tl;
                        q.pix[slot] = (uint32_t)px | ((uint32_t)py << 11) | ((uint32_t)axis << 22) |
                                      ((uint32_t)scene << 24);
                        q.l0[slot] = l[0];
                        q.l1[slot] = l[1];
                        q.l2[slot] = l[2];
                        q.z[slot] = zf;
                    }
                    qn += __popc(m);
                    pending += (unsigned)__popc(m);
                    if (qn >= 32) {
                        shade32(32);
                        head = (head + 32) & (kQueue - 1);
                        qn -= 32;
                    }
                }
            }
        }
    }
    shade32(qn);
    flush_count();
    __syncthreads();
    for (int i = threadIdx.x; i < nscenes; i += blockDim.x)
        if (frag_count[i]) atomicAdd(&S.get(i).stats->total_voxel_fragments, frag_count[i]);
}

template <class Scenes>
void launch_voxelize(const Scenes& S, const VoxWork& W, int num_sms, int blocks_per_sm, cudaStream_t s) {
    if (W.ntri <= 0) return;
    const int nblocks = (int)((W.ntri + kSetupThreads - 1) / kSetupThreads);
    voxelize_setup_kernel<Scenes><<<nblocks, kSetupThreads, 0, s>>>(S, W);
    voxelize_scan_kernel<<<1, 1024, 0, s>>>(W.block_off, nblocks);
    const int bps = blocks_per_sm < 1 ? 1 : (blocks_per_sm > kRasterBlocksPerSM ? kRasterBlocksPerSM : blocks_per_sm);
    voxelize_raster_kernel<Scenes><<<num_sms * bps, kWarps * 32, 0, s>>>(S, W, nblocks);
    note_launches(3);
}

// ================================================ warp-map occupancy pass
// voxelize.frag:187-192: the occupancy voxelisation that the warp map is
// built from (Application.cpp:235-285), the same rasterisation rule as above
// at a 32^2 viewport, unwarped and unshaded.  Nearly every triangle of a
// scene covers a handful of pixels at that size, so the persistent raster's
// work units (one shared-counter grab, a search and three dependent loads
// each) would cost far more than the pixels: one thread takes one triangle,
// sets it up and walks a bounding box of up to kOccLanePixels pixels itself;
// the warp walks the larger ones together, 32 pixels at a time.  The result
// is an OR of bits, so the order of the walks does not matter.
constexpr int kOccThreads = 256;
constexpr int kOccLanePixels = 32;

__device__ __forceinline__ void occupancy_fragment(const AccumParams& P, int axis, int px, int py, float zf) {
    int vx, vy, vz;
    if (!fragment_voxel(P, px, py, axis, zf, vx, vy, vz)) return;
    const long long v = ((long long)vz * P.dim + vy) * P.dim + vx;
    atomicOr(P.occ + (v >> 5), 1u << (v & 31));
}

template <class Scenes>
__global__ void __launch_bounds__(kOccThreads) occupancy_kernel(const Scenes S, long long ntri) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const long long g = (long long)blockIdx.x * kOccThreads + threadIdx.x;
    RasterTri rt;
    float z[3] = {0.f, 0.f, 0.f};
    int axis = 0, scene = 0;
    bool ok = false;
    if (g < ntri) {
        long long t;
        scene = S.find(g, t);
        const AccumParams& P = S.get(scene);
        ok = P.occ != nullptr && project_triangle(P, t, rt, z, axis);  // scenes without a map: no occupancy
    }
    int X[3] = {0, 0, 0}, Y[3] = {0, 0, 0}, dX[3], dY[3];
    int bias = 0, perm1 = 0, px0 = 0, py0 = 0, bw = 0, bh = 0;
    float inv = 0.f;
    if (ok) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            X[k] = (int)rt.X[k];
            Y[k] = (int)rt.Y[k];
        }
        bias = (rt.bias[0] ? 1 : 0) | (rt.bias[1] ? 2 : 0) | (rt.bias[2] ? 4 : 0);
        perm1 = rt.perm1;
        inv = __fdiv_rn(1.0f, __ll2float_rn(rt.area));
        px0 = rt.px0;
        py0 = rt.py0;
        bw = rt.px1 - rt.px0 + 1;
        bh = rt.py1 - rt.py0 + 1;
    }
    const int npix = bw * bh;
    if (npix <= kOccLanePixels) {
        const AccumParams& P = S.get(scene);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            dX[k] = X[(k + 2) % 3] - X[(k + 1) % 3];
            dY[k] = Y[(k + 2) % 3] - Y[(k + 1) % 3];
        }
        for (int py = py0; py < py0 + bh; ++py)
            for (int px = px0; px < px0 + bw; ++px) {
                float l[3], zf;
                if (pixel_fragment(X, Y, dX, dY, bias, perm1, inv, z, px, py, l, zf))
                    occupancy_fragment(P, axis, px, py, zf);
            }
    }
    unsigned big = __ballot_sync(FULL, npix > kOccLanePixels);
    while (big) {
        const int src = __ffs(big) - 1;
        big &= big - 1;
        int sX[3], sY[3], sdX[3], sdY[3];
        float sz[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            sX[k] = __shfl_sync(FULL, X[k], src);
            sY[k] = __shfl_sync(FULL, Y[k], src);
            sz[k] = __shfl_sync(FULL, z[k], src);
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            sdX[k] = sX[(k + 2) % 3] - sX[(k + 1) % 3];
            sdY[k] = sY[(k + 2) % 3] - sY[(k + 1) % 3];
        }
        const int sbias = __shfl_sync(FULL, bias, src), sperm1 = __shfl_sync(FULL, perm1, src);
        const float sinv = __shfl_sync(FULL, inv, src);
        const int saxis = __shfl_sync(FULL, axis, src), sscene = __shfl_sync(FULL, scene, src);
        const int spx0 = __shfl_sync(FULL, px0, src), spy0 = __shfl_sync(FULL, py0, src);
        const int sbw = __shfl_sync(FULL, bw, src), sn = __shfl_sync(FULL, npix, src);
        const AccumParams& SP = S.get(sscene);
        for (int idx = lane; idx < sn; idx += 32) {
            const int row = idx / sbw;
            const int px = spx0 + (idx - row * sbw), py = spy0 + row;
            float l[3], zf;
            if (pixel_fragment(sX, sY, sdX, sdY, sbias, sperm1, sinv, sz, px, py, l, zf))
                occupancy_fragment(SP, saxis, px, py, zf);
        }
    }
}

// ====================================================== tessellation voxeliser
// testTesselation.tesc/.tese (Application.cpp:585-662) in three launches of
// the same shape as the rasteriser's: per-triangle tessellation levels and
// point counts (tess_setup_kernel), the scan of the block totals, and a
// persistent kernel in which every warp takes an equal range of 32-point
// work units, queues the points of its units and stores 32 at a time.
//
// Tessellation levels after GL's equal_spacing rounding, packed 7 bits each:
// inner n | outer[0] << 7 | outer[1] << 14 | outer[2] << 21 (1..64 each).
constexpr int kTessUnit = 32;

// Float-to-int truncation of ivec3(): NaN -> 0, saturating (cvt.rzi.s32.f32).
__device__ __forceinline__ int trunc_sat(float x) { return __float2int_rz(x); }

// equal_spacing: clamp to [1, max], round up (OpenGL 4.6, 11.2.2).
__device__ __forceinline__ int tess_round(float level, float max_level) {
    return (int)ceilf(fminf(fmaxf(level, 1.0f), max_level));
}

// Points of the triangle primitive generator in point mode for inner level
// n and outer levels m0..m2: the outer ring (3 corners and m - 1 points per
// edge) plus the concentric inner rings k = 1.. of n - 2k segments each
// (3 (n - 2k) points, or the centre when n - 2k = 0).
__device__ __forceinline__ uint32_t tess_point_count(int n, int m0, int m1, int m2) {
    uint32_t c = (uint32_t)(m0 + m1 + m2);
    if (n >= 2) {
        const int K = (n & 1) ? (n - 1) / 2 : n / 2 - 1;
        c += 3u * (uint32_t)(K * n - K * (K + 1)) + ((n & 1) ? 0u : 1u);
    }
    return c;
}

// testTesselation.tesc:33-78: levels of one triangle; false if discarded
// (all three vertices truncate to one voxel: levels 0).
__device__ __forceinline__ bool tess_levels(const AccumParams& P, const float* Pp, uint32_t& packed, uint32_t& npts) {
    const f3 a = ld3(Pp), b = ld3(Pp + 3), c = ld3(Pp + 6);
    const float fN = (float)P.dim;
    const f3 vtx[3] = {a, b, c};
    int vi[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {  // ivec3(voxelDim * getVoxelPosition(p)), the shader's own linear mapping
        vi[k][0] = trunc_sat(fN * __fdiv_rn((vtx[k].x - P.vcenter.x) - P.vmin.x, P.ext.x));
        vi[k][1] = trunc_sat(fN * __fdiv_rn((vtx[k].y - P.vcenter.y) - P.vmin.y, P.ext.y));
        vi[k][2] = trunc_sat(fN * __fdiv_rn((vtx[k].z - P.vcenter.z) - P.vmin.z, P.ext.z));
    }
    if (vi[0][0] == vi[1][0] && vi[0][1] == vi[1][1] && vi[0][2] == vi[1][2] && vi[0][0] == vi[2][0] &&
        vi[0][1] == vi[2][1] && vi[0][2] == vi[2][2])
        return false;
    const f3 A = sub(c, b), B = sub(c, a), C = sub(b, a);
    const float lx = length(A), ly = length(B), lz = length(C);
    const float sp = ((lx + ly) + lz) * 0.5f;  // semiperimeter
    const float area = __fsqrt_rn(((sp * (sp - lx)) * (sp - ly)) * (sp - lz));  // Heron
    const float ax = __fdiv_rn(2.0f * area, lx), ay = __fdiv_rn(2.0f * area, ly), az = __fdiv_rn(2.0f * area, lz);
    const float max_alt = fmaxf(ax, fmaxf(ay, az));
    const f3 vs = mk(__fdiv_rn(P.ext.x, fN), __fdiv_rn(P.ext.y, fN), __fdiv_rn(P.ext.z, fN));
    const float dx = fabsf(length(mulv(normalize(A), vs))), dy = fabsf(length(mulv(normalize(B), vs))),
                dz = fabsf(length(mulv(normalize(C), vs)));
    const float ox = fmaxf(1.0f, __fdiv_rn(lx, dx)), oy = fmaxf(1.0f, __fdiv_rn(ly, dy)),
                oz = fmaxf(1.0f, __fdiv_rn(lz, dz));
    const float inner = fmaxf(1.0f, __fdiv_rn(max_alt, vs.x));
    // gl_TessLevelOuter[0] = outer.z, [1] = outer.x, [2] = outer.y
    const int m0 = tess_round(oz, P.max_tess_level), m1 = tess_round(ox, P.max_tess_level),
              m2 = tess_round(oy, P.max_tess_level);
    int n = tess_round(inner, P.max_tess_level);
    if (n == 1 && (m0 > 1 || m1 > 1 || m2 > 1)) n = 2;  // inner 1 + epsilon
    packed = (uint32_t)n | ((uint32_t)m0 << 7) | ((uint32_t)m1 << 14) | ((uint32_t)m2 << 21);
    npts = tess_point_count(n, m0, m1, m2);
    return true;
}

// gl_TessCoord of point `i` in the order of tess_point_count.  The outer
// edges are u = 0 (from vertex 1 to 2, outer[0]), v = 0 (2 to 0, outer[1]),
// w = 0 (0 to 1, outer[2]), at j / m.  Ring k's corners lie where the
// perpendiculars through the inner subdivision points nearest each corner
// meet: (1 - 2t, t, t) and rotations, t = 2k / (3n); its edges are split
// into n - 2k equal segments.
__device__ __forceinline__ f3 tess_coord(uint32_t packed, int i) {
    const int n = (int)(packed & 127u), m0 = (int)((packed >> 7) & 127u), m1 = (int)((packed >> 14) & 127u),
              m2 = (int)((packed >> 21) & 127u);
    if (i < 3) return i == 0 ? mk(1.0f, 0.0f, 0.0f) : i == 1 ? mk(0.0f, 1.0f, 0.0f) : mk(0.0f, 0.0f, 1.0f);
    i -= 3;
    if (i < m0 - 1) {
        const float s = __fdiv_rn((float)(i + 1), (float)m0);
        return mk(0.0f, 1.0f - s, s);
    }
    i -= m0 - 1;
    if (i < m1 - 1) {
        const float s = __fdiv_rn((float)(i + 1), (float)m1);
        return mk(s, 0.0f, 1.0f - s);
    }
    i -= m1 - 1;
    if (i < m2 - 1) {
        const float s = __fdiv_rn((float)(i + 1), (float)m2);
        return mk(1.0f - s, s, 0.0f);
    }
    i -= m2 - 1;
    int k = 1, q = n - 2;
    while (q > 0 && i >= 3 * q) {
        i -= 3 * q;
        ++k;
        q -= 2;
    }
    if (q <= 0) {  // the centre of an even inner level
        const float third = __fdiv_rn(1.0f, 3.0f);
        return mk(third, third, third);
    }
    const float t = __fdiv_rn((float)(2 * k), (float)(3 * n));
    const float h = 1.0f - 2.0f * t;
    const int e = i / q, j = i - e * q;
    const float s = __fdiv_rn((float)j, (float)q);
    // corners c_e and c_{e+1} of the ring: c0 = (h,t,t), c1 = (t,h,t), c2 = (t,t,h)
    const int e1 = e == 2 ? 0 : e + 1;
    const float a0 = e == 0 ? h : t, a1 = e == 1 ? h : t, a2 = e == 2 ? h : t;
    const float b0 = e1 == 0 ? h : t, b1 = e1 == 1 ? h : t, b2 = e1 == 2 ? h : t;
    return mk(a0 + s * (b0 - a0), a1 + s * (b1 - a1), a2 + s * (b2 - a2));
}

// Record of a triangle: {packed levels, points, scene, index within its scene}.
template <class Scenes>
__global__ void __launch_bounds__(kSetupThreads) tess_setup_kernel(const Scenes S, const VoxWork W) {
    const long long g = (long long)blockIdx.x * kSetupThreads + threadIdx.x;
    uint32_t units = 0;
    if (g < W.ntri) {
        long long t;
        const int scene = S.find(g, t);
        const AccumParams& P = S.get(scene);
        uint32_t packed = 0, npts = 0;
        if (!tess_levels(P, P.pos + t * 9, packed, npts)) npts = 0;
        W.tri_rec[3 * g] = make_uint4(packed, npts, (uint32_t)scene, (uint32_t)t);
        units = (npts + kTessUnit - 1) / kTessUnit;
        W.tri_units[g] = units;
    }
    block_scan_units(W, g, units);
}

struct TessQueue {
    int tri[2 * kTessUnit];       // triangle index within its scene
    uint32_t pt[2 * kTessUnit];   // point index within the triangle | scene << 16
    uint32_t lev[2 * kTessUnit];  // packed levels
};

// testTesselation.tese:101-133 for the queued points, one per lane (lanes
// >= nact idle), stored with 64-bit reductions.  Summing every group of
// lanes that hit one voxel first (__match_any_sync, __reduce_add_sync)
// measured 2.2x slower on the large frame than plain reductions; merging
// adjacent pairs, and setting the occupancy bit only on a voxel's first
// store, are what pays.  Integer sums: any grouping gives the same record.
template <class Scenes>
__device__ __forceinline__ void tess_store32(const Scenes& S, const TessQueue& q, int nact, int lane) {
    bool valid = false;
    uint32_t v = 0, qr = 0, qg = 0, qb = 0, qx = 0, qy = 0, qz = 0;
    const AccumParams& P = S.get(lane < nact ? (int)(q.pt[lane] >> 16) : 0);
    if (lane < nact) {
        const long long t = q.tri[lane];
        const f3 bc = tess_coord(q.lev[lane], (int)(q.pt[lane] & 0xffffu));
        const float* Pp = P.pos + t * 9;
        const float* Pn = P.nrm + t * 9;
        const f3 p0 = ld3(Pp), p1 = ld3(Pp + 3), p2 = ld3(Pp + 6);
        const f3 n0 = ld3(Pn), n1 = ld3(Pn + 3), n2 = ld3(Pn + 6);
        const f3 pos = add(add(mul(p0, bc.x), mul(p1, bc.y)), mul(p2, bc.z));
        const f3 nrm = add(add(mul(n0, bc.x), mul(n1, bc.y)), mul(n2, bc.z));
        const int N = P.dim;
        const float fN = (float)N;
        f3 tc;
        if (P.warp.mode == VCT_WARP_PERSPECTIVE) {  // voxelTesselationWarpedPosition
            tc = perspective_tc(P.warp, pos);
        } else {  // voxelLinearPosition (the evaluation shader passes warpVoxels = false)
            tc = mk(__fdiv_rn((pos.x - P.vcenter.x) - P.vmin.x, P.ext.x),
                    __fdiv_rn((pos.y - P.vcenter.y) - P.vmin.y, P.ext.y),
                    __fdiv_rn((pos.z - P.vcenter.z) - P.vmin.z, P.ext.z));
        }
        const int vx = trunc_sat(fN * tc.x), vy = trunc_sat(fN * tc.y), vz = trunc_sat(fN * tc.z);
        if (!(vx < 0 || vy < 0 || vz < 0 || vx >= N || vy >= N || vz >= N)) {
            valid = true;
            v = (uint32_t)(((long long)vz * N + vy) * N + vx);
            const f3 Nf = normalize(nrm);  // voxelStore: normalize(normal) * 0.5 + 0.5
            const f3 col = ld3(P.albedo + t * 3);
            qr = quant16(col.x);
            qg = quant16(col.y);
            qb = quant16(col.z);
            qx = quant16(Nf.x * 0.5f + 0.5f);
            qy = quant16(Nf.y * 0.5f + 0.5f);
            qz = quant16(Nf.z * 0.5f + 0.5f);
        }
    }
    // Neighbouring points of a ring edge often share a voxel: an even lane
    // takes its odd neighbour's sums when both hit the same voxel (one
    // shuffle per word), so the pair costs one set of reductions.
    const unsigned key = valid ? v : 0xffffffffu;
    const unsigned partner = __shfl_xor_sync(0xffffffffu, key, 1);  // every lane takes part
    const bool pair = valid && partner == key;
    const uint32_t pr = __shfl_xor_sync(0xffffffffu, qr, 1), pg = __shfl_xor_sync(0xffffffffu, qg, 1),
                   pb = __shfl_xor_sync(0xffffffffu, qb, 1), px = __shfl_xor_sync(0xffffffffu, qx, 1),
                   py = __shfl_xor_sync(0xffffffffu, qy, 1), pz = __shfl_xor_sync(0xffffffffu, qz, 1);
    if (!valid || (pair && (lane & 1))) return;
    unsigned long long cnt = 1;
    if (pair) {
        cnt = 2;
        qr += pr;
        qg += pg;
        qb += pb;
        qx += px;
        qy += py;
        qz += pz;
    }
    unsigned long long* rec = reinterpret_cast<unsigned long long*>(P.acc + kAccWords * record_slot(v, P.dim));
    const unsigned long long a0 = cnt | ((unsigned long long)qr << 32);
    const unsigned long long a1 = (unsigned long long)qg | ((unsigned long long)qb << 32);
    const unsigned long long a2 = (unsigned long long)qx | ((unsigned long long)qy << 32);
    const unsigned long long was = atomicAdd(rec + 0, a0);
    if (P.carry) {
        // Exact past 65,536 points: the old values show every crossing of
        // 2^32 by r, g, b, nx and ny (the count itself never gets near one;
        // nz's carries land in the last word's unused high half).  The store
        // that takes the count past 65,536 lists the voxel even without a
        // crossing, so that the carry pass rewrites every voxel whose nz may
        // have carried.
        const unsigned long long w1 = atomicAdd(rec + 1, a1), w2 = atomicAdd(rec + 2, a2);
        atomicAdd(rec + 3, (unsigned long long)qz);
        const uint32_t ev[kCarryEvents] = {wrap_hi(was, a0), carry_lo(w1, a1), wrap_hi(w1, a1),
                                           carry_lo(w2, a2), wrap_hi(w2, a2)};
        const unsigned long long c0 = was & 0xffffffffull;
        if ((ev[0] | ev[1] | ev[2] | ev[3] | ev[4]) || (c0 <= 65536ull && c0 + cnt > 65536ull))
            carry_add(P.carry, v, ev, P.stats);
    } else {
        atomicAdd(rec + 1, a1);
        atomicAdd(rec + 2, a2);
        atomicAdd(rec + 3, (unsigned long long)qz);
    }
    // The voxel's occupancy bit, once: by the store that found its count at 0.
    if ((was & 0xffffffffull) == 0ull) atomicOr(P.occ + (v >> 5), 1u << (v & 31));
}

// The carry pass: every voxel listed in a scene's carry table gets its six
// 64-bit sums rebuilt from its record and its crossings of 2^32, its record
// rewritten with their float values (the resolve's dividend) and bit 31 of
// the count set, and its brick flagged for the resolve's exact pass.  One
// thread per table slot, blockIdx.y the scene.
template <class Scenes>
__global__ void __launch_bounds__(256) carry_fixup_kernel(const Scenes S) {
    const AccumParams& P = S.get(blockIdx.y);
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (!P.carry || slot >= kCarrySlots) return;
    const uint32_t* e = P.carry + 8 * slot;
    if (e[0] == 0u) return;
    const long long v = (long long)e[0] - 1;
    uint4* r = reinterpret_cast<uint4*>(P.acc + kAccWords * record_slot(v, P.dim));
    const uint4 r0 = r[0], r1 = r[1];
    const unsigned long long t = 1ull << 32;
    // {count | r}, {g | b}, {nx | ny}, {nz | nz's carries}: a high field holds
    // its own sum plus the low field's carries, modulo 2^32
    const unsigned long long sr = r0.y + t * e[1], sg = r0.z + t * e[2], sb = r0.w + t * e[3] - e[2],
                             sx = r1.x + t * e[4], sy = r1.y + t * e[5] - e[4], sz = r1.z + t * r1.w;
    r[0] = make_uint4(r0.x | 0x80000000u, __float_as_uint(__ull2float_rn(sr)), __float_as_uint(__ull2float_rn(sg)),
                      __float_as_uint(__ull2float_rn(sb)));
    r[1] = make_uint4(__float_as_uint(__ull2float_rn(sx)), __float_as_uint(__ull2float_rn(sy)),
                      __float_as_uint(__ull2float_rn(sz)), 0u);
    const long long N = P.dim, bpa = N / 16;  // the voxel's 16^3 brick, in the resolve's brick order
    const long long x = v % N, y = (v / N) % N, z = v / (N * N);
    P.brick_exact[((z / 16) * bpa + y / 16) * bpa + x / 16] = 1u;
}

template <class Scenes>
__global__ void __launch_bounds__(kWarps * 32, 4) tess_points_kernel(const Scenes S, const VoxWork W, int nblocks) {
    __shared__ TessQueue queues[kWarps];
    __shared__ unsigned point_count[kMaxBatchScenes];  // generated points per scene
    const int lane = threadIdx.x & 31;
    TessQueue& q = queues[threadIdx.x >> 5];
    const int nscenes = S.count();
    for (int i = threadIdx.x; i < nscenes; i += blockDim.x) point_count[i] = 0;
    __syncthreads();
    const long long nw = (long long)gridDim.x * kWarps;
    const long long w = (long long)blockIdx.x * kWarps + (threadIdx.x >> 5);
    const long long total = W.block_off[nblocks];
    const long long u0 = total * w / nw, u1 = total * (w + 1) / nw;
    int qn = 0;                // queued points (warp-uniform)
    int cur_scene = 0;         // generated points of the current scene, not yet counted
    unsigned pending = 0;
    if (u0 < u1) {
        int lo = 0, hi = nblocks - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if ((long long)W.block_off[mid] <= u0)
                lo = mid;
            else
                hi = mid - 1;
        }
        long long glo = (long long)lo * kSetupThreads;
        long long ghi = min(glo + kSetupThreads, W.ntri) - 1;
        while (glo < ghi) {
            const long long mid = (glo + ghi + 1) >> 1;
            if (unit_start<Scenes>(W, mid) <= u0)
                glo = mid;
            else
                ghi = mid - 1;
        }
        long long g = glo;
        long long start = unit_start<Scenes>(W, g);
        uint32_t nunits = W.tri_units[g];
        for (long long u = u0; u < u1; ++u) {
            while (u >= start + nunits) {
                ++g;
                start = unit_start<Scenes>(W, g);
                nunits = W.tri_units[g];
            }
            const uint4 r = __ldg(W.tri_rec + 3 * g);
            const int base = (int)(u - start) * kTessUnit;
            const int cnt = min(kTessUnit, (int)r.y - base);
            if (lane < cnt) {
                q.tri[qn + lane] = (int)r.w;
                q.pt[qn + lane] = (uint32_t)(base + lane) | (r.z << 16);
                q.lev[qn + lane] = r.x;
            }
            if ((int)r.z != cur_scene) {
                if (lane == 0 && pending) atomicAdd(&point_count[cur_scene], pending);
                cur_scene = (int)r.z;
                pending = 0;
            }
            pending += (unsigned)cnt;
            __syncwarp();
            qn += cnt;
            if (qn >= kTessUnit) {
                tess_store32(S, q, kTessUnit, lane);
                __syncwarp();
                if (lane < qn - kTessUnit) {
                    q.tri[lane] = q.tri[kTessUnit + lane];
                    q.pt[lane] = q.pt[kTessUnit + lane];
                    q.lev[lane] = q.lev[kTessUnit + lane];
                }
                __syncwarp();
                qn -= kTessUnit;
            }
        }
    }
    tess_store32(S, q, qn, lane);
    if (lane == 0 && pending) atomicAdd(&point_count[cur_scene], pending);
    __syncthreads();
    for (int i = threadIdx.x; i < nscenes; i += blockDim.x)
        if (point_count[i] && S.get(i).stats) atomicAdd(&S.get(i).stats->total_voxel_fragments, point_count[i]);
}

template <class Scenes>
void launch_tess(const Scenes& S, const VoxWork& W, int num_sms, cudaStream_t s) {
    if (W.ntri <= 0) return;
    const int nblocks = (int)((W.ntri + kSetupThreads - 1) / kSetupThreads);
    tess_setup_kernel<Scenes><<<nblocks, kSetupThreads, 0, s>>>(S, W);
    voxelize_scan_kernel<<<1, 1024, 0, s>>>(W.block_off, nblocks);
    tess_points_kernel<Scenes><<<num_sms * 4, kWarps * 32, 0, s>>>(S, W, nblocks);
    note_launches(3);
}

}  // namespace

// The tessellation voxeliser: setup, scan, points (the same scratch as the
// rasteriser's).
void launch_tesselate(const AccumParams& P, cudaStream_t s) {
    const VoxWork W = {P.tri_rec, P.tri_units, P.tri_scan, P.block_off, P.ntri, 0};
    launch_tess(OneScene<AccumParams>{P}, W, P.num_sms, s);
    if (P.carry) {
        carry_fixup_kernel<<<dim3(kCarrySlots / 256, 1), 256, 0, s>>>(OneScene<AccumParams>{P});
        note_launches(1);
    }
}

void launch_tesselate_batch(const SceneBatch<AccumParams>& B, const VoxWork& W, int num_sms, cudaStream_t s) {
    launch_tess(ManyScenes<AccumParams>{B}, W, num_sms, s);
    carry_fixup_kernel<<<dim3(kCarrySlots / 256, B.n), 256, 0, s>>>(ManyScenes<AccumParams>{B});
    note_launches(1);
}

void accumulate_bind_scratch(AccumParams& P, void* scratch) {
    char* p = static_cast<char*>(scratch);
    const long long ntri = P.ntri;
    P.tri_rec = reinterpret_cast<uint4*>(p);
    p += align256(ntri * 48);
    P.tri_units = reinterpret_cast<uint32_t*>(p);
    p += align256(ntri * 4);
    P.tri_scan = reinterpret_cast<uint32_t*>(p);
    p += align256(ntri * 4);
    P.block_off = reinterpret_cast<uint32_t*>(p);
}

void launch_occupancy(const AccumParams& P, cudaStream_t s) {
    if (P.ntri <= 0) return;
    occupancy_kernel<<<(unsigned)((P.ntri + kOccThreads - 1) / kOccThreads), kOccThreads, 0, s>>>(
        OneScene<AccumParams>{P}, P.ntri);
    note_launches(1);
}

void launch_occupancy_batch(const SceneBatch<AccumParams>& B, long long ntri, cudaStream_t s) {
    if (ntri <= 0) return;
    occupancy_kernel<<<(unsigned)((ntri + kOccThreads - 1) / kOccThreads), kOccThreads, 0, s>>>(
        ManyScenes<AccumParams>{B}, ntri);
    note_launches(1);
}

void launch_accumulate(const AccumParams& P, cudaStream_t s) {
    const VoxWork W = {P.tri_rec, P.tri_units, P.tri_scan, P.block_off, P.ntri, P.unit_log2};
    launch_voxelize(OneScene<AccumParams>{P}, W, P.num_sms, P.blocks_per_sm, s);
}

int accumulate_batch_max_scenes() { return kMaxBatchScenes; }

void launch_accumulate_batch(const SceneBatch<AccumParams>& B, const VoxWork& W, int num_sms, int blocks_per_sm,
                             cudaStream_t s) {
    launch_voxelize(ManyScenes<AccumParams>{B}, W, num_sms, blocks_per_sm, s);
}

}  // namespace vct
