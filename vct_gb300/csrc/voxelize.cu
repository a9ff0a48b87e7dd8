// Triangle voxelisation: shaders/voxelize.geom:25-73 + voxelize.frag:75-280.
//
// Three launches, balanced at fragment granularity (triangle sizes vary by
// more than three orders of magnitude in one scene), for one scene or for the
// concatenated triangles of a batch of scenes:
//  1. voxelize_setup_kernel, one thread per triangle: the geometry-shader
//     part (dominant axis from the summed vertex normals, per-axis ortho
//     projection, snapping to the 1/256 sub-pixel grid, bounding box) into a
//     48-byte record, and the triangle's share of work: its bounding box in
//     units of 2^unit_log2 pixels (a tuning setting), with a block-local
//     exclusive scan;
//  2. voxelize_scan_kernel, one CTA: exclusive scan of the per-block totals;
//  3. voxelize_raster_kernel, persistent: every warp takes an equal
//     contiguous range of work units, tests 32 pixel centres at a time for
//     coverage, compacts covered fragments (clipped to the depth range) with
//     a ballot into a per-warp queue in shared memory, and whenever 32 are
//     queued each lane lights one fragment (all enabled lights, 5-tap PCF for
//     shadow casters) and adds it into the voxel's 32-byte accumulator record
//     with fire-and-forget 64-bit reductions.
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

struct FragQueue {
    int tri[kQueue];       // triangle index within its scene
    uint32_t pix[kQueue];  // px | py << 11 | axis << 22 | scene << 24
    float l0[kQueue], l1[kQueue], l2[kQueue], z[kQueue];
};

__device__ __forceinline__ float shadow_factor(const AccumParams& P, f3 wp) {
    return pcf5(P.shadowmap, P.sw, P.sh, P.ls, wp);
}

// ------------------------------------------------------------- 1. setup
template <class Scenes>
__global__ void __launch_bounds__(kSetupThreads) voxelize_setup_kernel(const Scenes S, const VoxWork W) {
    const long long g = (long long)blockIdx.x * kSetupThreads + threadIdx.x;
    uint32_t units = 0;
    if (g < W.ntri) {
        long long t;
        const AccumParams& P = S.get(S.find(g, t));
        const float* Pp = P.pos + t * 9;
        const float* Pn = P.nrm + t * 9;
        f3 n0 = ld3(Pn), n1 = ld3(Pn + 3), n2 = ld3(Pn + 6);
        f3 fn = normalize(add(add(n0, n1), n2));
        float ax = fabsf(fn.x), ay = fabsf(fn.y), az = fabsf(fn.z);
        int axis = 2;
        if (ax > ay && ax > az)
            axis = 0;
        else if (ay > ax && ay > az)
            axis = 1;
        if (P.axis_override >= 0 && P.axis_override <= 2) axis = P.axis_override;
        const float* M = P.mvp + 16 * axis;
        const int N = P.dim;
        float wx[3], wy[3], z[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float c[4];
            mat_vec(M, Pp[3 * k], Pp[3 * k + 1], Pp[3 * k + 2], 1.0f, c);
            float nx = __fdiv_rn(c[0], c[3]), ny = __fdiv_rn(c[1], c[3]);
            z[k] = __fdiv_rn(c[2], c[3]);
            wx[k] = (nx + 1.0f) * 0.5f * (float)N;
            wy[k] = (ny + 1.0f) * 0.5f * (float)N;
        }
        RasterTri rt;
        if (raster_setup(wx, wy, N, N, rt)) {
            const uint32_t bw = rt.px1 - rt.px0 + 1, bh = rt.py1 - rt.py0 + 1;
            const uint32_t bias = (rt.bias[0] ? 1u : 0u) | (rt.bias[1] ? 2u : 0u) | (rt.bias[2] ? 4u : 0u);
            const float inv = __fdiv_rn(1.0f, __ll2float_rn(rt.area));
            uint4* rec = W.tri_rec + 3 * g;
            rec[0] = make_uint4((uint32_t)rt.X[0], (uint32_t)rt.Y[0], (uint32_t)rt.X[1], (uint32_t)rt.Y[1]);
            rec[1] = make_uint4((uint32_t)rt.X[2], (uint32_t)rt.Y[2], __float_as_uint(z[0]), __float_as_uint(z[1]));
            rec[2] = make_uint4(__float_as_uint(z[2]), __float_as_uint(inv),
                                (uint32_t)rt.px0 | ((uint32_t)rt.py0 << 11) | ((uint32_t)axis << 22) |
                                    ((uint32_t)rt.perm1 << 24) | (bias << 25),
                                bw | (bh << 11));
            units = (bw * bh + (1u << W.unit_log2) - 1) >> W.unit_log2;
        }
        W.tri_units[g] = units;
    }
    // Block-local exclusive scan of the unit counts.
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
    if (P.warp.mode == VCT_WARP_NONE) {
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
    if (P.occupancy_only) {  // voxelize.frag:187-192
        atomicOr(P.occ + (v >> 5), 1u << (v & 31));
        return;
    }
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
            if (L.shadow_caster) lit = mul(lit, 1.0f - shadow_factor(P, wp));
            fin = add(fin, lit);
        }
        color = mk(clampf(fin.x, 0.0f, 1.0f), clampf(fin.y, 0.0f, 1.0f), clampf(fin.z, 0.0f, 1.0f));
    }
    const f3 n01 = mk((Nf.x + 1.0f) * 0.5f, (Nf.y + 1.0f) * 0.5f, (Nf.z + 1.0f) * 0.5f);
    unsigned long long* rec = reinterpret_cast<unsigned long long*>(P.acc + (long long)kAccWords * v);
    const unsigned long long qr = quant16(color.x), qg = quant16(color.y), qb = quant16(color.z);
    const unsigned long long qx = quant16(n01.x), qy = quant16(n01.y), qz = quant16(n01.z);
    // Fire-and-forget reductions: no result is waited for.
    atomicAdd(rec + 0, 1ull | (qr << 32));
    atomicAdd(rec + 1, qg | (qb << 32));
    atomicAdd(rec + 2, qx | (qy << 32));
    atomicAdd(rec + 3, qz);
    atomicOr(P.occ + (v >> 5), 1u << (v & 31));
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
    const int lane = threadIdx.x & 31;
    FragQueue& q = queues[threadIdx.x >> 5];
    const unsigned FULL = 0xffffffffu;
    const int nscenes = S.count();
    for (int i = threadIdx.x; i < nscenes; i += blockDim.x) frag_count[i] = 0;
    __syncthreads();
    const long long nw = (long long)gridDim.x * kWarps;
    const long long w = (long long)blockIdx.x * kWarps + (threadIdx.x >> 5);
    const long long total = W.block_off[nblocks];
    const long long u0 = total * w / nw, u1 = total * (w + 1) / nw;
    int qn = 0;  // queued fragments (warp-uniform)

    // Shades the first 32 queued fragments, one per lane, and counts them
    // per scene (one shared-memory atomic per distinct scene in the warp).
    auto shade32 = [&](int nact) {
        __syncwarp();
        if (lane < nact) {
            const int s = (int)(q.pix[lane] >> 24);
            const AccumParams& P = S.get(s);
            shade_fragment(P, q, lane);
            const unsigned same = __match_any_sync(__activemask(), s);
            if (lane == __ffs(same) - 1 && !P.occupancy_only) atomicAdd(&frag_count[s], (unsigned)__popc(same));
        }
        __syncwarp();
    };

    if (u0 < u1) {
        // Triangle owning unit u0: binary search over the block offsets, then
        // over the block-local scan.
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
            long long tl;
            const int scene = S.find(g, tl);
            const uint4* rp = W.tri_rec + 3 * g;
            const uint4 r0 = __ldg(rp), r1 = __ldg(rp + 1), r2 = __ldg(rp + 2);
            const int X[3] = {(int)r0.x, (int)r0.z, (int)r1.x};
            const int Y[3] = {(int)r0.y, (int)r0.w, (int)r1.y};
            const float z[3] = {__uint_as_float(r1.z), __uint_as_float(r1.w), __uint_as_float(r2.x)};
            const float inv = __uint_as_float(r2.y);
            const int px0 = (int)(r2.z & 0x7ffu), py0 = (int)((r2.z >> 11) & 0x7ffu);
            const int axis = (int)((r2.z >> 22) & 3u), perm1 = (int)((r2.z >> 24) & 1u), bias = (int)(r2.z >> 25);
            const int bw = (int)(r2.w & 0x7ffu), bh = (int)(r2.w >> 11);
            const int p_begin = (int)(u - start) << W.unit_log2;
            const int p_end = min(p_begin + (1 << W.unit_log2), bw * bh);
            for (int c = p_begin; c < p_end; c += 32) {
                const int idx = c + lane;
                bool cov = false;
                float l[3] = {0.f, 0.f, 0.f}, zf = 0.f;
                int px = 0, py = 0;
                if (idx < p_end) {
                    const int row = idx / bw;
                    py = py0 + row;
                    px = px0 + (idx - row * bw);
                    const long long sx = (long long)px * kSub + kSub / 2, sy = (long long)py * kSub + kSub / 2;
                    long long e[3];
                    cov = true;
#pragma unroll
                    for (int k = 0; k < 3; ++k) {
                        const int a = (k + 1) % 3, b = (k + 2) % 3;
                        e[k] = (long long)(X[b] - X[a]) * (sy - Y[a]) - (long long)(Y[b] - Y[a]) * (sx - X[a]);
                        cov = cov && (e[k] - ((bias >> k) & 1) >= 0);
                    }
                    if (cov) {
                        const float w0 = __ll2float_rn(e[0]) * inv, w1 = __ll2float_rn(e[1]) * inv,
                                    w2 = __ll2float_rn(e[2]) * inv;
                        l[0] = w0;
                        l[1] = perm1 ? w2 : w1;
                        l[2] = perm1 ? w1 : w2;
                        zf = interp(l, z[0], z[1], z[2]);
                        cov = zf >= -1.0f && zf <= 1.0f;  // GL clipping
                    }
                }
                const unsigned m = __ballot_sync(FULL, cov);
                if (cov) {
                    const int slot = qn + __popc(m & ((1u << lane) - 1u));
                    q.tri[slot] = (int)tl;
                    q.pix[slot] = (uint32_t)px | ((uint32_t)py << 11) | ((uint32_t)axis << 22) |
                                  ((uint32_t)scene << 24);
                    q.l0[slot] = l[0];
                    q.l1[slot] = l[1];
                    q.l2[slot] = l[2];
                    q.z[slot] = zf;
                }
                qn += __popc(m);
                if (qn >= 32) {
                    shade32(32);
                    if (lane < qn - 32) {
                        const int src = 32 + lane;
                        q.tri[lane] = q.tri[src];
                        q.pix[lane] = q.pix[src];
                        q.l0[lane] = q.l0[src];
                        q.l1[lane] = q.l1[src];
                        q.l2[lane] = q.l2[src];
                        q.z[lane] = q.z[src];
                    }
                    __syncwarp();
                    qn -= 32;
                }
            }
        }
    }
    shade32(qn);
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

}  // namespace

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
