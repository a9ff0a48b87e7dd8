// Triangle voxelisation: shaders/voxelize.geom:25-73 + voxelize.frag:75-280.
//
// One warp per triangle (grid-stride).  All lanes run the geometry-shader
// part (dominant axis, per-axis projection, snapping) redundantly, then the
// lanes stride over the triangle's pixel bounding box and each covered pixel
// centre becomes one fragment: it is lit by every enabled light (shadowed by
// the 5-tap PCF for shadow casters), and its colour, normal and a count of 1
// are added into the integer accumulators with atomics.  Integer sums make
// the result independent of fragment order: it is bit-exact against the CPU
// oracle.  Compiled with --fmad=false (see vct_device.cuh).
#include "vct_device.cuh"

namespace vct {

__device__ __forceinline__ float shadow_factor(const AccumParams& P, f3 wp) {
    float c[4];
    mat_vec(P.ls, wp.x, wp.y, wp.z, 1.0f, c);
    float sx = (__fdiv_rn(c[0], c[3]) + 1.0f) * 0.5f;
    float sy = (__fdiv_rn(c[1], c[3]) + 1.0f) * 0.5f;
    float sz = (__fdiv_rn(c[2], c[3]) + 1.0f) * 0.5f;
    float frag = sz - 0.01f;
    if (frag > 1.0f) return 0.0f;
    const int ox[5] = {0, 1, 0, -1, 0};
    const int oy[5] = {0, 0, 1, 0, -1};
    float f = 0.0f;
#pragma unroll
    for (int s = 0; s < 5; ++s)
        if (frag > shadow_bilinear(P.shadowmap, P.sw, P.sh, sx, sy, ox[s], oy[s])) f += 1.0f;
    return __fdiv_rn(f, 5.0f);
}

__global__ void __launch_bounds__(256) accumulate_kernel(const AccumParams P) {
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    const int N = P.dim;
    const long long NV = (long long)N * N * N;
    unsigned frag_count = 0;

    for (long long t = warp; t < P.ntri; t += nwarps) {
        const float* Pp = P.pos + t * 9;
        const float* Pn = P.nrm + t * 9;
        f3 p[3] = {ld3(Pp), ld3(Pp + 3), ld3(Pp + 6)};
        f3 n[3] = {ld3(Pn), ld3(Pn + 3), ld3(Pn + 6)};
        f3 fn = normalize(add(add(n[0], n[1]), n[2]));
        float ax = fabsf(fn.x), ay = fabsf(fn.y), az = fabsf(fn.z);
        int axis = 2;
        if (ax > ay && ax > az)
            axis = 0;
        else if (ay > ax && ay > az)
            axis = 1;
        if (P.axis_override >= 0 && P.axis_override <= 2) axis = P.axis_override;
        const float* M = P.mvp + 16 * axis;
        float wx[3], wy[3], z[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float c[4];
            mat_vec(M, p[k].x, p[k].y, p[k].z, 1.0f, c);
            float nx = __fdiv_rn(c[0], c[3]), ny = __fdiv_rn(c[1], c[3]);
            z[k] = __fdiv_rn(c[2], c[3]);
            wx[k] = (nx + 1.0f) * 0.5f * (float)N;
            wy[k] = (ny + 1.0f) * 0.5f * (float)N;
        }
        RasterTri rt;
        if (!raster_setup(wx, wy, N, N, rt)) continue;
        const f3 col0 = ld3(P.albedo + t * 3);
        const int bw = rt.px1 - rt.px0 + 1;
        const int npx = bw * (rt.py1 - rt.py0 + 1);
        for (int idx = lane; idx < npx; idx += 32) {
            const int py = rt.py0 + idx / bw;
            const int px = rt.px0 + idx % bw;
            long long e[3];
            if (!raster_cover(rt, px, py, e)) continue;
            float l[3];
            raster_weights(rt, e, l);
            float zf = interp(l, z[0], z[1], z[2]);
            if (!(zf >= -1.0f && zf <= 1.0f)) continue;
            ++frag_count;
            f3 wp = mk(interp(l, p[0].x, p[1].x, p[2].x), interp(l, p[0].y, p[1].y, p[2].y),
                       interp(l, p[0].z, p[1].z, p[2].z));
            f3 ni = mk(interp(l, n[0].x, n[1].x, n[2].x), interp(l, n[0].y, n[1].y, n[2].y),
                       interp(l, n[0].z, n[1].z, n[2].z));
            f3 Nf = normalize(ni);
            f3 color = col0;
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
                        float att = 1.0f - smoothstep(0.75f * L.range, L.range, length(d));
                        lit = mul(lit, att);
                    } else if (L.type == 1u) {
                        float ndl = fmaxf(0.0f, dot(Nf, normalize(mk(-L.direction.x, -L.direction.y, -L.direction.z))));
                        lit = mul(mul(mulv(color, L.color), L.intensity), ndl);
                    }
                    if (L.shadow_caster) lit = mul(lit, 1.0f - shadow_factor(P, wp));
                    fin = add(fin, lit);
                }
                color = mk(clampf(fin.x, 0.0f, 1.0f), clampf(fin.y, 0.0f, 1.0f), clampf(fin.z, 0.0f, 1.0f));
            }
            f3 n01 = mk((Nf.x + 1.0f) * 0.5f, (Nf.y + 1.0f) * 0.5f, (Nf.z + 1.0f) * 0.5f);
            float uz = (zf + 1.0f) * 0.5f;
            float dz = (float)N * (1.0f - uz);
            int iz = __float2int_rz(dz);
            int vx, vy, vz;
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
            if (vx < 0 || vy < 0 || vz < 0 || vx >= N || vy >= N || vz >= N) continue;
            const long long v = ((long long)vz * N + vy) * N + vx;
            atomicAdd(P.count + v, 1u);
            atomicAdd(P.sums + 0 * NV + v, quant16(color.x));
            atomicAdd(P.sums + 1 * NV + v, quant16(color.y));
            atomicAdd(P.sums + 2 * NV + v, quant16(color.z));
            atomicAdd(P.sums + 3 * NV + v, quant16(n01.x));
            atomicAdd(P.sums + 4 * NV + v, quant16(n01.y));
            atomicAdd(P.sums + 5 * NV + v, quant16(n01.z));
        }
    }
    // Warp-aggregated fragment counter (VoxelizeInfo.totalVoxelFragments).
    unsigned total = __reduce_add_sync(0xffffffffu, frag_count);
    if (lane == 0 && total) atomicAdd(&P.stats->total_voxel_fragments, total);
}

void launch_accumulate(const AccumParams& P, cudaStream_t s) {
    if (P.ntri <= 0) return;
    long long warps_needed = P.ntri;
    long long blocks = (warps_needed * 32 + 255) / 256;
    int maxb = P.num_sms * 8;
    if (blocks > maxb) blocks = maxb;
    accumulate_kernel<<<(unsigned)blocks, 256, 0, s>>>(P);
    note_launches(1);
}

}  // namespace vct
