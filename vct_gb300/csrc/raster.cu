// Frame set-up passes that the reference performs with the GL rasteriser:
// the depth-only shadow pass (src/Application.cpp:213-233) and a camera
// G-buffer (world position, normal, albedo) that replaces the depth prepass
// and the per-fragment inputs of phong.frag.  Not part of the timed path.
//
// Both use the pixel-centre integer rasteriser of vct_device.cuh with one
// warp per triangle.  Depth tests are atomicMin on keys: the shadow map keys
// are the bits of non-negative fp32 depths (ordered like the floats), the
// G-buffer keys are (depth bits << 32 | triangle id), which also makes the
// nearest-triangle choice deterministic.  Compiled with --fmad=false.
#include "vct_device.cuh"

namespace vct {

namespace {

__global__ void __launch_bounds__(256) shadow_raster_kernel(const ShadowRasterParams P) {
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long t = warp; t < P.ntri; t += nwarps) {
        const float* Pp = P.pos + t * 9;
        float wx[3], wy[3], d[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float c[4];
            mat_vec(P.ls, Pp[3 * k], Pp[3 * k + 1], Pp[3 * k + 2], 1.0f, c);
            float nx = __fdiv_rn(c[0], c[3]), ny = __fdiv_rn(c[1], c[3]), nz = __fdiv_rn(c[2], c[3]);
            wx[k] = (nx + 1.0f) * 0.5f * (float)P.w;
            wy[k] = (ny + 1.0f) * 0.5f * (float)P.h;
            d[k] = (nz + 1.0f) * 0.5f;
        }
        RasterTri rt;
        if (!raster_setup(wx, wy, P.w, P.h, rt)) continue;
        const int bw = rt.px1 - rt.px0 + 1;
        const long long npx = (long long)bw * (rt.py1 - rt.py0 + 1);
        for (long long idx = lane; idx < npx; idx += 32) {
            const int py = rt.py0 + (int)(idx / bw);
            const int px = rt.px0 + (int)(idx % bw);
            long long e[3];
            if (!raster_cover(rt, px, py, e)) continue;
            float l[3];
            raster_weights(rt, e, l);
            float z = interp(l, d[0], d[1], d[2]);
            if (!(z >= 0.0f && z <= 1.0f)) continue;
            atomicMin(P.depth_bits + (long long)py * P.w + px, __float_as_uint(z));
        }
    }
}

__global__ void __launch_bounds__(256) gbuffer_raster_kernel(const GbufferRasterParams P) {
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long t = warp; t < P.ntri; t += nwarps) {
        const float* Pp = P.pos + t * 9;
        float cv[3][4];
#pragma unroll
        for (int k = 0; k < 3; ++k) mat_vec(P.vp, Pp[3 * k], Pp[3 * k + 1], Pp[3 * k + 2], 1.0f, cv[k]);
        // Near-plane clip z >= -w (Sutherland-Hodgman), as the CPU oracle does.
        float poly[4][4];
        int np = 0;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float* a = cv[k];
            const float* b = cv[(k + 1) % 3];
            float da = a[2] + a[3], db = b[2] + b[3];
            if (da >= 0.0f) {
#pragma unroll
                for (int c = 0; c < 4; ++c) poly[np][c] = a[c];
                ++np;
            }
            if ((da >= 0.0f) != (db >= 0.0f)) {
                float s = __fdiv_rn(da, da - db);
#pragma unroll
                for (int c = 0; c < 4; ++c) poly[np][c] = a[c] + s * (b[c] - a[c]);
                ++np;
            }
        }
        for (int f = 1; f + 1 < np; ++f) {
            const float* vv[3] = {poly[0], poly[f], poly[f + 1]};
            float wx[3], wy[3], d[3];
            bool ok = true;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (!(vv[k][3] > 0.0f)) ok = false;
                float nx = __fdiv_rn(vv[k][0], vv[k][3]), ny = __fdiv_rn(vv[k][1], vv[k][3]);
                float nz = __fdiv_rn(vv[k][2], vv[k][3]);
                wx[k] = (nx + 1.0f) * 0.5f * (float)P.w;
                wy[k] = (ny + 1.0f) * 0.5f * (float)P.h;
                d[k] = (nz + 1.0f) * 0.5f;
            }
            if (!ok) continue;
            RasterTri rt;
            if (!raster_setup(wx, wy, P.w, P.h, rt)) continue;
            const int bw = rt.px1 - rt.px0 + 1;
            const long long npx = (long long)bw * (rt.py1 - rt.py0 + 1);
            for (long long idx = lane; idx < npx; idx += 32) {
                const int py = rt.py0 + (int)(idx / bw);
                const int px = rt.px0 + (int)(idx % bw);
                long long e[3];
                if (!raster_cover(rt, px, py, e)) continue;
                float l[3];
                raster_weights(rt, e, l);
                float z = interp(l, d[0], d[1], d[2]);
                if (!(z >= 0.0f && z <= 1.0f)) continue;
                unsigned long long key = ((unsigned long long)__float_as_uint(z) << 32) | (unsigned long long)(unsigned)t;
                atomicMin(P.keys + (long long)py * P.w + px, key);
            }
        }
    }
}

__device__ __forceinline__ f3 crossf(f3 a, f3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

__global__ void gbuffer_resolve_kernel(const GbufferRasterParams P) {
    const long long n = (long long)P.w * P.h;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long key = P.keys[i];
        if (key == ~0ull) {
            P.gpos[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            P.gnrm[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            P.galb[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            continue;
        }
        const int px = (int)(i % P.w), py = (int)(i / P.w);
        const long long t = (long long)(key & 0xffffffffull);
        const float* Pp = P.pos + t * 9;
        const float* Pn = P.nrm + t * 9;
        f3 p0 = ld3(Pp), p1 = ld3(Pp + 3), p2 = ld3(Pp + 6);
        float ndx = __fdiv_rn((float)px + 0.5f, (float)P.w) * 2.0f - 1.0f;
        float ndy = __fdiv_rn((float)py + 0.5f, (float)P.h) * 2.0f - 1.0f;
        float fw[4];
        mat_vec(P.ivp, ndx, ndy, 1.0f, 1.0f, fw);
        f3 dir = sub(mk(__fdiv_rn(fw[0], fw[3]), __fdiv_rn(fw[1], fw[3]), __fdiv_rn(fw[2], fw[3])), P.eye);
        f3 e1 = sub(p1, p0), e2 = sub(p2, p0);
        f3 pv = crossf(dir, e2);
        float det = dot(e1, pv);
        float u = __fdiv_rn(1.0f, 3.0f), v = u;
        if (det != 0.0f) {
            float inv = __fdiv_rn(1.0f, det);
            f3 tv = sub(P.eye, p0);
            u = dot(tv, pv) * inv;
            f3 qv = crossf(tv, e1);
            v = dot(dir, qv) * inv;
            u = clampf(u, 0.0f, 1.0f);
            v = clampf(v, 0.0f, 1.0f - u);
        }
        float w0 = 1.0f - u - v;
        f3 wp = add(add(mul(p0, w0), mul(p1, u)), mul(p2, v));
        f3 nn = normalize(add(add(mul(ld3(Pn), w0), mul(ld3(Pn + 3), u)), mul(ld3(Pn + 6), v)));
        P.gpos[i] = make_float4(wp.x, wp.y, wp.z, 1.0f);
        P.gnrm[i] = make_float4(nn.x, nn.y, nn.z, 0.0f);
        P.galb[i] = make_float4(P.albedo[3 * t], P.albedo[3 * t + 1], P.albedo[3 * t + 2], 1.0f);
    }
}

}  // namespace

void launch_shadow_raster(const ShadowRasterParams& P, cudaStream_t s) {
    launch_fill_u32(P.depth_bits, 0x3f800000u, (long long)P.w * P.h, s);  // 1.0f
    if (P.ntri <= 0) return;
    long long blocks = (P.ntri * 32 + 255) / 256;
    long long maxb = (long long)P.num_sms * 8;
    shadow_raster_kernel<<<(unsigned)(blocks < maxb ? blocks : maxb), 256, 0, s>>>(P);
    note_launches(1);
}

void launch_gbuffer_raster(const GbufferRasterParams& P, cudaStream_t s) {
    long long n = (long long)P.w * P.h;
    launch_fill_u32(reinterpret_cast<uint32_t*>(P.keys), 0xffffffffu, 2 * n, s);
    if (P.ntri > 0) {
        long long blocks = (P.ntri * 32 + 255) / 256;
        long long maxb = (long long)P.num_sms * 8;
        gbuffer_raster_kernel<<<(unsigned)(blocks < maxb ? blocks : maxb), 256, 0, s>>>(P);
        note_launches(1);
    }
    long long rb = (n + 255) / 256;
    if (rb > 8192) rb = 8192;
    gbuffer_resolve_kernel<<<(unsigned)rb, 256, 0, s>>>(P);
    note_launches(1);
}

}  // namespace vct
