// CPU oracle of the VCT hot path (test infrastructure only; see vct_oracle.h).
//
// Compiled with -ffp-contract=off so that every a*b+c below is two rounded
// operations, on x86 and on Arm alike.  The order of every fp32 operation in
// the bit-exact stages (rasterisation, voxelisation, normalisation,
// injection, mips) is part of the contract the CUDA kernels follow.
#include "vct_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------- helpers
struct f3 {
    float x, y, z;
};
static inline f3 mk(float x, float y, float z) { return {x, y, z}; }
static inline f3 add(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline f3 sub(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline f3 mul(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
static inline f3 mulv(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
static inline float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline f3 cross(f3 a, f3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// normalize(v) = v * (1 / sqrt(dot(v, v))): two IEEE-rounded operations.
static inline f3 normalize(f3 v) {
    float inv = 1.0f / std::sqrt(dot(v, v));
    return mul(v, inv);
}
static inline float length(f3 v) { return std::sqrt(dot(v, v)); }
static inline f3 ld3(const float* p) { return {p[0], p[1], p[2]}; }

// glm-style mat4 (column-major) times vec4, summed over columns in order.
static inline void mat_vec(const float* m, float x, float y, float z, float w, float out[4]) {
    for (int r = 0; r < 4; ++r) out[r] = m[0 + r] * x + m[4 + r] * y + m[8 + r] * z + m[12 + r] * w;
}

static inline float clampf(float x, float lo, float hi) { return std::fmin(std::fmax(x, lo), hi); }

// GLSL smoothstep.
static inline float smoothstep(float e0, float e1, float x) {
    float t = clampf((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

template <typename F>
static void parallel_for(int64_t n, int nthreads, F&& fn) {
    if (nthreads <= 1 || n < 2) {
        fn(0, n);
        return;
    }
    int nt = (int)std::min<int64_t>(nthreads, n);
    // Items differ in cost by orders of magnitude (a column sliver rasterises thousands of
    // fragments, a small box triangle a few; a covered pixel traces cones, a background one
    // nothing), so the threads take chunks from a shared counter. Every caller's result is
    // independent of which thread handles an item.
    const int64_t chunk = std::max<int64_t>(1, n / ((int64_t)nt * 64));
    std::atomic<int64_t> next{0};
    std::vector<std::thread> th;
    th.reserve(nt);
    for (int t = 0; t < nt; ++t) {
        th.emplace_back([&fn, &next, n, chunk] {
            for (int64_t a = next.fetch_add(chunk); a < n; a = next.fetch_add(chunk)) fn(a, std::min(n, a + chunk));
        });
    }
    for (auto& t : th) t.join();
}

// ------------------------------------------------------------ binary16
uint16_t f2h(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t exp = (x >> 23) & 0xffu;
    uint32_t man = x & 0x7fffffu;
    if (exp == 0xffu) return (uint16_t)(man ? 0x7fffu : (sign | 0x7c00u));
    int e = (int)exp - 127 + 15;
    if (e >= 31) return (uint16_t)(sign | 0x7c00u);
    if (e <= 0) {
        if (e < -10) return (uint16_t)sign;
        uint32_t full = man | 0x800000u;
        int shift = 14 - e;
        uint32_t hm = full >> shift;
        uint32_t rem = full & ((1u << shift) - 1u);
        uint32_t half = 1u << (shift - 1);
        if (rem > half || (rem == half && (hm & 1u))) hm++;
        return (uint16_t)(sign | hm);
    }
    uint32_t h = sign | ((uint32_t)e << 10) | (man >> 13);
    uint32_t rem = man & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
    return (uint16_t)h;
}

float h2f(uint16_t h) {
    uint32_t sign = ((uint32_t)h & 0x8000u) << 16;
    uint32_t exp = (h >> 10) & 0x1fu;
    uint32_t man = h & 0x3ffu;
    uint32_t x;
    if (exp == 0) {
        if (man == 0) {
            x = sign;
        } else {  // subnormal: renormalise
            int e = -1;
            do {
                man <<= 1;
                ++e;
            } while (!(man & 0x400u));
            man &= 0x3ffu;
            x = sign | ((uint32_t)(127 - 15 - e) << 23) | (man << 13);
        }
    } else if (exp == 31) {
        x = sign | 0x7f800000u | (man << 13);
    } else {
        x = sign | ((exp - 15 + 127) << 23) | (man << 13);
    }
    float f;
    std::memcpy(&f, &x, 4);
    return f;
}

// ---------------------------------------------------------- matrices (glm)
void lookat(const float e[3], const float c[3], const float u[3], float* m) {
    f3 eye = ld3(e), ctr = ld3(c), up = ld3(u);
    f3 f = normalize(sub(ctr, eye));
    f3 s = normalize(cross(f, up));
    f3 uu = cross(s, f);
    for (int i = 0; i < 16; ++i) m[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    m[0] = s.x;
    m[4] = s.y;
    m[8] = s.z;
    m[1] = uu.x;
    m[5] = uu.y;
    m[9] = uu.z;
    m[2] = -f.x;
    m[6] = -f.y;
    m[10] = -f.z;
    m[12] = -dot(s, eye);
    m[13] = -dot(uu, eye);
    m[14] = dot(f, eye);
}

void ortho(float l, float r, float b, float t, float n, float f, float* m) {
    for (int i = 0; i < 16; ++i) m[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    m[0] = 2.0f / (r - l);
    m[5] = 2.0f / (t - b);
    m[10] = -2.0f / (f - n);
    m[12] = -(r + l) / (r - l);
    m[13] = -(t + b) / (t - b);
    m[14] = -(f + n) / (f - n);
}

void matmul(const float* a, const float* b, float* out) {
    float r[16];
    for (int c = 0; c < 4; ++c)
        for (int row = 0; row < 4; ++row)
            r[c * 4 + row] = a[0 * 4 + row] * b[c * 4 + 0] + a[1 * 4 + row] * b[c * 4 + 1] +
                             a[2 * 4 + row] * b[c * 4 + 2] + a[3 * 4 + row] * b[c * 4 + 3];
    std::memcpy(out, r, sizeof r);
}

// src/Application.cpp:689-692.
void voxel_mvp(const orc_volume* v, float* out) {
    float proj[16], view[16];
    ortho(v->vmin[0], v->vmax[0], v->vmin[1], v->vmax[1], 0.0f, v->vmax[2] - v->vmin[2], proj);
    const float* c = v->vcenter;
    float ex[3] = {v->vmax[0] + c[0], 0.0f + c[1], 0.0f + c[2]};
    float ey[3] = {0.0f + c[0], v->vmax[1] + c[1], 0.0f + c[2]};
    float ez[3] = {0.0f + c[0], 0.0f + c[1], v->vmax[2] + c[2]};
    float upy[3] = {0, 1, 0}, upz[3] = {0, 0, -1};
    lookat(ex, c, upy, view);
    matmul(proj, view, out + 0);
    lookat(ey, c, upz, view);
    matmul(proj, view, out + 16);
    lookat(ez, c, upy, view);
    matmul(proj, view, out + 32);
}

// ------------------------------------------------------ rasterisation core
// Pixel-centre coverage on a 1/256 sub-pixel grid with a top-left tie rule.
// Window coordinates have the origin at the bottom-left (GL).
constexpr int64_t kSub = 256;

static inline int64_t snap(float w) {
    w = clampf(w, -1048576.0f, 1048576.0f);
    return (int64_t)std::rint(w * 256.0f);
}

static inline int64_t floordiv(int64_t a, int64_t b) {
    int64_t q = a / b;
    if ((a % b != 0) && ((a < 0) != (b < 0))) --q;
    return q;
}

struct RasterTri {
    int64_t X[3], Y[3];
    int64_t area;
    int64_t bias[3];  // 0 for top-left edges, -1 otherwise (edge k is opposite vertex k)
    int px0, px1, py0, py1;
    int perm[3];      // vertex order after orientation fix
};

// Edge function of edge a->b at p: > 0 on the interior side of a CCW triangle.
static inline int64_t edge(int64_t ax, int64_t ay, int64_t bx, int64_t by, int64_t px, int64_t py) {
    return (bx - ax) * (py - ay) - (by - ay) * (px - ax);
}

static bool raster_setup(const float wx[3], const float wy[3], int W, int H, RasterTri& t) {
    int64_t X[3], Y[3];
    for (int k = 0; k < 3; ++k) {
        X[k] = snap(wx[k]);
        Y[k] = snap(wy[k]);
    }
    int64_t area = edge(X[0], Y[0], X[1], Y[1], X[2], Y[2]);
    if (area == 0) return false;
    int p[3] = {0, 1, 2};
    if (area < 0) {
        p[1] = 2;
        p[2] = 1;
        area = -area;
    }
    for (int k = 0; k < 3; ++k) {
        t.X[k] = X[p[k]];
        t.Y[k] = Y[p[k]];
        t.perm[k] = p[k];
    }
    t.area = area;
    for (int k = 0; k < 3; ++k) {
        int a = (k + 1) % 3, b = (k + 2) % 3;
        int64_t dx = t.X[b] - t.X[a], dy = t.Y[b] - t.Y[a];
        bool tl = (dy < 0) || (dy == 0 && dx < 0);
        t.bias[k] = tl ? 0 : -1;
    }
    int64_t minx = std::min({t.X[0], t.X[1], t.X[2]}), maxx = std::max({t.X[0], t.X[1], t.X[2]});
    int64_t miny = std::min({t.Y[0], t.Y[1], t.Y[2]}), maxy = std::max({t.Y[0], t.Y[1], t.Y[2]});
    int64_t x0 = -floordiv(-(minx - kSub / 2), kSub);  // ceil
    int64_t x1 = floordiv(maxx - kSub / 2, kSub);
    int64_t y0 = -floordiv(-(miny - kSub / 2), kSub);
    int64_t y1 = floordiv(maxy - kSub / 2, kSub);
    x0 = std::max<int64_t>(x0, 0);
    y0 = std::max<int64_t>(y0, 0);
    x1 = std::min<int64_t>(x1, W - 1);
    y1 = std::min<int64_t>(y1, H - 1);
    if (x0 > x1 || y0 > y1) return false;
    t.px0 = (int)x0;
    t.px1 = (int)x1;
    t.py0 = (int)y0;
    t.py1 = (int)y1;
    return true;
}

// Barycentric edge values at pixel (px,py); returns false when not covered.
static inline bool raster_cover(const RasterTri& t, int px, int py, int64_t e[3]) {
    int64_t sx = (int64_t)px * kSub + kSub / 2, sy = (int64_t)py * kSub + kSub / 2;
    for (int k = 0; k < 3; ++k) {
        int a = (k + 1) % 3, b = (k + 2) % 3;
        e[k] = edge(t.X[a], t.Y[a], t.X[b], t.Y[b], sx, sy);
        if (e[k] + t.bias[k] < 0) return false;
    }
    return true;
}

// Interpolation weights l_k = e_k * (1 / area), in the original vertex order.
static inline void raster_weights(const RasterTri& t, const int64_t e[3], float l[3]) {
    float inv = 1.0f / (float)t.area;
    float lp[3];
    for (int k = 0; k < 3; ++k) lp[k] = (float)e[k] * inv;
    for (int k = 0; k < 3; ++k) l[t.perm[k]] = lp[k];
}

static inline float interp(const float l[3], float a, float b, float c) { return l[0] * a + l[1] * b + l[2] * c; }

// ------------------------------------------------ bilinear shadow-map fetch
// texture(shadowmap, uv) with GL_LINEAR, clamp-to-border 1.0 and a texel
// offset as textureOffset adds it (src/Application.cpp:45-53).
static inline float shadow_fetch(const float* sm, int W, int H, int i, int j) {
    if (i < 0 || j < 0 || i >= W || j >= H) return 1.0f;
    return sm[(int64_t)j * W + i];
}
static inline float shadow_bilinear(const float* sm, int W, int H, float u, float v, int ox, int oy) {
    float x = (u * (float)W + (float)ox) - 0.5f;
    float y = (v * (float)H + (float)oy) - 0.5f;
    float fx = std::floor(x), fy = std::floor(y);
    float a = x - fx, b = y - fy;
    int i = (int)fx, j = (int)fy;
    float t00 = shadow_fetch(sm, W, H, i, j), t10 = shadow_fetch(sm, W, H, i + 1, j);
    float t01 = shadow_fetch(sm, W, H, i, j + 1), t11 = shadow_fetch(sm, W, H, i + 1, j + 1);
    float bot = t00 * (1.0f - a) + t10 * a;
    float top = t01 * (1.0f - a) + t11 * a;
    return bot * (1.0f - b) + top * b;
}

// shaders/voxelize.frag:160-184 (identical to phong.frag:183-207).
static float shadow_factor(const float* sm, int W, int H, const float ls[16], f3 wp) {
    float c[4];
    mat_vec(ls, wp.x, wp.y, wp.z, 1.0f, c);
    float sx = (c[0] / c[3] + 1.0f) * 0.5f;
    float sy = (c[1] / c[3] + 1.0f) * 0.5f;
    float sz = (c[2] / c[3] + 1.0f) * 0.5f;
    float frag = sz - 0.01f;
    if (frag > 1.0f) return 0.0f;
    static const int off[5][2] = {{0, 0}, {1, 0}, {0, 1}, {-1, 0}, {0, -1}};
    float f = 0.0f;
    for (int s = 0; s < 5; ++s)
        if (frag > shadow_bilinear(sm, W, H, sx, sy, off[s][0], off[s][1])) f += 1.0f;
    return f / 5.0f;
}

static inline uint32_t quant16(float x) { return (uint32_t)std::rint(clampf(x, 0.0f, 1.0f) * 65535.0f); }

// ------------------------------------------------------------------- warping
// voxelWarpFn (common.glsl:11-18), alpha = 0.25, in the GLSL's order.
template <typename T>
static inline T warp_fn(T x) {
    T y = (T(0.25) * x + T(2.25) * x * x) + T(-1.5) * x * x * x;
    return std::min(std::max(y, T(0)), T(1));
}
// voxelWarp (common.glsl:20-27).
template <typename T>
static inline void voxel_warp(const T p[3], const float c[3], T out[3]) {
    for (int k = 0; k < 3; ++k) {
        T off = p[k] - (T)c[k];
        off = T(0.5) * off + T(0.5);
        off = warp_fn(off);
        off = T(2) * off - T(1);
        out[k] = (T)c[k] + off;
    }
}
// texture(warpmap, p).xyz: GL_LINEAR, clamp-to-edge, texel c / 65535.
template <typename T>
static inline void warp_lookup(const uint16_t* map, const T p[3], T out[3]) {
    const int D = 32;
    T f[3], a[3];
    int i0[3], i1[3];
    for (int k = 0; k < 3; ++k) {
        T u = p[k] * (T)D - T(0.5);
        f[k] = std::floor(u);
        a[k] = u - f[k];
        int i = (int)f[k];
        i0[k] = std::min(std::max(i, 0), D - 1);
        i1[k] = std::min(std::max(i + 1, 0), D - 1);
    }
    T t[8][3];
    for (int n = 0; n < 8; ++n) {
        int x = (n & 1) ? i1[0] : i0[0], y = ((n >> 1) & 1) ? i1[1] : i0[1], z = (n >> 2) ? i1[2] : i0[2];
        const uint16_t* q = map + 4 * (((int64_t)z * D + y) * D + x);
        for (int c = 0; c < 3; ++c) t[n][c] = (T)q[c] / (T)65535;
    }
    for (int c = 0; c < 3; ++c) {
        T x00 = t[0][c] * (T(1) - a[0]) + t[1][c] * a[0];
        T x10 = t[2][c] * (T(1) - a[0]) + t[3][c] * a[0];
        T x01 = t[4][c] * (T(1) - a[0]) + t[5][c] * a[0];
        T x11 = t[6][c] * (T(1) - a[0]) + t[7][c] * a[0];
        T y0 = x00 * (T(1) - a[1]) + x10 * a[1];
        T y1 = x01 * (T(1) - a[1]) + x11 * a[1];
        out[c] = y0 * (T(1) - a[2]) + y1 * a[2];
    }
}
// voxelTesselationWarpedPosition (common.glsl:37-42) of a world position:
// (pv (p, 1)).xyz / w * 0.5 + 0.5.  Results outside [-1, 2] (off the grid for
// every consumer), infinities and NaN become -1.
template <typename T>
static inline void perspective_tc(const orc_warp* w, const T p[3], T out[3]) {
    const float* m = w->pv;
    T c[4];
    for (int r = 0; r < 4; ++r)
        c[r] = (((T)m[r] * p[0] + (T)m[4 + r] * p[1]) + (T)m[8 + r] * p[2]) + (T)m[12 + r] * T(1);
    bool inside = true;
    for (int k = 0; k < 3; ++k) {
        out[k] = c[k] / c[3] * T(0.5) + T(0.5);
        inside = inside && out[k] >= T(-1) && out[k] <= T(2);
    }
    if (!inside) out[0] = out[1] = out[2] = T(-1);
}
template <typename T>
static inline void apply_warp(const orc_warp* w, T p[3]) {
    if (!w || w->mode == 0) return;
    T o[3];
    if (w->mode == 1) {
        voxel_warp(p, w->eye_tc, o);
    } else if (w->mode == 3) {
        // phong.frag:159: back to world space, then projected
        T wp[3];
        for (int k = 0; k < 3; ++k) wp[k] = (p[k] * (T)w->ext[k] + (T)w->vcenter[k]) + (T)w->vmin[k];
        perspective_tc(w, wp, o);
    } else {
        warp_lookup(w->map, p, o);
    }
    p[0] = o[0];
    p[1] = o[1];
    p[2] = o[2];
}

}  // namespace

// ================================================================ C API
extern "C" {

uint16_t orc_f32_to_f16(float f) { return f2h(f); }
float orc_f16_to_f32(uint16_t h) { return h2f(h); }
void orc_f32_to_f16_array(const float* in, uint16_t* out, int64_t n) {
    for (int64_t i = 0; i < n; ++i) out[i] = f2h(in[i]);
}
void orc_voxel_mvp(const orc_volume* vol, float out[48]) { voxel_mvp(vol, out); }
void orc_lookat(const float eye[3], const float center[3], const float up[3], float out[16]) {
    lookat(eye, center, up, out);
}
void orc_ortho(float l, float r, float b, float t, float n, float f, float out[16]) { ortho(l, r, b, t, n, f, out); }
void orc_perspective(float fovy, float aspect, float zn, float zf, float* m) {
    float th = std::tan(fovy / 2.0f);
    for (int i = 0; i < 16; ++i) m[i] = 0.0f;
    m[0] = 1.0f / (aspect * th);
    m[5] = 1.0f / th;
    m[10] = -(zf + zn) / (zf - zn);
    m[11] = -1.0f;
    m[14] = -(2.0f * zf * zn) / (zf - zn);
}
void orc_mat4_mul(const float a[16], const float b[16], float out[16]) { matmul(a, b, out); }

// --------------------------------------------------------------- voxelize
// voxelize.geom picks the axis; GL rasterises at pixel centres in a dim x dim
// viewport; voxelize.frag lights the fragment and accumulates it.
void orc_voxelize(const orc_volume* vol, const float* pos, const float* nrm, const float* albedo,
                  int64_t ntri, const orc_light* lights, int32_t nlights, int32_t lighting,
                  int32_t axis_override, const float* sm, int32_t sw, int32_t sh, const float ls[16],
                  uint32_t* count, uint64_t* sums, uint32_t* total_fragments, int32_t nthreads,
                  const orc_warp* warp) {
    // voxelize.frag reads warpVoxels and warpTexture; voxelizeTesselationWarp
    // (mode 3) leaves the rasterised grid linear.
    const bool warped = warp && warp->mode != 0 && warp->mode != 3;
    const int N = vol->dim;
    const int64_t NV = (int64_t)N * N * N;
    float mvp[48];
    voxel_mvp(vol, mvp);
    std::atomic<uint64_t> total{0};
    const bool atomic = nthreads > 1;
    auto addu = [atomic](auto* p, uint32_t v) {
        if (atomic)
            __atomic_fetch_add(p, v, __ATOMIC_RELAXED);
        else
            *p += v;
    };
    parallel_for(ntri, nthreads, [&](int64_t t0, int64_t t1) {
        uint64_t local_total = 0;
        for (int64_t t = t0; t < t1; ++t) {
            const float* P = pos + t * 9;
            const float* Nn = nrm + t * 9;
            f3 p[3] = {ld3(P), ld3(P + 3), ld3(P + 6)};
            f3 n[3] = {ld3(Nn), ld3(Nn + 3), ld3(Nn + 6)};
            // voxelize.geom:28-45 (strict >, ties fall to z).
            f3 fn = normalize(add(add(n[0], n[1]), n[2]));
            float ax = std::fabs(fn.x), ay = std::fabs(fn.y), az = std::fabs(fn.z);
            int axis = 2;
            if (ax > ay && ax > az)
                axis = 0;
            else if (ay > ax && ay > az)
                axis = 1;
            if (axis_override >= 0 && axis_override <= 2) axis = axis_override;
            const float* M = mvp + 16 * axis;
            float wx[3], wy[3], z[3];
            for (int k = 0; k < 3; ++k) {
                float c[4];
                mat_vec(M, p[k].x, p[k].y, p[k].z, 1.0f, c);
                float nx = c[0] / c[3], ny = c[1] / c[3];
                z[k] = c[2] / c[3];
                wx[k] = (nx + 1.0f) * 0.5f * (float)N;
                wy[k] = (ny + 1.0f) * 0.5f * (float)N;
            }
            RasterTri rt;
            if (!raster_setup(wx, wy, N, N, rt)) continue;
            f3 col0 = ld3(albedo + t * 3);
            for (int py = rt.py0; py <= rt.py1; ++py) {
                for (int px = rt.px0; px <= rt.px1; ++px) {
                    int64_t e[3];
                    if (!raster_cover(rt, px, py, e)) continue;
                    float l[3];
                    raster_weights(rt, e, l);
                    float zf = interp(l, z[0], z[1], z[2]);
                    if (!(zf >= -1.0f && zf <= 1.0f)) continue;  // clipped by GL
                    ++local_total;
                    f3 wp = mk(interp(l, p[0].x, p[1].x, p[2].x), interp(l, p[0].y, p[1].y, p[2].y),
                               interp(l, p[0].z, p[1].z, p[2].z));
                    f3 ni = mk(interp(l, n[0].x, n[1].x, n[2].x), interp(l, n[0].y, n[1].y, n[2].y),
                               interp(l, n[0].z, n[1].z, n[2].z));
                    f3 Nf = normalize(ni);
                    f3 color = col0;
                    if (lighting) {  // voxelize.frag:200-225
                        f3 fin = mk(0, 0, 0);
                        for (int li = 0; li < nlights; ++li) {
                            const orc_light& L = lights[li];
                            if (!L.enabled) continue;
                            f3 lc = ld3(L.color);
                            f3 lit = mk(0, 0, 0);
                            if (L.type == 0u) {
                                f3 lp = ld3(L.position);
                                f3 d = sub(lp, wp);
                                float ndl = std::fmax(0.0f, dot(Nf, normalize(d)));
                                lit = mul(mulv(mul(color, L.intensity), lc), ndl);
                                float att = 1.0f - smoothstep(0.75f * L.range, L.range, length(d));
                                lit = mul(lit, att);
                            } else if (L.type == 1u) {
                                f3 dir = ld3(L.direction);
                                float ndl = std::fmax(0.0f, dot(Nf, normalize(mk(-dir.x, -dir.y, -dir.z))));
                                lit = mul(mul(mulv(color, lc), L.intensity), ndl);
                            }
                            if (L.shadow_caster) {
                                float s = 1.0f - shadow_factor(sm, sw, sh, ls, wp);
                                lit = mul(lit, s);
                            }
                            fin = add(fin, lit);
                        }
                        color = mk(clampf(fin.x, 0.0f, 1.0f), clampf(fin.y, 0.0f, 1.0f), clampf(fin.z, 0.0f, 1.0f));
                    }
                    f3 n01 = mk((Nf.x + 1.0f) * 0.5f, (Nf.y + 1.0f) * 0.5f, (Nf.z + 1.0f) * 0.5f);
                    // voxelize.frag:79-108 with the swizzle resolved per axis.
                    float uz = (zf + 1.0f) * 0.5f;
                    float dz = (float)N * (1.0f - uz);
                    int iz = (int)dz;
                    int vx, vy, vz;
                    if (warped) {
                        // the fragment's volume coordinate: pixel centre, depth,
                        // swizzled, z flipped, warped, scaled
                        const float fN = (float)N;
                        const float ux = ((float)px + 0.5f) / fN, uy = ((float)py + 0.5f) / fN;
                        float u[3];
                        if (axis == 0) {
                            u[0] = 1.0f - uz; u[1] = uy; u[2] = ux;
                        } else if (axis == 1) {
                            u[0] = ux; u[1] = 1.0f - uz; u[2] = uy;
                        } else {
                            u[0] = ux; u[1] = uy; u[2] = uz;
                        }
                        u[2] = 1.0f - u[2];
                        apply_warp(warp, u);
                        vx = (int)(fN * u[0]);
                        vy = (int)(fN * u[1]);
                        vz = (int)(fN * u[2]);
                    } else if (axis == 0) {
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
                    int64_t v = ((int64_t)vz * N + vy) * N + vx;
                    addu(count + v, 1u);
                    addu(sums + 0 * NV + v, quant16(color.x));
                    addu(sums + 1 * NV + v, quant16(color.y));
                    addu(sums + 2 * NV + v, quant16(color.z));
                    addu(sums + 3 * NV + v, quant16(n01.x));
                    addu(sums + 4 * NV + v, quant16(n01.y));
                    addu(sums + 5 * NV + v, quant16(n01.z));
                }
            }
        }
        total.fetch_add(local_total);
    });
    if (total_fragments) *total_fragments += (uint32_t)total.load();
}

// ------------------------------------------------- tessellation voxeliser
// simpleTesselated.vert -> testTesselation.tesc -> GL's triangle primitive
// generator (point_mode, equal_spacing) -> testTesselation.tese.

// ivec3(x): truncation toward zero; NaN gives 0 and values beyond the int
// range saturate, as the GPU's conversion does.
static inline int trunc_sat(float x) {
    if (!(x == x)) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x <= -2147483648.0f) return (-2147483647 - 1);
    return (int)x;
}

// Level after clamping to [1, max] and rounding up (equal_spacing).
static inline int round_level(float level, float max_level) {
    return (int)std::ceil(std::fmin(std::fmax(level, 1.0f), max_level));
}

int32_t orc_tess_levels(const orc_volume* vol, const float* tri, float max_level, int32_t out[4]) {
    const f3 vmin = ld3(vol->vmin), vmax = ld3(vol->vmax), vc = ld3(vol->vcenter);
    const f3 ext = sub(vmax, vmin);
    const float fN = (float)vol->dim;
    const f3 a = ld3(tri), b = ld3(tri + 3), c = ld3(tri + 6);
    // testTesselation.tesc:15-21,42-43: ivec3(voxelDim * getVoxelPosition(p))
    auto vox = [&](f3 p, int v[3]) {
        v[0] = trunc_sat(fN * (((p.x - vc.x) - vmin.x) / ext.x));
        v[1] = trunc_sat(fN * (((p.y - vc.y) - vmin.y) / ext.y));
        v[2] = trunc_sat(fN * (((p.z - vc.z) - vmin.z) / ext.z));
    };
    int va[3], vb[3], vcc[3];
    vox(a, va);
    vox(b, vb);
    vox(c, vcc);
    if (va[0] == vb[0] && va[1] == vb[1] && va[2] == vb[2] && va[0] == vcc[0] && va[1] == vcc[1] &&
        va[2] == vcc[2])
        return 0;  // all levels 0: the patch is discarded
    // :51-71, edges opposite each vertex, Heron's area, altitudes
    const f3 A = sub(c, b), B = sub(c, a), C = sub(b, a);
    const float la = length(A), lb = length(B), lc = length(C);
    const float s = ((la + lb) + lc) * 0.5f;
    const float area = std::sqrt(((s * (s - la)) * (s - lb)) * (s - lc));
    const float alt[3] = {2.0f * area / la, 2.0f * area / lb, 2.0f * area / lc};
    const float max_alt = std::fmax(alt[0], std::fmax(alt[1], alt[2]));  // GLSL max: a NaN operand loses
    const f3 vs = mk(ext.x / fN, ext.y / fN, ext.z / fN);
    auto div_factor = [&](f3 e) { return std::fabs(length(mulv(normalize(e), vs))); };
    const float outer[3] = {std::fmax(1.0f, la / div_factor(A)), std::fmax(1.0f, lb / div_factor(B)),
                            std::fmax(1.0f, lc / div_factor(C))};
    const float inner = std::fmax(1.0f, max_alt / vs.x);
    // :73-76: TessLevelOuter[0] = outer.z, [1] = outer.x, [2] = outer.y
    int n = round_level(inner, max_level);
    const int m0 = round_level(outer[2], max_level), m1 = round_level(outer[0], max_level),
              m2 = round_level(outer[1], max_level);
    // An inner level of 1 with any outer level above 1 counts as 1 + epsilon.
    if (n == 1 && (m0 > 1 || m1 > 1 || m2 > 1)) n = 2;
    out[0] = n;
    out[1] = m0;
    out[2] = m1;
    out[3] = m2;
    return 1;
}

int32_t orc_tess_point_count(const int32_t lv[4]) {
    int32_t total = lv[1] + lv[2] + lv[3];  // outer ring: corners + (m - 1) per edge
    for (int q = lv[0] - 2; q >= 0; q -= 2) total += q > 0 ? 3 * q : 1;  // inner rings
    return total;
}

// OpenGL 4.6 section 11.2.2.1, point mode.  Order: the corners (1,0,0),
// (0,1,0), (0,0,1); the inner points of the u = 0 edge (outer[0], from
// vertex 1 to vertex 2), of the v = 0 edge (outer[1], vertex 2 to 0) and of
// the w = 0 edge (outer[2], vertex 0 to 1), at j/m; then the inner rings from
// the outside in.  In the equilateral domain the inner subdivision has n
// segments per edge; ring k's corner next to vertex 0 is where the
// perpendiculars to the two adjacent edges through their subdivision points
// at distance k/n from ring k-1's corners meet, which in barycentric
// coordinates is (1 - 2t, t, t) with t = 2k / (3n).  Its edges keep the
// spacing 1/n: n - 2k segments, 3 (n - 2k) points, and a single centre point
// when n - 2k = 0.
void orc_tess_coords(const int32_t lv[4], float* out) {
    const int n = lv[0];
    int64_t o = 0;
    auto put = [&](float u, float v, float w) {
        out[o++] = u;
        out[o++] = v;
        out[o++] = w;
    };
    put(1.0f, 0.0f, 0.0f);
    put(0.0f, 1.0f, 0.0f);
    put(0.0f, 0.0f, 1.0f);
    for (int j = 1; j < lv[1]; ++j) {
        const float s = (float)j / (float)lv[1];
        put(0.0f, 1.0f - s, s);
    }
    for (int j = 1; j < lv[2]; ++j) {
        const float s = (float)j / (float)lv[2];
        put(s, 0.0f, 1.0f - s);
    }
    for (int j = 1; j < lv[3]; ++j) {
        const float s = (float)j / (float)lv[3];
        put(1.0f - s, s, 0.0f);
    }
    for (int k = 1; n - 2 * k >= 0; ++k) {
        const int q = n - 2 * k;
        if (q == 0) {
            const float third = 1.0f / 3.0f;
            put(third, third, third);
            break;
        }
        const float t = (float)(2 * k) / (float)(3 * n);
        const float h = 1.0f - 2.0f * t;
        const float corner[3][3] = {{h, t, t}, {t, h, t}, {t, t, h}};
        for (int e = 0; e < 3; ++e) {
            const float* p0 = corner[e];
            const float* p1 = corner[(e + 1) % 3];
            for (int j = 0; j < q; ++j) {
                const float s = (float)j / (float)q;
                put(p0[0] + s * (p1[0] - p0[0]), p0[1] + s * (p1[1] - p0[1]), p0[2] + s * (p1[2] - p0[2]));
            }
        }
    }
}

void orc_voxelize_tess(const orc_volume* vol, const float* pos, const float* nrm, const float* albedo,
                       int64_t ntri, float max_level, const orc_warp* warp, uint32_t* count, uint64_t* sums,
                       uint64_t* total_points, int32_t nthreads) {
    const int N = vol->dim;
    const int64_t NV = (int64_t)N * N * N;
    const f3 vmin = ld3(vol->vmin), vmax = ld3(vol->vmax), vc = ld3(vol->vcenter);
    const f3 ext = sub(vmax, vmin);
    const bool persp = warp && warp->mode == 3;  // the other warps are off in the evaluation shader
    std::atomic<uint64_t> total{0};
    const bool atomic = nthreads > 1;
    auto addu = [atomic](auto* p, uint32_t v) {
        if (atomic)
            __atomic_fetch_add(p, v, __ATOMIC_RELAXED);
        else
            *p += v;
    };
    parallel_for(ntri, nthreads, [&](int64_t t0, int64_t t1) {
        uint64_t local = 0;
        std::vector<float> bc;
        for (int64_t t = t0; t < t1; ++t) {
            int32_t lv[4];
            if (!orc_tess_levels(vol, pos + t * 9, max_level, lv)) continue;
            const int32_t np = orc_tess_point_count(lv);
            bc.resize((size_t)np * 3);
            orc_tess_coords(lv, bc.data());
            local += (uint64_t)np;
            const float* P = pos + t * 9;
            const float* Nn = nrm + t * 9;
            const f3 p0 = ld3(P), p1 = ld3(P + 3), p2 = ld3(P + 6);
            const f3 n0 = ld3(Nn), n1 = ld3(Nn + 3), n2 = ld3(Nn + 6);
            const f3 col = ld3(albedo + t * 3);
            const uint32_t qc[3] = {quant16(col.x), quant16(col.y), quant16(col.z)};
            for (int32_t i = 0; i < np; ++i) {
                const float u = bc[3 * i], v = bc[3 * i + 1], w = bc[3 * i + 2];
                // testTesselation.tese:102-110: u P0 + v P1 + w P2
                const f3 p = add(add(mul(p0, u), mul(p1, v)), mul(p2, w));
                const f3 nn = add(add(mul(n0, u), mul(n1, v)), mul(n2, w));
                float tc[3];
                if (persp) {
                    const float wp[3] = {p.x, p.y, p.z};
                    perspective_tc(warp, wp, tc);
                } else {
                    tc[0] = ((p.x - vc.x) - vmin.x) / ext.x;
                    tc[1] = ((p.y - vc.y) - vmin.y) / ext.y;
                    tc[2] = ((p.z - vc.z) - vmin.z) / ext.z;
                }
                const int x = trunc_sat((float)N * tc[0]), y = trunc_sat((float)N * tc[1]),
                          z = trunc_sat((float)N * tc[2]);
                if (x < 0 || y < 0 || z < 0 || x >= N || y >= N || z >= N) continue;
                const int64_t vi = ((int64_t)z * N + y) * N + x;
                // voxelStore: normal = normalize(normal) * 0.5 + 0.5
                const f3 Nf = normalize(nn);
                addu(count + vi, 1u);
                addu(sums + 0 * NV + vi, qc[0]);
                addu(sums + 1 * NV + vi, qc[1]);
                addu(sums + 2 * NV + vi, qc[2]);
                addu(sums + 3 * NV + vi, quant16(Nf.x * 0.5f + 0.5f));
                addu(sums + 4 * NV + vi, quant16(Nf.y * 0.5f + 0.5f));
                addu(sums + 5 * NV + vi, quant16(Nf.z * 0.5f + 0.5f));
            }
        }
        total.fetch_add(local);
    });
    if (total_points) *total_points += total.load();
}

// --------------------------------------------------------------- normalize
void orc_normalize(const orc_volume* vol, float opacity, int32_t temporal, float decay,
                   const uint32_t* count, const uint64_t* sums, uint16_t* color, uint16_t* normal,
                   uint16_t* radiance, orc_stats* stats, int32_t nthreads) {
    const int64_t NV = (int64_t)vol->dim * vol->dim * vol->dim;
    std::atomic<uint32_t> uniq{0}, mx{0}, flags{0};
    parallel_for(NV, nthreads, [&](int64_t a, int64_t b) {
        uint32_t lu = 0, lm = 0, lf = 0;
        for (int64_t v = a; v < b; ++v) {
            uint32_t c = count[v];
            float alpha = 0.0f;
            uint16_t* C = color + 4 * v;
            uint16_t* Nn = normal + 4 * v;
            if (c > 0) {
                ++lu;
                lm = std::max(lm, c);
                // the sums are 64-bit: exact for any number of fragments
                float denom = 65535.0f * (float)c;
                alpha = opacity > 0.0f ? opacity : 1.0f;
                for (int k = 0; k < 3; ++k) C[k] = f2h((float)sums[k * NV + v] / denom);
                C[3] = f2h(alpha);
                for (int k = 0; k < 3; ++k) Nn[k] = f2h((float)sums[(3 + k) * NV + v] / denom);
                Nn[3] = f2h(1.0f);
            } else {
                for (int k = 0; k < 4; ++k) C[k] = Nn[k] = 0;
            }
            uint16_t* R = radiance + 4 * v;
            if (temporal) {
                // transferVoxels.comp:55-62: mix(previous, (0,0,0,a), 1 - decay)
                float w = 1.0f - decay;
                float nv[4] = {0.0f, 0.0f, 0.0f, alpha};
                for (int k = 0; k < 4; ++k) {
                    float prev = h2f(R[k]);
                    R[k] = f2h(prev * (1.0f - w) + nv[k] * w);
                }
            } else {
                R[0] = R[1] = R[2] = 0;
                R[3] = c > 0 ? f2h(alpha) : (uint16_t)0;
            }
        }
        uniq.fetch_add(lu);
        uint32_t cur = mx.load();
        while (lm > cur && !mx.compare_exchange_weak(cur, lm)) {
        }
        flags.fetch_or(lf);
    });
    if (stats) {
        stats->unique_voxels += uniq.load();
        stats->max_fragments_per_voxel = std::max(stats->max_fragments_per_voxel, mx.load());
        stats->error_flags |= flags.load();
    }
}

// ------------------------------------------------------------------ inject
// injectRadiance.comp:40-103.  Stores are idempotent per voxel, so threads
// are split by shadow-map rows and the (equal) racing stores are harmless;
// each thread writes through relaxed atomics to stay well defined.
void orc_inject(const orc_volume* vol, const float* sm, int32_t sw, int32_t sh, const float li[16],
                const float lpos[3], const float lint[3], int32_t lighting, int32_t dilate,
                const uint16_t* color, const uint16_t* normal, uint16_t* radiance, int32_t nthreads,
                const orc_warp* warp, int32_t temporal, float decay) {
    const int N = vol->dim;
    // With the temporal filter the relit colour mixes with the radiance
    // transferVoxels seeded this frame (injectRadiance.comp:86-93); every
    // store reads that seeded value (a snapshot), so racing stores agree.
    std::vector<uint16_t> seeded;
    if (temporal && lighting && !dilate) seeded.assign(radiance, radiance + 4 * (int64_t)N * N * N);
    // The dispatch covers ceil(size/16)*16 threads and the bounds test is
    // `>`: thread index == size also runs when size is not a multiple of 16.
    const int nx = std::min(((sw + 15) / 16) * 16, sw + 1);
    const int ny = std::min(((sh + 15) / 16) * 16, sh + 1);
    f3 vmin = ld3(vol->vmin), vmax = ld3(vol->vmax), vc = ld3(vol->vcenter);
    f3 ext = sub(vmax, vmin);
    auto vindex = [&](f3 w) {
        float tc[3] = {((w.x - vc.x) - vmin.x) / ext.x, ((w.y - vc.y) - vmin.y) / ext.y,
                       ((w.z - vc.z) - vmin.z) / ext.z};
        if (warp && warp->mode == 3) {  // getVoxelPosition projects the world position
            const float wp[3] = {w.x, w.y, w.z};
            perspective_tc(warp, wp, tc);
        } else {
            apply_warp(warp, tc);  // getVoxelPosition (common.glsl:44-60)
        }
        return mk((float)N * tc[0], (float)N * tc[1], (float)N * tc[2]);
    };
    f3 lvox = vindex(ld3(lpos));
    auto store = [&](int x, int y, int z, const uint16_t v[4]) {
        if (x < 0 || y < 0 || z < 0 || x >= N || y >= N || z >= N) return;
        uint64_t w;
        std::memcpy(&w, v, 8);
        uint64_t* dst = (uint64_t*)(radiance + 4 * (((int64_t)z * N + y) * N + x));
        __atomic_store_n(dst, w, __ATOMIC_RELAXED);
    };
    auto load_c = [&](int x, int y, int z, uint16_t out[4]) {
        if (x < 0 || y < 0 || z < 0 || x >= N || y >= N || z >= N) {
            out[0] = out[1] = out[2] = out[3] = 0;
            return;
        }
        std::memcpy(out, color + 4 * (((int64_t)z * N + y) * N + x), 8);
    };
    parallel_for(ny, nthreads, [&](int64_t y0, int64_t y1) {
        for (int y = (int)y0; y < (int)y1; ++y) {
            for (int x = 0; x < nx; ++x) {
                float u = (float)x / (float)sw, v = (float)y / (float)sh;
                float depth = shadow_bilinear(sm, sw, sh, u, v, 0, 0);
                float ndx = u * 2.0f - 1.0f, ndy = v * 2.0f - 1.0f, ndz = depth * 2.0f - 1.0f;
                float w4[4];
                mat_vec(li, ndx, ndy, ndz, 1.0f, w4);
                f3 vi = vindex(mk(w4[0], w4[1], w4[2]));
                int ix = (int)vi.x, iy = (int)vi.y, iz = (int)vi.z;
                if (ix >= N || iy >= N || iz >= N || ix < 0 || iy < 0 || iz < 0) continue;
                if (dilate) {
                    static const int off[7][3] = {{0, 0, 0}, {0, 0, 1}, {-1, 0, 0}, {0, 1, 0},
                                                  {0, -1, 0}, {1, 0, 0}, {-1, 0, 0}};
                    for (int k = 0; k < 7; ++k) {
                        uint16_t c[4];
                        load_c(ix + off[k][0], iy + off[k][1], iz + off[k][2], c);
                        store(ix + off[k][0], iy + off[k][1], iz + off[k][2], c);
                    }
                } else {
                    uint16_t c[4];
                    load_c(ix, iy, iz, c);
                    if (lighting) {
                        const uint16_t* Nn = normal + 4 * (((int64_t)iz * N + iy) * N + ix);
                        f3 n = mk(2.0f * h2f(Nn[0]) - 1.0f, 2.0f * h2f(Nn[1]) - 1.0f, 2.0f * h2f(Nn[2]) - 1.0f);
                        f3 L = normalize(sub(lvox, mk((float)ix, (float)iy, (float)iz)));
                        float diff = std::fmax(dot(n, L), 0.0f);
                        float rgb[3];
                        for (int k = 0; k < 3; ++k) rgb[k] = (diff * lint[k]) * h2f(c[k]);
                        uint16_t o[4];
                        o[3] = c[3];
                        if (!seeded.empty()) {
                            const uint16_t* p = seeded.data() + 4 * (((int64_t)iz * N + iy) * N + ix);
                            for (int k = 0; k < 3; ++k) rgb[k] = (1.0f - decay) * rgb[k] + decay * h2f(p[k]);
                            o[3] = p[3];
                        }
                        for (int k = 0; k < 3; ++k) o[k] = f2h(rgb[k]);
                        store(ix, iy, iz, o);
                    } else {
                        store(ix, iy, iz, c);
                    }
                }
            }
        }
    });
}

// -------------------------------------------------------------------- mips
// filterRadiance.comp BOX2: dst = 0.125 * sum of the 8 children, summed in
// the shader's offset order (z fastest, then y, then x), rounded to binary16.
void orc_build_mips(int32_t dim, int32_t levels, uint16_t* chain, int32_t nthreads) {
    int64_t off = 0;
    int S = dim;
    for (int l = 0; l + 1 < levels; ++l) {
        const uint16_t* src = chain + 4 * off;
        int D = S / 2;
        uint16_t* dst = chain + 4 * (off + (int64_t)S * S * S);
        parallel_for(D, nthreads, [&](int64_t z0, int64_t z1) {
            for (int z = (int)z0; z < (int)z1; ++z)
                for (int y = 0; y < D; ++y)
                    for (int x = 0; x < D; ++x) {
                        float acc[4] = {0, 0, 0, 0};
                        for (int ox = 0; ox < 2; ++ox)
                            for (int oy = 0; oy < 2; ++oy)
                                for (int oz = 0; oz < 2; ++oz) {
                                    const uint16_t* s =
                                        src + 4 * (((int64_t)(2 * z + oz) * S + (2 * y + oy)) * S + (2 * x + ox));
                                    for (int k = 0; k < 4; ++k) acc[k] += h2f(s[k]);
                                }
                        uint16_t* d = dst + 4 * (((int64_t)z * D + y) * D + x);
                        for (int k = 0; k < 4; ++k) d[k] = f2h(acc[k] * 0.125f);
                    }
        });
        off += (int64_t)S * S * S;
        S = D;
    }
}

}  // extern "C"

// ------------------------------------------------------------------ trace
namespace {

template <typename T>
struct V {
    T x, y, z;
};
template <typename T>
static inline V<T> vadd(V<T> a, V<T> b) {
    return {a.x + b.x, a.y + b.y, a.z + b.z};
}
template <typename T>
static inline V<T> vsub(V<T> a, V<T> b) {
    return {a.x - b.x, a.y - b.y, a.z - b.z};
}
template <typename T>
static inline V<T> vmul(V<T> a, T s) {
    return {a.x * s, a.y * s, a.z * s};
}
template <typename T>
static inline T vdot(V<T> a, V<T> b) {
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename T>
static inline V<T> vnorm(V<T> a) {
    T inv = T(1) / std::sqrt(vdot(a, a));
    return vmul(a, inv);
}

template <typename T>
struct Sampler {
    const uint16_t* chain;
    int dim, levels;
    int64_t off[16];

    void init(const uint16_t* c, int d, int l) {
        chain = c;
        dim = d;
        levels = l;
        int64_t o = 0;
        for (int i = 0; i < l; ++i) {
            off[i] = o;
            int64_t s = d >> i;
            o += s * s * s;
        }
    }
    inline void texel(int l, int S, int x, int y, int z, T out[4]) const {
        if (x < 0 || y < 0 || z < 0 || x >= S || y >= S || z >= S) {
            out[0] = out[1] = out[2] = out[3] = T(0);
            return;
        }
        const uint16_t* p = chain + 4 * (off[l] + ((int64_t)z * S + y) * S + x);
        for (int k = 0; k < 4; ++k) out[k] = (T)h2f(p[k]);
    }
    // GL_LINEAR within one level, clamp-to-border (0,0,0,0).
    void trilinear(int l, V<T> p, T out[4]) const {
        int S = dim >> l;
        T u = p.x * (T)S - T(0.5), v = p.y * (T)S - T(0.5), w = p.z * (T)S - T(0.5);
        T fu = std::floor(u), fv = std::floor(v), fw = std::floor(w);
        T a = u - fu, b = v - fv, c = w - fw;
        int i = (int)fu, j = (int)fv, k = (int)fw;
        T t[8][4];
        for (int n = 0; n < 8; ++n) texel(l, S, i + (n & 1), j + ((n >> 1) & 1), k + (n >> 2), t[n]);
        for (int ch = 0; ch < 4; ++ch) {
            T x00 = t[0][ch] * (T(1) - a) + t[1][ch] * a;
            T x10 = t[2][ch] * (T(1) - a) + t[3][ch] * a;
            T x01 = t[4][ch] * (T(1) - a) + t[5][ch] * a;
            T x11 = t[6][ch] * (T(1) - a) + t[7][ch] * a;
            T y0 = x00 * (T(1) - b) + x10 * b;
            T y1 = x01 * (T(1) - b) + x11 * b;
            out[ch] = y0 * (T(1) - c) + y1 * c;
        }
    }
    // textureLod with GL_LINEAR_MIPMAP_LINEAR minification, GL_NEAREST
    // magnification, levels [0, levels-1].
    void sample(V<T> p, T lambda, T out[4]) const {
        int q = levels - 1;
        if (lambda <= T(0)) {
            int S = dim;
            T u = p.x * (T)S, v = p.y * (T)S, w = p.z * (T)S;
            texel(0, S, (int)std::floor(u), (int)std::floor(v), (int)std::floor(w), out);
            return;
        }
        if (lambda >= (T)q) {
            trilinear(q, p, out);
            return;
        }
        T fl = std::floor(lambda);
        int d1 = (int)fl;
        T f = lambda - fl;
        T a[4], b[4];
        trilinear(d1, p, a);
        trilinear(d1 + 1, p, b);
        for (int ch = 0; ch < 4; ++ch) out[ch] = a[ch] * (T(1) - f) + b[ch] * f;
    }
};

// phong.frag:135-180 plus a length limit `maxd` in texture units.
template <typename T>
static void trace_cone(const Sampler<T>& s, V<T> pos, V<T> n, V<T> dir, const orc_cone& c, T maxd, T out[4],
                       uint64_t& samples, const orc_warp* warp) {
    dir = vnorm(dir);
    T col[3] = {0, 0, 0};
    T alpha = 0;
    T scale = T(1) / (T)s.dim;
    V<T> start = vadd(pos, vmul(vmul(n, (T)c.bias), scale));
    T h = (T)c.h0;
    T tanh = std::tan((T)c.angle / T(2));
    for (int i = 0; i < c.steps && alpha < T(0.95); ++i) {
        T r = h * tanh;
        T lod = std::log2(std::max(T(1), T(2) * r));
        V<T> sp = vadd(start, vmul(vmul(dir, h), scale));
        // any(notEqual(p, clamp(p, 0, 1))): leaves the volume, or is NaN.
        if (!(sp.x >= T(0) && sp.y >= T(0) && sp.z >= T(0) && sp.x <= T(1) && sp.y <= T(1) && sp.z <= T(1))) break;
        if (h * scale > maxd) break;
        T sc[4];
        if (warp && warp->mode != 0) {  // phong.frag:150-157
            T q[3] = {sp.x, sp.y, sp.z};
            apply_warp(warp, q);
            sp = {q[0], q[1], q[2]};
        }
        s.sample(sp, lod + (T)c.lod_offset, sc);
        ++samples;
        T a = T(1) - alpha;
        for (int k = 0; k < 3; ++k) col[k] += sc[k] * a;
        alpha += a * sc[3];
        h += r;
    }
    out[0] = col[0];
    out[1] = col[1];
    out[2] = col[2];
    out[3] = alpha;
}

// phong.frag:470-478; the -0.5909037 typo is kept.
static const double kConeDirs[6][3] = {{0, 1, 0},
                                       {0, 0.5, 0.866025},
                                       {0.823639, 0.5, 0.267617},
                                       {0.509037, 0.5, -0.700629},
                                       {-0.5909037, 0.5, -0.700629},
                                       {-0.823639, 0.5, 0.267617}};
static const double kConeWeights[6] = {0.25, 0.15, 0.15, 0.15, 0.15, 0.15};

template <typename T>
static void trace_rows(const orc_volume* vol, int levels, const uint16_t* chain, const orc_trace_params* tp,
                       const float* gpos, const float* gnrm, const float* galb, int W, int H, int row0, int row1,
                       int row_step, const float eye[3], float* irr, float* spec, float* colr, uint64_t* samples_out,
                       int nthreads, const orc_warp* warp) {
    Sampler<T> s;
    s.init(chain, vol->dim, levels);
    V<T> vmin = {(T)vol->vmin[0], (T)vol->vmin[1], (T)vol->vmin[2]};
    V<T> vmax = {(T)vol->vmax[0], (T)vol->vmax[1], (T)vol->vmax[2]};
    V<T> vc = {(T)vol->vcenter[0], (T)vol->vcenter[1], (T)vol->vcenter[2]};
    V<T> E = {(T)eye[0], (T)eye[1], (T)eye[2]};
    T maxd = tp->max_distance > 0 ? (T)tp->max_distance : std::sqrt(T(3));
    std::vector<int> rows;
    for (int r = row0; r < row1; r += std::max(1, row_step)) rows.push_back(r);
    std::atomic<uint64_t> total{0};
    parallel_for((int64_t)rows.size(), nthreads, [&](int64_t a, int64_t b) {
        uint64_t ns = 0;
        for (int64_t ri = a; ri < b; ++ri) {
            int y = rows[ri];
            for (int x = 0; x < W; ++x) {
                int64_t p = (int64_t)y * W + x;
                float ir[4] = {0, 0, 0, 0}, sp[4] = {0, 0, 0, 0}, co[4] = {0, 0, 0, 0};
                if (gpos[4 * p + 3] != 0.0f) {
                    V<T> P = {(T)gpos[4 * p], (T)gpos[4 * p + 1], (T)gpos[4 * p + 2]};
                    V<T> Nn = vnorm(V<T>{(T)gnrm[4 * p], (T)gnrm[4 * p + 1], (T)gnrm[4 * p + 2]});
                    V<T> alb = {(T)galb[4 * p], (T)galb[4 * p + 1], (T)galb[4 * p + 2]};
                    V<T> out;
                    if (tp->enable_indirect) {
                        V<T> vp = {((P.x - vc.x) - vmin.x) / (vmax.x - vmin.x), ((P.y - vc.y) - vmin.y) / (vmax.y - vmin.y),
                                   ((P.z - vc.z) - vmin.z) / (vmax.z - vmin.z)};
                        // Orthonormal basis from N: Duff et al. 2017, "Building an
                        // Orthonormal Basis, Revisited" (JCGT 6(1)).
                        T sgn = Nn.z >= T(0) ? T(1) : T(-1);
                        T ca = T(-1) / (sgn + Nn.z);
                        T cb = Nn.x * Nn.y * ca;
                        V<T> Tg = {T(1) + sgn * Nn.x * Nn.x * ca, sgn * cb, -sgn * Nn.x};
                        V<T> Bt = {cb, sgn + Nn.y * Nn.y * ca, -Nn.y};
                        T ind[4] = {0, 0, 0, 0};
                        for (int c = 0; c < 6; ++c) {
                            T dx = (T)kConeDirs[c][0], dy = (T)kConeDirs[c][1], dz = (T)kConeDirs[c][2];
                            V<T> d;
                            if (tp->ref_tbn_quirk)  // mat3(T, B, N) * d
                                d = vadd(vadd(vmul(Tg, dx), vmul(Bt, dy)), vmul(Nn, dz));
                            else  // y -> N, z -> -B (a proper rotation of the set)
                                d = vsub(vadd(vmul(Tg, dx), vmul(Nn, dy)), vmul(Bt, dz));
                            d = vnorm(d);
                            T cr[4];
                            trace_cone(s, vp, Nn, d, tp->diffuse, maxd, cr, ns, warp);
                            T w = (T)kConeWeights[c];
                            for (int k = 0; k < 4; ++k) ind[k] += w * cr[k];
                        }
                        for (int k = 0; k < 4; ++k) ir[k] = (float)ind[k];
                        T occ = T(1) - std::min(std::max(ind[3], T(0)), T(1));
                        V<T> rgb = {ind[0], ind[1], ind[2]};
                        if (tp->enable_reflections) {
                            V<T> I = vsub(P, E);
                            V<T> R = vsub(I, vmul(Nn, T(2) * vdot(Nn, I)));
                            T sr[4];
                            trace_cone(s, vp, Nn, R, tp->specular, maxd, sr, ns, warp);
                            for (int k = 0; k < 4; ++k) sp[k] = (float)sr[k];
                            rgb = vadd(rgb, vmul(V<T>{sr[0], sr[1], sr[2]}, (T)tp->reflect_scale));
                        }
                        T as = (T)tp->ambient_scale;
                        rgb = {rgb.x * (as * alb.x), rgb.y * (as * alb.y), rgb.z * (as * alb.z)};
                        out = rgb;
                        if (tp->draw_occlusion) out = vmul(out, occ);
                    } else {
                        T as = (T)tp->ambient_scale;
                        out = {as * alb.x, as * alb.y, as * alb.z};
                    }
                    if (tp->enable_postprocess) {
                        T g = T(1) / T(2.2);
                        out = {std::pow(out.x / (out.x + T(1)), g), std::pow(out.y / (out.y + T(1)), g),
                               std::pow(out.z / (out.z + T(1)), g)};
                    }
                    co[0] = (float)out.x;
                    co[1] = (float)out.y;
                    co[2] = (float)out.z;
                    co[3] = 1.0f;
                }
                if (irr) std::memcpy(irr + 4 * p, ir, 16);
                if (spec) std::memcpy(spec + 4 * p, sp, 16);
                if (colr) std::memcpy(colr + 4 * p, co, 16);
            }
        }
        total.fetch_add(ns);
    });
    if (samples_out) *samples_out += total.load();
}

// Cone set around the normal of listed pixels: dirs[c] = (x, y, z, weight)
// in the frame (T, B, N) of the Duff et al. basis; irradiance = sum of
// weight * cone rgba.  The learned path's 16-cone reference uses it.
template <typename T>
static void trace_set_pixels(const orc_volume* vol, int levels, const uint16_t* chain, const float* dirs, int ncones,
                             const orc_cone& cone, T maxd, const float* gpos, const float* gnrm, int W,
                             const int32_t* pixels, int64_t npix, float* out, uint64_t* samples_out, int nthreads,
                             const orc_warp* warp) {
    Sampler<T> s;
    s.init(chain, vol->dim, levels);
    V<T> vmin = {(T)vol->vmin[0], (T)vol->vmin[1], (T)vol->vmin[2]};
    V<T> vmax = {(T)vol->vmax[0], (T)vol->vmax[1], (T)vol->vmax[2]};
    V<T> vc = {(T)vol->vcenter[0], (T)vol->vcenter[1], (T)vol->vcenter[2]};
    (void)W;
    std::atomic<uint64_t> total{0};
    parallel_for(npix, nthreads, [&](int64_t a, int64_t b) {
        uint64_t ns = 0;
        for (int64_t i = a; i < b; ++i) {
            const int64_t p = pixels[i];
            T acc[4] = {0, 0, 0, 0};
            if (gpos[4 * p + 3] != 0.0f) {
                V<T> P = {(T)gpos[4 * p], (T)gpos[4 * p + 1], (T)gpos[4 * p + 2]};
                V<T> Nn = vnorm(V<T>{(T)gnrm[4 * p], (T)gnrm[4 * p + 1], (T)gnrm[4 * p + 2]});
                V<T> vp = {((P.x - vc.x) - vmin.x) / (vmax.x - vmin.x), ((P.y - vc.y) - vmin.y) / (vmax.y - vmin.y),
                           ((P.z - vc.z) - vmin.z) / (vmax.z - vmin.z)};
                T sgn = Nn.z >= T(0) ? T(1) : T(-1);
                T ca = T(-1) / (sgn + Nn.z);
                T cb = Nn.x * Nn.y * ca;
                V<T> Tg = {T(1) + sgn * Nn.x * Nn.x * ca, sgn * cb, -sgn * Nn.x};
                V<T> Bt = {cb, sgn + Nn.y * Nn.y * ca, -Nn.y};
                for (int c = 0; c < ncones; ++c) {
                    V<T> d = vadd(vadd(vmul(Tg, (T)dirs[4 * c]), vmul(Bt, (T)dirs[4 * c + 1])),
                                  vmul(Nn, (T)dirs[4 * c + 2]));
                    T cr[4];
                    trace_cone(s, vp, Nn, d, cone, maxd, cr, ns, warp);
                    for (int k = 0; k < 4; ++k) acc[k] += (T)dirs[4 * c + 3] * cr[k];
                }
            }
            for (int k = 0; k < 4; ++k) out[4 * i + k] = (float)acc[k];
        }
        total.fetch_add(ns);
    });
    if (samples_out) *samples_out += total.load();
}

}  // namespace

extern "C" {

void orc_trace_cone_set(const orc_volume* vol, int32_t levels, const uint16_t* chain, const float* dirs,
                        int32_t ncones, const orc_cone* cone, float max_distance, const float* gpos, const float* gnrm,
                        int32_t width, const int32_t* pixels, int64_t npix, int32_t precision, float* out,
                        uint64_t* samples, int32_t nthreads, const orc_warp* warp) {
    if (precision == 64)
        trace_set_pixels<double>(vol, levels, chain, dirs, ncones, *cone, (double)max_distance, gpos, gnrm, width,
                                 pixels, npix, out, samples, nthreads, warp);
    else
        trace_set_pixels<float>(vol, levels, chain, dirs, ncones, *cone, max_distance, gpos, gnrm, width, pixels,
                                npix, out, samples, nthreads, warp);
}

// Cheap features of the learned path (fp32): per 4x4 block, at its first
// covered pixel (order 5, 10, 6, 9, 0, 1, ... of the block, index 4 dy + dx),
// two cones along normalize(N + T) and normalize(N - T); step s samples mip
// level min(s + 1, levels - 1) trilinearly at start + dir * 2^s / dim (start
// = position + N / dim), 8 steps composited front to back (no early out;
// nothing is added once the cone has left [0,1]^3); the accumulated RGBA
// after steps 1, 3, 5 and 7 are the cone's 16 features.
void orc_learned_features(const orc_volume* vol, int32_t levels, const uint16_t* chain, const float* gpos,
                          const float* gnrm, int32_t W, int32_t H, float* out, const orc_warp* warp) {
    Sampler<float> s;
    s.init(chain, vol->dim, levels);
    static const int order[16] = {5, 10, 6, 9, 0, 1, 2, 3, 4, 7, 8, 11, 12, 13, 14, 15};
    const int wq = (W + 3) / 4, hq = (H + 3) / 4;
    const float scale = 1.0f / (float)vol->dim;
    for (int qy = 0; qy < hq; ++qy)
        for (int qx = 0; qx < wq; ++qx) {
            float* f = out + ((int64_t)qy * wq + qx) * 32;
            for (int k = 0; k < 32; ++k) f[k] = 0.0f;
            int64_t pix = -1;
            for (int k = 0; k < 16 && pix < 0; ++k) {
                const int x = 4 * qx + (order[k] & 3), y = 4 * qy + (order[k] >> 2);
                if (x < W && y < H && gpos[4 * ((int64_t)y * W + x) + 3] != 0.0f) pix = (int64_t)y * W + x;
            }
            if (pix < 0) continue;
            const float* gp = gpos + 4 * pix;
            const float* gn = gnrm + 4 * pix;
            V<float> N = vnorm(V<float>{gn[0], gn[1], gn[2]});
            const float sgn = N.z >= 0.0f ? 1.0f : -1.0f;
            const float ca = -1.0f / (sgn + N.z);
            const float cb = N.x * N.y * ca;
            V<float> Tg = {1.0f + sgn * N.x * N.x * ca, sgn * cb, -sgn * N.x};
            V<float> vp = {((gp[0] - vol->vcenter[0]) - vol->vmin[0]) / (vol->vmax[0] - vol->vmin[0]),
                           ((gp[1] - vol->vcenter[1]) - vol->vmin[1]) / (vol->vmax[1] - vol->vmin[1]),
                           ((gp[2] - vol->vcenter[2]) - vol->vmin[2]) / (vol->vmax[2] - vol->vmin[2])};
            V<float> start = vadd(vp, vmul(N, scale));
            for (int c = 0; c < 2; ++c) {
                V<float> d = vnorm(c == 0 ? vadd(N, Tg) : vsub(N, Tg));
                float h = 1.0f, alpha = 0.0f, col[3] = {0, 0, 0};
                bool inside = true;
                for (int i = 0; i < 8; ++i) {
                    V<float> sp = vadd(start, vmul(d, h * scale));
                    inside = inside && sp.x >= 0.f && sp.y >= 0.f && sp.z >= 0.f && sp.x <= 1.f && sp.y <= 1.f &&
                             sp.z <= 1.f;
                    if (inside) {
                        float smp[4];
                        float q[3] = {sp.x, sp.y, sp.z};
                        apply_warp(warp, q);
                        s.trilinear(std::min(i + 1, levels - 1), V<float>{q[0], q[1], q[2]}, smp);
                        const float a = 1.0f - alpha;
                        for (int k = 0; k < 3; ++k) col[k] += smp[k] * a;
                        alpha += a * smp[3];
                    }
                    if (i & 1) {
                        float* o = f + c * 16 + (i >> 1) * 4;
                        o[0] = col[0];
                        o[1] = col[1];
                        o[2] = col[2];
                        o[3] = alpha;
                    }
                    h *= 2.0f;
                }
            }
        }
}

void orc_trace(const orc_volume* vol, int32_t levels, const uint16_t* chain, const orc_trace_params* tp,
               const float* gpos, const float* gnrm, const float* galb, int32_t width, int32_t height,
               int32_t row0, int32_t row1, int32_t row_step, const float eye[3], int32_t precision, float* irradiance,
               float* specular, float* color, uint64_t* samples, int32_t nthreads, const orc_warp* warp) {
    row0 = std::max(0, row0);
    row1 = std::min(height, row1);
    if (precision == 64)
        trace_rows<double>(vol, levels, chain, tp, gpos, gnrm, galb, width, height, row0, row1, row_step, eye,
                           irradiance, specular, color, samples, nthreads, warp);
    else
        trace_rows<float>(vol, levels, chain, tp, gpos, gnrm, galb, width, height, row0, row1, row_step, eye,
                          irradiance, specular, color, samples, nthreads, warp);
}

// ------------------------------------------------------------------ shade
// phong.frag:183-344 (direct lighting: Cook-Torrance with GGX / Schlick-GGX /
// Schlick, or Blinn-Phong; point-light range and attenuation; PCF) and the
// composite of main (430-520).
namespace {
const float kPiRef = 3.1415982f;  // common.glsl:1 (sic)
struct Lit {
    f3 d, s;
};
inline float sq(float x) { return x * x; }
Lit cook_torrance(f3 dc, f3 lc, f3 N, f3 V, f3 L, f3 H, float r, float m) {
    const float n_dot_l = std::fmax(0.0f, dot(N, L));
    const float n_dot_v = std::fmax(0.0f, dot(N, V));
    const float n_dot_h = std::fmax(0.0f, dot(N, H));
    const float h_dot_v = std::fmax(0.0f, dot(H, V));
    const f3 fl = mk(dc.x / kPiRef, dc.y / kPiRef, dc.z / kPiRef);
    const float alpha2 = sq(r);
    const float D = alpha2 / (kPiRef * sq(sq(n_dot_h) * (alpha2 - 1.0f) + 1.0f));
    const float k = sq(r + 1.0f) / 8.0f;
    const float g1v = n_dot_v / (n_dot_v * (1.0f - k) + k);
    const float g1l = n_dot_l / (n_dot_l * (1.0f - k) + k);
    const float G = g1v * g1l;
    const float f0[3] = {0.04f * (1.0f - m) + dc.x * m, 0.04f * (1.0f - m) + dc.y * m, 0.04f * (1.0f - m) + dc.z * m};
    const float p5 = std::pow(1.0f - h_dot_v, 5.0f);
    float F[3], fct[3], kd[3];
    const float den = std::fmax(4.0f * n_dot_l * n_dot_v, 0.001f);
    for (int c = 0; c < 3; ++c) {
        F[c] = f0[c] + (1.0f - f0[c]) * p5;
        fct[c] = D * G * F[c] / den;
        kd[c] = (1.0f - F[c]) * (1.0f - m);
    }
    const float lcv[3] = {lc.x, lc.y, lc.z}, flv[3] = {fl.x, fl.y, fl.z};
    float d[3], sp[3];
    for (int c = 0; c < 3; ++c) {
        d[c] = lcv[c] * n_dot_l * kd[c] * flv[c];
        sp[c] = lcv[c] * n_dot_l * fct[c];
    }
    return {mk(d[0], d[1], d[2]), mk(sp[0], sp[1], sp[2])};
}
Lit blinn_phong(f3 dc, const orc_light& Lt, f3 N, f3 V, f3 L, float shininess, float att) {
    const float diff = std::fmax(dot(N, L), 0.0f);
    const f3 H = normalize(add(V, L));
    const float spec = std::pow(std::fmax(dot(N, H), 0.0f), shininess);
    const float lc[3] = {Lt.color[0], Lt.color[1], Lt.color[2]}, d[3] = {dc.x, dc.y, dc.z};
    float a[3], b[3];
    for (int c = 0; c < 3; ++c) {
        a[c] = diff * att * lc[c] * Lt.intensity * d[c];
        b[c] = spec * att * lc[c] * Lt.intensity * d[c];
    }
    return {mk(a[0], a[1], a[2]), mk(b[0], b[1], b[2])};
}
}  // namespace

void orc_shade(const float* gpos, const float* gnrm, const float* galb, int32_t W, int32_t H, const float eye[3],
               const orc_light* lights, int32_t nl, const float* sm, int32_t sw, int32_t sh, const float ls[16],
               const float* irr, const float* spec, const orc_shade_params* sp, float* color) {
    const f3 E = ld3(eye);
    for (int64_t p = 0; p < (int64_t)W * H; ++p) {
        float* out = color + 4 * p;
        if (gpos[4 * p + 3] == 0.0f) {
            out[0] = out[1] = out[2] = out[3] = 0.0f;
            continue;
        }
        const f3 Pw = ld3(gpos + 4 * p);
        const f3 N = normalize(ld3(gnrm + 4 * p));
        const f3 dc = ld3(galb + 4 * p);
        const f3 V = normalize(sub(E, Pw));
        f3 dsum = mk(0, 0, 0), ssum = mk(0, 0, 0);
        for (int i = 0; i < nl; ++i) {
            const orc_light& Lt = lights[i];
            if (!Lt.enabled) continue;
            Lit lg = {mk(0, 0, 0), mk(0, 0, 0)};
            if (Lt.type == 0u) {
                const f3 lp = ld3(Lt.position);
                const float dist = length(sub(lp, Pw));
                if (dist > Lt.range) continue;
                const float att = 1.0f - smoothstep(0.75f * Lt.range, Lt.range, dist);
                const f3 L = normalize(sub(lp, Pw));
                if (sp->cooktorrance) {
                    lg = cook_torrance(dc, ld3(Lt.color), N, V, L, normalize(add(V, L)), sp->roughness, sp->metallic);
                    lg.d = mul(lg.d, att);
                    lg.s = mul(lg.s, att);
                } else {
                    lg = blinn_phong(dc, Lt, N, V, L, sp->shininess, att);
                }
            } else if (Lt.type == 1u) {
                const f3 dir = ld3(Lt.direction);
                const f3 L = normalize(mk(-dir.x, -dir.y, -dir.z));
                if (sp->cooktorrance)
                    lg = cook_torrance(dc, ld3(Lt.color), N, V, L, normalize(add(V, L)), sp->roughness, sp->metallic);
                else
                    lg = blinn_phong(dc, Lt, N, V, L, sp->shininess, 1.0f);
            }
            if (Lt.shadow_caster) {
                const float sf = 1.0f - shadow_factor(sm, sw, sh, ls, Pw);
                lg.d = mul(lg.d, sf);
                lg.s = mul(lg.s, sf);
            }
            dsum = add(dsum, lg.d);
            ssum = add(ssum, lg.s);
        }
        const f3 dl = sp->enable_diffuse ? dsum : mk(0, 0, 0);
        const f3 sl = sp->enable_specular ? ssum : mk(0, 0, 0);
        f3 rgb;
        if (sp->enable_indirect && irr) {
            const float* ir = irr + 4 * p;
            const float occ = 1.0f - clampf(ir[3], 0.0f, 1.0f);
            f3 ind = ld3(ir);
            if (sp->enable_reflections && spec) ind = add(ind, mul(ld3(spec + 4 * p), sp->reflect_scale));
            const float as = sp->ambient_scale;
            ind = mk(ind.x * (as * dc.x), ind.y * (as * dc.y), ind.z * (as * dc.z));
            rgb = add(add(ind, dl), sl);
            if (sp->draw_occlusion) rgb = mul(rgb, occ);
        } else {
            rgb = add(add(mul(dc, sp->ambient_scale), dl), sl);
        }
        if (sp->enable_postprocess) {
            const float g = 1.0f / 2.2f;
            rgb = mk(std::pow(rgb.x / (rgb.x + 1.0f), g), std::pow(rgb.y / (rgb.y + 1.0f), g),
                     std::pow(rgb.z / (rgb.z + 1.0f), g));
        }
        out[0] = rgb.x;
        out[1] = rgb.y;
        out[2] = rgb.z;
        out[3] = 1.0f;
    }
}

// temporalRadianceFilter.comp: every voxel of level 0 scaled by decay.
void orc_decay_radiance(uint16_t* radiance, int64_t nv, float decay) {
    for (int64_t i = 0; i < 4 * nv; ++i) radiance[i] = f2h(h2f(radiance[i]) * decay);
}

// Normal matrix mat3(transpose(inverse(model))) of an affine model matrix:
// the transposed inverse of its upper 3x3, i.e. its cofactors / determinant.
void orc_normal_matrix(const float m[16], float out[9]) {
    float a[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) a[r][c] = m[c * 4 + r];
    float C[3][3];
    C[0][0] = a[1][1] * a[2][2] - a[1][2] * a[2][1];
    C[0][1] = -(a[1][0] * a[2][2] - a[1][2] * a[2][0]);
    C[0][2] = a[1][0] * a[2][1] - a[1][1] * a[2][0];
    C[1][0] = -(a[0][1] * a[2][2] - a[0][2] * a[2][1]);
    C[1][1] = a[0][0] * a[2][2] - a[0][2] * a[2][0];
    C[1][2] = -(a[0][0] * a[2][1] - a[0][1] * a[2][0]);
    C[2][0] = a[0][1] * a[1][2] - a[0][2] * a[1][1];
    C[2][1] = -(a[0][0] * a[1][2] - a[0][2] * a[1][0]);
    C[2][2] = a[0][0] * a[1][1] - a[0][1] * a[1][0];
    const float det = a[0][0] * C[0][0] + a[0][1] * C[0][1] + a[0][2] * C[0][2];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) out[c * 3 + r] = C[r][c] / det;
}

// voxelize.vert:15-22 for rigid actors: triangles [first, first + count) of
// actor k transformed by model k (positions) and its normal matrix (normals).
void orc_transform_actors(const float* src_pos, const float* src_nrm, const int64_t* first, const int64_t* count,
                          const float* models, int32_t n, float* dst_pos, float* dst_nrm) {
    for (int k = 0; k < n; ++k) {
        const float* M = models + 16 * k;
        float Nm[9];
        orc_normal_matrix(M, Nm);
        for (int64_t t = first[k]; t < first[k] + count[k]; ++t)
            for (int v = 0; v < 3; ++v) {
                const float* p = src_pos + t * 9 + 3 * v;
                const float* q = src_nrm + t * 9 + 3 * v;
                float o[4];
                mat_vec(M, p[0], p[1], p[2], 1.0f, o);
                for (int r = 0; r < 3; ++r) dst_pos[t * 9 + 3 * v + r] = o[r];
                for (int r = 0; r < 3; ++r) dst_nrm[t * 9 + 3 * v + r] = Nm[0 + r] * q[0] + Nm[3 + r] * q[1] + Nm[6 + r] * q[2];
            }
    }
}

void orc_warpmap(const uint8_t* occ, float high, float low, uint16_t* map) {
    const int D = 32;
    // Application.cpp:313-344: inclusive prefix sums of the occupancy along x, y, z
    std::vector<int> px(D * D * D), py(D * D * D), pz(D * D * D);
    auto at = [&](int x, int y, int z) { return (z * D + y) * D + x; };
    for (int z = 0; z < D; ++z)
        for (int y = 0; y < D; ++y) {
            int sx = 0;
            for (int x = 0; x < D; ++x) px[at(x, y, z)] = (sx += occ[at(x, y, z)] ? 1 : 0);
        }
    for (int z = 0; z < D; ++z)
        for (int x = 0; x < D; ++x) {
            int sy = 0;
            for (int y = 0; y < D; ++y) py[at(x, y, z)] = (sy += occ[at(x, y, z)] ? 1 : 0);
        }
    for (int y = 0; y < D; ++y)
        for (int x = 0; x < D; ++x) {
            int sz = 0;
            for (int z = 0; z < D; ++z) pz[at(x, y, z)] = (sz += occ[at(x, y, z)] ? 1 : 0);
        }
    // Application.cpp:346-371: per occupied count, the low and high cell
    // widths; generateWarpmapWeights.frag stores them in RGBA16F targets.
    float wl[D + 1], wh[D + 1];
    for (int o = 0; o <= D; ++o) {
        float l = 1.0f, h = 1.0f;
        if (o != 0 && o != D) {
            const int occupied = o, empty = D - o, total = D;
            h = high;
            l = (total - h * occupied) / (float)empty;
            if (l < low) {
                l = low;
                h = (total - l * empty) / (float)occupied;
            }
        }
        wl[o] = h2f(f2h(l));
        wh[o] = h2f(f2h(h));
    }
    // generateWarpmap.frag at the texel centres
    for (int z = 0; z < D; ++z)
        for (int y = 0; y < D; ++y)
            for (int x = 0; x < D; ++x) {
                const int i = at(x, y, z);
                const bool o = occ[i] != 0;
                const int idx[3] = {x, y, z};
                const int tot[3] = {px[at(D - 1, y, z)], py[at(x, D - 1, z)], pz[at(x, y, D - 1)]};
                const int part[3] = {px[i], py[i], pz[i]};
                uint16_t* t = map + 4 * (int64_t)i;
                for (int k = 0; k < 3; ++k) {
                    const float lo = wl[tot[k]], hi = wh[tot[k]];
                    const float res = o ? hi : lo;
                    const float prev = (float)(o ? part[k] - 1 : part[k]);
                    const float offset = lo * ((float)idx[k] - prev) + hi * prev;
                    const float inner = 0.5f * res;
                    const float w = (offset + inner) / (float)D;
                    t[k] = (uint16_t)std::rint(clampf(w, 0.0f, 1.0f) * 65535.0f);
                }
                t[3] = (uint16_t)((tot[0] & 0x1F) | ((tot[1] & 0x1F) << 5) | ((tot[2] & 0x1F) << 10) | ((o ? 1 : 0) << 15));
            }
}

// ------------------------------------------------------------ set-up passes
// Depth-only shadow pass (src/Application.cpp:213-233): window depth
// (ndc.z + 1) / 2, fragments outside [0,1] clipped, LESS test, clear 1.0.
void orc_render_shadowmap(const float* pos, int64_t ntri, const float ls[16], int32_t W, int32_t H, float* depth,
                          int32_t nthreads) {
    for (int64_t i = 0; i < (int64_t)W * H; ++i) depth[i] = 1.0f;
    // Rows are split across threads; each thread rasterises every triangle
    // restricted to its rows, so the depth test needs no synchronisation.
    parallel_for(H, nthreads, [&](int64_t r0, int64_t r1) {
        for (int64_t t = 0; t < ntri; ++t) {
            const float* P = pos + t * 9;
            float wx[3], wy[3], d[3];
            for (int k = 0; k < 3; ++k) {
                float c[4];
                mat_vec(ls, P[3 * k], P[3 * k + 1], P[3 * k + 2], 1.0f, c);
                float nx = c[0] / c[3], ny = c[1] / c[3], nz = c[2] / c[3];
                wx[k] = (nx + 1.0f) * 0.5f * (float)W;
                wy[k] = (ny + 1.0f) * 0.5f * (float)H;
                d[k] = (nz + 1.0f) * 0.5f;
            }
            RasterTri rt;
            if (!raster_setup(wx, wy, W, H, rt)) continue;
            int y0 = std::max<int>(rt.py0, (int)r0), y1 = std::min<int>(rt.py1, (int)r1 - 1);
            for (int py = y0; py <= y1; ++py)
                for (int px = rt.px0; px <= rt.px1; ++px) {
                    int64_t e[3];
                    if (!raster_cover(rt, px, py, e)) continue;
                    float l[3];
                    raster_weights(rt, e, l);
                    float z = interp(l, d[0], d[1], d[2]);
                    if (!(z >= 0.0f && z <= 1.0f)) continue;
                    float& dst = depth[(int64_t)py * W + px];
                    if (z < dst) dst = z;
                }
        }
    });
}

// Camera G-buffer: nearest triangle per pixel centre (key = depth bits, then
// triangle id), resolved by intersecting the pixel's ray with that triangle.
void orc_render_gbuffer(const float* pos, const float* nrm, const float* albedo, int64_t ntri, const float vp[16],
                        const float eye[3], const float ivp[16], int32_t W, int32_t H, float* gpos, float* gnrm,
                        float* galb) {
    std::vector<uint64_t> keys((size_t)W * H, ~0ull);
    for (int64_t t = 0; t < ntri; ++t) {
        const float* P = pos + t * 9;
        float cv[3][4];
        for (int k = 0; k < 3; ++k) mat_vec(vp, P[3 * k], P[3 * k + 1], P[3 * k + 2], 1.0f, cv[k]);
        // Clip against the near plane z >= -w (Sutherland-Hodgman).
        float poly[4][4];
        int np = 0;
        for (int k = 0; k < 3; ++k) {
            const float* a = cv[k];
            const float* b = cv[(k + 1) % 3];
            float da = a[2] + a[3], db = b[2] + b[3];
            if (da >= 0.0f) {
                std::memcpy(poly[np++], a, 16);
            }
            if ((da >= 0.0f) != (db >= 0.0f)) {
                float s = da / (da - db);
                for (int c = 0; c < 4; ++c) poly[np][c] = a[c] + s * (b[c] - a[c]);
                ++np;
            }
        }
        for (int f = 1; f + 1 < np; ++f) {
            const float* vv[3] = {poly[0], poly[f], poly[f + 1]};
            float wx[3], wy[3], d[3];
            bool ok = true;
            for (int k = 0; k < 3; ++k) {
                if (!(vv[k][3] > 0.0f)) ok = false;
                float nx = vv[k][0] / vv[k][3], ny = vv[k][1] / vv[k][3], nz = vv[k][2] / vv[k][3];
                wx[k] = (nx + 1.0f) * 0.5f * (float)W;
                wy[k] = (ny + 1.0f) * 0.5f * (float)H;
                d[k] = (nz + 1.0f) * 0.5f;
            }
            if (!ok) continue;
            RasterTri rt;
            if (!raster_setup(wx, wy, W, H, rt)) continue;
            for (int py = rt.py0; py <= rt.py1; ++py)
                for (int px = rt.px0; px <= rt.px1; ++px) {
                    int64_t e[3];
                    if (!raster_cover(rt, px, py, e)) continue;
                    float l[3];
                    raster_weights(rt, e, l);
                    float z = interp(l, d[0], d[1], d[2]);
                    if (!(z >= 0.0f && z <= 1.0f)) continue;
                    uint32_t zb;
                    std::memcpy(&zb, &z, 4);
                    uint64_t key = ((uint64_t)zb << 32) | (uint64_t)(uint32_t)t;
                    uint64_t& dst = keys[(size_t)py * W + px];
                    if (key < dst) dst = key;
                }
        }
    }
    f3 E = ld3(eye);
    for (int py = 0; py < H; ++py)
        for (int px = 0; px < W; ++px) {
            size_t i = (size_t)py * W + px;
            float* gp = gpos + 4 * i;
            float* gn = gnrm + 4 * i;
            float* ga = galb + 4 * i;
            if (keys[i] == ~0ull) {
                for (int k = 0; k < 4; ++k) gp[k] = gn[k] = ga[k] = 0.0f;
                continue;
            }
            int64_t t = (int64_t)(keys[i] & 0xffffffffull);
            const float* P = pos + t * 9;
            const float* Nn = nrm + t * 9;
            f3 p0 = ld3(P), p1 = ld3(P + 3), p2 = ld3(P + 6);
            float ndx = ((float)px + 0.5f) / (float)W * 2.0f - 1.0f;
            float ndy = ((float)py + 0.5f) / (float)H * 2.0f - 1.0f;
            float fw[4];
            mat_vec(ivp, ndx, ndy, 1.0f, 1.0f, fw);
            f3 dir = sub(mk(fw[0] / fw[3], fw[1] / fw[3], fw[2] / fw[3]), E);
            f3 e1 = sub(p1, p0), e2 = sub(p2, p0);
            f3 pv = cross(dir, e2);
            float det = dot(e1, pv);
            float u = 1.0f / 3.0f, v = 1.0f / 3.0f;
            if (det != 0.0f) {
                float inv = 1.0f / det;
                f3 tv = sub(E, p0);
                u = dot(tv, pv) * inv;
                f3 qv = cross(tv, e1);
                v = dot(dir, qv) * inv;
                u = clampf(u, 0.0f, 1.0f);
                v = clampf(v, 0.0f, 1.0f - u);
            }
            float w0 = 1.0f - u - v;
            f3 wp = add(add(mul(p0, w0), mul(p1, u)), mul(p2, v));
            f3 nn = normalize(add(add(mul(ld3(Nn), w0), mul(ld3(Nn + 3), u)), mul(ld3(Nn + 6), v)));
            gp[0] = wp.x;
            gp[1] = wp.y;
            gp[2] = wp.z;
            gp[3] = 1.0f;
            gn[0] = nn.x;
            gn[1] = nn.y;
            gn[2] = nn.z;
            gn[3] = 0.0f;
            ga[0] = albedo[3 * t];
            ga[1] = albedo[3 * t + 1];
            ga[2] = albedo[3 * t + 2];
            ga[3] = 1.0f;
        }
}

}  // extern "C"
