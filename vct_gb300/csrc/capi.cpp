// C ABI of the VCT hot path (include/vct.h): context lifetime, argument
// validation, stream-ordered launches.  Compiled with -ffp-contract=off: the
// host-side matrices and the voxel position of the light are computed with
// the same fp32 operation order as the GLSL host code they replace.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "host.h"

using namespace vct;
using namespace vct::host;


namespace vct {
static std::atomic<unsigned long long> g_launches{0};
void note_launches(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }
}  // namespace vct

namespace vct {
namespace host {

thread_local std::string g_err;

vct_status fail(vct_status s, const std::string& msg) {
    g_err = msg;
    return s;
}


// ----------------------------------------------------------- glm-style math
struct hf3 {
    float x, y, z;
};
inline hf3 hsub(hf3 a, hf3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float hdot(hf3 a, hf3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline hf3 hcross(hf3 a, hf3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline hf3 hnorm(hf3 v) {
    float inv = 1.0f / std::sqrt(hdot(v, v));
    return {v.x * inv, v.y * inv, v.z * inv};
}

void mat_identity(float* m) {
    for (int i = 0; i < 16; ++i) m[i] = (i % 5 == 0) ? 1.0f : 0.0f;
}
// glm::lookAt (right handed).
void look_at(hf3 eye, hf3 center, hf3 up, float* m) {
    hf3 f = hnorm(hsub(center, eye));
    hf3 s = hnorm(hcross(f, up));
    hf3 u = hcross(s, f);
    mat_identity(m);
    m[0] = s.x;
    m[4] = s.y;
    m[8] = s.z;
    m[1] = u.x;
    m[5] = u.y;
    m[9] = u.z;
    m[2] = -f.x;
    m[6] = -f.y;
    m[10] = -f.z;
    m[12] = -hdot(s, eye);
    m[13] = -hdot(u, eye);
    m[14] = hdot(f, eye);
}
// glm::ortho (depth range -1..1).
void ortho(float l, float r, float b, float t, float n, float f, float* m) {
    mat_identity(m);
    m[0] = 2.0f / (r - l);
    m[5] = 2.0f / (t - b);
    m[10] = -2.0f / (f - n);
    m[12] = -(r + l) / (r - l);
    m[13] = -(t + b) / (t - b);
    m[14] = -(f + n) / (f - n);
}
// glm operator* for mat4: column c of a*b = sum_k a[k] * b[c][k], in order.
void mat_mul(const float* a, const float* b, float* out) {
    float r[16];
    for (int c = 0; c < 4; ++c)
        for (int row = 0; row < 4; ++row)
            r[c * 4 + row] = a[row] * b[c * 4 + 0] + a[4 + row] * b[c * 4 + 1] + a[8 + row] * b[c * 4 + 2] +
                             a[12 + row] * b[c * 4 + 3];
    std::memcpy(out, r, sizeof r);
}

// src/Application.cpp:689-692.
void voxel_mvp(const vct_config& c, float* out) {
    float proj[16], view[16];
    ortho(c.voxel_min[0], c.voxel_max[0], c.voxel_min[1], c.voxel_max[1], 0.0f, c.voxel_max[2] - c.voxel_min[2], proj);
    hf3 ctr = {c.voxel_center[0], c.voxel_center[1], c.voxel_center[2]};
    hf3 ex = {c.voxel_max[0] + ctr.x, 0.0f + ctr.y, 0.0f + ctr.z};
    hf3 ey = {0.0f + ctr.x, c.voxel_max[1] + ctr.y, 0.0f + ctr.z};
    hf3 ez = {0.0f + ctr.x, 0.0f + ctr.y, c.voxel_max[2] + ctr.z};
    look_at(ex, ctr, {0, 1, 0}, view);
    mat_mul(proj, view, out);
    look_at(ey, ctr, {0, 0, -1}, view);
    mat_mul(proj, view, out + 16);
    look_at(ez, ctr, {0, 1, 0}, view);
    mat_mul(proj, view, out + 32);
}

bool is_pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }
int ilog2(int v) {
    int l = 0;
    while ((1 << (l + 1)) <= v) ++l;
    return l;
}

vct_status validate_config(const vct_config* c) {
    if (!c) return fail(VCT_ERR_INVALID_ARGUMENT, "config is NULL");
    if (!is_pow2(c->voxel_dim) || c->voxel_dim < 16 || c->voxel_dim > 1024)
        return fail(VCT_ERR_INVALID_ARGUMENT, "voxel_dim must be a power of two in [16, 1024]");
    for (int k = 0; k < 3; ++k) {
        if (!std::isfinite(c->voxel_min[k]) || !std::isfinite(c->voxel_max[k]) || !std::isfinite(c->voxel_center[k]))
            return fail(VCT_ERR_INVALID_ARGUMENT, "volume bounds must be finite");
        if (!(c->voxel_max[k] > c->voxel_min[k])) return fail(VCT_ERR_INVALID_ARGUMENT, "voxel_max must exceed voxel_min");
        // voxelize.frag maps fragments to voxels through the per-axis ortho
        // projections; that equals voxelLinearPosition only for a symmetric
        // cubic volume (min = -max, equal extents).
        if (c->voxel_min[k] != -c->voxel_max[k])
            return fail(VCT_ERR_INVALID_ARGUMENT, "volume must be symmetric: voxel_min = -voxel_max");
        if (c->voxel_max[k] != c->voxel_max[0]) return fail(VCT_ERR_INVALID_ARGUMENT, "volume must be cubic");
    }
    if (c->voxel_levels < 0) return fail(VCT_ERR_INVALID_ARGUMENT, "voxel_levels must be >= 0");
    return VCT_OK;
}

vct_status validate_params(const vct_params* p) {
    if (!p) return fail(VCT_ERR_INVALID_ARGUMENT, "params is NULL");
    const vct_cone_settings* cs[2] = {&p->diffuse_cone, &p->specular_cone};
    for (auto c : cs) {
        if (c->steps < 0 || c->steps > 4096) return fail(VCT_ERR_INVALID_ARGUMENT, "cone steps must be in [0, 4096]");
        if (!(c->cone_angle > 0.0f) || !(c->cone_angle < 3.14159f))
            return fail(VCT_ERR_INVALID_ARGUMENT, "cone angle must be in (0, pi)");
        if (!std::isfinite(c->bias) || !std::isfinite(c->lod_offset) || !(c->cone_initial_height > 0.0f))
            return fail(VCT_ERR_INVALID_ARGUMENT, "cone bias/lod offset must be finite, initial height > 0");
    }
    if (p->trace_filter != VCT_FILTER_SOFTWARE && p->trace_filter != VCT_FILTER_HARDWARE &&
        p->trace_filter != VCT_FILTER_HARDWARE_LEVELS && p->trace_filter != VCT_FILTER_HYBRID)
        return fail(VCT_ERR_INVALID_ARGUMENT, "trace_filter must be one of VCT_FILTER_*");
    if (p->axis_override < -1 || p->axis_override > 2) return fail(VCT_ERR_INVALID_ARGUMENT, "axis_override in [-1, 2]");
    if (!std::isfinite(p->voxel_set_opacity) || !std::isfinite(p->temporal_decay))
        return fail(VCT_ERR_INVALID_ARGUMENT, "opacity/decay must be finite");
    if (p->warp_mode < VCT_WARP_NONE || p->warp_mode > VCT_WARP_PERSPECTIVE)
        return fail(VCT_ERR_INVALID_ARGUMENT, "warp_mode must be one of VCT_WARP_*");
    if (p->voxelize_tesselation != 0 && p->voxelize_tesselation != 1)
        return fail(VCT_ERR_INVALID_ARGUMENT, "voxelize_tesselation must be 0 or 1");
    if (!(p->max_tess_level >= 1.0f && p->max_tess_level <= (float)VCT_MAX_TESS_LEVEL))
        return fail(VCT_ERR_INVALID_ARGUMENT, "max_tess_level must be in [1, VCT_MAX_TESS_LEVEL]");
    for (int i = 0; i < 16; ++i)
        if (!std::isfinite(p->pv[i])) return fail(VCT_ERR_INVALID_ARGUMENT, "pv must be finite");
    if (!std::isfinite(p->roughness) || !std::isfinite(p->metallic) || !std::isfinite(p->shininess))
        return fail(VCT_ERR_INVALID_ARGUMENT, "roughness, metallic and shininess must be finite");
    if (!(p->warp_high_resolution > 0.0f && p->warp_high_resolution <= 32.0f) ||
        !(p->warp_low_resolution > 0.0f && p->warp_low_resolution <= 32.0f))
        return fail(VCT_ERR_INVALID_ARGUMENT, "warp resolutions must be in (0, 32]");
    return VCT_OK;
}

vct_status validate_tris(const vct_triangles* t) {
    if (!t) return fail(VCT_ERR_INVALID_ARGUMENT, "triangles is NULL");
    if (t->count < 0 || t->count > 0x7fffffffLL) return fail(VCT_ERR_INVALID_ARGUMENT, "triangle count out of range");
    if (t->count > 0 && (!t->positions_dev || !t->normals_dev || !t->albedo_dev))
        return fail(VCT_ERR_INVALID_ARGUMENT, "triangle arrays must be non-NULL");
    return VCT_OK;
}

vct_status validate_shadow(const vct_shadow_desc* s, bool needed) {
    if (!needed) return VCT_OK;
    if (!s) return fail(VCT_ERR_INVALID_ARGUMENT, "shadow description is NULL");
    if (!s->shadowmap_dev || s->width <= 0 || s->height <= 0 || s->width > 32768 || s->height > 32768)
        return fail(VCT_ERR_INVALID_ARGUMENT, "shadow map pointer/size invalid");
    return VCT_OK;
}

vct_status validate_lights(const vct_light* lights, int n, bool* needs_shadow) {
    *needs_shadow = false;
    if (n < 0 || n > VCT_MAX_LIGHTS) return fail(VCT_ERR_INVALID_ARGUMENT, "n_lights must be in [0, 16]");
    if (n > 0 && !lights) return fail(VCT_ERR_INVALID_ARGUMENT, "lights is NULL");
    for (int i = 0; i < n; ++i) {
        if (lights[i].type > 1u) return fail(VCT_ERR_INVALID_ARGUMENT, "light type must be 0 (point) or 1 (directional)");
        if (lights[i].enabled && lights[i].shadow_caster) *needs_shadow = true;
    }
    return VCT_OK;
}

vct_status validate_gbuffer(const vct_gbuffer* g) {
    if (!g) return fail(VCT_ERR_INVALID_ARGUMENT, "gbuffer is NULL");
    if (g->width <= 0 || g->height <= 0 || g->width > 16384 || g->height > 16384)
        return fail(VCT_ERR_INVALID_ARGUMENT, "gbuffer size out of range");
    if (!g->position_dev || !g->normal_dev || !g->albedo_dev)
        return fail(VCT_ERR_INVALID_ARGUMENT, "gbuffer planes must be non-NULL");
    return VCT_OK;
}

uint2* level_ptr(uint2* chain, const vct_ctx* ctx, int l) { return chain + ctx->level_off[l]; }

f3 to_f3(const float* p) { return {p[0], p[1], p[2]}; }

}  // namespace host
}  // namespace vct

namespace vct {

vct_status set_error(vct_status s, const char* msg) { return fail(s, msg); }

void voxel_mvp_host(const vct_config& c, float out[48]) { voxel_mvp(c, out); }

vct_status validate_voxelize_inputs(const vct_config* cfg, const vct_params* p, const vct_triangles* t,
                                    const vct_light* lights, int n, const vct_shadow_desc* shadow, bool* need_shadow) {
    vct_status s = validate_config(cfg);
    if (s == VCT_OK) s = validate_params(p);
    if (s == VCT_OK) s = validate_tris(t);
    if (s == VCT_OK) s = validate_lights(lights, n, need_shadow);
    if (s != VCT_OK) return s;
    *need_shadow = *need_shadow && p->voxelize_lighting;
    return validate_shadow(shadow, *need_shadow);
}

void fill_accum_inputs(const vct_config& cfg, const vct_params& prm, const float mvp[48], const vct_triangles* t,
                       const vct_light* lights, int n, const vct_shadow_desc* sh, AccumParams& P) {
    std::memset(&P, 0, sizeof P);
    P.pos = t->positions_dev;
    P.nrm = t->normals_dev;
    P.albedo = t->albedo_dev;
    P.ntri = t->count;
    P.dim = cfg.voxel_dim;
    P.lighting = prm.voxelize_lighting;
    P.axis_override = prm.axis_override;
    P.nlights = n;
    P.unit_log2 = 9;
    P.blocks_per_sm = 3;
    for (int i = 0; i < n; ++i) {
        LightDev& L = P.lights[i];
        L.position = to_f3(lights[i].position);
        L.direction = to_f3(lights[i].direction);
        L.color = to_f3(lights[i].color);
        L.range = lights[i].range;
        L.intensity = lights[i].intensity;
        L.enabled = lights[i].enabled;
        L.shadow_caster = lights[i].shadow_caster;
        L.type = lights[i].type;
        // Hoisted per-light terms of voxelize.frag, same fp32 operations.
        hf3 nd = {-lights[i].direction[0], -lights[i].direction[1], -lights[i].direction[2]};
        hf3 ndn = hnorm(nd);
        L.neg_dir_n = {ndn.x, ndn.y, ndn.z};
        L.range075 = 0.75f * lights[i].range;
    }
    std::memcpy(P.mvp, mvp, sizeof P.mvp);
    P.vmin = to_f3(cfg.voxel_min);
    P.vcenter = to_f3(cfg.voxel_center);
    P.ext = {cfg.voxel_max[0] - cfg.voxel_min[0], cfg.voxel_max[1] - cfg.voxel_min[1],
             cfg.voxel_max[2] - cfg.voxel_min[2]};
    P.max_tess_level = prm.max_tess_level;
    if (sh) {
        std::memcpy(P.ls, sh->ls, sizeof P.ls);
        P.shadowmap = sh->shadowmap_dev;
        P.sw = sh->width;
        P.sh = sh->height;
    }
}

}  // namespace vct

namespace vct {
namespace host {

void default_tuning(vct_tuning& t) {
    t.voxel_unit_pixels = 512;
    t.voxel_blocks_per_sm = 3;
    t.trace_tile_w = 16;
    t.trace_tile_h = 16;
    t.trace_warp_w = 8;
}

vct_status validate_tuning(const vct_tuning* t) {
    if (!t) return fail(VCT_ERR_INVALID_ARGUMENT, "tuning is NULL");
    if (!is_pow2(t->voxel_unit_pixels) || t->voxel_unit_pixels < 32 || t->voxel_unit_pixels > 8192)
        return fail(VCT_ERR_INVALID_ARGUMENT, "voxel_unit_pixels must be a power of two in [32, 8192]");
    if (t->voxel_blocks_per_sm < 1 || t->voxel_blocks_per_sm > 3)
        return fail(VCT_ERR_INVALID_ARGUMENT, "voxel_blocks_per_sm must be in [1, 3]");
    const int tw = t->trace_tile_w, th = t->trace_tile_h, ww = t->trace_warp_w;
    if (!is_pow2(tw) || tw < 4 || tw > 64 || tw * th != 256)
        return fail(VCT_ERR_INVALID_ARGUMENT, "trace tile must be tile_w x tile_h = 256 with tile_w in [4, 64]");
    if (!is_pow2(ww) || ww * 8 < tw || ww > tw || ww > 32)
        return fail(VCT_ERR_INVALID_ARGUMENT, "trace_warp_w must be a power of two in [tile_w/8, min(tile_w, 32)]");
    return VCT_OK;
}

void apply_tuning(const vct_tuning& t, AccumParams& P) {
    P.unit_log2 = ilog2(t.voxel_unit_pixels);
    P.blocks_per_sm = t.voxel_blocks_per_sm;
}

void apply_tuning(const vct_tuning& t, TraceParams& P) {
    P.tile_w_log2 = ilog2(t.trace_tile_w);
    P.tile_h_log2 = ilog2(t.trace_tile_h);
    P.warp_w_log2 = ilog2(t.trace_warp_w);
}

WarpDev warp_dev(const vct_ctx* ctx, const float* eye) {
    WarpDev W;
    std::memset(&W, 0, sizeof W);
    W.mode = ctx->params.warp_mode;
    W.mapf = ctx->warpmap_f;
    std::memcpy(W.pv, ctx->params.pv, sizeof W.pv);
    W.vmin = to_f3(ctx->cfg.voxel_min);
    W.vcenter = to_f3(ctx->cfg.voxel_center);
    W.ext = {ctx->cfg.voxel_max[0] - ctx->cfg.voxel_min[0], ctx->cfg.voxel_max[1] - ctx->cfg.voxel_min[1],
             ctx->cfg.voxel_max[2] - ctx->cfg.voxel_min[2]};
    if (eye) {  // voxelLinearPosition(eye) (common.glsl:6-9)
        float tc[3];
        for (int k = 0; k < 3; ++k)
            tc[k] = ((eye[k] - ctx->cfg.voxel_center[k]) - ctx->cfg.voxel_min[k]) /
                    (ctx->cfg.voxel_max[k] - ctx->cfg.voxel_min[k]);
        W.eye_tc = {tc[0], tc[1], tc[2]};
    }
    return W;
}

vct_status build_warpmap(vct_ctx* ctx, const AccumParams& A, cudaStream_t st) {
    // voxelize.frag:187-192 into the 32^3 occupancy grid (Application.cpp:
    // 235-285): the rasteriser's rule at a 32^2 viewport, unwarped.
    AccumParams O = A;
    O.dim = VCT_WARP_DIM;
    O.occ = ctx->occ32;
    O.acc = nullptr;
    O.stats = nullptr;
    O.warp.mode = VCT_WARP_NONE;
    VCT_CUDA(cudaMemsetAsync(ctx->occ32, 0, (VCT_WARP_DIM * VCT_WARP_DIM * VCT_WARP_DIM / 32) * 4, st));
    launch_occupancy(O, st);
    VCT_CHECK_LAUNCH("warp occupancy");
    launch_warpmap(ctx->occ32, ctx->params.warp_high_resolution, ctx->params.warp_low_resolution, ctx->warpmap,
                   ctx->warpmap_f, st);
    VCT_CHECK_LAUNCH("warp map");
    return VCT_OK;
}

// The voxeliser the parameters select: rasterising (voxelize.geom/.frag) or
// tessellating (testTesselation.tesc/.tese).
void launch_voxelizer(const vct_ctx* ctx, const AccumParams& P, cudaStream_t st) {
    if (ctx->params.voxelize_tesselation) {
        // (errors of these clears surface at the launch check)
        cudaMemsetAsync(P.carry, 0, (size_t)kCarryBytes, st);
        cudaMemsetAsync(P.brick_exact, 0, (size_t)(ctx->nv / 4096 + 1) * 4, st);
        launch_tesselate(P, st);
    } else {
        launch_accumulate(P, st);
    }
}

vct_status fill_accum(vct_ctx* ctx, const vct_triangles* t, const vct_light* lights, int n,
                      const vct_shadow_desc* sh, const float* eye, AccumParams& P) {
    if (ctx->params.voxelize_tesselation && t->count > (1LL << 24))
        return fail(VCT_ERR_UNSUPPORTED, "the tessellation voxeliser takes at most 2^24 triangles per call");
    fill_accum_inputs(ctx->cfg, ctx->params, ctx->mvp, t, lights, n, sh, P);
    P.warp = warp_dev(ctx, eye);
    apply_tuning(ctx->tuning, P);
    P.acc = ctx->acc;
    P.occ = ctx->occ;
    P.carry = ctx->params.voxelize_tesselation ? ctx->carry : nullptr;
    P.brick_exact = ctx->params.voxelize_tesselation ? ctx->brick_exact : nullptr;
    P.stats = ctx->stats;
    P.num_sms = ctx->num_sms;
    const long long need = accumulate_scratch_bytes(t->count);
    if (need > ctx->vox_scratch_bytes) {
        if (ctx->vox_scratch) cudaFree(ctx->vox_scratch);
        ctx->vox_scratch = nullptr;
        ctx->vox_scratch_bytes = 0;
        cudaError_t e = cudaMalloc(&ctx->vox_scratch, (size_t)need);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(VCT_ERR_OUT_OF_MEMORY, std::string("voxeliser scratch: ") + cudaGetErrorString(e));
        }
        ctx->vox_scratch_bytes = need;
    }
    accumulate_bind_scratch(P, ctx->vox_scratch);
    return VCT_OK;
}

void fill_norm(vct_ctx* ctx, NormalizeParams& P) {
    P.dim = ctx->dim;
    P.opacity = ctx->params.voxel_set_opacity;
    P.temporal = ctx->params.temporal_filter;
    P.decay = ctx->params.temporal_decay;
    P.acc = ctx->acc;
    P.occ = ctx->occ;
    P.brick_exact = ctx->params.voxelize_tesselation ? ctx->brick_exact : nullptr;
    P.color = ctx->color;
    P.normal = ctx->normal;
    P.radiance = ctx->radiance;
    P.stats = ctx->stats;
    P.num_sms = ctx->num_sms;
}

// voxelIndex(p) of common.glsl:62-64 with warping off: dim * (p - center - min) / (max - min).
f3 voxel_index_host(const vct_config& c, int dim, const float* p) {
    float out[3];
    for (int k = 0; k < 3; ++k) {
        float ext = c.voxel_max[k] - c.voxel_min[k];
        float tc = ((p[k] - c.voxel_center[k]) - c.voxel_min[k]) / ext;
        out[k] = tc * (float)dim;
    }
    return {out[0], out[1], out[2]};
}

void fill_inject(vct_ctx* ctx, const vct_shadow_desc* s, const float* eye, InjectParams& P) {
    std::memset(&P, 0, sizeof P);
    P.warp = warp_dev(ctx, eye);
    for (int k = 0; k < 3; ++k)  // voxelLinearPosition(lightPos)
        (&P.light_tc.x)[k] = ((s->light_pos[k] - ctx->cfg.voxel_center[k]) - ctx->cfg.voxel_min[k]) /
                             (ctx->cfg.voxel_max[k] - ctx->cfg.voxel_min[k]);
    P.light_pos = to_f3(s->light_pos);
    P.dim = ctx->dim;
    P.shadowmap = s->shadowmap_dev;
    P.sw = s->width;
    P.sh = s->height;
    // The dispatch covers ceil(size/16)*16 invocations and the bounds test in
    // injectRadiance.comp:44 is `>`, so index == size also runs when size is
    // not a multiple of 16.
    P.nx = std::min(((s->width + 15) / 16) * 16, s->width + 1);
    P.ny = std::min(((s->height + 15) / 16) * 16, s->height + 1);
    std::memcpy(P.ls_inverse, s->ls_inverse, sizeof P.ls_inverse);
    P.vmin = to_f3(ctx->cfg.voxel_min);
    P.vmax = to_f3(ctx->cfg.voxel_max);
    P.vcenter = to_f3(ctx->cfg.voxel_center);
    P.light_vox = voxel_index_host(ctx->cfg, ctx->dim, s->light_pos);
    P.light_int = to_f3(s->light_int);
    P.lighting = ctx->params.radiance_lighting;
    P.dilate = ctx->params.radiance_dilate;
    P.temporal = ctx->params.temporal_filter;
    P.decay = ctx->params.temporal_decay;
    P.color = ctx->color;
    P.normal = ctx->normal;
    P.radiance = ctx->radiance;
    P.lit = ctx->lit;
}

MipLevels mip_levels(vct_ctx* ctx, uint2* chain, int levels) {
    MipLevels M;
    std::memset(&M, 0, sizeof M);
    M.dim = ctx->dim;
    M.levels = levels;
    for (int l = 0; l < levels; ++l) M.level[l] = level_ptr(chain, ctx, l);
    return M;
}

// The samplers' copies of the radiance chain: the texture array (texture-unit
// filtering) and the bordered fp32 chain (software filtering).
bool filter_uses_texture(int filter) { return filter != VCT_FILTER_SOFTWARE; }
bool filter_uses_bordered(int filter) { return filter == VCT_FILTER_SOFTWARE || filter == VCT_FILTER_HYBRID; }

vct_status ensure_texture(vct_ctx* ctx) {
    if (ctx->tex_array) return VCT_OK;
    cudaChannelFormatDesc desc = cudaCreateChannelDescHalf4();
    cudaExtent ext = make_cudaExtent(ctx->dim, ctx->dim, ctx->dim);
    VCT_CUDA(cudaMallocMipmappedArray(&ctx->tex_array, &desc, ext, ctx->levels, cudaArraySurfaceLoadStore));
    for (int l = 0; l < ctx->levels; ++l) {
        cudaArray_t arr;
        VCT_CUDA(cudaGetMipmappedArrayLevel(&arr, ctx->tex_array, l));
        cudaResourceDesc sres;
        std::memset(&sres, 0, sizeof sres);
        sres.resType = cudaResourceTypeArray;
        sres.res.array.array = arr;
        VCT_CUDA(cudaCreateSurfaceObject(&ctx->surf[l], &sres));
    }
    cudaResourceDesc res;
    std::memset(&res, 0, sizeof res);
    res.resType = cudaResourceTypeMipmappedArray;
    res.res.mipmap.mipmap = ctx->tex_array;
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof td);
    for (int k = 0; k < 3; ++k) td.addressMode[k] = cudaAddressModeBorder;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 1;
    td.mipmapFilterMode = cudaFilterModeLinear;
    td.minMipmapLevelClamp = 0.0f;
    td.maxMipmapLevelClamp = (float)(ctx->levels - 1);
    td.maxAnisotropy = 1;
    VCT_CUDA(cudaCreateTextureObject(&ctx->tex, &res, &td, nullptr));
    return VCT_OK;
}

// A fused frame whose sampler reads both the texture array and the bordered
// chain writes the linear chain only from level `linear_stale` on: the levels
// below are in the texture array, texel for texel the same binary16 values.
// Entry points that read the linear chain copy them back first.
vct_status sync_linear(vct_ctx* ctx, cudaStream_t s) {
    if (ctx->linear_stale <= 0) return VCT_OK;
    for (int l = 0; l < ctx->linear_stale; ++l) {
        cudaArray_t arr;
        VCT_CUDA(cudaGetMipmappedArrayLevel(&arr, ctx->tex_array, l));
        int S = ctx->dim >> l;
        cudaMemcpy3DParms p;
        std::memset(&p, 0, sizeof p);
        p.srcArray = arr;
        p.dstPtr = make_cudaPitchedPtr(level_ptr(ctx->radiance, ctx, l), (size_t)S * 8, S, S);
        p.extent = make_cudaExtent(S, S, S);
        p.kind = cudaMemcpyDeviceToDevice;
        VCT_CUDA(cudaMemcpy3DAsync(&p, s));
    }
    ctx->linear_stale = 0;
    return VCT_OK;
}

// Copies the linear radiance chain into the mip-mapped array of the
// texture-unit sampler.
vct_status refresh_texture(vct_ctx* ctx, cudaStream_t s) {
    vct_status st = ensure_texture(ctx);
    if (st != VCT_OK) return st;
    if ((st = sync_linear(ctx, s)) != VCT_OK) return st;
    for (int l = 0; l < ctx->levels; ++l) {
        cudaArray_t arr;
        VCT_CUDA(cudaGetMipmappedArrayLevel(&arr, ctx->tex_array, l));
        int S = ctx->dim >> l;
        cudaMemcpy3DParms p;
        std::memset(&p, 0, sizeof p);
        p.srcPtr = make_cudaPitchedPtr(level_ptr(ctx->radiance, ctx, l), (size_t)S * 8, S, S);
        p.dstArray = arr;
        p.extent = make_cudaExtent(S, S, S);
        p.kind = cudaMemcpyDeviceToDevice;
        VCT_CUDA(cudaMemcpy3DAsync(&p, s));
    }
    ctx->tex_ready = true;
    return VCT_OK;
}

vct_status fill_trace(vct_ctx* ctx, const vct_gbuffer* g, const float eye[3], const vct_trace_out* out,
                      TraceParams& P) {
    std::memset(&P, 0, sizeof P);
    P.gpos = reinterpret_cast<const float4*>(g->position_dev);
    P.gnrm = reinterpret_cast<const float4*>(g->normal_dev);
    P.galb = reinterpret_cast<const float4*>(g->albedo_dev);
    P.width = g->width;
    P.height = g->height;
    P.irradiance = reinterpret_cast<float4*>(out->irradiance_dev);
    P.specular = reinterpret_cast<float4*>(out->specular_dev);
    P.color = reinterpret_cast<float4*>(out->color_dev);
    P.samples = out->sample_count_dev;
    P.pchain = ctx->pchain;
    P.dim = ctx->dim;
    P.levels = ctx->levels;
    P.vmin = to_f3(ctx->cfg.voxel_min);
    P.vmax = to_f3(ctx->cfg.voxel_max);
    P.vcenter = to_f3(ctx->cfg.voxel_center);
    P.eye = to_f3(eye);
    const vct_params& pr = ctx->params;
    P.diffuse = pr.diffuse_cone;
    P.specular_cone = pr.specular_cone;
    P.enable_indirect = pr.enable_indirect;
    P.enable_reflections = pr.enable_reflections;
    P.draw_occlusion = pr.draw_occlusion;
    P.enable_postprocess = pr.enable_postprocess;
    P.ambient_scale = pr.ambient_scale;
    P.reflect_scale = pr.reflect_scale;
    P.max_distance = pr.max_distance > 0.0f ? pr.max_distance : std::sqrt(3.0f);
    P.ref_tbn_quirk = pr.ref_tbn_quirk;
    P.filter = pr.trace_filter;
    P.tex = ctx->tex;
    P.warp = warp_dev(ctx, eye);
    apply_tuning(ctx->tuning, P);
    for (auto p : {(const void*)g->position_dev, (const void*)g->normal_dev, (const void*)g->albedo_dev,
                   (const void*)out->irradiance_dev, (const void*)out->specular_dev, (const void*)out->color_dev})
        if (reinterpret_cast<uintptr_t>(p) % 16 != 0) return fail(VCT_ERR_INVALID_ARGUMENT, "float4 planes must be 16-byte aligned");
    return VCT_OK;
}

vct_status ensure_padded_chain(vct_ctx* c, cudaStream_t st) {
    if (c->pad_ready) return VCT_OK;
    vct_status s = sync_linear(c, st);
    if (s != VCT_OK) return s;
    launch_pad_copy(c->radiance, c->pchain, c->dim, c->levels, st);
    VCT_CHECK_LAUNCH("bordered chain copy");
    c->pad_ready = true;
    return VCT_OK;
}

}  // namespace host
}  // namespace vct

// ==================================================================== API
extern "C" {

int32_t vct_abi_version(void) { return VCT_ABI_VERSION; }

const char* vct_status_string(vct_status s) {
    switch (s) {
        case VCT_OK: return "ok";
        case VCT_ERR_INVALID_ARGUMENT: return "invalid argument";
        case VCT_ERR_OUT_OF_MEMORY: return "out of device memory";
        case VCT_ERR_CUDA: return "CUDA error";
        case VCT_ERR_STATE: return "invalid call order";
        case VCT_ERR_TIMEOUT: return "device wait timed out";
        case VCT_ERR_UNSUPPORTED: return "unsupported";
        case VCT_ERR_OVERFLOW: return "accumulator overflow";
    }
    return "unknown status";
}

const char* vct_last_error(void) { return g_err.c_str(); }

void vct_struct_sizes(int64_t* light, int64_t* config, int64_t* params, int64_t* triangles, int64_t* gbuffer,
                      int64_t* trace_out, int64_t* shadow_desc, int64_t* stats) {
    if (light) *light = sizeof(vct_light);
    if (config) *config = sizeof(vct_config);
    if (params) *params = sizeof(vct_params);
    if (triangles) *triangles = sizeof(vct_triangles);
    if (gbuffer) *gbuffer = sizeof(vct_gbuffer);
    if (trace_out) *trace_out = sizeof(vct_trace_out);
    if (shadow_desc) *shadow_desc = sizeof(vct_shadow_desc);
    if (stats) *stats = sizeof(vct_stats);
}

int64_t vct_struct_layout(const char* name) {
    if (!name) return -1;
    struct Entry {
        const char* name;
        size_t value;
    };
#define VCT_SZ(T) {#T, sizeof(T)}
#define VCT_OFF(T, f) {#T "." #f, offsetof(T, f)}
    static const Entry table[] = {
        VCT_SZ(vct_light),  VCT_SZ(vct_config),         VCT_SZ(vct_cone_settings),  VCT_SZ(vct_params),
        VCT_SZ(vct_triangles), VCT_SZ(vct_gbuffer),     VCT_SZ(vct_trace_out),      VCT_SZ(vct_shadow_desc),
        VCT_SZ(vct_stats),  VCT_SZ(vct_timers),         VCT_SZ(vct_tuning),         VCT_SZ(vct_scene_desc),
        VCT_OFF(vct_scene_desc, lights), VCT_OFF(vct_scene_desc, n_lights), VCT_OFF(vct_scene_desc, shadow),
        VCT_OFF(vct_scene_desc, eye),    VCT_OFF(vct_scene_desc, gbuffer),  VCT_OFF(vct_scene_desc, out),
        VCT_OFF(vct_params, trace_filter), VCT_OFF(vct_params, pv), VCT_OFF(vct_tuning, trace_warp_w),
        VCT_SZ(vct_adam), VCT_SZ(vct_learned_stats), VCT_OFF(vct_learned_stats, max_tile_error),
    };
#undef VCT_SZ
#undef VCT_OFF
    for (const Entry& e : table)
        if (std::strcmp(e.name, name) == 0) return (int64_t)e.value;
    return -1;
}

void vct_default_params(vct_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    const float deg = 3.14159265358979323846f / 180.0f;
    p->voxelize_lighting = 1;
    p->axis_override = -1;
    p->voxel_set_opacity = 0.5f;
    p->temporal_filter = 0;
    p->temporal_decay = 0.8f;
    p->radiance_lighting = 0;
    p->radiance_dilate = 0;
    p->diffuse_cone = {16, 60.0f * deg, 1.0f, 1.0f, 0.5f};
    p->specular_cone = {32, 30.0f * deg, 1.7f, 0.5f, 0.1f};
    p->enable_indirect = 1;
    p->enable_reflections = 1;
    p->draw_occlusion = 1;
    p->enable_postprocess = 1;
    p->ambient_scale = 1.0f;
    p->reflect_scale = 1.0f;
    p->max_distance = 0.0f;
    p->ref_tbn_quirk = 0;
    p->trace_filter = VCT_FILTER_SOFTWARE;
    p->warp_mode = VCT_WARP_NONE;
    p->warp_high_resolution = 2.0f;  // src/Application.h:81-82
    p->warp_low_resolution = 0.5f;
    p->cooktorrance = 1;  // src/Application.h:60-68
    p->enable_diffuse = 1;
    p->enable_specular = 1;
    p->roughness = 0.5f;  // phong.frag:310 without a roughness map
    p->metallic = 0.0f;
    p->shininess = 32.0f;  // src/Graphics/Mesh.h:29
    p->voxelize_tesselation = 0;  // the reference's default is 1 (Application.h:100); see vct.h
    p->max_tess_level = (float)VCT_MAX_TESS_LEVEL;
    for (int i = 0; i < 16; ++i) p->pv[i] = (i % 5 == 0) ? 1.0f : 0.0f;
}

vct_status vct_voxel_mvp(const vct_config* cfg, float mvp_xyz[48]) {
    vct_status s = validate_config(cfg);
    if (s != VCT_OK) return s;
    if (!mvp_xyz) return fail(VCT_ERR_INVALID_ARGUMENT, "output is NULL");
    voxel_mvp(*cfg, mvp_xyz);
    return VCT_OK;
}

vct_status vct_create(const vct_config* cfg, vct_ctx** out) {
    if (!out) return fail(VCT_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    vct_status s = validate_config(cfg);
    if (s != VCT_OK) return s;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(VCT_ERR_CUDA, "no CUDA device available");
    }
    if (cfg->device < 0 || cfg->device >= ndev) return fail(VCT_ERR_INVALID_ARGUMENT, "device ordinal out of range");
    DeviceScope ds(cfg->device);
    VCT_CUDA(ds.err);
    vct_ctx* c = new (std::nothrow) vct_ctx;
    if (!c) return fail(VCT_ERR_OUT_OF_MEMORY, "host allocation failed");
    c->cfg = *cfg;
    c->dim = cfg->voxel_dim;
    int maxl = ilog2(c->dim) + 1;
    c->levels = cfg->voxel_levels == 0 ? maxl : std::min(std::max(cfg->voxel_levels, 1), maxl);
    default_tuning(c->tuning);
    c->color_levels = (cfg->flags & VCT_CONFIG_COLOR_MIPS) ? c->levels : 1;
    c->device = cfg->device;
    c->nv = (long long)c->dim * c->dim * c->dim;
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
    vct_default_params(&c->params);
    voxel_mvp(*cfg, c->mvp);
    long long off = 0;
    for (int l = 0; l < c->levels; ++l) {
        c->level_off[l] = off;
        long long S = c->dim >> l;
        off += S * S * S;
    }
    long long chain_vox = off;
    long long color_vox = c->color_levels > 1 ? chain_vox : c->nv;
    struct Alloc {
        void** p;
        size_t bytes;
    } allocs[] = {
        {(void**)&c->acc, (size_t)c->nv * 4 * kAccWords},
        {(void**)&c->occ, (size_t)((c->nv + 31) / 32) * 4},
        {(void**)&c->lit, (size_t)((c->nv + 31) / 32) * 4},
        {(void**)&c->color, (size_t)color_vox * 8},
        {(void**)&c->normal, (size_t)c->nv * 8},
        {(void**)&c->radiance, (size_t)chain_vox * 8},
        {(void**)&c->stats, sizeof(StatsDev)},
        {(void**)&c->pchain, (size_t)padded_level_offset(c->dim, c->levels) * 16},
        {(void**)&c->occ32, (size_t)(VCT_WARP_DIM * VCT_WARP_DIM * VCT_WARP_DIM / 32) * 4},
        {(void**)&c->warpmap, (size_t)VCT_WARP_DIM * VCT_WARP_DIM * VCT_WARP_DIM * 8},
        {(void**)&c->warpmap_f, (size_t)(VCT_WARP_DIM + 2) * (VCT_WARP_DIM + 2) * (VCT_WARP_DIM + 2) * 16},
        {(void**)&c->carry, (size_t)kCarryBytes},
        {(void**)&c->brick_exact, (size_t)(c->nv / 4096 + 1) * 4},
    };
    for (auto& a : allocs) {
        cudaError_t e = cudaMalloc(a.p, a.bytes);
        if (e == cudaSuccess) e = cudaMemset(*a.p, 0, a.bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            std::string msg = std::string("device allocation failed: ") + cudaGetErrorString(e);
            vct_destroy(c);
            return fail(e == cudaErrorMemoryAllocation ? VCT_ERR_OUT_OF_MEMORY : VCT_ERR_CUDA, msg);
        }
    }
    cudaError_t e = cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->join, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        cudaGetLastError();
        std::string msg = std::string("stream/event creation failed: ") + cudaGetErrorString(e);
        vct_destroy(c);
        return fail(VCT_ERR_CUDA, msg);
    }
    *out = c;
    return VCT_OK;
}

vct_status vct_destroy(vct_ctx* c) {
    if (!c) return VCT_OK;
    DeviceScope ds(c->device);
    for (auto e : c->ev)
        if (e) cudaEventDestroy(e);
    if (c->fork) cudaEventDestroy(c->fork);
    if (c->join) cudaEventDestroy(c->join);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->tex) cudaDestroyTextureObject(c->tex);
    if (c->tex_array) cudaFreeMipmappedArray(c->tex_array);
    for (auto sf : c->surf)
        if (sf) cudaDestroySurfaceObject(sf);
    void* ptrs[] = {c->acc,    c->occ,   c->lit,         c->color,  c->normal,  c->radiance, c->stats,
                    c->vox_scratch, c->pchain, c->learned, c->occ32, c->warpmap, c->warpmap_f, c->carry,
                    c->brick_exact};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete c;
    return VCT_OK;
}

vct_status vct_set_params(vct_ctx* c, const vct_params* p) {
    if (!c) return fail(VCT_ERR_INVALID_ARGUMENT, "ctx is NULL");
    vct_status s = validate_params(p);
    if (s != VCT_OK) return s;
    c->params = *p;
    return VCT_OK;
}

vct_status vct_get_params(const vct_ctx* c, vct_params* out) {
    if (!c || !out) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = c->params;
    return VCT_OK;
}

vct_status vct_get_config(const vct_ctx* c, vct_config* out) {
    if (!c || !out) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = c->cfg;
    out->voxel_levels = c->levels;
    return VCT_OK;
}

vct_status vct_volume_level(const vct_ctx* c, int32_t volume, int32_t level, const uint16_t** data, int32_t* dim) {
    if (!c || !data) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    uint2* base = nullptr;
    int nl = 0;
    switch (volume) {
        case VCT_VOLUME_COLOR: base = c->color; nl = c->color_levels; break;
        case VCT_VOLUME_NORMAL: base = c->normal; nl = 1; break;
        case VCT_VOLUME_RADIANCE: base = c->radiance; nl = c->levels; break;
        default: return fail(VCT_ERR_INVALID_ARGUMENT, "unknown volume");
    }
    if (level < 0 || level >= nl) return fail(VCT_ERR_INVALID_ARGUMENT, "level out of range for this volume");
    if (volume == VCT_VOLUME_RADIANCE && level < c->linear_stale) {
        // The level is in the texture array only (a fused frame's hybrid
        // sampler): copied back once, after all work queued on the device.
        vct_ctx* m = const_cast<vct_ctx*>(c);
        DeviceScope ds(m->device);
        VCT_CUDA(ds.err);
        VCT_CUDA(cudaDeviceSynchronize());
        vct_status s = sync_linear(m, nullptr);
        if (s != VCT_OK) return s;
        VCT_CUDA(cudaStreamSynchronize(nullptr));
    }
    *data = reinterpret_cast<const uint16_t*>(base + c->level_off[level]);
    if (dim) *dim = c->dim >> level;
    return VCT_OK;
}

int64_t vct_record_slot(int64_t v, int32_t dim) { return record_slot(v, dim); }

vct_status vct_accumulators(const vct_ctx* c, const uint32_t** records, const uint32_t** occupancy) {
    if (!c) return fail(VCT_ERR_INVALID_ARGUMENT, "ctx is NULL");
    if (records) *records = c->acc;
    if (occupancy) *occupancy = c->occ;
    return VCT_OK;
}

vct_status vct_voxelize_accumulate(vct_ctx* c, const vct_triangles* tris, const vct_light* lights, int32_t n,
                                   const vct_shadow_desc* shadow, const float eye[3], void* stream) {
    if (!c) return fail(VCT_ERR_INVALID_ARGUMENT, "ctx is NULL");
    if (!eye && c->params.warp_mode == VCT_WARP_ANALYTIC)
        return fail(VCT_ERR_INVALID_ARGUMENT, "the analytic warp needs the eye position");
    vct_status s = validate_tris(tris);
    if (s != VCT_OK) return s;
    bool need_shadow = false;
    if ((s = validate_lights(lights, n, &need_shadow)) != VCT_OK) return s;
    need_shadow = need_shadow && c->params.voxelize_lighting;
    if ((s = validate_shadow(shadow, need_shadow)) != VCT_OK) return s;
    DeviceScope ds(c->device);
    VCT_CUDA(ds.err);
    cudaStream_t st = as_stream(stream);
    if (c->stats_reset_pending) {
        VCT_CUDA(cudaMemsetAsync(c->stats, 0, sizeof(StatsDev), st));
        c->stats_reset_pending = false;
    }
    AccumParams P;
    if ((s = fill_accum(c, tris, lights, n, need_shadow ? shadow : nullptr, eye, P)) != VCT_OK) return s;
    if (c->params.warp_mode == VCT_WARP_TEXTURE && (s = build_warpmap(c, P, st)) != VCT_OK) return s;
    launch_voxelizer(c, P, st);
    VCT_CHECK_LAUNCH("voxelize accumulate");
    c->radiance_ready = false;
    c->mips_ready = false;
    c->pad_ready = false;
    c->tex_ready = false;
    return VCT_OK;
}

vct_status vct_normalize(vct_ctx* c, void* stream) {
    if (!c) return fail(VCT_ERR_INVALID_ARGUMENT, "ctx is NULL");
    DeviceScope ds(c->device);
    VCT_CUDA(ds.err);
    cudaStream_t st = as_stream(stream);
    vct_status s = sync_linear(c, st);  // the temporal filter reads last frame's level 0
    if (s != VCT_OK) return s;
    if (c->stats_reset_pending) VCT_CUDA(cudaMemsetAsync(c->stats, 0, sizeof(StatsDev), st));
    NormalizeParams P;
    fill_norm(c, P);
    launch_normalize(P, st);
    VCT_CHECK_LAUNCH("normalize");
    // Records of occupied voxels were zeroed by the kernel; the mask is
    // cleared here so that the next accumulate starts from an empty grid.
    VCT_CUDA(cudaMemsetAsync(c->occ, 0, (size_t)((c->nv + 31) / 32) * 4, st));
    c->stats_reset_pending = true;
    c->radiance_ready = true;
    c->mips_ready = false;
    c->pad_ready = false;
    c->tex_ready = false;
    return VCT_OK;
}

vct_status vct_clear_accumulators(vct_ctx* c, void* stream) {
    if (!c) return fail(VCT_ERR_INVALID_ARGUMENT, "ctx is NULL");
    DeviceScope ds(c->device);
    VCT_CUDA(ds.err);
    cudaStream_t st = as_stream(stream);
    VCT_CUDA(cudaMemsetAsync(c->acc, 0, (size_t)c->nv * 4 * kAccWords, st));
    VCT_CUDA(cudaMemsetAsync(c->occ, 0, (size_t)((c->nv + 31) / 32) * 4, st));
    c->stats_reset_pending = true;
    return VCT_OK;
}

vct_status vct_voxelize(vct_ctx* c, const vct_triangles* tris, const vct_light* lights, int32_t n,
                        const vct_shadow_desc* shadow, const float eye[3], void* stream) {
    vct_status s = vct_voxelize_accumulate(c, tris, lights, n, shadow, eye, stream);
    if (s != VCT_OK) return s;
    return vct_normalize(c, stream);
}

vct_status vct_inject(vct_ctx* c, const vct_shadow_desc* shadow, const float eye[3], void* stream) {
    if (!c) return fail(VCT_ERR_INVALID_ARGUMENT, "ctx is NULL");
    if (!eye && c->params.warp_mode == VCT_WARP_ANALYTIC)
        return fail(VCT_ERR_INVALID_ARGUMENT, "the analytic warp needs the eye position");
    vct_status s = validate_shadow(shadow, true);
    if (s != VCT_OK) return s;
    DeviceScope ds(c->device);
    VCT_CUDA(ds.err);
    InjectParams P;
    fill_inject(c, shadow, eye, P);
    cudaStream_t st = as_stream(stream);
    if ((s = sync_linear(c, st)) != VCT_OK) return s;
    if (P.temporal && P.lighting && !P.dilate) {
        // the relit stores read the seeded radiance: one store per marked voxel
        VCT_CUDA(cudaMemsetAsync(c->lit, 0, (size_t)((c->nv + 31) / 32) * 4, st));
        launch_inject_mark(P, st);
        launch_inject_apply(P, st);
    } else {
        launch_inject(P, st);
    }
    VCT_CHECK_LAUNCH("inject");
    c->mips_ready = false;
    c->pad_ready = false;
    c->tex_ready = false;
    return VCT_OK;
}

vct_status vct_build_mips(vct_ctx* c, int32_t volume, void* stream) {
    if (!c) return fail(VCT_ERR_INVALID_ARGUMENT, "ctx is NULL");
    DeviceScope ds(c->device);
    VCT_CUDA(ds.err);
    cudaStream_t st = as_stream(stream);
    if (volume == VCT_VOLUME_RADIANCE) {
        vct_status s = sync_linear(c, st);
        if (s != VCT_OK) return s;
        launch_mips(mip_levels(c, c->radiance, c->levels), 0, st);
        VCT_CHECK_LAUNCH("build mips");
        if (filter_uses_texture(c->params.trace_filter)) {
            vct_status s = refresh_texture(c, st);
            if (s != VCT_OK) return s;
        }
        if (filter_uses_bordered(c->params.trace_filter)) {
            launch_pad_copy(c->radiance, c->pchain, c->dim, c->levels, st);
            VCT_CHECK_LAUNCH("bordered chain copy");
            c->pad_ready = true;
        }
        c->mips_ready = true;
        return VCT_OK;
    }
    if (volume == VCT_VOLUME_COLOR) {
        if (c->color_levels < 2) return fail(VCT_ERR_UNSUPPORTED, "context created without VCT_CONFIG_COLOR_MIPS");
        launch_mips(mip_levels(c, c->color, c->color_levels), 0, st);
        VCT_CHECK_LAUNCH("build colour mips");
        return VCT_OK;
    }
    return fail(VCT_ERR_INVALID_ARGUMENT, "volume must be VCT_VOLUME_RADIANCE or VCT_VOLUME_COLOR");
}

vct_status vct_trace(vct_ctx* c, const vct_gbuffer* g, const float eye[3], const vct_trace_out* out, void* stream) {
    if (!c || !eye || !out) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    vct_status s = validate_gbuffer(g);
    if (s != VCT_OK) return s;
    DeviceScope ds(c->device);
    VCT_CUDA(ds.err);
    cudaStream_t st = as_stream(stream);
    if (filter_uses_texture(c->params.trace_filter) && !c->tex_ready) {
        if ((s = refresh_texture(c, st)) != VCT_OK) return s;
    }
    if (filter_uses_bordered(c->params.trace_filter) && (s = ensure_padded_chain(c, st)) != VCT_OK) return s;
    TraceParams P;
    if ((s = fill_trace(c, g, eye, out, P)) != VCT_OK) return s;
    launch_trace(P, st);
    VCT_CHECK_LAUNCH("trace");
    if (c->timers_on && c->volume_timed) {  // render stage of a timed vct_frame_volume
        VCT_CUDA(cudaEventRecord(c->ev[4], st));
        c->timers_recorded = true;
    }
    return VCT_OK;
}

vct_status vct_trace_views(vct_ctx* c, int32_t n, const vct_gbuffer* gbuffers, const float* eyes,
                           const vct_trace_out* outs, void* stream) {
    if (!c || (n > 0 && (!gbuffers || !eyes || !outs))) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n < 0) return fail(VCT_ERR_INVALID_ARGUMENT, "n must be >= 0");
    vct_status s = VCT_OK;
    for (int i = 0; i < n; ++i)
        if ((s = validate_gbuffer(&gbuffers[i])) != VCT_OK) return s;
    DeviceScope ds(c->device);
    VCT_CUDA(ds.err);
    cudaStream_t st = as_stream(stream);
    if (n == 0) return VCT_OK;
    if (filter_uses_texture(c->params.trace_filter) && !c->tex_ready) {
        if ((s = refresh_texture(c, st)) != VCT_OK) return s;
    }
    if (filter_uses_bordered(c->params.trace_filter) && (s = ensure_padded_chain(c, st)) != VCT_OK) return s;
    // kMaxViews viewpoints per launch, their parameters in kernel-parameter space
    for (int first = 0; first < n; first += kMaxViews) {
        ViewSet V;
        std::memset(&V, 0, sizeof V);
        V.n = std::min(kMaxViews, n - first);
        for (int k = 0; k < V.n; ++k) {
            TraceParams& P = V.p[k];
            if ((s = fill_trace(c, &gbuffers[first + k], eyes + 3 * (first + k), &outs[first + k], P)) != VCT_OK)
                return s;
            V.off[k + 1] = V.off[k] + trace_tiles(P.width, P.height, P.tile_w_log2, P.tile_h_log2);
        }
        launch_trace_views(V, c->params.trace_filter, st);
        VCT_CHECK_LAUNCH("trace views");
    }
    return VCT_OK;
}

namespace {

// The volume pass of vct_frame: voxelise, inject (marked), normalise +
// inject resolve + mips.  Inputs are validated by the callers.
vct_status frame_volume(vct_ctx* c, const vct_triangles* tris, const vct_light* lights, int32_t n,
                        const vct_shadow_desc* shadow, const float eye[3], cudaStream_t st) {
    vct_status s = VCT_OK;
    const bool timed = c->timers_on;
    c->volume_timed = false;
    if (timed) VCT_CUDA(cudaEventRecord(c->ev[0], st));
    VCT_CUDA(cudaMemsetAsync(c->stats, 0, sizeof(StatsDev), st));
    AccumParams A;
    if ((s = fill_accum(c, tris, lights, n, shadow, eye, A)) != VCT_OK) return s;
    if (c->params.warp_mode == VCT_WARP_TEXTURE && (s = build_warpmap(c, A, st)) != VCT_OK) return s;
    // The shadow-map half of injection (the lit mask) needs neither the
    // voxeliser's output nor its SMs' full attention: it runs on the side
    // stream, forked after everything the caller enqueued so far (the last
    // frame's resolve read the mask) and joined before the resolve.
    VCT_CUDA(cudaEventRecord(c->fork, st));
    VCT_CUDA(cudaStreamWaitEvent(c->side, c->fork, 0));
    VCT_CUDA(cudaMemsetAsync(c->lit, 0, (size_t)((c->nv + 31) / 32) * 4, c->side));
    InjectParams I;
    fill_inject(c, shadow, eye, I);
    launch_inject_mark(I, c->side);
    VCT_CHECK_LAUNCH("frame: inject mark");
    VCT_CUDA(cudaEventRecord(c->join, c->side));
    launch_voxelizer(c, A, st);
    VCT_CHECK_LAUNCH("frame: accumulate");
    if (timed) VCT_CUDA(cudaEventRecord(c->ev[1], st));
    VCT_CUDA(cudaStreamWaitEvent(st, c->join, 0));
    if (timed) VCT_CUDA(cudaEventRecord(c->ev[2], st));
    const bool hw = filter_uses_texture(c->params.trace_filter);
    const bool pad = filter_uses_bordered(c->params.trace_filter);
    if (hw && (s = ensure_texture(c)) != VCT_OK) return s;
    // The temporal filter reads last frame's level 0 from the linear chain.
    if (c->params.temporal_filter && (s = sync_linear(c, st)) != VCT_OK) return s;
    ResolveParams R;
    std::memset(&R, 0, sizeof R);
    fill_norm(c, R.norm);
    R.fused = 1;
    R.lighting = c->params.radiance_lighting;
    R.dilate = c->params.radiance_dilate;
    R.light_vox = I.light_vox;
    R.light_int = I.light_int;
    R.warp = I.warp;
    R.light_tc = I.light_tc;
    R.light_pos = I.light_pos;
    R.lit = c->lit;
    R.mip_levels = std::min(4, c->levels - 1);
    // The sampler's own copy of the chain is written by the same kernels:
    // texture-unit surfaces, or the bordered chain of the software sampler.
    // When the sampler reads both (hybrid) and no temporal filter reads last
    // frame's radiance, the linear copy of the levels below the resolve's last
    // one is not written: they are in the texture array, texel for texel, and
    // sync_linear copies them back for the entry points that read them.  The
    // last level stays, as the mip tail's source.
    const int stale = (hw && pad && !c->params.temporal_filter) ? R.mip_levels : 0;
    for (int l = 0; l <= R.mip_levels; ++l) {
        R.radiance_levels[l] = l < stale ? nullptr : level_ptr(c->radiance, c, l);
        R.surf[l] = hw ? c->surf[l] : 0;
        R.pad_levels[l] = pad ? c->pchain + padded_level_offset(c->dim, l) : nullptr;
    }
    launch_resolve(R, st);
    VCT_CHECK_LAUNCH("frame: resolve");
    VCT_CUDA(cudaMemsetAsync(c->occ, 0, (size_t)((c->nv + 31) / 32) * 4, st));
    if (c->levels > 5) {
        MipLevels M = mip_levels(c, c->radiance, c->levels);
        for (int l = 0; l < c->levels; ++l) {
            M.surf[l] = hw ? c->surf[l] : 0;
            M.pad[l] = pad ? c->pchain + padded_level_offset(c->dim, l) : nullptr;
        }
        launch_mips(M, 4, st);
        VCT_CHECK_LAUNCH("frame: coarse mips");
    }
    c->tex_ready = hw;
    c->pad_ready = pad;
    c->linear_stale = stale;
    c->stats_reset_pending = true;
    c->radiance_ready = true;
    c->mips_ready = true;
    if (timed) VCT_CUDA(cudaEventRecord(c->ev[3], st));
    c->volume_timed = timed;
    return VCT_OK;
}

vct_status validate_volume_inputs(const vct_ctx* c, const vct_triangles* tris, const vct_light* lights, int32_t n,
                                  const vct_shadow_desc* shadow, const float* eye) {
    if (!c || !eye) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    vct_status s = validate_tris(tris);
    if (s != VCT_OK) return s;
    bool need_shadow = false;
    if ((s = validate_lights(lights, n, &need_shadow)) != VCT_OK) return s;
    return validate_shadow(shadow, true);
}

}  // namespace

vct_status vct_frame_volume(vct_ctx* c, const vct_triangles* tris, const vct_light* lights, int32_t n,
                            const vct_shadow_desc* shadow, const float eye[3], void* stream) {
    vct_status s = validate_volume_inputs(c, tris, lights, n, shadow, eye);
    if (s != VCT_OK) return s;
    DeviceScope ds(c->device);
    VCT_CUDA(ds.err);
    return frame_volume(c, tris, lights, n, shadow, eye, as_stream(stream));
}

vct_status vct_frame(vct_ctx* c, const vct_triangles* tris, const vct_light* lights, int32_t n,
                     const vct_shadow_desc* shadow, const float eye[3], const vct_gbuffer* g,
                     const vct_trace_out* out, void* stream) {
    vct_status s = validate_volume_inputs(c, tris, lights, n, shadow, eye);
    if (s != VCT_OK) return s;
    if (!out) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    if ((s = validate_gbuffer(g)) != VCT_OK) return s;
    DeviceScope ds(c->device);
    VCT_CUDA(ds.err);
    cudaStream_t st = as_stream(stream);
    if ((s = frame_volume(c, tris, lights, n, shadow, eye, st)) != VCT_OK) return s;
    TraceParams T;
    if ((s = fill_trace(c, g, eye, out, T)) != VCT_OK) return s;
    launch_trace(T, st);
    VCT_CHECK_LAUNCH("frame: trace");
    if (c->volume_timed) {
        VCT_CUDA(cudaEventRecord(c->ev[4], st));
        c->timers_recorded = true;
    }
    return VCT_OK;
}

vct_status vct_sampler_rate(vct_ctx* c, int32_t filter, int64_t samples, double* rate, void* stream) {
    if (!c || !rate) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (filter < VCT_FILTER_SOFTWARE || filter > VCT_FILTER_HYBRID)
        return fail(VCT_ERR_INVALID_ARGUMENT, "filter must be one of VCT_FILTER_*");
    if (samples < 1 || samples > (1LL << 40)) return fail(VCT_ERR_INVALID_ARGUMENT, "samples out of range");
    if (!c->mips_ready) return fail(VCT_ERR_STATE, "no radiance chain: run vct_frame or vct_build_mips first");
    DeviceScope ds(c->device);
    VCT_CUDA(ds.err);
    cudaStream_t st = as_stream(stream);
    vct_status s = VCT_OK;
    if (filter_uses_texture(filter) && !c->tex_ready && (s = refresh_texture(c, st)) != VCT_OK) return s;
    if (filter_uses_bordered(filter) && (s = ensure_padded_chain(c, st)) != VCT_OK) return s;
    vct_gbuffer g;
    std::memset(&g, 0, sizeof g);
    g.width = g.height = 1;
    vct_trace_out o;
    std::memset(&o, 0, sizeof o);
    TraceParams P;
    const float eye[3] = {0.f, 0.f, 0.f};
    if ((s = fill_trace(c, &g, eye, &o, P)) != VCT_OK) return s;
    P.filter = filter;
    const int blocks = c->num_sms * 4;
    const long long threads = (long long)blocks * 256;
    const int iters = (int)std::max<long long>(1, std::min<long long>(1 << 20, samples / threads));
    float* sink = nullptr;
    VCT_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&sink), (size_t)threads * sizeof(float), st));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t err = cudaEventCreate(&e0);
    if (err == cudaSuccess) err = cudaEventCreate(&e1);
    if (err == cudaSuccess) {
        launch_sampler_rate(P, filter, blocks, std::max(1, iters / 8), sink, st);  // warm-up
        err = cudaEventRecord(e0, st);
    }
    if (err == cudaSuccess) {
        launch_sampler_rate(P, filter, blocks, iters, sink, st);
        err = cudaEventRecord(e1, st);
    }
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFreeAsync(sink, st);
    if (err != cudaSuccess) return fail(VCT_ERR_CUDA, std::string("sampler rate: ") + cudaGetErrorString(err));
    *rate = ms > 0.0f ? (double)threads * (double)iters / (ms * 1e-3) : 0.0;
    return VCT_OK;
}

vct_status vct_enable_timers(vct_ctx* c, int32_t enable) {
    if (!c) return fail(VCT_ERR_INVALID_ARGUMENT, "ctx is NULL");
    DeviceScope ds(c->device);
    VCT_CUDA(ds.err);
    if (enable && !c->ev[0]) {
        for (auto& e : c->ev) VCT_CUDA(cudaEventCreate(&e));
    }
    c->timers_on = enable != 0;
    c->timers_recorded = false;
    return VCT_OK;
}

vct_status vct_get_timers(vct_ctx* c, vct_timers* out) {
    if (!c || !out) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!c->timers_recorded) return fail(VCT_ERR_STATE, "no timed vct_frame since timers were enabled");
    DeviceScope ds(c->device);
    VCT_CUDA(ds.err);
    VCT_CUDA(cudaEventSynchronize(c->ev[4]));
    float* dst[5] = {&out->voxelize_ms, &out->radiance_ms, &out->mipmap_ms, &out->render_ms, &out->total_ms};
    const int a[5] = {0, 1, 2, 3, 0}, b[5] = {1, 2, 3, 4, 4};
    for (int i = 0; i < 5; ++i) VCT_CUDA(cudaEventElapsedTime(dst[i], c->ev[a[i]], c->ev[b[i]]));
    return VCT_OK;
}

uint64_t vct_launch_count(void) { return g_launches.load(); }

vct_status vct_shade(vct_ctx* c, const vct_gbuffer* g, const float eye[3], const vct_light* lights, int32_t n,
                     const vct_shadow_desc* shadow, const float* irradiance, const float* specular, float* color,
                     void* stream) {
    if (!c || !eye || !color) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    vct_status s = validate_gbuffer(g);
    if (s != VCT_OK) return s;
    bool need_shadow = false;
    if ((s = validate_lights(lights, n, &need_shadow)) != VCT_OK) return s;
    if ((s = validate_shadow(shadow, need_shadow)) != VCT_OK) return s;
    for (const void* p : {(const void*)irradiance, (const void*)specular, (const void*)color})
        if (reinterpret_cast<uintptr_t>(p) % 16 != 0) return fail(VCT_ERR_INVALID_ARGUMENT, "float4 planes must be 16-byte aligned");
    DeviceScope ds(c->device);
    VCT_CUDA(ds.err);
    // the lights as the voxeliser holds them (neg_dir_n = normalize(-direction))
    AccumParams A;
    vct_triangles none = {};
    fill_accum_inputs(c->cfg, c->params, c->mvp, &none, lights, n, need_shadow ? shadow : nullptr, A);
    ShadeParams P;
    std::memset(&P, 0, sizeof P);
    P.gpos = reinterpret_cast<const float4*>(g->position_dev);
    P.gnrm = reinterpret_cast<const float4*>(g->normal_dev);
    P.galb = reinterpret_cast<const float4*>(g->albedo_dev);
    P.irradiance = reinterpret_cast<const float4*>(irradiance);
    P.specular = reinterpret_cast<const float4*>(specular);
    P.color = reinterpret_cast<float4*>(color);
    P.width = g->width;
    P.height = g->height;
    P.eye = to_f3(eye);
    P.nlights = n;
    std::memcpy(P.lights, A.lights, sizeof P.lights);
    P.shadowmap = A.shadowmap;
    P.sw = A.sw;
    P.sh = A.sh;
    std::memcpy(P.ls, A.ls, sizeof P.ls);
    const vct_params& pr = c->params;
    P.cooktorrance = pr.cooktorrance;
    P.enable_diffuse = pr.enable_diffuse;
    P.enable_specular = pr.enable_specular;
    P.enable_indirect = pr.enable_indirect;
    P.enable_reflections = pr.enable_reflections;
    P.draw_occlusion = pr.draw_occlusion;
    P.enable_postprocess = pr.enable_postprocess;
    P.roughness = pr.roughness;
    P.metallic = pr.metallic;
    P.shininess = pr.shininess;
    P.ambient_scale = pr.ambient_scale;
    P.reflect_scale = pr.reflect_scale;
    launch_shade(P, as_stream(stream));
    VCT_CHECK_LAUNCH("shade");
    return VCT_OK;
}

vct_status vct_decay_radiance(vct_ctx* c, void* stream) {
    if (!c) return fail(VCT_ERR_INVALID_ARGUMENT, "ctx is NULL");
    DeviceScope ds(c->device);
    VCT_CUDA(ds.err);
    vct_status s = sync_linear(c, as_stream(stream));
    if (s != VCT_OK) return s;
    launch_decay(c->radiance, c->nv, c->params.temporal_decay, as_stream(stream));
    VCT_CHECK_LAUNCH("decay radiance");
    c->mips_ready = false;
    c->pad_ready = false;
    c->tex_ready = false;
    return VCT_OK;
}

// mat3(transpose(inverse(model))) from the upper 3x3's cofactors / determinant.
static void normal_matrix(const float m[16], float out[9]) {
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

vct_status vct_transform_actors(const vct_triangles* local, const vct_actor* actors, int32_t n, float* pos, float* nrm,
                                void* stream) {
    vct_status s = validate_tris(local);
    if (s != VCT_OK) return s;
    if (!actors || !pos || !nrm) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n < 0 || n > VCT_MAX_ACTORS) return fail(VCT_ERR_INVALID_ARGUMENT, "n_actors must be in [0, VCT_MAX_ACTORS]");
    ActorsDev A;
    std::memset(&A, 0, sizeof A);
    A.src_pos = local->positions_dev;
    A.src_nrm = local->normals_dev;
    A.dst_pos = pos;
    A.dst_nrm = nrm;
    A.n = n;
    long long prev_end = 0;
    for (int k = 0; k < n; ++k) {
        const vct_actor& a = actors[k];
        if (a.first_triangle < prev_end || a.triangle_count < 0 || a.first_triangle + a.triangle_count > local->count)
            return fail(VCT_ERR_INVALID_ARGUMENT, "actor triangle ranges must be ascending, disjoint and inside the triangles");
        for (float v : a.model)
            if (!std::isfinite(v)) return fail(VCT_ERR_INVALID_ARGUMENT, "actor models must be finite");
        A.start[k] = a.first_triangle;
        A.end[k] = a.first_triangle + a.triangle_count;
        prev_end = A.end[k];
        std::memcpy(A.model[k], a.model, sizeof a.model);
        normal_matrix(a.model, A.normal[k]);
    }
    launch_transform_actors(A, as_stream(stream));
    VCT_CHECK_LAUNCH("transform actors");
    return VCT_OK;
}

vct_status vct_warpmap(const vct_ctx* c, const uint16_t** map) {
    if (!c || !map) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    *map = c->warpmap;
    return VCT_OK;
}

vct_status vct_get_stats(vct_ctx* c, vct_stats* out, void* stream) {
    if (!c || !out) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    DeviceScope ds(c->device);
    VCT_CUDA(ds.err);
    StatsDev h;
    VCT_CUDA(cudaMemcpyAsync(&h, c->stats, sizeof h, cudaMemcpyDeviceToHost, as_stream(stream)));
    VCT_CUDA(cudaStreamSynchronize(as_stream(stream)));
    out->total_voxel_fragments = h.total_voxel_fragments;
    out->unique_voxels = h.unique_voxels;
    out->max_fragments_per_voxel = h.max_fragments_per_voxel;
    out->error_flags = h.error_flags;
    return VCT_OK;
}

vct_status vct_render_shadowmap(const vct_triangles* tris, const float ls[16], float* depth, int32_t w, int32_t h,
                                void* stream) {
    vct_status s = validate_tris(tris);
    if (s != VCT_OK) return s;
    if (!ls || !depth || w <= 0 || h <= 0 || w > 32768 || h > 32768)
        return fail(VCT_ERR_INVALID_ARGUMENT, "shadow map arguments invalid");
    int dev = 0;
    VCT_CUDA(cudaGetDevice(&dev));
    ShadowRasterParams P;
    std::memset(&P, 0, sizeof P);
    P.pos = tris->positions_dev;
    P.ntri = tris->count;
    std::memcpy(P.ls, ls, sizeof P.ls);
    P.depth_bits = reinterpret_cast<unsigned int*>(depth);
    P.w = w;
    P.h = h;
    cudaDeviceGetAttribute(&P.num_sms, cudaDevAttrMultiProcessorCount, dev);
    launch_shadow_raster(P, as_stream(stream));
    VCT_CHECK_LAUNCH("shadow map");
    return VCT_OK;
}

vct_status vct_render_gbuffer(const vct_triangles* tris, const float vp[16], const float eye[3], const float ivp[16],
                              int32_t w, int32_t h, unsigned long long* keys, float* gpos, float* gnrm, float* galb,
                              void* stream) {
    vct_status s = validate_tris(tris);
    if (s != VCT_OK) return s;
    if (!vp || !eye || !ivp || !keys || !gpos || !gnrm || !galb || w <= 0 || h <= 0 || w > 16384 || h > 16384)
        return fail(VCT_ERR_INVALID_ARGUMENT, "gbuffer arguments invalid");
    int dev = 0;
    VCT_CUDA(cudaGetDevice(&dev));
    GbufferRasterParams P;
    std::memset(&P, 0, sizeof P);
    P.pos = tris->positions_dev;
    P.nrm = tris->normals_dev;
    P.albedo = tris->albedo_dev;
    P.ntri = tris->count;
    std::memcpy(P.vp, vp, sizeof P.vp);
    std::memcpy(P.ivp, ivp, sizeof P.ivp);
    P.eye = to_f3(eye);
    P.keys = keys;
    P.gpos = reinterpret_cast<float4*>(gpos);
    P.gnrm = reinterpret_cast<float4*>(gnrm);
    P.galb = reinterpret_cast<float4*>(galb);
    P.w = w;
    P.h = h;
    cudaDeviceGetAttribute(&P.num_sms, cudaDevAttrMultiProcessorCount, dev);
    launch_gbuffer_raster(P, as_stream(stream));
    VCT_CHECK_LAUNCH("gbuffer");
    return VCT_OK;
}

}  // extern "C"
