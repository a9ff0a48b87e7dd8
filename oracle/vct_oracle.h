/*
 * CPU oracle of the VCT hot path.  TEST INFRASTRUCTURE ONLY: it is the
 * correctness reference of the CUDA library and the timed CPU baseline; nothing
 * in the product links or calls it.
 *
 * It restates, in plain single-threaded C++17, the GLSL of sfreed141/vct:
 *   shaders/common.glsl:1-64          voxel coordinate mapping
 *   shaders/voxelize.geom:25-73       dominant-axis projection
 *   shaders/voxelize.frag:75-108,159-280  fragment lighting, PCF, accumulation
 *   shaders/testTesselation.tesc/.tese    the tessellation voxeliser
 *   shaders/transferVoxels.comp:29-70 normalisation / opacity / radiance seed
 *   shaders/injectRadiance.comp:40-103 shadow-map injection
 *   shaders/filterRadiance.comp:14-65 2x2x2 box mip
 *   shaders/phong.frag:135-180,470-511 cone tracing and composite
 *   src/Application.cpp:200-210,689-692 host matrices
 * plus the GL fixed-function pieces those shaders rely on (pixel-centre
 * rasterisation, bilinear / trilinear-mipmap filtering with clamp-to-border,
 * binary16 rounding).
 *
 * Parity is unpinned by the reference: it has no tests, fixtures or golden
 * outputs, and its OpenGL program cannot run without a graphics stack.  The
 * oracle is pinned instead by hand-computed known answers (tests/golden).
 *
 * Volumes are binary16 RGBA, x fastest, exactly as include/vct.h describes.
 * Every function with an `nthreads` argument gives bit-identical results for
 * any thread count (integer accumulation, disjoint outputs).
 */
#ifndef VCT_ORACLE_H
#define VCT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_volume {
    int32_t dim;
    float vmin[3], vmax[3], vcenter[3];
} orc_volume;

/* Voxel warping: mode 0 none, 1 voxelWarp about eye_tc (warpVoxels),
 * 2 the 32^3 RGBA16 unorm warp map (warpTexture), 3 the perspective
 * projection pv of voxelizeTesselationWarp (common.glsl:37-42; volume
 * coordinates go back to world space through vmin, vcenter, ext). */
typedef struct orc_warp {
    int32_t mode;
    const uint16_t* map;
    float eye_tc[3];
    float pv[16];
    float vmin[3], vcenter[3], ext[3];
} orc_warp;

/* Same layout as vct_light (80 bytes). */
typedef struct orc_light {
    float position[3], _p0;
    float direction[3], _p1;
    float color[3];
    float range, intensity;
    uint32_t enabled, selected, shadow_caster, type;
    uint32_t _p2[3];
} orc_light;

typedef struct orc_cone {
    int32_t steps;
    float angle, bias, h0, lod_offset;
} orc_cone;

typedef struct orc_trace_params {
    orc_cone diffuse, specular;
    int32_t enable_indirect, enable_reflections, draw_occlusion, enable_postprocess;
    float ambient_scale, reflect_scale, max_distance;
    int32_t ref_tbn_quirk;
} orc_trace_params;

typedef struct orc_stats {
    uint32_t total_voxel_fragments, unique_voxels, max_fragments_per_voxel, error_flags;
} orc_stats;

uint16_t orc_f32_to_f16(float f);
float orc_f16_to_f32(uint16_t h);
void orc_f32_to_f16_array(const float* in, uint16_t* out, int64_t n);

void orc_voxel_mvp(const orc_volume* vol, float out[48]);
void orc_lookat(const float eye[3], const float center[3], const float up[3], float out[16]);
void orc_ortho(float l, float r, float b, float t, float n, float f, float out[16]);
void orc_perspective(float fovy, float aspect, float znear, float zfar, float out[16]);
void orc_mat4_mul(const float a[16], const float b[16], float out[16]);

/* count[dim^3] (uint32), sums[6*dim^3] (uint64, SoA r,g,b,nx,ny,nz) are ADDED
 * to; the sums are exact for any number of fragments per voxel. */
void orc_voxelize(const orc_volume* vol, const float* pos, const float* nrm, const float* albedo,
                  int64_t ntri, const orc_light* lights, int32_t nlights, int32_t lighting,
                  int32_t axis_override, const float* shadowmap, int32_t sw, int32_t sh,
                  const float ls[16], uint32_t* count, uint64_t* sums, uint32_t* total_fragments,
                  int32_t nthreads, const orc_warp* warp);

/* Tessellation voxeliser (testTesselation.tesc/.tese): levels of one
 * triangle (9 floats) after GL's equal_spacing rounding, out = {inner,
 * outer0, outer1, outer2}; returns 0 when the control shader discards the
 * patch (all three vertices in one voxel). */
int32_t orc_tess_levels(const orc_volume* vol, const float* tri, float max_level, int32_t out[4]);
/* Number of points of GL's triangle tessellation in point mode, and their
 * gl_TessCoord (3 floats each) in this oracle's enumeration order. */
int32_t orc_tess_point_count(const int32_t levels[4]);
void orc_tess_coords(const int32_t levels[4], float* out);
/* Every generated point stores the triangle's albedo and its normal into
 * the voxel holding it (linear mapping, or warp mode 3).  count/sums as for
 * orc_voxelize; total_points counts the generated points. */
void orc_voxelize_tess(const orc_volume* vol, const float* pos, const float* nrm, const float* albedo,
                       int64_t ntri, float max_level, const orc_warp* warp, uint32_t* count, uint64_t* sums,
                       uint64_t* total_points, int32_t nthreads);

/* transferVoxels.comp; radiance/colour/normal are dim^3 RGBA16F (uint16 x4). */
void orc_normalize(const orc_volume* vol, float voxel_set_opacity, int32_t temporal_filter,
                   float temporal_decay, const uint32_t* count, const uint64_t* sums,
                   uint16_t* color, uint16_t* normal, uint16_t* radiance, orc_stats* stats,
                   int32_t nthreads);

void orc_inject(const orc_volume* vol, const float* shadowmap, int32_t sw, int32_t sh,
                const float ls_inverse[16], const float light_pos[3], const float light_int[3],
                int32_t radiance_lighting, int32_t radiance_dilate, const uint16_t* color,
                const uint16_t* normal, uint16_t* radiance, int32_t nthreads, const orc_warp* warp,
                int32_t temporal, float decay);
/* phong.frag's composite with direct lighting (see vct_shade). */
typedef struct orc_shade_params {
    int32_t cooktorrance, enable_diffuse, enable_specular, enable_indirect, enable_reflections, draw_occlusion,
        enable_postprocess;
    float roughness, metallic, shininess, ambient_scale, reflect_scale;
} orc_shade_params;
void orc_shade(const float* gpos, const float* gnrm, const float* galb, int32_t width, int32_t height,
               const float eye[3], const orc_light* lights, int32_t nlights, const float* shadowmap, int32_t sw,
               int32_t sh, const float ls[16], const float* irradiance, const float* specular,
               const orc_shade_params* sp, float* color);
/* temporalRadianceFilter.comp: radiance (nv RGBA16F voxels) *= decay. */
void orc_decay_radiance(uint16_t* radiance, int64_t nv, float decay);
/* mat3(transpose(inverse(model))) of an affine model (column-major in and out). */
void orc_normal_matrix(const float model[16], float out[9]);
/* Rigid actors: triangles [first[k], first[k] + count[k]) transformed by model k. */
void orc_transform_actors(const float* src_pos, const float* src_nrm, const int64_t* first, const int64_t* count,
                          const float* models, int32_t n, float* dst_pos, float* dst_nrm);

/* chain: all `levels` levels contiguous; level 0 is read, 1.. are written. */
void orc_build_mips(int32_t dim, int32_t levels, uint16_t* chain, int32_t nthreads);

/* Rows [row0, row1) of the G-buffer are traced; outputs are full-size float4
 * images (rows outside the range untouched).  Any output may be NULL.
 * precision: 32 = the fp32 transcription, 64 = the fp64 reference. */
void orc_trace(const orc_volume* vol, int32_t levels, const uint16_t* chain,
               const orc_trace_params* tp, const float* gpos, const float* gnrm,
               const float* galb, int32_t width, int32_t height, int32_t row0, int32_t row1,
               int32_t row_step, const float eye[3], int32_t precision, float* irradiance,
               float* specular, float* color, uint64_t* samples, int32_t nthreads, const orc_warp* warp);

/* Cone set of the learned path's 16-cone reference: for each listed pixel,
 * sum over cones c of dirs[4c+3] * traceCone(dir = T dirs[4c] + B dirs[4c+1]
 * + N dirs[4c+2]) in the Duff et al. frame; float4 per listed pixel. */
void orc_trace_cone_set(const orc_volume* vol, int32_t levels, const uint16_t* chain, const float* dirs,
                        int32_t ncones, const orc_cone* cone, float max_distance, const float* gpos,
                        const float* gnrm, int32_t width, const int32_t* pixels, int64_t npix, int32_t precision,
                        float* out, uint64_t* samples, int32_t nthreads, const orc_warp* warp);
/* Cheap quarter-resolution features of the learned path, fp32,
 * ceil(W/4) x ceil(H/4) x 32. */
void orc_learned_features(const orc_volume* vol, int32_t levels, const uint16_t* chain, const float* gpos,
                          const float* gnrm, int32_t width, int32_t height, float* out, const orc_warp* warp);
/* The 32^3 warp map (RGBA16 unorm, x fastest) from a 32^3 occupancy grid
 * (bytes, nonzero = occupied): Application.cpp:313-371, generateWarpmapWeights.frag
 * (weights stored binary16), generateWarpmap.frag. */
void orc_warpmap(const uint8_t* occupancy, float high, float low, uint16_t* map);

void orc_render_shadowmap(const float* pos, int64_t ntri, const float ls[16], int32_t w, int32_t h,
                          float* depth, int32_t nthreads);
void orc_render_gbuffer(const float* pos, const float* nrm, const float* albedo, int64_t ntri,
                        const float vp[16], const float eye[3], const float inv_vp[16], int32_t w,
                        int32_t h, float* gpos, float* gnrm, float* galb);

#ifdef __cplusplus
}
#endif

#endif
