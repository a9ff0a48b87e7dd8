/*
 * vct.h - C ABI of the GB300 voxel cone tracing hot path.
 *
 * The reference (sfreed141/vct) drives this path through OpenGL programs whose
 * operator surface is a set of named uniforms, image/texture bindings and an
 * SSBO of lights (src/Application.cpp:666-1067).  This header replaces that
 * surface with plain C entry points over device pointers:
 *
 *   reference program / call site                         entry point here
 *   voxelize.vert/.geom/.frag   src/Application.cpp:666-754   vct_voxelize_accumulate
 *   simpleTesselated.vert, testTesselation.tesc/.tese
 *                               src/Application.cpp:585-662   vct_voxelize_accumulate with
 *                                                             params.voxelize_tesselation
 *   transferVoxels.comp         src/Application.cpp:757-785   vct_normalize
 *   (both, back to back)                                      vct_voxelize
 *   injectRadiance.comp         src/Application.cpp:788-837   vct_inject
 *   filterRadiance.comp loop    src/Application.cpp:877-921   vct_build_mips
 *   phong.frag cone tracing     src/Application.cpp:967-1067  vct_trace
 *   the four timed regions      src/Application.cpp:583-1067  vct_frame
 *   VoxelizeInfo SSBO readback  src/Overlay.cpp:104-116       vct_get_stats
 *   Settings / VCTSettings      src/Application.h:28-103      vct_params
 *   class VCT (volumes, dims)   src/Application.h:107-156     vct_config + vct_ctx
 *   struct Light (std140, 80 B) src/Scene.h:13-34             vct_light
 *
 * Conventions
 *  - Every function returns vct_status; nothing throws across the ABI.
 *  - Pointers named *_dev are CUDA device pointers owned by the caller.
 *    Volumes (accumulators, colour/normal/radiance mip chains) are owned by
 *    the context.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default
 *    stream).  Calls are stream ordered; host arguments are copied before
 *    the call returns.
 *  - A context is bound to the CUDA device given at creation and is not
 *    thread safe: use one context per host thread.
 *  - Matrices are column-major float[16], as glm / GLSL store them.
 *  - Volumes are RGBA16F (IEEE binary16 x4, 8 bytes per voxel), x fastest:
 *    voxel (x,y,z) of level l lives at level_offset[l] + (z*S + y)*S + x
 *    with S = dim >> l.
 */
#ifndef VCT_H
#define VCT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VCT_ABI_VERSION 1
#define VCT_MAX_LIGHTS 16
#define VCT_MAX_LEVELS 11 /* dim <= 1024 */

typedef enum vct_status {
    VCT_OK = 0,
    VCT_ERR_INVALID_ARGUMENT = 1,
    VCT_ERR_OUT_OF_MEMORY = 2,
    VCT_ERR_CUDA = 3,
    VCT_ERR_STATE = 4,       /* call order violated (e.g. trace before mips) */
    VCT_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
    VCT_ERR_UNSUPPORTED = 6,
    VCT_ERR_OVERFLOW = 7     /* a voxel received more fragments than the exact range */
} vct_status;

typedef struct vct_ctx vct_ctx;

/* Light types, as `uint type` in the reference Light block (src/Scene.h:14). */
#define VCT_LIGHT_POINT 0u
#define VCT_LIGHT_DIRECTIONAL 1u

/* Byte-for-byte the std140 record the reference writes into its light SSBO
 * (src/Scene.cpp:64-76, shaders/voxelize.frag:31-44): 80 bytes per light. */
typedef struct vct_light {
    float position[3];
    float _pad0;
    float direction[3];
    float _pad1;
    float color[3];
    float range;           /* offset 44 */
    float intensity;       /* offset 48 */
    uint32_t enabled;      /* offset 52 */
    uint32_t selected;     /* offset 56 (unused by the path) */
    uint32_t shadow_caster;/* offset 60 */
    uint32_t type;         /* offset 64 */
    uint32_t _pad2[3];
} vct_light;

/* Volume set-up: the reference's class VCT (src/Application.h:107-156). */
#define VCT_CONFIG_COLOR_MIPS 1u /* also keep a colour mip chain (reference's second filter loop) */

typedef struct vct_config {
    int32_t voxel_dim;     /* power of two in [16, 1024]  (VCT::voxelDim) */
    int32_t voxel_levels;  /* 0 = full chain log2(dim)+1; clamped like VCT::remake */
    float voxel_min[3];    /* VCT::min, must equal -voxel_max (symmetric, cubic) */
    float voxel_max[3];    /* VCT::max */
    float voxel_center[3]; /* VCT::center */
    int32_t device;        /* CUDA device ordinal */
    uint32_t flags;        /* VCT_CONFIG_* */
} vct_config;

/* One cone family: the reference's VCTSettings (src/Application.h:28-34). */
typedef struct vct_cone_settings {
    int32_t steps;
    float cone_angle;          /* radians, full aperture */
    float bias;                /* start offset along the normal, in voxels */
    float cone_initial_height; /* in voxels */
    float lod_offset;
} vct_cone_settings;

#define VCT_FILTER_SOFTWARE 0 /* fp32 trilinear (exact GL semantics) from a bordered fp32 copy of the chain */
#define VCT_FILTER_HARDWARE 1 /* texture units' trilinear-mip filtering */
#define VCT_FILTER_HARDWARE_LEVELS 2 /* texture units' trilinear filtering per level, levels blended in fp32 */
#define VCT_FILTER_HYBRID 3 /* of the two levels of each trilinear-mip sample, the one with the larger weight in
                               exact fp32 (as SOFTWARE), the other by the texture units, blended in fp32 */

/* Voxel warping: positions in [0,1]^3 volume coordinates are remapped before
 * they index or sample the grid, in the voxeliser (voxelize.frag:100-106),
 * injection (getVoxelPosition) and the cone tracer (phong.frag:150-157).
 *  - ANALYTIC (warpVoxels): voxelWarp about the eye, a cubic per axis
 *    (common.glsl:11-31).
 *  - TEXTURE (warpTexture): a 32^3 warp map built every voxelisation from a
 *    32^3 occupancy voxelisation of the same triangles: per axis, occupied
 *    warp cells get warp_high_resolution and empty ones a resolution that
 *    keeps each row's total (Application.cpp:346-371), the weights stored as
 *    binary16 (the RGBA16F weight textures), cell centres warped by the
 *    prefix sums of the widths (generateWarpmap.frag), stored RGBA16 unorm
 *    and read with trilinear filtering and clamp-to-edge. */
/*  - PERSPECTIVE (voxelizeTesselationWarp): the grid is laid over the camera
 *    frustum of `pv`; a world position maps to (pv p).xyz / (pv p).w * 0.5
 *    + 0.5 (common.glsl:37-42).  Injection and the cone tracer use it as the
 *    reference does (getVoxelPosition, phong.frag:158-160), and so does the
 *    tessellation voxeliser; the rasterising voxeliser ignores it, as
 *    voxelize.frag does.  Projected coordinates outside [-1, 2] (all of them
 *    off the grid) are replaced by -1 so that points on or behind the camera
 *    plane stay well defined. */
#define VCT_WARP_NONE 0
#define VCT_WARP_ANALYTIC 1
#define VCT_WARP_TEXTURE 2
#define VCT_WARP_PERSPECTIVE 3
#define VCT_WARP_DIM 32

/* Tessellation voxeliser (voxelizeTesselation: simpleTesselated.vert,
 * testTesselation.tesc/.tese; Application.cpp:585-662).  Every triangle is a
 * patch whose tessellation levels follow the control shader (each outer
 * level the edge length in voxels along the edge direction, the inner level
 * the longest altitude in voxels, all at least 1; a triangle whose three
 * vertices truncate to one voxel is discarded), tessellated as GL's
 * triangle primitive generator does in point mode with equal spacing (levels
 * clamped to [1, max_tess_level] and rounded up; concentric inner rings built
 * from the perpendiculars of the inner subdivision, OpenGL 4.6 section
 * 11.2.2.1).  Every generated point stores the triangle's albedo and its
 * interpolated normal into the voxel that contains it, unlit, like the
 * evaluation shader.  The rasterising voxeliser stays the default of
 * vct_default_params because the benchmark frame is defined on its
 * pixel-centre rule; the reference's own default is the tessellation one
 * (Application.h:100). */
#define VCT_MAX_TESS_LEVEL 64 /* GL_MAX_TESS_GEN_LEVEL of the reference's GL implementation */

/* Every hot-path uniform of the reference, with vct_default_params giving the
 * reference defaults of src/Application.h:36-103. */
typedef struct vct_params {
    /* voxelize.geom / voxelize.frag */
    int32_t voxelize_lighting;   /* voxelizeLighting (default 1) */
    int32_t axis_override;       /* axis_override (-1: dominant axis) */
    /* transferVoxels.comp */
    float voxel_set_opacity;     /* voxelSetOpacity (0.5) */
    int32_t temporal_filter;     /* temporalFilterRadiance (0) */
    float temporal_decay;        /* temporalDecay (0.8) */
    /* injectRadiance.comp */
    int32_t radiance_lighting;   /* radianceLighting (0) */
    int32_t radiance_dilate;     /* radianceDilate (0) */
    /* phong.frag */
    vct_cone_settings diffuse_cone;  /* {16, 60 deg, 1.0, 1.0, 0.5} */
    vct_cone_settings specular_cone; /* {32, 30 deg, 1.7, 0.5, 0.1} */
    int32_t enable_indirect;     /* 1 */
    int32_t enable_reflections;  /* 1 */
    int32_t draw_occlusion;      /* 1 */
    int32_t enable_postprocess;  /* 1 */
    float ambient_scale;         /* 1.0 */
    float reflect_scale;         /* 1.0 */
    float max_distance;          /* cone length limit in texture units; <= 0: grid diagonal */
    int32_t ref_tbn_quirk;       /* 1: map the cone set's y axis to the bitangent as phong.vert's TBN does */
    int32_t trace_filter;        /* VCT_FILTER_* */
    /* voxel warping (common.glsl:11-64, generateWarpmap.frag, Application.cpp:300-580) */
    int32_t warp_mode;           /* VCT_WARP_* (warpVoxels / warpTexture; default none) */
    float warp_high_resolution;  /* warpTextureHighResolution (2.0) */
    float warp_low_resolution;   /* warpTextureLowResolution (0.5) */
    /* direct lighting of vct_shade (phong.frag:183-344) */
    int32_t cooktorrance;        /* cooktorrance (1): GGX Cook-Torrance, else Blinn-Phong */
    int32_t enable_diffuse;      /* enableDiffuse (1) */
    int32_t enable_specular;     /* enableSpecular (1) */
    float roughness;             /* 0.5: phong.frag's value without a roughness map */
    float metallic;              /* 0.0: without a metallic map */
    float shininess;             /* material.shininess (32, src/Graphics/Mesh.h:29) */
    /* tessellation voxeliser and the perspective warp (Application.cpp:202,585-662) */
    int32_t voxelize_tesselation; /* voxelizeTesselation (0 here; see VCT_MAX_TESS_LEVEL) */
    float max_tess_level;         /* GL_MAX_TESS_GEN_LEVEL, in [1, VCT_MAX_TESS_LEVEL] (64) */
    float pv[16];                 /* 'pv' = perspective(fov, aspect, 1, 20) * view, column-major */
} vct_params;

/* Caller-owned triangle soup on the device. */
typedef struct vct_triangles {
    const float* positions_dev; /* count*9 floats: v0.xyz v1.xyz v2.xyz (world space) */
    const float* normals_dev;   /* count*9 floats: per-vertex normals */
    const float* albedo_dev;    /* count*3 floats: diffuse colour per triangle */
    int64_t count;
} vct_triangles;

/* G-buffer: one float4 per pixel in each plane, row 0 at the bottom. */
typedef struct vct_gbuffer {
    const float* position_dev; /* world xyz, w = 1 covered / 0 background */
    const float* normal_dev;   /* unit normal xyz */
    const float* albedo_dev;   /* diffuse rgb */
    int32_t width, height;
} vct_gbuffer;

/* Trace outputs, float4 per pixel; any pointer may be NULL. */
typedef struct vct_trace_out {
    float* irradiance_dev; /* sum of weighted diffuse cones: rgb, a = accumulated opacity */
    float* specular_dev;   /* specular cone rgba */
    float* color_dev;      /* composite (indirect*albedo [*occlusion], post-processed) */
    unsigned long long* sample_count_dev; /* optional: += number of trilinear-mip samples */
} vct_trace_out;

/* Light-space inputs of one frame (the mainlight of src/Application.cpp:205-210). */
typedef struct vct_shadow_desc {
    const float* shadowmap_dev; /* width*height fp32 depths in [0,1], row 0 at the bottom */
    int32_t width, height;
    float ls[16];         /* light projection * view */
    float ls_inverse[16]; /* inverse(ls), as the host computes it */
    float light_pos[3];   /* injectRadiance 'lightPos' */
    float light_int[3];   /* injectRadiance 'lightInt' */
} vct_shadow_desc;

/* VoxelizeInfo block (shaders/voxelize.frag:53-59). */
typedef struct vct_stats {
    uint32_t total_voxel_fragments;
    uint32_t unique_voxels;
    uint32_t max_fragments_per_voxel;
    uint32_t error_flags; /* VCT_STATS_* */
} vct_stats;

/* Some voxel's colour and normal sums are not exact: the rasterising
 * voxeliser put VCT_MAX_EXACT_FRAGMENTS or more fragments into it (its
 * packed 32-bit sums carry), or the tessellation voxeliser, whose sums stay
 * exact past that bound, found no free slot in its table of voxels whose
 * sums passed 2^32 (65,536 slots). */
#define VCT_STATS_COUNT_OVERFLOW 1u
#define VCT_MAX_EXACT_FRAGMENTS 65537u

/* Device time of the last vct_frame's stages, the reference's GLBufferedTimer
 * regions (src/Application.h:192): voxelize = rasterise + accumulate,
 * radiance = what remains of injection marking after the voxeliser (the
 * marking runs concurrently with it, so usually about 0), mipmap = normalise
 * + inject resolve + mip chain, render = cone tracing, total = all of them. */
typedef struct vct_timers {
    float voxelize_ms;
    float radiance_ms;
    float mipmap_ms;
    float render_ms;
    float total_ms;
} vct_timers;

#define VCT_VOLUME_COLOR 0
#define VCT_VOLUME_NORMAL 1
#define VCT_VOLUME_RADIANCE 2

/* ---- library ---------------------------------------------------------- */
int32_t vct_abi_version(void);
const char* vct_status_string(vct_status s);
/* Message of the last failing call on this host thread ("" if none). */
const char* vct_last_error(void);
/* sizeof of the public structs, for FFI layout checks. */
void vct_struct_sizes(int64_t* light, int64_t* config, int64_t* params,
                      int64_t* triangles, int64_t* gbuffer, int64_t* trace_out,
                      int64_t* shadow_desc, int64_t* stats);
/* sizeof of a public struct by name ("vct_tuning"), or offsetof of one of its
 * fields ("vct_scene_desc.eye"); -1 for an unknown name. */
int64_t vct_struct_layout(const char* name);
/* Reference defaults (src/Application.h:36-103). */
void vct_default_params(vct_params* out);
/* The three per-axis voxelisation matrices of src/Application.cpp:689-692. */
vct_status vct_voxel_mvp(const vct_config* cfg, float mvp_xyz[48]);

/* ---- context ---------------------------------------------------------- */
vct_status vct_create(const vct_config* cfg, vct_ctx** out);
vct_status vct_destroy(vct_ctx* ctx);
vct_status vct_set_params(vct_ctx* ctx, const vct_params* params);
vct_status vct_get_params(const vct_ctx* ctx, vct_params* out);
vct_status vct_get_config(const vct_ctx* ctx, vct_config* out);
/* Device pointer of one level of a volume (read-only view for callers).
 * With VCT_FILTER_HYBRID and no temporal filter, vct_frame / vct_frame_volume
 * leave the linear copy of radiance levels 0-3 to the sampler's texture array
 * (the same binary16 texels); the first call for such a level synchronises
 * the device and copies them back.  The stage entry points that read the
 * radiance chain (vct_normalize, vct_inject, vct_build_mips,
 * vct_decay_radiance) do the same copy on their stream. */
vct_status vct_volume_level(const vct_ctx* ctx, int32_t volume, int32_t level,
                            const uint16_t** data_dev, int32_t* dim);
/* Device pointers of the integer accumulators: one 8 x uint32 record per
 * voxel {count, r, g, b, nx, ny, nz, 0} (sums of round(x * 65535)), and the
 * occupancy bit mask (bit v%32 of word v/32 for voxel v = (z*dim + y)*dim + x).
 * Voxel v's record is at records_dev[8*s], s being v with bit 1 (bit 1 of x)
 * and bit log2(dim) (bit 0 of y) exchanged: each 128-byte line of records
 * holds a 2 x 2 block of voxels in x and y.
 * Between vct_voxelize_accumulate and vct_normalize they hold the sums of
 * the frame; vct_normalize / vct_frame leave them zeroed. */
vct_status vct_accumulators(const vct_ctx* ctx, const uint32_t** records_dev,
                            const uint32_t** occupancy_dev);
/* The slot s of voxel v's record (records_dev[8*s]) in a dim^3 grid. */
int64_t vct_record_slot(int64_t v, int32_t dim);

/* ---- stages ----------------------------------------------------------- */
/* voxelize.geom/.frag: rasterise every triangle along its dominant axis and
 * add colour, normal and count of each fragment into the accumulators.  With
 * params.voxelize_tesselation the triangles are tessellated into points
 * instead (testTesselation.tesc/.tese) and lights and shadow map are not
 * read; total_voxel_fragments then counts the generated points. */
vct_status vct_voxelize_accumulate(vct_ctx* ctx, const vct_triangles* tris,
                                   const vct_light* lights, int32_t n_lights,
                                   const vct_shadow_desc* shadow, const float eye[3],
                                   void* stream);
/* transferVoxels.comp: divide by count, set opacity, seed radiance level 0,
 * update the VoxelizeInfo counters and zero the accumulators. */
vct_status vct_normalize(vct_ctx* ctx, void* stream);
/* Clear accumulators (only needed after an abandoned accumulate). */
vct_status vct_clear_accumulators(vct_ctx* ctx, void* stream);
/* vct_voxelize_accumulate + vct_normalize. */
vct_status vct_voxelize(vct_ctx* ctx, const vct_triangles* tris, const vct_light* lights,
                        int32_t n_lights, const vct_shadow_desc* shadow, const float eye[3],
                        void* stream);
/* injectRadiance.comp: one thread per shadow-map texel. */
vct_status vct_inject(vct_ctx* ctx, const vct_shadow_desc* shadow, const float eye[3],
                      void* stream);
/* filterRadiance.comp over all levels of VCT_VOLUME_RADIANCE or VCT_VOLUME_COLOR. */
vct_status vct_build_mips(vct_ctx* ctx, int32_t volume, void* stream);
/* phong.frag indirect term: six diffuse cones + one specular cone per pixel. */
vct_status vct_trace(vct_ctx* ctx, const vct_gbuffer* gbuffer, const float eye[3],
                     const vct_trace_out* out, void* stream);
/* No counterpart in the reference, which draws one camera per frame.  The
 * phong.frag trace of n viewpoints of the same volumes (gbuffers[i], eye
 * eyes[3*i..3*i+2], outputs outs[i]) in one launch per 8 viewpoints:
 * equal, bit for bit, to n vct_trace calls. */
vct_status vct_trace_views(vct_ctx* ctx, int32_t n, const vct_gbuffer* gbuffers, const float* eyes,
                           const vct_trace_out* outs, void* stream);
/* All four stages; normalisation, injection and the first mip levels are
 * fused.  Results equal vct_voxelize + vct_inject + vct_build_mips +
 * vct_trace on the same inputs. */
vct_status vct_frame(vct_ctx* ctx, const vct_triangles* tris, const vct_light* lights,
                     int32_t n_lights, const vct_shadow_desc* shadow, const float eye[3],
                     const vct_gbuffer* gbuffer, const vct_trace_out* out, void* stream);
/* The volume half of vct_frame (voxelise, inject, mips; the reference's
 * passes before phong.frag), for callers that overlap the upload of the
 * G-buffer with it: vct_frame = vct_frame_volume + vct_trace, with the same
 * results.  With timers enabled, the next vct_trace records the render
 * stage. */
vct_status vct_frame_volume(vct_ctx* ctx, const vct_triangles* tris, const vct_light* lights,
                            int32_t n_lights, const vct_shadow_desc* shadow, const float eye[3],
                            void* stream);
/* Peak rate of the cone tracer's textureLod samples on this GPU, the
 * denominator of its roofline (the tracer is bound by sample filtering, not
 * HBM): `samples` samples spread over the GPU, each through the sampler of
 * `filter` (VCT_FILTER_*), at positions inside one small region of the
 * current radiance chain (so its texels stay in L1) and at the levels and
 * fractions cone steps use.  Needs a built chain (vct_frame, or
 * vct_build_mips).  Synchronises `stream`. */
vct_status vct_sampler_rate(vct_ctx* ctx, int32_t filter, int64_t samples, double* samples_per_second,
                            void* stream);
/* Synchronises `stream` and returns the VoxelizeInfo counters of the last
 * vct_normalize / vct_frame. */
vct_status vct_get_stats(vct_ctx* ctx, vct_stats* out, void* stream);

/* Per-stage CUDA-event timers of vct_frame (off by default). */
vct_status vct_enable_timers(vct_ctx* ctx, int32_t enable);
/* Waits for the last timed vct_frame and returns its stage times. */
vct_status vct_get_timers(vct_ctx* ctx, vct_timers* out);
/* phong.frag's full composite (main, 430-520) for a G-buffer: direct
 * lighting of every enabled light (Cook-Torrance with GGX and Schlick-GGX, or
 * Blinn-Phong; point-light range and smoothstep attenuation; 5-tap PCF for
 * shadow casters, phong.frag:183-207) plus the indirect term from a previous
 * vct_trace: color = (irradiance.rgb + specular.rgb * reflect_scale) *
 * ambient_scale * albedo + diffuse + specular, times the occlusion
 * 1 - clamp(irradiance.a) with draw_occlusion; without irradiance (NULL, or
 * enable_indirect 0): ambient_scale * albedo + diffuse + specular; then the
 * tone map and gamma with enable_postprocess.  color_dev: float4 per pixel. */
vct_status vct_shade(vct_ctx* ctx, const vct_gbuffer* gbuffer, const float eye[3], const vct_light* lights,
                     int32_t n_lights, const vct_shadow_desc* shadow, const float* irradiance_dev,
                     const float* specular_dev, float* color_dev, void* stream);

/* temporalRadianceFilter.comp: radiance level 0 *= temporal_decay (every
 * voxel, RGBA16F rounded).  The coarser levels are stale until the next
 * vct_build_mips. */
vct_status vct_decay_radiance(vct_ctx* ctx, void* stream);

/* ---- rigid actors (src/Actor.h, src/Transform.h, voxelize.vert) --------- */
/* Triangles [first_triangle, first_triangle + triangle_count) of `local`
 * move with `model` (column-major): positions = model * p, normals =
 * mat3(transpose(inverse(model))) * n (computed here from the upper 3x3's
 * cofactors and determinant), written to the same triangle indices of
 * positions_dev / normals_dev (count * 9 floats each; other triangles are
 * not written).  Ranges ascending and non-overlapping, at most
 * VCT_MAX_ACTORS per call. */
#define VCT_MAX_ACTORS 64 /* = the kernel's per-launch table */
typedef struct vct_actor {
    int64_t first_triangle;
    int64_t triangle_count;
    float model[16];
} vct_actor;
vct_status vct_transform_actors(const vct_triangles* local, const vct_actor* actors, int32_t n_actors,
                                float* positions_dev, float* normals_dev, void* stream);

/* The warp map of the last voxelisation with VCT_WARP_TEXTURE: 32^3 texels,
 * x fastest, RGBA16 unorm (xyz = warped coordinate * 65535, w = the packed
 * cell information of generateWarpmap.frag). */
vct_status vct_warpmap(const vct_ctx* ctx, const uint16_t** map_dev);
/* Number of kernels this library has launched since it was loaded. */
uint64_t vct_launch_count(void);

/* ---- batched scenes ---------------------------------------------------- */
/* No counterpart in the reference (it renders one scene per frame).  A batch
 * owns one context per scene (grids may differ, each <= 256^3, all on one
 * device) and runs vct_frame for every scene with one launch per stage:
 * the voxeliser's work units, the shadow texels, the resolve bricks and the
 * pixel tiles of all scenes are concatenated and each launch maps a global
 * work index back to its scene.  Results equal vct_frame per scene. */
typedef struct vct_batch vct_batch;

typedef struct vct_scene_desc {
    vct_triangles triangles;
    const vct_light* lights; /* host array */
    int32_t n_lights;
    vct_shadow_desc shadow;
    float eye[3];
    vct_gbuffer gbuffer;
    vct_trace_out out;
} vct_scene_desc;

vct_status vct_batch_create(const vct_config* scene_cfg, int32_t n_scenes, vct_batch** out);
vct_status vct_batch_destroy(vct_batch* batch);
/* Parameters of one scene (scene = -1: every scene); all scenes must use the
 * same trace_filter and voxeliser; warp modes may differ (scenes with
 * VCT_WARP_TEXTURE build their maps inside the batched frame). */
vct_status vct_batch_set_params(vct_batch* batch, int32_t scene, const vct_params* params);
vct_status vct_batch_frame(vct_batch* batch, const vct_scene_desc* scenes, int32_t n_scenes, void* stream);
/* Records vct_batch_frame for `scenes` into a CUDA graph owned by the batch
 * (the descriptors are copied: replays run the captured scenes). */
vct_status vct_batch_capture(vct_batch* batch, const vct_scene_desc* scenes, int32_t n_scenes, void* stream);
vct_status vct_batch_replay(vct_batch* batch, void* stream);
/* The context of one scene (volumes, stats) for reading. */
vct_status vct_batch_context(vct_batch* batch, int32_t scene, vct_ctx** ctx);
/* CUDA-event stage timers of vct_batch_frame (not of graph replays):
 * voxelize_ms (all scenes' voxelisation), mipmap_ms (injection, resolve and
 * mip chains), render_ms (cone tracing), total_ms; radiance_ms is 0. */
vct_status vct_batch_enable_timers(vct_batch* batch, int32_t enable);
vct_status vct_batch_get_timers(vct_batch* batch, vct_timers* out);

/* ---- launch shapes and the autotuner ----------------------------------- */
/* No counterpart in the reference (its launch shapes are fixed by the GL
 * pipeline and the compute shaders' local sizes).  Every setting gives
 * bit-identical results; only speed differs. */
typedef struct vct_tuning {
    int32_t voxel_unit_pixels;   /* candidate pixels (rows' spans of the triangle) per voxeliser work unit, about: power of two in [32, 8192] (512) */
    int32_t voxel_blocks_per_sm; /* resident voxeliser raster CTAs per SM: 1..3 (3) */
    int32_t trace_tile_w;        /* pixel tile of one 256-thread trace CTA, tile_w * tile_h = 256: */
    int32_t trace_tile_h;        /*   tile_w a power of two in [4, 64] (16 x 16) */
    int32_t trace_warp_w;        /* pixel tile of one warp: warp_w x 32/warp_w, warp_w a power of two with */
                                 /*   tile_w/8 <= warp_w <= min(tile_w, 32) (8) */
} vct_tuning;

void vct_default_tuning(vct_tuning* out);
vct_status vct_get_tuning(const vct_ctx* ctx, vct_tuning* out);
vct_status vct_set_tuning(vct_ctx* ctx, const vct_tuning* tuning);
vct_status vct_batch_get_tuning(const vct_batch* batch, vct_tuning* out);
vct_status vct_batch_set_tuning(vct_batch* batch, const vct_tuning* tuning);
/* Times vct_frame under each candidate voxeliser setting and each candidate
 * trace tile shape (`reps` frames each, median of the stage's CUDA-event
 * time; the two stages are tuned independently), keeps the fastest as the
 * context's tuning and returns it in `best` (may be NULL).  Synchronises
 * `stream`; the frame's outputs are written as by vct_frame. */
vct_status vct_autotune(vct_ctx* ctx, const vct_triangles* tris, const vct_light* lights, int32_t n_lights,
                        const vct_shadow_desc* shadow, const float eye[3], const vct_gbuffer* gbuffer,
                        const vct_trace_out* out, int32_t reps, void* stream, vct_tuning* best);
/* The same for a batch, timing vct_batch_frame; drops a captured graph. */
vct_status vct_batch_autotune(vct_batch* batch, const vct_scene_desc* scenes, int32_t n_scenes, int32_t reps,
                              void* stream, vct_tuning* best);

/* ---- learned path ------------------------------------------------------ */
/* No counterpart in the reference.  Diagnostic of the tensor-core path the
 * MLP kernels use: one 128 x n x k BF16 GEMM with FP32 accumulation on the
 * fifth-generation tensor cores (tcgen05.mma, accumulator in tensor memory):
 * d_dev (128 x n, row-major fp32) = a_dev (128 x k) * b_dev (n x k)^T, the
 * operands row-major BF16 bit patterns; k, n in {16, 32, 48, 64}.  variant 1
 * exchanges the two stride fields of the shared-memory descriptors (a check
 * of the layout convention: it must NOT reproduce the product).
 * Synchronises `stream`; VCT_ERR_TIMEOUT if the MMA did not complete. */
vct_status vct_tensor_core_check(const uint16_t* a_dev, const uint16_t* b_dev, int32_t k, int32_t n,
                                 int32_t variant, float* d_dev, void* stream);
/* No counterpart in the reference.  Exercises the timeout path of the
 * bounded device-side waits (the tensor-core kernels' mbarrier waits): one
 * thread waits on an mbarrier that nothing arrives on, gives up after
 * limit_ns (in [1e3, 1e9]) and records it.  Synchronises `stream` and
 * returns VCT_ERR_TIMEOUT, the expected outcome; the device stays usable. */
vct_status vct_timeout_probe(int64_t limit_ns, void* stream);

/* The network: 42 inputs, three hidden layers of 64 with ReLU, 4 linear
 * outputs: irradiance RGB and the network's estimate of its own error there
 * (|irradiance - target|, Euclidean over RGB); BF16 weights and activations,
 * FP32 accumulation on the tensor cores, FP32 master parameters and Adam
 * state.  Parameters are packed fp32: W1[64][42] b1[64] W2[64][64] b2[64]
 * W3[64][64] b3[64] W4[4][64] b4[4] (W[out][in]).  Training minimises the
 * mean squared error over the n x 3 irradiance outputs plus
 * VCT_MLP_CONFIDENCE_WEIGHT times the mean over the n rows of
 * (estimate - |irradiance - target|)^2, the second term's |irradiance -
 * target| held constant.  Feature rows: n x 42 fp32, row-major, 8-byte
 * aligned; targets: n x 3 fp32. */
#define VCT_MLP_INPUTS 42
#define VCT_MLP_HIDDEN 64
#define VCT_MLP_OUTPUTS 4
#define VCT_MLP_PARAMS 11332
#define VCT_MLP_CONFIDENCE_WEIGHT 0.5f
typedef struct vct_mlp vct_mlp;
typedef struct vct_adam {
    float lr, beta1, beta2, eps;
} vct_adam;

/* He-uniform weights from `seed` (splitmix64), zero biases. */
vct_status vct_mlp_create(int32_t device, uint64_t seed, vct_mlp** out);
vct_status vct_mlp_destroy(vct_mlp* mlp);
/* Host copies of the packed parameters (set also resets the Adam state);
 * get synchronises `stream` and reports VCT_ERR_TIMEOUT if an earlier
 * training or inference launch gave up waiting for the tensor core. */
vct_status vct_mlp_set_params(vct_mlp* mlp, const float* params, int64_t count);
vct_status vct_mlp_get_params(vct_mlp* mlp, float* params, int64_t count, void* stream);
/* out_dev (n x 4, 16-byte aligned) = network(rows_dev). */
vct_status vct_mlp_forward(vct_mlp* mlp, const float* rows_dev, int64_t n, float* out_dev, void* stream);
/* grad_dev (VCT_MLP_PARAMS fp32) = d loss / d params and loss_dev (1 fp32,
 * may be NULL) for rows_dev and targets_dev (n x 3); parameters unchanged.
 * Synchronises `stream`. */
vct_status vct_mlp_gradients(vct_mlp* mlp, const float* rows_dev, const float* targets_dev, int64_t n,
                             float* grad_dev, float* loss_dev, void* stream);
/* One Adam step on the n rows index_dev[0..n) of rows_dev / targets_dev
 * (index_dev NULL: rows 0..n); loss_dev (may be NULL) receives the step's
 * loss before the update.  No synchronisation. */
vct_status vct_mlp_train_step(vct_mlp* mlp, const float* rows_dev, const float* targets_dev, const int32_t* index_dev,
                              int64_t n, const vct_adam* opt, float* loss_dev, void* stream);

/* Learned trace of a frame whose radiance chain is built (>= 5 levels).
 * Cheap features: per 4x4 pixel block (ceil(w/4) x ceil(h/4) blocks, row
 * major), at its first covered pixel, two 90-degree cones along
 * normalize(N +- T), each marched 8 steps (step s samples mip level s + 1,
 * 2^s voxels out) and composited front to back; the accumulated RGBA after
 * levels 2, 4, 6 and 8 are 4 x 4 features per cone: 32 BF16 values, 64 bytes
 * per block, 16-byte aligned. */
#define VCT_LEARNED_CHEAP_FEATURES 32
vct_status vct_learned_features(vct_ctx* ctx, const vct_gbuffer* gbuffer, const float eye[3], uint16_t* features_dev,
                                void* stream);
/* Feature rows (n x 42 fp32) of the listed pixels (index y * width + x):
 * the 32 cheap features of the pixel's block, unit normal N, eye distance /
 * volume extent, albedo, and the near-field radiance RGB (one trilinear
 * sample of mip level 1 at position + 2 N / dim, where the diffuse cones
 * take their first sample; zero outside the volume); all zero for
 * background.  Every value is BF16-representable. */
vct_status vct_learned_rows(vct_ctx* ctx, const vct_gbuffer* gbuffer, const float eye[3],
                            const uint16_t* features_dev, const int32_t* pixels_dev, int64_t n, float* rows_dev,
                            void* stream);
/* The plain 16-cone irradiance (the learned path's target and fallback):
 * 16 cones of equal solid angle (aperture 2 acos(15/16)) on a Fibonacci
 * hemisphere around the normal, cosine weighted, 24 steps, bias / initial
 * height / LOD offset of the diffuse cones; float4 per pixel (rgb, 0). */
vct_status vct_trace_reference16(vct_ctx* ctx, const vct_gbuffer* gbuffer, const float eye[3],
                                 float* irradiance_dev, void* stream);
typedef struct vct_learned_stats {
    int32_t tiles;           /* 16 x 16 pixel tiles */
    int32_t fallback_tiles;  /* tiles re-traced with the 16-cone reference */
    float mean_tile_error;   /* mean estimated relative L2 error per tile, each capped at 1 (-1: no probes) */
    float max_tile_error;
} vct_learned_stats;
/* Learned irradiance: cheap features, the network on every pixel, then per
 * 16 x 16 tile an error estimate (16-cone irradiance at 4 probe pixels vs the
 * network, relative L2) and the 16-cone trace of every tile whose estimate
 * exceeds `threshold` (INFINITY: no probes, no fallback).  stats (may be
 * NULL) synchronises `stream`. */
vct_status vct_learned_trace(vct_ctx* ctx, vct_mlp* mlp, const vct_gbuffer* gbuffer, const float eye[3],
                             float threshold, float* irradiance_dev, vct_learned_stats* stats, void* stream);
/* Learned irradiance with a per-pixel fallback: cheap features and the
 * network on every pixel as in vct_learned_trace; then every covered pixel
 * whose error estimate (the network's fourth output) exceeds `threshold`
 * times the root-mean-square of the network's irradiance over the frame's
 * covered pixels is listed and re-traced with the 16-cone reference
 * (INFINITY: no fallback).  fallback_pixels (host, may be NULL) receives the
 * number of re-traced pixels and synchronises `stream`. */
vct_status vct_learned_trace_pixels(vct_ctx* ctx, vct_mlp* mlp, const vct_gbuffer* gbuffer, const float eye[3],
                                    float threshold, float* irradiance_dev, int64_t* fallback_pixels,
                                    void* stream);

/* ---- voxelisation without allocation ---------------------------------- */
/* No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (a host application whose device memory is all reserved up front by its
 * own allocator, a plugin in a process whose CUDA memory pool belongs to
 * someone else, or a frame loop that must not allocate): vct_voxelize
 * (accumulate + normalise) into volumes the caller owns, with no context and
 * no device allocation by this library or anything it calls.  Its scratch
 * (accumulator records, occupancy mask, work-distribution arrays, counters)
 * is one fixed __device__ array of about 9 MiB that every GPU that loads the
 * library keeps until the process exits.
 *  - cfg->voxel_dim <= VCT_STATIC_MAX_DIM and tris->count <=
 *    VCT_STATIC_MAX_TRIANGLES, otherwise VCT_ERR_INVALID_ARGUMENT.
 *  - color_dev, normal_dev, radiance_dev: dim^3 RGBA16F voxels each
 *    (8 bytes per voxel, x fastest), 32-byte aligned; radiance_dev receives
 *    level 0 as transferVoxels.comp seeds it (and is read first when the
 *    temporal filter is on).
 *  - Runs on the current CUDA device, which must be cfg->device (checked;
 *    this call never changes the current device).  The first call on a device looks up
 *    the array's device address (cudaGetSymbolAddress) for that device; make
 *    that first call before any stream capture.
 *  - With CUDA's lazy module loading (the default since CUDA 12.2) the array
 *    comes into being at that first call on each device: the driver then
 *    allocates its ~9 MiB.  Make the first call before reserving the rest of
 *    the device's memory, or run with CUDA_MODULE_LOADING=EAGER so that the
 *    array is allocated when the context is created.  Later calls allocate
 *    nothing.
 *  - The address looked up at the first call is kept for the life of the
 *    process: do not use this entry point across a cudaDeviceReset (or any
 *    other tear-down of the device's primary context).
 *  - All calls share the one array: calls whose work overlaps on the GPU
 *    (different streams, or different host threads) race.  Each call clears
 *    the parts of the array that must start at zero.
 *  - stats (host pointer) may be NULL; when given, the call synchronises
 *    `stream` and returns the VoxelizeInfo counters of this call.  While
 *    `stream` is being captured, stats must be NULL (VCT_ERR_INVALID_ARGUMENT
 *    otherwise, before any work is enqueued). */
#define VCT_STATIC_MAX_DIM 64
#define VCT_STATIC_MAX_TRIANGLES 16384
vct_status vct_voxelize_static(const vct_config* cfg, const vct_params* params,
                               const vct_triangles* tris, const vct_light* lights,
                               int32_t n_lights, const vct_shadow_desc* shadow,
                               uint16_t* color_dev, uint16_t* normal_dev,
                               uint16_t* radiance_dev, vct_stats* stats, void* stream);

/* ---- frame set-up (not part of the timed path) ------------------------ */
/* Depth-only render of the scene from the light (the reference's shadow
 * pass, src/Application.cpp:213-233): fp32 depth in [0,1], cleared to 1. */
vct_status vct_render_shadowmap(const vct_triangles* tris, const float ls[16],
                                float* depth_dev, int32_t width, int32_t height,
                                void* stream);
/* Camera G-buffer (world position, normal, albedo) with a depth test.
 * `keys_dev` is caller scratch of width*height uint64. */
vct_status vct_render_gbuffer(const vct_triangles* tris, const float view_proj[16],
                              const float eye[3], const float inv_view_proj[16],
                              int32_t width, int32_t height, unsigned long long* keys_dev,
                              float* position_dev, float* normal_dev, float* albedo_dev,
                              void* stream);

#ifdef __cplusplus
}
#endif

#endif /* VCT_H */
