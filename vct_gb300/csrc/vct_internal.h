// Internal declarations shared by the C ABI (capi.cpp) and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/vct.h"

#ifdef __CUDACC__
#define VCT_HD __host__ __device__
#else
#define VCT_HD
#endif

namespace vct {

struct f3 {
    float x, y, z;
};

// The software cone sampler reads a private copy of the radiance mip chain in
// which every level of side S is stored as (S+2)^3 voxels: the level plus a
// one-voxel shell of zeros (the GL clamp-to-border colour), so that any
// trilinear footprint of a position in [0,1]^3 lies inside the array.
// Each level starts at an odd texel offset: with rows of an even number of
// 16-byte texels, the interior of every row then starts on a 32-byte sector,
// and the resolve's rows of 16 texels fill whole sectors instead of sharing
// one with the border or the neighbouring brick.  Offset (in texels) of
// padded level l:
VCT_HD inline long long padded_level_offset(int N, int l) {
    long long off = 1;
    for (int i = 0; i < l; ++i) {
        const long long p = (N >> i) + 2;
        off += p * p * p;
        off += (off & 1) ? 0 : 1;
    }
    return off;
}

// Voxel warping (VCT_WARP_*): the texture mode's map is 32^3 RGBA16 unorm
// texels, x fastest, read through its fp32 copy (c / 65535 per channel); the
// analytic mode warps about the eye's volume coordinate; the perspective mode
// projects world positions with `pv` (volume coordinates are first mapped
// back to world space with vmin, vcenter and ext = vmax - vmin).
struct WarpDev {
    int mode;
    const float4* mapf;
    f3 eye_tc;
    float pv[16];
    f3 vmin, vcenter, ext;
};

struct LightDev {
    f3 position;
    f3 direction;
    f3 color;
    float range, intensity;
    uint32_t enabled, shadow_caster, type;
    // normalize(-direction) and 0.75 * range, computed on the host with the
    // same fp32 operations the shader evaluates per fragment.
    f3 neg_dir_n;
    float range075;
};

struct StatsDev {
    uint32_t total_voxel_fragments;
    uint32_t unique_voxels;
    uint32_t max_fragments_per_voxel;
    uint32_t error_flags;
};

struct AccumParams {
    const float* pos;
    const float* nrm;
    const float* albedo;
    long long ntri;
    int dim;
    int lighting;
    int axis_override;
    int nlights;
    LightDev lights[VCT_MAX_LIGHTS];
    float mvp[48];
    float ls[16];
    const float* shadowmap;
    int sw, sh;
    uint32_t* acc;  // accumulator records, kAccWords uint32 per voxel
    uint32_t* occ;  // occupancy bit mask, one bit per voxel
    uint32_t* carry;  // tessellation voxeliser: crossings of 2^32 per record field (kCarrySlots entries), or nullptr
    uint32_t* brick_exact;  // with `carry`: per 16^3 brick, set by the carry pass for the bricks it rewrote
    StatsDev* stats;
    int num_sms;
    int unit_log2;      // log2 of the candidate pixels per work unit (whole rows of the bounding box)
    int blocks_per_sm;  // raster CTAs per SM (1..3)
    WarpDev warp;
    f3 vmin, vcenter, ext;  // voxelLinearPosition of the tessellation voxeliser
    float max_tess_level;   // GL_MAX_TESS_GEN_LEVEL
    // Work distribution scratch (sized for ntri; see voxelize.cu).
    uint4* tri_rec;          // 3 x uint4 per triangle
    uint32_t* tri_units;     // work units per triangle
    uint32_t* tri_scan;      // block-local exclusive scan of tri_units
    uint32_t* block_off;     // exclusive scan of per-block unit totals (+ total at [nblocks])
};

// Several independent scenes processed by one launch per stage: `off` is the
// exclusive prefix sum (n + 1 entries, in device memory) of the scenes' work
// items (triangles, shadow texels, bricks or pixel tiles) and `p` their
// parameters.  A global work index w belongs to scene s with
// off[s] <= w < off[s+1].
template <class Params>
struct SceneBatch {
    const Params* p;
    const long long* off;
    int n;
};

// Voxeliser work distribution over all triangles of one launch (one scene, or
// the concatenated triangles of a batch).
struct VoxWork {
    uint4* tri_rec;
    uint32_t* tri_units;
    uint32_t* tri_scan;
    uint32_t* block_off;
    long long ntri;
    int unit_log2;
};

constexpr int kSetupThreads = 256;  // triangles per setup block
constexpr long long align256(long long b) { return (b + 255) & ~255LL; }
// Scratch bytes the voxeliser needs for `ntri` triangles: a 48-byte setup
// record, a unit count and a scan entry per triangle, one offset per block
// (+ the total), then an 8-byte work counter.
constexpr long long accumulate_scratch_bytes(long long ntri) {
    return align256(ntri * 48) + align256(ntri * 4) * 2 +
           align256(((ntri + kSetupThreads - 1) / kSetupThreads + 2) * 4 + 8);
}
// Carves the scratch buffer into the AccumParams work arrays.
void accumulate_bind_scratch(AccumParams& P, void* scratch);

// One 32-byte accumulator record per voxel: {count, r, g, b, nx, ny, nz, 0}.
// Sums are of 16-bit fixed point (round(x * 65535)); they are updated as
// four 64-bit atomics whose low halves (count, g, nx, nz) never carry into
// the high halves while a voxel receives fewer than VCT_MAX_EXACT_FRAGMENTS
// fragments, so the record then equals seven independent 32-bit sums.  The
// last word's high half only ever receives nz's carries, so {nz, pad} is
// nz's exact 64-bit sum.
constexpr int kAccWords = 8;

// Record slot of voxel v = (z * N + y) * N + x (N = dim, a power of two of
// at least 16): bit 1 of x and bit 0 of y change places, so the four 32-byte
// records of each 128-byte line hold a 2 x 2 block in x and y instead of a
// run of four along x.  DRAM moves whole lines around the records of the
// occupied voxels, and a surface's occupied voxels fill more of each line in
// 2 x 2 blocks: on the 262,144-triangle 256^3 frame, 5.18 M records touch
// 1.99 M lines instead of 2.37 M.
VCT_HD inline long long record_slot(long long v, int N) {
    const long long d = ((v >> 1) ^ ((v & N) ? 1 : 0)) & 1;
    return v ^ (d * (N + 2));
}

// Exact sums past VCT_MAX_EXACT_FRAGMENTS (the tessellation voxeliser, whose
// slivers put up to ~10^5 points into one voxel): every 64-bit add returns
// the word's old value, from which the adder sees whether its low field
// crossed 2^32 (a carry into the high field) and whether the high field
// wrapped.  Such crossings (rare: only voxels past 65,536 points have them)
// are counted per voxel in an open-addressing table of kCarrySlots entries
// {voxel + 1, r wraps, g carries, b wraps, nx carries, ny wraps, 0, 0}; nz's
// carries need no count (they accumulate in the last word's high half), and
// every voxel past 65,536 points is listed, crossing or not.  After the voxeliser, a carry pass rebuilds each listed voxel's six
// 64-bit sums and rewrites its record: the sums' float values (the value
// the resolve divides) in the six sum fields and bit 31 set in the count;
// it flags the voxel's 16^3 brick, which a second instantiation of the
// resolve handles (the common one skips it).
// A table with no free slot within kCarryProbes probes raises
// VCT_STATS_COUNT_OVERFLOW.
constexpr int kCarrySlotsLog2 = 16, kCarrySlots = 1 << kCarrySlotsLog2, kCarryProbes = 64;
constexpr long long kCarryBytes = (long long)kCarrySlots * 8 * 4;
constexpr int kCarryEvents = 5;

struct NormalizeParams {
    int dim;
    float opacity;
    int temporal;
    float decay;
    uint32_t* acc;
    const uint32_t* occ;
    const uint32_t* brick_exact;  // per 16^3 brick: the carry pass rewrote one of its records; nullptr: no carry pass
    uint2* color;     // level 0 of the colour volume
    uint2* normal;
    uint2* radiance;  // level 0 of the radiance chain
    StatsDev* stats;
    int num_sms;
};

struct InjectParams {
    int dim;
    const float* shadowmap;
    int sw, sh;
    int nx, ny;  // texel threads that pass the shader's bounds test
    float ls_inverse[16];
    f3 vmin, vmax, vcenter;
    f3 light_vox;  // voxelIndex(lightPos)
    f3 light_int;
    int lighting, dilate;
    const uint2* color;
    const uint2* normal;
    uint2* radiance;
    uint32_t* lit;  // fused path: bit mask of voxels the shader would store to
    WarpDev warp;
    f3 light_tc;    // voxelLinearPosition(lightPos): light_vox is warped on the device when warping
    f3 light_pos;   // lightPos (the perspective warp projects the world position)
    int temporal;   // temporalFilterRadiance: relit voxels mix with the radiance seeded this frame
    float decay;
};

// Fused normalisation + injection resolve + first mip levels (vct_frame).
struct ResolveParams {
    NormalizeParams norm;
    int fused;  // 0: plain normalisation (transferVoxels.comp)
    int lighting, dilate;
    f3 light_vox, light_int;
    const uint32_t* lit;
    uint2* radiance_levels[5];  // levels 0..4 of the radiance chain
    int mip_levels;             // number of levels below 0 to write from the brick (<= 4)
    cudaSurfaceObject_t surf[5];  // texture-unit copy of levels 0..4 (0 = none)
    float4* pad_levels[5];        // bordered fp32 copy of levels 0..4 (nullptr = none)
    WarpDev warp;
    f3 light_tc;
    f3 light_pos;
};

struct MipLevels {
    uint2* level[VCT_MAX_LEVELS];
    cudaSurfaceObject_t surf[VCT_MAX_LEVELS];  // optional texture-unit copy (0 = none)
    float4* pad[VCT_MAX_LEVELS];               // optional bordered fp32 copy (nullptr = none)
    int dim;
    int levels;
    int first;  // mip tail: the level the remaining levels are built from
};

struct TraceParams {
    const float4* gpos;
    const float4* gnrm;
    const float4* galb;
    int width, height;
    float4* irradiance;
    float4* specular;
    float4* color;
    unsigned long long* samples;
    const float4* pchain;  // bordered fp32 chain (software trilinear, nearest-level magnification)
    int dim, levels;
    f3 vmin, vmax, vcenter, eye;
    vct_cone_settings diffuse, specular_cone;
    int enable_indirect, enable_reflections, draw_occlusion, enable_postprocess;
    float ambient_scale, reflect_scale, max_distance;
    int ref_tbn_quirk;
    int filter;  // VCT_FILTER_*
    cudaTextureObject_t tex;
    // Pixel tile of one 256-thread CTA (tile_w x tile_h) and of one warp
    // (warp_w x 32/warp_w), as log2.
    int tile_w_log2, tile_h_log2, warp_w_log2;
    WarpDev warp;
};

// Several viewpoints of one volume traced by one launch (vct_trace_views):
// the views' parameters travel in kernel-parameter space, `off` is the
// exclusive prefix sum of their pixel tiles.
constexpr int kMaxViews = 8;
struct ViewSet {
    TraceParams p[kMaxViews];
    long long off[kMaxViews + 1];
    int n;
};

struct ShadowRasterParams {
    const float* pos;
    long long ntri;
    float ls[16];
    unsigned int* depth_bits;
    int w, h;
    int num_sms;
};

struct GbufferRasterParams {
    const float* pos;
    const float* nrm;
    const float* albedo;
    long long ntri;
    float vp[16];
    float ivp[16];
    f3 eye;
    unsigned long long* keys;
    float4* gpos;
    float4* gnrm;
    float4* galb;
    int w, h;
    int num_sms;
};

// Counts kernel launches (vct_launch_count).
void note_launches(int n);

// Host helpers of the C ABI (capi.cpp), shared with the other entry points.
vct_status set_error(vct_status s, const char* msg);
void voxel_mvp_host(const vct_config& c, float out[48]);
vct_status validate_voxelize_inputs(const vct_config* cfg, const vct_params* p, const vct_triangles* t,
                                    const vct_light* lights, int n, const vct_shadow_desc* shadow, bool* need_shadow);
// Fills every input field of AccumParams (not the accumulators, stats or scratch).
void fill_accum_inputs(const vct_config& cfg, const vct_params& prm, const float mvp[48], const vct_triangles* t,
                       const vct_light* lights, int n, const vct_shadow_desc* sh, AccumParams& P);

void launch_accumulate(const AccumParams& P, cudaStream_t s);
// The warp map's 32^3 occupancy voxelisation into P.occ (P.dim = 32, unwarped):
// one thread per triangle, no scratch.
void launch_occupancy(const AccumParams& P, cudaStream_t s);
// The tessellation voxeliser into the same accumulators (testTesselation.tesc/.tese).
void launch_tesselate(const AccumParams& P, cudaStream_t s);
void launch_normalize(const NormalizeParams& P, cudaStream_t s);
void launch_inject(const InjectParams& P, cudaStream_t s);
void launch_inject_mark(const InjectParams& P, cudaStream_t s);
void launch_resolve(const ResolveParams& P, cudaStream_t s);
// Builds levels [first+1, levels) from level `first`.
void launch_mips(const MipLevels& M, int first, cudaStream_t s);
void launch_trace(const TraceParams& P, cudaStream_t s);
// Sampler throughput microbenchmark (vct_sampler_rate): blocks x 256 threads x iters samples.
void launch_sampler_rate(const TraceParams& P, int filter, int blocks, int iters, float* sink, cudaStream_t s);
void launch_shadow_raster(const ShadowRasterParams& P, cudaStream_t s);
void launch_gbuffer_raster(const GbufferRasterParams& P, cudaStream_t s);
void launch_fill_u32(uint32_t* p, uint32_t v, long long n, cudaStream_t s);

// Batched frame stages: one launch covers the work of every scene.
int accumulate_batch_max_scenes();
void launch_accumulate_batch(const SceneBatch<AccumParams>& B, const VoxWork& W, int num_sms, int blocks_per_sm,
                             cudaStream_t s);
void launch_tesselate_batch(const SceneBatch<AccumParams>& B, const VoxWork& W, int num_sms, cudaStream_t s);
void launch_inject_mark_batch(const SceneBatch<InjectParams>& B, long long ntexels, cudaStream_t s);
void launch_resolve_batch(const SceneBatch<ResolveParams>& B, long long nbricks, bool exact, cudaStream_t s);
void launch_mip_tail_batch(const SceneBatch<MipLevels>& B, cudaStream_t s);
// A device range of 32-bit words to zero (p 16-byte aligned, as cudaMalloc returns).
struct ClearRange {
    uint32_t* p;
    long long words;
};
// Zeroes n ranges (a device array) in one launch; max_words sizes the grid.
void launch_clear_ranges(const ClearRange* ranges, int n, long long max_words, cudaStream_t s);
long long trace_tiles(int width, int height, int tile_w_log2, int tile_h_log2);
void launch_trace_batch(const SceneBatch<TraceParams>& B, int filter, long long tiles, cudaStream_t s);
void launch_trace_views(const ViewSet& V, int filter, cudaStream_t s);
// ------------------------------------------------------------- learned path
// MLP 42-64-64-64-4: irradiance RGB and the network's estimate of its own
// error.  Packed fp32 parameters: W1[64][42] b1[64] W2[64][64] b2[64]
// W3[64][64] b3[64] W4[4][64] b4[4].
constexpr int kMlpIn = 42, kMlpInPad = 48, kMlpHidden = 64, kMlpOut = 4, kMlpOutPad = 16;
constexpr int kOffW1 = 0, kOffB1 = 2688, kOffW2 = 2752, kOffB2 = 6848, kOffW3 = 6912, kOffB3 = 11008,
              kOffW4 = 11072, kOffB4 = 11328, kMlpParams = 11332;
// Weight of the error-estimate term in the training loss (relative to the
// mean squared error of the irradiance).
constexpr float kMlpConfidenceWeight = 0.5f;
// BF16 operand images in the tensor core's shared-memory tile layout:
// forward B operands W1 (64 x 48), W2, W3 (64 x 64), W4 (16 x 64), then the
// transposes used by the backward pass W4^T (64 x 16), W3^T, W2^T (64 x 64).
constexpr int kImgW1 = 0, kImgW2 = 6144, kImgW3 = 14336, kImgW4 = 22528, kImgFwd = 24576, kImgW4t = 24576,
              kImgW3t = 26624, kImgW2t = 34816, kImgAll = 43008;
// Bias vector padded for the kernels: b1 | b2 | b3 | b4 (16).
constexpr int kBiasPad = 208;
// Quarter-resolution cheap trace: 2 cones x 4 levels x RGBA, BF16.
constexpr int kCheapFeatures = 32;
// Per-tile error probes of the learned trace and its 16 x 16 tiles.
constexpr int kProbes = 4, kLearnTile = 16;

struct MlpDev {
    float* params;  // fp32 master
    float* grad;
    float* m;
    float* v;
    uint8_t* img;   // kImgAll bytes
    float* bias;    // kBiasPad floats
    float* loss;
};

struct LearnedParams {
    TraceParams T;             // G-buffer, eye, volume, software sampler chain
    const uint16_t* qfeat;     // quarter-res features, kCheapFeatures bf16 per quarter pixel
    int wq, hq;
    float depth_scale;         // 1 / volume extent
    float dirs16[16][4];       // 16-cone set in the (T, B, N) frame: xyz + weight
    vct_cone_settings ref_cone;
    const uint8_t* img;
    const float* bias;
    const float* rows;         // feature rows (vct_mlp_forward), or nullptr: pixels of the frame
    long long n;               // rows or pixels
    float* out_rows;           // n x 3
    float4* out;               // irradiance per pixel
    const int* pixels;         // rows kernel: pixel indices
    float* rows_out;           // rows kernel: n x 42
    float threshold;           // per-tile relative error bound, or the per-pixel bound relative to the frame's RMS
    float* tile_err;           // per 16x16 tile
    uint32_t* list;            // fallback tiles or pixels; their count at `count`
    uint32_t* count;
    float* est;                // per pixel: the network's error estimate (-1: background), or nullptr
    float* frame_sums;         // sum of squared network irradiance over covered pixels, covered pixels
    uint32_t* status;
};

struct TrainParams {
    MlpDev mlp;
    const float* rows;     // n x 42
    const float* targets;  // n x 3
    const int* index;      // optional permutation of rows
    long long n;
    float scale;           // 2 / (3 n): d loss / d irradiance output = scale * (output - target)
    float conf_scale;      // 2 w / n: d loss / d error estimate = conf_scale * (estimate - |output - target|)
    uint32_t* status;
};

void launch_learned_features(const LearnedParams& P, cudaStream_t s);
void launch_learned_rows(const LearnedParams& P, cudaStream_t s);
void launch_mlp_infer(const LearnedParams& P, int num_sms, cudaStream_t s);
void launch_learned_probe(const LearnedParams& P, cudaStream_t s);
void launch_trace16(const LearnedParams& P, bool listed, int num_sms, cudaStream_t s);
// The per-pixel fallback after inference with `est` set: the list of flagged
// pixels, then their 16-cone trace.
void launch_trace16_pixels(const LearnedParams& P, cudaStream_t s);
void launch_mlp_train(const TrainParams& P, int num_sms, cudaStream_t s);
void launch_mlp_update(const MlpDev& M, int step, float lr, float beta1, float beta2, float eps, int update,
                       cudaStream_t s);

// Injection through the lit mask (marked by launch_inject_mark): every marked
// voxel's store computed once from the radiance seeded this frame.
void launch_inject_apply(const InjectParams& P, cudaStream_t s);
// temporalRadianceFilter.comp: radiance level 0 *= decay.
void launch_decay(uint2* radiance, long long nv, float decay, cudaStream_t s);

// Rigid actors: world = model * local for positions, mat3(transpose(inverse(
// model))) * local for normals (voxelize.vert), per triangle range.
constexpr int kMaxActors = 64;
struct ActorsDev {
    const float* src_pos;
    const float* src_nrm;
    float* dst_pos;
    float* dst_nrm;
    long long start[kMaxActors], end[kMaxActors];  // ascending, non-overlapping triangle ranges
    float model[kMaxActors][16];                    // column-major
    float normal[kMaxActors][9];      // column-major 3x3
    int n;
};
void launch_transform_actors(const ActorsDev& A, cudaStream_t s);

// phong.frag's composite with direct lighting (vct_shade).
struct ShadeParams {
    const float4* gpos;
    const float4* gnrm;
    const float4* galb;
    const float4* irradiance;  // nullptr: no indirect term
    const float4* specular;
    float4* color;
    int width, height;
    f3 eye;
    int nlights;
    LightDev lights[VCT_MAX_LIGHTS];
    const float* shadowmap;
    int sw, sh;
    float ls[16];
    int cooktorrance, enable_diffuse, enable_specular, enable_indirect, enable_reflections, draw_occlusion,
        enable_postprocess;
    float roughness, metallic, shininess, ambient_scale, reflect_scale;
};
void launch_shade(const ShadeParams& P, cudaStream_t s);

// Warp map of VCT_WARP_TEXTURE from a 32^3 occupancy bit mask.
void launch_warpmap(const uint32_t* occ32, float high, float low, uint16_t* map, float4* mapf, cudaStream_t s);
// The warp map of one scene: its 32^3 occupancy mask, the high and low cell
// widths, the RGBA16 unorm map and its bordered fp32 copy ((32+2)^3).
struct WarpmapArgs {
    const uint32_t* occ;
    float high, low;
    uint16_t* map;  // nullptr: the scene builds no map
    float4* mapf;
};
// One map per scene of a batch (a device array of n arguments).
void launch_warpmap_batch(const WarpmapArgs* args, int n, cudaStream_t s);
// The 32^3 occupancy voxelisation of every scene of a batch whose occupancy
// parameters name a mask (occ), over all the batch's triangles.
void launch_occupancy_batch(const SceneBatch<AccumParams>& B, long long ntri, cudaStream_t s);

// Tensor-core GEMM check: D (128 x n, fp32) = A (128 x k) B^T (n x k), bf16.
// One bounded mbarrier wait that nothing completes: sets status to 1 after limit_ns.
void launch_wait_probe(uint32_t* status, unsigned long long limit_ns, cudaStream_t s);
void launch_umma_check(const uint16_t* A, const uint16_t* B, int K, int N, int swap, float* D, uint32_t* status,
                       cudaStream_t s);
// Copies every level of a linear chain into the interior of the bordered chain.
void launch_pad_copy(const uint2* chain, float4* pchain, int dim, int levels, cudaStream_t s);

}  // namespace vct
