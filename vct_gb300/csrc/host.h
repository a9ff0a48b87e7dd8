// Host-side internals shared by the C ABI translation units (capi.cpp,
// batch.cpp, learned_capi.cpp): the context object, error reporting,
// argument validation and the fillers of the kernels' parameter structs.
#pragma once

#include <string>

#include "vct_internal.h"

struct vct_ctx {
    vct_config cfg;
    vct_params params;
    int dim = 0, levels = 0, color_levels = 1, device = 0, num_sms = 0;
    long long nv = 0;
    uint32_t* acc = nullptr;  // accumulator records (kAccWords uint32 per voxel)
    uint32_t* occ = nullptr;  // occupancy bit mask
    uint32_t* lit = nullptr;
    uint2* color = nullptr;     // colour chain (color_levels levels)
    uint2* normal = nullptr;    // one level
    uint2* radiance = nullptr;  // radiance chain (levels levels)
    long long level_off[VCT_MAX_LEVELS] = {};
    vct::StatsDev* stats = nullptr;
    bool stats_reset_pending = true;
    bool radiance_ready = false;  // level 0 written since the last accumulate
    bool mips_ready = false;
    float mvp[48];
    cudaMipmappedArray_t tex_array = nullptr;
    cudaTextureObject_t tex = 0;
    cudaSurfaceObject_t surf[VCT_MAX_LEVELS] = {};
    bool tex_ready = false;
    bool timers_on = false;
    bool timers_recorded = false;
    bool volume_timed = false;  // the last volume pass recorded ev[0..3]: a trace after it records ev[4]
    cudaEvent_t ev[5] = {};
    // vct_frame runs the shadow-map half of injection on `side`, concurrently
    // with the voxeliser: `fork` / `join` order it against the caller's stream.
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    void* vox_scratch = nullptr;  // voxeliser work-distribution arrays
    long long vox_scratch_bytes = 0;
    float4* pchain = nullptr;  // bordered fp32 radiance chain read by the software sampler
    bool pad_ready = false;   // pchain holds the current radiance chain
    // Levels [0, linear_stale) of the linear radiance chain were left to the
    // texture array by the last fused frame (sync_linear copies them back).
    int linear_stale = 0;
    vct_tuning tuning;        // launch shapes (vct_set_tuning / vct_autotune)
    void* learned = nullptr;  // learned-trace scratch (quarter-res features, tile errors, fallback list)
    size_t learned_bytes = 0;
    uint32_t* occ32 = nullptr;   // VCT_WARP_TEXTURE: 32^3 occupancy bit mask
    uint16_t* warpmap = nullptr; // VCT_WARP_TEXTURE: 32^3 RGBA16 unorm warp map
    float4* warpmap_f = nullptr; // its bordered fp32 copy read by the lookups ((32+2)^3)
    uint32_t* carry = nullptr;   // the tessellation voxeliser's carry table (kCarrySlots entries)
    uint32_t* brick_exact = nullptr;  // per 16^3 brick: flagged by the carry pass for the exact resolve
};

namespace vct {
namespace host {

extern thread_local std::string g_err;
vct_status fail(vct_status s, const std::string& msg);

#define VCT_CUDA(expr)                                                                      \
    do {                                                                                    \
        cudaError_t e_ = (expr);                                                            \
        if (e_ != cudaSuccess) return ::vct::host::fail(VCT_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define VCT_CHECK_LAUNCH(what)                                                               \
    do {                                                                                     \
        cudaError_t e_ = cudaGetLastError();                                                 \
        if (e_ != cudaSuccess) return ::vct::host::fail(VCT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Makes the context's device current for the duration of a call and
// restores the caller's device afterwards.
struct DeviceScope {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceScope(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) err = cudaSetDevice(dev);
    }
    ~DeviceScope() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

bool is_pow2(int v);
int ilog2(int v);
f3 to_f3(const float* p);
vct_status validate_config(const vct_config* c);
vct_status validate_params(const vct_params* p);
vct_status validate_tris(const vct_triangles* t);
vct_status validate_shadow(const vct_shadow_desc* s, bool needed);
vct_status validate_lights(const vct_light* lights, int n, bool* needs_shadow);
vct_status validate_gbuffer(const vct_gbuffer* g);
uint2* level_ptr(uint2* chain, const vct_ctx* ctx, int l);

void default_tuning(vct_tuning& t);
vct_status validate_tuning(const vct_tuning* t);
void apply_tuning(const vct_tuning& t, AccumParams& P);
void apply_tuning(const vct_tuning& t, TraceParams& P);

vct_status fill_accum(vct_ctx* ctx, const vct_triangles* t, const vct_light* lights, int n,
                      const vct_shadow_desc* sh, const float* eye, AccumParams& P);
void fill_norm(vct_ctx* ctx, NormalizeParams& P);
void fill_inject(vct_ctx* ctx, const vct_shadow_desc* s, const float* eye, InjectParams& P);
// Warp state of the context's parameters for an eye position (may be NULL
// unless the mode is VCT_WARP_ANALYTIC).
WarpDev warp_dev(const vct_ctx* ctx, const float* eye);
// VCT_WARP_TEXTURE: the 32^3 occupancy voxelisation of `A`'s triangles and
// the warp map built from it (A: the main pass's parameters, scratch bound).
bool filter_uses_texture(int filter);
bool filter_uses_bordered(int filter);
vct_status build_warpmap(vct_ctx* ctx, const AccumParams& A, cudaStream_t s);
MipLevels mip_levels(vct_ctx* ctx, uint2* chain, int levels);
vct_status ensure_texture(vct_ctx* ctx);
vct_status fill_trace(vct_ctx* ctx, const vct_gbuffer* g, const float eye[3], const vct_trace_out* out,
                      TraceParams& P);
// Makes the bordered fp32 chain of the software sampler current.
vct_status ensure_padded_chain(vct_ctx* ctx, cudaStream_t s);
// Makes every level of the linear radiance chain current (copies back the
// levels a fused frame left in the texture array).
vct_status sync_linear(vct_ctx* ctx, cudaStream_t s);

}  // namespace host
}  // namespace vct
