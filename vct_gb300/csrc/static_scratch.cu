// vct_voxelize_static: voxelisation that allocates no device memory.
//
// Some callers of this library cannot call cudaMalloc: code that runs under
// an allocator it does not control (a host application that pre-reserves all
// device memory at start-up and hands out sub-ranges, a plugin inside a
// process whose CUDA memory pool is owned elsewhere), or code that must not
// allocate once a frame loop has started.  For them this entry point
// voxelises a scene into output volumes the caller already owns, and keeps
// everything else it needs (the 32-byte accumulator records, the occupancy
// mask, the triangle set-up records and scans of the work distribution, and
// the VoxelizeInfo counters) in one file-scope __device__ array of fixed
// size.  Every GPU that loads the library holds that array until the process
// exits.
//
// Limits: grids up to VCT_STATIC_MAX_DIM^3 voxels and up to
// VCT_STATIC_MAX_TRIANGLES triangles (about 9 MiB of device memory).
#include <mutex>

#include "vct_device.cuh"

namespace vct {

namespace {

constexpr long long kMaxVoxels = (long long)VCT_STATIC_MAX_DIM * VCT_STATIC_MAX_DIM * VCT_STATIC_MAX_DIM;
constexpr long long kRecordBytes = align256(kMaxVoxels * kAccWords * 4);
constexpr long long kOccBytes = align256((kMaxVoxels + 31) / 32 * 4);
constexpr long long kStatsBytes = align256(sizeof(StatsDev));
constexpr long long kWorkBytes = accumulate_scratch_bytes(VCT_STATIC_MAX_TRIANGLES);
constexpr long long kScratchBytes = kRecordBytes + kOccBytes + kStatsBytes + kWorkBytes;

// The shared scratch.  Host code must not use this name as a device address:
// on the host it is only a stand-in symbol, so the device address is looked
// up with cudaGetSymbolAddress (per device) and passed to the kernels.
static __device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_static_scratch on the current device `dev`, looked up
// on the first call made on that device (with lazy module loading, that
// lookup is also when the driver loads this file's module and allocates the
// array).  The cached address is not invalidated: it does not survive a
// cudaDeviceReset of that device.
vct_status scratch_address(int dev, char** out) {
    if (dev < 0 || dev >= kMaxDevices) return set_error(VCT_ERR_UNSUPPORTED, "device ordinal too large");
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return set_error(VCT_ERR_CUDA, "cudaGetSymbolAddress of the static scratch failed");
        }
        g_scratch_addr[dev] = p;
    }
    *out = static_cast<char*>(g_scratch_addr[dev]);
    return VCT_OK;
}

}  // namespace

}  // namespace vct

using namespace vct;

extern "C" vct_status vct_voxelize_static(const vct_config* cfg, const vct_params* params, const vct_triangles* tris,
                                          const vct_light* lights, int32_t n_lights, const vct_shadow_desc* shadow,
                                          uint16_t* color_dev, uint16_t* normal_dev, uint16_t* radiance_dev,
                                          vct_stats* stats, void* stream) {
    bool need_shadow = false;
    vct_status s = validate_voxelize_inputs(cfg, params, tris, lights, n_lights, shadow, &need_shadow);
    if (s != VCT_OK) return s;
    if (params->warp_mode != VCT_WARP_NONE)
        return set_error(VCT_ERR_UNSUPPORTED, "vct_voxelize_static: voxel warping needs a context (vct_voxelize)");
    if (params->voxelize_tesselation)
        return set_error(VCT_ERR_UNSUPPORTED, "vct_voxelize_static: the tessellation voxeliser needs a context");
    if (cfg->voxel_dim > VCT_STATIC_MAX_DIM)
        return set_error(VCT_ERR_INVALID_ARGUMENT, "vct_voxelize_static: voxel_dim exceeds VCT_STATIC_MAX_DIM (64)");
    if (tris->count > VCT_STATIC_MAX_TRIANGLES)
        return set_error(VCT_ERR_INVALID_ARGUMENT,
                         "vct_voxelize_static: triangle count exceeds VCT_STATIC_MAX_TRIANGLES (16384)");
    if (!color_dev || !normal_dev || !radiance_dev)
        return set_error(VCT_ERR_INVALID_ARGUMENT, "vct_voxelize_static: output volumes must be non-NULL");
    for (const void* p : {(const void*)color_dev, (const void*)normal_dev, (const void*)radiance_dev})
        if (reinterpret_cast<uintptr_t>(p) % 32 != 0)  // the resolve writes 4 voxels per 32-byte store
            return set_error(VCT_ERR_INVALID_ARGUMENT, "vct_voxelize_static: output volumes must be 32-byte aligned");

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return set_error(VCT_ERR_CUDA, "vct_voxelize_static: no current CUDA device");
    }
    if (dev != cfg->device)
        return set_error(VCT_ERR_INVALID_ARGUMENT, "vct_voxelize_static: cfg->device must be the current device");
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (stats) {  // the counters' read-back synchronises the stream, which a capture forbids
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
            cudaGetLastError();
            return set_error(VCT_ERR_CUDA, "vct_voxelize_static: cudaStreamIsCapturing failed");
        }
        if (cs != cudaStreamCaptureStatusNone)
            return set_error(VCT_ERR_INVALID_ARGUMENT,
                             "vct_voxelize_static: stats must be NULL while the stream is being captured");
    }
    char* base = nullptr;
    if ((s = scratch_address(dev, &base)) != VCT_OK) return s;
    const long long nv = (long long)cfg->voxel_dim * cfg->voxel_dim * cfg->voxel_dim;
    uint32_t* acc = reinterpret_cast<uint32_t*>(base);
    uint32_t* occ = reinterpret_cast<uint32_t*>(base + kRecordBytes);
    StatsDev* st_dev = reinterpret_cast<StatsDev*>(base + kRecordBytes + kOccBytes);
    void* work = base + kRecordBytes + kOccBytes + kStatsBytes;

    // The array keeps whatever the previous call left; the records, the mask
    // and the counters must start at zero.
    cudaError_t e = cudaMemsetAsync(acc, 0, (size_t)(nv * kAccWords * 4), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(occ, 0, (size_t)((nv + 31) / 32 * 4), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(st_dev, 0, sizeof(StatsDev), st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(VCT_ERR_CUDA, "vct_voxelize_static: clearing the static scratch failed");
    }

    int num_sms = 0;
    cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
    float mvp[48];
    voxel_mvp_host(*cfg, mvp);
    AccumParams A;
    fill_accum_inputs(*cfg, *params, mvp, tris, lights, n_lights, need_shadow ? shadow : nullptr, A);
    A.acc = acc;
    A.occ = occ;
    A.stats = st_dev;
    A.num_sms = num_sms;
    accumulate_bind_scratch(A, work);
    launch_accumulate(A, st);

    NormalizeParams N;
    N.dim = cfg->voxel_dim;
    N.opacity = params->voxel_set_opacity;
    N.temporal = params->temporal_filter;
    N.decay = params->temporal_decay;
    N.acc = acc;
    N.occ = occ;
    N.brick_exact = nullptr;  // the rasterising voxeliser only: no carry pass
    N.color = reinterpret_cast<uint2*>(color_dev);
    N.normal = reinterpret_cast<uint2*>(normal_dev);
    N.radiance = reinterpret_cast<uint2*>(radiance_dev);
    N.stats = st_dev;
    N.num_sms = num_sms;
    launch_normalize(N, st);
    if ((e = cudaGetLastError()) != cudaSuccess)
        return set_error(VCT_ERR_CUDA, cudaGetErrorString(e));

    if (stats) {
        StatsDev h;
        e = cudaMemcpyAsync(&h, st_dev, sizeof h, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return set_error(VCT_ERR_CUDA, cudaGetErrorString(e));
        }
        stats->total_voxel_fragments = h.total_voxel_fragments;
        stats->unique_voxels = h.unique_voxels;
        stats->max_fragments_per_voxel = h.max_fragments_per_voxel;
        stats->error_flags = h.error_flags;
    }
    return VCT_OK;
}
