// Batched scenes (vct_batch_*) and the launch-shape autotuner of the C ABI
// (include/vct.h).
#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "host.h"

using namespace vct;
using namespace vct::host;

// ==================================================================== batches
// vct_batch: one context per scene, every frame stage one launch over all
// scenes.  Per-scene parameter structs and the work-offset tables of the
// launches travel in one blob: staged in pinned host memory, copied to the
// device with one stream-ordered copy per frame.
struct vct_batch {
    int n = 0, device = 0, num_sms = 0;
    std::vector<vct_ctx*> ctx;
    size_t off_accum = 0, off_inject = 0, off_resolve = 0, off_mips = 0, off_trace = 0, off_tables = 0, off_clear = 0;
    size_t off_occ = 0, off_wmap = 0;  // warp maps: occupancy parameters and map arguments per scene
    size_t blob_bytes = 0;
    char* d_blob = nullptr;
    char* h_blob = nullptr;        // staging of vct_batch_frame
    char* h_graph_blob = nullptr;  // staging read by the captured graph
    void* work = nullptr;          // voxeliser work arrays over all triangles
    long long work_bytes = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    vct_tuning tuning;
    cudaEvent_t ev[4] = {};  // voxeliser start/end, trace start/end (timers, autotuner)
    bool timers_on = false, timers_recorded = false;
    int graph_launches = 0;  // kernels in the captured graph
};

namespace {

size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }

struct BatchTotals {
    long long tris = 0, texels = 0, bricks = 0, tiles = 0;
    // The frame's clears, zeroed by one launch each: before the voxeliser
    // (statistics, lit masks; carry tables and brick flags of the tessellation
    // voxeliser; the occupancy masks of the warp maps) at [0, n_pre) of the blob's clear list, and after the resolve
    // (occupancy masks, for the next frame's accumulation) at [kClearPre n, +n).
    int n_pre = 0;
    long long max_pre = 0, max_post = 0;
    bool any_map = false;  // some scene builds a warp map (VCT_WARP_TEXTURE)
};

constexpr int kClearPre = 5;  // clear-list entries per scene before the voxeliser (one more after the resolve)

// Validates the scene descriptors and fills the staging blob `h` (parameter
// structs and prefix tables).  Allocates the voxeliser work arrays when the
// batch grew (never during a capture: `allow_alloc` false).
vct_status batch_stage(vct_batch* b, const vct_scene_desc* sc, int n, char* h, BatchTotals& tot, bool allow_alloc) {
    if (!sc || n != b->n) return fail(VCT_ERR_INVALID_ARGUMENT, "scene descriptors must match the batch's scene count");
    const int filter = b->ctx[0]->params.trace_filter;
    long long* tri_off = reinterpret_cast<long long*>(h + b->off_tables);
    long long* tex_off = tri_off + (n + 1);
    long long* brick_off = tex_off + (n + 1);
    long long* tile_off = brick_off + (n + 1);
    tot = BatchTotals();
    for (int i = 0; i < n; ++i) {
        vct_ctx* c = b->ctx[i];
        const vct_scene_desc& d = sc[i];
        vct_status s = validate_tris(&d.triangles);
        bool need_shadow = false;
        if (s == VCT_OK) s = validate_lights(d.lights, d.n_lights, &need_shadow);
        if (s == VCT_OK) s = validate_shadow(&d.shadow, true);
        if (s == VCT_OK) s = validate_gbuffer(&d.gbuffer);
        if (s != VCT_OK) return s;
        if (c->params.trace_filter != filter) return fail(VCT_ERR_INVALID_ARGUMENT, "all scenes of a batch must use the same trace_filter");
        // The resolve and mip kernels write the chain copies the sampler reads:
        // the texture-unit surfaces, the bordered fp32 chain, or both (hybrid).
        const bool hw = filter_uses_texture(filter), pad = filter_uses_bordered(filter);
        if (hw && (s = ensure_texture(c)) != VCT_OK) return s;
        if (c->params.voxelize_tesselation != b->ctx[0]->params.voxelize_tesselation)
            return fail(VCT_ERR_INVALID_ARGUMENT, "all scenes of a batch must use the same voxeliser");
        if (c->params.voxelize_tesselation && d.triangles.count > (1LL << 24))
            return fail(VCT_ERR_UNSUPPORTED, "the tessellation voxeliser takes at most 2^24 triangles per scene");
        AccumParams A;
        fill_accum_inputs(c->cfg, c->params, c->mvp, &d.triangles, d.lights, d.n_lights, &d.shadow, A);
        A.warp = warp_dev(c, d.eye);
        apply_tuning(b->tuning, A);
        A.acc = c->acc;
        A.occ = c->occ;
        A.carry = c->params.voxelize_tesselation ? c->carry : nullptr;
        A.brick_exact = c->params.voxelize_tesselation ? c->brick_exact : nullptr;
        A.stats = c->stats;
        A.num_sms = c->num_sms;
        InjectParams I;
        fill_inject(c, &d.shadow, d.eye, I);
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
        for (int l = 0; l <= R.mip_levels; ++l) {
            R.radiance_levels[l] = level_ptr(c->radiance, c, l);
            R.surf[l] = hw ? c->surf[l] : 0;
            R.pad_levels[l] = pad ? c->pchain + padded_level_offset(c->dim, l) : nullptr;
        }
        MipLevels M = mip_levels(c, c->radiance, c->levels);
        for (int l = 0; l < c->levels; ++l) {
            M.surf[l] = hw ? c->surf[l] : 0;
            M.pad[l] = pad ? c->pchain + padded_level_offset(c->dim, l) : nullptr;
        }
        M.first = std::min(4, c->levels - 1);
        TraceParams T;
        if ((s = fill_trace(c, &d.gbuffer, d.eye, &d.out, T)) != VCT_OK) return s;
        apply_tuning(b->tuning, T);
        std::memcpy(h + b->off_accum + i * sizeof(AccumParams), &A, sizeof A);
        std::memcpy(h + b->off_inject + i * sizeof(InjectParams), &I, sizeof I);
        std::memcpy(h + b->off_resolve + i * sizeof(ResolveParams), &R, sizeof R);
        std::memcpy(h + b->off_mips + i * sizeof(MipLevels), &M, sizeof M);
        std::memcpy(h + b->off_trace + i * sizeof(TraceParams), &T, sizeof T);
        // VCT_WARP_TEXTURE: the 32^3 occupancy voxelisation (the rasteriser's rule at a
        // 32^2 viewport, unwarped) and the map built from it, as build_warpmap does
        AccumParams O = A;
        WarpmapArgs WM;
        std::memset(&WM, 0, sizeof WM);
        O.occ = nullptr;
        if (c->params.warp_mode == VCT_WARP_TEXTURE) {
            O.dim = VCT_WARP_DIM;
            O.occ = c->occ32;
            O.acc = nullptr;
            O.stats = nullptr;
            O.warp.mode = VCT_WARP_NONE;
            WM = WarpmapArgs{c->occ32, c->params.warp_high_resolution, c->params.warp_low_resolution, c->warpmap,
                             c->warpmap_f};
            tot.any_map = true;
        }
        std::memcpy(h + b->off_occ + i * sizeof(AccumParams), &O, sizeof O);
        std::memcpy(h + b->off_wmap + i * sizeof(WarpmapArgs), &WM, sizeof WM);
        tri_off[i] = tot.tris;
        tex_off[i] = tot.texels;
        brick_off[i] = tot.bricks;
        tile_off[i] = tot.tiles;
        tot.tris += d.triangles.count;
        tot.texels += (long long)I.nx * I.ny;
        const long long bpa = c->dim / 16;
        tot.bricks += bpa * bpa * bpa;
        tot.tiles += trace_tiles(d.gbuffer.width, d.gbuffer.height, T.tile_w_log2, T.tile_h_log2);
    }
    ClearRange* clr = reinterpret_cast<ClearRange*>(h + b->off_clear);
    auto pre = [&](void* p, long long words) {
        clr[tot.n_pre++] = ClearRange{static_cast<uint32_t*>(p), words};
        tot.max_pre = std::max(tot.max_pre, words);
    };
    for (int i = 0; i < n; ++i) {
        vct_ctx* c = b->ctx[i];
        const long long mask_words = (c->nv + 31) / 32;
        pre(c->stats, (long long)(sizeof(StatsDev) / 4));
        pre(c->lit, mask_words);
        if (c->params.warp_mode == VCT_WARP_TEXTURE) pre(c->occ32, VCT_WARP_DIM * VCT_WARP_DIM * VCT_WARP_DIM / 32);
        if (c->params.voxelize_tesselation) {
            pre(c->carry, (long long)(kCarryBytes / 4));
            pre(c->brick_exact, c->nv / 4096 + 1);
        }
        clr[kClearPre * n + i] = ClearRange{c->occ, mask_words};
        tot.max_post = std::max(tot.max_post, mask_words);
    }
    tri_off[n] = tot.tris;
    tex_off[n] = tot.texels;
    brick_off[n] = tot.bricks;
    tile_off[n] = tot.tiles;
    if (tot.tris > 0x7fffffffLL) return fail(VCT_ERR_INVALID_ARGUMENT, "a batch holds at most 2^31-1 triangles");
    if (b->ctx[0]->params.voxelize_tesselation && tot.tris > (1LL << 24))
        return fail(VCT_ERR_UNSUPPORTED, "the tessellation voxeliser takes at most 2^24 triangles per batch");
    const long long need = accumulate_scratch_bytes(std::max(tot.tris, 1LL));
    if (need > b->work_bytes) {
        if (!allow_alloc) return fail(VCT_ERR_STATE, "batch work arrays too small for the captured scenes");
        // A captured graph points at the old arrays: it goes with them.
        if (b->exec) cudaGraphExecDestroy(b->exec);
        if (b->graph) cudaGraphDestroy(b->graph);
        b->exec = nullptr;
        b->graph = nullptr;
        if (b->work) cudaFree(b->work);
        b->work = nullptr;
        b->work_bytes = 0;
        cudaError_t e = cudaMalloc(&b->work, (size_t)need);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(VCT_ERR_OUT_OF_MEMORY, std::string("batch work arrays: ") + cudaGetErrorString(e));
        }
        b->work_bytes = need;
    }
    return VCT_OK;
}

// Enqueues one batched frame; `h` holds the staged blob.
vct_status batch_enqueue(vct_batch* b, const char* h, const BatchTotals& tot, cudaStream_t st, bool timed = false) {
    const int n = b->n;
    VCT_CUDA(cudaMemcpyAsync(b->d_blob, h, b->blob_bytes, cudaMemcpyHostToDevice, st));
    // A batched frame writes every level of the linear chain; the temporal
    // filter reads last frame's level 0 from it.
    for (vct_ctx* c : b->ctx) {
        if (c->params.temporal_filter) {
            vct_status s = sync_linear(c, st);
            if (s != VCT_OK) return s;
        }
        c->linear_stale = 0;
    }
    const ClearRange* d_clear = reinterpret_cast<const ClearRange*>(b->d_blob + b->off_clear);
    launch_clear_ranges(d_clear, tot.n_pre, tot.max_pre, st);
    VCT_CHECK_LAUNCH("batch: clear");
    if (tot.any_map) {
        const long long* d_tri = reinterpret_cast<const long long*>(b->d_blob + b->off_tables);
        launch_occupancy_batch(SceneBatch<AccumParams>{reinterpret_cast<const AccumParams*>(b->d_blob + b->off_occ),
                                                       d_tri, n},
                               tot.tris, st);
        VCT_CHECK_LAUNCH("batch: warp occupancy");
        launch_warpmap_batch(reinterpret_cast<const WarpmapArgs*>(b->d_blob + b->off_wmap), n, st);
        VCT_CHECK_LAUNCH("batch: warp maps");
    }
    const long long* d_tables = reinterpret_cast<const long long*>(b->d_blob + b->off_tables);
    AccumParams W0;
    W0.ntri = tot.tris;
    accumulate_bind_scratch(W0, b->work);
    const VoxWork W = {W0.tri_rec, W0.tri_units, W0.tri_scan, W0.block_off, tot.tris,
                       ilog2(b->tuning.voxel_unit_pixels)};
    if (timed) VCT_CUDA(cudaEventRecord(b->ev[0], st));
    if (tot.tris > 0) {
        const SceneBatch<AccumParams> SB{reinterpret_cast<const AccumParams*>(b->d_blob + b->off_accum), d_tables, n};
        if (b->ctx[0]->params.voxelize_tesselation)
            launch_tesselate_batch(SB, W, b->num_sms, st);
        else
            launch_accumulate_batch(SB, W, b->num_sms, b->tuning.voxel_blocks_per_sm, st);
        VCT_CHECK_LAUNCH("batch: accumulate");
    }
    if (timed) VCT_CUDA(cudaEventRecord(b->ev[1], st));
    launch_inject_mark_batch(
        SceneBatch<InjectParams>{reinterpret_cast<const InjectParams*>(b->d_blob + b->off_inject), d_tables + (n + 1), n},
        tot.texels, st);
    VCT_CHECK_LAUNCH("batch: inject mark");
    launch_resolve_batch(SceneBatch<ResolveParams>{reinterpret_cast<const ResolveParams*>(b->d_blob + b->off_resolve),
                                                  d_tables + 2 * (n + 1), n},
                         tot.bricks, b->ctx[0]->params.voxelize_tesselation != 0, st);
    VCT_CHECK_LAUNCH("batch: resolve");
    launch_clear_ranges(d_clear + kClearPre * n, n, tot.max_post, st);
    VCT_CHECK_LAUNCH("batch: clear occupancy");
    launch_mip_tail_batch(SceneBatch<MipLevels>{reinterpret_cast<const MipLevels*>(b->d_blob + b->off_mips), nullptr, n},
                          st);
    VCT_CHECK_LAUNCH("batch: coarse mips");
    if (timed) VCT_CUDA(cudaEventRecord(b->ev[2], st));
    launch_trace_batch(SceneBatch<TraceParams>{reinterpret_cast<const TraceParams*>(b->d_blob + b->off_trace),
                                              d_tables + 3 * (n + 1), n},
                       b->ctx[0]->params.trace_filter, tot.tiles, st);
    VCT_CHECK_LAUNCH("batch: trace");
    if (timed) VCT_CUDA(cudaEventRecord(b->ev[3], st));
    const int filter = b->ctx[0]->params.trace_filter;
    for (vct_ctx* c : b->ctx) {
        c->stats_reset_pending = true;
        c->radiance_ready = c->mips_ready = true;
        c->tex_ready = filter_uses_texture(filter);
        c->pad_ready = filter_uses_bordered(filter);
    }
    return VCT_OK;
}

}  // namespace

extern "C" {

vct_status vct_batch_create(const vct_config* scene_cfg, int32_t n, vct_batch** out) {
    if (!out) return fail(VCT_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (!scene_cfg || n < 1 || n > accumulate_batch_max_scenes())
        return fail(VCT_ERR_INVALID_ARGUMENT, "a batch holds 1..256 scenes");
    for (int i = 0; i < n; ++i) {
        vct_status s = validate_config(&scene_cfg[i]);
        if (s != VCT_OK) return s;
        if (scene_cfg[i].voxel_dim > 256) return fail(VCT_ERR_UNSUPPORTED, "batched scenes are limited to 256^3 grids");
        if (scene_cfg[i].device != scene_cfg[0].device) return fail(VCT_ERR_INVALID_ARGUMENT, "a batch lives on one device");
    }
    vct_batch* b = new (std::nothrow) vct_batch;
    if (!b) return fail(VCT_ERR_OUT_OF_MEMORY, "host allocation failed");
    b->n = n;
    b->device = scene_cfg[0].device;
    default_tuning(b->tuning);
    for (int i = 0; i < n; ++i) {
        vct_ctx* c = nullptr;
        vct_status s = vct_create(&scene_cfg[i], &c);
        if (s != VCT_OK) {
            std::string msg = g_err;
            vct_batch_destroy(b);
            return fail(s, msg);
        }
        b->ctx.push_back(c);
    }
    b->num_sms = b->ctx[0]->num_sms;
    size_t off = 0;
    b->off_accum = off;
    off = up256(off + sizeof(AccumParams) * n);
    b->off_inject = off;
    off = up256(off + sizeof(InjectParams) * n);
    b->off_resolve = off;
    off = up256(off + sizeof(ResolveParams) * n);
    b->off_mips = off;
    off = up256(off + sizeof(MipLevels) * n);
    b->off_trace = off;
    off = up256(off + sizeof(TraceParams) * n);
    b->off_tables = off;
    off = up256(off + sizeof(long long) * 4 * (n + 1));
    b->off_clear = off;
    off = up256(off + sizeof(ClearRange) * (kClearPre + 1) * n);
    b->off_occ = off;
    off = up256(off + sizeof(AccumParams) * n);
    b->off_wmap = off;
    off = up256(off + sizeof(WarpmapArgs) * n);
    b->blob_bytes = off;
    DeviceScope ds(b->device);
    cudaError_t e = cudaMalloc(&b->d_blob, off);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_blob, off);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_graph_blob, off);
    if (e != cudaSuccess) {
        cudaGetLastError();
        vct_batch_destroy(b);
        return fail(VCT_ERR_OUT_OF_MEMORY, std::string("batch parameter blob: ") + cudaGetErrorString(e));
    }
    std::memset(b->h_blob, 0, off);
    std::memset(b->h_graph_blob, 0, off);
    *out = b;
    return VCT_OK;
}

vct_status vct_batch_destroy(vct_batch* b) {
    if (!b) return VCT_OK;
    DeviceScope ds(b->device);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (cudaEvent_t e : b->ev)
        if (e) cudaEventDestroy(e);
    for (vct_ctx* c : b->ctx) vct_destroy(c);
    if (b->d_blob) cudaFree(b->d_blob);
    if (b->h_blob) cudaFreeHost(b->h_blob);
    if (b->h_graph_blob) cudaFreeHost(b->h_graph_blob);
    if (b->work) cudaFree(b->work);
    delete b;
    return VCT_OK;
}

vct_status vct_batch_set_params(vct_batch* b, int32_t scene, const vct_params* p) {
    if (!b) return fail(VCT_ERR_INVALID_ARGUMENT, "batch is NULL");
    if (scene < -1 || scene >= b->n) return fail(VCT_ERR_INVALID_ARGUMENT, "scene index out of range");
    for (int i = 0; i < b->n; ++i)
        if (scene == -1 || scene == i) {
            vct_status s = vct_set_params(b->ctx[i], p);
            if (s != VCT_OK) return s;
        }
    return VCT_OK;
}

vct_status vct_batch_frame(vct_batch* b, const vct_scene_desc* scenes, int32_t n, void* stream) {
    if (!b) return fail(VCT_ERR_INVALID_ARGUMENT, "batch is NULL");
    DeviceScope ds(b->device);
    VCT_CUDA(ds.err);
    cudaStream_t st = as_stream(stream);
    // The staging blob may still be read by the previous frame's copy.
    VCT_CUDA(cudaStreamSynchronize(st));
    BatchTotals tot;
    vct_status s = batch_stage(b, scenes, n, b->h_blob, tot, true);
    if (s != VCT_OK) return s;
    if ((s = batch_enqueue(b, b->h_blob, tot, st, b->timers_on)) != VCT_OK) return s;
    b->timers_recorded = b->timers_on;
    return VCT_OK;
}

vct_status vct_batch_enable_timers(vct_batch* b, int32_t enable) {
    if (!b) return fail(VCT_ERR_INVALID_ARGUMENT, "batch is NULL");
    DeviceScope ds(b->device);
    VCT_CUDA(ds.err);
    if (enable && !b->ev[0])
        for (auto& e : b->ev) VCT_CUDA(cudaEventCreate(&e));
    b->timers_on = enable != 0;
    b->timers_recorded = false;
    return VCT_OK;
}

vct_status vct_batch_get_timers(vct_batch* b, vct_timers* out) {
    if (!b || !out) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!b->timers_recorded) return fail(VCT_ERR_STATE, "no timed vct_batch_frame since timers were enabled");
    DeviceScope ds(b->device);
    VCT_CUDA(ds.err);
    VCT_CUDA(cudaEventSynchronize(b->ev[3]));
    VCT_CUDA(cudaEventElapsedTime(&out->voxelize_ms, b->ev[0], b->ev[1]));
    VCT_CUDA(cudaEventElapsedTime(&out->mipmap_ms, b->ev[1], b->ev[2]));
    VCT_CUDA(cudaEventElapsedTime(&out->render_ms, b->ev[2], b->ev[3]));
    VCT_CUDA(cudaEventElapsedTime(&out->total_ms, b->ev[0], b->ev[3]));
    out->radiance_ms = 0.0f;
    return VCT_OK;
}

vct_status vct_batch_capture(vct_batch* b, const vct_scene_desc* scenes, int32_t n, void* stream) {
    if (!b) return fail(VCT_ERR_INVALID_ARGUMENT, "batch is NULL");
    if (!stream) return fail(VCT_ERR_INVALID_ARGUMENT, "capture needs a non-default stream");
    DeviceScope ds(b->device);
    VCT_CUDA(ds.err);
    cudaStream_t st = as_stream(stream);
    VCT_CUDA(cudaStreamSynchronize(st));
    BatchTotals tot;
    vct_status s = batch_stage(b, scenes, n, b->h_graph_blob, tot, true);
    if (s != VCT_OK) return s;
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    VCT_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const unsigned long long launches0 = vct_launch_count();
    s = batch_enqueue(b, b->h_graph_blob, tot, st);
    b->graph_launches = (int)(vct_launch_count() - launches0);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (s != VCT_OK) {
        if (g) cudaGraphDestroy(g);
        return s;
    }
    if (e != cudaSuccess) return fail(VCT_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    b->graph = g;
    VCT_CUDA(cudaGraphInstantiate(&b->exec, g, 0));
    return VCT_OK;
}

vct_status vct_batch_replay(vct_batch* b, void* stream) {
    if (!b) return fail(VCT_ERR_INVALID_ARGUMENT, "batch is NULL");
    if (!b->exec) return fail(VCT_ERR_STATE, "no captured graph: call vct_batch_capture first");
    DeviceScope ds(b->device);
    VCT_CUDA(ds.err);
    VCT_CUDA(cudaGraphLaunch(b->exec, as_stream(stream)));
    note_launches(b->graph_launches);
    return VCT_OK;
}

vct_status vct_batch_context(vct_batch* b, int32_t scene, vct_ctx** ctx) {
    if (!b || !ctx) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (scene < 0 || scene >= b->n) return fail(VCT_ERR_INVALID_ARGUMENT, "scene index out of range");
    *ctx = b->ctx[scene];
    return VCT_OK;
}


}  // extern "C"

// ==================================================================== tuning
namespace {

// Candidate settings of the autotuner.  Voxeliser: work-unit size (smaller
// units balance scenes of few large triangles, larger ones cut per-unit
// overhead) x raster CTAs per SM.  Trace: CTA tile and warp sub-tile shapes
// (the warp's footprint decides how coherent its 32 cones' texel fetches are).
const int kUnitCand[] = {128, 256, 512, 1024, 2048};
const int kBpsCand[] = {2, 3};
const int kTileCand[][3] = {{16, 16, 8}, {16, 16, 4}, {16, 16, 16}, {32, 8, 8}, {32, 8, 4},  {32, 8, 16},
                            {8, 32, 4},  {8, 32, 8},  {64, 4, 8},   {64, 4, 16}, {64, 4, 32}, {4, 64, 4}};

float median(std::vector<float> v) {
    std::sort(v.begin(), v.end());
    return v.empty() ? 0.0f : v[v.size() / 2];
}

// Runs one timed frame and returns (voxeliser ms, trace ms).
using TimedFrame = vct_status (*)(void* obj, const void* args, float* vox_ms, float* trace_ms);

vct_status tune(vct_tuning& cur, int reps, void* obj, const void* args, TimedFrame run, vct_tuning* set_into) {
    reps = std::max(1, std::min(reps, 64));
    std::vector<float> vox, trc;
    float v = 0, t = 0;
    // Voxeliser settings.
    vct_tuning best = cur;
    float best_ms = 3.0e38f;
    for (int u : kUnitCand)
        for (int bps : kBpsCand) {
            vct_tuning c = best;
            c.voxel_unit_pixels = u;
            c.voxel_blocks_per_sm = bps;
            *set_into = c;
            vct_status s = run(obj, args, &v, &t);  // warm-up
            if (s != VCT_OK) return s;
            vox.clear();
            for (int r = 0; r < reps; ++r) {
                if ((s = run(obj, args, &v, &t)) != VCT_OK) return s;
                vox.push_back(v);
            }
            const float m = median(vox);
            if (m < best_ms) {
                best_ms = m;
                best.voxel_unit_pixels = u;
                best.voxel_blocks_per_sm = bps;
            }
        }
    // Trace tile shapes.
    best_ms = 3.0e38f;
    vct_tuning best2 = best;
    for (const auto& tc : kTileCand) {
        vct_tuning c = best;
        c.trace_tile_w = tc[0];
        c.trace_tile_h = tc[1];
        c.trace_warp_w = tc[2];
        *set_into = c;
        vct_status s = run(obj, args, &v, &t);
        if (s != VCT_OK) return s;
        trc.clear();
        for (int r = 0; r < reps; ++r) {
            if ((s = run(obj, args, &v, &t)) != VCT_OK) return s;
            trc.push_back(t);
        }
        const float m = median(trc);
        if (m < best_ms) {
            best_ms = m;
            best2 = c;
        }
    }
    cur = best2;
    *set_into = best2;
    return VCT_OK;
}

struct CtxFrameArgs {
    const vct_triangles* tris;
    const vct_light* lights;
    int32_t n;
    const vct_shadow_desc* shadow;
    const float* eye;
    const vct_gbuffer* g;
    const vct_trace_out* out;
    void* stream;
};

vct_status ctx_timed_frame(void* obj, const void* a, float* vox_ms, float* trace_ms) {
    vct_ctx* c = static_cast<vct_ctx*>(obj);
    const CtxFrameArgs& f = *static_cast<const CtxFrameArgs*>(a);
    vct_status s = vct_frame(c, f.tris, f.lights, f.n, f.shadow, f.eye, f.g, f.out, f.stream);
    if (s != VCT_OK) return s;
    vct_timers t;
    if ((s = vct_get_timers(c, &t)) != VCT_OK) return s;
    *vox_ms = t.voxelize_ms;
    *trace_ms = t.render_ms;
    return VCT_OK;
}

struct BatchFrameArgs {
    const vct_scene_desc* scenes;
    int32_t n;
    void* stream;
};

vct_status batch_timed_frame(void* obj, const void* a, float* vox_ms, float* trace_ms) {
    vct_batch* b = static_cast<vct_batch*>(obj);
    const BatchFrameArgs& f = *static_cast<const BatchFrameArgs*>(a);
    cudaStream_t st = as_stream(f.stream);
    VCT_CUDA(cudaStreamSynchronize(st));
    BatchTotals tot;
    vct_status s = batch_stage(b, f.scenes, f.n, b->h_blob, tot, true);
    if (s != VCT_OK) return s;
    if ((s = batch_enqueue(b, b->h_blob, tot, st, true)) != VCT_OK) return s;
    VCT_CUDA(cudaEventSynchronize(b->ev[3]));
    VCT_CUDA(cudaEventElapsedTime(vox_ms, b->ev[0], b->ev[1]));
    VCT_CUDA(cudaEventElapsedTime(trace_ms, b->ev[2], b->ev[3]));
    return VCT_OK;
}

}  // namespace

extern "C" {

void vct_default_tuning(vct_tuning* out) {
    if (out) default_tuning(*out);
}

vct_status vct_get_tuning(const vct_ctx* c, vct_tuning* out) {
    if (!c || !out) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = c->tuning;
    return VCT_OK;
}

vct_status vct_set_tuning(vct_ctx* c, const vct_tuning* t) {
    if (!c) return fail(VCT_ERR_INVALID_ARGUMENT, "ctx is NULL");
    vct_status s = validate_tuning(t);
    if (s != VCT_OK) return s;
    c->tuning = *t;
    return VCT_OK;
}

vct_status vct_batch_get_tuning(const vct_batch* b, vct_tuning* out) {
    if (!b || !out) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = b->tuning;
    return VCT_OK;
}

vct_status vct_batch_set_tuning(vct_batch* b, const vct_tuning* t) {
    if (!b) return fail(VCT_ERR_INVALID_ARGUMENT, "batch is NULL");
    vct_status s = validate_tuning(t);
    if (s != VCT_OK) return s;
    b->tuning = *t;
    return VCT_OK;
}

vct_status vct_autotune(vct_ctx* c, const vct_triangles* tris, const vct_light* lights, int32_t n_lights,
                        const vct_shadow_desc* shadow, const float eye[3], const vct_gbuffer* g,
                        const vct_trace_out* out, int32_t reps, void* stream, vct_tuning* best) {
    if (!c) return fail(VCT_ERR_INVALID_ARGUMENT, "ctx is NULL");
    const bool timers_were_on = c->timers_on;
    vct_status s = vct_enable_timers(c, 1);
    if (s != VCT_OK) return s;
    const CtxFrameArgs args = {tris, lights, n_lights, shadow, eye, g, out, stream};
    const vct_tuning orig = c->tuning;
    vct_tuning cur = orig;
    s = tune(cur, reps, c, &args, ctx_timed_frame, &c->tuning);
    c->tuning = s == VCT_OK ? cur : orig;
    vct_enable_timers(c, timers_were_on ? 1 : 0);
    if (s == VCT_OK && best) *best = c->tuning;
    return s;
}

vct_status vct_batch_autotune(vct_batch* b, const vct_scene_desc* scenes, int32_t n, int32_t reps, void* stream,
                              vct_tuning* best) {
    if (!b) return fail(VCT_ERR_INVALID_ARGUMENT, "batch is NULL");
    DeviceScope ds(b->device);
    VCT_CUDA(ds.err);
    if (!b->ev[0])
        for (auto& e : b->ev) VCT_CUDA(cudaEventCreate(&e));
    b->timers_recorded = false;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    const BatchFrameArgs args = {scenes, n, stream};
    const vct_tuning orig = b->tuning;
    vct_tuning cur = orig;
    vct_status s = tune(cur, reps, b, &args, batch_timed_frame, &b->tuning);
    b->tuning = s == VCT_OK ? cur : orig;
    if (s == VCT_OK && best) *best = cur;
    return s;
}

}  // extern "C"
