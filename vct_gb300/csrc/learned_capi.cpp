// C ABI of the learned path (include/vct.h): the tensor-core GEMM check, the
// MLP object (inference, gradients, Adam training steps) and the traces of
// the learned configuration (cheap quarter-resolution features, the 16-cone
// reference, the learned trace with its per-tile or per-pixel fallback).
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "host.h"

using namespace vct;
using namespace vct::host;

struct vct_mlp {
    int device = 0, num_sms = 0;
    MlpDev dev = {};
    uint32_t* status = nullptr;
    int step = 0;
};

namespace {

// splitmix64 (Steele, Lea, Flood 2014): seeded uniform numbers for the
// initial weights.
uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// He-uniform weights (bound sqrt(6 / fan_in)), zero biases.
void init_params(uint64_t seed, std::vector<float>& p) {
    p.assign(kMlpParams, 0.0f);
    uint64_t s = seed;
    auto fill = [&](int off, int nout, int nin) {
        const double a = std::sqrt(6.0 / nin);
        for (int i = 0; i < nout * nin; ++i) {
            const double u = (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0);
            p[off + i] = (float)((2.0 * u - 1.0) * a);
        }
    };
    fill(kOffW1, kMlpHidden, kMlpIn);
    fill(kOffW2, kMlpHidden, kMlpHidden);
    fill(kOffW3, kMlpHidden, kMlpHidden);
    fill(kOffW4, kMlpOut, kMlpHidden);
}

vct_status upload_params(vct_mlp* m, const float* host, cudaStream_t st) {
    VCT_CUDA(cudaMemcpyAsync(m->dev.params, host, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, st));
    VCT_CUDA(cudaMemsetAsync(m->dev.m, 0, sizeof(float) * kMlpParams, st));
    VCT_CUDA(cudaMemsetAsync(m->dev.v, 0, sizeof(float) * kMlpParams, st));
    launch_mlp_update(m->dev, 1, 0.f, 0.f, 0.f, 0.f, 0, st);
    VCT_CHECK_LAUNCH("mlp operand images");
    m->step = 0;
    return VCT_OK;
}

vct_status check_status(vct_mlp* m, cudaStream_t st) {
    uint32_t h = 0;
    VCT_CUDA(cudaMemcpyAsync(&h, m->status, sizeof h, cudaMemcpyDeviceToHost, st));
    VCT_CUDA(cudaStreamSynchronize(st));
    if (h) {
        VCT_CUDA(cudaMemsetAsync(m->status, 0, sizeof h, st));
        return fail(VCT_ERR_TIMEOUT, "a tensor-core completion wait timed out");
    }
    return VCT_OK;
}

vct_status validate_rows(const float* rows, int64_t n) {
    if (n < 0 || n > (1LL << 31)) return fail(VCT_ERR_INVALID_ARGUMENT, "row count out of range");
    if (n > 0 && !rows) return fail(VCT_ERR_INVALID_ARGUMENT, "rows is NULL");
    if (reinterpret_cast<uintptr_t>(rows) % 8 != 0) return fail(VCT_ERR_INVALID_ARGUMENT, "rows must be 8-byte aligned");
    return VCT_OK;
}

// The 16-cone reference set: Fibonacci hemisphere directions
// (z_i = 1 - (i + 1/2)/16, azimuth i times the golden angle) in the
// (T, B, N) frame, weighted by cos(theta) / sum cos(theta); cones of equal
// solid angle 2 pi / 16 (aperture 2 acos(15/16)).
void fill_learned(vct_ctx* c, const TraceParams& T, LearnedParams& L) {
    std::memset(&L, 0, sizeof L);
    L.T = T;
    L.wq = (T.width + 3) / 4;
    L.hq = (T.height + 3) / 4;
    L.depth_scale = 1.0f / (c->cfg.voxel_max[0] - c->cfg.voxel_min[0]);
    const double golden = 3.14159265358979323846 * (3.0 - std::sqrt(5.0));
    double wsum = 0.0;
    for (int i = 0; i < 16; ++i) wsum += 1.0 - (i + 0.5) / 16.0;
    for (int i = 0; i < 16; ++i) {
        const double z = 1.0 - (i + 0.5) / 16.0, r = std::sqrt(1.0 - z * z), phi = golden * i;
        L.dirs16[i][0] = (float)(r * std::cos(phi));
        L.dirs16[i][1] = (float)(r * std::sin(phi));
        L.dirs16[i][2] = (float)z;
        L.dirs16[i][3] = (float)(z / wsum);
    }
    L.ref_cone = c->params.diffuse_cone;
    L.ref_cone.steps = 24;
    L.ref_cone.cone_angle = (float)(2.0 * std::acos(15.0 / 16.0));
}

vct_status learned_setup(vct_ctx* c, const vct_gbuffer* g, const float eye[3], cudaStream_t st, LearnedParams& L) {
    if (!c || !eye) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    vct_status s = validate_gbuffer(g);
    if (s != VCT_OK) return s;
    if (c->levels < 5) return fail(VCT_ERR_UNSUPPORTED, "the learned path samples mip levels 1..4: needs >= 5 levels");
    if ((s = ensure_padded_chain(c, st)) != VCT_OK) return s;
    vct_trace_out none = {};
    TraceParams T;
    if ((s = fill_trace(c, g, eye, &none, T)) != VCT_OK) return s;
    fill_learned(c, T, L);
    return VCT_OK;
}


// The learned traces' scratch in the context: quarter-resolution features,
// the per-tile error estimates, the fallback list (tiles, or pixels: one
// entry per pixel of the frame), the per-pixel error estimates, the frame's
// two sums and the list's length.
vct_status learned_scratch(vct_ctx* c, long long W, long long H, LearnedParams& L) {
    const long long tiles = ((W + kLearnTile - 1) / kLearnTile) * ((H + kLearnTile - 1) / kLearnTile);
    const long long entries = tiles > W * H ? tiles : W * H;
    auto a256 = [](long long b) { return (size_t)((b + 255) & ~255LL); };
    const size_t qbytes = (size_t)L.wq * L.hq * kCheapFeatures * 2;
    const size_t need = a256((long long)qbytes) + a256(tiles * 4) + a256(entries * 4) + a256(W * H * 4) + 256 + 256;
    if (need > c->learned_bytes) {
        if (c->learned) cudaFree(c->learned);
        c->learned = nullptr;
        c->learned_bytes = 0;
        cudaError_t e = cudaMalloc(&c->learned, need);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(VCT_ERR_OUT_OF_MEMORY, std::string("learned scratch: ") + cudaGetErrorString(e));
        }
        c->learned_bytes = need;
    }
    char* p = static_cast<char*>(c->learned);
    L.qfeat = reinterpret_cast<uint16_t*>(p);
    p += a256((long long)qbytes);
    L.tile_err = reinterpret_cast<float*>(p);
    p += a256(tiles * 4);
    L.list = reinterpret_cast<uint32_t*>(p);
    p += a256(entries * 4);
    L.est = reinterpret_cast<float*>(p);
    p += a256(W * H * 4);
    L.frame_sums = reinterpret_cast<float*>(p);
    p += 256;
    L.count = reinterpret_cast<uint32_t*>(p);
    return VCT_OK;
}

vct_status learned_check(vct_ctx* c, vct_mlp* m, float* irradiance, float threshold) {
    if (!c || !m || !irradiance) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (reinterpret_cast<uintptr_t>(irradiance) % 16 != 0) return fail(VCT_ERR_INVALID_ARGUMENT, "irradiance must be 16-byte aligned");
    if (m->device != c->device) return fail(VCT_ERR_INVALID_ARGUMENT, "context and MLP live on different devices");
    if (!(threshold >= 0.0f)) return fail(VCT_ERR_INVALID_ARGUMENT, "threshold must be >= 0 (infinity: no fallback)");
    return VCT_OK;
}

}  // namespace

extern "C" {

vct_status vct_tensor_core_check(const uint16_t* a_dev, const uint16_t* b_dev, int32_t k, int32_t n, int32_t variant,
                                 float* d_dev, void* stream) {
    if (!a_dev || !b_dev || !d_dev) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (k < 16 || k > 64 || k % 16 != 0) return fail(VCT_ERR_INVALID_ARGUMENT, "k must be 16, 32, 48 or 64");
    if (n < 16 || n > 64 || n % 16 != 0) return fail(VCT_ERR_INVALID_ARGUMENT, "n must be 16, 32, 48 or 64");
    if (variant != 0 && variant != 1) return fail(VCT_ERR_INVALID_ARGUMENT, "variant must be 0 or 1");
    cudaStream_t st = as_stream(stream);
    uint32_t* status = nullptr;
    VCT_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&status), sizeof(uint32_t), st));
    VCT_CUDA(cudaMemsetAsync(status, 0, sizeof(uint32_t), st));
    launch_umma_check(a_dev, b_dev, k, n, variant, d_dev, status, st);
    VCT_CHECK_LAUNCH("tensor core check");
    uint32_t h = 0;
    VCT_CUDA(cudaMemcpyAsync(&h, status, sizeof h, cudaMemcpyDeviceToHost, st));
    VCT_CUDA(cudaFreeAsync(status, st));
    VCT_CUDA(cudaStreamSynchronize(st));
    if (h) return fail(VCT_ERR_TIMEOUT, "tensor core check: MMA completion wait timed out");
    return VCT_OK;
}

vct_status vct_timeout_probe(int64_t limit_ns, void* stream) {
    if (limit_ns < 1000 || limit_ns > 1000000000) return fail(VCT_ERR_INVALID_ARGUMENT, "limit_ns must be in [1e3, 1e9]");
    cudaStream_t st = as_stream(stream);
    uint32_t* status = nullptr;
    VCT_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&status), sizeof(uint32_t), st));
    VCT_CUDA(cudaMemsetAsync(status, 0, sizeof(uint32_t), st));
    launch_wait_probe(status, (unsigned long long)limit_ns, st);
    VCT_CHECK_LAUNCH("timeout probe");
    uint32_t h = 0;
    VCT_CUDA(cudaMemcpyAsync(&h, status, sizeof h, cudaMemcpyDeviceToHost, st));
    VCT_CUDA(cudaFreeAsync(status, st));
    VCT_CUDA(cudaStreamSynchronize(st));
    if (h) return fail(VCT_ERR_TIMEOUT, "timeout probe: the bounded wait gave up, as designed");
    return VCT_OK;
}

vct_status vct_mlp_create(int32_t device, uint64_t seed, vct_mlp** out) {
    if (!out) return fail(VCT_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    DeviceScope ds(device);
    VCT_CUDA(ds.err);
    vct_mlp* m = new (std::nothrow) vct_mlp;
    if (!m) return fail(VCT_ERR_OUT_OF_MEMORY, "host allocation failed");
    m->device = device;
    cudaDeviceGetAttribute(&m->num_sms, cudaDevAttrMultiProcessorCount, device);
    const size_t pf = sizeof(float) * kMlpParams;
    struct {
        void** p;
        size_t bytes;
    } allocs[] = {{(void**)&m->dev.params, pf},           {(void**)&m->dev.grad, pf},
                  {(void**)&m->dev.m, pf},                {(void**)&m->dev.v, pf},
                  {(void**)&m->dev.img, (size_t)kImgAll}, {(void**)&m->dev.bias, sizeof(float) * kBiasPad},
                  {(void**)&m->dev.loss, sizeof(float)},  {(void**)&m->status, sizeof(uint32_t)}};
    for (auto& a : allocs) {
        cudaError_t e = cudaMalloc(a.p, a.bytes);
        if (e == cudaSuccess) e = cudaMemset(*a.p, 0, a.bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            vct_mlp_destroy(m);
            return fail(VCT_ERR_OUT_OF_MEMORY, std::string("mlp buffers: ") + cudaGetErrorString(e));
        }
    }
    std::vector<float> p;
    init_params(seed, p);
    vct_status s = upload_params(m, p.data(), nullptr);
    if (s == VCT_OK && cudaDeviceSynchronize() != cudaSuccess) s = fail(VCT_ERR_CUDA, "mlp initialisation");
    if (s != VCT_OK) {
        std::string msg = g_err;
        vct_mlp_destroy(m);
        return fail(s, msg);
    }
    *out = m;
    return VCT_OK;
}

vct_status vct_mlp_destroy(vct_mlp* m) {
    if (!m) return VCT_OK;
    DeviceScope ds(m->device);
    void* ptrs[] = {m->dev.params, m->dev.grad, m->dev.m, m->dev.v, m->dev.img, m->dev.bias, m->dev.loss, m->status};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete m;
    return VCT_OK;
}

vct_status vct_mlp_set_params(vct_mlp* m, const float* host, int64_t count) {
    if (!m || !host) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (count != kMlpParams) return fail(VCT_ERR_INVALID_ARGUMENT, "count must be VCT_MLP_PARAMS");
    for (int64_t i = 0; i < count; ++i)
        if (!std::isfinite(host[i])) return fail(VCT_ERR_INVALID_ARGUMENT, "parameters must be finite");
    DeviceScope ds(m->device);
    VCT_CUDA(ds.err);
    vct_status s = upload_params(m, host, nullptr);
    if (s != VCT_OK) return s;
    VCT_CUDA(cudaDeviceSynchronize());
    return VCT_OK;
}

vct_status vct_mlp_get_params(vct_mlp* m, float* host, int64_t count, void* stream) {
    if (!m || !host) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (count != kMlpParams) return fail(VCT_ERR_INVALID_ARGUMENT, "count must be VCT_MLP_PARAMS");
    DeviceScope ds(m->device);
    VCT_CUDA(ds.err);
    cudaStream_t st = as_stream(stream);
    VCT_CUDA(cudaMemcpyAsync(host, m->dev.params, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, st));
    return check_status(m, st);
}

vct_status vct_mlp_forward(vct_mlp* m, const float* rows, int64_t n, float* out, void* stream) {
    if (!m || (n > 0 && !out)) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (reinterpret_cast<uintptr_t>(out) % 16 != 0) return fail(VCT_ERR_INVALID_ARGUMENT, "out must be 16-byte aligned");
    vct_status s = validate_rows(rows, n);
    if (s != VCT_OK) return s;
    DeviceScope ds(m->device);
    VCT_CUDA(ds.err);
    LearnedParams L;
    std::memset(&L, 0, sizeof L);
    L.img = m->dev.img;
    L.bias = m->dev.bias;
    L.rows = rows;
    L.n = n;
    L.out_rows = out;
    L.status = m->status;
    launch_mlp_infer(L, m->num_sms, as_stream(stream));
    VCT_CHECK_LAUNCH("mlp forward");
    return VCT_OK;
}

static vct_status train_launch(vct_mlp* m, const float* rows, const float* targets, const int32_t* index, int64_t n,
                               cudaStream_t st) {
    vct_status s = validate_rows(rows, n);
    if (s != VCT_OK) return s;
    if (n < 1) return fail(VCT_ERR_INVALID_ARGUMENT, "training needs at least one row");
    if (!targets) return fail(VCT_ERR_INVALID_ARGUMENT, "targets is NULL");
    VCT_CUDA(cudaMemsetAsync(m->dev.grad, 0, sizeof(float) * kMlpParams, st));
    VCT_CUDA(cudaMemsetAsync(m->dev.loss, 0, sizeof(float), st));
    TrainParams P;
    std::memset(&P, 0, sizeof P);
    P.mlp = m->dev;
    P.rows = rows;
    P.targets = targets;
    P.index = index;
    P.n = n;
    P.scale = (float)(2.0 / (3.0 * (double)n));
    P.conf_scale = (float)(2.0 * (double)kMlpConfidenceWeight / (double)n);
    P.status = m->status;
    launch_mlp_train(P, m->num_sms, st);
    VCT_CHECK_LAUNCH("mlp training kernel");
    return VCT_OK;
}

vct_status vct_mlp_gradients(vct_mlp* m, const float* rows, const float* targets, int64_t n, float* grad_dev,
                             float* loss_dev, void* stream) {
    if (!m || !grad_dev) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    DeviceScope ds(m->device);
    VCT_CUDA(ds.err);
    cudaStream_t st = as_stream(stream);
    vct_status s = train_launch(m, rows, targets, nullptr, n, st);
    if (s != VCT_OK) return s;
    VCT_CUDA(cudaMemcpyAsync(grad_dev, m->dev.grad, sizeof(float) * kMlpParams, cudaMemcpyDeviceToDevice, st));
    if (loss_dev) VCT_CUDA(cudaMemcpyAsync(loss_dev, m->dev.loss, sizeof(float), cudaMemcpyDeviceToDevice, st));
    return check_status(m, st);
}

vct_status vct_mlp_train_step(vct_mlp* m, const float* rows, const float* targets, const int32_t* index, int64_t n,
                              const vct_adam* opt, float* loss_dev, void* stream) {
    if (!m || !opt) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!(opt->lr >= 0.0f) || !(opt->beta1 >= 0.0f && opt->beta1 < 1.0f) || !(opt->beta2 >= 0.0f && opt->beta2 < 1.0f) ||
        !(opt->eps > 0.0f))
        return fail(VCT_ERR_INVALID_ARGUMENT, "Adam settings out of range");
    DeviceScope ds(m->device);
    VCT_CUDA(ds.err);
    cudaStream_t st = as_stream(stream);
    vct_status s = train_launch(m, rows, targets, index, n, st);
    if (s != VCT_OK) return s;
    ++m->step;
    launch_mlp_update(m->dev, m->step, opt->lr, opt->beta1, opt->beta2, opt->eps, 1, st);
    VCT_CHECK_LAUNCH("adam");
    if (loss_dev) VCT_CUDA(cudaMemcpyAsync(loss_dev, m->dev.loss, sizeof(float), cudaMemcpyDeviceToDevice, st));
    return VCT_OK;
}

vct_status vct_learned_features(vct_ctx* c, const vct_gbuffer* g, const float eye[3], uint16_t* features, void* stream) {
    if (!features) return fail(VCT_ERR_INVALID_ARGUMENT, "features is NULL");
    if (reinterpret_cast<uintptr_t>(features) % 16 != 0) return fail(VCT_ERR_INVALID_ARGUMENT, "features must be 16-byte aligned");
    if (!c) return fail(VCT_ERR_INVALID_ARGUMENT, "ctx is NULL");
    DeviceScope ds(c->device);
    VCT_CUDA(ds.err);
    cudaStream_t st = as_stream(stream);
    LearnedParams L;
    vct_status s = learned_setup(c, g, eye, st, L);
    if (s != VCT_OK) return s;
    L.qfeat = features;
    launch_learned_features(L, st);
    VCT_CHECK_LAUNCH("learned features");
    return VCT_OK;
}

vct_status vct_learned_rows(vct_ctx* c, const vct_gbuffer* g, const float eye[3], const uint16_t* features,
                            const int32_t* pixels, int64_t n, float* rows, void* stream) {
    if (!features || (n > 0 && (!pixels || !rows))) return fail(VCT_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n < 0) return fail(VCT_ERR_INVALID_ARGUMENT, "n must be >= 0");
    if (!c) return fail(VCT_ERR_INVALID_ARGUMENT, "ctx is NULL");
    DeviceScope ds(c->device);
    VCT_CUDA(ds.err);
    cudaStream_t st = as_stream(stream);
    LearnedParams L;
    vct_status s = learned_setup(c, g, eye, st, L);
    if (s != VCT_OK) return s;
    L.qfeat = features;
    L.pixels = pixels;
    L.n = n;
    L.rows_out = rows;
    launch_learned_rows(L, st);
    VCT_CHECK_LAUNCH("learned rows");
    return VCT_OK;
}

vct_status vct_trace_reference16(vct_ctx* c, const vct_gbuffer* g, const float eye[3], float* irradiance, void* stream) {
    if (!irradiance) return fail(VCT_ERR_INVALID_ARGUMENT, "irradiance is NULL");
    if (reinterpret_cast<uintptr_t>(irradiance) % 16 != 0) return fail(VCT_ERR_INVALID_ARGUMENT, "irradiance must be 16-byte aligned");
    if (!c) return fail(VCT_ERR_INVALID_ARGUMENT, "ctx is NULL");
    DeviceScope ds(c->device);
    VCT_CUDA(ds.err);
    cudaStream_t st = as_stream(stream);
    LearnedParams L;
    vct_status s = learned_setup(c, g, eye, st, L);
    if (s != VCT_OK) return s;
    L.out = reinterpret_cast<float4*>(irradiance);
    launch_trace16(L, false, c->num_sms, st);
    VCT_CHECK_LAUNCH("16-cone trace");
    return VCT_OK;
}


vct_status vct_learned_trace_pixels(vct_ctx* c, vct_mlp* m, const vct_gbuffer* g, const float eye[3], float threshold,
                                    float* irradiance, int64_t* fallback_pixels, void* stream) {
    vct_status s = learned_check(c, m, irradiance, threshold);
    if (s != VCT_OK) return s;
    DeviceScope ds(c->device);
    VCT_CUDA(ds.err);
    cudaStream_t st = as_stream(stream);
    LearnedParams L;
    if ((s = learned_setup(c, g, eye, st, L)) != VCT_OK) return s;
    if ((s = learned_scratch(c, g->width, g->height, L)) != VCT_OK) return s;
    const bool fallback = !std::isinf(threshold);
    L.img = m->dev.img;
    L.bias = m->dev.bias;
    L.n = (long long)g->width * g->height;
    L.out = reinterpret_cast<float4*>(irradiance);
    L.threshold = threshold;
    L.status = m->status;
    if (!fallback) L.est = nullptr;
    VCT_CUDA(cudaMemsetAsync(L.count, 0, sizeof(uint32_t), st));
    if (fallback) VCT_CUDA(cudaMemsetAsync(L.frame_sums, 0, 2 * sizeof(float), st));
    launch_learned_features(L, st);
    VCT_CHECK_LAUNCH("learned features");
    launch_mlp_infer(L, m->num_sms, st);
    VCT_CHECK_LAUNCH("mlp inference");
    if (fallback) {
        launch_trace16_pixels(L, st);
        VCT_CHECK_LAUNCH("16-cone pixel fallback");
    }
    if (fallback_pixels) {
        uint32_t count = 0;
        VCT_CUDA(cudaMemcpyAsync(&count, L.count, sizeof count, cudaMemcpyDeviceToHost, st));
        if ((s = check_status(m, st)) != VCT_OK) return s;
        *fallback_pixels = fallback ? (int64_t)count : 0;
    }
    return VCT_OK;
}

vct_status vct_learned_trace(vct_ctx* c, vct_mlp* m, const vct_gbuffer* g, const float eye[3], float threshold,
                             float* irradiance, vct_learned_stats* stats, void* stream) {
    vct_status s = learned_check(c, m, irradiance, threshold);
    if (s != VCT_OK) return s;
    DeviceScope ds(c->device);
    VCT_CUDA(ds.err);
    cudaStream_t st = as_stream(stream);
    LearnedParams L;
    if ((s = learned_setup(c, g, eye, st, L)) != VCT_OK) return s;
    const long long W = g->width, H = g->height;
    const long long tiles = ((W + kLearnTile - 1) / kLearnTile) * ((H + kLearnTile - 1) / kLearnTile);
    if ((s = learned_scratch(c, W, H, L)) != VCT_OK) return s;
    L.est = nullptr;
    L.img = m->dev.img;
    L.bias = m->dev.bias;
    L.n = W * H;
    L.out = reinterpret_cast<float4*>(irradiance);
    L.threshold = std::isinf(threshold) ? 3.0e38f : threshold;
    L.status = m->status;
    VCT_CUDA(cudaMemsetAsync(L.count, 0, sizeof(uint32_t), st));
    launch_learned_features(L, st);
    VCT_CHECK_LAUNCH("learned features");
    launch_mlp_infer(L, m->num_sms, st);
    VCT_CHECK_LAUNCH("mlp inference");
    if (!std::isinf(threshold)) {
        launch_learned_probe(L, st);
        VCT_CHECK_LAUNCH("learned error probes");
        launch_trace16(L, true, c->num_sms, st);
        VCT_CHECK_LAUNCH("16-cone fallback");
    }
    if (stats) {
        std::vector<float> err((size_t)tiles);
        uint32_t count = 0;
        if (!std::isinf(threshold)) {
            VCT_CUDA(cudaMemcpyAsync(err.data(), L.tile_err, sizeof(float) * tiles, cudaMemcpyDeviceToHost, st));
            VCT_CUDA(cudaMemcpyAsync(&count, L.count, sizeof count, cudaMemcpyDeviceToHost, st));
        }
        if ((s = check_status(m, st)) != VCT_OK) return s;
        // Estimates are relative: a tile whose probes see almost no light can
        // report a huge one; each counts as at most 1 in the mean.
        double sum = 0.0, mx = 0.0;
        for (float e : err) {
            const double v = (double)e;
            sum += v < 1.0 ? v : 1.0;
            mx = v > mx ? v : mx;
        }
        stats->tiles = (int32_t)tiles;
        stats->fallback_tiles = (int32_t)count;
        stats->mean_tile_error = std::isinf(threshold) ? -1.0f : (float)(sum / (double)tiles);
        stats->max_tile_error = std::isinf(threshold) ? -1.0f : (float)mx;
    }
    return VCT_OK;
}

}  // extern "C"
