// C ABI of the learned path (include/vct.h): the tensor-core GEMM check, the
// MLP object, the cheap and the 16-cone traces and the learned frame.
#include <cstring>
#include <string>

#include "host.h"

using namespace vct;
using namespace vct::host;

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

}  // extern "C"
