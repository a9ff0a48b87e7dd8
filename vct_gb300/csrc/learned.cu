// Learned indirect light (the "learned" configuration): a cheap two-cone
// quarter-resolution trace plus G-buffer features feed a small BF16 MLP
// (42-64-64-64-3, FP32 accumulation) that predicts the 16-cone full-resolution
// irradiance.  Inference and training run on the fifth-generation tensor
// cores (tcgen05.mma, accumulators in TMEM; umma.cuh).
//
// Compiled with --fmad=false: the cone marching (cone.cuh) writes its fused
// multiply-adds out.
#include "cone.cuh"
#include "umma.cuh"

namespace vct {

namespace {

using namespace umma;

// ------------------------------------------------------------ GEMM check
// One 128 x N x K BF16 GEMM through the tensor core: A (128 x K) and B (N x K)
// row-major in global memory, D = A B^T (128 x N, FP32) back to global.
// `swap` exchanges the two descriptor strides (a diagnostic of the layout
// convention; both variants stay inside the zero-filled operand regions).
constexpr int kCheckSmemA = 32768, kCheckSmemB = 16384;

__global__ void __launch_bounds__(128) umma_check_kernel(const uint16_t* __restrict__ A,
                                                          const uint16_t* __restrict__ B, int K, int N, int swap,
                                                          float* __restrict__ D, uint32_t* __restrict__ status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint8_t* sa = smem;
    uint8_t* sb = smem + kCheckSmemA;
    for (int i = threadIdx.x; i < (kCheckSmemA + kCheckSmemB) / 16; i += blockDim.x)
        reinterpret_cast<uint4*>(smem)[i] = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    for (int i = threadIdx.x; i < 128 * K; i += blockDim.x)
        *reinterpret_cast<uint16_t*>(sa + tile_offset(i / K, i % K, 128)) = A[i];
    for (int i = threadIdx.x; i < N * K; i += blockDim.x)
        *reinterpret_cast<uint16_t*>(sb + tile_offset(i / K, i % K, N)) = B[i];
    fence_async_smem();
    if (threadIdx.x == 0) {
        mbar_init(smem_u32(&mbar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(smem_u32(&tmem_base), 64);
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tbase = tmem_base;
    if (threadIdx.x == 0) {
        const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
        const uint32_t idesc = idesc_bf16_f32(128, N);
        for (int j = 0; j < K / 16; ++j) {
            const uint64_t da = swap ? smem_desc(a0 + j * 2 * 128 * 16, 128, 128 * 16) : tile_desc(a0, 128, j);
            const uint64_t db = swap ? smem_desc(b0 + j * 2 * N * 16, 128, N * 16) : tile_desc(b0, N, j);
            mma_bf16(tbase, da, db, idesc, j > 0 ? 1u : 0u);
        }
        commit(smem_u32(&mbar));
    }
    const int ok = __syncthreads_and(mbar_wait(smem_u32(&mbar), 0) ? 1 : 0);
    fence_after_sync();
    if (ok) {
        for (int c = 0; c < N; c += 16) {
            float v[16];
            tmem_ld16(tmem_addr(tbase, warp, c), v);
#pragma unroll
            for (int i = 0; i < 16; ++i) D[(32 * warp + lane) * N + c + i] = v[i];
        }
    } else if (threadIdx.x == 0) {
        atomicOr(status, 1u);
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tbase, 64);
}

}  // namespace

void launch_umma_check(const uint16_t* A, const uint16_t* B, int K, int N, int swap, float* D, uint32_t* status,
                       cudaStream_t s) {
    cudaFuncSetAttribute(umma_check_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kCheckSmemA + kCheckSmemB);
    umma_check_kernel<<<1, 128, kCheckSmemA + kCheckSmemB, s>>>(A, B, K, N, swap, D, status);
    note_launches(1);
}

}  // namespace vct
