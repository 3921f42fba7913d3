// Learned Poisson preconditioner: tensor-core (tcgen05) kernels.
//
// This translation unit holds the tcgen05 GEMM tile used by the preconditioner network's
// channel-mixing convolutions, and a check entry point that multiplies one tile so the
// operand layout can be verified against a host GEMM.
#include <cuda_bf16.h>
#include "pic_kernels.h"
#include "pic_tc.cuh"

namespace pic {

constexpr long long kTcWaitLimit = 1ll << 24;

// D (128 x N, FP32, row-major) = A (128 x K, bf16, row-major) * B^T (B: N x K, bf16, row-major)
// 128 threads; K a multiple of 16, N in {16, 32, 64, 128}
__global__ void __launch_bounds__(128) k_tc_gemm_tile(const __nv_bfloat16* __restrict__ A,
                                                      const __nv_bfloat16* __restrict__ B, float* __restrict__ D,
                                                      int N, int K, unsigned* err) {
    extern __shared__ __align__(128) unsigned char smem[];
    __nv_bfloat16* sA = reinterpret_cast<__nv_bfloat16*>(smem);
    const int slices = K / 16;
    __nv_bfloat16* sB = sA + slices * 128 * 16;
    __shared__ uint32_t tmem_base;
    __shared__ __align__(8) uint64_t bar;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int idx = tid; idx < 128 * K; idx += 128) {
        int m = idx / K, k = idx - m * K;
        sA[(k >> 4) * 2048 + tc_slice_offset(m, k & 15)] = A[idx];
    }
    for (int idx = tid; idx < N * K; idx += 128) {
        int nn = idx / K, k = idx - nn * K;
        sB[(k >> 4) * (N * 16) + tc_slice_offset(nn, k & 15)] = B[idx];
    }
    tc_fence_smem();
    const uint32_t ncols = N < 32 ? 32 : N;
    if (warp == 0) {
        tc_alloc(&tmem_base, ncols);
        tc_relinquish();
    }
    if (tid == 0) tc_mbar_init(&bar, 1);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tm = tmem_base;
    if (tid == 0) {
        const uint32_t idesc = tc_idesc_bf16(128, N);
        for (int s = 0; s < slices; s++)
            tc_mma_bf16(tm, tc_smem_desc(sA + s * 2048, 128, 256), tc_smem_desc(sB + s * N * 16, 128, 256), idesc,
                        s > 0 ? 1u : 0u);
        tc_commit(&bar);
    }
    bool ok = tc_mbar_wait(&bar, 0, kTcWaitLimit);
    if (!ok) {
        if (tid == 0) set_error(err, kErrBarrierTimeout);
        tc_mbar_wait(&bar, 0, kTcWaitLimit);  // bounded wait for the MMAs in flight before freeing TMEM
    }
    tc_fence_after();
    if (ok) {
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tc_ld16(tm + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
#pragma unroll
            for (int c = 0; c < 16; c++) D[(32 * warp + lane) * N + c0 + c] = v[c];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tc_dealloc(tm, ncols);
}

}  // namespace pic

using namespace pic;

// Multiplies one 128 x N tile on the tensor cores (device pointers, current device); used by the
// tests to check the tcgen05 operand layout.  Returns 0, 1 for bad sizes, 2 for a CUDA error,
// 5 when the MMA completion wait ran out.
extern "C" int pic_tc_gemm_check(const void* A, const void* B, void* D, int N, int K, void* stream) {
    if (!A || !B || !D || K <= 0 || K % 16 || K > 256 || (N != 16 && N != 32 && N != 64 && N != 128)) return 1;
    unsigned* err = nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMallocAsync((void**)&err, sizeof(unsigned), s) != cudaSuccess) return 2;
    cudaMemsetAsync(err, 0, sizeof(unsigned), s);
    size_t smem = (size_t)(K / 16) * (128 + N) * 16 * sizeof(__nv_bfloat16);
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_tc_gemm_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_tc_gemm_tile<<<1, 128, smem, s>>>((const __nv_bfloat16*)A, (const __nv_bfloat16*)B, (float*)D, N, K, err);
    unsigned h = 0;
    cudaMemcpyAsync(&h, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    cudaFreeAsync(err, s);
    if (e != cudaSuccess) return 2;
    return h ? 5 : 0;
}
