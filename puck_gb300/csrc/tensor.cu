// Tensor-core (tcgen05) parts of the library.
//
// puck_tc_selftest: one CTA multiplies a 128 x k BF16 tile by a k x n BF16
// tile into FP32 through shared memory, one tcgen05.mma per 16 of k, a TMEM
// accumulator and tcgen05.ld.  It is the building block of the sum-product
// rule application and lets a caller check the tensor-core path of a device
// against a host product before parsing with it.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "../../include/puck_gpu.h"
#include "puck_internal.h"
#include "tcgen05.cuh"

namespace puck {
namespace {

constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s for any tensor-core wait

__device__ __forceinline__ int pow2_cols(int n) {
  int c = 32;
  while (c < n) c <<= 1;
  return c;
}

// D[128 x n] = A[128 x k] * B[n x k]^T; A and B row-major BF16, D row-major
// FP32.  k a multiple of 16 (<= 256), n a multiple of 16 (<= 256).  128
// threads.  err: 0 ok, 1 the MMA did not complete within the wait limit.
__global__ void __launch_bounds__(128, 1)
    k_tc_selftest(const __nv_bfloat16* A, const __nv_bfloat16* B, float* D, int k, int n, int* err) {
  extern __shared__ __align__(1024) unsigned char sm_raw[];
  __shared__ uint64_t bar;
  __shared__ uint32_t taddr_s;
  unsigned char* sA = sm_raw;
  unsigned char* sB = sm_raw + 128 * k * 2;
  for (int i = threadIdx.x; i < 128 * k; i += blockDim.x) {
    const int r = i / k, kk = i - r * k;
    *reinterpret_cast<__nv_bfloat16*>(sA + tc::tile_offset(r, kk, k)) = A[i];
  }
  for (int i = threadIdx.x; i < n * k; i += blockDim.x) {
    const int r = i / k, kk = i - r * k;
    *reinterpret_cast<__nv_bfloat16*>(sB + tc::tile_offset(r, kk, k)) = B[i];
  }
  const int ncols = pow2_cols(n);
  if (threadIdx.x < 32) tc::tmem_alloc(&taddr_s, ncols);
  if (threadIdx.x == 0) tc::mbar_init(&bar, 1);
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = taddr_s;
  if (threadIdx.x == 0) {
    const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB);
    const uint32_t sbo = (uint32_t)k * 16, idesc = tc::idesc_bf16_f32(128, n);
    for (int s = 0; s < k / 16; ++s)
      tc::mma_bf16(taddr, tc::smem_desc(a0 + s * 256, 128, sbo), tc::smem_desc(b0 + s * 256, 128, sbo), idesc,
                   s > 0);
    tc::mma_commit(&bar);
  }
  const bool ok = tc::mbar_wait(&bar, 0, kWaitNs);
  tc::fence_after_sync();
  if (!ok) {
    if (threadIdx.x == 0) atomicExch(err, 1);
    tc::mbar_wait(&bar, 0, kWaitNs);  // its reads of shared memory may still be in flight
  } else {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, row = w * 32 + lane;
    for (int c0 = 0; c0 < n; c0 += 16) {
      float v[16];
      tc::tmem_ld16(taddr + ((uint32_t)(w * 32) << 16) + c0, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) D[row * n + c0 + i] = v[i];
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32) tc::tmem_dealloc(taddr, ncols);
}

}  // namespace
}  // namespace puck

extern "C" puck_status puck_tc_selftest(int32_t device, int32_t k, int32_t n, const uint16_t* a, const uint16_t* b,
                                        float* d) {
  if (!a || !b || !d || k <= 0 || k > 256 || k % 16 || n <= 0 || n > 256 || n % 16) {
    puck::set_last_error("puck_tc_selftest: k and n must be multiples of 16 in [16, 256]");
    return PUCK_ERR_INVALID_ARG;
  }
  __nv_bfloat16 *dA = nullptr, *dB = nullptr;
  float* dD = nullptr;
  int* dErr = nullptr;
  puck_status st = PUCK_OK;
  auto fail = [&](cudaError_t e) {
    if (e != cudaSuccess && st == PUCK_OK) {
      puck::set_last_error(std::string("puck_tc_selftest: ") + cudaGetErrorString(e));
      st = PUCK_ERR_CUDA;
    }
    return e != cudaSuccess;
  };
  const size_t smem = (size_t)(128 + n) * k * 2;
  int herr = 0;
  if (!fail(cudaSetDevice(device)) && !fail(cudaMalloc(&dA, 128 * k * 2)) && !fail(cudaMalloc(&dB, (size_t)n * k * 2)) &&
      !fail(cudaMalloc(&dD, (size_t)128 * n * 4)) && !fail(cudaMalloc(&dErr, 4)) &&
      !fail(cudaMemcpy(dA, a, 128 * k * 2, cudaMemcpyHostToDevice)) &&
      !fail(cudaMemcpy(dB, b, (size_t)n * k * 2, cudaMemcpyHostToDevice)) && !fail(cudaMemset(dErr, 0, 4)) &&
      !fail(cudaFuncSetAttribute(puck::k_tc_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem))) {
    puck::k_tc_selftest<<<1, 128, smem>>>(dA, dB, dD, k, n, dErr);
    if (!fail(cudaGetLastError()) && !fail(cudaDeviceSynchronize()) &&
        !fail(cudaMemcpy(d, dD, (size_t)128 * n * 4, cudaMemcpyDeviceToHost)) &&
        !fail(cudaMemcpy(&herr, dErr, 4, cudaMemcpyDeviceToHost)) && herr) {
      puck::set_last_error("puck_tc_selftest: the tensor-core wait gave up");
      st = PUCK_ERR_DEVICE_TIMEOUT;
    }
  }
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dD);
  cudaFree(dErr);
  return st;
}
