// Max-constituent (MBR) tree decoding into caller-owned device buffers, with
// no device allocation at all.
//
// Some callers cannot allocate device memory at the point where they decode:
// a JVM host that runs the parser inside a device arena its own pool carved
// out up front (every byte of the device already belongs to that pool), or a
// serving loop whose request path must never enter the CUDA allocator (a
// cudaMalloc can synchronize the device and stall every stream).  puck_parse's MBR path
// allocates its dynamic-programming tables with the rest of its batch
// buffers; this entry point runs the same per-sentence decode
// (mbr_decode_sentence) but keeps that scratch -- the sentences' lengths and
// offsets and the tables -- in one fixed-size array in the library's device
// memory.  Every GPU that loads the library holds the array until the process
// exits.
//
// The array's address is resolved once per device with cudaGetSymbolAddress,
// with that device current, by the first call made on it; make that first
// call before any stream capture.  Calls share the array: two calls whose
// work overlaps on the GPU (on different streams, or from different host
// threads) race on it and must be serialized by the caller.  Nothing in the
// array is read before the call writes it, so stale contents of an earlier
// call never leak into a result.

#include "mbr_dp.cuh"
#include "../../include/puck_gpu.h"

#include <cstddef>
#include <cstdint>
#include <mutex>
#include <string>

namespace {

constexpr int kStaticMaxSentences = 65536;
constexpr long long kStaticDpFloats = 4LL << 20;  // 16 MiB of tables: sum of 3 * (n+1)^2 over a call

struct StaticScratch {
  int lengths[kStaticMaxSentences];
  long long cell_off[kStaticMaxSentences + 1];
  long long node_off[kStaticMaxSentences + 1];
  long long dp_off[kStaticMaxSentences + 1];
  float dp[kStaticDpFloats];
};

__device__ __align__(256) StaticScratch g_mbr_static_scratch;

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
StaticScratch* g_scratch_ptr[kMaxDevices] = {nullptr};

// Exclusive prefix sums of the per-sentence cell, node and table sizes (one
// CTA walks the sentences in chunks of its size).
__global__ void k_static_offsets(StaticScratch* S, int nsent) {
  __shared__ long long part[3][1024];
  __shared__ long long carry[3];
  if (threadIdx.x < 3) carry[threadIdx.x] = 0;
  __syncthreads();
  for (int base = 0; base < nsent; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const long long n = i < nsent ? S->lengths[i] : 0;
    long long v[3] = {n * (n + 1), n > 0 ? 2 * n - 1 : 0, n > 0 ? 3 * (n + 1) * (n + 1) : 0};
    for (int k = 0; k < 3; ++k) part[k][threadIdx.x] = v[k];
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
      long long add[3] = {0, 0, 0};
      if ((int)threadIdx.x >= o)
        for (int k = 0; k < 3; ++k) add[k] = part[k][threadIdx.x - o];
      __syncthreads();
      for (int k = 0; k < 3; ++k) part[k][threadIdx.x] += add[k];
      __syncthreads();
    }
    if (i < nsent) {
      S->cell_off[i] = carry[0] + part[0][threadIdx.x] - v[0];
      S->node_off[i] = carry[1] + part[1][threadIdx.x] - v[1];
      S->dp_off[i] = carry[2] + part[2][threadIdx.x] - v[2];
    }
    __syncthreads();
    if (threadIdx.x == 0)
      for (int k = 0; k < 3; ++k) carry[k] += part[k][blockDim.x - 1];
    __syncthreads();
  }
}

__global__ void k_mbr_decode_static(const StaticScratch* S, int nsent, const float2* decode, const float* iscale,
                                    const float* oscale, int scaling, puck::DevNode* nodes) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsent) return;
  // the tables live in the file-scope array (reached here through S, whose
  // value the host resolved with cudaGetSymbolAddress)
  float* dp = const_cast<StaticScratch*>(S)->dp + S->dp_off[s];
  puck::dev::mbr_decode_sentence(S->lengths[s], S->cell_off[s], decode, iscale, oscale, scaling, dp,
                                 nodes + S->node_off[s]);
}

puck_status fail(puck_status st, const std::string& msg) {
  puck::set_last_error(msg);
  return st;
}

}  // namespace

extern "C" puck_status puck_mbr_decode_static(const float* cell_decode, const float* iscale, const float* oscale,
                                              const int32_t* lengths, int32_t nsent, puck_tree_node* nodes,
                                              void* stream) {
  if (nsent < 0 || (nsent > 0 && (!cell_decode || !lengths || !nodes)))
    return fail(PUCK_ERR_INVALID_ARG, "puck_mbr_decode_static: null argument or negative sentence count");
  if ((iscale == nullptr) != (oscale == nullptr))
    return fail(PUCK_ERR_INVALID_ARG, "puck_mbr_decode_static: give both scale arrays or neither");
  // the kernels read cell_decode as {score, symbol} pairs (8-byte loads)
  auto misaligned = [](const void* p, uintptr_t a) { return reinterpret_cast<uintptr_t>(p) % a != 0; };
  if (misaligned(cell_decode, 8) || misaligned(nodes, 4) || misaligned(iscale, 4) || misaligned(oscale, 4))
    return fail(PUCK_ERR_INVALID_ARG,
                "puck_mbr_decode_static: cell_decode must be 8-byte aligned, nodes and scales 4-byte aligned");
  if (nsent > kStaticMaxSentences)
    return fail(PUCK_ERR_INVALID_ARG, "puck_mbr_decode_static: more than " + std::to_string(kStaticMaxSentences) +
                                          " sentences in one call");
  long long dp = 0;
  for (int i = 0; i < nsent; ++i) {
    const long long n = lengths[i];
    if (n < 1 || n > puck::kMaxLen)
      return fail(PUCK_ERR_INVALID_ARG, "puck_mbr_decode_static: sentence " + std::to_string(i) + " has length " +
                                            std::to_string(n) + " (1.." + std::to_string(puck::kMaxLen) + ")");
    dp += 3 * (n + 1) * (n + 1);
  }
  if (dp > kStaticDpFloats)
    return fail(PUCK_ERR_INVALID_ARG, "puck_mbr_decode_static: the call needs " + std::to_string(dp) +
                                          " table floats, the fixed scratch holds " + std::to_string(kStaticDpFloats) +
                                          " (sum of 3*(n+1)^2 over the sentences); split the call");
  if (nsent == 0) return PUCK_OK;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(PUCK_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(PUCK_ERR_INVALID_ARG, "device ordinal out of range");
  StaticScratch* S = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_mbr_static_scratch);
      if (e != cudaSuccess)
        return fail(PUCK_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_scratch_ptr[dev] = static_cast<StaticScratch*>(p);
    }
    S = g_scratch_ptr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int* dev_lengths = reinterpret_cast<int*>(reinterpret_cast<char*>(S) + offsetof(StaticScratch, lengths));
  e = cudaMemcpyAsync(dev_lengths, lengths, (size_t)nsent * sizeof(int32_t), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return fail(PUCK_ERR_CUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
  k_static_offsets<<<1, 1024, 0, st>>>(S, nsent);
  k_mbr_decode_static<<<(nsent + 63) / 64, 64, 0, st>>>(S, nsent, reinterpret_cast<const float2*>(cell_decode),
                                                        iscale, oscale, iscale ? 1 : 0,
                                                        reinterpret_cast<puck::DevNode*>(nodes));
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(PUCK_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return PUCK_OK;
}
