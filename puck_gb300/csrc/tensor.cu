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
#include "device_common.cuh"
#include "tcgen05.cuh"

namespace puck {
namespace {

constexpr unsigned long long kWaitNs = 500000000ull;  // 0.5 s for any tensor-core wait

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

// ---------------------------------------------------------------------------
// Sum-product inside pass on tensor cores: binary sums of a tile of 128 cells
// of one span, for the targets of one TMEM part (see DevTc).  For every coarse
// pair with rule blocks in the part, the CUDA cores build the pair's
// outer-product rows M_c[j*nz + k] = sum_s scale_s * A_s[Y_j] * B_s[Z_k] over
// each cell's live splits (FP32, rounded to BF16 into the A operand; a cell
// for which the pair is dead gets a zero row), the block weights are copied
// into the B operand, and one elected thread issues the MMAs that add
// A x B^T into the block's TMEM slot.  Two A/B buffers alternate, so the
// CUDA cores fill one while the tensor core reads the other.  The
// accumulator is read out once, gated per target by the cell mask, into the
// bot cells; launch_inside_span (tc_binary) then finishes the cells.
//
// Reference: the inside binary pass (src/main/scala/puck/parser/
// CLParser.scala:489-504) with the Real semiring's scaled products
// (src/main/java/puck/parser/gen/SimpleGenRuleMultiply.java:213-214).
struct TcCells {
  long long pbot[kTcRows];
  int sent[kTcRows], beg[kTcRows], len[kTcRows];
  float ps[kTcRows];
  int flag[kTcRows];                        // valid and unpruned
  int gate[kTcRows][kMaxMask];
  unsigned allow[kTcRows][kMaxLen / 32];    // NN: split b + 1 + i has both operand cells unpruned
  unsigned char allow1[kTcRows][4];         // NT, TN, TT
  unsigned m[kTcRows][kMaxLen / 32];        // this pair's live splits per cell
  int live[kTcRows];
  uint32_t taddr;
  int err;
  uint64_t bar[2], bar_fin;
};

// Operand cells of split i of cell r for a job; false if the split is out of
// range or not allowed (an operand cell pruned).
__device__ __forceinline__ bool split_cells(const TcCells& X, const DevBatch& B, int r, int job, int span, int i,
                                            int nsplit, long long& lc, long long& rc) {
  using namespace dev;
  lc = rc = 0;
  if (i >= nsplit) return false;
  const int b = X.beg[r], n = X.len[r], e = b + span;
  const long long off = B.cell_off[X.sent[r]], toff = off + tri(n);
  if (job == IN_NN) {
    lc = toff + chart_index(b, b + 1 + i, n);
    rc = toff + chart_index(b + 1 + i, e, n);
    return (X.allow[r][i >> 5] >> (i & 31)) & 1;
  }
  if (job == IN_NT) {
    lc = toff + chart_index(b, e - 1, n);
    rc = off + chart_index(e - 1, e, n);
    return X.allow1[r][0];
  }
  lc = off + chart_index(b, b + 1, n);
  if (job == IN_TN) {
    rc = toff + chart_index(b + 1, e, n);
    return X.allow1[r][1];
  }
  rc = off + chart_index(b + 1, e, n);
  return X.allow1[r][2];
}

constexpr int kTcRounds = 3;  // outer-product tasks per lane: ny * ceil(nz / 4) <= 96

// per warp: two splits' staged member values of A_s and B_s
__shared__ __align__(16) float g_stage[kTcThreads / 32][2][2][32];

__global__ void __launch_bounds__(kTcThreads, 1)
    k_inside_tc(DevLevel L, DevTc T, DevBatch B, int span, const int* cells, int ncells, DevMask M, float* inside,
                DevLive V, Counters C) {
  using namespace dev;
  extern __shared__ __align__(1024) unsigned char sm_raw[];
  __shared__ TcCells X;
  const int cs = L.cell_size, ms = L.mask_size, h = blockIdx.y;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const size_t abytes = (size_t)kTcRows * T.max_kpad * 2;
  unsigned char* sA[2] = {sm_raw, sm_raw + abytes};
  unsigned char* sB[2] = {sm_raw + 2 * abytes, sm_raw + 2 * abytes + T.bcap};
  // --- the tile's cells ----------------------------------------------------
  if (tid < kTcRows) {
    const int c = blockIdx.x * kTcRows + tid;
    const bool valid = c < ncells;
    const int s = valid ? cells[2 * c] : 0, b = valid ? cells[2 * c + 1] : 0;
    const int n = valid ? B.len[s] : 0, e = b + span;
    const long long off = valid ? B.cell_off[s] : 0, toff = off + tri(n);
    const long long pbot = valid ? off + chart_index(b, e, n) : 0;
    const bool f = valid && mask_any(M, pbot);
    X.pbot[tid] = pbot;
    X.sent[tid] = s;
    X.beg[tid] = b;
    X.len[tid] = n;
    X.flag[tid] = f;
    X.ps[tid] = f ? scale_of(M.iscale, pbot) : 0.f;
    for (int i = 0; i < ms; ++i) X.gate[tid][i] = f && M.bits ? M.bits[pbot * ms + i] : -1;
    for (int w = 0; w < kMaxLen / 32; ++w) X.allow[tid][w] = 0u;
    if (f) {
      auto BOT = [&](int x, int y) { return off + chart_index(x, y, n); };
      auto TOP = [&](int x, int y) { return toff + chart_index(x, y, n); };
      for (int sp = b + 1; sp < e; ++sp)
        if (mask_any(M, TOP(b, sp)) && mask_any(M, TOP(sp, e))) X.allow[tid][(sp - b - 1) >> 5] |= 1u << ((sp - b - 1) & 31);
      X.allow1[tid][0] = mask_any(M, TOP(b, e - 1)) && mask_any(M, BOT(e - 1, e));
      X.allow1[tid][1] = mask_any(M, BOT(b, b + 1)) && mask_any(M, TOP(b + 1, e));
      X.allow1[tid][2] = span == 2 && mask_any(M, BOT(b, b + 1)) && mask_any(M, BOT(b + 1, e));
    } else {
      X.allow1[tid][0] = X.allow1[tid][1] = X.allow1[tid][2] = 0;
    }
  }
  // a wait of an earlier CTA gave up: this launch's results are void
  if (tid == 0) X.err = *reinterpret_cast<volatile int*>(T.err);
  __syncthreads();
  if (X.err) {
    if (tid < kTcRows && X.flag[tid] && C.status) C.status[X.sent[tid]] = 5;  // PUCK_ERR_DEVICE_TIMEOUT
    return;
  }
  if (warp == 0) tc::tmem_alloc(&X.taddr, T.ncols);
  if (tid == 0) {
    tc::mbar_init(&X.bar[0], 1);
    tc::mbar_init(&X.bar[1], 1);
    tc::mbar_init(&X.bar_fin, 1);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = X.taddr;
  // --- zero the accumulator --------------------------------------------------
  {
    const int q = warp & 3, chunk = warp >> 2, per = T.ncols / (kTcThreads / 128);
    for (int c = chunk * per; c < (chunk + 1) * per; c += 16) tc::tmem_st16_zero(taddr + ((uint32_t)(q * 32) << 16) + c);
    tc::tmem_wait_st();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  // --- the part's pairs -------------------------------------------------------
  const uint32_t idesc = tc::idesc_bf16_f32(kTcRows, T.slot_w);
  unsigned ncommit[2] = {0u, 0u};
  int it = 0;
  bool issued = false;
  for (int e = T.part_off[h]; e < T.part_off[h + 1]; ++e) {
    const int4 tp = __ldg(T.tpair + e);
    const int job = tp.x & 3, p = tp.x >> 2, kpad = tp.y, nb = tp.w - tp.z;
    if (job == IN_TT && span != 2) continue;
    const DevJob& J = L.jobs[job];
    const int buf = it & 1;
    if (ncommit[buf] && !X.err && !tc::mbar_wait(&X.bar[buf], (ncommit[buf] - 1) & 1, kWaitNs)) {
      atomicExch(&X.err, 1);
      atomicExch(T.err, 1);
    }
    tc::fence_after_sync();
    // B operands of the entry's blocks, contiguous in bmat
    {
      const uint4* src = reinterpret_cast<const uint4*>(T.bmat + __ldg(T.tpair_b + e));
      uint4* dst = reinterpret_cast<uint4*>(sB[buf]);
      const int n16 = nb * T.slot_w * kpad * 2 / 16;
      for (int i = tid; i < n16; i += kTcThreads) dst[i] = __ldg(src + i);
    }
    // A operand: one row per cell
    const int key = __ldg(J.pair_key + p);
    const int ca = key & 255, cb = (key >> 8) & 255;
    const int* aoff = J.a_is_t ? L.t_mem_off : L.nt_mem_off;
    const int* amem = J.a_is_t ? L.t_mem : L.nt_mem;
    const int* boff = J.b_is_t ? L.t_mem_off : L.nt_mem_off;
    const int* bmem = J.b_is_t ? L.t_mem : L.nt_mem;
    const int a0 = __ldg(aoff + ca), ny = __ldg(aoff + ca + 1) - a0;
    const int b0 = __ldg(boff + cb), nz = __ldg(boff + cb + 1) - b0;
    const int kk = ny * nz, nkq = (nz + 3) >> 2, ntask = ny * nkq;
    const int* pg = T.tpair_gate + (size_t)e * ms;
    // phase 1: per cell, the live splits of this pair.  A warp takes eight
    // cells and issues all their liveness loads before the first ballot.
    unsigned pgw[kMaxMask];
#pragma unroll
    for (int w = 0; w < kMaxMask; ++w) pgw[w] = w < ms ? (unsigned)__ldg(pg + w) : 0u;
    {
      constexpr int kPer = kTcRows / (kTcThreads / 32);
      const int nsplit = job == IN_NN ? span - 1 : 1;
      for (int ch = 0; ch < nsplit; ch += 32) {
        bool ok[kPer];
        int lw[kPer], rw[kPer];
#pragma unroll
        for (int i = 0; i < kPer; ++i) {
          const int r = warp * kPer + i;
          bool on = X.flag[r] != 0;
          if (on && M.bits) {
            bool hit = false;
#pragma unroll
            for (int w = 0; w < kMaxMask; ++w) hit |= w < ms && (pgw[w] & (unsigned)X.gate[r][w]) != 0;
            on = hit;
          }
          long long lc = 0, rc = 0;
          ok[i] = on && split_cells(X, B, r, job, span, ch + lane, nsplit, lc, rc);
          lw[i] = ok[i] ? __ldg(V.in + lc * ms + (ca >> 5)) : 0;
          rw[i] = ok[i] ? __ldg(V.in + rc * ms + (cb >> 5)) : 0;
        }
#pragma unroll
        for (int i = 0; i < kPer; ++i) {
          const int r = warp * kPer + i;
          const unsigned m = __ballot_sync(kFull, ok[i] && ((lw[i] >> (ca & 31)) & 1) && ((rw[i] >> (cb & 31)) & 1));
          if (lane == 0) {
            X.m[r][ch >> 5] = m;
            X.live[r] = (ch == 0 ? 0 : X.live[r]) | (m != 0);
          }
        }
      }
    }
    __syncthreads();
    // phase 2: (live cell, task round) items over all warps; dead rows zeroed
    unsigned lm[kTcRows / 32];
    int nlive = 0;
#pragma unroll
    for (int i = 0; i < kTcRows / 32; ++i) {
      lm[i] = __ballot_sync(kFull, X.live[i * 32 + lane] != 0);
      nlive += __popc(lm[i]);
    }
    // the pair's member indices, one per lane (rows of A_s and B_s it stages)
    const int my_a = lane < ny ? __ldg(amem + a0 + lane) : -1;
    const int my_b = lane < nz ? __ldg(bmem + b0 + lane) : -1;
    const int nrounds = (ntask + 31) >> 5;
    float(*stg)[2][32] = g_stage[warp];  // [split][A or B][member]
    for (int k = warp; k < nlive; k += kTcThreads / 32) {
      int r = 0;
      for (int i = 0, acc0 = 0; i < kTcRows / 32; ++i) {
        const int c = __popc(lm[i]);
        if (k < acc0 + c) {
          unsigned mm = lm[i];
          for (int z = acc0; z < k; ++z) mm &= mm - 1;  // drop the live cells before the k-th
          r = i * 32 + __ffs(mm) - 1;
          break;
        }
        acc0 += c;
      }
      float acc[kTcRounds][4];
#pragma unroll
      for (int u = 0; u < kTcRounds; ++u)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[u][q] = 0.f;
      const int nsplit = job == IN_NN ? span - 1 : 1;
      for (int ch = 0; ch < nsplit; ch += 32) {
        const unsigned m = X.m[r][ch >> 5];
        if (!m) continue;
        long long lc = 0, rc = 0;
        float scl = 0.f;
        if ((m >> lane) & 1) {
          split_cells(X, B, r, job, span, ch + lane, nsplit, lc, rc);
          scl = __expf(-X.ps[r] + scale_of(M.iscale, lc) + scale_of(M.iscale, rc));
        }
        const int lci = (int)lc, rci = (int)rc;
        // two live splits per step: each lane stages one member value of
        // A_s and of B_s (scaled), then computes its tasks from shared memory
        for (unsigned mm = m; mm;) {
          const int s0 = __ffs(mm) - 1;
          mm &= mm - 1;
          const bool two = mm != 0;
          const int s1 = two ? __ffs(mm) - 1 : s0;
          if (two) mm &= mm - 1;
          const long long L0 = __shfl_sync(kFull, lci, s0), R0 = __shfl_sync(kFull, rci, s0);
          const long long L1 = __shfl_sync(kFull, lci, s1), R1 = __shfl_sync(kFull, rci, s1);
          const float sc0 = __shfl_sync(kFull, scl, s0), sc1 = __shfl_sync(kFull, scl, s1);
          const float av0 = my_a >= 0 ? __ldg(inside + L0 * cs + my_a) * sc0 : 0.f;
          const float bv0 = my_b >= 0 ? __ldg(inside + R0 * cs + my_b) : 0.f;
          const float av1 = two && my_a >= 0 ? __ldg(inside + L1 * cs + my_a) * sc1 : 0.f;
          const float bv1 = two && my_b >= 0 ? __ldg(inside + R1 * cs + my_b) : 0.f;
          stg[0][0][lane] = av0;
          stg[0][1][lane] = bv0;
          stg[1][0][lane] = av1;
          stg[1][1][lane] = bv1;
          __syncwarp();
#pragma unroll
          for (int u = 0; u < kTcRounds; ++u) {
            const int t = lane + 32 * u;
            if (u < nrounds && t < ntask) {
              const int j = t / nkq, k0 = (t - j * nkq) * 4;
              const float x0 = stg[0][0][j], x1 = stg[1][0][j];
              const float4 y0 = *reinterpret_cast<const float4*>(&stg[0][1][k0]);
              const float4 y1 = *reinterpret_cast<const float4*>(&stg[1][1][k0]);
              acc[u][0] = fmaf(x1, y1.x, fmaf(x0, y0.x, acc[u][0]));
              acc[u][1] = fmaf(x1, y1.y, fmaf(x0, y0.y, acc[u][1]));
              acc[u][2] = fmaf(x1, y1.z, fmaf(x0, y0.z, acc[u][2]));
              acc[u][3] = fmaf(x1, y1.w, fmaf(x0, y0.w, acc[u][3]));
            }
          }
          __syncwarp();
        }
      }
      unsigned char* row0 = sA[buf];
#pragma unroll
      for (int u = 0; u < kTcRounds; ++u) {
        const int t = lane + 32 * u;
        if (u < nrounds && t < ntask) {
          const int j = t / nkq, k0 = (t - j * nkq) * 4;
#pragma unroll
          for (int q = 0; q < 4; ++q)
            if (k0 + q < nz)
              *reinterpret_cast<__nv_bfloat16*>(row0 + tc::tile_offset(r, j * nz + k0 + q, kpad)) =
                  __float2bfloat16_rn(acc[u][q]);
        }
      }
      for (int jk = kk + lane; jk < kpad; jk += 32)
        *reinterpret_cast<__nv_bfloat16*>(row0 + tc::tile_offset(r, jk, kpad)) = __float2bfloat16_rn(0.f);
    }
    {
      const int c8n = kpad >> 3;
      for (int i = tid; i < kTcRows * c8n; i += kTcThreads) {
        const int r = i / c8n, c8 = i - r * c8n;
        if (!X.live[r])
          *reinterpret_cast<uint4*>(sA[buf] + ((r >> 3) * c8n + c8) * 128 + (r & 7) * 16) = make_uint4(0, 0, 0, 0);
      }
    }
    const int local_any = nlive > 0;
    tc::fence_async_smem();
    tc::fence_before_sync();
    const int any = __syncthreads_or(local_any);
    tc::fence_after_sync();
    if (!any) continue;
    if (tid == 0) {
      const uint32_t abase = tc::smem_u32(sA[buf]), bbase = tc::smem_u32(sB[buf]);
      const uint32_t sbo = (uint32_t)kpad * 16, bstride = (uint32_t)T.slot_w * kpad * 2;
      for (int i = 0; i < nb; ++i) {
        const uint32_t d = taddr + (uint32_t)(__ldg(T.tblk + tp.z + i) * T.slot_w);
        for (int k16 = 0; k16 < kpad / 16; ++k16)
          tc::mma_bf16(d, tc::smem_desc(abase + k16 * 256, 128, sbo),
                       tc::smem_desc(bbase + i * bstride + k16 * 256, 128, sbo), idesc, 1u);
      }
      tc::mma_commit(&X.bar[buf]);
    }
    ++ncommit[buf];
    ++it;
    issued = true;
  }
  // --- read out ---------------------------------------------------------------
  if (issued) {
    if (tid == 0) tc::mma_commit(&X.bar_fin);
    if (!tc::mbar_wait(&X.bar_fin, 0, kWaitNs)) {
      atomicExch(&X.err, 1);
      atomicExch(T.err, 1);
    }
  }
  tc::fence_after_sync();
  __syncthreads();
  const bool failed = X.err != 0;
  {
    const int q = warp & 3, chunk = warp >> 2, per = T.ncols / (kTcThreads / 128), r = q * 32 + lane;
    const bool mine = X.flag[r] && !failed;
    for (int c = chunk * per; c < (chunk + 1) * per; c += 16) {
      float v[16];
      tc::tmem_ld16(taddr + ((uint32_t)(q * 32) << 16) + c, v);
      if (!mine) continue;
      float* row = inside + X.pbot[r] * cs;
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int t = __ldg(T.col_tgt + h * T.ncols + c + i);
        if (t < 0) continue;
        bool g = true;
        if (M.bits) {
          g = false;
          for (int w = 0; w < ms; ++w) g |= (__ldg(T.tgt_gate + t * ms + w) & X.gate[r][w]) != 0;
        }
        row[t] = g ? v[i] : 0.f;
      }
    }
    if (h == 0 && chunk == 0 && mine)
      for (int u = 0; u < T.n_uncovered; ++u) inside[X.pbot[r] * cs + __ldg(T.uncovered + u)] = 0.f;
    if (failed && tid < kTcRows && X.flag[tid] && C.status) C.status[X.sent[tid]] = 5;  // PUCK_ERR_DEVICE_TIMEOUT
  }
  // a failed wait: the MMAs may still be running; give them another bounded
  // wait before the columns are freed
  if (failed && issued) tc::mbar_wait(&X.bar_fin, 0, kWaitNs);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, T.ncols);
}

}  // namespace

size_t tc_static_smem_bytes() { return sizeof(TcCells) + sizeof(g_stage); }

size_t tc_smem_bytes(const DevTc& T) { return 2 * (size_t)kTcRows * T.max_kpad * 2 + 2 * (size_t)T.bcap; }

cudaError_t launch_inside_tc(const DevLevel& L, const DevTc& T, const DevBatch& B, int span, const int* cells,
                             int ncells, const DevMask& M, float* inside, DevLive V, Counters C, cudaStream_t st) {
  if (ncells <= 0 || span < 2) return cudaSuccess;
  const size_t smem = tc_smem_bytes(T);
  if (cudaError_t e = cudaFuncSetAttribute(k_inside_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      e != cudaSuccess)
    return e;
  const dim3 grid((unsigned)((ncells + kTcRows - 1) / kTcRows), (unsigned)T.nparts);
  k_inside_tc<<<grid, kTcThreads, smem, st>>>(L, T, B, span, cells, ncells, M, inside, V, C);
  return cudaGetLastError();
}

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
