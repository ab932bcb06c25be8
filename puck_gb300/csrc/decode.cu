// Decode-side kernels on sm_103a: pruning masks, scaling, Viterbi backtrace,
// MBR (max-constituent) decoding and root scores.
//
// Reference semantics restated (dlwh/puck paths):
//   masks         src/main/scala/puck/parser/gen/CLMaskKernels.scala:172-236
//   scaling       src/main/scala/puck/parser/gen/CLScalingKernels.scala:51-69
//   backtrace     src/main/scala/puck/parser/gen/CLViterbi.scala:383-605
//   MBR           src/main/scala/puck/parser/gen/CLMBRKernels.scala:118-170,
//                 src/main/scala/puck/parser/CLParser.scala:587-696
//   root scores   src/main/scala/puck/parser/gen/CLParserUtils.scala:64-78,
//                 CLParser.scala:189-206

#include "mbr_dp.cuh"

namespace puck {
namespace {

using namespace dev;

// Adds a block's count of fully pruned cells to the launch counter (every
// thread of the block calls this once).
__device__ __forceinline__ void flush_pruned(unsigned& block_pruned, unsigned long long* pruned) {
  __syncthreads();
  if (threadIdx.x == 0 && pruned && block_pruned) atomicAdd(pruned, (unsigned long long)block_pruned);
}

// ---------------------------------------------------------------------------
// Pruning masks: one warp per cell (max-marginal test against root + thresh).
// Cell c of sentence s (unit i of a per-cell work list).
struct CellRef { int s; long long c, first, last; };
__device__ __forceinline__ CellRef cell_ref(const DevBatch& B, const DevWork& W, int i) {
  const int k = entry_of(W, i);
  CellRef r;
  r.s = W.sent[k];
  const int n = B.len[r.s];
  r.first = B.cell_off[r.s];
  r.last = r.first + 2 * tri(n);
  r.c = r.first + (i - W.pref[k]);
  return r;
}

__global__ void k_masks(DevLevel L, DevBatch B, DevWork W, const float* inside, const float* outside, float thresh,
                        int* out, unsigned long long* pruned) {
  __shared__ unsigned block_pruned;
  if (threadIdx.x == 0) block_pruned = 0;
  __syncthreads();
  const long long unit = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (unit >= W.nunits) {
    flush_pruned(block_pruned, pruned);
    return;
  }
  const CellRef R = cell_ref(B, W, (int)unit);
  const int s = R.s;
  const long long c = R.c, first = R.first, last = R.last;
  const int cs = L.cell_size;
  const float root_score = inside[(last - 1) * cs + L.root];
  const float cutoff = root_score + thresh;
  const bool term = (c - first) < B.len[s];
  unsigned words[kMaxMask];
#pragma unroll
  for (int i = 0; i < kMaxMask; ++i) words[i] = 0u;
  for (int sym = lane; sym < L.num_syms; sym += 32) {
    const float score = inside[c * cs + sym] + outside[c * cs + sym];
    if (score >= cutoff) {
      const int f = term ? (sym < L.n_t ? L.t_coarse[sym] : 0) : (sym < L.n_nt ? L.nt_coarse[sym] : 0);
#pragma unroll
      for (int i = 0; i < kMaxMask; ++i)
        if ((f >> 5) == i) words[i] |= 1u << (f & 31);
    }
  }
  unsigned any = 0u;
#pragma unroll
  for (int i = 0; i < kMaxMask; ++i) {
    const unsigned v = __reduce_or_sync(kFull, words[i]);
    any |= v;
    if (lane == 0 && i < L.mask_size) out[c * L.mask_size + i] = (int)v;
  }
  if (lane == 0 && !any) atomicAdd(&block_pruned, 1u);  // no coarse symbol survives: the next level skips the cell
  flush_pruned(block_pruned, pruned);
}

// Per-cell log-scale: max over the cell, -9000 floor mapped to 0.
__global__ void k_scaling(int cs, DevBatch B, DevWork W, const float* chart, float* out) {
  const long long unit = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (unit >= W.nunits) return;
  const long long c = cell_ref(B, W, (int)unit).c;
  float m = -100000.0f;
  for (int k = lane; k < cs; k += 32) m = fmaxf(chart[c * cs + k], m);
  m = warp_reduce<SEMI_VITERBI>(m);
  if (lane == 0) out[c] = m < -9000.0f ? 0.f : m;
}

// ---------------------------------------------------------------------------
// Viterbi backtrace: one CTA per sentence, nodes in preorder.  Candidates are
// numbered in the reference's sequential scan order (NT, TN, TT, then NN by
// split) and compared with ">=", so the winner is the last candidate that
// attains the maximum; the CTA's threads split the candidates and a (score,
// sequence index) reduction recovers that order.
struct Best { float score; int idx; int a, b, code; };

__device__ __forceinline__ bool better(const Best& o, const Best& v) {
  return o.score > v.score || (o.score == v.score && o.idx > v.idx);
}

__device__ __forceinline__ Best warp_argmax_last(Best v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    Best w;
    w.score = __shfl_xor_sync(kFull, v.score, o);
    w.idx = __shfl_xor_sync(kFull, v.idx, o);
    w.a = __shfl_xor_sync(kFull, v.a, o);
    w.b = __shfl_xor_sync(kFull, v.b, o);
    w.code = __shfl_xor_sync(kFull, v.code, o);
    if (better(w, v)) v = w;
  }
  return v;
}

constexpr int kVitThreads = 256;

// CTA-wide argmax; every thread gets the result.
__device__ __forceinline__ Best block_argmax_last(Best v, Best* red) {
  v = warp_argmax_last(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();  // red is reused node after node
  if (lane == 0) red[warp] = v;
  __syncthreads();
  Best r = red[0];
  for (int w = 1; w < kVitThreads / 32; ++w)
    if (better(red[w], r)) r = red[w];
  return r;
}

__global__ void __launch_bounds__(kVitThreads) k_viterbi(DevLevel L, DevBatch B, DevWork W, int max_len,
                                                         const float* inside, DevNode* nodes) {
  extern __shared__ DevNode tn[];
  __shared__ Best red[kVitThreads / 32];
  const int k = blockIdx.x;
  if (k >= W.nent) return;
  const int s = W.sent[k];
  const int n = B.len[s];
  const int cs = L.cell_size;
  const float* ibot = inside + B.cell_off[s] * cs;
  const float* itop = ibot + tri(n) * cs;
  auto CELL = [&](const float* base, int x, int y) { return base + (long long)cs * chart_index(x, y, n); };
  const int nnt = L.n_nt;
  if (threadIdx.x == 0) { tn[0].top = L.root; tn[0].width = n; tn[0].bot = 0; tn[0].score = 0.f; }
  __syncthreads();
  int begin = 0;
  for (int p = 0; p < 2 * n - 1; ++p) {
    const DevNode nd = tn[p];
    const int width = nd.width, end = begin + width;
    int botSym = nd.bot;
    if (nd.top != -1) {
      const int uoff = (width == 1 ? 5 : 4) * nnt + nd.top;
      const float* child = CELL(ibot, begin, end);
      const int r0 = L.v_off[uoff], r1 = L.v_off[uoff + 1];
      Best bst{-30000.0f, -1, 0, 0, 0};
      for (int r = r0 + threadIdx.x; r < r1; r += kVitThreads) {
        const int c = L.v_left[r];
        const float scr = L.v_score[r] + child[c];
        if (scr >= bst.score) { bst.score = scr; bst.idx = r; bst.a = c; }
      }
      bst = block_argmax_last(bst, red);
      botSym = bst.idx < 0 ? 0 : bst.a;
      if (threadIdx.x == 0) { tn[p].bot = botSym; tn[p].score = bst.score; }
    }
    if (width == 1) {
      if (threadIdx.x == 0) tn[p].score = ibot[(long long)cs * begin + botSym];
      begin += 1;
    } else {
      // candidate t in [0, total): NT rules, TN rules, TT rules (width 2), then
      // (width - 1) copies of the NN rules, one per split in ascending order
      const int oNT = L.v_off[1 * nnt + botSym], nNT = L.v_off[1 * nnt + botSym + 1] - oNT;
      const int oTN = L.v_off[2 * nnt + botSym], nTN = L.v_off[2 * nnt + botSym + 1] - oTN;
      const int oTT = L.v_off[3 * nnt + botSym], nTT = width == 2 ? L.v_off[3 * nnt + botSym + 1] - oTT : 0;
      const int oNN = L.v_off[botSym], nNN = L.v_off[botSym + 1] - oNN;
      const int first = nNT + nTN + nTT;
      const int total = first + (width - 1) * nNN;
      const float* ntL = CELL(itop, begin, end - 1);
      const float* ntR = CELL(ibot, end - 1, end);
      const float* tnL = CELL(ibot, begin, begin + 1);
      const float* tnR = CELL(itop, begin + 1, end);
      const float* ttR = CELL(ibot, begin + 1, end);
      Best bst{-300000.0f, -1, 10, 10, begin + 1};
      for (int t = threadIdx.x; t < total; t += kVitThreads) {
        int r, code;
        const float *lc, *rc;
        if (t < nNT) { r = oNT + t; lc = ntL; rc = ntR; code = -1; }
        else if (t < nNT + nTN) { r = oTN + (t - nNT); lc = tnL; rc = tnR; code = -2; }
        else if (t < first) { r = oTT + (t - nNT - nTN); lc = tnL; rc = ttR; code = -3; }
        else {
          const int q = t - first, j = q / nNN;
          r = oNN + (q - j * nNN);
          code = begin + 1 + j;
          lc = CELL(itop, begin, code);
          rc = CELL(itop, code, end);
        }
        const int a = L.v_left[r], bb = L.v_right[r];
        const float scr = (L.v_score[r] + lc[a]) + rc[bb];
        if (scr >= bst.score) { bst.score = scr; bst.idx = t; bst.a = a; bst.b = bb; bst.code = code; }
      }
      bst = block_argmax_last(bst, red);
      if (bst.idx < 0) { bst.a = 10; bst.b = 10; bst.code = begin + 1; }
      if (threadIdx.x == 0) {
        tn[p].score = bst.score;
        int bestSplit = bst.code;
        const int cfg = bestSplit < 0 ? -bestSplit : 0;
        bestSplit = cfg == 0 ? bestSplit : (cfg == 2 ? begin + 1 : end - 1);
        DevNode& ln = tn[p + 1];
        DevNode& rn = tn[p + 2 * (bestSplit - begin)];
        if ((cfg >> 1) == 0) ln.top = bst.a; else { ln.top = -1; ln.bot = bst.a; }
        if ((cfg & 1) == 0) rn.top = bst.b; else { rn.top = -1; rn.bot = bst.b; }
        ln.width = bestSplit - begin;
        rn.width = end - bestSplit;
      }
    }
    __syncthreads();
  }
  DevNode* out = nodes + B.node_off[s];
  for (int q = threadIdx.x; q < 2 * n - 1; q += kVitThreads) out[q] = tn[q];
}

// ---------------------------------------------------------------------------
// MBR: per cell best coarse marginal (warp per cell), then a per-sentence
// max-constituent CKY with on-device extraction.
template <int S>
__global__ void k_mbr_cells(DevLevel L, DevBatch B, DevWork W, const float* inside, const float* outside,
                            float2* decode) {
  extern __shared__ float margs_all[];
  const long long unit = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  float* margs = margs_all + wib * L.n_coarse;
  if (unit >= W.nunits) return;
  for (int k = lane; k < L.n_coarse; k += 32) margs[k] = 0.f;
  __syncwarp();
  const CellRef R = cell_ref(B, W, (int)unit);
  const int s = R.s;
  const long long c = R.c, first = R.first, last = R.last;
  const int cs = L.cell_size;
  const float root_score = inside[(last - 1) * cs + L.root];
  const bool term = (c - first) < B.len[s];
  for (int k = lane; k < L.num_syms; k += 32) {
    const int proj = term ? (k < L.n_t ? L.t_coarse[k] : 0) : (k < L.n_nt ? L.nt_coarse[k] : 0);
    const float in = inside[c * cs + k], ou = outside[c * cs + k];
    const float v = S == SEMI_LOGSUM ? __expf(in - root_score + ou) : in / root_score * ou;
    atomicAdd(&margs[proj], v);
  }
  __syncwarp();
  float best = -CUDART_INF_F;
  int bsym = -1;
  for (int k = lane; k < L.n_coarse; k += 32)
    if (margs[k] > best) { best = margs[k]; bsym = k; }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    float ob = __shfl_xor_sync(kFull, best, o);
    int oy = __shfl_xor_sync(kFull, bsym, o);
    if (ob > best || (ob == best && oy >= 0 && (bsym < 0 || oy < bsym))) { best = ob; bsym = oy; }
  }
  if (lane == 0) decode[c] = make_float2(best, __int_as_float(bsym));
}

__global__ void k_mbr_decode(DevBatch B, DevWork W, DevMask M, int scaling, const float2* decode,
                             const long long* mbr_off, float* scratch, DevNode* nodes) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= W.nent) return;
  const int s = W.sent[k];
  mbr_decode_sentence(B.len[s], B.cell_off[s], decode, M.iscale, M.oscale, scaling, scratch + mbr_off[s],
                      nodes + B.node_off[s]);
}

// log Z per sentence (CLParser.scala:189-206), accumulated in FP64.
__global__ void k_root_scores(DevLevel L, DevBatch B, DevWork W, DevMask M, const float* inside,
                              const double* part_scale, float* log_z) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= W.nent) return;
  const int s = W.sent[k];
  const int n = B.len[s];
  const long long root_cell = B.cell_off[s] + tri(n) + chart_index(0, n, n);
  const float v = inside[root_cell * L.cell_size + L.root];
  if (L.semiring == SEMI_REAL) {
    const double sc = M.iscale ? (double)M.iscale[root_cell] : 0.0;
    log_z[s] = (float)(log((double)v) + sc + part_scale[s]);
  } else {
    log_z[s] = v;
  }
}

template <class K>
cudaError_t set_smem(K kernel, size_t bytes) {
  // static + dynamic shared memory above 48 KB needs the opt-in, whatever
  // the dynamic part alone is
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

}  // namespace

cudaError_t launch_masks(const DevLevel& L, const DevBatch& B, const DevWork& W, const float* inside,
                         const float* outside, float thresh, int* masks_out, cudaStream_t st,
                         unsigned long long* pruned) {
  const int blocks = (int)((W.nunits * 32 + 255) / 256);
  if (blocks == 0) return cudaSuccess;
  k_masks<<<blocks, 256, 0, st>>>(L, B, W, inside, outside, thresh, masks_out, pruned);
  return cudaGetLastError();
}

cudaError_t launch_scaling(int cell_size, const DevBatch& B, const DevWork& W, const float* chart, float* out,
                           cudaStream_t st) {
  const int blocks = (int)((W.nunits * 32 + 255) / 256);
  if (blocks == 0) return cudaSuccess;
  k_scaling<<<blocks, 256, 0, st>>>(cell_size, B, W, chart, out);
  return cudaGetLastError();
}

cudaError_t launch_viterbi(const DevLevel& L, const DevBatch& B, const DevWork& W, int max_len, const float* inside,
                           DevNode* nodes, cudaStream_t st) {
  if (W.nent == 0) return cudaSuccess;
  const size_t smem = (size_t)(2 * max_len - 1) * sizeof(DevNode);
  if (cudaError_t e = set_smem(k_viterbi, smem); e != cudaSuccess) return e;
  k_viterbi<<<W.nent, kVitThreads, smem, st>>>(L, B, W, max_len, inside, nodes);
  return cudaGetLastError();
}

cudaError_t launch_mbr_cells(const DevLevel& L, const DevBatch& B, const DevWork& W, const float* inside,
                             const float* outside, float2* decode, cudaStream_t st) {
  const int wpb = 8;
  const int blocks = (int)((W.nunits + wpb - 1) / wpb);
  if (blocks == 0) return cudaSuccess;
  const size_t smem = (size_t)wpb * L.n_coarse * sizeof(float);
  if (L.semiring == SEMI_LOGSUM)
    k_mbr_cells<SEMI_LOGSUM><<<blocks, wpb * 32, smem, st>>>(L, B, W, inside, outside, decode);
  else
    k_mbr_cells<SEMI_REAL><<<blocks, wpb * 32, smem, st>>>(L, B, W, inside, outside, decode);
  return cudaGetLastError();
}

cudaError_t launch_mbr_decode(const DevBatch& B, const DevWork& W, const DevMask& M, int scaling,
                              const float2* decode, const long long* mbr_off, float* scratch, DevNode* nodes,
                              cudaStream_t st) {
  const int blocks = (W.nent + 63) / 64;
  if (blocks == 0) return cudaSuccess;
  k_mbr_decode<<<blocks, 64, 0, st>>>(B, W, M, scaling, decode, mbr_off, scratch, nodes);
  return cudaGetLastError();
}

cudaError_t launch_root_scores(const DevLevel& L, const DevBatch& B, const DevWork& W, const DevMask& M,
                               const float* inside, const double* part_scale, float* log_z, cudaStream_t st) {
  const int blocks = (W.nent + 127) / 128;
  if (blocks == 0) return cudaSuccess;
  k_root_scores<<<blocks, 128, 0, st>>>(L, B, W, M, inside, part_scale, log_z);
  return cudaGetLastError();
}

}  // namespace puck
