// Decode-side kernels on sm_103a: pruning masks, scaling, Viterbi backtrace,
// MBR (max-constituent) decoding and root scores.
//
// Reference semantics restated (dlwh/puck paths):
//   masks         src/main/scala/puck/parser/gen/CLMaskKernels.scala:172-236
//   scaling       src/main/scala/puck/parser/gen/CLScalingKernels.scala:225-243
//   backtrace     src/main/scala/puck/parser/gen/CLViterbi.scala:383-605
//   MBR           src/main/scala/puck/parser/gen/CLMBRKernels.scala:118-170,
//                 src/main/scala/puck/parser/CLParser.scala:587-696
//   root scores   src/main/scala/puck/parser/gen/CLParserUtils.scala:305-316,
//                 CLParser.scala:189-206

#include "mbr_dp.cuh"

namespace puck {
namespace {

using namespace dev;

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
                        int* out) {
  const long long unit = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (unit >= W.nunits) return;
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
#pragma unroll
  for (int i = 0; i < kMaxMask; ++i) {
    const unsigned v = __reduce_or_sync(kFull, words[i]);
    if (lane == 0 && i < L.mask_size) out[c * L.mask_size + i] = (int)v;
  }
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
// Viterbi backtrace: one warp per sentence.  Candidates are scanned in the
// reference's sequential order (NT, TN, TT, NN by split) with ">=" ties, so
// the winner is the last candidate that attains the maximum; lanes split the
// rule lists and a (score, sequence index) reduction recovers that order.
struct Best { float score; int idx; int a, b, code; };

__device__ __forceinline__ Best warp_argmax_last(Best v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    float os = __shfl_xor_sync(kFull, v.score, o);
    int oi = __shfl_xor_sync(kFull, v.idx, o);
    int oa = __shfl_xor_sync(kFull, v.a, o);
    int ob = __shfl_xor_sync(kFull, v.b, o);
    int oc = __shfl_xor_sync(kFull, v.code, o);
    if (os > v.score || (os == v.score && oi > v.idx)) { v.score = os; v.idx = oi; v.a = oa; v.b = ob; v.code = oc; }
  }
  return v;
}

__global__ void k_viterbi(DevLevel L, DevBatch B, DevWork W, int max_len, const float* inside, DevNode* nodes) {
  extern __shared__ DevNode tn_all[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int k = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (k >= W.nent) return;
  const int s = W.sent[k];
  const int n = B.len[s];
  DevNode* tn = tn_all + wib * (2 * max_len - 1);
  const int cs = L.cell_size;
  const float* ibot = inside + B.cell_off[s] * cs;
  const float* itop = ibot + tri(n) * cs;
  auto CELL = [&](const float* base, int x, int y) { return base + (long long)cs * chart_index(x, y, n); };
  const int nnt = L.n_nt;
  if (lane == 0) { tn[0].top = L.root; tn[0].width = n; tn[0].bot = 0; tn[0].score = 0.f; }
  __syncwarp();
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
      for (int r = r0 + lane; r < r1; r += 32) {
        const int c = L.v_left[r];
        const float scr = L.v_score[r] + child[c];
        if (scr >= bst.score) { bst.score = scr; bst.idx = r; bst.a = c; }
      }
      bst = warp_argmax_last(bst);
      botSym = bst.idx < 0 ? 0 : bst.a;
      if (lane == 0) { tn[p].bot = botSym; tn[p].score = bst.score; }
    }
    if (width == 1) {
      if (lane == 0) tn[p].score = ibot[(long long)cs * begin + botSym];
      begin += 1;
    } else {
      Best bst{-300000.0f, -1, 10, 10, begin + 1};
      int base = 0;
      auto scan = [&](const float* lc, const float* rc, int grp, int code) {
        const int r0 = L.v_off[grp * nnt + botSym], r1 = L.v_off[grp * nnt + botSym + 1];
        for (int r = r0 + lane; r < r1; r += 32) {
          const int a = L.v_left[r], bb = L.v_right[r];
          const float scr = (L.v_score[r] + lc[a]) + rc[bb];
          if (scr >= bst.score) { bst.score = scr; bst.idx = base + (r - r0); bst.a = a; bst.b = bb; bst.code = code; }
        }
        base += r1 - r0;
      };
      scan(CELL(itop, begin, end - 1), CELL(ibot, end - 1, end), 1, -1);
      scan(CELL(ibot, begin, begin + 1), CELL(itop, begin + 1, end), 2, -2);
      if (width == 2) scan(CELL(ibot, begin, begin + 1), CELL(ibot, begin + 1, end), 3, -3);
      for (int sp = begin + 1; sp < end; ++sp) scan(CELL(itop, begin, sp), CELL(itop, sp, end), 0, sp);
      bst = warp_argmax_last(bst);
      if (bst.idx < 0) { bst.a = 10; bst.b = 10; bst.code = begin + 1; }
      if (lane == 0) {
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
    __syncwarp();
  }
  DevNode* out = nodes + B.node_off[s];
  for (int p = lane; p < 2 * n - 1; p += 32) out[p] = tn[p];
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
void set_smem(K kernel, size_t bytes) {
  if (bytes > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

}  // namespace

cudaError_t launch_masks(const DevLevel& L, const DevBatch& B, const DevWork& W, const float* inside,
                         const float* outside, float thresh, int* masks_out, cudaStream_t st) {
  const int blocks = (int)((W.nunits * 32 + 255) / 256);
  if (blocks == 0) return cudaSuccess;
  k_masks<<<blocks, 256, 0, st>>>(L, B, W, inside, outside, thresh, masks_out);
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
  const int wpb = 4;
  const int blocks = (W.nent + wpb - 1) / wpb;
  if (blocks == 0) return cudaSuccess;
  const size_t smem = (size_t)wpb * (2 * max_len - 1) * sizeof(DevNode);
  set_smem(k_viterbi, smem);
  k_viterbi<<<blocks, wpb * 32, smem, st>>>(L, B, W, max_len, inside, nodes);
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
