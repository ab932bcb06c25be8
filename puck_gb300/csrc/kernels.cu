// Device kernels of the chart-parsing hot path (sm_103a).
//
// Every pass runs one CTA per chart cell of a span-length wavefront.  The
// binary passes are written in *gather* form: the CTA that owns a target cell
// stages the child (or parent/sibling) cells of every allowed split in shared
// memory and reduces all rule applications into the cell in one place, so no
// global atomics are needed and the cell is written exactly once.  Max-plus
// (Viterbi) results are bit-identical to the reference's per-rule
// ``max(p, (L + R) + w)`` (SimpleGenRuleMultiply.java:151) because x -> fl(x + w)
// is monotone: max_s fl(fl(L_s + R_s) + w) == fl(max_s fl(L_s + R_s) + w).
//
// Reference semantics restated here (dlwh/puck paths):
//   gating        CLParser.scala:845-855,885-901 (segment bits vs cell mask, child "any")
//   inside pass   CLParser.scala:256-314,489-504
//   outside pass  CLParser.scala:316-369,506-522
//   unaries       CLParser.scala:698-763, SimpleGenRuleMultiply.java:255-319
//   lexicon       CLParser.scala:411-467
//   masks         CLMaskKernels.scala:172-236
//   scaling       CLScalingKernels.scala:225-243
//   backtrace     CLViterbi.scala:383-605
//   MBR           CLMBRKernels.scala:118-170, CLParser.scala:587-696

#include "puck_internal.h"

#include <math_constants.h>

namespace puck {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ long long tri(int n) { return (long long)n * (n + 1) / 2; }
__device__ __forceinline__ int chart_index(int b, int e, int n) {
  int sp = abs(e - b) - 1;
  return min(b, e) + sp * n - sp * (sp - 1) / 2;
}

struct SentCell { int s, b; };

__device__ __forceinline__ SentCell span_cell(const DevBatch& B, int span, int i) {
  const int* pref = B.span_pref + B.span_base[span];
  int lo = 0, hi = B.span_count[span];
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (pref[mid] <= i) lo = mid; else hi = mid;
  }
  return {B.order[lo], i - pref[lo]};
}

__device__ __forceinline__ int sentence_of_cell(const DevBatch& B, long long c) {
  int lo = 0, hi = B.nsent;  // cell_off[lo] <= c < cell_off[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (B.cell_off[mid] <= c) lo = mid; else hi = mid;
  }
  return lo;
}

template <int S> struct Sr;
template <> struct Sr<SEMI_VITERBI> {
  static __device__ __forceinline__ float zero() { return -CUDART_INF_F; }
  static __device__ __forceinline__ float one() { return 0.f; }
  static __device__ __forceinline__ float add(float x, float y) { return fmaxf(x, y); }
  static __device__ __forceinline__ float mad(float acc, float child, float w) { return fmaxf(acc, child + w); }
};
template <> struct Sr<SEMI_REAL> {
  static __device__ __forceinline__ float zero() { return 0.f; }
  static __device__ __forceinline__ float one() { return 1.f; }
  static __device__ __forceinline__ float add(float x, float y) { return x + y; }
  static __device__ __forceinline__ float mad(float acc, float child, float w) { return fmaf(child, w, acc); }
};
template <> struct Sr<SEMI_LOGSUM> {
  static __device__ __forceinline__ float zero() { return -1000000.0f; }
  static __device__ __forceinline__ float one() { return 0.f; }
  static __device__ __forceinline__ float add(float x, float y) {
    float lo = fminf(x, y), hi = fmaxf(x, y);
    return hi + log1pf(expf(lo - hi));
  }
  static __device__ __forceinline__ float mad(float acc, float child, float w) { return add(acc, child + w); }
};

template <int S> __device__ __forceinline__ float warp_reduce(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = Sr<S>::add(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

__device__ __forceinline__ bool mask_any(const DevMask& M, long long c) {
  if (!M.bits) return true;
  const int* m = M.bits + c * M.mask_size;
  for (int i = 0; i < M.mask_size; ++i)
    if (m[i]) return true;
  return false;
}

// Shared bookkeeping of one target cell's pass.
struct CellCtx {
  const float* aptr[kMaxLen];  // operand cells of each allowed split
  const float* bptr[kMaxLen];
  float scl[kMaxLen];          // Real semiring: per-split scale exp(-p + l + r)
  int gate[kMaxMask];
  int nsp;
  int flag0, flag1;
  unsigned long long work;
  unsigned long long corner;
};

// Reduce every rule of job J over the staged splits into P (one warp per
// target symbol, lanes over the target's rules).
template <int S>
__device__ void gather_job(const DevJob& J, int cs, int ms, bool gated, int merged, float* P, float* stA,
                           float* stB, int chunk, CellCtx& X) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int nsp = X.nsp;
  const int n4 = cs >> 2;
  unsigned long long work = 0, corner = 0;
  for (int c0 = 0; c0 < nsp; c0 += chunk) {
    const int nc = min(chunk, nsp - c0);
    for (int idx = threadIdx.x; idx < nc * n4; idx += blockDim.x) {
      int s = idx / n4, k = idx - s * n4;
      reinterpret_cast<float4*>(stA + s * cs)[k] = __ldg(reinterpret_cast<const float4*>(X.aptr[c0 + s]) + k);
      reinterpret_cast<float4*>(stB + s * cs)[k] = __ldg(reinterpret_cast<const float4*>(X.bptr[c0 + s]) + k);
    }
    __syncthreads();
    for (int t = warp; t < J.n_tgt; t += nwarps) {
      const int seg = __ldg(J.tgt_seg + t);
      if (seg < 0) continue;
      if (gated) {
        const int* bits = J.seg_bits + (merged ? 0 : seg) * ms;
        bool hit = false;
        for (int i = 0; i < ms; ++i) hit |= (__ldg(bits + i) & X.gate[i]) != 0;
        if (!hit) continue;
      }
      const int r0 = __ldg(J.rowptr + t), r1 = __ldg(J.rowptr + t + 1);
      float acc = Sr<S>::zero();
      for (int r = r0 + lane; r < r1; r += 32) {
        const int2 rr = __ldg(J.rules + r);
        const int a = rr.x & 0xffff, b = (int)((unsigned)rr.x >> 16);
        const float w = __int_as_float(rr.y);
        if (S == SEMI_VITERBI) {
          float v = -CUDART_INF_F;
          for (int s = 0; s < nc; ++s) v = fmaxf(v, stA[s * cs + a] + stB[s * cs + b]);
          acc = fmaxf(acc, v + w);
        } else if (S == SEMI_REAL) {
          float v = 0.f;
          for (int s = 0; s < nc; ++s) v = fmaf(X.scl[c0 + s], stA[s * cs + a] * stB[s * cs + b], v);
          acc = fmaf(v, w, acc);
        } else {
          float v = Sr<S>::zero();
          for (int s = 0; s < nc; ++s) v = Sr<S>::add(v, stA[s * cs + a] + stB[s * cs + b]);
          acc = Sr<S>::add(acc, v + w);
        }
      }
      acc = warp_reduce<S>(acc);
      if (lane == 0) {
        P[t] = Sr<S>::add(P[t], acc);
        work += (unsigned long long)(r1 - r0) * nc;
        if (S == SEMI_VITERBI && acc >= 0.f) corner++;
      }
    }
    __syncthreads();
  }
  if (lane == 0 && (work | corner)) {
    atomicAdd(&X.work, work);
    atomicAdd(&X.corner, corner);
  }
}

template <int S>
__device__ __forceinline__ void add_split(CellCtx& X, const float* a, const float* b, float ls, float rs, float ps) {
  int k = X.nsp++;
  X.aptr[k] = a;
  X.bptr[k] = b;
  if (S == SEMI_REAL) X.scl[k] = __expf(-ps + rs + ls);
}

__device__ __forceinline__ float scale_of(const float* sc, long long c) { return sc ? sc[c] : 0.f; }

template <int S>
__device__ void unary_into(const DevUJob& U, const float* src, float* dst, int cs, bool allowed, float scale) {
  for (int k = threadIdx.x; k < cs; k += blockDim.x) dst[k] = Sr<S>::zero();
  if (!allowed) return;
  for (int t = threadIdx.x; t < U.n_tgt; t += blockDim.x) {
    const int r0 = __ldg(U.rowptr + t), r1 = __ldg(U.rowptr + t + 1);
    if (r0 == r1) continue;
    float acc = Sr<S>::zero();
    for (int r = r0; r < r1; ++r) {
      const int2 rr = __ldg(U.rules + r);
      acc = Sr<S>::mad(acc, src[rr.x], __int_as_float(rr.y));
    }
    if (S == SEMI_REAL) acc *= scale;
    dst[t] = acc;
  }
}

__device__ __forceinline__ void store_cell(float* dst, const float* src, int cs) {
  const int n4 = cs >> 2;
  for (int k = threadIdx.x; k < n4; k += blockDim.x)
    reinterpret_cast<float4*>(dst)[k] = reinterpret_cast<const float4*>(src)[k];
}

__device__ __forceinline__ void flush_counters(CellCtx& X, const Counters& C) {
  if (threadIdx.x == 0) {
    if (X.work && C.work) atomicAdd(C.work, X.work);
    if (X.corner && C.corner) atomicAdd(C.corner, X.corner);
  }
}

// ---------------------------------------------------------------------------
// Inside pass for one span length (span 1: unary TU over the lexicon cells).
template <int S>
__global__ void __launch_bounds__(256) k_inside_span(DevLevel L, DevBatch B, DevMask M, int span, float* inside,
                                                     Counters C, int chunk) {
  extern __shared__ __align__(16) float smem[];
  __shared__ CellCtx X;
  const int cs = L.cell_size, ms = L.mask_size;
  float* P = smem;
  float* Q = P + cs;
  float* stA = Q + cs;
  float* stB = stA + chunk * cs;
  const SentCell sc = span_cell(B, span, blockIdx.x);
  const int s = sc.s, b = sc.b, e = b + span, n = B.len[s];
  const long long off = B.cell_off[s], toff = off + tri(n);
  const long long pbot = off + chart_index(b, e, n), ptop = toff + chart_index(b, e, n);
  if (threadIdx.x == 0) {
    X.flag0 = span == 1 ? 1 : mask_any(M, pbot);
    X.flag1 = mask_any(M, ptop);
    X.work = 0;
    X.corner = 0;
    if (M.bits)
      for (int i = 0; i < ms; ++i) X.gate[i] = M.bits[pbot * ms + i];
  }
  for (int k = threadIdx.x; k < cs; k += blockDim.x) P[k] = Sr<S>::zero();
  __syncthreads();
  const bool gated = M.bits != nullptr;
  const float ps = S == SEMI_REAL ? scale_of(M.iscale, pbot) : 0.f;
  if (span == 1) {
    for (int k = threadIdx.x; k < cs; k += blockDim.x) P[k] = inside[pbot * cs + k];
  } else if (X.flag0) {
    const float* ch = inside;
    auto BOT = [&](int x, int y) { return off + chart_index(x, y, n); };
    auto TOP = [&](int x, int y) { return toff + chart_index(x, y, n); };
    for (int job = 0; job < 4; ++job) {
      const int jid = job == 0 ? IN_TT : job == 1 ? IN_NT : job == 2 ? IN_TN : IN_NN;
      if (jid == IN_TT && span != 2) continue;
      if (L.jobs[jid].n_tgt == 0) continue;
      if (threadIdx.x == 0) {
        X.nsp = 0;
        if (jid == IN_NT) {
          long long lc = TOP(b, e - 1), rc = BOT(e - 1, e);
          if (mask_any(M, lc) && mask_any(M, rc))
            add_split<S>(X, ch + lc * cs, ch + rc * cs, scale_of(M.iscale, lc), scale_of(M.iscale, rc), ps);
        } else if (jid == IN_TN || jid == IN_TT) {
          long long lc = BOT(b, b + 1), rc = jid == IN_TN ? TOP(b + 1, e) : BOT(b + 1, e);
          if (mask_any(M, lc) && mask_any(M, rc))
            add_split<S>(X, ch + lc * cs, ch + rc * cs, scale_of(M.iscale, lc), scale_of(M.iscale, rc), ps);
        } else {
          for (int sp = b + 1; sp < e; ++sp) {
            long long lc = TOP(b, sp), rc = TOP(sp, e);
            if (mask_any(M, lc) && mask_any(M, rc))
              add_split<S>(X, ch + lc * cs, ch + rc * cs, scale_of(M.iscale, lc), scale_of(M.iscale, rc), ps);
          }
        }
      }
      __syncthreads();
      gather_job<S>(L.jobs[jid], cs, ms, gated, L.gate_merged, P, stA, stB, chunk, X);
    }
  }
  __syncthreads();
  if (span >= 2) store_cell(inside + pbot * cs, P, cs);
  // unary layer: top cell (whole row replaced, CLParser.scala:721-727)
  const float us = S == SEMI_REAL ? __expf(-scale_of(M.iscale, ptop) + scale_of(M.iscale, pbot)) : 1.f;
  unary_into<S>(L.ujobs[span == 1 ? IN_TU : IN_NU], P, Q, cs, X.flag1 != 0, us);
  __syncthreads();
  store_cell(inside + ptop * cs, Q, cs);
  flush_counters(X, C);
}

// ---------------------------------------------------------------------------
// Outside pass for one span length: outside-top of each cell gathered from its
// parents, then the unary layer to outside-bot (and, at span 1, the
// terminal-child binaries that the reference runs after its span loop).
template <int S>
__global__ void __launch_bounds__(256) k_outside_span(DevLevel L, DevBatch B, DevMask M, int span,
                                                      const float* inside, float* outside, Counters C, int chunk) {
  extern __shared__ __align__(16) float smem[];
  __shared__ CellCtx X;
  const int cs = L.cell_size, ms = L.mask_size;
  float* P = smem;
  float* Q = P + cs;
  float* stA = Q + cs;
  float* stB = stA + chunk * cs;
  const SentCell sc = span_cell(B, span, blockIdx.x);
  const int s = sc.s, b = sc.b, e = b + span, n = B.len[s];
  const long long off = B.cell_off[s], toff = off + tri(n);
  const long long cbot = off + chart_index(b, e, n), ctop = toff + chart_index(b, e, n);
  auto BOT = [&](int x, int y) { return off + chart_index(x, y, n); };
  auto TOP = [&](int x, int y) { return toff + chart_index(x, y, n); };
  const bool gated = M.bits != nullptr;
  if (threadIdx.x == 0) {
    X.flag0 = mask_any(M, ctop);
    X.flag1 = mask_any(M, cbot);
    X.work = 0;
    X.corner = 0;
    if (M.bits)
      for (int i = 0; i < ms; ++i) X.gate[i] = M.bits[ctop * ms + i];
  }
  for (int k = threadIdx.x; k < cs; k += blockDim.x) P[k] = Sr<S>::zero();
  __syncthreads();
  const float* in = inside;
  const float* ou = outside;
  const float* IS = M.iscale;
  const float* OS = M.oscale;
  if (span == n) {
    if (threadIdx.x == 0) P[L.root] = Sr<S>::one();  // setRootScores
  } else if (X.flag0) {
    const float ps = S == SEMI_REAL ? scale_of(OS, ctop) : 0.f;
    for (int job = 0; job < 4; ++job) {
      const int jid = job == 0 ? OUT_R_TN : job == 1 ? OUT_L_NT : job == 2 ? OUT_L_NN : OUT_R_NN;
      if (L.jobs[jid].n_tgt == 0) continue;
      if (threadIdx.x == 0) {
        X.nsp = 0;
        if (jid == OUT_R_TN) {
          if (b >= 1) {
            long long lc = BOT(b - 1, b), rc = BOT(b - 1, e);
            if (mask_any(M, lc) && mask_any(M, rc))
              add_split<S>(X, in + lc * cs, ou + rc * cs, scale_of(IS, lc), scale_of(OS, rc), ps);
          }
        } else if (jid == OUT_L_NT) {
          if (e + 1 <= n) {
            long long lc = BOT(b, e + 1), rc = BOT(e, e + 1);
            if (mask_any(M, lc) && mask_any(M, rc))
              add_split<S>(X, ou + lc * cs, in + rc * cs, scale_of(OS, lc), scale_of(IS, rc), ps);
          }
        } else if (jid == OUT_L_NN) {
          for (int sp = e + 1; sp <= n; ++sp) {
            long long lc = BOT(b, sp), rc = TOP(e, sp);
            if (mask_any(M, lc) && mask_any(M, rc))
              add_split<S>(X, ou + lc * cs, in + rc * cs, scale_of(OS, lc), scale_of(IS, rc), ps);
          }
        } else {
          for (int sp = 0; sp < b; ++sp) {
            long long lc = TOP(sp, b), rc = BOT(sp, e);
            if (mask_any(M, lc) && mask_any(M, rc))
              add_split<S>(X, in + lc * cs, ou + rc * cs, scale_of(IS, lc), scale_of(OS, rc), ps);
          }
        }
      }
      __syncthreads();
      gather_job<S>(L.jobs[jid], cs, ms, gated, L.gate_merged, P, stA, stB, chunk, X);
    }
  }
  __syncthreads();
  store_cell(outside + ctop * cs, P, cs);
  // unary layer: outside-bot from outside-top.  With a batch of one-word
  // sentences only, the reference's first unary call (at span == maxLength)
  // uses the nonterminal unaries and the span loop never runs.
  const bool use_tu = span == 1 && B.max_len > 1;
  const float us = S == SEMI_REAL ? __expf(-scale_of(OS, cbot) + scale_of(OS, ctop)) : 1.f;
  unary_into<S>(L.ujobs[use_tu ? OUT_TU : OUT_NU], P, Q, cs, X.flag0 != 0, us);
  __syncthreads();
  if (span == 1 && X.flag1) {
    // terminal-child buckets, gated by the bot cell's mask (CLParser.scala:345-355)
    if (threadIdx.x == 0 && M.bits)
      for (int i = 0; i < ms; ++i) X.gate[i] = M.bits[cbot * ms + i];
    const float ps = S == SEMI_REAL ? scale_of(OS, cbot) : 0.f;
    for (int job = 0; job < 4; ++job) {
      const int jid = job == 0 ? OUT_L_TT : job == 1 ? OUT_R_NT : job == 2 ? OUT_L_TN : OUT_R_TT;
      if (L.jobs[jid].n_tgt == 0) continue;
      if (threadIdx.x == 0) {
        X.nsp = 0;
        if (jid == OUT_L_TT) {
          if (b + 2 <= n) {
            long long lc = BOT(b, b + 2), rc = BOT(b + 1, b + 2);
            if (mask_any(M, lc) && mask_any(M, rc))
              add_split<S>(X, ou + lc * cs, in + rc * cs, scale_of(OS, lc), scale_of(IS, rc), ps);
          }
        } else if (jid == OUT_R_NT) {
          for (int sp = 0; sp < b; ++sp) {
            long long lc = TOP(sp, b), rc = BOT(sp, b + 1);
            if (mask_any(M, lc) && mask_any(M, rc))
              add_split<S>(X, in + lc * cs, ou + rc * cs, scale_of(IS, lc), scale_of(OS, rc), ps);
          }
        } else if (jid == OUT_L_TN) {
          for (int sp = b + 2; sp <= n; ++sp) {
            long long lc = BOT(b, sp), rc = TOP(b + 1, sp);
            if (mask_any(M, lc) && mask_any(M, rc))
              add_split<S>(X, ou + lc * cs, in + rc * cs, scale_of(OS, lc), scale_of(IS, rc), ps);
          }
        } else {
          if (b >= 1) {
            long long lc = BOT(b - 1, b), rc = BOT(b - 1, b + 1);
            if (mask_any(M, lc) && mask_any(M, rc))
              add_split<S>(X, in + lc * cs, ou + rc * cs, scale_of(IS, lc), scale_of(OS, rc), ps);
          }
        }
      }
      __syncthreads();
      gather_job<S>(L.jobs[jid], cs, ms, gated, L.gate_merged, Q, stA, stB, chunk, X);
    }
  }
  __syncthreads();
  store_cell(outside + cbot * cs, Q, cs);
  flush_counters(X, C);
}

// ---------------------------------------------------------------------------
// Lexicon: one warp per token writes the bot span-1 cell.
template <int S>
__global__ void k_lexicon(DevLevel L, DevBatch B, DevMask M, float* inside, double* part_scale, int* status) {
  const long long tok = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (tok >= B.num_tokens) return;
  int lo = 0, hi = B.nsent;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (B.word_off[mid] <= tok) lo = mid; else hi = mid;
  }
  const int s = lo, pos = (int)(tok - B.word_off[s]), n = B.len[s];
  const int cs = L.cell_size;
  const long long cell = B.cell_off[s] + pos;  // chartIndex(pos, pos + 1) == pos
  float* row = inside + cell * cs;
  for (int k = lane; k < cs; k += 32) row[k] = Sr<S>::zero();
  __syncwarp();
  const int w = B.words[tok];
  if (w < 0 || w >= L.n_words) {
    if (lane == 0 && status) status[s] = 4;  // PUCK_ERR_OOV
    return;
  }
  const long long x0 = L.lex_off[w], x1 = L.lex_off[w + 1];
  if (S == SEMI_REAL) {
    const float my_scale = __expf(-scale_of(M.iscale, cell));
    float total = 0.f;
    for (long long x = x0 + lane; x < x1; x += 32) {
      float v = __expf(L.lex_score[x]) * my_scale;
      row[L.lex_term[x]] = v;
      total += v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) total += __shfl_xor_sync(kFull, total, o);
    __syncwarp();
    const float half = total / 2.f;
    for (long long x = x0 + lane; x < x1; x += 32) row[L.lex_term[x]] /= half;
    if (lane == 0) atomicAdd(part_scale + s, log((double)half));
  } else {
    for (long long x = x0 + lane; x < x1; x += 32) row[L.lex_term[x]] = L.lex_score[x];
  }
  (void)n;
}

// ---------------------------------------------------------------------------
// Pruning masks: one warp per cell (max-marginal test against root + thresh).
__global__ void k_masks(DevLevel L, DevBatch B, const float* inside, const float* outside, float thresh,
                        int* out) {
  const long long c = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= B.num_cells) return;
  const int s = sentence_of_cell(B, c);
  const long long first = B.cell_off[s], last = B.cell_off[s + 1];
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
__global__ void k_scaling(int cs, long long num_cells, const float* chart, float* out) {
  const long long c = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= num_cells) return;
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

__global__ void k_viterbi(DevLevel L, DevBatch B, const float* inside, DevNode* nodes) {
  extern __shared__ DevNode tn_all[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int s = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (s >= B.nsent) return;
  const int n = B.len[s];
  DevNode* tn = tn_all + wib * (2 * B.max_len - 1);
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
__global__ void k_mbr_cells(DevLevel L, DevBatch B, const float* inside, const float* outside, float2* decode) {
  extern __shared__ float margs_all[];
  const long long c = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  float* margs = margs_all + wib * L.n_coarse;
  if (c >= B.num_cells) return;
  for (int k = lane; k < L.n_coarse; k += 32) margs[k] = 0.f;
  __syncwarp();
  const int s = sentence_of_cell(B, c);
  const long long first = B.cell_off[s], last = B.cell_off[s + 1];
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

__global__ void k_mbr_decode(DevBatch B, DevMask M, int scaling, const float2* decode, const long long* mbr_off,
                             float* scratch, DevNode* nodes) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= B.nsent) return;
  const int n = B.len[s];
  const long long off = B.cell_off[s], toff = off + tri(n);
  // per-sentence scratch: best scores, best splits, unary flags ((n+1)^2 each)
  float* bs = scratch + mbr_off[s];
  int* bsplit = reinterpret_cast<int*>(bs + (n + 1) * (n + 1));
  int* uu = bsplit + (n + 1) * (n + 1);
  auto idx = [n](int x, int y) { return x * (n + 1) + y; };
  const float root_i = scaling ? M.iscale[toff + chart_index(0, n, n)] : 0.f;
  for (int span = 1; span <= n; ++span) {
    for (int bg = 0; bg + span <= n; ++bg) {
      const int en = bg + span;
      const long long ct = toff + chart_index(bg, en, n), cb = off + chart_index(bg, en, n);
      float topS = decode[ct].x, botS = decode[cb].x;
      if (scaling) {
        topS *= (float)exp((double)M.iscale[ct] + (double)M.oscale[ct] - (double)root_i);
        botS *= (float)exp((double)M.iscale[cb] + (double)M.oscale[cb] - (double)root_i);
      }
      if (isnan(topS)) topS = 0.f;
      if (isnan(botS)) botS = 0.f;
      topS = fminf(topS, 1.0f);
      botS = fminf(botS, 1.0f);
      const bool useU = (bg + 1 < en) || (double)topS > 0.4;
      uu[idx(bg, en)] = useU;
      float sc = useU ? topS + botS : botS;
      if (span > 1) {
        float bss = 0.0f;
        int bsp = bg + 1;
        for (int sp = bg + 1; sp < en; ++sp) {
          const float v = bs[idx(bg, sp)] + bs[idx(sp, en)];
          if (v > bss) { bsp = sp; bss = v; }
        }
        bsplit[idx(bg, en)] = bsp;
        sc += bss;
      }
      bs[idx(bg, en)] = sc;
    }
  }
  DevNode* out = nodes + B.node_off[s];
  int stack_b[kMaxLen], stack_e[kMaxLen];
  int top = 0, p = 0;
  stack_b[0] = 0; stack_e[0] = n; top = 1;
  while (top > 0) {
    --top;
    const int bg = stack_b[top], en = stack_e[top];
    const long long ct = toff + chart_index(bg, en, n), cb = off + chart_index(bg, en, n);
    DevNode nd;
    nd.top = uu[idx(bg, en)] ? __float_as_int(decode[ct].y) : -1;
    nd.bot = __float_as_int(decode[cb].y);
    nd.width = en - bg;
    nd.score = bs[idx(bg, en)];
    out[p++] = nd;
    if (en - bg > 1) {
      const int sp = bsplit[idx(bg, en)];
      stack_b[top] = sp; stack_e[top] = en; ++top;
      stack_b[top] = bg; stack_e[top] = sp; ++top;
    }
  }
}

// log Z per sentence (CLParser.scala:189-206), accumulated in FP64.
__global__ void k_root_scores(DevLevel L, DevBatch B, DevMask M, const float* inside, const double* part_scale,
                              float* log_z) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= B.nsent) return;
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

size_t inside_smem_bytes(int cell_size, int chunk) {
  return (size_t)(2 * cell_size + 2 * (size_t)chunk * cell_size) * sizeof(float);
}

int pick_split_chunk(int cell_size, int max_len) {
  const int budget = 96 * 1024 / 4;
  int chunk = (budget - 2 * cell_size) / (2 * cell_size);
  chunk = chunk < 2 ? 2 : chunk;
  chunk = chunk > kMaxSplitChunk ? kMaxSplitChunk : chunk;
  if (max_len > 1 && chunk > max_len) chunk = max_len;
  return chunk;
}

static constexpr int kThreads = 256;

cudaError_t launch_lexicon(const DevLevel& L, const DevBatch& B, const DevMask& M, float* inside,
                           double* part_scale, Counters C, cudaStream_t st) {
  const long long warps = B.num_tokens;
  const int blocks = (int)((warps * 32 + 127) / 128);
  if (blocks == 0) return cudaSuccess;
  switch (L.semiring) {
    case SEMI_VITERBI: k_lexicon<SEMI_VITERBI><<<blocks, 128, 0, st>>>(L, B, M, inside, part_scale, C.status); break;
    case SEMI_REAL: k_lexicon<SEMI_REAL><<<blocks, 128, 0, st>>>(L, B, M, inside, part_scale, C.status); break;
    default: k_lexicon<SEMI_LOGSUM><<<blocks, 128, 0, st>>>(L, B, M, inside, part_scale, C.status); break;
  }
  return cudaGetLastError();
}

cudaError_t launch_inside_span(const DevLevel& L, const DevBatch& B, const DevMask& M, int span, int ncells,
                               float* inside, Counters C, cudaStream_t st) {
  if (ncells == 0) return cudaSuccess;
  const int chunk = pick_split_chunk(L.cell_size, B.max_len);
  const size_t smem = inside_smem_bytes(L.cell_size, chunk);
  switch (L.semiring) {
    case SEMI_VITERBI:
      set_smem(k_inside_span<SEMI_VITERBI>, smem);
      k_inside_span<SEMI_VITERBI><<<ncells, kThreads, smem, st>>>(L, B, M, span, inside, C, chunk);
      break;
    case SEMI_REAL:
      set_smem(k_inside_span<SEMI_REAL>, smem);
      k_inside_span<SEMI_REAL><<<ncells, kThreads, smem, st>>>(L, B, M, span, inside, C, chunk);
      break;
    default:
      set_smem(k_inside_span<SEMI_LOGSUM>, smem);
      k_inside_span<SEMI_LOGSUM><<<ncells, kThreads, smem, st>>>(L, B, M, span, inside, C, chunk);
      break;
  }
  return cudaGetLastError();
}

cudaError_t launch_outside_span(const DevLevel& L, const DevBatch& B, const DevMask& M, int span, int ncells,
                                const float* inside, float* outside, Counters C, cudaStream_t st) {
  if (ncells == 0) return cudaSuccess;
  const int chunk = pick_split_chunk(L.cell_size, B.max_len);
  const size_t smem = inside_smem_bytes(L.cell_size, chunk);
  switch (L.semiring) {
    case SEMI_VITERBI:
      set_smem(k_outside_span<SEMI_VITERBI>, smem);
      k_outside_span<SEMI_VITERBI><<<ncells, kThreads, smem, st>>>(L, B, M, span, inside, outside, C, chunk);
      break;
    case SEMI_REAL:
      set_smem(k_outside_span<SEMI_REAL>, smem);
      k_outside_span<SEMI_REAL><<<ncells, kThreads, smem, st>>>(L, B, M, span, inside, outside, C, chunk);
      break;
    default:
      set_smem(k_outside_span<SEMI_LOGSUM>, smem);
      k_outside_span<SEMI_LOGSUM><<<ncells, kThreads, smem, st>>>(L, B, M, span, inside, outside, C, chunk);
      break;
  }
  return cudaGetLastError();
}

cudaError_t launch_masks(const DevLevel& L, const DevBatch& B, const float* inside, const float* outside,
                         float thresh, int* masks_out, cudaStream_t st) {
  const long long threads = B.num_cells * 32;
  const int blocks = (int)((threads + 255) / 256);
  if (blocks == 0) return cudaSuccess;
  k_masks<<<blocks, 256, 0, st>>>(L, B, inside, outside, thresh, masks_out);
  return cudaGetLastError();
}

cudaError_t launch_scaling(int cell_size, long long num_cells, const float* chart, float* out, cudaStream_t st) {
  const int blocks = (int)((num_cells * 32 + 255) / 256);
  if (blocks == 0) return cudaSuccess;
  k_scaling<<<blocks, 256, 0, st>>>(cell_size, num_cells, chart, out);
  return cudaGetLastError();
}

cudaError_t launch_viterbi(const DevLevel& L, const DevBatch& B, const float* inside, DevNode* nodes,
                           cudaStream_t st) {
  const int wpb = 4;
  const int blocks = (B.nsent + wpb - 1) / wpb;
  if (blocks == 0) return cudaSuccess;
  const size_t smem = (size_t)wpb * (2 * B.max_len - 1) * sizeof(DevNode);
  set_smem(k_viterbi, smem);
  k_viterbi<<<blocks, wpb * 32, smem, st>>>(L, B, inside, nodes);
  return cudaGetLastError();
}

cudaError_t launch_mbr_cells(const DevLevel& L, const DevBatch& B, const float* inside, const float* outside,
                             float2* decode, cudaStream_t st) {
  const int wpb = 8;
  const int blocks = (int)((B.num_cells + wpb - 1) / wpb);
  if (blocks == 0) return cudaSuccess;
  const size_t smem = (size_t)wpb * L.n_coarse * sizeof(float);
  if (L.semiring == SEMI_LOGSUM)
    k_mbr_cells<SEMI_LOGSUM><<<blocks, wpb * 32, smem, st>>>(L, B, inside, outside, decode);
  else
    k_mbr_cells<SEMI_REAL><<<blocks, wpb * 32, smem, st>>>(L, B, inside, outside, decode);
  return cudaGetLastError();
}

cudaError_t launch_mbr_decode(const DevBatch& B, const DevMask& M, int scaling, const float2* decode,
                              const long long* mbr_off, float* scratch, DevNode* nodes, cudaStream_t st) {
  const int blocks = (B.nsent + 63) / 64;
  if (blocks == 0) return cudaSuccess;
  k_mbr_decode<<<blocks, 64, 0, st>>>(B, M, scaling, decode, mbr_off, scratch, nodes);
  return cudaGetLastError();
}

cudaError_t launch_root_scores(const DevLevel& L, const DevBatch& B, const DevMask& M, const float* inside,
                               const double* part_scale, float* log_z, cudaStream_t st) {
  const int blocks = (B.nsent + 127) / 128;
  if (blocks == 0) return cudaSuccess;
  k_root_scores<<<blocks, 128, 0, st>>>(L, B, M, inside, part_scale, log_z);
  return cudaGetLastError();
}

}  // namespace puck
