// Chart passes of the hot path on sm_103a: lexicon, inside and outside span
// wavefronts (binary rules + unary layer).
//
// One CTA owns one target cell of a span-length wavefront and reduces every
// rule application into it in *gather* form, so there are no global atomics
// and the cell is written exactly once.  Max-plus (Viterbi) cells are
// bit-identical to the reference's per-rule ``max(p, (L + R) + w)``
// (SimpleGenRuleMultiply.java:151) because x -> fl(x + w) is monotone:
//     max_s fl(fl(L_s + R_s) + w) == fl(max_s fl(L_s + R_s) + w).
//
// Split grammars use the pair-factored form.  Rules are grouped by the coarse
// projection (Y, Z) of their operands.  For a target cell, a warp computes the
// max-plus outer product M[j][k] = max_s A_s[Y_j] + B_s[Z_k] over the splits s
// once per pair, then applies every rule of the pair as M[j][k] + w.  Both
// steps are exact in max-plus arithmetic.  Every producing kernel records, per
// cell, which coarse symbols hold a non-zero value (its liveness bitset).  A
// pair is skipped for a split whose left operand has no live Y or right operand
// no live Z.  This is exact too, because every skipped term is the semiring
// zero.  Operand values are read through L1, so the pass needs little shared
// memory and several CTAs share an SM.  Grammars without split structure keep
// target-major rule scans over operand cells staged in shared memory.
//
// Kernel modes: 0 target-major scans; 2 the pair form (whole-pair tiles, one
// task of one j and four k per lane); 3 the flat-tile form (pairs cut into
// 16 x 16 sub-tiles, an 8 x 4 lane grid over each, four-split groups staged
// per warp, four-rule records), for both the max-plus and the sum-product
// semiring and for both passes.  The host picks the mode per level and per
// span launch.  Within mode 0, an ungated job (no coarse mask, not LogSum)
// with few rules per target scans its distinct child pairs instead of its
// targets (gather_pairmajor).
//
// Reference semantics restated (dlwh/puck paths):
//   gating        CLParser.scala:845-855,885-901 (segment bits vs cell mask, child "any")
//   inside pass   CLParser.scala:256-314,489-504
//   outside pass  CLParser.scala:316-369,506-522
//   unaries       CLParser.scala:698-763, SimpleGenRuleMultiply.java:255-319
//   lexicon       CLParser.scala:411-467

#include "device_common.cuh"

namespace puck {
namespace {

using namespace dev;

constexpr int kPairChunk = 64;   // splits per liveness chunk (two ballots)
constexpr int kThreads = 256;
constexpr int kRuleBatch = 4;   // rules per lane whose loads are in flight together
// Per-warp operand stage of the flat-tile kernels: two buffers of 34 rows
// of four floats (A members 0-15, a -inf row, B members 0-15, a -inf row).
constexpr int kStageRows = 34;
constexpr int kStageFloats = 2 * kStageRows * 4;
constexpr int kStageRowB = 17;
// Per-warp list of a pair's live splits (chunk positions, one byte each),
// padded by three repeats of the last one for the groups of four.
constexpr int kSplitList = 68;

// Shared bookkeeping of one target cell.
struct __align__(16) CellCtx {
  // operand cells of each allowed split, and four more entries that repeat
  // the last split (the flat-tile path reads splits in groups of four)
  const float* aptr[kMaxLen + 4];
  const float* bptr[kMaxLen + 4];
  const int* alive[kMaxLen];    // their liveness words
  const int* blive[kMaxLen];
  float scl[kMaxLen];           // Real semiring: per-split scale exp(-p + l + r)
  int la[kPairChunk][kMaxMask];
  int lb[kPairChunk][kMaxMask];
  int gate[kMaxMask];
  unsigned words[kMaxMask];
  int nsp, nlive;
  int next;   // next live-pair draw of the flat-tile path
  int flag0, flag1;
  int g, G;   // this CTA is part g of the cell's G parts
  int last;
  int wcnt[kThreads / 32];
  unsigned segpass[kMaxSeg / 32];  // bit s: segment s of the current job is gated in for this cell
  unsigned long long work, corner;
};

// Dynamic shared memory of a pass kernel: [P | Q | mode 0: staged operand
// cells | mode 2: per-warp outer-product tiles, pair liveness, live list].
struct Smem {
  float* P;
  float* Q;
  float* stA;
  float* stB;
  float* M;
  float* stage;  // per warp kStageFloats: staged A and B members of four splits (16-byte aligned)
  unsigned* pl;
  int* list;
  unsigned char* slist;  // per warp kSplitList: the live splits of the warp's current pair (flat-tile path)
  float* sclist;         // sum-product levels, per warp kSplitList: the scale of each listed split, 0 for
                         // the list's repeats (16-byte aligned)
  int mtile;             // floats of each warp's M tile
};

// Floats of each warp's outer-product tile: the flat-tile sub-tiles (at most
// 16 x 16) in a flat-tile kernel (MODE 3), else the level's largest pair.
__host__ __device__ __forceinline__ int mtile_floats(const DevLevel& L, bool flat) {
  return flat ? L.flat_mtile : L.max_mtile;
}

// with_stage: the per-warp operand stage (the Viterbi inside pass and the
// flat-tile kernels); pairs: a pair-factored kernel (MODE 2 or 3; the outside
// kernel tests the level's mode at run time instead, which keeps its
// target-major register allocation free of spills); flat: a flat-tile kernel
// (MODE 3)
__device__ __forceinline__ Smem carve(float* base, const DevLevel& L, int chunk, bool with_stage, bool pairs,
                                      bool flat) {
  Smem m;
  const int cs = L.cell_size;
  m.P = base;
  m.Q = base + cs;
  float* rest = base + 2 * cs;
  m.stA = m.stB = m.M = m.stage = nullptr;
  m.pl = nullptr;
  m.list = nullptr;
  m.slist = nullptr;
  m.sclist = nullptr;
  m.mtile = mtile_floats(L, flat);
  if (pairs) {
    if (with_stage) {
      m.stage = rest;
      rest += (blockDim.x >> 5) * kStageFloats;
    }
    m.M = rest;
    m.pl = reinterpret_cast<unsigned*>(rest + (blockDim.x >> 5) * m.mtile);
    m.list = reinterpret_cast<int*>(m.pl + L.n_coarse * L.mask_size);
    if (with_stage) {
      m.slist = reinterpret_cast<unsigned char*>(m.list + L.max_npair);
      if (L.semiring == SEMI_REAL) {
        const size_t end = reinterpret_cast<size_t>(m.slist + (blockDim.x >> 5) * kSplitList);
        m.sclist = reinterpret_cast<float*>((end + 15) & ~(size_t)15);
      }
    }
  } else {
    m.stA = rest;
    m.stB = rest + chunk * cs;
  }
  return m;
}

// Two FP32 additions in one instruction (sm_100+ packed f32x2, round to
// nearest: each lane of the pair is rounded exactly as a scalar add).
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;"
      : "=l"(r)
      : "l"(*reinterpret_cast<unsigned long long*>(&a)), "l"(*reinterpret_cast<unsigned long long*>(&b)));
  return *reinterpret_cast<float2*>(&r);
}

// max(a, b, c) in one instruction (sm_100+); exact, like fmaxf
__device__ __forceinline__ float max3(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// float max through integer atomics (valid for every non-NaN value)
__device__ __forceinline__ void atomic_fmax(float* addr, float v) {
  if (__float_as_int(v) >= 0) atomicMax(reinterpret_cast<int*>(addr), __float_as_int(v));
  else atomicMin(reinterpret_cast<unsigned*>(addr), __float_as_uint(v));
}

template <int S>
__device__ __forceinline__ void put_split(CellCtx& X, int k, const float* a, const float* b, const int* la,
                                          const int* lb, float ls, float rs, float ps) {
  X.aptr[k] = a;
  X.bptr[k] = b;
  X.alive[k] = la;
  X.blive[k] = lb;
  if (S == SEMI_REAL) X.scl[k] = __expf(-ps + rs + ls);
}

template <int S>
__device__ __forceinline__ void add_split(CellCtx& X, const float* a, const float* b, const int* la,
                                          const int* lb, float ls, float rs, float ps) {
  int k = X.nsp++;
  X.aptr[k] = a;
  X.bptr[k] = b;
  X.alive[k] = la;
  X.blive[k] = lb;
  if (S == SEMI_REAL) X.scl[k] = __expf(-ps + rs + ls);
}

__device__ __forceinline__ void stage(CellCtx& X, int c0, int nc, int cs, float* stA, float* stB) {
  const int n4 = cs >> 2;
  for (int idx = threadIdx.x; idx < nc * n4; idx += blockDim.x) {
    const int s = idx / n4, k = idx - s * n4;
    reinterpret_cast<float4*>(stA + s * cs)[k] = __ldg(reinterpret_cast<const float4*>(X.aptr[c0 + s]) + k);
    reinterpret_cast<float4*>(stB + s * cs)[k] = __ldg(reinterpret_cast<const float4*>(X.bptr[c0 + s]) + k);
  }
}

__device__ __forceinline__ bool gate_hit(const DevJob& J, int seg, int ms, int merged, const int* gate) {
  const int* bits = J.seg_bits + (merged ? 0 : seg) * ms;
  bool hit = false;
  for (int i = 0; i < ms; ++i) hit |= (__ldg(bits + i) & gate[i]) != 0;
  return hit;
}

// Target-major layout: one warp per target symbol, lanes over its rules.
template <int S>
__device__ void gather_targets(const DevJob& J, const DevLevel& L, bool gated, float* P, float* stA, float* stB,
                               int chunk, CellCtx& X) {
  const int cs = L.cell_size, ms = L.mask_size;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int nsp = X.nsp;
  unsigned long long work = 0, corner = 0;
  for (int c0 = 0; c0 < nsp; c0 += chunk) {
    const int nc = min(chunk, nsp - c0);
    stage(X, c0, nc, cs, stA, stB);
    __syncthreads();
    for (int t = X.g * nwarps + warp; t < J.n_tgt; t += X.G * nwarps) {
      const int seg = __ldg(J.tgt_seg + t);
      if (seg < 0) continue;
      if (gated && !gate_hit(J, seg, ms, L.gate_merged, X.gate)) continue;
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
  if (nsp == 0) __syncthreads();  // see gather()
  if (lane == 0 && (work | corner)) {
    atomicAdd(&X.work, work);
    atomicAdd(&X.corner, corner);
  }
}

template <int S>
__device__ __forceinline__ void flush_run(float* P, int t, float v, unsigned long long& corner);

// Pair-major layout (DevJob::pm_*), for an ungated target-major level: every
// thread takes distinct child pairs (a, b), computes max_s fl(A_s[a] +
// B_s[b]) over the chunk's staged splits once (sum-product: the scaled sum),
// and applies the pair's rules to their targets with shared-memory atomics.
// Exact in max-plus: fl(max_s fl(A + B) + w) = max_s fl(fl(A + B) + w), as
// for the pair-factored form.  The parts of a split cell take every G-th
// pair.
template <int S>
__device__ void gather_pairmajor(const DevJob& J, const DevLevel& L, float* P, float* stA, float* stB, int chunk,
                                 CellCtx& X) {
  const int cs = L.cell_size;
  const int lane = threadIdx.x & 31;
  const int nsp = X.nsp;
  unsigned long long work = 0, corner = 0;
  for (int c0 = 0; c0 < nsp; c0 += chunk) {
    const int nc = min(chunk, nsp - c0);
    stage(X, c0, nc, cs, stA, stB);
    __syncthreads();
    for (int p = X.g * blockDim.x + threadIdx.x; p < J.pm_npair; p += X.G * blockDim.x) {
      const int ab = __ldg(J.pm_ab + p);
      const int a = ab & 0xffff, b = (int)((unsigned)ab >> 16);
      float v = Sr<S>::zero();
      if (S == SEMI_VITERBI) {
        for (int s = 0; s < nc; ++s) v = fmaxf(v, stA[s * cs + a] + stB[s * cs + b]);
      } else {
        for (int s = 0; s < nc; ++s) v = fmaf(X.scl[c0 + s], stA[s * cs + a] * stB[s * cs + b], v);
      }
      const int r0 = __ldg(J.pm_off + p), r1 = __ldg(J.pm_off + p + 1);
      work += (unsigned long long)nc + (r1 - r0);
      if (v == Sr<S>::zero()) continue;
      for (int r = r0; r < r1; ++r) {
        const int2 R = __ldg(J.pm_rule + r);
        const float w = __int_as_float(R.y);
        flush_run<S>(P, R.x, S == SEMI_VITERBI ? v + w : v * w, corner);
      }
    }
    __syncthreads();
  }
  if (nsp == 0) __syncthreads();  // see gather()
  for (int o = 16; o > 0; o >>= 1) {
    work += __shfl_down_sync(kFull, work, o);
    corner += __shfl_down_sync(kFull, corner, o);
  }
  if (lane == 0 && (work | corner)) {
    atomicAdd(&X.work, work);
    atomicAdd(&X.corner, corner);
  }
}

__device__ __forceinline__ bool bit(const int* words, int c) { return (words[c >> 5] >> (c & 31)) & 1; }

// Whether pair key c has a live member in the liveness words: key = one
// coarse symbol (grp 1), or the group of 16 coarse ids 16c .. 16c + 15
// (grp 16, DevLevel::pair_group).
__device__ __forceinline__ bool key_live(const int* words, int c, int grp) {
  return grp <= 1 ? bit(words, c) : (((unsigned)words[c >> 1] >> ((c & 1) * 16)) & 0xffffu) != 0u;
}

template <int S>
__device__ __forceinline__ void flush_run(float* P, int t, float v, unsigned long long& corner) {
  if (S == SEMI_VITERBI) {
    if (v != -CUDART_INF_F) {
      atomic_fmax(P + t, v);
      if (v >= 0.f) ++corner;
    }
  } else if (v != 0.f) {
    atomicAdd(P + t, v);
  }
}

// This lane's operand value for each of the four splits of group g (see
// grid_outer): one 4-byte load fetches the group's split positions from the
// warp's live-split list, then their row pointers.
// Sum-product: the left operand (sc != nullptr, the warp's scale list)
// carries each listed split's scale, and the list's repeats have scale 0, so
// they add nothing.
template <int S>
__device__ __forceinline__ float4 load_group(const float* const* rows, const float* sc, const unsigned char* sl,
                                             int g, unsigned src, bool ok) {
  const unsigned q = *reinterpret_cast<const unsigned*>(sl + 4 * g);
  const float z = Sr<S>::zero();
  float4 v;
  v.x = ok ? __ldg(rows[q & 255u] + src) : z;
  v.y = ok ? __ldg(rows[(q >> 8) & 255u] + src) : z;
  v.z = ok ? __ldg(rows[(q >> 16) & 255u] + src) : z;
  v.w = ok ? __ldg(rows[q >> 24] + src) : z;
  if (S == SEMI_REAL && sc) {
    const float4 f = *reinterpret_cast<const float4*>(sc + 4 * g);
    v.x *= f.x;
    v.y *= f.y;
    v.z *= f.z;
    v.w *= f.w;
  }
  return v;
}

// Outer product of one pair in the flat-tile layout (DevJob::pair_desc) into
// the warp's M tile: M[j * nz + k] = max over the pair's live splits s of
// fl(A_s[Y_j] + B_s[Z_k]).  The lanes form an 8 x 4 grid: lane (jg, kg) =
// (lane / 4, lane % 4) holds the RJ x RK entries j = jg + 8a, k = kg + 4b, so
// that each A row it reads serves RK entries and each B row RJ entries.  The
// n live splits (the warp's list sl, padded by repeats of the last one: max
// is idempotent) go in groups of four.  Per group, lanes 0-15 stage the A
// members of the four splits as one float4 row each, lanes 16-31 the B
// members; a lane then reads its RJ A rows and RK B rows (one 16-byte load
// each) and folds four sums into each entry with two packed adds and two
// 3-input maxes.  The operand loads of the next group are issued before the
// current group's arithmetic, into the other of the warp's two stage buffers.
// Rows past the tile read the -inf rows; their entries are not stored.
// Sum-product: M[j * nz + k] = sum over the live splits of scale_s A_s[Y_j]
// B_s[Z_k], four fused multiply-adds per entry and group, the scale applied
// to A when it is staged.
template <int S, int RJ, int RK>
__device__ __forceinline__ void grid_outer(const CellCtx& X, int c0, const unsigned char* sl, const float* scl_list,
                                           int n, int4 D, float4* st4, float* Mw) {
  const int lane = threadIdx.x & 31;
  const int ny = D.z & 255, nz = (D.z >> 8) & 255;
  const int jg = lane >> 2, kg = lane & 3;
  unsigned offA[RJ], offB[RK];  // byte offsets of the lane's rows in buffer 0
#pragma unroll
  for (int a = 0; a < RJ; ++a) offA[a] = (unsigned)((jg + 8 * a < ny ? jg + 8 * a : 16) * 16);
#pragma unroll
  for (int b = 0; b < RK; ++b) offB[b] = (unsigned)((kStageRowB + (kg + 4 * b < nz ? kg + 4 * b : 16)) * 16);
  float acc[RJ][RK];
#pragma unroll
  for (int a = 0; a < RJ; ++a)
#pragma unroll
    for (int b = 0; b < RK; ++b) acc[a][b] = Sr<S>::zero();
  const bool a_side = lane < 16;
  const int mem = a_side ? lane : lane - 16;
  const bool ok = mem < (a_side ? ny : nz);
  const unsigned src = (a_side ? (unsigned)D.x & 0xffffu : (unsigned)D.x >> 16) + mem;
  const float* const* rows = (a_side ? X.aptr : X.bptr) + c0;
  const float* sc = S == SEMI_REAL && a_side ? scl_list : nullptr;
  const int my_row = a_side ? mem : kStageRowB + mem;
  int g = 0;
  float4 v = load_group<S>(rows, sc, sl, 0, src, ok);
  for (int buf = 0;; buf ^= 1) {
    float4* sb = st4 + buf * kStageRows;
    sb[my_row] = v;
    __syncwarp();
    const bool rest = 4 * (g + 1) < n;
    if (rest) {
      ++g;
      v = load_group<S>(rows, sc, sl, g, src, ok);
    }
    const char* stb = reinterpret_cast<const char*>(sb);
    float4 A[RJ];
#pragma unroll
    for (int a = 0; a < RJ; ++a) A[a] = *reinterpret_cast<const float4*>(stb + offA[a]);
#pragma unroll
    for (int b = 0; b < RK; ++b) {
      const float4 B = *reinterpret_cast<const float4*>(stb + offB[b]);
#pragma unroll
      for (int a = 0; a < RJ; ++a) {
        if (S == SEMI_VITERBI) {
          const float2 t01 = add2(make_float2(A[a].x, A[a].y), make_float2(B.x, B.y));
          const float2 t23 = add2(make_float2(A[a].z, A[a].w), make_float2(B.z, B.w));
          acc[a][b] = max3(acc[a][b], t01.x, t01.y);
          acc[a][b] = max3(acc[a][b], t23.x, t23.y);
        } else {
          acc[a][b] = fmaf(A[a].x, B.x, acc[a][b]);
          acc[a][b] = fmaf(A[a].y, B.y, acc[a][b]);
          acc[a][b] = fmaf(A[a].z, B.z, acc[a][b]);
          acc[a][b] = fmaf(A[a].w, B.w, acc[a][b]);
        }
      }
    }
    if (!rest) break;
  }
#pragma unroll
  for (int a = 0; a < RJ; ++a)
#pragma unroll
    for (int b = 0; b < RK; ++b)
      if (jg + 8 * a < ny && kg + 4 * b < nz) Mw[(jg + 8 * a) * nz + kg + 4 * b] = acc[a][b];
  __syncwarp();
}

// The gated-in blocks of one flat-tile pair: each lane runs its one-target
// slice four rules per record, fl(M[e] + w) folded with packed adds and
// 3-input maxes (sum-product: M[e] w summed with fused multiply-adds; a
// padding rule, weight 0, adds nothing even where M[e] overflowed), and
// flushes once per block.  A block's descriptor {segment, first record, end
// record, rules} is read one block ahead.
template <int S>
__device__ __forceinline__ void flat_rules(const DevJob& J, const CellCtx& X, int4 D, const float* Mw, float* P,
                                           unsigned long long& work, unsigned long long& corner) {
  const int lane = threadIdx.x & 31;
  const int b0 = D.y, nb = (int)((unsigned)D.z >> 16);
  int4 nxt = nb > 0 ? __ldg(J.fr_blk + b0) : make_int4(0, 0, 0, 0);
  for (int q = 0; q < nb; ++q) {
    const int4 B = nxt;
    if (q + 1 < nb) nxt = __ldg(J.fr_blk + b0 + q + 1);
    if (!((X.segpass[B.x >> 5] >> (B.x & 31)) & 1u)) continue;
    const int t = __ldg(J.fr_tgt + (b0 + q) * 32 + lane);
    float best = Sr<S>::zero();
#pragma unroll 2
    for (int g = B.y + lane; g < B.z; g += 32) {
      const unsigned o = __ldg(J.fr_idx + g);
      const float4 w = __ldg(J.fr_w + g);
      if (S == SEMI_VITERBI) {
        const float2 t01 = add2(make_float2(Mw[o & 255u], Mw[(o >> 8) & 255u]), make_float2(w.x, w.y));
        const float2 t23 = add2(make_float2(Mw[(o >> 16) & 255u], Mw[o >> 24]), make_float2(w.z, w.w));
        best = max3(best, t01.x, t01.y);
        best = max3(best, t23.x, t23.y);
      } else {
        best = fmaf(w.x != 0.f ? Mw[o & 255u] : 0.f, w.x, best);
        best = fmaf(w.y != 0.f ? Mw[(o >> 8) & 255u] : 0.f, w.y, best);
        best = fmaf(w.z != 0.f ? Mw[(o >> 16) & 255u] : 0.f, w.z, best);
        best = fmaf(w.w != 0.f ? Mw[o >> 24] : 0.f, w.w, best);
      }
    }
    if (t >= 0) flush_run<S>(P, t, best, corner);
    if (lane == 0) work += (unsigned long long)B.w;
  }
  __syncwarp();
}

// The live pairs of a flat-tile job for one chunk of splits.  Warps take
// pairs from a shared counter (this part's pairs are list positions g,
// g + G, g + 2G, ...), so a warp that drew cheap pairs takes more of them.
template <int S>
__device__ __forceinline__ void flat_pairs(const DevJob& J, const Smem& sm, CellCtx& X, int c0, int nc, int nlive,
                                           int grp, float* Mw, float* P, unsigned long long& work,
                                           unsigned long long& corner) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float4* st4 = reinterpret_cast<float4*>(sm.stage + warp * kStageFloats);
  unsigned char* sl = sm.slist + warp * kSplitList;
  float* sc = S == SEMI_REAL ? sm.sclist + warp * kSplitList : nullptr;
  for (;;) {
    int k = 0;
    if (lane == 0) k = atomicAdd(&X.next, 1);
    const int i = X.g + __shfl_sync(kFull, k, 0) * X.G;
    if (i >= nlive) break;
    const int p = sm.list[i];
    const int4 D = __ldg(J.pair_desc + p);
    const int ca = D.w & 255, cb = (D.w >> 8) & 255;
    const unsigned lo =
        __ballot_sync(kFull, lane < nc && key_live(X.la[lane], ca, grp) && key_live(X.lb[lane], cb, grp));
    const unsigned hi = __ballot_sync(
        kFull, lane + 32 < nc && key_live(X.la[lane + 32], ca, grp) && key_live(X.lb[lane + 32], cb, grp));
    const unsigned long long m = (unsigned long long)lo | ((unsigned long long)hi << 32);
    // the pair's live splits in order, then three repeats of the last one
    // (sum-product: with their scales, and scale 0 for the repeats)
    const unsigned below = (1u << lane) - 1u;
    const int nlo = __popc(lo), n = nlo + __popc(hi);
    if ((lo >> lane) & 1u) {
      const int at = __popc(lo & below);
      sl[at] = (unsigned char)lane;
      if (S == SEMI_REAL) sc[at] = X.scl[c0 + lane];
    }
    if ((hi >> lane) & 1u) {
      const int at = nlo + __popc(hi & below);
      sl[at] = (unsigned char)(32 + lane);
      if (S == SEMI_REAL) sc[at] = X.scl[c0 + 32 + lane];
    }
    if (lane < 3) {
      sl[n + lane] = (unsigned char)(hi ? 63 - __clz(hi) : 31 - __clz(lo));
      if (S == SEMI_REAL) sc[n + lane] = 0.f;
    }
    __syncwarp();
    const int ny = D.z & 255, nz = (D.z >> 8) & 255, E = ny * nz;
    const int shape = (ny > 8 ? 3 : 0) + (nz > 12 ? 2 : nz > 8 ? 1 : 0);  // RJ in {1, 2} x RK in {2, 3, 4}
    switch (shape) {
      case 0: grid_outer<S, 1, 2>(X, c0, sl, sc, n, D, st4, Mw); break;
      case 1: grid_outer<S, 1, 3>(X, c0, sl, sc, n, D, st4, Mw); break;
      case 2: grid_outer<S, 1, 4>(X, c0, sl, sc, n, D, st4, Mw); break;
      case 3: grid_outer<S, 2, 2>(X, c0, sl, sc, n, D, st4, Mw); break;
      case 4: grid_outer<S, 2, 3>(X, c0, sl, sc, n, D, st4, Mw); break;
      default: grid_outer<S, 2, 4>(X, c0, sl, sc, n, D, st4, Mw); break;
    }
    if (lane == 0) work += (unsigned long long)__popcll(m) * E;
    flat_rules<S>(J, X, D, Mw, P, work, corner);
  }
}

// Pair-factored gather (level mode 2), see the file comment.  FLAT: every
// job this kernel runs is in the flat-tile form, so the other pair loops are
// not compiled in (a smaller kernel for the instruction cache).
template <int S, bool FLAT = false>
__device__ void gather_pairs(const DevJob& J, const DevLevel& L, bool gated, float* P, const Smem& sm,
                             CellCtx& X) {
  const int ms = L.mask_size, grp = FLAT ? L.pair_group : 1;
  const int nkeys = grp <= 1 ? L.n_coarse : (L.n_coarse + 15) >> 4;  // pair keys: coarse symbols or groups
  // the pair list of this kernel's form (the flat-tile form has its own, of sub-tiles)
  const int npair = FLAT ? J.fnpair : J.npair;
  const int* pair_key = FLAT ? J.fpair_key : J.pair_key;
  const int* pair_gate = FLAT ? J.fpair_gate : J.pair_gate;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int* aoff = J.a_is_t ? L.t_mem_off : L.nt_mem_off;
  const int* amem = J.a_is_t ? L.t_mem : L.nt_mem;
  const int* boff = J.b_is_t ? L.t_mem_off : L.nt_mem_off;
  const int* bmem = J.b_is_t ? L.t_mem : L.nt_mem;
  float* Mw = sm.M + warp * sm.mtile;
  const int nsp = X.nsp;
  unsigned long long work = 0, corner = 0;
  if (FLAT && threadIdx.x < 4 && nsp > 0) {
    // the split lists run in groups of four: repeat the last split
    X.aptr[nsp + threadIdx.x] = X.aptr[nsp - 1];
    X.bptr[nsp + threadIdx.x] = X.bptr[nsp - 1];
  }
  if (FLAT && lane < 16) {
    // the -inf rows of the flat-tile stage (rows 16 and kStageRowB + 16 of both buffers)
    const int row = (lane >> 3) * kStageRows + ((lane & 4) ? kStageRowB + 16 : 16);
    sm.stage[warp * kStageFloats + row * 4 + (lane & 3)] = -CUDART_INF_F;
  }
  // the cell's gate per segment, one ballot per 32 segments (read after the
  // first barrier below)
  for (int base = 0; base < J.nseg; base += blockDim.x) {
    const int sg = base + threadIdx.x;
    const bool hit = sg < J.nseg && (!gated || gate_hit(J, sg, ms, L.gate_merged, X.gate));
    const unsigned b = __ballot_sync(kFull, hit);
    if (lane == 0 && sg < J.nseg) X.segpass[sg >> 5] = b;
  }
  for (int c0 = 0; c0 < nsp; c0 += kPairChunk) {
    const int nc = min(kPairChunk, nsp - c0);
    for (int i = threadIdx.x; i < nc * ms; i += blockDim.x) {
      const int s = i / ms, w = i - s * ms;
      X.la[s][w] = __ldg(X.alive[c0 + s] + w);
      X.lb[s][w] = __ldg(X.blive[c0 + s] + w);
    }
    if (threadIdx.x == 0) {
      X.nlive = 0;
      X.next = 0;
    }
    __syncthreads();
    // pl[ca] = union over splits with a live key ca on the left of the right-hand live sets
    for (int ca = threadIdx.x; ca < nkeys; ca += blockDim.x) {
      unsigned acc[kMaxMask];
#pragma unroll
      for (int w = 0; w < kMaxMask; ++w) acc[w] = 0u;
      for (int s = 0; s < nc; ++s) {
        if (key_live(X.la[s], ca, grp)) {
#pragma unroll
          for (int w = 0; w < kMaxMask; ++w)
            if (w < ms) acc[w] |= (unsigned)X.lb[s][w];
        }
      }
#pragma unroll
      for (int w = 0; w < kMaxMask; ++w)
        if (w < ms) sm.pl[ca * ms + w] = acc[w];
    }
    __syncthreads();
    // compact the live pairs (coarse liveness, then the OR of their segments' bits)
    for (int base = 0; base < npair; base += blockDim.x) {
      const int k = base + threadIdx.x;
      bool live = false;
      if (k < npair) {
        const int key = __ldg(pair_key + k);
        const int ca = key & 255, cb = (key >> 8) & 255;
        live = key_live(reinterpret_cast<const int*>(sm.pl) + ca * ms, cb, grp);
        if (live && gated) {
          bool hit = false;
          for (int i = 0; i < ms; ++i) hit |= (__ldg(pair_gate + k * ms + i) & X.gate[i]) != 0;
          live = hit;
        }
      }
      // the list keeps pair order (a prefix over warps, not an atomic
      // counter): the parts of a split cell index the same list
      const unsigned bal = __ballot_sync(kFull, live);
      if (lane == 0) X.wcnt[warp] = __popc(bal);
      __syncthreads();
      int wb = X.nlive, total = 0;
      for (int w = 0; w < nwarps; ++w) {
        const int c = X.wcnt[w];
        wb += w < warp ? c : 0;
        total += c;
      }
      if (live) sm.list[wb + __popc(bal & ((1u << lane) - 1u))] = k;
      __syncthreads();  // every thread has read X.nlive and X.wcnt
      if (threadIdx.x == 0) X.nlive += total;
    }
    __syncthreads();
    const int nlive = X.nlive;
    if (FLAT) {
      flat_pairs<S>(J, sm, X, c0, nc, nlive, grp, Mw, P, work, corner);
      __syncthreads();
      continue;
    }
    for (int i = X.g * nwarps + warp; i < nlive; i += X.G * nwarps) {
      const int p = sm.list[i];
      const int key = __ldg(J.pair_key + p);
      const int ca = key & 255, cb = (key >> 8) & 255;
      const unsigned lo = __ballot_sync(kFull, lane < nc && bit(X.la[lane], ca) && bit(X.lb[lane], cb));
      const unsigned hi =
          __ballot_sync(kFull, lane + 32 < nc && bit(X.la[lane + 32], ca) && bit(X.lb[lane + 32], cb));
      const unsigned long long m = (unsigned long long)lo | ((unsigned long long)hi << 32);
      const int a0 = __ldg(aoff + ca), ny = __ldg(aoff + ca + 1) - a0;
      const int b0 = __ldg(boff + cb), nz = __ldg(boff + cb + 1) - b0;
      const int nkq = (nz + 3) >> 2, ntask = ny * nkq;
      if (S == SEMI_VITERBI && J.interleaved && sm.stage && ntask <= 64 && ny <= 32 && nz <= 32) {
        // outer product with each split's member values staged in shared
        // memory: per step a lane loads one A and one B member of two live
        // splits, then every task reads its operands from the stage
        float(*st)[2][32] = reinterpret_cast<float(*)[2][32]>(sm.stage + warp * kStageFloats);
        // ny, nz <= 16: one load per lane stages both operands (lanes 0-15 the
        // A members, lanes 16-31 the B members) into st[s][0]
        const bool narrow = ny <= 16 && nz <= 16;
        const int my_a = lane < ny ? __ldg(amem + a0 + lane) : -1;
        const int my_b = lane < nz ? __ldg(bmem + b0 + lane) : -1;
        const int my_n = lane < 16 ? (lane < ny ? __ldg(amem + a0 + lane) : -1)
                                   : (lane - 16 < nz ? __ldg(bmem + b0 + lane - 16) : -1);
        const int yoff = narrow ? 16 : 0;
        int tj[2], tk[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int t = lane + 32 * u;
          tj[u] = t < ntask ? t / nkq : -1;
          tk[u] = t < ntask ? (t - tj[u] * nkq) * 4 : 0;
        }
        float acc[2][4];
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[u][q] = -CUDART_INF_F;
        for (unsigned long long mm = m; mm;) {
          const int s0 = __ffsll(mm) - 1;
          mm &= mm - 1;
          const int s1 = mm ? __ffsll(mm) - 1 : s0;
          if (mm) mm &= mm - 1;
          if (narrow) {
            const float* r0 = lane < 16 ? X.aptr[c0 + s0] : X.bptr[c0 + s0];
            const float* r1 = lane < 16 ? X.aptr[c0 + s1] : X.bptr[c0 + s1];
            st[0][0][lane] = my_n >= 0 ? __ldg(r0 + my_n) : -CUDART_INF_F;
            st[1][0][lane] = my_n >= 0 ? __ldg(r1 + my_n) : -CUDART_INF_F;
          } else {
            st[0][0][lane] = my_a >= 0 ? __ldg(X.aptr[c0 + s0] + my_a) : -CUDART_INF_F;
            st[0][1][lane] = my_b >= 0 ? __ldg(X.bptr[c0 + s0] + my_b) : -CUDART_INF_F;
            st[1][0][lane] = my_a >= 0 ? __ldg(X.aptr[c0 + s1] + my_a) : -CUDART_INF_F;
            st[1][1][lane] = my_b >= 0 ? __ldg(X.bptr[c0 + s1] + my_b) : -CUDART_INF_F;
          }
          __syncwarp();
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            if (tj[u] < 0) continue;
            const float x0 = st[0][0][tj[u]], x1 = st[1][0][tj[u]];
            const float4 y0 = *reinterpret_cast<const float4*>(&st[0][narrow ? 0 : 1][yoff + tk[u]]);
            const float4 y1 = *reinterpret_cast<const float4*>(&st[1][narrow ? 0 : 1][yoff + tk[u]]);
            acc[u][0] = fmaxf(acc[u][0], fmaxf(x0 + y0.x, x1 + y1.x));
            acc[u][1] = fmaxf(acc[u][1], fmaxf(x0 + y0.y, x1 + y1.y));
            acc[u][2] = fmaxf(acc[u][2], fmaxf(x0 + y0.z, x1 + y1.z));
            acc[u][3] = fmaxf(acc[u][3], fmaxf(x0 + y0.w, x1 + y1.w));
          }
          __syncwarp();
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          if (tj[u] < 0) continue;
#pragma unroll
          for (int q = 0; q < 4; ++q)
            if (tk[u] + q < nz) Mw[tj[u] * nz + tk[u] + q] = acc[u][q];
        }
      } else
      // outer product over the live splits: M[j][k] = max_s A_s[Y_j] + B_s[Z_k]
      for (int t = lane; t < ntask; t += 32) {
        const int j = t / nkq, k0 = (t - j * nkq) * 4;
        const int ai = __ldg(amem + a0 + j);
        int bi[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) bi[q] = k0 + q < nz ? __ldg(bmem + b0 + k0 + q) : -1;
        float acc[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q] = Sr<S>::zero();
        if (S != SEMI_VITERBI || !J.interleaved) {
          // one split per step (the sum-product pass and the outside jobs)
          for (unsigned long long mm = m; mm; mm &= mm - 1) {
            const int s = __ffsll(mm) - 1;
            const float* A = X.aptr[c0 + s];
            const float* B = X.bptr[c0 + s];
            const float a = __ldg(A + ai);
            if (S == SEMI_VITERBI) {
#pragma unroll
              for (int q = 0; q < 4; ++q)
                if (bi[q] >= 0) acc[q] = fmaxf(acc[q], a + __ldg(B + bi[q]));
            } else {
              const float as = a * X.scl[c0 + s];
#pragma unroll
              for (int q = 0; q < 4; ++q)
                if (bi[q] >= 0) acc[q] = fmaf(as, __ldg(B + bi[q]), acc[q]);
            }
          }
        } else
        // two live splits per step, their loads issued together; an odd last
        // split is paired with itself (max is idempotent)
        for (unsigned long long mm = m; mm;) {
          const int s0 = __ffsll(mm) - 1;
          mm &= mm - 1;
          const bool two = mm != 0;
          const int s1 = two ? __ffsll(mm) - 1 : s0;
          if (two) mm &= mm - 1;
          const float* A0 = X.aptr[c0 + s0];
          const float* B0 = X.bptr[c0 + s0];
          const float* A1 = X.aptr[c0 + s1];
          const float* B1 = X.bptr[c0 + s1];
          const float a0v = __ldg(A0 + ai), a1v = __ldg(A1 + ai);
          float b0v[4], b1v[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            b0v[q] = bi[q] >= 0 ? __ldg(B0 + bi[q]) : 0.f;
            b1v[q] = bi[q] >= 0 ? __ldg(B1 + bi[q]) : 0.f;
          }
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[q] = fmaxf(acc[q], fmaxf(a0v + b0v[q], a1v + b1v[q]));
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (bi[q] >= 0) Mw[j * nz + k0 + q] = acc[q];
      }
      __syncwarp();
      if (lane == 0) work += (unsigned long long)__popcll(m) * ny * nz;
      // every rule of the pair's gated-in blocks: M[j][k] (x) w into its target
      const int bk1 = __ldg(J.pair_blk + p + 1);
      for (int bk = __ldg(J.pair_blk + p); bk < bk1; ++bk) {
        {
          const int sg = __ldg(J.blk_seg + bk);
          if (!((X.segpass[sg >> 5] >> (sg & 31)) & 1u)) continue;
        }
        int cur = -1;
        float run = Sr<S>::zero();
        if (!J.interleaved) {
          // rules stored block after block (sum-product levels and outside
          // jobs): lane l reads its contiguous slice one rule per step, rule
          // form j | k << 8
          const int r0 = __ldg(J.blk_ptr + bk), r1 = __ldg(J.blk_ptr + bk + 1);
          const int per = (r1 - r0 + 31) >> 5;
          const int rs = r0 + lane * per, re = min(r1, rs + per);
          for (int r = rs; r < re; ++r) {
            const int2 R = __ldg(J.pair_rules + r);
            const int jj = R.x & 255, kk = (R.x >> 8) & 255, t = (int)((unsigned)R.x >> 16);
            const float w = __int_as_float(R.y);
            const float v = S == SEMI_VITERBI ? Mw[jj * nz + kk] + w : Mw[jj * nz + kk] * w;
            if (t != cur) {
              if (cur >= 0) flush_run<S>(P, cur, run, corner);
              cur = t;
              run = v;
            } else {
              run = Sr<S>::add(run, v);
            }
          }
          if (cur >= 0) flush_run<S>(P, cur, run, corner);
          if (lane == 0) work += (unsigned long long)(r1 - r0);
          continue;
        }
        // lane l runs its contiguous, target-sorted slice of the block; the
        // slices are stored interleaved, so each step's loads are coalesced
        const int r0 = __ldg(J.blk_ptr + bk), per = (__ldg(J.blk_ptr + bk + 1) - r0) >> 5;
        if (J.interleaved == 2) {
          // every rule of the lane's slice has the same target: one running
          // max, flushed once (padding rules carry the zero weight)
          float best = Sr<S>::zero();
          int tl = 0;
          for (int i0 = 0; i0 < per; i0 += kRuleBatch) {
            int2 R[kRuleBatch];
#pragma unroll
            for (int q = 0; q < kRuleBatch; ++q) R[q] = __ldg(J.pair_rules + r0 + (i0 + q) * 32 + lane);
            float m4[kRuleBatch];
#pragma unroll
            for (int q = 0; q < kRuleBatch; ++q) m4[q] = Mw[R[q].x & 0xffff];
#pragma unroll
            for (int q = 0; q < kRuleBatch; ++q) best = Sr<S>::add(best, m4[q] + __int_as_float(R[q].y));
            tl = (int)((unsigned)R[0].x >> 16);
          }
          flush_run<S>(P, tl, best, corner);
          if (lane == 0) work += (unsigned long long)__ldg(J.blk_nrule + bk);
          continue;
        }
        // kRuleBatch rules per step: their loads are issued before any is used
        // (the step count `per` is the same for every lane of the warp)
        for (int i0 = 0; i0 < per; i0 += kRuleBatch) {
          int2 R[kRuleBatch];
#pragma unroll
          for (int q = 0; q < kRuleBatch; ++q)
            R[q] = i0 + q < per ? __ldg(J.pair_rules + r0 + (i0 + q) * 32 + lane) : make_int2(0, 0);
          float m4[kRuleBatch];
#pragma unroll
          for (int q = 0; q < kRuleBatch; ++q) m4[q] = Mw[R[q].x & 0xffff];
#pragma unroll
          for (int q = 0; q < kRuleBatch; ++q) {
            if (i0 + q >= per) break;
            const int t = (int)((unsigned)R[q].x >> 16);
            const float w = __int_as_float(R[q].y);
            const float v = m4[q] + w;
            if (t != cur) {
              if (cur >= 0) flush_run<S>(P, cur, run, corner);
              cur = t;
              run = v;
            } else {
              run = Sr<S>::add(run, v);
            }
          }
        }
        if (cur >= 0) flush_run<S>(P, cur, run, corner);
        if (lane == 0) work += (unsigned long long)__ldg(J.blk_nrule + bk);
      }
      __syncwarp();
    }
    __syncthreads();
  }
  if (nsp == 0) __syncthreads();  // see gather()
  if (lane == 0 && (work | corner)) {
    atomicAdd(&X.work, work);
    atomicAdd(&X.corner, corner);
  }
}

// MODE 0 target-major, 2 pair-factored, 3 pair-factored with every job in
// the flat-tile form (Viterbi inside passes).
//
// The span kernels run their jobs one after another in one CTA, and one warp
// (or one thread) writes each job's split count, operand pointers, gates and
// pair list into the CTA's shared bookkeeping.  Every warp must leave a job
// before the next job's setup is written, or a warp still reading this job's
// split count would run its tables over the next job's splits and pair list.
// A gather with splits ends on a barrier that every warp reaches after its
// last read of them (the last barrier of its chunk loop); one without splits
// ends on a barrier of its own.  Each warp's copy of the split count is this
// job's: the next one is written only after all warps passed one of those
// barriers.
template <int S, int MODE>
__device__ __forceinline__ void gather(const DevJob& J, const DevLevel& L, bool gated, float* P, const Smem& sm,
                                       int chunk, CellCtx& X) {
  if constexpr (MODE == 3) gather_pairs<S, true>(J, L, gated, P, sm, X);
  else if constexpr (MODE == 2 && S != SEMI_LOGSUM) gather_pairs<S>(J, L, gated, P, sm, X);
  else if (S != SEMI_LOGSUM && !gated && J.pm_npair > 0) gather_pairmajor<S>(J, L, P, sm.stA, sm.stB, chunk, X);
  else gather_targets<S>(J, L, gated, P, sm.stA, sm.stB, chunk, X);
}

// Liveness bitset of a shared-memory row (n_valid symbols projected by proj).
template <int S>
__device__ void live_bits(const float* row, int n_valid, const int* proj, int ms, CellCtx& X, int* dst) {
  if (threadIdx.x < kMaxMask) X.words[threadIdx.x] = 0u;
  __syncthreads();
  unsigned w[kMaxMask];
#pragma unroll
  for (int i = 0; i < kMaxMask; ++i) w[i] = 0u;
  for (int k = threadIdx.x; k < n_valid; k += blockDim.x) {
    if (Sr<S>::live(row[k])) {
      const int c = __ldg(proj + k);
#pragma unroll
      for (int i = 0; i < kMaxMask; ++i)
        if ((c >> 5) == i) w[i] |= 1u << (c & 31);
    }
  }
#pragma unroll
  for (int i = 0; i < kMaxMask; ++i) {
    const unsigned v = __reduce_or_sync(kFull, w[i]);
    if ((threadIdx.x & 31) == 0 && v) atomicOr(&X.words[i], v);
  }
  __syncthreads();
  if (dst && threadIdx.x < ms) dst[threadIdx.x] = (int)X.words[threadIdx.x];
}

template <int S>
__device__ void unary_into(const DevUJob& U, const float* src, float* dst, int cs, bool allowed, float scale) {
  for (int k = threadIdx.x; k < cs; k += blockDim.x) dst[k] = Sr<S>::zero();
  if (!allowed) return;
  for (int t = threadIdx.x; t < U.n_tgt; t += blockDim.x) {
    const int r0 = __ldg(U.rowptr + t), r1 = __ldg(U.rowptr + t + 1);
    if (r0 == r1) continue;
    float acc = Sr<S>::zero();
    int r = r0;
    if (S == SEMI_VITERBI) {
      // four independent running maxima (max is exact in any order), so four
      // rule loads are in flight at once
      float a1 = acc, a2 = acc, a3 = acc;
      for (; r + 4 <= r1; r += 4) {
        const int2 q0 = __ldg(U.rules + r), q1 = __ldg(U.rules + r + 1);
        const int2 q2 = __ldg(U.rules + r + 2), q3 = __ldg(U.rules + r + 3);
        acc = fmaxf(acc, src[q0.x] + __int_as_float(q0.y));
        a1 = fmaxf(a1, src[q1.x] + __int_as_float(q1.y));
        a2 = fmaxf(a2, src[q2.x] + __int_as_float(q2.y));
        a3 = fmaxf(a3, src[q3.x] + __int_as_float(q3.y));
      }
      acc = fmaxf(fmaxf(acc, a1), fmaxf(a2, a3));
    }
    for (; r < r1; ++r) {
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

// Parts of a cell split over several CTAs: each part publishes its partial
// row; the last part to arrive combines the rows in part order into P and
// goes on to finish the cell.  Returns false for the parts that stop here.
template <int S>
__device__ bool combine_parts(const DevWork& W, CellCtx& X, float* P, int cs, long long cell) {
  if (X.G == 1) return true;
  store_cell(W.part_rows + (size_t)blockIdx.x * cs, P, cs);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) X.last = atomicAdd(W.cell_cnt + cell, 1) == X.G - 1;
  __syncthreads();
  if (!X.last) return false;
  __threadfence();
  const float* base = W.part_rows + (size_t)(blockIdx.x - X.g) * cs;
  for (int k = threadIdx.x; k < cs; k += blockDim.x) {
    float acc = Sr<S>::zero();
    for (int j = 0; j < X.G; ++j) acc = Sr<S>::add(acc, j == X.g ? P[k] : __ldcg(base + (size_t)j * cs + k));
    P[k] = acc;
  }
  if (threadIdx.x == 0) W.cell_cnt[cell] = 0;
  __syncthreads();
  return true;
}

__device__ __forceinline__ void flush_counters(CellCtx& X, const Counters& C) {
  if (threadIdx.x == 0) {
    if (X.work && C.work) atomicAdd(C.work, X.work);
    if (X.corner && C.corner) atomicAdd(C.corner, X.corner);
  }
}

// ---------------------------------------------------------------------------
// Inside pass over the cells of a work list (span 1: the unary layer over
// lexicon cells).  Register budgets: five CTAs per SM for the pair-factored
// passes (48 registers: the flat-tile path keeps up to eight tile entries
// and their stage offsets in registers; the sum-product one spills 32 bytes
// there and is still 18% faster than four CTAs at 63 registers), six for the
// target-major ones.
template <int S, int MODE>
__global__ void __launch_bounds__(256, MODE >= 2 ? 5 : 6)
    k_inside_span(DevLevel L, DevBatch B, DevWork W, DevMask M, float* inside, DevLive V, Counters C, int chunk) {
  extern __shared__ __align__(16) float smem[];
  __shared__ CellCtx X;
  const int cs = L.cell_size, ms = L.mask_size;
  const Smem sm = carve(smem, L, chunk, S == SEMI_VITERBI || MODE == 3, MODE >= 2, MODE == 3);
  float* P = sm.P;
  float* Q = sm.Q;
  const int ent = entry_of(W, blockIdx.x);
  const int s = W.sent[ent], span = span_of(W, ent), n = B.len[s];
  const int G = ways_of(W, ent), local = (int)blockIdx.x - W.pref[ent];
  const int b = local / G, e = b + span, g = local - (local / G) * G;
  const long long off = B.cell_off[s], toff = off + tri(n);
  const long long pbot = off + chart_index(b, e, n), ptop = toff + chart_index(b, e, n);
  if (threadIdx.x == 0) {
    X.flag0 = span == 1 ? 1 : mask_any(M, pbot);
    X.flag1 = mask_any(M, ptop);
    X.work = 0;
    X.corner = 0;
    // a pruned cell has no rule work: part 0 finishes it alone
    X.G = X.flag0 && span >= 2 && !(S == SEMI_REAL && L.tc_binary) ? G : 1;
    X.g = X.flag0 && span >= 2 ? g : 0;
    if (M.bits)
      for (int i = 0; i < ms; ++i) X.gate[i] = M.bits[pbot * ms + i];
  }
  for (int k = threadIdx.x; k < cs; k += blockDim.x) P[k] = Sr<S>::zero();
  __syncthreads();
  if (X.G == 1 && g != 0) return;  // a spare part of a pruned cell
  const bool gated = M.bits != nullptr;
  const float ps = S == SEMI_REAL ? scale_of(M.iscale, pbot) : 0.f;
  auto BOT = [&](int x, int y) { return off + chart_index(x, y, n); };
  auto TOP = [&](int x, int y) { return toff + chart_index(x, y, n); };
  auto split = [&](long long lc, long long rc) {
    if (mask_any(M, lc) && mask_any(M, rc))
      add_split<S>(X, inside + lc * cs, inside + rc * cs, V.in + lc * ms, V.in + rc * ms, scale_of(M.iscale, lc),
                   scale_of(M.iscale, rc), ps);
  };
  if (span == 1 || (S == SEMI_REAL && L.tc_binary && X.flag0)) {
    // lexicon scores, or binary sums the tensor-core pass left in the bot cell
    for (int k = threadIdx.x; k < cs; k += blockDim.x) P[k] = inside[pbot * cs + k];
  } else if (X.flag0) {
    for (int job = 0; job < 4; ++job) {
      const int jid = job == 0 ? IN_TT : job == 1 ? IN_NT : job == 2 ? IN_TN : IN_NN;
      if (jid == IN_TT && span != 2) continue;
      if (L.jobs[jid].n_tgt == 0 || L.jobs[jid].nseg == 0) continue;
      if (jid != IN_NN) {
        if (threadIdx.x == 0) {
          X.nsp = 0;
          if (jid == IN_NT) split(TOP(b, e - 1), BOT(e - 1, e));
          else if (jid == IN_TN) split(BOT(b, b + 1), TOP(b + 1, e));
          else split(BOT(b, b + 1), BOT(b + 1, e));
        }
      } else if (threadIdx.x < 32) {
        // the allowed splits, 32 at a time (their mask loads in parallel),
        // kept in split order
        const int lane = threadIdx.x;
        int k0 = 0;
        for (int sp0 = b + 1; sp0 < e; sp0 += 32) {
          const int sp = sp0 + lane;
          const long long lc = sp < e ? TOP(b, sp) : 0, rc = sp < e ? TOP(sp, e) : 0;
          const bool ok = sp < e && mask_any(M, lc) && mask_any(M, rc);
          const unsigned bal = __ballot_sync(kFull, ok);
          if (ok)
            put_split<S>(X, k0 + __popc(bal & ((1u << lane) - 1u)), inside + lc * cs, inside + rc * cs,
                         V.in + lc * ms, V.in + rc * ms, scale_of(M.iscale, lc), scale_of(M.iscale, rc), ps);
          k0 += __popc(bal);
        }
        if (lane == 0) X.nsp = k0;
      }
      __syncthreads();
      gather<S, MODE>(L.jobs[jid], L, gated, P, sm, chunk, X);
    }
  }
  __syncthreads();
  if (!combine_parts<S>(W, X, P, cs, pbot)) {
    flush_counters(X, C);
    return;
  }
  if (span >= 2) {
    store_cell(inside + pbot * cs, P, cs);
    live_bits<S>(P, L.n_nt, L.nt_coarse, ms, X, V.in + pbot * ms);
  }
  // unary layer: top cell (whole row replaced, CLParser.scala:721-727)
  const float us = S == SEMI_REAL ? __expf(-scale_of(M.iscale, ptop) + scale_of(M.iscale, pbot)) : 1.f;
  unary_into<S>(L.ujobs[span == 1 ? IN_TU : IN_NU], P, Q, cs, X.flag1 != 0, us);
  __syncthreads();
  store_cell(inside + ptop * cs, Q, cs);
  live_bits<S>(Q, L.n_nt, L.nt_coarse, ms, X, V.in + ptop * ms);
  flush_counters(X, C);
}

// ---------------------------------------------------------------------------
// Outside pass over the cells of a work list: outside-top of each cell gathered from its
// parents, then the unary layer to outside-bot (and, at span 1, the
// terminal-child binaries that the reference runs after its span loop).
// Register budgets: five CTAs per SM for the pair-factored passes, six for
// the target-major Viterbi pass (40 registers; 15% faster than four CTAs at
// 64 on the bench's coarse level despite a few spilled bytes), four for the
// target-major sum-product passes.
template <int S, int MODE>
__global__ void __launch_bounds__(256, MODE >= 2 ? 5 : S == SEMI_VITERBI ? 6 : 4)
    k_outside_span(DevLevel L, DevBatch B, DevWork W, DevMask M, const float* inside, float* outside, DevLive V,
                   Counters C, int chunk) {
  extern __shared__ __align__(16) float smem[];
  __shared__ CellCtx X;
  const int cs = L.cell_size, ms = L.mask_size;
  const Smem sm = carve(smem, L, chunk, MODE == 3, MODE == 3 || L.mode == 2, MODE == 3);
  float* P = sm.P;
  float* Q = sm.Q;
  const int ent = entry_of(W, blockIdx.x);
  const int s = W.sent[ent], span = span_of(W, ent), n = B.len[s];
  const int G = ways_of(W, ent), local = (int)blockIdx.x - W.pref[ent];
  const int b = local / G, e = b + span, g = local - (local / G) * G;
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
    // parts split the parent gathers of span >= 2 (span 1 runs a second
    // gather after its unary layer and is never split)
    const bool parts = X.flag0 && span >= 2 && span != n;
    X.G = parts ? G : 1;
    X.g = parts ? g : 0;
    if (M.bits)
      for (int i = 0; i < ms; ++i) X.gate[i] = M.bits[ctop * ms + i];
  }
  for (int k = threadIdx.x; k < cs; k += blockDim.x) P[k] = Sr<S>::zero();
  __syncthreads();
  if (X.G == 1 && g != 0) return;  // a spare part of a cell without parent gathers
  const float* IS = M.iscale;
  const float* OS = M.oscale;
  // operand helpers: (outside parent, inside sibling) or (inside sibling, outside parent)
  float ps = 0.f;
  auto split_oi = [&](long long oc, long long ic) {
    if (mask_any(M, oc) && mask_any(M, ic))
      add_split<S>(X, outside + oc * cs, inside + ic * cs, V.out + oc * ms, V.in + ic * ms, scale_of(OS, oc),
                   scale_of(IS, ic), ps);
  };
  auto split_io = [&](long long ic, long long oc) {
    if (mask_any(M, ic) && mask_any(M, oc))
      add_split<S>(X, inside + ic * cs, outside + oc * cs, V.in + ic * ms, V.out + oc * ms, scale_of(IS, ic),
                   scale_of(OS, oc), ps);
  };
  // the allowed splits sp in [lo, hi) of a range job, built by warp 0 32 at a
  // time (mask loads in parallel) in split order; cells(sp, c1, c2) names the
  // operand cells, outside-then-inside when oi
  auto range_splits = [&](int lo, int hi, bool oi, auto cells) {
    if (threadIdx.x >= 32) return;
    const int lane = threadIdx.x;
    int k0 = 0;
    for (int s0 = lo; s0 < hi; s0 += 32) {
      const int sp = s0 + lane;
      long long c1 = 0, c2 = 0;
      if (sp < hi) cells(sp, c1, c2);
      const bool ok = sp < hi && mask_any(M, c1) && mask_any(M, c2);
      const unsigned bal = __ballot_sync(kFull, ok);
      if (ok) {
        const int k = k0 + __popc(bal & ((1u << lane) - 1u));
        if (oi)
          put_split<S>(X, k, outside + c1 * cs, inside + c2 * cs, V.out + c1 * ms, V.in + c2 * ms, scale_of(OS, c1),
                       scale_of(IS, c2), ps);
        else
          put_split<S>(X, k, inside + c1 * cs, outside + c2 * cs, V.in + c1 * ms, V.out + c2 * ms, scale_of(IS, c1),
                       scale_of(OS, c2), ps);
      }
      k0 += __popc(bal);
    }
    if (lane == 0) X.nsp = k0;
  };
  if (span == n) {
    if (threadIdx.x == 0) P[L.root] = Sr<S>::one();  // setRootScores
  } else if (X.flag0) {
    ps = S == SEMI_REAL ? scale_of(OS, ctop) : 0.f;
    for (int job = 0; job < 4; ++job) {
      const int jid = job == 0 ? OUT_R_TN : job == 1 ? OUT_L_NT : job == 2 ? OUT_L_NN : OUT_R_NN;
      if (L.jobs[jid].n_tgt == 0 || L.jobs[jid].nseg == 0) continue;
      // no split at the sentence's edges: a right-child job needs a parent
      // starting before b, a left-child job one ending after e
      if ((jid == OUT_R_TN || jid == OUT_R_NN) ? b < 1 : e + 1 > n) continue;
      if (jid == OUT_L_NN) {
        range_splits(e + 1, n + 1, true, [&](int sp, long long& c1, long long& c2) {
          c1 = BOT(b, sp);
          c2 = TOP(e, sp);
        });
      } else if (jid == OUT_R_NN) {
        range_splits(0, b, false, [&](int sp, long long& c1, long long& c2) {
          c1 = TOP(sp, b);
          c2 = BOT(sp, e);
        });
      } else if (threadIdx.x == 0) {
        X.nsp = 0;
        if (jid == OUT_R_TN) {
          if (b >= 1) split_io(BOT(b - 1, b), BOT(b - 1, e));
        } else if (e + 1 <= n) {
          split_oi(BOT(b, e + 1), BOT(e, e + 1));
        }
      }
      __syncthreads();
      gather<S, MODE>(L.jobs[jid], L, gated, P, sm, chunk, X);
    }
  }
  __syncthreads();
  if (!combine_parts<S>(W, X, P, cs, ctop)) {
    flush_counters(X, C);
    return;
  }
  store_cell(outside + ctop * cs, P, cs);
  live_bits<S>(P, L.n_nt, L.nt_coarse, ms, X, V.out ? V.out + ctop * ms : nullptr);
  // unary layer: outside-bot from outside-top.  With a batch of one-word
  // sentences only, the reference's first unary call (at span == maxLength)
  // uses the nonterminal unaries and its span loop never runs.
  const bool use_tu = span == 1 && !W.one_word_batch;
  const float us = S == SEMI_REAL ? __expf(-scale_of(OS, cbot) + scale_of(OS, ctop)) : 1.f;
  unary_into<S>(L.ujobs[use_tu ? OUT_TU : OUT_NU], P, Q, cs, X.flag0 != 0, us);
  __syncthreads();
  if (span == 1 && X.flag1) {
    // terminal-child buckets, gated by the bot cell's mask (CLParser.scala:345-355)
    if (threadIdx.x == 0 && M.bits)
      for (int i = 0; i < ms; ++i) X.gate[i] = M.bits[cbot * ms + i];
    ps = S == SEMI_REAL ? scale_of(OS, cbot) : 0.f;
    for (int job = 0; job < 4; ++job) {
      const int jid = job == 0 ? OUT_L_TT : job == 1 ? OUT_R_NT : job == 2 ? OUT_L_TN : OUT_R_TT;
      if (L.jobs[jid].n_tgt == 0 || L.jobs[jid].nseg == 0) continue;
      if ((jid == OUT_R_NT || jid == OUT_R_TT) ? b < 1 : b + 2 > n) continue;  // as above
      if (jid == OUT_R_NT) {
        range_splits(0, b, false, [&](int sp, long long& c1, long long& c2) {
          c1 = TOP(sp, b);
          c2 = BOT(sp, b + 1);
        });
      } else if (jid == OUT_L_TN) {
        range_splits(b + 2, n + 1, true, [&](int sp, long long& c1, long long& c2) {
          c1 = BOT(b, sp);
          c2 = TOP(b + 1, sp);
        });
      } else if (threadIdx.x == 0) {
        X.nsp = 0;
        if (jid == OUT_L_TT) {
          if (b + 2 <= n) split_oi(BOT(b, b + 2), BOT(b + 1, b + 2));
        } else if (b >= 1) {
          split_io(BOT(b - 1, b), BOT(b - 1, b + 1));
        }
      }
      __syncthreads();
      gather<S, MODE>(L.jobs[jid], L, gated, Q, sm, chunk, X);
    }
  }
  __syncthreads();
  store_cell(outside + cbot * cs, Q, cs);
  const bool term = span == 1 && use_tu;
  live_bits<S>(Q, term ? L.n_t : L.n_nt, term ? L.t_coarse : L.nt_coarse, ms, X,
               V.out ? V.out + cbot * ms : nullptr);
  flush_counters(X, C);
}

// ---------------------------------------------------------------------------
// Lexicon (CLParser.scala:426-467): one warp per token writes its bot span-1
// cell: the semiring zero except the word's allowed preterminals.
template <int S>
__global__ void k_lexicon(DevLevel L, DevBatch B, DevWork W, DevMask M, float* inside, double* part_scale,
                          DevLive V, int* status) {
  const long long unit = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (unit >= W.nunits) return;
  const int ent = entry_of(W, (int)unit);
  const int s = W.sent[ent], pos = (int)unit - W.pref[ent];
  const long long tok = B.word_off[s] + pos;
  const int cs = L.cell_size, ms = L.mask_size;
  const long long cell = B.cell_off[s] + pos;  // chartIndex(pos, pos + 1) == pos
  float* row = inside + cell * cs;
  for (int k = lane; k < cs; k += 32) row[k] = Sr<S>::zero();
  __syncwarp();
  const int w = B.words[tok];
  unsigned bits[kMaxMask];
#pragma unroll
  for (int i = 0; i < kMaxMask; ++i) bits[i] = 0u;
  if (w < 0 || w >= L.n_words) {
    if (lane == 0 && status) status[s] = 4;  // PUCK_ERR_OOV
  } else {
    const long long x0 = L.lex_off[w], x1 = L.lex_off[w + 1];
    for (long long x = x0 + lane; x < x1; x += 32) {
      const int c = L.t_coarse[L.lex_term[x]];
#pragma unroll
      for (int i = 0; i < kMaxMask; ++i)
        if ((c >> 5) == i) bits[i] |= 1u << (c & 31);
    }
    if (S == SEMI_REAL) {
      const float my_scale = __expf(-scale_of(M.iscale, cell));
      float total = 0.f;
      for (long long x = x0 + lane; x < x1; x += 32) {
        const float v = __expf(L.lex_score[x]) * my_scale;
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
  }
#pragma unroll
  for (int i = 0; i < kMaxMask; ++i) {
    const unsigned v = __reduce_or_sync(kFull, bits[i]);
    if (lane == 0 && i < ms) V.in[cell * ms + i] = (int)v;
  }
}

template <class K>
cudaError_t set_smem(K kernel, size_t bytes) {
  // static + dynamic shared memory above 48 KB needs the opt-in, whatever
  // the dynamic part alone is
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

}  // namespace

size_t pass_smem_bytes(const DevLevel& L, int chunk, bool with_stage, bool pairs, bool flat) {
  const size_t cs = L.cell_size;
  if (pairs)
    return (2 * cs + (size_t)(kThreads / 32) * ((with_stage ? kStageFloats : 0) + mtile_floats(L, flat))) *
               sizeof(float) +
           (size_t)L.n_coarse * L.mask_size * sizeof(unsigned) + (size_t)L.max_npair * sizeof(int) +
           (with_stage ? (size_t)(kThreads / 32) * kSplitList : 0) +
           (with_stage && L.semiring == SEMI_REAL ? (size_t)(kThreads / 32) * kSplitList * sizeof(float) + 16 : 0);
  return (2 * cs + 2 * (size_t)chunk * cs) * sizeof(float);
}

// Splits staged per chunk by the target-major mode: as many as fit with two
// CTAs per SM.
int pick_split_chunk(int cell_size, int max_len) {
  const int static_bytes = (int)sizeof(CellCtx);
  const int budget = (112 * 1024 - static_bytes) / 4;
  int chunk = (budget - 2 * cell_size) / (2 * cell_size);
  chunk = chunk < 2 ? 2 : chunk;
  chunk = chunk > kMaxSplitChunk ? kMaxSplitChunk : chunk;
  if (max_len > 1 && chunk > max_len) chunk = max_len;
  return chunk;
}

cudaError_t launch_lexicon(const DevLevel& L, const DevBatch& B, const DevWork& W, const DevMask& M, float* inside,
                           double* part_scale, DevLive V, Counters C, cudaStream_t st) {
  const long long warps = W.nunits;
  const int blocks = (int)((warps * 32 + 127) / 128);
  if (blocks == 0) return cudaSuccess;
  switch (L.semiring) {
    case SEMI_VITERBI: k_lexicon<SEMI_VITERBI><<<blocks, 128, 0, st>>>(L, B, W, M, inside, part_scale, V, C.status); break;
    case SEMI_REAL: k_lexicon<SEMI_REAL><<<blocks, 128, 0, st>>>(L, B, W, M, inside, part_scale, V, C.status); break;
    default: k_lexicon<SEMI_LOGSUM><<<blocks, 128, 0, st>>>(L, B, W, M, inside, part_scale, V, C.status); break;
  }
  return cudaGetLastError();
}

namespace {

template <int S, int MODE>
cudaError_t launch_pass(bool inside_pass, const DevLevel& L, const DevBatch& B, const DevWork& W, const DevMask& M,
                        int max_span, const float* inside_c, float* inside, float* outside, DevLive V, Counters C,
                        cudaStream_t st) {
  const int chunk = pick_split_chunk(L.cell_size, max_span);
  const size_t smem =
      pass_smem_bytes(L, chunk, (inside_pass && S == SEMI_VITERBI) || MODE == 3, MODE >= 2, MODE == 3);
  const unsigned grid = (unsigned)W.nunits;
  if (inside_pass) {
    if (cudaError_t e = set_smem(k_inside_span<S, MODE>, smem); e != cudaSuccess) return e;
    k_inside_span<S, MODE><<<grid, kThreads, smem, st>>>(L, B, W, M, inside, V, C, chunk);
  } else {
    if (cudaError_t e = set_smem(k_outside_span<S, MODE>, smem); e != cudaSuccess) return e;
    k_outside_span<S, MODE><<<grid, kThreads, smem, st>>>(L, B, W, M, inside_c, outside, V, C, chunk);
  }
  return cudaGetLastError();
}

cudaError_t launch_any(bool inside_pass, const DevLevel& L, const DevBatch& B, const DevWork& W, const DevMask& M,
                       int max_span, const float* inside_c, float* inside, float* outside, DevLive V, Counters C,
                       cudaStream_t st) {
  if (W.nunits == 0) return cudaSuccess;
  const bool pairs = L.mode == 2;
  switch (L.semiring) {
    case SEMI_VITERBI:
      // the flat-tile passes (their pairs: of coarse symbols, or of groups
      // of coarse ids on a target-major level)
      if (inside_pass ? L.flat_inside : L.flat_outside)
        return launch_pass<SEMI_VITERBI, 3>(inside_pass, L, B, W, M, max_span, inside_c, inside, outside, V, C, st);
      return pairs ? launch_pass<SEMI_VITERBI, 2>(inside_pass, L, B, W, M, max_span, inside_c, inside, outside, V, C, st)
                   : launch_pass<SEMI_VITERBI, 0>(inside_pass, L, B, W, M, max_span, inside_c, inside, outside, V, C, st);
    case SEMI_REAL:
      if (inside_pass ? L.flat_inside : L.flat_outside)
        return launch_pass<SEMI_REAL, 3>(inside_pass, L, B, W, M, max_span, inside_c, inside, outside, V, C, st);
      return pairs ? launch_pass<SEMI_REAL, 2>(inside_pass, L, B, W, M, max_span, inside_c, inside, outside, V, C, st)
                   : launch_pass<SEMI_REAL, 0>(inside_pass, L, B, W, M, max_span, inside_c, inside, outside, V, C, st);
    default:
      return launch_pass<SEMI_LOGSUM, 0>(inside_pass, L, B, W, M, max_span, inside_c, inside, outside, V, C, st);
  }
}

}  // namespace

cudaError_t launch_inside_span(const DevLevel& L, const DevBatch& B, const DevWork& W, const DevMask& M,
                               int max_span, float* inside, DevLive V, Counters C, cudaStream_t st) {
  return launch_any(true, L, B, W, M, max_span, inside, inside, nullptr, V, C, st);
}

cudaError_t launch_outside_span(const DevLevel& L, const DevBatch& B, const DevWork& W, const DevMask& M,
                                int max_span, const float* inside, float* outside, DevLive V, Counters C,
                                cudaStream_t st) {
  return launch_any(false, L, B, W, M, max_span, inside, nullptr, outside, V, C, st);
}

}  // namespace puck
