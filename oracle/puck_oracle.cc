// CPU oracle for the chart-parsing hot path -- TEST INFRASTRUCTURE ONLY.
//
// A restatement of the reference's host loops and generated OpenCL kernels
// (paths relative to the dlwh/puck project), used by the test-suite as the
// parity checker and by bench.py as the timed CPU baseline.  Nothing in the
// product library links or calls this file.
//
// Parity status: UNPINNED.  The reference (Scala 2.10 + JavaCL + epic) cannot
// be built or run here and its tests hold no golden vectors for this path,
// so this restatement is checked only against hand-derived cases and an FP64
// self-consistency check, not against reference outputs.
//
// Restated pieces:
//   span loops          src/main/scala/puck/parser/CLParser.scala:256-369,489-522
//   work queues/gating  CLParser.scala:845-923 (block gating, child "any" tests, split ranges)
//   binary kernel       src/main/java/puck/parser/gen/SimpleGenRuleMultiply.java:103-229
//                       (per sub-segment partial per parent, semiring_mad, atomic write)
//   Viterbi atomic      SimpleGenRuleMultiply.java:340-365 (atomic_min on float bits:
//                       a partial >= +0.0 is dropped, which this file emulates)
//   unary kernel        SimpleGenRuleMultiply.java:255-319 + CLParser.scala:698-763
//   semirings           src/main/scala/puck/parser/RuleSemiring.scala:22-98
//   lexicon scoring     CLParser.scala:411-467
//   masks               src/main/scala/puck/parser/gen/CLMaskKernels.scala:172-236
//   scaling             src/main/scala/puck/parser/gen/CLScalingKernels.scala:51-69
//   root scores         src/main/scala/puck/parser/gen/CLParserUtils.scala:64-78
//   Viterbi backtrace   src/main/scala/puck/parser/gen/CLViterbi.scala:383-605 (WG_SIZE = 1)
//   MBR                 src/main/scala/puck/parser/gen/CLMBRKernels.scala:118-170 + CLParser.scala:587-696
//   partitions          CLParser.scala:189-206
//   chart indexing      src/main/scala/puck/parser/ParseChart.scala:58-65, Batch.scala:23,50-58
//
// The engine is templated on the float type: F = float is the bit-level
// restatement; F = double is the FP64 reference of the same computation.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum { VITERBI = 0, REAL = 1, LOGSUM = 2 };
enum JobId { IN_NN, IN_NT, IN_TN, IN_TT, OUT_L_NN, OUT_R_NN, OUT_L_NT, OUT_R_NT,
             OUT_L_TN, OUT_R_TN, OUT_L_TT, OUT_R_TT, NJOBS };
enum UJobId { IN_NU, IN_TU, OUT_NU, OUT_TU, NUJOBS };

struct Job {
  std::vector<int> tgt, ia, ib;
  std::vector<float> w;
  int nseg = 0;
  std::vector<int> seg_bits;                    // nseg * mask_size
  std::vector<int> sub_seg, sub_off, sub_rules;  // sub-segments in generator order
};

struct UJob {
  std::vector<int> tgt, src;
  std::vector<float> w;
};

struct Level {
  int semiring, n_nt, n_t, cell_size, mask_size, n_coarse, root;
  std::vector<int> nt_coarse, t_coarse;
  Job jobs[NJOBS];
  UJob ujobs[NUJOBS];
  std::vector<int64_t> lex_off;
  std::vector<int> lex_term;
  std::vector<float> lex_score;
  std::vector<int> v_off, v_left, v_right;
  std::vector<float> v_score;
  int num_syms() const { return std::max(n_nt, n_t); }
};

inline int chart_index(int begin, int end, int length) {
  int span = std::abs(end - begin) - 1;
  return std::min(begin, end) + span * length - span * (span - 1) / 2;
}
inline int64_t tri(int n) { return (int64_t)n * (n + 1) / 2; }

inline int32_t fbits(float f) { int32_t i; std::memcpy(&i, &f, 4); return i; }
inline float bitsf(int32_t i) { float f; std::memcpy(&f, &i, 4); return f; }

// fmax/fmin with OpenCL semantics for non-NaN inputs.
template <class F> inline F cl_max(F a, F b) { return a > b ? a : (b > a ? b : (std::signbit(a) ? b : a)); }
template <class F> inline F cl_min(F a, F b) { return a < b ? a : (b < a ? b : (std::signbit(a) ? a : b)); }

template <class F> struct Semi {
  int kind;
  F zero() const { return kind == VITERBI ? -std::numeric_limits<F>::infinity() : (kind == REAL ? F(0) : F(-1000000.0)); }
  F one() const { return kind == REAL ? F(1) : F(0); }
  F times(F a, F b) const { return kind == REAL ? a * b : a + b; }
  F add(F x, F y) const {
    if (kind == VITERBI) return cl_max(x, y);
    if (kind == REAL) return x + y;
    F lo = cl_min(x, y), hi = cl_max(x, y);
    return hi + std::log(F(1) + std::exp(lo - hi));
  }
  // semiring_mad(x, y, z)
  F mad(F x, F y, F z) const {
    if (kind == VITERBI) return cl_max(x, y + z);
    if (kind == REAL) return y * z + x;
    F yy = y + z;
    F lo = cl_min(x, yy), hi = cl_max(x, yy);
    return hi + std::log(F(1) + std::exp(lo - hi));
  }
};

struct Batch {
  int nsent = 0, max_len = 0;
  std::vector<int> len;
  std::vector<int64_t> cell_off;   // nsent + 1
  std::vector<int64_t> word_off;
  std::vector<int> words;
  int64_t num_cells() const { return cell_off.back(); }
  int64_t bot(int s, int b, int e) const { return cell_off[s] + chart_index(b, e, len[s]); }
  int64_t top(int s, int b, int e) const { return cell_off[s] + tri(len[s]) + chart_index(b, e, len[s]); }
  int64_t bot_off(int s) const { return cell_off[s]; }
  int64_t top_off(int s) const { return cell_off[s] + tri(len[s]); }
};

// Incoming pruning mask from the previous level (DenseMatrixMask,
// src/main/scala/puck/parser/PruningMask.scala:71-114).
struct MaskIn {
  const std::vector<int32_t>* bits = nullptr;  // num_cells * mask_size
  int mask_size = 0;
  const std::vector<float>* iscale = nullptr;  // per cell log-scales (Real semiring)
  const std::vector<float>* oscale = nullptr;
  bool has() const { return bits != nullptr; }
  const int32_t* cell(int64_t c) const { return bits->data() + c * mask_size; }
  bool any(int64_t c) const {
    if (!bits) return true;
    const int32_t* m = cell(c);
    for (int i = 0; i < mask_size; ++i) if (m[i]) return true;
    return false;
  }
};

enum Half { BOT, TOP };

template <class F> struct Engine {
  const Level& L;
  const Batch& B;
  const MaskIn& M;
  bool merged;  // non-final level of a multi-level cascade: one block gated by segment 0's bits
  Semi<F> S;
  int threads;
  std::vector<F> inside, outside;
  std::vector<F> iscale, oscale;     // scale buffers of this level's charts
  std::vector<double> partition_scales;
  int64_t corner_drops = 0;          // atomic_min writes of a value >= +0.0 that were dropped
  // (rule, split) applications the reference's queues run: rows queued for a
  // block times the block's rules, summed per pass (0 inside, 1 outside)
  int64_t rule_apps[2] = {0, 0};
  int apps_pass = 0;

  Engine(const Level& l, const Batch& b, const MaskIn& m, bool mg, int th)
      : L(l), B(b), M(m), merged(mg), S{l.semiring}, threads(th) {
    int64_t nc = B.num_cells();
    iscale.assign(nc, F(0));
    oscale.assign(nc, F(0));
    if (M.iscale && L.semiring == REAL) {
      for (int64_t c = 0; c < nc; ++c) { iscale[c] = (*M.iscale)[c]; oscale[c] = (*M.oscale)[c]; }
    }
    partition_scales.assign(B.nsent, 0.0);
  }

  F* cellp(std::vector<F>& chart, int64_t c) { return chart.data() + c * L.cell_size; }

  bool allowed_bot(int s, int b, int e) const { return M.any(B.bot(s, b, e)); }
  bool allowed_top(int s, int b, int e) const { return M.any(B.top(s, b, e)); }

  // Parent write of the generated binary kernel (SimpleGenRuleMultiply.java:158-165,324-365).
  void write_parent(F* loc, F value) {
    if (S.kind == VITERBI) {
      if constexpr (sizeof(F) == 4) {
        int32_t cur = fbits(*loc), v = fbits(value);
        if (v < cur) *loc = value;
        else if (value >= F(0) && cur != v) {
#pragma omp atomic
          corner_drops++;
        }
      } else {
        *loc = cl_max(*loc, value);
      }
    } else {
      *loc = S.add(*loc, value);
    }
  }

  struct Row { int64_t p, l, r; };

  // BinaryUpdateManager.doUpdates + flushQueue + CLBinaryRuleUpdater.update.
  template <class Ranger>
  void binary_update(int job, int span, bool parent_is_bot,
                     std::vector<F>& pchart, Half phalf,
                     std::vector<F>& lchart, Half lhalf, bool l_is_inside,
                     std::vector<F>& rchart, Half rhalf, bool r_is_inside,
                     const std::vector<F>& pscale, const std::vector<F>& lscale, const std::vector<F>& rscale,
                     Ranger ranger) {
    const Job& J = L.jobs[job];
    if (J.nseg == 0) return;
    bool l_top = l_is_inside && lhalf == TOP;
    bool r_top = r_is_inside && rhalf == TOP;
    // block queues: one per segment (segments with equal bits are grouped in
    // the reference; gating is per bits, so per-segment queues are equivalent)
    int nblocks = merged ? 1 : J.nseg;
    std::vector<std::vector<Row>> queues(nblocks);
    for (int s = 0; s < B.nsent; ++s) {
      int len = B.len[s];
      for (int start = 0; start + span <= len; ++start) {
        int end = start + span;
        int64_t mcell = parent_is_bot ? B.bot(s, start, end) : B.top(s, start, end);
        std::vector<int> blockids;
        if (!M.has()) {
          for (int k = 0; k < nblocks; ++k) blockids.push_back(k);
        } else {
          const int32_t* m = M.cell(mcell);
          for (int k = 0; k < nblocks; ++k) {
            const int* bits = &J.seg_bits[(size_t)k * L.mask_size];
            bool hit = false;
            for (int i = 0; i < L.mask_size; ++i) if (bits[i] & m[i]) { hit = true; break; }
            if (hit) blockids.push_back(k);
          }
        }
        if (blockids.empty()) continue;
        int64_t pcell = (phalf == BOT ? B.bot_off(s) : B.top_off(s)) + chart_index(start, end, len);
        int64_t loff = lhalf == BOT ? B.bot_off(s) : B.top_off(s);
        int64_t roff = rhalf == BOT ? B.bot_off(s) : B.top_off(s);
        int lo, hi;
        ranger(start, end, len, lo, hi);
        for (int split = lo; split <= hi; ++split) {
          if (split < 0 || split > len) continue;
          bool la, ra;
          if (split < start) la = l_top ? allowed_top(s, split, start) : allowed_bot(s, split, start);
          else la = l_top ? allowed_top(s, start, split) : allowed_bot(s, start, split);
          if (split < end) ra = r_top ? allowed_top(s, split, end) : allowed_bot(s, split, end);
          else ra = r_top ? allowed_top(s, end, split) : allowed_bot(s, end, split);
          if (!(la && ra)) continue;
          Row row{pcell, loff + chart_index(split, start, len), roff + chart_index(split, end, len)};
          for (int k : blockids) queues[k].push_back(row);
        }
      }
    }
    for (int k = 0; k < nblocks; ++k) {
      auto& q = queues[k];
      if (q.empty()) continue;
      // rows sharing a parent cell are contiguous; run groups in parallel
      std::vector<size_t> gstart;
      for (size_t i = 0; i < q.size(); ++i) if (i == 0 || q[i].p != q[i - 1].p) gstart.push_back(i);
      gstart.push_back(q.size());
      int seg_lo = merged ? 0 : k, seg_hi = merged ? J.nseg : k + 1;
      int64_t block_rules = 0;
      for (size_t sub = 0; sub < J.sub_seg.size(); ++sub)
        if (J.sub_seg[sub] >= seg_lo && J.sub_seg[sub] < seg_hi) block_rules += J.sub_off[sub + 1] - J.sub_off[sub];
      rule_apps[apps_pass] += (int64_t)q.size() * block_rules;
      const int64_t ngroups = (int64_t)gstart.size() - 1;
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads)
      for (int64_t g = 0; g < ngroups; ++g) {
        for (int seg = seg_lo; seg < seg_hi; ++seg) {
          for (size_t sub = 0; sub < J.sub_seg.size(); ++sub) {
            if (J.sub_seg[sub] != seg) continue;
            for (size_t ri = gstart[g]; ri < gstart[g + 1]; ++ri) {
              const Row& row = q[ri];
              F* parents = cellp(pchart, row.p);
              const F* left = cellp(lchart, row.l);
              const F* right = cellp(rchart, row.r);
              F scale = F(1);
              if (S.kind == REAL) scale = (F)std::exp(-pscale[row.p] + rscale[row.r] + lscale[row.l]);
              int cur = -1;
              F acc = S.zero();
              for (int x = J.sub_off[sub]; x < J.sub_off[sub + 1]; ++x) {
                int r = J.sub_rules[x];
                int t = J.tgt[r];
                if (t != cur) {
                  if (cur >= 0) {
                    if (S.kind == REAL) acc *= scale;
                    write_parent(parents + cur, acc);
                  }
                  cur = t;
                  acc = S.zero();
                }
                acc = S.mad(acc, S.times(left[J.ia[r]], right[J.ib[r]]), (F)J.w[r]);
              }
              if (cur >= 0) {
                if (S.kind == REAL) acc *= scale;
                write_parent(parents + cur, acc);
              }
            }
          }
        }
      }
    }
  }

  // UnaryUpdateManager.doUpdates + unary kernel: the parent cell is replaced by
  // a fresh row (semiring zero except rule parents).
  void unary_update(int ujob, int span, std::vector<F>& chart, Half phalf, Half chalf,
                    const std::vector<F>& scale) {
    const UJob& U = L.ujobs[ujob];
    std::vector<std::pair<int64_t, int64_t>> rows;
    for (int s = 0; s < B.nsent; ++s) {
      int len = B.len[s];
      for (int start = 0; start + span <= len; ++start) {
        if (!allowed_top(s, start, start + span)) continue;
        int64_t pc = (phalf == BOT ? B.bot_off(s) : B.top_off(s)) + chart_index(start, start + span, len);
        int64_t cc = (chalf == BOT ? B.bot_off(s) : B.top_off(s)) + chart_index(start, start + span, len);
        rows.push_back({pc, cc});
      }
    }
#pragma omp parallel for schedule(static) num_threads(threads)
    for (size_t i = 0; i < rows.size(); ++i) {
      std::vector<F> out(L.cell_size, S.zero());
      std::vector<F> acc(L.cell_size, S.zero());
      std::vector<char> declared(L.cell_size, 0);
      const F* child = cellp(chart, rows[i].second);
      F sc = F(1);
      if (S.kind == REAL) sc = (F)std::exp(-scale[rows[i].first] + scale[rows[i].second]);
      for (size_t r = 0; r < U.tgt.size(); ++r) {
        int t = U.tgt[r];
        declared[t] = 1;
        acc[t] = S.mad(acc[t], child[U.src[r]], (F)U.w[r]);
      }
      for (int t = 0; t < L.cell_size; ++t) {
        if (!declared[t]) continue;
        if (S.kind == REAL) out[t] += acc[t] * sc;
        else out[t] = acc[t];
      }
      std::memcpy(cellp(chart, rows[i].first), out.data(), sizeof(F) * L.cell_size);
    }
  }

  // computeTagScores + writeTagScores (CLParser.scala:411-467).
  void tag_scores() {
#pragma omp parallel for schedule(static) num_threads(threads)
    for (int s = 0; s < B.nsent; ++s) {
      double score_scale = 0.0;
      for (int pos = 0; pos < B.len[s]; ++pos) {
        int w = B.words[B.word_off[s] + pos];
        F* cell = cellp(inside, B.bot(s, pos, pos + 1));
        for (int k = 0; k < L.cell_size; ++k) cell[k] = S.zero();
        F my_scale = F(1);
        if (S.kind == REAL) my_scale = (F)std::exp(-(double)iscale[B.bot(s, pos, pos + 1)]);
        F total = S.zero();
        for (int64_t x = L.lex_off[w]; x < L.lex_off[w + 1]; ++x) {
          F v = (S.kind == REAL) ? (F)std::exp((double)L.lex_score[x]) : (F)L.lex_score[x];
          cell[L.lex_term[x]] = v * my_scale;
          total = total + cell[L.lex_term[x]];
        }
        if (S.kind == REAL) {
          score_scale += std::log((double)(total / F(2)));
          for (int64_t x = L.lex_off[w]; x < L.lex_off[w + 1]; ++x) cell[L.lex_term[x]] /= (total / F(2));
        }
      }
      partition_scales[s] = score_scale;
    }
  }

  void run_inside() {
    apps_pass = 0;
    int64_t nc = B.num_cells();
    inside.assign((size_t)nc * L.cell_size, S.zero());
    outside.assign((size_t)nc * L.cell_size, S.zero());
    tag_scores();
    unary_update(IN_TU, 1, inside, TOP, BOT, iscale);
    for (int span = 2; span <= B.max_len; ++span) {
      auto r_nt = [](int b, int e, int, int& lo, int& hi) { lo = e - 1; hi = e - 1; };
      auto r_tn = [](int b, int e, int, int& lo, int& hi) { lo = b + 1; hi = b + 1; };
      auto r_nn = [](int b, int e, int, int& lo, int& hi) { lo = b + 1; hi = e - 1; };
      if (span == 2)
        binary_update(IN_TT, span, true, inside, BOT, inside, BOT, true, inside, BOT, true, iscale, iscale, iscale, r_tn);
      binary_update(IN_NT, span, true, inside, BOT, inside, TOP, true, inside, BOT, true, iscale, iscale, iscale, r_nt);
      binary_update(IN_TN, span, true, inside, BOT, inside, BOT, true, inside, TOP, true, iscale, iscale, iscale, r_tn);
      binary_update(IN_NN, span, true, inside, BOT, inside, TOP, true, inside, TOP, true, iscale, iscale, iscale, r_nn);
      unary_update(IN_NU, span, inside, TOP, BOT, iscale);
    }
  }

  void run_outside() {
    apps_pass = 1;
    // setRootScores
    for (int s = 0; s < B.nsent; ++s) cellp(outside, B.top(s, 0, B.len[s]))[L.root] = S.one();
    unary_update(OUT_NU, B.max_len, outside, BOT, TOP, oscale);
    auto r_next = [](int b, int e, int, int& lo, int& hi) { lo = e + 1; hi = e + 1; };
    auto r_prev = [](int b, int e, int, int& lo, int& hi) { lo = b - 1; hi = b - 1; };
    auto r_after = [](int b, int e, int l, int& lo, int& hi) { lo = e + 1; hi = l; };
    auto r_before = [](int b, int e, int, int& lo, int& hi) { lo = 0; hi = b - 1; };
    for (int span = B.max_len - 1; span >= 1; --span) {
      // outsideBinaryPass (CLParser.scala:506-522)
      binary_update(OUT_R_TN, span, false, outside, TOP, inside, BOT, true, outside, BOT, false,
                    oscale, iscale, oscale, r_prev);
      binary_update(OUT_L_NT, span, false, outside, TOP, outside, BOT, false, inside, BOT, true,
                    oscale, oscale, iscale, r_next);
      binary_update(OUT_L_NN, span, false, outside, TOP, outside, BOT, false, inside, TOP, true,
                    oscale, oscale, iscale, r_after);
      binary_update(OUT_R_NN, span, false, outside, TOP, inside, TOP, true, outside, BOT, false,
                    oscale, iscale, oscale, r_before);
      if (span == 1) unary_update(OUT_TU, span, outside, BOT, TOP, oscale);
      else unary_update(OUT_NU, span, outside, BOT, TOP, oscale);
    }
    // terminal-child buckets after the span loop (CLParser.scala:345-355)
    binary_update(OUT_L_TT, 1, true, outside, BOT, outside, BOT, false, inside, BOT, true, oscale, oscale, iscale, r_next);
    binary_update(OUT_R_NT, 1, true, outside, BOT, inside, TOP, true, outside, BOT, false, oscale, iscale, oscale, r_before);
    binary_update(OUT_L_TN, 1, true, outside, BOT, outside, BOT, false, inside, TOP, true, oscale, oscale, iscale, r_after);
    binary_update(OUT_R_TT, 1, true, outside, BOT, inside, BOT, true, outside, BOT, false, oscale, iscale, oscale, r_prev);
  }

  // computeMasks kernel (Viterbi charts).
  void masks(float thresh, std::vector<int32_t>& out) {
    int64_t nc = B.num_cells();
    out.assign((size_t)nc * L.mask_size, 0);
    int ns = L.num_syms();
    for (int s = 0; s < B.nsent; ++s) {
      int64_t first = B.cell_off[s], last = B.cell_off[s + 1];
      F root_score = inside[(size_t)(last - 1) * L.cell_size + L.root];
      F cutoff = root_score + (F)thresh;
      for (int64_t c = first; c < last; ++c) {
        bool term = (c - first) < B.len[s];
        const F* in = inside.data() + c * L.cell_size;
        const F* ou = outside.data() + c * L.cell_size;
        int32_t* m = out.data() + c * L.mask_size;
        for (int sym = 0; sym < ns; ++sym) {
          F score = in[sym] + ou[sym];
          int keep = score >= cutoff;
          int field = term ? (sym < L.n_t ? L.t_coarse[sym] : 0) : (sym < L.n_nt ? L.nt_coarse[sym] : 0);
          m[field / 32] |= (int32_t)((uint32_t)keep << (field % 32));
        }
      }
    }
  }

  // getScalingConstants kernel.
  void scaling(const std::vector<F>& chart, std::vector<float>& out) {
    int64_t nc = B.num_cells();
    out.assign(nc, 0.f);
    for (int64_t c = 0; c < nc; ++c) {
      F m = F(-100000.0);
      for (int sym = 0; sym < L.cell_size; ++sym) m = cl_max(chart[(size_t)c * L.cell_size + sym], m);
      if (m < F(-9000.0)) m = F(0);
      out[c] = (float)m;
    }
  }

  // CLViterbi kernel with WG_SIZE = 1.
  void viterbi(std::vector<int32_t>& nodes, const std::vector<int64_t>& node_off) {
    const int* po = L.v_off.data();
    const int UNARY_OFFSET = 4 * L.n_nt, UNARY_OFFSET_T = 5 * L.n_nt;
    const int NN_OFF = 0, NT_OFF = L.n_nt, TN_OFF = 2 * L.n_nt, TT_OFF = 3 * L.n_nt;
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
    for (int s = 0; s < B.nsent; ++s) {
      int length = B.len[s];
      int32_t* tree = nodes.data() + node_off[s] * 4;
      const F* ibot = inside.data() + B.bot_off(s) * L.cell_size;
      const F* itop = inside.data() + B.top_off(s) * L.cell_size;
      auto CELL = [&](const F* base, int b, int e) { return base + (size_t)L.cell_size * chart_index(b, e, length); };
      tree[0] = L.root;
      tree[2] = length;
      int begin = 0;
      for (int p = 0; p < 2 * length - 1; ++p) {
        int32_t* node = tree + 4 * p;
        int width = node[2];
        int end = begin + width;
        int botSym = node[1];
        if (node[0] != -1) {
          int uoff = width == 1 ? UNARY_OFFSET_T : UNARY_OFFSET;
          const F* child = CELL(ibot, begin, end);
          F best = F(-30000.0f);
          int bestSym = 0;
          for (int r = po[uoff + node[0]]; r < po[uoff + node[0] + 1]; ++r) {
            int c = L.v_left[r];
            F sc = (F)L.v_score[r] + child[c];
            if (sc >= best) { best = sc; bestSym = c; }
          }
          node[3] = fbits((float)best);
          botSym = bestSym;
          node[1] = botSym;
        }
        if (width == 1) {
          node[3] = fbits((float)ibot[(size_t)L.cell_size * begin + botSym]);
          begin += 1;
        } else {
          int il = 10, ir = 10, isplit = begin + 1;
          F iscore = F(-300000.0f);
          auto best_binary = [&](const F* lc, const F* rc, int off, int split) {
            for (int r = po[off + botSym]; r < po[off + botSym + 1]; ++r) {
              int a = L.v_left[r], b = L.v_right[r];
              F sc = (F)L.v_score[r] + lc[a] + rc[b];
              if (sc >= iscore) { iscore = sc; il = a; ir = b; isplit = split; }
            }
          };
          best_binary(CELL(itop, begin, end - 1), CELL(ibot, end - 1, end), NT_OFF, -1);
          best_binary(CELL(ibot, begin, begin + 1), CELL(itop, begin + 1, end), TN_OFF, -2);
          if (width == 2) best_binary(CELL(ibot, begin, begin + 1), CELL(ibot, begin + 1, end), TT_OFF, -3);
          for (int split = begin + 1; split < end; ++split)
            best_binary(CELL(itop, begin, split), CELL(itop, split, end), NN_OFF, split);
          node[3] = fbits((float)iscore);
          int bestSplit = isplit;
          int cfg = bestSplit < 0 ? -bestSplit : 0;
          bestSplit = cfg == 0 ? bestSplit : (cfg == 2 ? begin + 1 : end - 1);
          int32_t* lnode = tree + 4 * (p + 1);
          int32_t* rnode = tree + 4 * (p + 2 * (bestSplit - begin));
          if ((cfg >> 1) == 0) lnode[0] = il; else { lnode[0] = -1; lnode[1] = il; }
          if ((cfg & 1) == 0) rnode[0] = ir; else { rnode[0] = -1; rnode[1] = ir; }
          lnode[2] = bestSplit - begin;
          rnode[2] = end - bestSplit;
        }
      }
    }
  }

  // computeMBR kernel: per cell best coarse marginal {score, symbol}.
  void mbr_cells(std::vector<float>& score, std::vector<int>& sym) {
    int64_t nc = B.num_cells();
    score.assign(nc, 0.f);
    sym.assign(nc, -1);
    int ns = L.num_syms();
    for (int s = 0; s < B.nsent; ++s) {
      int64_t first = B.cell_off[s], last = B.cell_off[s + 1];
      F root_score = inside[(size_t)(last - 1) * L.cell_size + L.root];
      std::vector<F> margs(L.n_coarse);
      for (int64_t c = first; c < last; ++c) {
        bool term = (c - first) < B.len[s];
        const F* in = inside.data() + c * L.cell_size;
        const F* ou = outside.data() + c * L.cell_size;
        std::fill(margs.begin(), margs.end(), F(0));
        for (int k = 0; k < ns; ++k) {
          int proj = term ? (k < L.n_t ? L.t_coarse[k] : 0) : (k < L.n_nt ? L.nt_coarse[k] : 0);
          if (S.kind == LOGSUM) margs[proj] += std::exp(in[k] - root_score + ou[k]);
          else margs[proj] += in[k] / root_score * ou[k];
        }
        F best = -std::numeric_limits<F>::infinity();
        int bs = -1;
        for (int cs = 0; cs < L.n_coarse; ++cs)
          if (margs[cs] > best) { best = margs[cs]; bs = cs; }
        score[c] = (float)best;
        sym[c] = bs;
      }
    }
  }
};

// extractMBRParses (CLParser.scala:589-696): host CKY over per-cell best
// coarse marginals.  Output nodes {top coarse or -1, bot coarse, width, score bits}.
void mbr_extract(const Batch& B, int s, const std::vector<float>& score, const std::vector<int>& sym,
                 const MaskIn& M, bool scaling, int32_t* out) {
  int n = B.len[s];
  auto idx = [n](int b, int e) { return (size_t)b * (n + 1) + e; };
  std::vector<float> best((n + 1) * (n + 1), 0.f);
  std::vector<int> bsplit((n + 1) * (n + 1), 0);
  std::vector<char> use_unary((n + 1) * (n + 1), 0);
  auto itop = [&](int b, int e) { return (*M.iscale)[B.top(s, b, e)]; };
  auto otop = [&](int b, int e) { return (*M.oscale)[B.top(s, b, e)]; };
  auto ibot = [&](int b, int e) { return (*M.iscale)[B.bot(s, b, e)]; };
  auto obot = [&](int b, int e) { return (*M.oscale)[B.bot(s, b, e)]; };
  for (int span = 1; span <= n; ++span) {
    for (int begin = 0; begin + span <= n; ++begin) {
      int end = begin + span;
      float topScaled = score[B.top(s, begin, end)];
      float botScaled = score[B.bot(s, begin, end)];
      if (scaling) {
        // FP32 sum of the scales, math.exp in FP64, rounded to FP32 (CLParser.scala:613-614)
        const float at = (itop(begin, end) + otop(begin, end)) - itop(0, n);
        const float ab = (ibot(begin, end) + obot(begin, end)) - itop(0, n);
        topScaled *= (float)std::exp((double)at);
        botScaled *= (float)std::exp((double)ab);
      }
      if (std::isnan(topScaled)) topScaled = 0.f;
      if (std::isnan(botScaled)) botScaled = 0.f;
      topScaled = std::min(topScaled, 1.0f);
      botScaled = std::min(botScaled, 1.0f);
      bool uu = (begin + 1 < end) || topScaled > 0.4;
      use_unary[idx(begin, end)] = uu;
      best[idx(begin, end)] = uu ? (topScaled + botScaled) : botScaled;
      if (span > 1) {
        float bestSplitScore = 0.0f;
        int bs = begin + 1;
        for (int split = begin + 1; split < end; ++split) {
          float sc = best[idx(begin, split)] + best[idx(split, end)];
          if (sc > bestSplitScore) { bs = split; bestSplitScore = sc; }
        }
        bsplit[idx(begin, end)] = bs;
        best[idx(begin, end)] += bestSplitScore;
      }
    }
  }
  int p = 0;
  // preorder emission
  struct Frame { int b, e; };
  std::vector<Frame> stack{{0, n}};
  while (!stack.empty()) {
    Frame f = stack.back();
    stack.pop_back();
    int32_t* node = out + 4 * p++;
    node[0] = use_unary[idx(f.b, f.e)] ? sym[B.top(s, f.b, f.e)] : -1;
    node[1] = sym[B.bot(s, f.b, f.e)];
    node[2] = f.e - f.b;
    node[3] = fbits(best[idx(f.b, f.e)]);
    if (f.e - f.b > 1) {
      int sp = bsplit[idx(f.b, f.e)];
      stack.push_back({sp, f.e});
      stack.push_back({f.b, sp});
    }
  }
}

struct LevelResult {
  std::vector<float> inside, outside;        // always stored as float for access
  std::vector<double> inside64, outside64;
  std::vector<int32_t> masks;                 // masks this level produced for the next
  std::vector<float> iscale, oscale;          // scales this level produced for the next
  std::vector<double> partition_scales;
  int64_t corner_drops = 0;
  int64_t rule_apps[2] = {0, 0};
  bool has_outside = false;
};

struct Run {
  std::vector<Level*> levels;
  Batch batch;
  int threads = 1;
  int precision = 32;
  std::vector<LevelResult> res;
  std::vector<int32_t> nodes;
  std::vector<int64_t> node_off;
  std::vector<int> status;
  std::vector<float> partitions;
  std::vector<float> mbr_score;
  std::vector<int> mbr_sym;
  // externally provided masks for the final level (FP64 runs reuse FP32 masks)
  std::vector<int32_t> ext_masks;
  std::vector<float> ext_iscale, ext_oscale;
  bool use_ext = false;
};

template <class F>
void store(LevelResult& r, Engine<F>& E, bool outside) {
  if constexpr (sizeof(F) == 4) {
    r.inside = E.inside;
    if (outside) r.outside = E.outside;
  } else {
    r.inside64 = E.inside;
    if (outside) r.outside64 = E.outside;
    r.inside.assign(E.inside.begin(), E.inside.end());
    if (outside) r.outside.assign(E.outside.begin(), E.outside.end());
  }
  r.partition_scales = E.partition_scales;
  r.corner_drops = E.corner_drops;
  r.rule_apps[0] = E.rule_apps[0];
  r.rule_apps[1] = E.rule_apps[1];
  r.has_outside = outside;
}

// mode: 0 = parse, 1 = partitions, 2 = insideOutside
template <class F>
int run_all(Run& R, int mode) {
  int nl = (int)R.levels.size();
  R.res.assign(nl, LevelResult());
  MaskIn mask;
  for (int li = 0; li < nl; ++li) {
    const Level& L = *R.levels[li];
    bool last = li == nl - 1;
    bool merged = !last && nl != 1;
    if (last && R.use_ext) {
      mask.bits = &R.ext_masks;
      mask.mask_size = L.mask_size;
      mask.iscale = &R.ext_iscale;
      mask.oscale = &R.ext_oscale;
    }
    Engine<F> E(L, R.batch, mask, merged, R.threads);
    if (!last) {
      if (R.use_ext && li == nl - 2) { continue; }
      // updateMasks -> computePruningMasks: inside, outside, masks(-9)
      E.run_inside();
      E.run_outside();
      LevelResult& lr = R.res[li];
      E.masks(-9.0f, lr.masks);
      bool next_scales = R.levels[li + 1]->semiring == REAL;
      if (next_scales) {
        E.scaling(E.inside, lr.iscale);
        E.scaling(E.outside, lr.oscale);
      } else {
        lr.iscale.assign(R.batch.num_cells(), 0.f);
        lr.oscale.assign(R.batch.num_cells(), 0.f);
      }
      store(lr, E, true);
      mask.bits = &lr.masks;
      mask.mask_size = L.mask_size;
      mask.iscale = &lr.iscale;
      mask.oscale = &lr.oscale;
      continue;
    }
    E.run_inside();
    LevelResult& lr = R.res[li];
    if (mode == 1) {
      R.partitions.assign(R.batch.nsent, 0.f);
      for (int s = 0; s < R.batch.nsent; ++s) {
        F v = E.inside[(size_t)R.batch.top(s, 0, R.batch.len[s]) * L.cell_size + L.root];
        if (L.semiring == REAL) {
          float sc = mask.iscale ? (*mask.iscale)[R.batch.top(s, 0, R.batch.len[s])] : 0.f;
          R.partitions[s] = ((float)std::log((double)v) + sc) + (float)E.partition_scales[s];
        } else {
          R.partitions[s] = (float)v;
        }
      }
      store(lr, E, false);
      return 0;
    }
    bool vit = L.semiring == VITERBI;
    if (!vit || mode == 2) E.run_outside();
    store(lr, E, !vit || mode == 2);
    R.node_off.assign(R.batch.nsent + 1, 0);
    for (int s = 0; s < R.batch.nsent; ++s) R.node_off[s + 1] = R.node_off[s] + 2 * R.batch.len[s] - 1;
    R.nodes.assign((size_t)R.node_off.back() * 4, 0);
    R.status.assign(R.batch.nsent, 0);
    if (vit) {
      E.viterbi(R.nodes, R.node_off);
    } else {
      E.mbr_cells(R.mbr_score, R.mbr_sym);
      if (mode == 0) {
        if (!mask.has()) return 2;  // "Can't use null pruning mask for parse extraction!"
        for (int s = 0; s < R.batch.nsent; ++s)
          mbr_extract(R.batch, s, R.mbr_score, R.mbr_sym, mask, L.semiring == REAL,
                      R.nodes.data() + R.node_off[s] * 4);
      }
    }
  }
  return 0;
}

}  // namespace

extern "C" {

void* po_level_new(int semiring, int n_nt, int n_t, int cell_size, int mask_size, int n_coarse, int root,
                   const int* nt_coarse, const int* t_coarse) {
  Level* L = new Level();
  L->semiring = semiring; L->n_nt = n_nt; L->n_t = n_t; L->cell_size = cell_size;
  L->mask_size = mask_size; L->n_coarse = n_coarse; L->root = root;
  L->nt_coarse.assign(nt_coarse, nt_coarse + n_nt);
  L->t_coarse.assign(t_coarse, t_coarse + n_t);
  return L;
}

void po_level_set_job(void* lv, int job, int n, const int* tgt, const int* ia, const int* ib, const float* w,
                      int nseg, const int* seg_bits, int nsub, const int* sub_seg, const int* sub_off,
                      const int* sub_rules) {
  Level* L = (Level*)lv;
  Job& J = L->jobs[job];
  J.tgt.assign(tgt, tgt + n); J.ia.assign(ia, ia + n); J.ib.assign(ib, ib + n); J.w.assign(w, w + n);
  J.nseg = nseg;
  J.seg_bits.assign(seg_bits, seg_bits + (size_t)nseg * L->mask_size);
  J.sub_seg.assign(sub_seg, sub_seg + nsub);
  J.sub_off.assign(sub_off, sub_off + nsub + 1);
  J.sub_rules.assign(sub_rules, sub_rules + (nsub ? sub_off[nsub] : 0));
}

void po_level_set_ujob(void* lv, int ujob, int n, const int* tgt, const int* src, const float* w) {
  Level* L = (Level*)lv;
  UJob& U = L->ujobs[ujob];
  U.tgt.assign(tgt, tgt + n); U.src.assign(src, src + n); U.w.assign(w, w + n);
}

void po_level_set_lexicon(void* lv, int nwords, const int64_t* off, const int* term, const float* score) {
  Level* L = (Level*)lv;
  L->lex_off.assign(off, off + nwords + 1);
  L->lex_term.assign(term, term + off[nwords]);
  L->lex_score.assign(score, score + off[nwords]);
}

void po_level_set_viterbi(void* lv, int n_off, const int* off, int n, const int* left, const int* right,
                          const float* score) {
  Level* L = (Level*)lv;
  L->v_off.assign(off, off + n_off);
  L->v_left.assign(left, left + n); L->v_right.assign(right, right + n); L->v_score.assign(score, score + n);
}

void po_level_free(void* lv) { delete (Level*)lv; }

void* po_run_new(int nlevels, void** levels, int nsent, const int64_t* word_off, const int* words,
                 int threads, int precision) {
  Run* R = new Run();
  for (int i = 0; i < nlevels; ++i) R->levels.push_back((Level*)levels[i]);
  Batch& B = R->batch;
  B.nsent = nsent;
  B.word_off.assign(word_off, word_off + nsent + 1);
  B.words.assign(words, words + word_off[nsent]);
  B.len.resize(nsent);
  B.cell_off.assign(nsent + 1, 0);
  for (int s = 0; s < nsent; ++s) {
    B.len[s] = (int)(word_off[s + 1] - word_off[s]);
    B.max_len = std::max(B.max_len, B.len[s]);
    B.cell_off[s + 1] = B.cell_off[s] + 2 * tri(B.len[s]);
  }
  R->threads = threads > 0 ? threads : 1;
  R->precision = precision;
  return R;
}

void po_run_set_final_masks(void* rv, const int32_t* masks, const float* iscale, const float* oscale) {
  Run* R = (Run*)rv;
  int64_t nc = R->batch.num_cells();
  int ms = R->levels.back()->mask_size;
  R->ext_masks.assign(masks, masks + nc * ms);
  R->ext_iscale.assign(iscale, iscale + nc);
  R->ext_oscale.assign(oscale, oscale + nc);
  R->use_ext = true;
}

int po_run(void* rv, int mode) {
  Run* R = (Run*)rv;
  return R->precision == 64 ? run_all<double>(*R, mode) : run_all<float>(*R, mode);
}

int64_t po_run_num_cells(void* rv) { return ((Run*)rv)->batch.num_cells(); }
int64_t po_run_num_nodes(void* rv) { return ((Run*)rv)->node_off.empty() ? 0 : ((Run*)rv)->node_off.back(); }

int po_run_get_chart(void* rv, int level, int which, float* out) {
  Run* R = (Run*)rv;
  LevelResult& r = R->res[level];
  const std::vector<float>& v = which == 0 ? r.inside : r.outside;
  if (v.empty()) return 1;
  std::memcpy(out, v.data(), v.size() * sizeof(float));
  return 0;
}

int po_run_get_chart64(void* rv, int level, int which, double* out) {
  Run* R = (Run*)rv;
  LevelResult& r = R->res[level];
  const std::vector<double>& v = which == 0 ? r.inside64 : r.outside64;
  if (v.empty()) return 1;
  std::memcpy(out, v.data(), v.size() * sizeof(double));
  return 0;
}

int po_run_get_masks(void* rv, int level, int32_t* out, float* iscale, float* oscale) {
  Run* R = (Run*)rv;
  LevelResult& r = R->res[level];
  if (r.masks.empty()) return 1;
  std::memcpy(out, r.masks.data(), r.masks.size() * 4);
  std::memcpy(iscale, r.iscale.data(), r.iscale.size() * 4);
  std::memcpy(oscale, r.oscale.data(), r.oscale.size() * 4);
  return 0;
}

void po_run_get_partition_scales(void* rv, int level, double* out) {
  Run* R = (Run*)rv;
  auto& v = R->res[level].partition_scales;
  std::memcpy(out, v.data(), v.size() * sizeof(double));
}

int64_t po_run_corner_drops(void* rv, int level) { return ((Run*)rv)->res[level].corner_drops; }

// pass 0 = inside, 1 = outside
int64_t po_run_rule_apps(void* rv, int level, int pass) { return ((Run*)rv)->res[level].rule_apps[pass & 1]; }

void po_run_get_trees(void* rv, int32_t* nodes) {
  Run* R = (Run*)rv;
  std::memcpy(nodes, R->nodes.data(), R->nodes.size() * 4);
}

void po_run_get_partitions(void* rv, float* out) {
  Run* R = (Run*)rv;
  std::memcpy(out, R->partitions.data(), R->partitions.size() * 4);
}

void po_run_get_mbr(void* rv, float* score, int32_t* sym) {
  Run* R = (Run*)rv;
  std::memcpy(score, R->mbr_score.data(), R->mbr_score.size() * 4);
  std::memcpy(sym, R->mbr_sym.data(), R->mbr_sym.size() * 4);
}

void po_run_free(void* rv) { delete (Run*)rv; }

}  // extern "C"
