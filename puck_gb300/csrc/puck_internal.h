// Internal device-side structures of libpuck_gb300 (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <string>

namespace puck {

enum { SEMI_VITERBI = 0, SEMI_REAL = 1, SEMI_LOGSUM = 2 };

// Binary gather jobs.  Inside jobs have the rule parent as target; outside
// jobs use the reference's rotated rules (the updated child is the target).
enum JobId { IN_NN, IN_NT, IN_TN, IN_TT, OUT_L_NN, OUT_R_NN, OUT_L_NT, OUT_R_NT,
             OUT_L_TN, OUT_R_TN, OUT_L_TT, OUT_R_TT, NJOBS };
enum UJobId { IN_NU, IN_TU, OUT_NU, OUT_TU, NUJOBS };

constexpr int kMaxMask = 8;        // up to 256 coarse symbols
constexpr int kMaxCoarse = 256;
constexpr int kMaxSplitChunk = 32;  // splits staged in shared memory at once
constexpr int kMaxLen = 256;        // longest sentence a parser accepts
constexpr int kMaxSeg = 2048;       // rule segments of one job (coarse parents x sub-segments)

// A job's rules in CSR over target symbols.  rules[k] = {a | b << 16, bits(w)}
// with value = (A[a] + B[b]) + w (Viterbi) or A[a] * B[b] * w (Real).
struct DevJob {
  int n_tgt;
  int nseg;
  const int* rowptr;    // [n_tgt + 1]
  const int2* rules;    // [rowptr[n_tgt]]
  const int* tgt_seg;   // [n_tgt] segment of the target's rules, -1 if none
  const int* seg_bits;  // [nseg * mask_size] coarse-parent bitset of each segment
  // pair-factored layout (level mode 2): rules grouped by the coarse
  // projection (ca, cb) of their operands ("pairs"), then by segment
  // ("blocks"), then by target; rules {j | k << 8 | target << 16, bits(w)}
  // with j, k the operands' positions among their coarse symbol's members.
  int npair;
  int a_is_t, b_is_t;
  int interleaved;        // pair_rules lane-interleaved, tile-index form (Viterbi inside jobs, pair form):
                          // 1 mixed-target slices, 2 one target per lane slice (slice length a
                          // multiple of 4)
  const int* pair_key;    // [npair] ca | cb << 8
  const int* pair_gate;   // [npair * mask_size] OR of the pair's segment bits
  const int* pair_blk;    // [npair + 1] block range
  const int* blk_seg;     // [nblk]
  const int* blk_ptr;     // [nblk + 1] rule range, each a multiple of 32 (lane-interleaved, padded)
  const int* blk_nrule;   // [nblk] rules of the block before padding
  const int2* pair_rules;   // {(j * nz + k) | target << 16, bits(w)}
  // Flat-tile layout (flat != 0; Viterbi inside jobs whose pairs have
  // contiguous operand members; run by the MODE 3 kernels).  Pairs with more
  // than 16 members on a side are cut into sub-tiles of at most 16 x 16, each
  // a pair of this layout's own list (fnpair, fpair_key, fpair_gate); on a
  // level with pair_group 16 the keys are groups of 16 coarse ids.  A
  // sub-tile's outer product M[e], e = j * nz + k, is held one entry per lane
  // and slot (e = lane + 32 * slot).  A block's rules (at most 32 targets)
  // keep one target per lane slice; each lane's slice is stored as records of
  // four rules: their tile entries e (one byte each) and their weights
  // (padding: weight -inf).  The rules of a record position are ordered so
  // that the 32 lanes' entries fall in distinct shared-memory banks where the
  // slices allow.
  int flat;
  int fnpair;
  const int* fpair_key;   // [fnpair] pair key ca | cb << 8 of each sub-tile
  const int* fpair_gate;  // [fnpair * mask_size] OR of the sub-tile's segment bits
  const int4* pair_desc;  // [fnpair] {first A member | first B member << 16, first block,
                          //          ny | nz << 8 | blocks << 16, ca | cb << 8}
  const int4* fr_blk;     // [nblk] {segment, first record, end record, rules}; records of a
                          // block: 32 lanes x steps
  const int* fr_tgt;      // [nblk * 32] target of each lane's slice, -1 for none
  const unsigned* fr_idx; // [records] four tile entries, byte q = rule q
  const float4* fr_w;     // [records] four weights
  // Pair-major layout (target-major levels, Viterbi and sum-product): the
  // job's rules grouped by their distinct child pair (a, b), for the scan of
  // an ungated level that computes each pair's split maximum (or sum) once.
  int pm_npair;
  const int* pm_ab;       // [pm_npair] a | b << 16
  const int* pm_off;      // [pm_npair + 1] rule range of each pair
  const int2* pm_rule;    // {target, bits(w)}
};

struct DevUJob {
  int n_tgt;
  const int* rowptr;    // [n_tgt + 1]
  const int2* rules;    // {src, bits(w)}
};

struct DevLevel {
  int semiring, n_nt, n_t, cell_size, mask_size, n_coarse, root, num_syms, n_words;
  int gate_merged;  // non-final level of a cascade: every target gated by segment 0's bits
  int mode;         // 0: target-major rule scans, 2: pair-factored
  int max_npair;    // largest pair count of any job (shared-memory list size)
  int max_mtile;    // largest ny * nz of any pair (per-warp outer-product tile)
  int tc_binary;    // sum-product inside pass: binary sums already in the bot cells (tensor-core form)
  int flat_inside;  // every inside job with rules has the flat-tile layout (DevJob::flat); the
                    // host clears it in its copy of a level for launches of the other form
  int flat_outside; // the same for the outside jobs
  int flat_mtile;   // largest ny * nz of any flat-tile sub-tile (<= 256): the M tile of the
                    // flat-tile (MODE 3) kernels
  int pair_group;   // coarse ids per pair key of the flat-tile tables: 1 (pairs of coarse
                    // symbols) or 16 (a target-major level whose coarse ids each have at
                    // most one member per role: pairs of groups of 16 coarse ids, liveness
                    // tested on 16-bit halves of the liveness words)
  const int* nt_mem_off;  // [n_coarse + 1] coarse -> nonterminal members
  const int* nt_mem;
  const int* t_mem_off;   // [n_coarse + 1] coarse -> terminal members
  const int* t_mem;
  const int* nt_coarse;
  const int* t_coarse;
  DevJob jobs[NJOBS];
  DevUJob ujobs[NUJOBS];
  const long long* lex_off;
  const int* lex_term;
  const float* lex_score;
  const int* v_off;
  const int* v_left;
  const int* v_right;
  const float* v_score;
};

// Tensor-core form of a sum-product level's inside binary pass.  The binary
// sums of a tile of 128 cells accumulate in TMEM, one FP32 column per target:
// targets are grouped by coarse parent into slots of slot_w columns, and the
// slots are split into nparts parts of at most ncols columns (one CTA per
// tile and part).  For every rule block of a coarse pair the block's weights
// form a BF16 B operand (slot_w rows = the parent's members, kpad columns =
// the pair's outer-product tile padded to 16), stored in the tcgen05 K-major
// core-matrix layout; the pair's outer products over the cell's live splits
// form the A operand (128 cells x kpad).  Gating by the cell mask is applied
// per target when the accumulator is read out: every target keeps the same
// segment bits in every job and block, which the builder checks.
struct DevTc {
  int nparts, slot_w, ncols;  // ncols: TMEM columns allocated (a power of two, <= 512)
  int max_kpad, bcap;         // largest kpad; bytes of one B staging buffer
  const int* part_off;        // [nparts + 1] into tpair
  const int4* tpair;          // {job | pair << 2, kpad, blk0, blk1}: a pair's blocks in one part
  const int* tpair_gate;      // [ntpair * mask_size] OR of those blocks' segment bits
  const int* tblk;            // [nblk] TMEM slot of a block; its B operand follows the previous one's
  const long long* tpair_b;   // [ntpair] byte offset of the entry's first B operand in bmat
  const unsigned char* bmat;  // B operands, BF16
  const int* col_tgt;         // [nparts * ncols] target of a column, -1 for none
  const int* tgt_gate;        // [n_nt * mask_size] segment bits of each binary target
  const int* uncovered;       // row positions no column covers (written as zero)
  int n_uncovered;
  int* err;                   // set when a tensor-core wait gave up; later CTAs then skip their tiles
};

// Sentences of a batch (or of a server's resident set).  Each sentence's
// chart is laid out like the reference's Batch (src/main/scala/puck/parser/
// Batch.scala:23,50-58): a bot half then a top half of n(n+1)/2 cells each, in
// span-major chartIndex order, starting at cell_off[s].  In batch mode the
// sentences are packed back to back; a server places them anywhere in its
// resident chart arena.
struct DevBatch {
  int nsent;
  const int* len;             // [nsent]
  const long long* cell_off;  // [nsent] first cell of each sentence
  const long long* word_off;  // [nsent] first word id of each sentence
  const int* words;
  const long long* node_off;  // [nsent] first tree node of each sentence
};

// The units of one launch: entries are sentences; unit i belongs to the entry
// k with pref[k] <= i < pref[k+1].  Units are cells of one span length per
// entry (span passes), tokens (lexicon), cells (per-cell kernels) or whole
// sentences (decoders).  One launch can mix sentences at different spans.
// A span pass may give each cell of an entry `ways` CTAs: unit
// pref[k] + c * ways + g is part g of cell c.  The parts split the cell's rule
// work, leave partial rows in part_rows (one row per unit), and the last part
// to finish (counted in cell_cnt, indexed by chart cell, zero between
// launches) combines them and finishes the cell.
struct DevWork {
  int nent;
  long long nunits;         // pref[nent], kept on the host side for grid sizes
  const int* sent;          // [nent] sentence index
  const int* span;          // [nent] span length of the entry's cells; null: span_all for every entry
  int span_all;
  const int* pref;          // [nent + 1]; null for per-sentence launches (unit k is entry k)
  const int* ways;          // [nent] CTAs per cell; null: ways_all
  int ways_all;
  float* part_rows;         // [nunits * cell_size] when any entry has ways > 1
  int* cell_cnt;            // [cells of the chart]
  int one_word_batch;       // outside pass: the reference's batch-of-one-word-sentences unary quirk
};

// Pruning mask and log-scales produced by the previous level.
struct DevMask {
  const int* bits;      // [num_cells * mask_size] or null (no pruning)
  int mask_size;
  const float* iscale;  // [num_cells] or null
  const float* oscale;
};

struct DevNode { int top, bot, width; float score; };

// Launch wrappers (kernels.cu).  All return cudaGetLastError() of the launch.
struct Counters {
  unsigned long long* corner;   // binary partials >= +0.0 written (the reference drops them)
  unsigned long long* work;     // (rule, split) applications
  int* status;                  // per-sentence status codes
};

// Liveness bitsets of a chart: per cell, bit c set iff some symbol that
// projects onto coarse symbol c is not the semiring zero.
struct DevLive {
  int* in;    // [num_cells * mask_size] inside chart
  int* out;   // [num_cells * mask_size] outside chart (may be null)
};

// Launch wrappers.  Every wrapper takes the host-side unit count of its work
// list (W.nunits) as the grid size; part_scale and log_z are indexed by
// sentence.
cudaError_t launch_lexicon(const DevLevel& L, const DevBatch& B, const DevWork& W, const DevMask& M, float* inside,
                           double* part_scale, DevLive V, Counters C, cudaStream_t st);
cudaError_t launch_inside_span(const DevLevel& L, const DevBatch& B, const DevWork& W, const DevMask& M,
                               int max_span, float* inside, DevLive V, Counters C, cudaStream_t st);
cudaError_t launch_outside_span(const DevLevel& L, const DevBatch& B, const DevWork& W, const DevMask& M,
                                int max_span, const float* inside, float* outside, DevLive V, Counters C,
                                cudaStream_t st);
// pruned (may be null) counts the cells whose mask has no bit set
cudaError_t launch_masks(const DevLevel& L, const DevBatch& B, const DevWork& W, const float* inside,
                         const float* outside, float thresh, int* masks_out, cudaStream_t st,
                         unsigned long long* pruned = nullptr);
cudaError_t launch_scaling(int cell_size, const DevBatch& B, const DevWork& W, const float* chart, float* out,
                           cudaStream_t st);
cudaError_t launch_viterbi(const DevLevel& L, const DevBatch& B, const DevWork& W, int max_len, const float* inside,
                           DevNode* nodes, cudaStream_t st);
cudaError_t launch_mbr_cells(const DevLevel& L, const DevBatch& B, const DevWork& W, const float* inside,
                             const float* outside, float2* decode, cudaStream_t st);
cudaError_t launch_mbr_decode(const DevBatch& B, const DevWork& W, const DevMask& M, int scaling,
                              const float2* decode, const long long* mbr_off, float* scratch, DevNode* nodes,
                              cudaStream_t st);
cudaError_t launch_root_scores(const DevLevel& L, const DevBatch& B, const DevWork& W, const DevMask& M,
                               const float* inside, const double* part_scale, float* log_z, cudaStream_t st);

size_t pass_smem_bytes(const DevLevel& L, int chunk, bool with_stage, bool pairs, bool flat);

// Tensor-core inside pass: the binary sums of the cells of one span.  cells
// holds (sentence, begin) pairs; 128 cells per tile, one CTA per tile and
// TMEM part.  The cells are finished by launch_inside_span with
// L.tc_binary set.
constexpr int kTcRows = 128;
constexpr int kTcThreads = 1024;
size_t tc_smem_bytes(const DevTc& T);
size_t tc_static_smem_bytes();
cudaError_t launch_inside_tc(const DevLevel& L, const DevTc& T, const DevBatch& B, int span, const int* cells,
                             int ncells, const DevMask& M, float* inside, DevLive V, Counters C, cudaStream_t st);

// CTAs per cell of a span launch.  A cell's rule work grows with its split
// count (span - 1).  part_target(total, sms, waves) is the work one part
// should get: the launch's total split count spread over `waves` waves of
// CTAs (five per SM; two waves unless the parser was autotuned),
// and at least four splits; cell_ways gives a cell enough parts for that, at
// most 16.  A launch that already fills the GPU keeps one CTA per cell.
inline double part_target(double total_splits, int sms, double waves = 2.0) {
  const double t = total_splits / (waves * sms * 5);
  return t < 4.0 ? 4.0 : t;
}
inline int cell_ways(int span, double target) {
  if (span < 4) return 1;
  int g = (int)((span - 1 + target - 1e-9) / target);
  if (g > 16) g = 16;
  return g < 1 ? 1 : g;
}

// Message returned by puck_last_error on the calling thread.
void set_last_error(const char* msg);
inline void set_last_error(const std::string& msg) { set_last_error(msg.c_str()); }
int pick_split_chunk(int cell_size, int max_len);

}  // namespace puck
