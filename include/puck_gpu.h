/*
 * puck_gpu.h -- C ABI of the GB300 chart-parsing library (libpuck_gb300.so).
 *
 * This is the drop-in boundary for the hot path of dlwh/puck: the Scala host
 * binds these symbols (Panama FFM or JNI) in place of JavaCL + the generated
 * OpenCL kernels.  Each entry point names the reference interface it replaces
 * (paths relative to the dlwh/puck project).
 *
 * Conventions: plain pointers and sizes, no ownership transfer unless stated.
 * Sentences are passed as word ids (see puck_grammar_word_id) with CSR
 * offsets: sentence i is word_ids[offsets[i] .. offsets[i+1]).
 * Calls on one puck_parser are not thread-safe (the reference's public
 * methods are `synchronized`, CLParser.scala:50-63); distinct parsers may be
 * used from distinct threads.  No call aborts the process or traps the GPU;
 * failures come back as puck_status codes with a message from
 * puck_last_error.
 */
#ifndef PUCK_GPU_H
#define PUCK_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum puck_status {
  PUCK_OK = 0,
  PUCK_ERR_OOM = 1,            /* device or host allocation failed */
  PUCK_ERR_BAD_GRAMMAR = 2,    /* unreadable or inconsistent grammar.grz */
  PUCK_ERR_SENT_TOO_LONG = 3,  /* sentence longer than the parser's max length */
  PUCK_ERR_OOV = 4,            /* word id outside the grammar's vocabulary */
  PUCK_ERR_DEVICE_TIMEOUT = 5, /* a bounded device wait gave up */
  PUCK_ERR_INVALID_ARG = 6,
  PUCK_ERR_CUDA = 7,           /* a CUDA runtime call failed */
  PUCK_ERR_INTERNAL = 8,
  PUCK_ERR_EMPTY = 9           /* empty sentence */
} puck_status;

typedef enum puck_decode {
  PUCK_DECODE_AUTO = 0,    /* Viterbi tree for a Viterbi fine level, MBR otherwise (CLParser.scala:151-164) */
  PUCK_DECODE_VITERBI = 1,
  PUCK_DECODE_MBR = 2
} puck_decode;

typedef struct puck_grammar puck_grammar;
typedef struct puck_parser puck_parser;

/* Options of `new CLParser(data, maxAllocSize, profile)` (CLParser.scala:46-48)
 * plus the RunParser/CLParser flags that shape a parse (RunParser.scala:34-43). */
typedef struct puck_options {
  int64_t mem_bytes;          /* device bytes the parser may use (--mem); <= 0: 80% of free memory */
  int32_t device;             /* CUDA device ordinal */
  int32_t profile;            /* non-zero: per-pass CUDA-event timings in puck_parser_stats */
  int32_t decode;             /* puck_decode */
  int32_t max_length;         /* longest sentence accepted (0: 100) */
  int32_t max_batch_sentences;/* cap on sentences per batch (0: no cap beyond memory) */
  float prune_threshold;      /* coarse-pass log max-marginal threshold (reference: -9, CLParser.scala:226) */
  int32_t use_graphs;         /* non-zero: capture each batch's pass sequence in a CUDA graph */
  int32_t tensor_cores;       /* non-zero: in puck_parse / puck_partitions / puck_inside_outside the
                                 sum-product fine level's inside binary sums run on tcgen05 tensor
                                 cores in BF16 with FP32 accumulation (levels whose structure the
                                 form does not cover, and the server, keep the FP32 path) */
  int32_t server_lanes;       /* puck_server_create: independent request loops ("lanes"), each with
                                 its own streams and a share of the memory and slots (0: 2; fewer
                                 when a share could not hold a few sentences of max_length) */
} puck_options;

/* One node of a preorder tree (the reference's tree_t, CLViterbi.scala:378):
 * top = nonterminal of the unary layer or -1 (no unary layer), bot = the
 * child symbol (terminal index when width == 1, else nonterminal index),
 * width = span length, score = the backtrace score.  A sentence of length n
 * has 2n-1 nodes; the left child of node p is p+1 and the right child is
 * p + 2*width(left).  MBR trees use the same layout with coarse symbol ids. */
typedef struct puck_tree_node {
  int32_t top;
  int32_t bot;
  int32_t width;
  float score;
} puck_tree_node;

/* Counters of the last call.  ms_* are CUDA-event times on the parser's
 * stream summed over batches: ms_device from the first to the last kernel
 * of each batch (no host work, no host<->device copies), ms_inside ..
 * ms_decode per pass kind over all levels. */
typedef struct puck_stats {
  double ms_total, ms_inside, ms_outside, ms_masks, ms_decode, ms_h2d, ms_d2h;
  int64_t cells;              /* chart cells (bot + top halves) of the batches */
  int64_t cells_pruned;       /* of those, cells the last coarse level's mask closes entirely */
  int64_t batches, kernel_launches;
  int64_t binary_work;        /* (rule, split) applications executed in the last call */
  double ms_device;
  int64_t h2d_bytes, d2h_bytes;
} puck_stats;

void puck_default_options(puck_options* opts);

/* --- grammar (CLParserData.readSequence, CLParser.scala:1302-1305) ------ */
puck_grammar* puck_grammar_load(const char* grz_path, puck_status* status);
void puck_grammar_free(puck_grammar* g);
int32_t puck_grammar_num_levels(const puck_grammar* g);
/* Per-level sizes: out[0..7] = semiring(0 viterbi,1 real,2 logsum), n_nt,
 * n_t, cell_size, mask_size, n_coarse, root, n_words. */
puck_status puck_grammar_level_info(const puck_grammar* g, int32_t level, int32_t out[8]);
/* Word string -> id in the vocabulary of the fine level; -1 if unknown. */
int32_t puck_grammar_word_id(const puck_grammar* g, const char* word);
/* The word's id, else the id of its unknown-word class for a word at
 * `position` in its sentence (0 = first), backing off to ever shorter
 * classes and finally "UNK", else -1.  The classes are those of the
 * Berkeley parser's English lexicons, which list one entry per class
 * (`UNK-INITC-KNOWNLC`, `UNK-LC-s`, ...): capitalisation (INITC with
 * KNOWNLC, CAPS, LC), digits (NUM), hyphens (DASH) and an English suffix.
 * The reference takes unknown-word scores from epic's lexicon model, which
 * is not present here, so this mapping is not checked against it. */
int32_t puck_grammar_word_id_at(const puck_grammar* g, const char* word, int32_t position);

/* --- grammar compiler (CompileGrammar.main, CompileGrammar.scala:20-72) -- */
/* Options of CompileGrammar (CompileGrammar.scala:20-25). */
typedef struct puck_compile_options {
  int32_t viterbi;    /* --viterbi (default 1): the fine level's semiring is Viterbi */
  int32_t logsum;     /* --logsum: with viterbi = 0, LogSum instead of Real (CompileGrammar.scala:45-51) */
  int32_t reproject;  /* --reproject: keep the first and last levels, the last projected onto the
                         first's substates through its .hierarchy file (CLParser.scala:1153-1209) */
  float threshold;    /* rules and lexicon entries with a lower log score are dropped (-12, as
                         CompileGrammar.scala:56 passes to parseBerkeleyText) */
} puck_compile_options;
void puck_default_compile_options(puck_compile_options* opts);
/* Compiles the Berkeley text grammars named by text_prefixes ("a:b", coarse
 * level first; each prefix has .numstates, .binary, .unary, .lexicon) into
 * the grammar.grz at out_grz, as `CompileGrammar --textGrammarPrefix a:b
 * --grammar out.grz` does (CLParserData.make + writeSequence,
 * CLParser.scala:1264-1285,1307-1317).  Coarse levels are Viterbi.  The
 * compiler is the library's host-side Python package, run in an embedded
 * CPython interpreter (the caller's, or libpython3.12 loaded on first use).
 * opts may be NULL (defaults).  Returns PUCK_ERR_BAD_GRAMMAR with a message
 * when the text grammars cannot be read. */
puck_status puck_compile_grammar(const char* text_prefixes, const char* out_grz, const puck_compile_options* opts);

/* --- parser (new CLParser / release, CLParser.scala:46-89) -------------- */
puck_parser* puck_parser_create(const puck_grammar* g, const puck_options* opts, puck_status* status);
void puck_parser_destroy(puck_parser* p);

/* CLParser.parse (CLParser.scala:50-53): coarse passes build pruning masks,
 * the last level decodes.  nodes_out holds sum(2*len_i - 1) nodes; node
 * block of sentence i starts at sum_{j<i}(2*len_j - 1).  sent_status (nsent
 * entries, may be NULL) gets a per-sentence puck_status; a sentence that
 * fails leaves its nodes zeroed (the reference prints "(())" for it). */
puck_status puck_parse(puck_parser* p, const int32_t* word_ids, const int64_t* offsets, int32_t nsent,
                       puck_tree_node* nodes_out, int32_t* sent_status);

/* CLParser.partitions (CLParser.scala:55-58,189-206): log partition (Viterbi:
 * best score) of each sentence under the last level, with the cascade's masks. */
puck_status puck_partitions(puck_parser* p, const int32_t* word_ids, const int64_t* offsets, int32_t nsent,
                            float* log_z, int32_t* sent_status);

/* CLParser.insideOutside (CLParser.scala:60-63,171-182): full inside and
 * outside passes of every level (results stay on the device). */
puck_status puck_inside_outside(puck_parser* p, const int32_t* word_ids, const int64_t* offsets, int32_t nsent);

/* Copies of the last call's device state, for tests and tools.  Valid only
 * when the call ran as a single batch.  which: 0 inside, 1 outside chart
 * (num_cells * cell_size floats), 2 masks produced by `level` for the next
 * level (num_cells * mask_size int32), 3 inside scales, 4 outside scales
 * (num_cells floats), 5 per-cell MBR {score, symbol} pairs (num_cells * 2). */
puck_status puck_debug_copy(puck_parser* p, int32_t level, int32_t which, void* host_out, size_t bytes);
int64_t puck_debug_num_cells(const puck_parser* p);
/* Host-only check of a job's rule tables (no device needed): builds them as
 * a parser would and rebuilds every rule they hold, which must equal the
 * job's target-major rule table exactly (target, operands, weight bits).
 * form: 0 the flat-tile tables over coarse pairs, 1 the flat-tile tables over
 * groups of 16 coarse ids (inside jobs 0-3 only), 2 the pair-major tables.
 * out[0..3] = rules, then sub-tiles, blocks, records (form 0-1) or distinct
 * pairs (form 2).  Returns 0 when they match, -1 when the job does not take
 * the layout, -2 on a mismatch or a broken invariant (an entry outside its
 * tile, more than 32 targets in a block, a pair listed twice), -3 for bad
 * arguments. */
int32_t puck_debug_flat_check(const puck_grammar* g, int32_t level, int32_t job, int32_t form, int64_t out[4]);

puck_status puck_parser_stats(const puck_parser* p, puck_stats* out);

/* Per-level pass times of the last call (CUDA events, summed over batches):
 * out[0] inside, out[1] outside, out[2] masks + scaling, out[3] decode (ms);
 * launches[0..3] the matching kernel launch counts. */
puck_status puck_parser_pass_ms(const puck_parser* p, int32_t level, double out[4], int64_t launches[4]);
/* Autotuner (no reference counterpart: the reference fixes its kernel shapes
 * when it compiles the grammar).  Parses the sample once per candidate and
 * keeps, for the whole parser, how many waves of CTAs the cells of a span
 * launch that does not fill the GPU are split to fill (1, 2 or 4).  chosen
 * (levels + 1 entries, may be NULL) receives each level's gather form (0
 * target-major, 2 pair-factored; the archive's choice) and the waves x 100.
 * Per level with the flat-tile layout it also chooses the span band whose
 * inside launches run the flat-tile form (puck_parser_flat_from).
 * Results do not depend on the choice (Viterbi bit-identical; Real sums
 * reorder). */
puck_status puck_parser_autotune(puck_parser* p, const int32_t* word_ids, const int64_t* offsets, int32_t nsent,
                                 int32_t* chosen);

/* First span whose inside launch of `level` runs the flat-tile form: 16 x 16
 * outer-product tiles (the sub-tiles of a pair-factored level's coarse
 * pairs, or groups of 16 coarse ids of a target-major Viterbi level) with
 * four-rule records; shorter spans run the level's own form.  0: no span
 * (or no flat-tile layout), -1: bad level.  By default every span of a
 * pair-factored Viterbi level; puck_parser_autotune may choose another band.
 * Results do not depend on it (max-plus, bit-identical). */
int32_t puck_parser_flat_from(const puck_parser* p, int32_t level);
/* Pins that band: span >= 2 runs the flat-tile form from that span on, 0 at
 * no span.  PUCK_ERR_INVALID_ARG for a bad level, span 1, or span > 0 on a
 * level without the flat-tile layout. */
puck_status puck_parser_set_flat_from(puck_parser* p, int32_t level, int32_t span);

/* 1 if `level` runs its inside binary sums on tensor cores (options
 * tensor_cores and a level the form covers), 0 if not (why, may be NULL,
 * receives the reason), -1 for a bad level. */
int32_t puck_parser_tensor_cores(const puck_parser* p, int32_t level, char* why, size_t len);

/* Binary-rule work of one level in the last call: out[0] = work units (the
 * pair-factored form: live split x child-pair elements plus applied rules;
 * the target-major form: rule x split applications), out[1] = binary partials
 * >= +0.0 (Viterbi), which the reference's atomic_min would have dropped. */
puck_status puck_parser_level_work(const puck_parser* p, int32_t level, int64_t out[2]);

/* Max-constituent (MBR) tree decode into caller-owned device buffers with no
 * device allocation, for callers that cannot allocate at the point where they
 * decode: a host running inside a device arena its own pool carved out (the
 * pool already owns the device's memory), or a serving loop that must keep
 * the CUDA allocator off its request path (a cudaMalloc can synchronize the
 * device).  No counterpart in the reference (its MBR decode runs on the host,
 * CLParser.scala:589-696).
 * Same decode as puck_parse's MBR path: cell_decode (device, 8-byte aligned)
 * holds per cell {best coarse marginal, coarse symbol as int bits} -- the
 * layout puck_debug_copy(which = 5) returns; iscale/oscale (device, per cell)
 * are the coarse level's log-scales for a Real fine level, or both NULL;
 * lengths is a host array; nodes (device) receives
 * sum(2*len_i - 1) preorder nodes.  Work is enqueued on `stream` (a
 * cudaStream_t, NULL = default stream).  Scratch lives in a fixed array in
 * the library's device memory, held by every device that loads the library
 * until the process exits: at most 65,536 sentences and sum of
 * 3*(len_i+1)^2 <= 4,194,304 floats (16 MiB) per call; larger calls are
 * rejected with PUCK_ERR_INVALID_ARG.  The first call on a device resolves
 * the array's address (cudaGetSymbolAddress, with that device current) and
 * should come before any stream capture.  All calls share the array: calls
 * whose work overlaps on the GPU (other streams, other host threads) race on
 * it and must be serialized by the caller. */
puck_status puck_mbr_decode_static(const float* cell_decode, const float* iscale, const float* oscale,
                                   const int32_t* lengths, int32_t nsent, puck_tree_node* nodes, void* stream);

/* Tensor-core check (no reference counterpart).  On `device`, one CTA
 * computes d[128 x n] = a[128 x k] * b[n x k]^T with tcgen05.mma from shared
 * memory into a TMEM accumulator, the building block of the BF16 sum-product
 * rule application.  a and b are row-major BF16 bit patterns, d row-major
 * FP32, all host memory; k and n are multiples of 16 in [16, 256].  Returns
 * PUCK_ERR_DEVICE_TIMEOUT if the tensor-core wait gave up. */
puck_status puck_tc_selftest(int32_t device, int32_t k, int32_t n, const uint16_t* a, const uint16_t* b, float* d);

/* --- continuous-batching server ------------------------------------------
 * Replaces the reference's batching front for parse requests,
 * BatchFunctionAnnotatorService (src/main/scala/puck/AnnotatorService.scala:
 * 29-78, one future per sentence, batches flushed by time or size), with
 * continuous batching: a request loop admits sentences as chart memory and
 * slots free up, keeps every admitted sentence's charts and pruning masks
 * resident on the device, and advances all resident sentences together, one
 * pass step per sentence per tick, each kernel of a tick covering the cells
 * of every sentence at that step (sentences at different span lengths share
 * one launch).  With a cascade, the coarse levels of the sentences admitted
 * in one tick run as one batch on a side stream and the sentences join the
 * ticks at the last level; the trees are decoded on a second side stream.
 * Options as for puck_parser_create: mem_bytes sizes the chart
 * arena, max_batch_sentences caps the resident sentences (0: 65,536),
 * max_length, decode and prune_threshold as for a parse.  submit, poll, take
 * and stats may be called from any thread.  The server runs several lanes
 * (opts.server_lanes): independent request loops on their own streams over
 * one copy of the device grammar tables, each with a share of the memory and
 * slots; a request goes to the lane with the fewest cells in hand, so one
 * lane's slow cells overlap the other lanes' ticks.  Stats sum over the lanes
 * (resident_peak and arena_cells_peak: the sum of the lanes' peaks; ms_device:
 * of their ticks, which overlap).  A result does not depend on which other
 * sentences were resident or on its lane; a one-word sentence parses as in a
 * batch that also holds longer sentences. */
typedef struct puck_server puck_server;

typedef struct puck_server_stats {
  int64_t submitted, completed, failed;
  int64_t ticks, kernel_launches;
  int64_t resident, resident_peak;       /* sentences holding charts now / at most */
  int64_t arena_cells, arena_cells_peak; /* chart arena capacity / most cells in use */
  double ms_device;                      /* CUDA-event time of all ticks */
  int64_t h2d_bytes, d2h_bytes;
} puck_server_stats;

puck_server* puck_server_create(const puck_grammar* g, const puck_options* opts, puck_status* status);
/* Finishes every admitted request, then stops the request loop. */
void puck_server_destroy(puck_server* s);
/* Clock of arrival and latency times (monotonic, nanoseconds). */
int64_t puck_server_now_ns(void);
/* Queues sentences i = 0..nsent-1 (word_ids[offsets[i] .. offsets[i+1])).
 * arrival_ns[i] is the time each request's latency counts from (NULL or 0:
 * now).  ids[i] receives the request id.  A sentence that cannot be parsed
 * (empty, too long, unknown word) still gets an id; its result carries the
 * failure status. */
puck_status puck_server_submit(puck_server* s, const int32_t* word_ids, const int64_t* offsets, int32_t nsent,
                               const int64_t* arrival_ns, int64_t* ids);
/* Waits up to wait_ms for finished requests and writes up to max_ids of their
 * ids (each id once); returns how many. */
int32_t puck_server_poll(puck_server* s, int64_t* ids, int32_t max_ids, int32_t wait_ms);
/* Copies a finished request's 2n-1 tree nodes (as puck_parse) and releases
 * it; sent_status and latency_ns (completion minus arrival) may be NULL. */
puck_status puck_server_take(puck_server* s, int64_t id, puck_tree_node* nodes, int32_t max_nodes,
                             int32_t* sent_status, int64_t* latency_ns);
puck_status puck_server_get_stats(const puck_server* s, puck_server_stats* out);
/* With opts.profile: CUDA-event ms of each step kind of one level summed over
 * ticks, out[0..4] = lexicon, inside, outside, masks (+ scaling), decode.
 * With a cascade the coarse levels run as per-admission batches; their whole
 * time is reported as level 0's inside entry. */
puck_status puck_server_pass_ms(const puck_server* s, int32_t level, double out[5]);
/* Lanes the server runs (see puck_options.server_lanes). */
int32_t puck_server_lanes(const puck_server* s);

/* Last error message of the calling thread; returns the full length. */
size_t puck_last_error(char* buf, size_t len);

#ifdef __cplusplus
}
#endif

#endif /* PUCK_GPU_H */
