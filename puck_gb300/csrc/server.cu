// Continuous-batching parse server (puck_server_* in puck_gpu.h).
//
// The reference batches parse requests in front of the parser:
// BatchFunctionAnnotatorService (dlwh/puck, src/main/scala/puck/
// AnnotatorService.scala:29-78) collects sentences until a time or size limit,
// hands the batch to CLParser.parse and completes one future per sentence.
// Here the request loop never waits for a batch to fill or drain:
//
//  * admission: a queued sentence is admitted as soon as a slot and a
//    contiguous range of 2*n(n+1)/2 cells of the chart arena are free (first
//    fit, FIFO order).  The arena holds every level's charts, liveness bits,
//    pruning masks and scales for the admitted sentences; they stay resident
//    until the sentence's tree is decoded.
//  * coarse groups: with a cascade, the sentences admitted in one tick run
//    their coarse levels as one batch on a coarse stream (every span back
//    to back), overlapping the ticks; they join the ticks at the last level
//    once that batch is done.
//  * ticks: every tick advances each resident sentence through its next pass
//    steps (lexicon, inside span k, outside span k, masks, decode).  One
//    kernel launch per step kind and level covers every sentence at that step,
//    whatever its span length, through the work lists the pass kernels take.
//    Launches of a tick run in the order lexicon, inside, outside, masks per
//    level, then decode, so a sentence can take several consecutive steps in
//    one tick (outside span 1, masks, next level's lexicon and inside span 1).
//  * pipelining: the host prepares tick t+1 while the GPU runs tick t; the
//    staging buffers and the tree output buffers are double-buffered.  A
//    finished sentence's cells and slot are reused by sentences admitted in
//    later ticks, which the single stream orders after its last kernel.
//  * results: decoded trees are written by the decode kernels straight into
//    mapped pinned host memory; the host hands them out once the tick's event
//    has completed.
//
// Every kernel computes a cell from that sentence's own cells only, so a
// result does not depend on which other sentences were resident with it.

#include "host_runtime.h"

#include <array>
#include <chrono>
#include <climits>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <numeric>
#include <thread>

using namespace puck_host;

namespace {

constexpr int kMaxLevels = 8;
constexpr int kDefaultSlots = 65536;

long long tri(long long n) { return n * (n + 1) / 2; }

int64_t now_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

// Per-slot metadata written at the start of a tick.
struct SlotUpdate {
  long long cell_off, node_off, mbr_off;
  int slot, len, words_at, fresh;
};

struct SlotTables {
  int* len;
  long long* cell_off;
  long long* node_off;
  long long* mbr_off;
  int* words;
  int* status;
  double* part[kMaxLevels];
  int nlevels;
};

__global__ void k_slot_update(SlotTables T, const SlotUpdate* U, const int* staged_words) {
  const SlotUpdate u = U[blockIdx.x];
  if (threadIdx.x == 0) {
    T.len[u.slot] = u.len;
    T.cell_off[u.slot] = u.cell_off;
    T.node_off[u.slot] = u.node_off;
    T.mbr_off[u.slot] = u.mbr_off;
    if (u.fresh) {
      T.status[u.slot] = 0;
      for (int l = 0; l < T.nlevels; ++l)
        if (T.part[l]) T.part[l][u.slot] = 0.0;
    }
  }
  if (u.words_at >= 0)  // words live at the sentence's first cell index
    for (int i = threadIdx.x; i < u.len; i += blockDim.x) T.words[u.cell_off + i] = staged_words[u.words_at + i];
}

// First-fit allocator of contiguous cell ranges.
class CellArena {
 public:
  void init(long long cap) {
    free_.clear();
    free_[0] = cap;
    cap_ = cap;
    used_ = peak_ = 0;
  }
  long long alloc(long long n) {
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < n) continue;
      const long long off = it->first, rest = it->second - n;
      free_.erase(it);
      if (rest) free_[off + n] = rest;
      used_ += n;
      peak_ = std::max(peak_, used_);
      return off;
    }
    return -1;
  }
  void release(long long off, long long n) {
    used_ -= n;
    auto next = free_.lower_bound(off);
    if (next != free_.end() && next->first == off + n) {
      n += next->second;
      next = free_.erase(next);
    }
    if (next != free_.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == off) {
        prev->second += n;
        return;
      }
    }
    free_[off] = n;
  }
  long long cap() const { return cap_; }
  long long peak() const { return peak_; }

 private:
  std::map<long long, long long> free_;
  long long cap_ = 0, used_ = 0, peak_ = 0;
};

struct Request {
  int n = 0;
  int status = PUCK_OK;
  int64_t t_arrival = 0, t_done = 0;
  std::vector<int> words;
  std::vector<puck_tree_node> nodes;
};

enum Stage { ST_LEX = 0, ST_IN = 1, ST_OUT = 2, ST_MASK = 3, ST_DEC = 4, ST_WAIT = 5 };

// Coarse groups in flight per lane.  Admission waits while both are busy, so
// under load the next group gathers more sentences and its coarse batch
// runs larger launches (two in flight against eight: at 6,000 sentences/s
// offered p50 latency 85 against 165 ms, and 5% more sentences/s at
// saturation on the C1 grammar).
constexpr int kGroups = 2;

// A resident sentence and its pass cursor (owned by the loop thread).
struct Resident {
  int64_t id;
  int slot, n;
  long long cell_off;
  int level, stage, span;
  int upd;  // index of this tick's admission record, -1 after the admitting tick
  int grp;  // coarse group while stage == ST_WAIT
};

// The coarse levels of the sentences admitted in one tick run as one batch
// on the coarse stream: lexicon, every inside span, every outside span and
// the masks, back to back.  They then join the ticks at the last level.
struct CoarseGroup {
  bool busy = false;
  int waiting = 0;                 // residents still in ST_WAIT
  cudaEvent_t begin = nullptr, done = nullptr;
  char* host = nullptr;
  size_t host_cap = 0;
  DevBuf dev, parts;
};

struct Finishing {
  int64_t id;
  long long node_at;
  int n;
  int slot;
  long long cell_off;
};

// Host and device buffers of one tick in flight.
struct TickBuf {
  char* host = nullptr;  // pinned staging
  size_t host_cap = 0;
  DevBuf dev;
  puck_tree_node* out_host = nullptr;  // mapped pinned tree output
  puck::DevNode* out_dev = nullptr;
  size_t out_cap = 0;  // nodes
  cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
  // the decode runs on its own stream once the last level's passes of the
  // tick are done, overlapping the next ticks
  cudaEvent_t ev_fine = nullptr, ev_dec_begin = nullptr, ev_dec_end = nullptr;
  bool decoded = false;
  std::vector<cudaEvent_t> ev_group;  // profile: after the slot update, then after each step group
  std::vector<Finishing> finishing;
  int64_t launches = 0, h2d = 0, d2h = 0;
};

struct LevelArena {
  DevBuf inside, outside, live_in, live_out, masks, iscale, oscale, part;
  bool need_out = false, next_real = false, last = false;
};

// One step list of a tick: entries (slot, span) and the unit prefix.
struct StepList {
  std::vector<int> sent, span, pref, ways;
  long long units = 0;
  size_t at_sent = 0, at_span = 0, at_pref = 0, at_ways = 0;  // byte offsets in the staging buffer
  void clear() {
    sent.clear();
    span.clear();
    pref.clear();
    ways.clear();
    units = 0;
  }
};

}  // namespace

// One lane of the server: a request loop thread with its own streams, chart
// arena, slots and tick buffers.  puck_server runs several lanes over one
// set of device grammar tables; a request stays in the lane it was given to.
struct Lane {
  const puck_grammar* g = nullptr;
  puck_options opt{};
  int nl = 0;
  bool mbr = false;
  cudaStream_t stream = nullptr, dstream = nullptr;
  std::vector<std::shared_ptr<LevelDev>> levels;  // shared by the lanes
  std::vector<LevelArena> la;
  DevBuf d_len, d_cell_off, d_node_off, d_mbr_off, d_words, d_status, d_counters, d_decode, d_scratch, d_parts,
      d_cell_cnt;
  int slots = 0, sms = 1, max_cs = 0;
  CellArena arena;
  std::vector<int> free_slots;
  TickBuf tb[2];
  CoarseGroup groups[kGroups];
  cudaStream_t cstream = nullptr;
  cudaEvent_t ev_slots[2] = {nullptr, nullptr};  // per tick buffer: after its slot updates
  std::vector<Resident> resident;  // loop thread only
  std::vector<StepList> lists;     // loop thread only

  mutable std::mutex mu;
  std::condition_variable cv_submit, cv_done;
  std::condition_variable* any_done = nullptr;  // the server's: notified with cv_done
  std::deque<int64_t> pending;
  std::unordered_map<int64_t, Request> reqs;
  std::deque<int64_t> done_q;
  int64_t next_id = 0;
  bool stopping = false;
  puck_server_stats stats{};
  std::vector<std::array<double, 5>> pass_ms;  // per level: lexicon, inside, outside, masks, decode
  std::thread loop;
};

namespace {

void ensure_host(char*& p, size_t& cap, size_t bytes) {
  if (bytes <= cap) return;
  if (p) cudaFreeHost(p);
  p = nullptr;
  cap = 0;
  const size_t want = std::max<size_t>(bytes + bytes / 2, 1 << 20);
  CUDA_TRY(cudaHostAlloc(reinterpret_cast<void**>(&p), want, cudaHostAllocDefault));
  cap = want;
}

void ensure_out(TickBuf& T, size_t nodes) {
  if (nodes <= T.out_cap) return;
  if (T.out_host) cudaFreeHost(T.out_host);
  T.out_host = nullptr;
  T.out_dev = nullptr;
  T.out_cap = 0;
  const size_t want = std::max<size_t>(nodes + nodes / 2, 1 << 16);
  void* h = nullptr;
  CUDA_TRY(cudaHostAlloc(&h, want * sizeof(puck_tree_node), cudaHostAllocMapped));
  void* d = nullptr;
  CUDA_TRY(cudaHostGetDevicePointer(&d, h, 0));
  T.out_host = static_cast<puck_tree_node*>(h);
  T.out_dev = static_cast<puck::DevNode*>(d);
  T.out_cap = want;
}

int group_of(const Lane* S, const Resident& r) {
  return r.stage == ST_DEC ? 4 * S->nl : 4 * r.level + r.stage;
}

long long units_of(const Resident& r) {
  switch (r.stage) {
    case ST_LEX: return r.n;
    case ST_IN:
    case ST_OUT: return r.n - r.span + 1;
    default: return 2 * tri(r.n);
  }
}

// Next pass step of a sentence (the order of CLParser.parse for one sentence:
// per level lexicon, inside spans 1..n, outside spans n..1 where needed,
// masks; then the decode of the last level).
void advance(const Lane* S, Resident& r) {
  const LevelArena& A = S->la[r.level];
  switch (r.stage) {
    case ST_LEX: r.stage = ST_IN; r.span = 1; return;
    case ST_IN:
      if (r.span < r.n) { ++r.span; return; }
      if (A.need_out) { r.stage = ST_OUT; r.span = r.n; return; }
      r.stage = A.last ? ST_DEC : ST_MASK;
      return;
    case ST_OUT:
      if (r.span > 1) { --r.span; return; }
      r.stage = A.last ? ST_DEC : ST_MASK;
      return;
    case ST_MASK: ++r.level; r.stage = ST_LEX; r.span = 0; return;
    default: return;
  }
}

void fail_all(Lane* S, puck_status st) {
  std::lock_guard<std::mutex> lk(S->mu);
  S->stopping = true;  // the request loop has ended: later submits are refused
  const int64_t t = now_ns();
  auto fail = [&](int64_t id) {
    Request& r = S->reqs[id];
    r.status = st;
    r.t_done = t;
    S->done_q.push_back(id);
    ++S->stats.failed;
    ++S->stats.completed;
  };
  for (int64_t id : S->pending) fail(id);
  S->pending.clear();
  for (const Resident& r : S->resident) fail(r.id);
  for (TickBuf& T : S->tb) {
    for (const Finishing& f : T.finishing) fail(f.id);
    T.finishing.clear();
  }
  S->resident.clear();
  S->stats.resident = 0;
  S->cv_done.notify_all();
  if (S->any_done) S->any_done->notify_all();
}

void harvest(Lane* S, int p) {
  TickBuf& T = S->tb[p];
  CUDA_TRY(cudaEventSynchronize(T.ev_end));
  float ms = 0.f, dms = 0.f;
  CUDA_TRY(cudaEventElapsedTime(&ms, T.ev_begin, T.ev_end));
  if (T.decoded) {
    CUDA_TRY(cudaEventSynchronize(T.ev_dec_end));
    CUDA_TRY(cudaEventElapsedTime(&dms, T.ev_dec_begin, T.ev_dec_end));
  }
  std::vector<float> gms(T.ev_group.size() > 1 ? T.ev_group.size() - 1 : 0, 0.f);
  for (size_t k = 0; k < gms.size(); ++k) CUDA_TRY(cudaEventElapsedTime(&gms[k], T.ev_group[k], T.ev_group[k + 1]));
  const int64_t t = now_ns();
  std::lock_guard<std::mutex> lk(S->mu);
  for (size_t k = 0; k < gms.size(); ++k) S->pass_ms[k / 4][k % 4] += gms[k];
  if (!T.ev_group.empty()) S->pass_ms[S->nl - 1][4] += dms;
  for (const Finishing& f : T.finishing) {
    Request& r = S->reqs[f.id];
    r.nodes.assign(T.out_host + f.node_at, T.out_host + f.node_at + (2 * f.n - 1));
    r.t_done = t;
    S->done_q.push_back(f.id);
    ++S->stats.completed;
    // the decode has read the sentence's cells: they and its slot are free
    S->arena.release(f.cell_off, 2 * tri(f.n));
    S->free_slots.push_back(f.slot);
  }
  S->stats.ms_device += ms + dms;
  S->stats.kernel_launches += T.launches;
  S->stats.h2d_bytes += T.h2d;
  S->stats.d2h_bytes += T.d2h;
  T.finishing.clear();
  S->cv_done.notify_all();
  if (S->any_done) S->any_done->notify_all();
}

// Launches the coarse levels of one group (the sentences admitted in one
// tick) as a batch on the coarse stream, once tick buffer p's slot updates
// have run: per level the lexicon, inside spans 1..n, outside spans n..1 and
// the masks (and scales for a Real next level), each launch covering every
// sentence of the group with cells of that span.
void launch_group(Lane* S, int gi, const std::vector<std::pair<int, int>>& members, int p) {
  CoarseGroup& Gp = S->groups[gi];
  cudaStream_t cs = S->cstream;
  const int ns = (int)members.size();
  std::vector<int> order(ns);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return members[a].second > members[b].second; });
  const int maxn = members[order[0]].second;
  std::vector<int> wl;
  struct ListAt {
    size_t sent, pref;
    int nent;
    long long nunits;
    int span, ways;
  };
  auto add_list = [&](int nent, int span, int ways, auto units) {
    ListAt at{wl.size(), 0, nent, 0, span, ways};
    for (int k = 0; k < nent; ++k) wl.push_back(members[order[k]].first);
    at.pref = wl.size();
    long long acc = 0;
    wl.push_back(0);
    for (int k = 0; k < nent; ++k) {
      acc += units(members[order[k]].second) * ways;
      wl.push_back((int)acc);
    }
    at.nunits = acc;
    return at;
  };
  std::vector<ListAt> spans(maxn + 1);
  long long part_units = 0;
  for (int L = 1; L <= maxn; ++L) {
    int k = 0;
    long long cells = 0;
    while (k < ns && members[order[k]].second >= L) cells += members[order[k++]].second - L + 1;
    const int G = puck::cell_ways(L, puck::part_target((double)cells * (L - 1), S->sms));
    if (G > 1) part_units = std::max(part_units, cells * G);
    spans[L] = add_list(k, L, G, [L](int n) { return (long long)(n - L + 1); });
  }
  const ListAt toks = add_list(ns, 1, 1, [](int n) { return (long long)n; });
  const ListAt cells = add_list(ns, 0, 1, [](int n) { return 2 * tri(n); });
  const size_t bytes = wl.size() * sizeof(int);
  ensure_host(Gp.host, Gp.host_cap, bytes);
  std::memcpy(Gp.host, wl.data(), bytes);
  Gp.dev.ensure(std::max<size_t>(bytes, 16));
  if (part_units > 0) Gp.parts.ensure(part_units * S->max_cs * sizeof(float));
  CUDA_TRY(cudaStreamWaitEvent(cs, S->ev_slots[p], 0));
  CUDA_TRY(cudaEventRecord(Gp.begin, cs));
  CUDA_TRY(cudaMemcpyAsync(Gp.dev.p, Gp.host, bytes, cudaMemcpyHostToDevice, cs));
  const int* wdev = Gp.dev.as<int>();
  auto work = [&](const ListAt& a) {
    puck::DevWork W{};
    W.nent = a.nent;
    W.nunits = a.nunits;
    W.sent = wdev + a.sent;
    W.span = nullptr;
    W.span_all = a.span;
    W.pref = wdev + a.pref;
    W.ways = nullptr;
    W.ways_all = a.ways;
    W.part_rows = Gp.parts.as<float>();
    W.cell_cnt = S->d_cell_cnt.as<int>();
    W.one_word_batch = 0;
    return W;
  };
  puck::DevBatch B{};
  B.nsent = S->slots;
  B.len = S->d_len.as<int>();
  B.cell_off = S->d_cell_off.as<long long>();
  B.word_off = S->d_cell_off.as<long long>();
  B.words = S->d_words.as<int>();
  B.node_off = S->d_node_off.as<long long>();
  const puck::Counters C{S->d_counters.as<unsigned long long>(), S->d_counters.as<unsigned long long>() + 1,
                         S->d_status.as<int>()};
  const int maxlen = S->opt.max_length;
  int64_t launches = 0;
  puck::DevMask M{nullptr, 0, nullptr, nullptr};
  for (int l = 0; l + 1 < S->nl; ++l) {
    const puck::DevLevel& D = S->levels[l]->d;
    LevelArena& A = S->la[l];
    float* inside = A.inside.as<float>();
    float* outside = A.outside.as<float>();
    const puck::DevLive V{A.live_in.as<int>(), A.live_out.as<int>()};
    puck::DevMask MM = M;
    if (D.semiring != puck::SEMI_REAL) { MM.iscale = nullptr; MM.oscale = nullptr; }
    CUDA_TRY(puck::launch_lexicon(D, B, work(toks), MM, inside, A.part.as<double>(), V, C, cs));
    for (int L = 1; L <= maxn; ++L) CUDA_TRY(puck::launch_inside_span(D, B, work(spans[L]), MM, maxlen, inside, V, C, cs));
    for (int L = maxn; L >= 1; --L)
      CUDA_TRY(puck::launch_outside_span(D, B, work(spans[L]), MM, maxlen, inside, outside, V, C, cs));
    const puck::DevWork Wc = work(cells);
    CUDA_TRY(puck::launch_masks(D, B, Wc, inside, outside, S->opt.prune_threshold, A.masks.as<int>(), cs));
    launches += 2 + 2 * maxn;
    if (A.next_real) {
      CUDA_TRY(puck::launch_scaling(D.cell_size, B, Wc, inside, A.iscale.as<float>(), cs));
      CUDA_TRY(puck::launch_scaling(D.cell_size, B, Wc, outside, A.oscale.as<float>(), cs));
      launches += 2;
    }
    M.bits = A.masks.as<int>();
    M.mask_size = D.mask_size;
    M.iscale = A.next_real ? A.iscale.as<float>() : nullptr;
    M.oscale = A.next_real ? A.oscale.as<float>() : nullptr;
  }
  CUDA_TRY(cudaEventRecord(Gp.done, cs));
  std::lock_guard<std::mutex> lk(S->mu);
  S->stats.kernel_launches += launches;
  S->stats.h2d_bytes += (int64_t)bytes;
}

// Builds, uploads and launches one tick into buffer p.  Returns false when
// nothing was resident.
bool run_tick(Lane* S, int p) {
  TickBuf& T = S->tb[p];
  T.launches = T.h2d = T.d2h = 0;
  std::vector<SlotUpdate> upd;
  std::vector<int> staged_words;
  // with a cascade, this tick's admissions form one coarse group
  const bool grouped = S->nl >= 2;
  int gi = -1;
  for (int k = 0; grouped && k < kGroups && gi < 0; ++k)
    if (!S->groups[k].busy) gi = k;
  std::vector<std::pair<int, int>> members;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    while ((!grouped || gi >= 0) && !S->pending.empty() && !S->free_slots.empty()) {
      const int64_t id = S->pending.front();
      Request& q = S->reqs[id];
      const long long off = S->arena.alloc(2 * tri(q.n));
      if (off < 0) break;
      const int slot = S->free_slots.back();
      S->free_slots.pop_back();
      if (grouped) {
        S->resident.push_back(Resident{id, slot, q.n, off, S->nl - 1, ST_WAIT, 0, (int)upd.size(), gi});
        members.emplace_back(slot, q.n);
      } else {
        S->resident.push_back(Resident{id, slot, q.n, off, 0, ST_LEX, 0, (int)upd.size(), -1});
      }
      upd.push_back(SlotUpdate{off, 0, 6 * off, slot, q.n, (int)staged_words.size(), 1});
      staged_words.insert(staged_words.end(), q.words.begin(), q.words.end());
      std::vector<int>().swap(q.words);
      S->pending.pop_front();
    }
    S->stats.resident = (int64_t)S->resident.size();
    S->stats.resident_peak = std::max(S->stats.resident_peak, S->stats.resident);
    S->stats.arena_cells_peak = S->arena.peak();
  }
  if (!members.empty()) {
    S->groups[gi].busy = true;
    S->groups[gi].waiting = (int)members.size();
  }
  if (S->resident.empty()) return false;

  // step lists: each sentence takes its next steps while their launch comes
  // later in the tick than the step it took before
  const int G = 4 * S->nl + 1;
  auto& lists = S->lists;
  lists.resize(G);
  for (auto& L : lists) L.clear();
  long long out_nodes = 0;
  std::vector<Resident> keep;
  keep.reserve(S->resident.size());
  for (Resident r : S->resident) {
    if (r.stage == ST_WAIT) {
      // admitted this tick (its group is not launched yet) or its coarse
      // batch still running: not in this tick
      CoarseGroup& Gp = S->groups[r.grp];
      if (r.upd >= 0 || cudaEventQuery(Gp.done) != cudaSuccess) {
        r.upd = -1;
        keep.push_back(r);
        continue;
      }
      r.stage = ST_LEX;  // level nl - 1: the coarse levels are done
      if (--Gp.waiting == 0) {
        float gms = 0.f;
        if (cudaEventElapsedTime(&gms, Gp.begin, Gp.done) == cudaSuccess) {
          std::lock_guard<std::mutex> lk(S->mu);
          S->stats.ms_device += gms;
          S->pass_ms[0][1] += gms;
        }
        Gp.busy = false;
      }
    }
    int last_g = -1;
    bool done = false;
    while (true) {
      const int g = group_of(S, r);
      if (g <= last_g) break;
      StepList& L = lists[g];
      L.sent.push_back(r.slot);
      if (r.stage == ST_IN || r.stage == ST_OUT) L.span.push_back(r.span);
      L.pref.push_back((int)units_of(r));  // per-entry units; prefix formed below
      last_g = g;
      if (r.stage == ST_DEC) {
        T.finishing.push_back(Finishing{r.id, out_nodes, r.n, r.slot, r.cell_off});
        // a sentence admitted in this tick keeps one record (two records of
        // one slot would race in k_slot_update)
        if (r.upd >= 0) upd[r.upd].node_off = out_nodes;
        else upd.push_back(SlotUpdate{r.cell_off, out_nodes, 6 * r.cell_off, r.slot, r.n, -1, 0});
        out_nodes += 2 * r.n - 1;
        done = true;
        break;
      }
      advance(S, r);
    }
    r.upd = -1;
    if (!done) keep.push_back(r);
  }
  S->resident.swap(keep);
  // every resident sentence is waiting for its coarse batch and nothing was
  // admitted: wait for the oldest running batch instead of an empty tick
  bool any = !upd.empty() || !T.finishing.empty();
  for (const auto& L : lists) any = any || !L.sent.empty();
  if (!any) {
    for (CoarseGroup& Gp : S->groups)
      if (Gp.busy) {
        CUDA_TRY(cudaEventSynchronize(Gp.done));
        break;
      }
    return false;
  }
  // span lists longest span first (their CTAs run longest)
  for (int g = 0; g < G; ++g) {
    StepList& L = lists[g];
    if (L.span.empty()) continue;
    std::vector<int> idx(L.sent.size());
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return L.span[a] > L.span[b]; });
    std::vector<int> s2(idx.size()), p2(idx.size()), u2(idx.size());
    for (size_t k = 0; k < idx.size(); ++k) {
      s2[k] = L.sent[idx[k]];
      p2[k] = L.span[idx[k]];
      u2[k] = L.pref[idx[k]];
    }
    L.sent.swap(s2);
    L.span.swap(p2);
    L.pref.swap(u2);
  }
  // span lists: CTAs per cell from the launch's total cell count
  long long part_units = 0;
  for (auto& L : lists) {
    if (L.span.empty()) continue;
    double splits = 0;
    for (size_t k = 0; k < L.sent.size(); ++k) splits += (double)L.pref[k] * std::max(L.span[k] - 1, 1);
    const double target = puck::part_target(splits, S->sms);
    L.ways.resize(L.sent.size());
    bool split = false;
    for (size_t k = 0; k < L.sent.size(); ++k) {
      L.ways[k] = puck::cell_ways(L.span[k], target);
      L.pref[k] *= L.ways[k];
      split |= L.ways[k] > 1;
    }
    if (split) {
      long long u = 0;
      for (int x : L.pref) u += x;
      part_units = std::max(part_units, u);
    }
  }
  for (auto& L : lists) {
    long long acc = 0;
    std::vector<int> pref(L.pref.size() + 1, 0);
    for (size_t k = 0; k < L.pref.size(); ++k) {
      acc += L.pref[k];
      if (acc > INT32_MAX) throw PuckError{PUCK_ERR_INTERNAL, "tick work list above 2^31 units"};
      pref[k + 1] = (int)acc;
    }
    L.pref.swap(pref);
    L.units = acc;
  }

  // staging layout: updates | words | per list sent, span, pref (16-byte aligned sections)
  size_t bytes = 0;
  auto section = [&](size_t n) {
    const size_t at = bytes;
    bytes += (n + 15) & ~size_t(15);
    return at;
  };
  const size_t at_upd = section(upd.size() * sizeof(SlotUpdate));
  const size_t at_words = section(staged_words.size() * sizeof(int));
  for (auto& L : lists) {
    L.at_sent = section(L.sent.size() * sizeof(int));
    L.at_span = section(L.span.size() * sizeof(int));
    L.at_pref = section(L.pref.size() * sizeof(int));
    L.at_ways = section(L.ways.size() * sizeof(int));
  }
  ensure_host(T.host, T.host_cap, bytes);
  std::memcpy(T.host + at_upd, upd.data(), upd.size() * sizeof(SlotUpdate));
  std::memcpy(T.host + at_words, staged_words.data(), staged_words.size() * sizeof(int));
  for (auto& L : lists) {
    std::memcpy(T.host + L.at_sent, L.sent.data(), L.sent.size() * sizeof(int));
    std::memcpy(T.host + L.at_span, L.span.data(), L.span.size() * sizeof(int));
    std::memcpy(T.host + L.at_pref, L.pref.data(), L.pref.size() * sizeof(int));
    std::memcpy(T.host + L.at_ways, L.ways.data(), L.ways.size() * sizeof(int));
  }
  if (part_units > 0) S->d_parts.ensure(part_units * S->max_cs * sizeof(float));
  T.dev.ensure(std::max<size_t>(bytes, 16));
  ensure_out(T, (size_t)out_nodes);
  cudaStream_t st = S->stream;
  CUDA_TRY(cudaEventRecord(T.ev_begin, st));
  CUDA_TRY(cudaMemcpyAsync(T.dev.p, T.host, bytes, cudaMemcpyHostToDevice, st));
  T.h2d = (int64_t)bytes;
  T.d2h = out_nodes * (int64_t)sizeof(puck_tree_node);
  const char* dbase = static_cast<const char*>(T.dev.p);
  if (!upd.empty()) {
    SlotTables tab{};
    tab.len = S->d_len.as<int>();
    tab.cell_off = S->d_cell_off.as<long long>();
    tab.node_off = S->d_node_off.as<long long>();
    tab.mbr_off = S->d_mbr_off.as<long long>();
    tab.words = S->d_words.as<int>();
    tab.status = S->d_status.as<int>();
    tab.nlevels = S->nl;
    for (int l = 0; l < S->nl; ++l) tab.part[l] = S->la[l].part.as<double>();
    k_slot_update<<<(unsigned)upd.size(), 128, 0, st>>>(tab, reinterpret_cast<const SlotUpdate*>(dbase + at_upd),
                                                        reinterpret_cast<const int*>(dbase + at_words));
    CUDA_TRY(cudaGetLastError());
    ++T.launches;
  }
  if (!members.empty()) {
    CUDA_TRY(cudaEventRecord(S->ev_slots[p], st));
    launch_group(S, gi, members, p);
  }

  puck::DevBatch B{};
  B.nsent = S->slots;
  B.len = S->d_len.as<int>();
  B.cell_off = S->d_cell_off.as<long long>();
  B.word_off = S->d_cell_off.as<long long>();
  B.words = S->d_words.as<int>();
  B.node_off = S->d_node_off.as<long long>();
  puck::Counters C{S->d_counters.as<unsigned long long>(), S->d_counters.as<unsigned long long>() + 1,
                   S->d_status.as<int>()};
  auto work = [&](const StepList& L) {
    puck::DevWork W{};
    W.nent = (int)L.sent.size();
    W.nunits = L.units;
    W.sent = reinterpret_cast<const int*>(dbase + L.at_sent);
    W.span = L.span.empty() ? nullptr : reinterpret_cast<const int*>(dbase + L.at_span);
    W.span_all = 0;
    W.pref = reinterpret_cast<const int*>(dbase + L.at_pref);
    W.ways = L.ways.empty() ? nullptr : reinterpret_cast<const int*>(dbase + L.at_ways);
    W.ways_all = 1;
    W.part_rows = S->d_parts.as<float>();
    W.cell_cnt = S->d_cell_cnt.as<int>();
    W.one_word_batch = 0;
    return W;
  };
  const int maxlen = S->opt.max_length;
  const bool prof = !T.ev_group.empty();
  auto mark = [&](int k) {
    if (prof) CUDA_TRY(cudaEventRecord(T.ev_group[k], st));
  };
  mark(0);
  puck::DevMask M{nullptr, 0, nullptr, nullptr};
  for (int l = 0; l < S->nl; ++l) {
    const puck::DevLevel& D = S->levels[l]->d;
    LevelArena& A = S->la[l];
    float* inside = A.inside.as<float>();
    float* outside = A.need_out ? A.outside.as<float>() : nullptr;
    const puck::DevLive V{A.live_in.as<int>(), A.need_out ? A.live_out.as<int>() : nullptr};
    puck::DevMask MM = M;
    if (D.semiring != puck::SEMI_REAL) { MM.iscale = nullptr; MM.oscale = nullptr; }
    const StepList& Llex = lists[4 * l + ST_LEX];
    const StepList& Lin = lists[4 * l + ST_IN];
    const StepList& Lout = lists[4 * l + ST_OUT];
    const StepList& Lmask = lists[4 * l + ST_MASK];
    if (!Llex.sent.empty()) {
      CUDA_TRY(puck::launch_lexicon(D, B, work(Llex), MM, inside, A.part.as<double>(), V, C, st));
      ++T.launches;
    }
    mark(4 * l + 1);
    if (!Lin.sent.empty()) {
      CUDA_TRY(puck::launch_inside_span(D, B, work(Lin), MM, maxlen, inside, V, C, st));
      ++T.launches;
    }
    mark(4 * l + 2);
    if (!Lout.sent.empty()) {
      CUDA_TRY(puck::launch_outside_span(D, B, work(Lout), MM, maxlen, inside, outside, V, C, st));
      ++T.launches;
    }
    mark(4 * l + 3);
    if (!A.last) {
      if (!Lmask.sent.empty()) {
        const puck::DevWork W = work(Lmask);
        CUDA_TRY(puck::launch_masks(D, B, W, inside, outside, S->opt.prune_threshold, A.masks.as<int>(), st));
        ++T.launches;
        if (A.next_real) {
          CUDA_TRY(puck::launch_scaling(D.cell_size, B, W, inside, A.iscale.as<float>(), st));
          CUDA_TRY(puck::launch_scaling(D.cell_size, B, W, outside, A.oscale.as<float>(), st));
          T.launches += 2;
        }
      }
      M.bits = A.masks.as<int>();
      M.mask_size = D.mask_size;
      M.iscale = A.next_real ? A.iscale.as<float>() : nullptr;
      M.oscale = A.next_real ? A.oscale.as<float>() : nullptr;
      mark(4 * l + 4);
      continue;
    }
    mark(4 * l + 4);
    const StepList& Ldec = lists[4 * S->nl];
    T.decoded = !Ldec.sent.empty();
    if (!T.decoded) continue;
    // decode on the side stream, after this tick's last-level passes
    cudaStream_t ds = S->dstream;
    CUDA_TRY(cudaEventRecord(T.ev_fine, st));
    CUDA_TRY(cudaStreamWaitEvent(ds, T.ev_fine, 0));
    CUDA_TRY(cudaEventRecord(T.ev_dec_begin, ds));
    puck::DevWork W = work(Ldec);
    if (!S->mbr) {
      CUDA_TRY(puck::launch_viterbi(D, B, W, maxlen, inside, T.out_dev, ds));
      ++T.launches;
    } else {
      CUDA_TRY(puck::launch_mbr_cells(D, B, W, inside, outside, S->d_decode.as<float2>(), ds));
      W.pref = nullptr;
      CUDA_TRY(puck::launch_mbr_decode(B, W, M, D.semiring == puck::SEMI_REAL ? 1 : 0, S->d_decode.as<float2>(),
                                       S->d_mbr_off.as<long long>(), S->d_scratch.as<float>(), T.out_dev, ds));
      T.launches += 2;
    }
    CUDA_TRY(cudaEventRecord(T.ev_dec_end, ds));
  }
  CUDA_TRY(cudaEventRecord(T.ev_end, st));
  {
    std::lock_guard<std::mutex> lk(S->mu);
    ++S->stats.ticks;
    S->stats.resident = (int64_t)S->resident.size();
  }
  return true;
}

void loop_main(Lane* S) {
  try {
    CUDA_TRY(cudaSetDevice(S->opt.device));
    std::deque<int> inflight;
    uint64_t tick = 0;
    while (true) {
      bool idle;
      {
        std::unique_lock<std::mutex> lk(S->mu);
        idle = S->resident.empty() && inflight.empty();
        if (idle) {
          S->cv_submit.wait(lk, [&] { return S->stopping || !S->pending.empty(); });
          if (S->pending.empty()) break;  // stopping with nothing left
        }
      }
      if (inflight.size() >= 2) {
        harvest(S, inflight.front());
        inflight.pop_front();
      }
      const int p = (int)(tick & 1);
      if (run_tick(S, p)) {
        inflight.push_back(p);
        ++tick;
      } else if (!inflight.empty()) {
        harvest(S, inflight.front());
        inflight.pop_front();
      } else if (S->resident.empty()) {
        // nothing resident and nothing admissible: wait for a submit
        std::unique_lock<std::mutex> lk(S->mu);
        S->cv_submit.wait_for(lk, std::chrono::milliseconds(1));
      }
    }
  } catch (const PuckError& e) {
    puck::set_last_error(e.msg);
    fail_all(S, e.status);
  }
}

int64_t server_bytes_per_cell(const Lane* S) {
  int64_t b = 8;  // the sentence's words at its first cells; the cell's part counter
  for (int l = 0; l < S->nl; ++l) {
    const HostLevel& L = S->g->levels[l];
    const LevelArena& A = S->la[l];
    const int k = A.need_out ? 2 : 1;
    b += (int64_t)(L.cell_size + L.mask_size) * 4 * k;
    if (!A.last) b += (int64_t)L.mask_size * 4;
    if (A.next_real) b += 8;
  }
  if (S->mbr) b += 8 + 24;  // per-cell decode pairs; decode tables (3(n+1)^2 <= 6 n(n+1) floats)
  return b;
}

void destroy_server(Lane* S) {
  cudaSetDevice(S->opt.device);
  for (TickBuf& T : S->tb) {
    if (T.host) cudaFreeHost(T.host);
    if (T.out_host) cudaFreeHost(T.out_host);
    T.dev.release();
    if (T.ev_begin) cudaEventDestroy(T.ev_begin);
    if (T.ev_end) cudaEventDestroy(T.ev_end);
    for (cudaEvent_t e : {T.ev_fine, T.ev_dec_begin, T.ev_dec_end})
      if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : T.ev_group) cudaEventDestroy(e);
  }
  for (LevelArena& A : S->la)
    for (DevBuf* b : {&A.inside, &A.outside, &A.live_in, &A.live_out, &A.masks, &A.iscale, &A.oscale, &A.part})
      b->release();
  for (DevBuf* b : {&S->d_len, &S->d_cell_off, &S->d_node_off, &S->d_mbr_off, &S->d_words, &S->d_status,
                    &S->d_counters, &S->d_decode, &S->d_scratch, &S->d_parts, &S->d_cell_cnt})
    b->release();
  S->levels.clear();
  if (S->stream) cudaStreamDestroy(S->stream);
  if (S->dstream) cudaStreamDestroy(S->dstream);
  if (S->cstream) cudaStreamDestroy(S->cstream);
  for (cudaEvent_t e : S->ev_slots)
    if (e) cudaEventDestroy(e);
  for (CoarseGroup& Gp : S->groups) {
    if (Gp.begin) cudaEventDestroy(Gp.begin);
    if (Gp.done) cudaEventDestroy(Gp.done);
    if (Gp.host) cudaFreeHost(Gp.host);
    Gp.dev.release();
    Gp.parts.release();
  }
  delete S;
}

// A lane over the server's device grammar tables; opt holds the lane's share
// of the memory budget (mem_bytes) and of the slots (max_batch_sentences).
Lane* lane_create(const puck_grammar* g, const puck_options& opt, const std::vector<std::shared_ptr<LevelDev>>& levels,
                  std::condition_variable* any_done, puck_status* status) {
  auto* S = new Lane();
  try {
    S->g = g;
    S->opt = opt;
    S->any_done = any_done;
    if (S->opt.max_length <= 0) S->opt.max_length = 100;
    if (S->opt.max_length > puck::kMaxLen)
      throw PuckError{PUCK_ERR_INVALID_ARG, "max_length above " + std::to_string(puck::kMaxLen)};
    S->nl = (int)g->levels.size();
    if (S->nl < 1 || S->nl > kMaxLevels) throw PuckError{PUCK_ERR_INVALID_ARG, "unsupported number of levels"};
    const HostLevel& fine = g->levels.back();
    const bool vit = S->opt.decode == PUCK_DECODE_VITERBI ||
                     (S->opt.decode == PUCK_DECODE_AUTO && fine.semiring == puck::SEMI_VITERBI);
    if (vit && fine.semiring != puck::SEMI_VITERBI)
      throw PuckError{PUCK_ERR_INVALID_ARG, "Viterbi decoding needs a Viterbi fine level"};
    if (!vit && fine.semiring == puck::SEMI_VITERBI)
      throw PuckError{PUCK_ERR_INVALID_ARG, "MBR decoding needs a sum-product fine level"};
    if (!vit && S->nl < 2) throw PuckError{PUCK_ERR_INVALID_ARG, "Can't use null pruning mask for parse extraction!"};
    S->mbr = !vit;
    int ndev = 0;
    CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (S->opt.device < 0 || S->opt.device >= ndev) throw PuckError{PUCK_ERR_INVALID_ARG, "no such CUDA device"};
    CUDA_TRY(cudaSetDevice(S->opt.device));
    CUDA_TRY(cudaDeviceGetAttribute(&S->sms, cudaDevAttrMultiProcessorCount, S->opt.device));
    CUDA_TRY(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking));
    CUDA_TRY(cudaStreamCreateWithFlags(&S->dstream, cudaStreamNonBlocking));
    CUDA_TRY(cudaStreamCreateWithFlags(&S->cstream, cudaStreamNonBlocking));
    for (cudaEvent_t& e : S->ev_slots) CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (CoarseGroup& Gp : S->groups) {
      CUDA_TRY(cudaEventCreate(&Gp.begin));
      CUDA_TRY(cudaEventCreate(&Gp.done));
    }
    for (TickBuf& T : S->tb) {
      CUDA_TRY(cudaEventCreate(&T.ev_begin));
      CUDA_TRY(cudaEventCreate(&T.ev_end));
      CUDA_TRY(cudaEventCreate(&T.ev_fine));
      CUDA_TRY(cudaEventCreate(&T.ev_dec_begin));
      CUDA_TRY(cudaEventCreate(&T.ev_dec_end));
    }
    S->nl = (int)g->levels.size();
    S->pass_ms.assign(S->nl, std::array<double, 5>{0, 0, 0, 0, 0});
    for (TickBuf& T : S->tb) {
      if (!S->opt.profile) continue;
      T.ev_group.resize(4 * S->nl + 1);
      for (cudaEvent_t& e : T.ev_group) CUDA_TRY(cudaEventCreate(&e));
    }
    S->levels = levels;
    S->la.resize(S->nl);
    for (int l = 0; l < S->nl; ++l) {
      LevelArena& A = S->la[l];
      A.last = l == S->nl - 1;
      A.need_out = !A.last || S->mbr;
      A.next_real = !A.last && g->levels[l + 1].semiring == puck::SEMI_REAL;
    }
    S->slots = S->opt.max_batch_sentences > 0 ? S->opt.max_batch_sentences : kDefaultSlots;
    size_t free_b = 0, total_b = 0;
    CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    const int64_t cap = (int64_t)(free_b * 0.8);
    const int64_t budget = S->opt.mem_bytes > 0 ? std::min<int64_t>(S->opt.mem_bytes, cap) : cap;
    const int64_t per_slot = 4 + 8 * 3 + 4 + 8 * S->nl;
    const int64_t per_cell = server_bytes_per_cell(S);
    const int64_t cells = std::min<int64_t>((budget - per_slot * S->slots) / per_cell, (int64_t)INT32_MAX - 1);
    if (cells < 2 * tri(S->opt.max_length))
      throw PuckError{PUCK_ERR_OOM, "memory budget holds no sentence of the maximum length"};
    S->arena.init(cells);
    for (int l = 0; l < S->nl; ++l) {
      const HostLevel& L = g->levels[l];
      LevelArena& A = S->la[l];
      A.inside.ensure(cells * L.cell_size * sizeof(float));
      A.live_in.ensure(cells * L.mask_size * sizeof(int));
      if (A.need_out) {
        A.outside.ensure(cells * L.cell_size * sizeof(float));
        A.live_out.ensure(cells * L.mask_size * sizeof(int));
      }
      if (!A.last) A.masks.ensure(cells * L.mask_size * sizeof(int));
      if (A.next_real) {
        A.iscale.ensure(cells * sizeof(float));
        A.oscale.ensure(cells * sizeof(float));
      }
      A.part.ensure(S->slots * sizeof(double));
    }
    S->d_len.ensure(S->slots * sizeof(int));
    S->d_cell_off.ensure(S->slots * sizeof(long long));
    S->d_node_off.ensure(S->slots * sizeof(long long));
    S->d_mbr_off.ensure(S->slots * sizeof(long long));
    S->d_status.ensure(S->slots * sizeof(int));
    S->d_words.ensure(cells * sizeof(int));
    S->d_counters.ensure(64);
    CUDA_TRY(cudaMemsetAsync(S->d_counters.p, 0, 64, S->stream));
    S->d_cell_cnt.ensure(cells * sizeof(int));
    CUDA_TRY(cudaMemsetAsync(S->d_cell_cnt.p, 0, cells * sizeof(int), S->stream));
    for (const HostLevel& HL : g->levels) S->max_cs = std::max(S->max_cs, HL.cell_size);
    if (S->mbr) {
      S->d_decode.ensure(cells * sizeof(float2));
      S->d_scratch.ensure(6 * cells * sizeof(float));
    }
    CUDA_TRY(cudaStreamSynchronize(S->stream));
    S->free_slots.resize(S->slots);
    for (int i = 0; i < S->slots; ++i) S->free_slots[i] = S->slots - 1 - i;
    S->stats.arena_cells = cells;
    S->loop = std::thread(loop_main, S);
    if (status) *status = PUCK_OK;
    return S;
  } catch (const PuckError& e) {
    puck::set_last_error(e.msg);
    if (status) *status = e.status;
  }
  destroy_server(S);
  return nullptr;
}

void lane_destroy(Lane* S) {
  if (!S) return;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stopping = true;
  }
  S->cv_submit.notify_all();
  if (S->loop.joinable()) S->loop.join();
  destroy_server(S);
}

// Queues sentences i = 0..nsent-1 in this lane; ids[i] receives the lane's
// id of each.
puck_status lane_submit(Lane* S, const int32_t* word_ids, const int64_t* offsets, int32_t nsent,
                        const int64_t* arrival_ns, int64_t* ids) {
  const int64_t t = now_ns();
  const int nwords = S->g->levels.back().n_words;
  const long long cap = S->arena.cap();
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stopping) {
      puck::set_last_error("puck_server_submit: server is stopping");
      return PUCK_ERR_INVALID_ARG;
    }
    for (int i = 0; i < nsent; ++i) {
      const int64_t id = S->next_id++;
      Request& r = S->reqs[id];
      const int64_t n = offsets[i + 1] - offsets[i];
      r.n = (int)std::max<int64_t>(n, 0);
      r.t_arrival = arrival_ns && arrival_ns[i] > 0 ? arrival_ns[i] : t;
      int st = PUCK_OK;
      if (n <= 0) st = PUCK_ERR_EMPTY;
      else if (n > S->opt.max_length) st = PUCK_ERR_SENT_TOO_LONG;
      else if (2 * tri(n) > cap) st = PUCK_ERR_OOM;
      else
        for (int64_t k = offsets[i]; k < offsets[i + 1]; ++k)
          if (word_ids[k] < 0 || word_ids[k] >= nwords) { st = PUCK_ERR_OOV; break; }
      ids[i] = id;
      ++S->stats.submitted;
      if (st != PUCK_OK) {
        r.status = st;
        r.t_done = t;
        S->done_q.push_back(id);
        ++S->stats.completed;
        ++S->stats.failed;
        continue;
      }
      r.words.assign(word_ids + offsets[i], word_ids + offsets[i + 1]);
      S->pending.push_back(id);
    }
  }
  S->cv_submit.notify_all();
  S->cv_done.notify_all();
  if (S->any_done) S->any_done->notify_all();
  return PUCK_OK;
}

int32_t lane_poll(Lane* S, int64_t* ids, int32_t max_ids, int32_t wait_ms) {
  if (max_ids <= 0) return 0;
  std::unique_lock<std::mutex> lk(S->mu);
  if (S->done_q.empty() && wait_ms > 0)
    S->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !S->done_q.empty(); });
  int32_t k = 0;
  while (k < max_ids && !S->done_q.empty()) {
    ids[k++] = S->done_q.front();
    S->done_q.pop_front();
  }
  return k;
}

puck_status lane_take(Lane* S, int64_t id, puck_tree_node* nodes, int32_t max_nodes, int32_t* sent_status,
                      int64_t* latency_ns) {
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->reqs.find(id);
  if (it == S->reqs.end() || it->second.t_done == 0) {
    puck::set_last_error("puck_server_take: no finished request with this id");
    return PUCK_ERR_INVALID_ARG;
  }
  Request& r = it->second;
  if (r.status == PUCK_OK && (!nodes || max_nodes < (int32_t)r.nodes.size())) {
    puck::set_last_error("puck_server_take: node buffer smaller than 2n-1");
    return PUCK_ERR_INVALID_ARG;
  }
  if (r.status == PUCK_OK) std::memcpy(nodes, r.nodes.data(), r.nodes.size() * sizeof(puck_tree_node));
  if (sent_status) *sent_status = r.status;
  if (latency_ns) *latency_ns = r.t_done - r.t_arrival;
  S->reqs.erase(it);
  return PUCK_OK;
}

puck_server_stats lane_stats(const Lane* S) {
  std::lock_guard<std::mutex> lk(S->mu);
  return S->stats;
}

void lane_pass_ms(const Lane* S, int32_t level, double out[5]) {
  std::lock_guard<std::mutex> lk(S->mu);
  for (int k = 0; k < 5; ++k) out[k] += S->pass_ms[level][k];
}

}  // namespace

// The server: lanes over one set of device grammar tables.  A request goes to
// the lane with the fewest cells queued or resident (ties: the lower lane);
// its id is the lane's id times the lane count plus the lane.  Each lane runs
// its own ticks on its own streams, so the tail of one lane's launches
// overlaps the other lanes' work instead of idling the GPU.
struct puck_server {
  std::vector<std::shared_ptr<LevelDev>> levels;
  std::vector<Lane*> lanes;
  std::vector<int64_t> load;  // per lane: cells of its submitted requests not yet taken
  std::unordered_map<int64_t, int64_t> cells_of;  // request id -> its cells (until taken)
  int nl = 0;
  std::mutex mu;
  std::condition_variable done;  // some lane finished a request
};

namespace {

// Lanes for a server: opts->server_lanes (0: two), fewer when a lane's share
// of the memory budget or of the slots would be too small for a sentence of
// the maximum length or for a useful batch.
int lane_count(const puck_options& o, int64_t budget, int64_t per_cell) {
  int lanes = o.server_lanes > 0 ? o.server_lanes : 2;
  lanes = std::min(lanes, 8);
  const int64_t maxlen = o.max_length > 0 ? o.max_length : 100;
  while (lanes > 1 && (budget / lanes) / std::max<int64_t>(per_cell, 1) < 8 * tri(maxlen)) --lanes;
  if (o.max_batch_sentences > 0) lanes = std::max(1, std::min(lanes, o.max_batch_sentences / 16));
  return lanes;
}

void destroy_all(puck_server* S) {
  for (Lane* L : S->lanes) lane_destroy(L);
  S->lanes.clear();
  S->levels.clear();
  delete S;
}

}  // namespace

extern "C" {

int64_t puck_server_now_ns(void) { return now_ns(); }

puck_server* puck_server_create(const puck_grammar* g, const puck_options* opts, puck_status* status) {
  auto* S = new puck_server();
  try {
    if (!g) throw PuckError{PUCK_ERR_INVALID_ARG, "null grammar"};
    puck_options o;
    if (opts) o = *opts;
    else puck_default_options(&o);
    S->nl = (int)g->levels.size();
    if (S->nl < 1 || S->nl > kMaxLevels) throw PuckError{PUCK_ERR_INVALID_ARG, "unsupported number of levels"};
    int ndev = 0;
    CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (o.device < 0 || o.device >= ndev) throw PuckError{PUCK_ERR_INVALID_ARG, "no such CUDA device"};
    CUDA_TRY(cudaSetDevice(o.device));
    for (int l = 0; l < S->nl; ++l) {
      S->levels.emplace_back(new LevelDev());
      build_level(*S->levels.back(), g->levels[l], l < S->nl - 1 && S->nl != 1);
    }
    size_t free_b = 0, total_b = 0;
    CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    const int64_t cap = (int64_t)(free_b * 0.8);
    const int64_t budget = o.mem_bytes > 0 ? std::min<int64_t>(o.mem_bytes, cap) : cap;
    int64_t per_cell = 8;
    for (const HostLevel& L : g->levels) per_cell += (int64_t)(L.cell_size + 2 * L.mask_size) * 8;
    const int n = lane_count(o, budget, per_cell);
    puck_options lo = o;
    lo.mem_bytes = budget / n;
    if (o.max_batch_sentences > 0) lo.max_batch_sentences = std::max(1, o.max_batch_sentences / n);
    for (int k = 0; k < n; ++k) {
      puck_status st = PUCK_OK;
      Lane* L = lane_create(g, lo, S->levels, &S->done, &st);
      if (!L) {
        char msg[512];
        puck_last_error(msg, sizeof msg);
        throw PuckError{st, msg};
      }
      S->lanes.push_back(L);
    }
    S->load.assign(n, 0);
    if (status) *status = PUCK_OK;
    return S;
  } catch (const PuckError& e) {
    puck::set_last_error(e.msg);
    if (status) *status = e.status;
  }
  destroy_all(S);
  return nullptr;
}

void puck_server_destroy(puck_server* S) {
  if (!S) return;
  destroy_all(S);
}

puck_status puck_server_submit(puck_server* S, const int32_t* word_ids, const int64_t* offsets, int32_t nsent,
                               const int64_t* arrival_ns, int64_t* ids) {
  if (!S || nsent < 0 || (nsent > 0 && (!word_ids || !offsets || !ids))) {
    puck::set_last_error("puck_server_submit: null argument or negative count");
    return PUCK_ERR_INVALID_ARG;
  }
  const int nlanes = (int)S->lanes.size();
  const int64_t t = now_ns();
  std::lock_guard<std::mutex> lk(S->mu);
  // each sentence to the least-loaded lane, then one submit per lane in order
  std::vector<std::vector<int>> pick(nlanes);
  std::vector<int64_t> cells(nsent);
  for (int i = 0; i < nsent; ++i) {
    const int64_t len = std::max<int64_t>(offsets[i + 1] - offsets[i], 0);
    cells[i] = 2 * tri(len);
    int best = 0;
    for (int k = 1; k < nlanes; ++k)
      if (S->load[k] < S->load[best]) best = k;
    S->load[best] += cells[i];
    pick[best].push_back(i);
  }
  std::vector<int32_t> w;
  std::vector<int64_t> off, arr, lid;
  for (int k = 0; k < nlanes; ++k) {
    if (pick[k].empty()) continue;
    w.clear();
    off.assign(1, 0);
    arr.clear();
    for (int i : pick[k]) {
      w.insert(w.end(), word_ids + offsets[i], word_ids + std::max(offsets[i], offsets[i + 1]));
      off.push_back((int64_t)w.size());
      arr.push_back(arrival_ns && arrival_ns[i] > 0 ? arrival_ns[i] : t);
    }
    lid.assign(pick[k].size(), 0);
    const puck_status st = lane_submit(S->lanes[k], w.data(), off.data(), (int32_t)pick[k].size(), arr.data(),
                                       lid.data());
    if (st != PUCK_OK) return st;
    for (size_t q = 0; q < pick[k].size(); ++q) {
      const int64_t id = lid[q] * nlanes + k;
      ids[pick[k][q]] = id;
      S->cells_of[id] = cells[pick[k][q]];
    }
  }
  return PUCK_OK;
}

int32_t puck_server_poll(puck_server* S, int64_t* ids, int32_t max_ids, int32_t wait_ms) {
  if (!S || !ids || max_ids <= 0) return 0;
  const int nlanes = (int)S->lanes.size();
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(std::max(wait_ms, 0));
  for (;;) {
    int32_t k = 0;
    for (int l = 0; l < nlanes && k < max_ids; ++l) {
      const int32_t got = lane_poll(S->lanes[l], ids + k, max_ids - k, 0);
      for (int32_t q = k; q < k + got; ++q) ids[q] = ids[q] * nlanes + l;
      k += got;
    }
    if (k > 0 || std::chrono::steady_clock::now() >= deadline) return k;
    // a lane notifies `done` when it finishes a request; the short timeout
    // covers a notification between the polls above and this wait
    std::unique_lock<std::mutex> lk(S->mu);
    S->done.wait_until(lk, std::min(deadline, std::chrono::steady_clock::now() + std::chrono::milliseconds(1)));
  }
}

puck_status puck_server_take(puck_server* S, int64_t id, puck_tree_node* nodes, int32_t max_nodes,
                             int32_t* sent_status, int64_t* latency_ns) {
  if (!S || id < 0) {
    puck::set_last_error("puck_server_take: no finished request with this id");
    return PUCK_ERR_INVALID_ARG;
  }
  const int nlanes = (int)S->lanes.size();
  const int l = (int)(id % nlanes);
  const puck_status st = lane_take(S->lanes[l], id / nlanes, nodes, max_nodes, sent_status, latency_ns);
  if (st == PUCK_OK) {
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->cells_of.find(id);
    if (it != S->cells_of.end()) {
      S->load[l] -= it->second;
      S->cells_of.erase(it);
    }
  }
  return st;
}

puck_status puck_server_get_stats(const puck_server* S, puck_server_stats* out) {
  if (!S || !out) return PUCK_ERR_INVALID_ARG;
  puck_server_stats sum{};
  for (const Lane* L : S->lanes) {
    const puck_server_stats s = lane_stats(L);
    sum.submitted += s.submitted;
    sum.completed += s.completed;
    sum.failed += s.failed;
    sum.ticks += s.ticks;
    sum.kernel_launches += s.kernel_launches;
    sum.resident += s.resident;
    sum.resident_peak += s.resident_peak;
    sum.arena_cells += s.arena_cells;
    sum.arena_cells_peak += s.arena_cells_peak;
    sum.ms_device += s.ms_device;
    sum.h2d_bytes += s.h2d_bytes;
    sum.d2h_bytes += s.d2h_bytes;
  }
  *out = sum;
  return PUCK_OK;
}

puck_status puck_server_pass_ms(const puck_server* S, int32_t level, double out[5]) {
  if (!S || !out || level < 0 || level >= S->nl) return PUCK_ERR_INVALID_ARG;
  for (int k = 0; k < 5; ++k) out[k] = 0.0;
  for (const Lane* L : S->lanes) lane_pass_ms(L, level, out);
  return PUCK_OK;
}

int32_t puck_server_lanes(const puck_server* S) { return S ? (int32_t)S->lanes.size() : 0; }

}  // extern "C"
