// Host runtime of libpuck_gb300: grammar.grz loading, device tables, sentence
// batching, the coarse-to-fine pass sequence and the C ABI of puck_gpu.h.
//
// Orchestration follows the reference's CLParser (dlwh/puck,
// src/main/scala/puck/parser/CLParser.scala):
//   parse      = masks from every coarse level, then the last level decodes (:50-53, :145-169)
//   coarse     = inside, outside, masks at the prune threshold, scales if the next level is Real (:208-250)
//   partitions = inside of the last level, root scores (:189-206)
// Batching packs sentences in input order until the chart budget is used
// (WorkSpace.getBatches, src/main/scala/puck/parser/WorkSpace.scala:20-41);
// results do not depend on how sentences are batched.

#include "host_runtime.h"

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <numeric>
#include <string>
#include <unordered_map>
#include <vector>

using namespace puck_host;

namespace {

thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }


// ---------------------------------------------------------------------------
// Minimal reader for zip archives with stored (uncompressed) entries.
struct ZipReader {
  std::vector<unsigned char> data;
  std::map<std::string, std::pair<size_t, size_t>> entries;  // name -> (offset, size)

  static uint32_t u32(const unsigned char* p) { return p[0] | (p[1] << 8) | (p[2] << 16) | ((uint32_t)p[3] << 24); }
  static uint16_t u16(const unsigned char* p) { return (uint16_t)(p[0] | (p[1] << 8)); }

  void open(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "cannot open " + path};
    data.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    if (data.size() < 22) throw PuckError{PUCK_ERR_BAD_GRAMMAR, path + ": not a zip archive"};
    size_t eocd = std::string::npos;
    for (size_t i = data.size() - 22 + 1; i-- > 0 && data.size() - i <= 22 + 65535;) {
      if (u32(&data[i]) == 0x06054b50u) { eocd = i; break; }
    }
    if (eocd == std::string::npos) throw PuckError{PUCK_ERR_BAD_GRAMMAR, path + ": no end of central directory"};
    const size_t n = u16(&data[eocd + 10]);
    size_t cd = u32(&data[eocd + 16]);
    for (size_t k = 0; k < n; ++k) {
      if (cd + 46 > data.size() || u32(&data[cd]) != 0x02014b50u)
        throw PuckError{PUCK_ERR_BAD_GRAMMAR, path + ": corrupt central directory"};
      const uint16_t method = u16(&data[cd + 10]);
      const uint32_t csize = u32(&data[cd + 20]);
      const uint16_t nl = u16(&data[cd + 28]), xl = u16(&data[cd + 30]), cl = u16(&data[cd + 32]);
      const size_t lho = u32(&data[cd + 42]);
      if (cd + 46 + nl > data.size()) throw PuckError{PUCK_ERR_BAD_GRAMMAR, path + ": corrupt central directory"};
      std::string name(reinterpret_cast<const char*>(&data[cd + 46]), nl);
      cd += 46 + nl + xl + cl;
      if (name.size() >= 8 && name.compare(name.size() - 8, 8, ".program") == 0) continue;  // never decoded
      if (method != 0)
        throw PuckError{PUCK_ERR_BAD_GRAMMAR, path + ": entry " + name + " is compressed (not a puck_gb300 artifact)"};
      if (csize == 0xffffffffu || lho == 0xffffffffu)
        throw PuckError{PUCK_ERR_BAD_GRAMMAR, path + ": zip64 entries are not supported"};
      if (lho + 30 > data.size() || u32(&data[lho]) != 0x04034b50u)
        throw PuckError{PUCK_ERR_BAD_GRAMMAR, path + ": corrupt local header"};
      const size_t start = lho + 30 + u16(&data[lho + 26]) + u16(&data[lho + 28]);
      if (start + csize > data.size()) throw PuckError{PUCK_ERR_BAD_GRAMMAR, path + ": truncated entry " + name};
      entries[name] = {start, csize};
    }
  }
  bool has(const std::string& name) const { return entries.count(name) != 0; }
  std::string text(const std::string& name) const {
    auto it = entries.find(name);
    if (it == entries.end()) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "missing entry " + name};
    return std::string(reinterpret_cast<const char*>(&data[it->second.first]), it->second.second);
  }
};


std::vector<std::string> split_lines(const std::string& s) {
  std::vector<std::string> out;
  size_t i = 0;
  while (i <= s.size()) {
    size_t j = s.find('\n', i);
    if (j == std::string::npos) j = s.size();
    out.push_back(s.substr(i, j - i));
    i = j + 1;
  }
  return out;
}

}  // namespace

void puck::set_last_error(const char* msg) { set_error(msg); }


namespace {

const char* kJobNames[puck::NJOBS] = {"in_NN", "in_NT", "in_TN", "in_TT", "out_L_NN", "out_R_NN",
                                      "out_L_NT", "out_R_NT", "out_L_TN", "out_R_TN", "out_L_TT", "out_R_TT"};
const char* kUJobNames[puck::NUJOBS] = {"in_NU", "in_TU", "out_NU", "out_TU"};

// Checks every array the device passes read: presence, dtype, sizes and
// index ranges (the kernels index shared memory with these values).
void validate_level(const HostLevel& L) {
  auto need = [&](const std::string& n, const char* tag, int64_t count) {
    int64_t c = 0;
    L.get<char>(n, tag, &c);
    if (count >= 0 && c != count) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "wrong size for " + n};
    return c;
  };
  auto range = [&](const std::string& n, int64_t hi) {
    int64_t c = 0;
    const int* v = L.get<int>(n, "i4", &c);
    for (int64_t k = 0; k < c; ++k)
      if (v[k] < 0 || v[k] >= hi) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "index out of range in " + n};
  };
  // offset tables the device walks: 0 first, never decreasing, ending at the
  // element count of the table they index
  auto offsets = [&](const std::string& n, int64_t last) {
    int64_t c = 0;
    if (L.arrays.at(n).tag[1] == '8') {
      const long long* v = L.get<long long>(n, "i8", &c);
      for (int64_t k = 0; k < c; ++k)
        if ((k == 0 && v[0] != 0) || (k > 0 && v[k] < v[k - 1]) || (k == c - 1 && v[k] != last))
          throw PuckError{PUCK_ERR_BAD_GRAMMAR, "bad offsets in " + n};
    } else {
      const int* v = L.get<int>(n, "i4", &c);
      for (int64_t k = 0; k < c; ++k)
        if ((k == 0 && v[0] != 0) || (k > 0 && v[k] < v[k - 1]) || (k == c - 1 && v[k] != last))
          throw PuckError{PUCK_ERR_BAD_GRAMMAR, "bad offsets in " + n};
    }
  };
  // weights: any value but NaN (-inf is a legal log weight)
  auto no_nan = [&](const std::string& n) {
    int64_t c = 0;
    const float* v = L.get<float>(n, "f4", &c);
    for (int64_t k = 0; k < c; ++k)
      if (std::isnan(v[k])) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "NaN weight in " + n};
  };
  need("nt_coarse", "i4", L.n_nt);
  need("t_coarse", "i4", L.n_t);
  range("nt_coarse", L.n_coarse);
  range("t_coarse", L.n_coarse);
  if (L.root < 0 || L.root >= L.n_nt) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "root out of range"};
  // coarse member lists first: the pair-table checks below read them
  need("nt_mem_off", "i4", L.n_coarse + 1);
  need("t_mem_off", "i4", L.n_coarse + 1);
  offsets("nt_mem_off", L.n_nt);
  offsets("t_mem_off", L.n_t);
  static const bool tgt_t[puck::NJOBS] = {false, false, false, false, false, false, false, true, true, false, true, true};
  static const bool a_t[puck::NJOBS] = {false, false, true, true, false, false, false, false, false, true, false, true};
  static const bool b_t[puck::NJOBS] = {false, true, false, true, false, false, true, false, false, false, true, false};
  for (int j = 0; j < puck::NJOBS; ++j) {
    const std::string n = kJobNames[j];
    const int ntgt = tgt_t[j] ? L.n_t : L.n_nt;
    const int64_t nr = need(n + "/rowptr", "i4", ntgt + 1);
    const int* rp = L.get<int>(n + "/rowptr", "i4", nullptr);
    const int64_t nab = need(n + "/ab", "i4", -1);
    need(n + "/w", "f4", nab);
    if (rp[0] != 0 || rp[nr - 1] != nab) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "bad rowptr for " + n};
    for (int64_t k = 0; k + 1 < nr; ++k)
      if (rp[k + 1] < rp[k]) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "bad rowptr for " + n};
    no_nan(n + "/w");
    const int* ab = L.get<int>(n + "/ab", "i4", nullptr);
    const int amax = a_t[j] ? L.n_t : L.n_nt, bmax = b_t[j] ? L.n_t : L.n_nt;
    for (int64_t k = 0; k < nab; ++k) {
      const int a = ab[k] & 0xffff, b = (int)((unsigned)ab[k] >> 16);
      if (a >= amax || b >= bmax) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "rule index out of range in " + n};
    }
    const int64_t nbits = need(n + "/seg_bits", "i4", -1);
    if (L.mask_size <= 0 || nbits % L.mask_size) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "bad seg_bits for " + n};
    need(n + "/tgt_seg", "i4", ntgt);
    need(n + "/pair_mode", "i4", 1);
    {
      const int64_t npk = need(n + "/pair_key", "i4", -1);
      need(n + "/pair_gate", "i4", npk * L.mask_size);
      const int64_t npb = need(n + "/pair_blk", "i4", npk + 1);
      const int64_t nbs = need(n + "/blk_seg", "i4", -1);
      const int64_t nbp = need(n + "/blk_ptr", "i4", nbs + 1);
      const int64_t npr = need(n + "/pair_rule", "i4", nab);
      need(n + "/pair_w", "f4", nab);
      no_nan(n + "/pair_w");
      // whole tables before the walk below indexes with them
      offsets(n + "/pair_blk", nbs);
      offsets(n + "/blk_ptr", npr);
      const int* pk = L.get<int>(n + "/pair_key", "i4", nullptr);
      const int* pb = L.get<int>(n + "/pair_blk", "i4", nullptr);
      const int* bs = L.get<int>(n + "/blk_seg", "i4", nullptr);
      const int* bp = L.get<int>(n + "/blk_ptr", "i4", nullptr);
      const int* pr = L.get<int>(n + "/pair_rule", "i4", nullptr);
      const int* ao = L.get<int>(a_t[j] ? "t_mem_off" : "nt_mem_off", "i4", nullptr);
      const int* bo = L.get<int>(b_t[j] ? "t_mem_off" : "nt_mem_off", "i4", nullptr);
      if (pb[0] != 0 || pb[npb - 1] != nbs || bp[0] != 0 || bp[nbp - 1] != npr)
        throw PuckError{PUCK_ERR_BAD_GRAMMAR, "bad pair tables for " + n};
      for (int64_t k = 0; k < npk; ++k) {
        const int ca = pk[k] & 255, cb = (pk[k] >> 8) & 255;
        if (ca >= L.n_coarse || cb >= L.n_coarse || pb[k + 1] < pb[k])
          throw PuckError{PUCK_ERR_BAD_GRAMMAR, "bad pair key for " + n};
        const int ny = ao[ca + 1] - ao[ca], nz = bo[cb + 1] - bo[cb];
        if (ny > 255 || nz > 255) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "coarse symbol with more than 255 members"};
        for (int b = pb[k]; b < pb[k + 1]; ++b) {
          if (bs[b] < 0 || bs[b] >= nbits / std::max(1, L.mask_size) || bp[b + 1] < bp[b])
            throw PuckError{PUCK_ERR_BAD_GRAMMAR, "bad block for " + n};
          for (int r = bp[b]; r < bp[b + 1]; ++r) {
            const int jj = pr[r] & 255, kk = (pr[r] >> 8) & 255, tt = (int)((unsigned)pr[r] >> 16);
            if (jj >= ny || kk >= nz || tt >= ntgt) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "pair rule out of range in " + n};
          }
        }
      }
    }
    int64_t c = 0;
    const int* ts = L.get<int>(n + "/tgt_seg", "i4", &c);
    for (int64_t k = 0; k < c; ++k)
      if (ts[k] < -1 || ts[k] >= nbits / L.mask_size) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "bad tgt_seg in " + n};
  }
  static const bool ut[puck::NUJOBS] = {false, false, false, true};
  static const bool us[puck::NUJOBS] = {false, true, false, false};
  for (int j = 0; j < puck::NUJOBS; ++j) {
    const std::string n = kUJobNames[j];
    const int64_t nr = need(n + "/rowptr", "i4", (ut[j] ? L.n_t : L.n_nt) + 1);
    const int* rp = L.get<int>(n + "/rowptr", "i4", nullptr);
    const int64_t ns = need(n + "/src", "i4", rp[nr - 1]);
    offsets(n + "/rowptr", ns);
    need(n + "/w", "f4", ns);
    no_nan(n + "/w");
    range(n + "/src", us[j] ? L.n_t : L.n_nt);
  }
  need("nt_mem", "i4", L.n_nt);
  need("t_mem", "i4", L.n_t);
  range("nt_mem", L.n_nt);
  range("t_mem", L.n_t);
  const int64_t nlo = need("lex_off", "i8", L.n_words + 1);
  const long long* lo = L.get<long long>("lex_off", "i8", nullptr);
  need("lex_term", "i4", lo[nlo - 1]);
  need("lex_score", "f4", lo[nlo - 1]);
  offsets("lex_off", lo[nlo - 1]);
  no_nan("lex_score");
  range("lex_term", L.n_t);
  const int64_t nvo = need("v_off", "i4", 6LL * L.n_nt + 1);
  const int* vo = L.get<int>("v_off", "i4", nullptr);
  need("v_left", "i4", vo[nvo - 1]);
  need("v_score", "f4", vo[nvo - 1]);
  need("v_right", "i4", vo[nvo - 1]);
  offsets("v_off", vo[nvo - 1]);
  no_nan("v_score");
  range("v_left", std::max(L.n_nt, L.n_t));
  range("v_right", std::max(L.n_nt, L.n_t));
}

void load_grammar(puck_grammar* g, const std::string& path) {
  ZipReader z;
  z.open(path);
  std::vector<std::string> names;
  for (auto& l : split_lines(z.text("parserNames")))
    if (!l.empty()) names.push_back(l);
  if (names.empty()) throw PuckError{PUCK_ERR_BAD_GRAMMAR, path + ": no levels"};
  for (auto& n : names) {
    if (!z.has(n + "/header"))
      throw PuckError{PUCK_ERR_BAD_GRAMMAR, path + ": level " + n +
                                                " has no header (reference archives with serialised objects are not decoded)"};
    HostLevel L;
    std::map<std::string, std::string> hdr;
    for (auto& line : split_lines(z.text(n + "/header"))) {
      size_t sp = line.find(' ');
      if (sp != std::string::npos) hdr[line.substr(0, sp)] = line.substr(sp + 1);
    }
    auto geti = [&](const char* k) {
      auto it = hdr.find(k);
      if (it == hdr.end()) throw PuckError{PUCK_ERR_BAD_GRAMMAR, std::string("header lacks ") + k};
      return std::stoi(it->second);
    };
    const std::string sr = hdr["semiring"];
    L.semiring = sr == "viterbi" ? 0 : sr == "real" ? 1 : sr == "logsum" ? 2 : -1;
    if (L.semiring < 0) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "unknown semiring " + sr};
    L.n_nt = geti("n_nt");
    L.n_t = geti("n_t");
    L.cell_size = geti("cell_size");
    L.mask_size = geti("mask_size");
    L.n_coarse = geti("n_coarse");
    L.root = geti("root");
    L.n_words = geti("n_words");
    if (L.mask_size > puck::kMaxMask || L.n_coarse > puck::kMaxCoarse)
      throw PuckError{PUCK_ERR_BAD_GRAMMAR, "too many coarse symbols"};
    // every coarse id needs a bit in a cell's mask words
    if (L.n_coarse < 1 || L.mask_size < 1 || L.n_coarse > 32 * L.mask_size)
      throw PuckError{PUCK_ERR_BAD_GRAMMAR, "mask size does not cover the coarse symbols"};
    if (L.cell_size % 32 != 0 || L.cell_size < std::max(L.n_nt, L.n_t))
      throw PuckError{PUCK_ERR_BAD_GRAMMAR, "bad cell size"};
    if (std::max(L.n_nt, L.n_t) > 65535) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "more than 65535 symbols"};
    const std::string pre = n + "/arrays/";
    for (auto& e : z.entries) {
      if (e.first.compare(0, pre.size(), pre) != 0) continue;
      const unsigned char* p = &z.data[e.second.first];
      if (e.second.second < 16 || std::memcmp(p, "PKA1", 4) != 0)
        throw PuckError{PUCK_ERR_BAD_GRAMMAR, "bad array entry " + e.first};
      Array a;
      std::memcpy(a.tag, p + 4, 4);
      std::memcpy(&a.count, p + 8, 8);
      size_t esz = (std::strncmp(a.tag, "i8", 2) == 0) ? 8 : 4;
      // the count comes from the file: bound it before any arithmetic on it
      if (a.count < 0 || (uint64_t)a.count > (e.second.second - 16) / esz)
        throw PuckError{PUCK_ERR_BAD_GRAMMAR, "truncated " + e.first};
      a.bytes.assign(p + 16, p + 16 + a.count * esz);
      L.arrays[e.first.substr(pre.size())] = std::move(a);
    }
    L.words = split_lines(z.text(n + "/words.txt"));
    if ((int)L.words.size() != L.n_words) {
      if (!(L.n_words == 0 && L.words.size() == 1)) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "word list size mismatch"};
      L.words.clear();
    }
    validate_level(L);
    g->levels.push_back(std::move(L));
  }
  const HostLevel& fine = g->levels.back();
  for (size_t i = 0; i < fine.words.size(); ++i) g->word_index.emplace(fine.words[i], (int)i);
  for (auto& L : g->levels)
    if (L.mask_size != g->levels.back().mask_size)
      throw PuckError{PUCK_ERR_BAD_GRAMMAR, "cascade levels disagree on the coarse symbol set"};
}

// ---------------------------------------------------------------------------


template <class T>
const T* up(LevelDev& D, const HostLevel& L, const std::string& name, const char* tag, int64_t* count = nullptr) {
  int64_t c = 0;
  const T* h = L.get<T>(name, tag, &c);
  if (count) *count = c;
  return reinterpret_cast<const T*>(D.upload(h, c * sizeof(T)));
}

// The flat-tile layout of a Viterbi inside job (DevJob::pair_desc, fr_*),
// built when every pair's operand members are contiguous index ranges.  A
// pair whose coarse symbols have more than 16 members on a side is cut into
// sub-tiles of at most 16 x 16 (16 members, then the rest): each sub-tile is
// a pair of its own, with the same coarse key (its liveness test), the rules
// whose two operands fall inside it and the OR of its blocks' segment bits
// as its gate.  A block with more than 32 targets is cut into runs of 32
// targets.  Each target of a block gets lanes in proportion to its rule
// count (at least one); a lane's slice is stored as records of four rules,
// padded with weight pad_w (the semiring's zero: -inf for max-plus, 0 for the
// sum-product, which the kernel skips), which never changes a cell.
// The sub-tiles form the layout's own pair list (fnpair, fpair_key,
// fpair_gate).  *mtile receives the largest sub-tile.  Returns false, uploading
// nothing, when the job does not qualify.
// ao/am and bo/bm: CSR from pair key to the operands' members (in the
// operand roles' index spaces) for the left and right operands.
struct FlatHost {
  std::vector<int4> desc, blk;
  std::vector<int> key, gate, tgt;
  std::vector<unsigned> idx;
  std::vector<float4> w;
  int max_tile = 1;
};

bool flat_tiles_host(FlatHost& F, int ntgt, int64_t npk, const int* pk, const int* pbk, const int* bs, const int* bp,
                     const int* pr, const float* pw, const int* seg_bits, int nseg, int ms, const int* ao,
                     const int* am, const int* bo, const int* bm, float pad_w) {
  constexpr int kSub = 16;  // largest sub-tile side
  auto contiguous = [](const int* off, const int* mem, int c) {
    for (int i = off[c]; i < off[c + 1]; ++i)
      if (mem[i] != mem[off[c]] + (i - off[c])) return false;
    return true;
  };
  struct FlatRule {
    int t, e;
    float w;
  };
  std::vector<int4>& desc = F.desc;
  std::vector<int4>& blk = F.blk;
  std::vector<int>& key = F.key;
  std::vector<int>& gate = F.gate;
  std::vector<int>& tgt = F.tgt;
  std::vector<unsigned>& idx = F.idx;
  std::vector<float4>& w = F.w;
  int& max_tile = F.max_tile;
  // One block of a sub-tile: rules sorted by target, at most 32 targets.
  auto emit_block = [&](int seg, const std::vector<FlatRule>& rs, int tile) -> bool {
    const int cnt = (int)rs.size();
    const size_t b = blk.size();
    tgt.resize((b + 1) * 32, -1);
    std::vector<int> tstart, tcnt, tlanes;
    for (int r = 0; r < cnt; ++r)
      if (r == 0 || rs[r].t != rs[r - 1].t) tstart.push_back(r);
    if (tstart.size() > 32) return false;
    for (size_t t = 0; t < tstart.size(); ++t) tcnt.push_back((t + 1 < tstart.size() ? tstart[t + 1] : cnt) - tstart[t]);
    tlanes.assign(tstart.size(), 1);
    auto slice = [&](size_t t) { return (tcnt[t] + tlanes[t] - 1) / tlanes[t]; };
    for (int free_lanes = 32 - (int)tstart.size(); free_lanes > 0 && !tstart.empty(); --free_lanes) {
      size_t best = 0;
      for (size_t t = 1; t < tstart.size(); ++t)
        if (slice(t) > slice(best)) best = t;
      if (slice(best) <= 1) break;
      ++tlanes[best];
    }
    int per = 0;
    for (size_t t = 0; t < tstart.size(); ++t) per = std::max(per, slice(t));
    const int steps = (per + 3) / 4, slots = 4 * steps;
    // each lane's rules (tile entry, weight), in any order: max is commutative
    std::vector<std::vector<std::pair<int, float>>> todo(32);
    int lane = 0;
    for (size_t t = 0; t < tstart.size(); ++t) {
      const int len = slice(t);
      for (int l = 0; l < tlanes[t]; ++l, ++lane) {
        const int a0 = tstart[t] + l * len, a1 = std::min(tstart[t] + tcnt[t], a0 + len);
        tgt[b * 32 + lane] = rs[tstart[t]].t;
        for (int r = a0; r < a1; ++r) todo[lane].push_back({rs[r].e, rs[r].w});
      }
    }
    // Each slot (one of the four loads of a record) is one warp-wide shared
    // load of M: its 32 tile entries should fall in distinct banks (e mod
    // 32), or read the same entry.  Slot by slot, lanes that must take a
    // rule now (as many rules left as slots) pick first; the others take a
    // rule only in a bank still free.  A lane without a rule this slot
    // reads an entry already read by the slot (weight -inf).
    const size_t base = idx.size();
    idx.resize(base + (size_t)steps * 32, 0u);
    w.resize(base + (size_t)steps * 32, make_float4(pad_w, pad_w, pad_w, pad_w));
    for (int sl = 0; sl < slots; ++sl) {
      int bank_e[32];
      std::fill(bank_e, bank_e + 32, -1);
      int pick[32];
      std::fill(pick, pick + 32, -1);
      auto choose = [&](int l, bool forced) {
        auto& v = todo[l];
        int best = -1;
        for (size_t r = 0; r < v.size(); ++r) {
          const int e = v[r].first, bk = e & 31;
          if (bank_e[bk] < 0 || bank_e[bk] == e) {
            best = (int)r;
            break;
          }
        }
        if (best < 0 && forced) best = 0;
        if (best < 0) return;
        pick[l] = best;
        const int e = v[best].first;
        if (bank_e[e & 31] < 0) bank_e[e & 31] = e;
      };
      for (int l = 0; l < 32; ++l)
        if (!todo[l].empty() && (int)todo[l].size() >= slots - sl) choose(l, true);
      for (int l = 0; l < 32; ++l)
        if (pick[l] < 0 && !todo[l].empty() && (int)todo[l].size() < slots - sl) choose(l, false);
      int any_e = 0;
      for (int k = 0; k < 32; ++k)
        if (bank_e[k] >= 0) {
          any_e = bank_e[k];
          break;
        }
      for (int l = 0; l < 32; ++l) {
        const size_t at = base + (size_t)(sl / 4) * 32 + l;
        int e = any_e;
        float wt = pad_w;
        if (pick[l] >= 0) {
          e = todo[l][pick[l]].first;
          wt = todo[l][pick[l]].second;
          todo[l].erase(todo[l].begin() + pick[l]);
        }
        idx[at] |= (unsigned)e << (8 * (sl % 4));
        (&w[at].x)[sl % 4] = wt;
      }
    }
    for (int l = 0; l < 32; ++l)
      if (!todo[l].empty()) return false;  // cannot happen: every lane has slots for all its rules
    // every tile entry inside the sub-tile (a byte each), every target below
    // the job's target count
    for (size_t q = base; q < idx.size(); ++q)
      for (int c = 0; c < 4; ++c)
        if ((int)((idx[q] >> (8 * c)) & 255u) >= tile) return false;
    for (int l = 0; l < 32; ++l)
      if (tgt[b * 32 + l] >= ntgt) return false;
    if (idx.size() > (size_t)INT32_MAX) return false;
    blk.push_back(make_int4(seg, (int)base, (int)idx.size(), cnt));
    return true;
  };
  std::vector<FlatRule> rs;
  std::vector<unsigned> g(std::max(ms, 1));
  for (int64_t k = 0; k < npk; ++k) {
    const int ca = pk[k] & 255, cb = (pk[k] >> 8) & 255;
    const int ny = ao[ca + 1] - ao[ca], nz = bo[cb + 1] - bo[cb];
    if (ny < 1 || nz < 1 || ny > 255 || nz > 255 || !contiguous(ao, am, ca) || !contiguous(bo, bm, cb)) return false;
    for (int y0 = 0; y0 < ny; y0 += kSub)
      for (int z0 = 0; z0 < nz; z0 += kSub) {
        const int sy = std::min(kSub, ny - y0), sz = std::min(kSub, nz - z0);
        const int a_first = am[ao[ca]] + y0, b_first = bm[bo[cb]] + z0;
        if (a_first > 0xffff || b_first > 0xffff) return false;
        const int b_first_blk = (int)blk.size();
        std::fill(g.begin(), g.end(), 0u);
        for (int b = pbk[k]; b < pbk[k + 1]; ++b) {
          if (bs[b] < 0 || bs[b] >= nseg) return false;
          // the block's rules inside this sub-tile, in target order
          rs.clear();
          for (int r = bp[b]; r < bp[b + 1]; ++r) {
            const unsigned x = (unsigned)pr[r];
            const int jj = (int)(x & 255u) - y0, kk = (int)((x >> 8) & 255u) - z0;
            if (jj >= 0 && jj < sy && kk >= 0 && kk < sz) rs.push_back({(int)(x >> 16), jj * sz + kk, pw[r]});
          }
          if (rs.empty()) continue;
          for (int i = 0; i < ms; ++i) g[i] |= (unsigned)seg_bits[(size_t)bs[b] * ms + i];
          // runs of at most 32 targets
          size_t r0 = 0;
          while (r0 < rs.size()) {
            size_t r1 = r0;
            int ntg = 0;
            while (r1 < rs.size() && (ntg < 32 || rs[r1].t == rs[r1 - 1].t)) {
              if (r1 == r0 || rs[r1].t != rs[r1 - 1].t) ++ntg;
              ++r1;
            }
            if (!emit_block(bs[b], std::vector<FlatRule>(rs.begin() + r0, rs.begin() + r1), sy * sz)) return false;
            r0 = r1;
          }
        }
        const int nb = (int)blk.size() - b_first_blk;
        if (nb == 0) continue;
        if (nb > 0xffff) return false;
        desc.push_back(make_int4(a_first | b_first << 16, b_first_blk, sy | sz << 8 | nb << 16, ca | cb << 8));
        key.push_back(ca | cb << 8);
        for (int i = 0; i < ms; ++i) gate.push_back((int)g[i]);
        max_tile = std::max(max_tile, sy * sz);
      }
  }
  return desc.size() <= (size_t)INT32_MAX / 32;
}

// Uploads the flat-tile tables of a job (DevJob::flat).
void upload_flat(LevelDev& D, puck::DevJob& J, FlatHost& F, int ms, float pad_w, int* mtile) {
  std::vector<int4>& desc = F.desc;
  std::vector<int4>& blk = F.blk;
  std::vector<int>& key = F.key;
  std::vector<int>& gate = F.gate;
  std::vector<int>& tgt = F.tgt;
  std::vector<unsigned>& idx = F.idx;
  std::vector<float4>& w = F.w;
  J.fnpair = (int)desc.size();
  if (desc.empty()) desc.push_back(make_int4(0, 0, 0, 0));  // a job without rules still gets (never read) tables
  if (key.empty()) key.push_back(0);
  if (gate.empty()) gate.assign(std::max(ms, 1), 0);
  if (blk.empty()) blk.push_back(make_int4(0, 0, 0, 0));
  if (tgt.empty()) tgt.assign(32, -1);
  if (idx.empty()) {
    idx.push_back(0u);
    w.push_back(make_float4(pad_w, pad_w, pad_w, pad_w));
  }
  J.fpair_key = static_cast<const int*>(D.upload(key.data(), key.size() * sizeof(int)));
  J.fpair_gate = static_cast<const int*>(D.upload(gate.data(), gate.size() * sizeof(int)));
  J.flat = 1;
  J.pair_desc = static_cast<const int4*>(D.upload(desc.data(), desc.size() * sizeof(int4)));
  J.fr_blk = static_cast<const int4*>(D.upload(blk.data(), blk.size() * sizeof(int4)));
  J.fr_tgt = static_cast<const int*>(D.upload(tgt.data(), tgt.size() * sizeof(int)));
  J.fr_idx = static_cast<const unsigned*>(D.upload(idx.data(), idx.size() * sizeof(unsigned)));
  J.fr_w = static_cast<const float4*>(D.upload(w.data(), w.size() * sizeof(float4)));
  *mtile = std::max(*mtile, F.max_tile);
}

bool build_flat_tiles(LevelDev& D, puck::DevJob& J, int ntgt, int64_t npk, const int* pk, const int* pbk,
                      const int* bs, const int* bp, const int* pr, const float* pw, const int* seg_bits, int nseg,
                      int ms, const int* ao, const int* am, const int* bo, const int* bm, float pad_w, int* mtile) {
  FlatHost F;
  if (!flat_tiles_host(F, ntgt, npk, pk, pbk, bs, bp, pr, pw, seg_bits, nseg, ms, ao, am, bo, bm, pad_w)) return false;
  upload_flat(D, J, F, ms, pad_w, mtile);
  return true;
}

// Flat-tile tables over groups of coarse ids for a target-major Viterbi
// level whose coarse map rises strictly along each role's symbols (the top
// level of a cascade: one symbol per coarse id).  Group g holds the symbols
// of coarse ids 16g .. 16g + 15, a contiguous run of at most 16 symbols per
// role, so every pair of groups is one flat tile.  Rules come from the
// job's target-major table, grouped by (group of a, group of b), then by
// segment and target.  Returns false, uploading nothing, when the level's
// coarse maps do not rise strictly.
// A job's segment bits as its per-pair gates see them.  On a merged level (a
// middle level of a cascade, the only merged level that receives masks) the
// reference runs every rule as one block gated by segment 0's bits
// (CLParser.scala:783-785), so every segment takes segment 0's row and a
// pair's gate becomes that row: all of the level's pairs pass or none do.
std::vector<int> gate_seg_bits(const HostLevel& L, const std::string& n, bool merged) {
  int64_t c = 0;
  const int* sb = L.get<int>(n + "/seg_bits", "i4", &c);
  std::vector<int> out(sb, sb + c);
  if (merged)
    for (int64_t k = L.mask_size; k < c; ++k) out[k] = sb[k % L.mask_size];
  return out;
}

bool group_tiles_host(FlatHost& F, const HostLevel& L, int j, int nseg, bool merged) {
  static const bool a_t[4] = {false, false, true, true};
  static const bool b_t[4] = {false, true, false, true};
  const std::string n = kJobNames[j];
  const int* ntc = L.get<int>("nt_coarse", "i4", nullptr);
  const int* tc = L.get<int>("t_coarse", "i4", nullptr);
  // CSR from group to its members, per role
  auto groups = [&](const int* coarse, int nsym, std::vector<int>& off, std::vector<int>& mem) {
    const int ng = (L.n_coarse + 15) / 16;
    off.assign(ng + 1, 0);
    mem.clear();
    for (int i = 0; i < nsym; ++i) {
      if (i > 0 && coarse[i] <= coarse[i - 1]) return false;
      ++off[coarse[i] / 16 + 1];
      mem.push_back(i);
    }
    for (int g = 0; g < ng; ++g) off[g + 1] += off[g];
    return true;
  };
  std::vector<int> nt_off, nt_mem, t_off, t_mem;
  if (!groups(ntc, L.n_nt, nt_off, nt_mem) || !groups(tc, L.n_t, t_off, t_mem)) return false;
  const std::vector<int>& ao = a_t[j] ? t_off : nt_off;
  const std::vector<int>& am = a_t[j] ? t_mem : nt_mem;
  const std::vector<int>& bo = b_t[j] ? t_off : nt_off;
  const std::vector<int>& bm = b_t[j] ? t_mem : nt_mem;
  const int* ca_of = a_t[j] ? tc : ntc;
  const int* cb_of = b_t[j] ? tc : ntc;
  int64_t nrow = 0, nab = 0;
  const int* rowptr = L.get<int>(n + "/rowptr", "i4", &nrow);
  const int* ab = L.get<int>(n + "/ab", "i4", &nab);
  const float* w = L.get<float>(n + "/w", "f4", nullptr);
  const int* tseg = L.get<int>(n + "/tgt_seg", "i4", nullptr);
  const int ntgt = (int)(nrow - 1);
  struct R {
    int key, seg, t, jk;
    float w;
  };
  std::vector<R> rs;
  rs.reserve(nab);
  for (int t = 0; t < ntgt; ++t)
    for (int r = rowptr[t]; r < rowptr[t + 1]; ++r) {
      const int a = ab[r] & 0xffff, b = (int)((unsigned)ab[r] >> 16);
      const int ga = ca_of[a] / 16, gb = cb_of[b] / 16;
      const int ja = a - am[ao[ga]], kb = b - bm[bo[gb]];
      if (tseg[t] < 0 || ja < 0 || ja >= ao[ga + 1] - ao[ga] || kb < 0 || kb >= bo[gb + 1] - bo[gb]) return false;
      rs.push_back({ga | gb << 8, tseg[t], t, ja | kb << 8, w[r]});
    }
  std::sort(rs.begin(), rs.end(), [](const R& x, const R& y) {
    if (x.key != y.key) return x.key < y.key;
    if (x.seg != y.seg) return x.seg < y.seg;
    if (x.t != y.t) return x.t < y.t;
    return x.jk < y.jk;
  });
  std::vector<int> pk, pbk, bs, bp, pr;
  std::vector<float> pw;
  for (size_t r = 0; r < rs.size(); ++r) {
    const bool new_pair = r == 0 || rs[r].key != rs[r - 1].key;
    if (new_pair) {
      pk.push_back(rs[r].key);
      pbk.push_back((int)bs.size());
    }
    if (new_pair || rs[r].seg != rs[r - 1].seg) {
      bs.push_back(rs[r].seg);
      bp.push_back((int)r);
    }
    pr.push_back(rs[r].jk | rs[r].t << 16);
    pw.push_back(rs[r].w);
  }
  pbk.push_back((int)bs.size());
  bp.push_back((int)rs.size());
  const std::vector<int> gbits = gate_seg_bits(L, n, merged);
  return flat_tiles_host(F, ntgt, (int64_t)pk.size(), pk.data(), pbk.data(), bs.data(), bp.data(), pr.data(),
                         pw.data(), gbits.data(), nseg, L.mask_size, ao.data(), am.data(), bo.data(), bm.data(),
                         -INFINITY);
}

bool build_group_tiles(LevelDev& D, puck::DevJob& J, const HostLevel& L, int j, int* mtile) {
  FlatHost F;
  if (!group_tiles_host(F, L, j, J.nseg, D.d.gate_merged != 0)) return false;
  upload_flat(D, J, F, L.mask_size, -INFINITY, mtile);
  return true;
}

// The unknown-word class of a word, in the scheme of the Berkeley parser's
// English lexicons, whose text grammars list one lexicon entry per class
// (`UNK-INITC-KNOWNLC`, `UNK-LC-s`, `UNK-CAPS-NUM`, ...):
//   "UNK";
//   a capitalisation class: -INITC for a sentence-initial word whose only
//   capital is its first letter (plus -KNOWNLC when its lowercase form is a
//   known word), -CAPS for any other word starting with a capital or for a
//   word with a capital after a non-letter start, -LC for other words with a
//   lowercase letter;
//   -NUM when it has a digit, -DASH when it has a hyphen;
//   one suffix class: -s for a final s after anything but s, i or u in a word
//   of three or more characters; otherwise, for words of five or more
//   characters without a hyphen and without both a digit and a capital, the
//   first of -ed, -ing, -ion, -er, -est, -ly, -ity, -y, -al that ends the
//   lowercased word.
// Letters are ASCII; other bytes count as neither letters nor digits.
std::string unknown_word_class(const std::string& w, int position,
                               const std::unordered_map<std::string, int>& known) {
  int caps = 0;
  bool digit = false, dash = false, lower = false;
  std::string lc(w);
  for (char& c : lc) {
    const unsigned char u = (unsigned char)c;
    if (u >= '0' && u <= '9') digit = true;
    else if (u == '-') dash = true;
    else if (u >= 'a' && u <= 'z') lower = true;
    else if (u >= 'A' && u <= 'Z') {
      ++caps;
      c = (char)(u - 'A' + 'a');
    }
  }
  const unsigned char first = (unsigned char)w[0];
  const bool first_cap = first >= 'A' && first <= 'Z';
  const bool first_letter = first_cap || (first >= 'a' && first <= 'z');
  std::string sig = "UNK";
  if (first_cap) {
    if (position == 0 && caps == 1) {
      sig += "-INITC";
      if (known.count(lc)) sig += "-KNOWNLC";
    } else {
      sig += "-CAPS";
    }
  } else if (!first_letter && caps > 0) {
    sig += "-CAPS";
  } else if (lower) {
    sig += "-LC";
  }
  if (digit) sig += "-NUM";
  if (dash) sig += "-DASH";
  const size_t n = lc.size();
  auto ends = [&](const char* suf) {
    const size_t k = std::strlen(suf);
    return n >= k && lc.compare(n - k, k, suf) == 0;
  };
  if (n >= 3 && lc[n - 1] == 's') {
    const char before = lc[n - 2];
    if (before != 's' && before != 'i' && before != 'u') sig += "-s";
  } else if (n >= 5 && !dash && !(digit && caps > 0)) {
    for (const char* suf : {"ed", "ing", "ion", "er", "est", "ly", "ity", "y", "al"})
      if (ends(suf)) {
        sig += "-";
        sig += suf;
        break;
      }
  }
  return sig;
}

// Pair-major tables of one job (DevJob::pm_*): the job's rules grouped by
// their child pair (a, b), each pair's rules as {target, bits(w)}.  Returns
// false for a job whose targets average more than kPairMajorRules rules
// (the atomic updates of each target would serialise) or that has none.
constexpr int kPairMajorRules = 48;
bool pm_tables_host(const HostLevel& L, int j, std::vector<int>& pab, std::vector<int>& poff,
                    std::vector<int2>& prule) {
  const std::string n = kJobNames[j];
  int64_t nrow = 0;
  const int* rowptr = L.get<int>(n + "/rowptr", "i4", &nrow);
  const int* ab = L.get<int>(n + "/ab", "i4", nullptr);
  const float* w = L.get<float>(n + "/w", "f4", nullptr);
  int with_rules = 0;
  for (int t = 0; t + 1 < nrow; ++t) with_rules += rowptr[t + 1] > rowptr[t];
  if (with_rules == 0 || rowptr[nrow - 1] > (int64_t)kPairMajorRules * with_rules) return false;
  std::vector<std::array<int, 3>> rs;  // (a | b << 16, target, rule)
  for (int t = 0; t + 1 < nrow; ++t)
    for (int r = rowptr[t]; r < rowptr[t + 1]; ++r) rs.push_back({ab[r], t, r});
  std::sort(rs.begin(), rs.end());
  pab.clear();
  poff.clear();
  prule.clear();
  for (size_t i = 0; i < rs.size(); ++i) {
    if (i == 0 || rs[i][0] != rs[i - 1][0]) {
      pab.push_back(rs[i][0]);
      poff.push_back((int)prule.size());
    }
    int2 v;
    v.x = rs[i][1];
    std::memcpy(&v.y, &w[rs[i][2]], 4);
    prule.push_back(v);
  }
  poff.push_back((int)prule.size());
  return true;
}

}  // namespace

void puck_host::build_level(LevelDev& D, const HostLevel& L, bool merged) {
  puck::DevLevel& d = D.d;
  d.semiring = L.semiring;
  d.n_nt = L.n_nt;
  d.n_t = L.n_t;
  d.cell_size = L.cell_size;
  d.mask_size = L.mask_size;
  d.n_coarse = L.n_coarse;
  d.root = L.root;
  d.num_syms = std::max(L.n_nt, L.n_t);
  d.n_words = L.n_words;
  d.gate_merged = merged ? 1 : 0;
  d.nt_coarse = up<int>(D, L, "nt_coarse", "i4");
  d.t_coarse = up<int>(D, L, "t_coarse", "i4");
  for (int j = 0; j < puck::NJOBS; ++j) {
    const std::string n = kJobNames[j];
    int64_t nrow = 0, nab = 0, nw = 0, nseg = 0;
    const int* rowptr_h = L.get<int>(n + "/rowptr", "i4", &nrow);
    const int* ab = L.get<int>(n + "/ab", "i4", &nab);
    const float* w = L.get<float>(n + "/w", "f4", &nw);
    if (nab != nw || nrow < 1 || rowptr_h[nrow - 1] != nab) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "inconsistent job " + n};
    std::vector<int2> packed(nab);
    for (int64_t k = 0; k < nab; ++k) {
      packed[k].x = ab[k];
      std::memcpy(&packed[k].y, &w[k], 4);
    }
    puck::DevJob& J = d.jobs[j];
    J.n_tgt = (int)(nrow - 1);
    J.rowptr = up<int>(D, L, n + "/rowptr", "i4");
    J.rules = reinterpret_cast<const int2*>(D.upload(packed.data(), packed.size() * sizeof(int2)));
    J.tgt_seg = up<int>(D, L, n + "/tgt_seg", "i4");
    J.seg_bits = up<int>(D, L, n + "/seg_bits", "i4", &nseg);
    J.nseg = (int)(nseg / std::max(1, L.mask_size));
    if (J.nseg > puck::kMaxSeg) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "more than 2048 rule segments in " + n};
    static const bool a_t[puck::NJOBS] = {false, false, true, true, false, false, false, false, false, true, false, true};
    static const bool b_t[puck::NJOBS] = {false, true, false, true, false, false, true, false, false, false, true, false};
    int64_t npk = 0, nr = 0, nbp = 0;
    const int* pk = L.get<int>(n + "/pair_key", "i4", &npk);
    const int* pr = L.get<int>(n + "/pair_rule", "i4", &nr);
    const float* pw = L.get<float>(n + "/pair_w", "f4", nullptr);
    const int* bp = L.get<int>(n + "/blk_ptr", "i4", &nbp);
    // Device layout of a block's rules: padded to a multiple of 32 and
    // interleaved, so that lane l's contiguous slice [l*per, (l+1)*per) is
    // read as rules[i*32 + l], i = 0..per-1 (coalesced across the warp).
    // Padding rules carry the semiring zero as weight and the block's last
    // target, so they never change a cell.
    // The device form of a rule is (j * nz + k) | target << 16: the index of
    // its operand pair in the pair's row-major outer-product tile.
    const float zero = L.semiring == puck::SEMI_REAL ? 0.f : -INFINITY;
    const int* pbk = L.get<int>(n + "/pair_blk", "i4", nullptr);
    // nz (and ny) of every block, from the member lists of the operand roles
    // the device uses for this job (DevJob::a_is_t / b_is_t = a_t[j] / b_t[j])
    const int* ao_ = L.get<int>(a_t[j] ? "t_mem_off" : "nt_mem_off", "i4", nullptr);
    const int* bo_ = L.get<int>(b_t[j] ? "t_mem_off" : "nt_mem_off", "i4", nullptr);
    std::vector<int> blk_nz(nbp > 0 ? nbp - 1 : 0, 1), blk_ny(nbp > 0 ? nbp - 1 : 0, 1);
    for (int64_t k = 0; k < npk; ++k) {
      const int ca = pk[k] & 255, cb = (pk[k] >> 8) & 255;
      for (int b = pbk[k]; b < pbk[k + 1]; ++b) {
        blk_nz[b] = bo_[cb + 1] - bo_[cb];
        blk_ny[b] = ao_[ca + 1] - ao_[ca];
      }
    }
    const int ntgt_j = (int)(nrow - 1);
    std::vector<int2> rr;
    std::vector<int> dev_bp(1, 0), blk_n;
    // Outside jobs and sum-product levels keep the archive's layout: blocks
    // back to back, rule form j | k << 8 | target << 16.  (The batched,
    // interleaved form faulted the GPU in those kernels; the cause is not
    // known, so they run the earlier, verified form.)
    const bool interleave = L.semiring == puck::SEMI_VITERBI && j < 4;  // Viterbi inside jobs
    if (!interleave) {
      rr.resize(nbp > 0 ? bp[nbp - 1] : 0);
      for (size_t k = 0; k < rr.size(); ++k) {
        rr[k].x = pr[k];
        std::memcpy(&rr[k].y, &pw[k], 4);
      }
      dev_bp.assign(bp, bp + nbp);
      for (int64_t b = 0; b + 1 < nbp; ++b) blk_n.push_back(bp[b + 1] - bp[b]);
    }
    // Viterbi inside jobs: each lane's slice holds rules of one target only
    // (per-target lanes), so the kernel keeps one running max per lane and
    // flushes it once.  A target gets lanes in proportion to its rules; the
    // slice length is padded to a multiple of four.  Blocks with more than 32
    // targets keep mixed slices (the job then uses the run-tracking loop).
    bool one_target_lanes = interleave;
    for (int64_t b = 0; one_target_lanes && b + 1 < nbp; ++b) {
      int ntg = 0;
      for (int r = bp[b]; r < bp[b + 1]; ++r)
        ntg += r == bp[b] || ((unsigned)pr[r] >> 16) != ((unsigned)pr[r - 1] >> 16);
      if (ntg > 32) one_target_lanes = false;
    }
    for (int64_t b = 0; interleave && b + 1 < nbp; ++b) {
      const int r0 = bp[b], cnt = bp[b + 1] - bp[b], nz = blk_nz[b];
      auto tile_form = [nz](int x) {
        const int jj = x & 255, kk = (x >> 8) & 255;
        return (jj * nz + kk) | (x & ~0xffff);
      };
      const size_t base = rr.size();
      if (one_target_lanes) {
        // targets of the block (its rules are sorted by target) and their lanes
        std::vector<int> tstart, tcnt, tlanes;
        for (int r = 0; r < cnt; ++r)
          if (r == 0 || ((unsigned)pr[r0 + r] >> 16) != ((unsigned)pr[r0 + r - 1] >> 16)) {
            tstart.push_back(r);
            tcnt.push_back(0);
          }
        for (size_t k = 0; k < tstart.size(); ++k)
          tcnt[k] = (k + 1 < tstart.size() ? tstart[k + 1] : cnt) - tstart[k];
        tlanes.assign(tstart.size(), 1);
        int free_lanes = 32 - (int)tstart.size();
        auto slice = [&](size_t k) { return (tcnt[k] + tlanes[k] - 1) / tlanes[k]; };
        while (free_lanes > 0 && !tstart.empty()) {
          size_t best = 0;
          for (size_t k = 1; k < tstart.size(); ++k)
            if (slice(k) > slice(best)) best = k;
          if (slice(best) <= 1) break;
          ++tlanes[best];
          --free_lanes;
        }
        int per = 0;
        for (size_t k = 0; k < tstart.size(); ++k) per = std::max(per, slice(k));
        per = (per + 3) / 4 * 4;
        rr.resize(base + (size_t)per * 32);
        const int pad_t = cnt ? (pr[r0] & ~0xffff) : 0;
        for (size_t slot = 0; slot < (size_t)per * 32; ++slot) {
          rr[base + slot].x = pad_t;  // a valid target, operand entry 0, zero weight
          std::memcpy(&rr[base + slot].y, &zero, 4);
        }
        int lane = 0;
        for (size_t k = 0; k < tstart.size(); ++k) {
          const int len = slice(k);
          for (int l = 0; l < tlanes[k]; ++l, ++lane) {
            const int a0 = tstart[k] + l * len, a1 = std::min(tstart[k] + tcnt[k], a0 + len);
            const int tpad = pr[r0 + tstart[k]] & ~0xffff;
            for (int i = 0; i < per; ++i) {
              int2 v;
              if (a0 + i < a1) {
                v.x = tile_form(pr[r0 + a0 + i]);
                std::memcpy(&v.y, &pw[r0 + a0 + i], 4);
              } else {
                v.x = tpad;
                std::memcpy(&v.y, &zero, 4);
              }
              rr[base + (size_t)i * 32 + lane] = v;
            }
          }
        }
      } else {
        const int per = (cnt + 31) / 32;
        rr.resize(base + (size_t)per * 32);
        for (int slot = 0; slot < per * 32; ++slot) {
          const int lane = slot % 32, i = slot / 32, logical = lane * per + i;
          int2 v;
          if (logical < cnt) {
            v.x = tile_form(pr[r0 + logical]);
            std::memcpy(&v.y, &pw[r0 + logical], 4);
          } else {
            v.x = cnt ? (pr[r0 + cnt - 1] & ~0xffff) : 0;  // target kept, operand entry 0
            std::memcpy(&v.y, &zero, 4);
          }
          rr[base + slot] = v;
        }
      }
      // every word the device decodes from this block: the tile index below
      // the pair's ny * nz (the warp's M tile holds max_mtile >= that) and
      // the target below the job's target count (<= cell_size)
      for (size_t q = base; q < rr.size(); ++q) {
        const unsigned x = (unsigned)rr[q].x;
        if ((int)(x & 0xffffu) >= blk_ny[b] * nz || (int)(x >> 16) >= ntgt_j)
          throw PuckError{PUCK_ERR_BAD_GRAMMAR, "pair rule out of its tile or target range in " + n};
      }
      dev_bp.push_back((int)rr.size());
      blk_n.push_back(cnt);
    }
    if (rr.size() > (size_t)INT32_MAX) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "pair rule table too large in " + n};
    J.npair = (int)npk;
    J.interleaved = !interleave ? 0 : one_target_lanes ? 2 : 1;
    J.a_is_t = a_t[j];
    J.b_is_t = b_t[j];
    J.pair_key = up<int>(D, L, n + "/pair_key", "i4");
    const std::vector<int> gbits = gate_seg_bits(L, n, merged);
    if (merged && J.nseg > 0) {
      std::vector<int> g((size_t)npk * L.mask_size);
      for (size_t k = 0; k < g.size(); ++k) g[k] = gbits[k % L.mask_size];
      J.pair_gate = static_cast<const int*>(D.upload(g.data(), g.size() * sizeof(int)));
    } else {
      J.pair_gate = up<int>(D, L, n + "/pair_gate", "i4");
    }
    // Viterbi and sum-product jobs (inside and outside) also get the
    // flat-tile layout where it applies
    if ((L.semiring == puck::SEMI_VITERBI || L.semiring == puck::SEMI_REAL) &&
        build_flat_tiles(D, J, ntgt_j, npk, pk, pbk, L.get<int>(n + "/blk_seg", "i4", nullptr), bp, pr, pw,
                         gbits.data(), J.nseg, L.mask_size,
                         L.get<int>(a_t[j] ? "t_mem_off" : "nt_mem_off", "i4", nullptr),
                         L.get<int>(a_t[j] ? "t_mem" : "nt_mem", "i4", nullptr),
                         L.get<int>(b_t[j] ? "t_mem_off" : "nt_mem_off", "i4", nullptr),
                         L.get<int>(b_t[j] ? "t_mem" : "nt_mem", "i4", nullptr),
                         L.semiring == puck::SEMI_REAL ? 0.f : -INFINITY, &d.flat_mtile))
      d.max_npair = std::max(d.max_npair, J.fnpair);
    J.pair_blk = up<int>(D, L, n + "/pair_blk", "i4");
    J.blk_seg = up<int>(D, L, n + "/blk_seg", "i4");
    J.blk_ptr = static_cast<const int*>(D.upload(dev_bp.data(), dev_bp.size() * sizeof(int)));
    if (blk_n.empty()) blk_n.push_back(0);  // a job without rules still gets a (never read) table
    J.blk_nrule = static_cast<const int*>(D.upload(blk_n.data(), blk_n.size() * sizeof(int)));
    J.pair_rules = reinterpret_cast<const int2*>(D.upload(rr.data(), rr.size() * sizeof(int2)));
    d.max_npair = std::max(d.max_npair, J.npair);
    const int* ao = L.get<int>(a_t[j] ? "t_mem_off" : "nt_mem_off", "i4", nullptr);
    const int* bo = L.get<int>(b_t[j] ? "t_mem_off" : "nt_mem_off", "i4", nullptr);
    for (int64_t k = 0; k < npk; ++k) {
      const int ca = pk[k] & 255, cb = (pk[k] >> 8) & 255;
      d.max_mtile = std::max(d.max_mtile, (ao[ca + 1] - ao[ca]) * (bo[cb + 1] - bo[cb]));
    }
  }
  d.flat_inside = 1;
  d.flat_outside = 1;
  for (int j = 0; j < puck::NJOBS; ++j)
    if (d.jobs[j].nseg > 0 && d.jobs[j].n_tgt > 0 && !d.jobs[j].flat) (j <= puck::IN_TT ? d.flat_inside : d.flat_outside) = 0;
  // Target-major levels also get each job's rules grouped by child pair (the
  // pair-major scan of an ungated level), for the jobs whose targets have at
  // most kPairMajorRules rules on average: with more, the atomic updates of
  // each target serialise (a 64 + 32-symbol grammar of 20,000 rules, 137 per
  // NN target, parsed 10% slower that way).
  if (L.semiring != puck::SEMI_LOGSUM && L.get<int>("in_NN/pair_mode", "i4", nullptr)[0] != 2) {
    std::vector<int> pab, poff;
    std::vector<int2> prule;
    for (int j = 0; j < puck::NJOBS; ++j) {
      if (!pm_tables_host(L, j, pab, poff, prule)) continue;
      puck::DevJob& J = d.jobs[j];
      J.pm_npair = (int)pab.size();
      J.pm_ab = static_cast<const int*>(D.upload(pab.data(), pab.size() * sizeof(int)));
      J.pm_off = static_cast<const int*>(D.upload(poff.data(), poff.size() * sizeof(int)));
      J.pm_rule = static_cast<const int2*>(D.upload(prule.data(), prule.size() * sizeof(int2)));
    }
  }
  d.pair_group = 1;
  {
    const int* nn_mode = L.get<int>("in_NN/pair_mode", "i4", nullptr);
    d.mode = (nn_mode[0] == 2 && L.semiring != puck::SEMI_LOGSUM) ? 2 : 0;
    // A target-major Viterbi level (the coarse level of a cascade, one
    // symbol per coarse id) gets its flat-tile layout over groups of 16
    // coarse ids, which replace its one-symbol pairs.
    if (d.mode == 0 && L.semiring == puck::SEMI_VITERBI) {
      int mt = 0;
      bool ok = true;
      for (int j = puck::IN_NN; ok && j <= puck::IN_TT; ++j)
        if (d.jobs[j].nseg > 0 && d.jobs[j].n_tgt > 0) ok = build_group_tiles(D, d.jobs[j], L, j, &mt);
      if (ok) {
        d.pair_group = 16;
        d.flat_mtile = mt;
        d.flat_inside = 1;
        for (int j = puck::IN_NN; j <= puck::IN_TT; ++j) d.max_npair = std::max(d.max_npair, d.jobs[j].fnpair);
      } else {
        d.flat_inside = 0;  // group tables in some jobs, one-symbol pairs in others: not used
      }
      d.flat_outside = 0;  // its outside jobs keep one-symbol pairs: the target-major scan is faster
    }
    // The flat-tile passes are ready; by default they run on the
    // pair-factored levels (the parser's autotuner chooses per span band).
    D.flat_ready_in = d.flat_inside != 0;
    D.flat_ready_out = d.flat_outside != 0;
    d.flat_inside = D.flat_ready_in && d.mode == 2;
    d.flat_outside = D.flat_ready_out && d.mode == 2;
    d.nt_mem_off = up<int>(D, L, "nt_mem_off", "i4");
    d.nt_mem = up<int>(D, L, "nt_mem", "i4");
    d.t_mem_off = up<int>(D, L, "t_mem_off", "i4");
    d.t_mem = up<int>(D, L, "t_mem", "i4");
  }
  for (int j = 0; j < puck::NUJOBS; ++j) {
    const std::string n = kUJobNames[j];
    int64_t nrow = 0, ns = 0, nw = 0;
    L.get<int>(n + "/rowptr", "i4", &nrow);
    const int* src = L.get<int>(n + "/src", "i4", &ns);
    const float* w = L.get<float>(n + "/w", "f4", &nw);
    if (ns != nw) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "inconsistent unary job " + n};
    std::vector<int2> packed(ns);
    for (int64_t k = 0; k < ns; ++k) {
      packed[k].x = src[k];
      std::memcpy(&packed[k].y, &w[k], 4);
    }
    puck::DevUJob& U = d.ujobs[j];
    U.n_tgt = (int)(nrow - 1);
    U.rowptr = up<int>(D, L, n + "/rowptr", "i4");
    U.rules = reinterpret_cast<const int2*>(D.upload(packed.data(), packed.size() * sizeof(int2)));
  }
  d.lex_off = up<long long>(D, L, "lex_off", "i8");
  d.lex_term = up<int>(D, L, "lex_term", "i4");
  d.lex_score = up<float>(D, L, "lex_score", "f4");
  d.v_off = up<int>(D, L, "v_off", "i4");
  d.v_left = up<int>(D, L, "v_left", "i4");
  d.v_right = up<int>(D, L, "v_right", "i4");
  d.v_score = up<float>(D, L, "v_score", "f4");
}

namespace {

uint16_t bf16_bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7fffffffu) > 0x7f800000u) return 0x7fc0;  // NaN
  return (uint16_t)((u + 0x7fffu + ((u >> 16) & 1u)) >> 16);  // round to nearest even
}

int tile_offset_host(int r, int k, int kpad) { return ((r >> 3) * (kpad >> 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2; }

}  // namespace

// Tensor-core tables of a sum-product level (DevTc).  Returns false, with the
// reason, for a level whose structure the tensor-core form does not cover.
bool puck_host::build_tc(LevelDev& D, const HostLevel& L, std::string* why) {
  auto no = [&](const std::string& m) {
    if (why) *why = m;
    return false;
  };
  const puck::DevLevel& d = D.d;
  if (L.semiring != puck::SEMI_REAL || d.mode != 2) return no("not a pair-factored sum-product level");
  if (d.gate_merged) return no("coarse level of a cascade");
  const int ms = L.mask_size, cs = L.cell_size;
  const int* nt_off = L.get<int>("nt_mem_off", "i4", nullptr);
  const int* nt_mem = L.get<int>("nt_mem", "i4", nullptr);
  const int* t_off = L.get<int>("t_mem_off", "i4", nullptr);
  const int* ntc = L.get<int>("nt_coarse", "i4", nullptr);
  // member index of each nonterminal within its coarse symbol
  std::vector<int> memidx(L.n_nt, -1);
  int maxmem = 0;
  for (int c = 0; c < L.n_coarse; ++c) {
    maxmem = std::max(maxmem, nt_off[c + 1] - nt_off[c]);
    for (int i = nt_off[c]; i < nt_off[c + 1]; ++i) memidx[nt_mem[i]] = i - nt_off[c];
  }
  const int slot_w = (maxmem + 15) / 16 * 16;
  if (slot_w > 32) return no("more than 32 refinements of a coarse symbol");
  // Gating.  A target whose segment bits are the same in every block of the
  // four inside jobs is gated when the accumulator is read out.  Rules of
  // any other target go into entries of their own, one per segment, whose
  // rows are zeroed for the cells the segment does not gate in.
  std::vector<std::vector<int>> tbits(L.n_nt);
  std::vector<char> incons(L.n_nt, 0), parent_used(L.n_coarse, 0);
  int max_kpad = 16;
  struct JobTabs {
    int64_t npk = 0;
    const int *pk, *pbk, *bp, *bs, *sb, *pr;
    const float* pw;
    const int *ao, *bo;
  };
  JobTabs jt[4];
  for (int j = 0; j < 4; ++j) {
    const std::string n = kJobNames[j];
    JobTabs& J = jt[j];
    J.pk = L.get<int>(n + "/pair_key", "i4", &J.npk);
    J.pbk = L.get<int>(n + "/pair_blk", "i4", nullptr);
    J.bp = L.get<int>(n + "/blk_ptr", "i4", nullptr);
    J.bs = L.get<int>(n + "/blk_seg", "i4", nullptr);
    J.sb = L.get<int>(n + "/seg_bits", "i4", nullptr);
    J.pr = L.get<int>(n + "/pair_rule", "i4", nullptr);
    J.pw = L.get<float>(n + "/pair_w", "f4", nullptr);
    const bool at = j == 2 || j == 3, bt = j == 1 || j == 3;
    J.ao = at ? t_off : nt_off;
    J.bo = bt ? t_off : nt_off;
    for (int64_t p = 0; p < J.npk; ++p) {
      const int ca = J.pk[p] & 255, cb = (J.pk[p] >> 8) & 255;
      const int kk = (J.ao[ca + 1] - J.ao[ca]) * (J.bo[cb + 1] - J.bo[cb]);
      if (kk > 256) return no("a coarse pair with more than 256 child pairs");
      if ((J.ao[ca + 1] - J.ao[ca]) * ((J.bo[cb + 1] - J.bo[cb] + 3) / 4) > 96 || J.ao[ca + 1] - J.ao[ca] > 32 ||
          J.bo[cb + 1] - J.bo[cb] > 32)
        return no("a coarse pair's outer product exceeds three tasks per lane");
      max_kpad = std::max(max_kpad, (kk + 15) / 16 * 16);
      for (int b = J.pbk[p]; b < J.pbk[p + 1]; ++b) {
        const std::vector<int> bits(J.sb + (size_t)J.bs[b] * ms, J.sb + (size_t)(J.bs[b] + 1) * ms);
        for (int r = J.bp[b]; r < J.bp[b + 1]; ++r) {
          const int t = (int)((unsigned)J.pr[r] >> 16);
          if (t < 0 || t >= L.n_nt) return no("binary target outside the nonterminals");
          parent_used[ntc[t]] = 1;
          if (tbits[t].empty()) tbits[t] = bits;
          else if (tbits[t] != bits) incons[t] = 1;
        }
      }
    }
  }
  std::vector<int> tgt_gate((size_t)L.n_nt * ms, -1);
  for (int t = 0; t < L.n_nt; ++t)
    if (!incons[t] && !tbits[t].empty()) std::memcpy(&tgt_gate[(size_t)t * ms], tbits[t].data(), ms * sizeof(int));
  // slots: coarse parents in order, split evenly over parts of <= 512 columns
  std::vector<int> parents;
  for (int c = 0; c < L.n_coarse; ++c)
    if (parent_used[c]) parents.push_back(c);
  if (parents.empty()) return no("no binary rules");
  const int per_part_max = 512 / slot_w;
  const int nparts = ((int)parents.size() + per_part_max - 1) / per_part_max;
  const int per_part = ((int)parents.size() + nparts - 1) / nparts;
  // each group of four warps zeroes and reads its share of the columns, 16 at
  // a time: a multiple of 16 per group
  int ncols = 16 * (puck::kTcThreads / 128);
  while (ncols < per_part * slot_w) ncols <<= 1;
  std::vector<int> part_of(L.n_coarse, -1), slot_of(L.n_coarse, -1);
  std::vector<int> col_tgt((size_t)nparts * ncols, -1);
  std::vector<char> covered(cs, 0);
  for (size_t i = 0; i < parents.size(); ++i) {
    const int c = parents[i], h = (int)i / per_part, sl = (int)i % per_part;
    part_of[c] = h;
    slot_of[c] = sl;
    for (int m = 0; m < nt_off[c + 1] - nt_off[c]; ++m) {
      col_tgt[(size_t)h * ncols + sl * slot_w + m] = nt_mem[nt_off[c] + m];
      covered[nt_mem[nt_off[c] + m]] = 1;
    }
  }
  std::vector<int> uncovered;
  for (int k = 0; k < cs; ++k)
    if (!covered[k]) uncovered.push_back(k);
  // shared memory: two A tiles (128 x max_kpad BF16) and two B buffers
  const size_t static_smem = puck::tc_static_smem_bytes() + 256;
  const size_t abytes = 2 * (size_t)puck::kTcRows * max_kpad * 2;
  const size_t blk_bytes = (size_t)slot_w * max_kpad * 2;
  if (abytes + static_smem + 2 * blk_bytes > 227 * 1024) return no("outer-product tiles too large for shared memory");
  size_t bcap = std::min<size_t>(40 * 1024, (227 * 1024 - static_smem - abytes) / 2) / 128 * 128;
  // a CTA holding more than half of TMEM keeps its SM to itself (a second
  // one would wait in tcgen05.alloc): shared memory for one CTA per SM
  if (ncols > 256 && abytes + 2 * bcap + static_smem < 120 * 1024)
    bcap = ((120 * 1024 - abytes - static_smem + 1) / 2 + 127) / 128 * 128;
  if (abytes + 2 * bcap + static_smem > 227 * 1024) return no("tensor-core buffers do not fit shared memory");
  // Entries, per part, job and pair: the pair's freely gated rules, then one
  // entry per segment for rules of targets with differing segments.  An
  // entry's B operands are one tile per coarse parent (slot), split into
  // several entries when they exceed a staging buffer.
  std::vector<int4> tpair;
  std::vector<int> tpair_gate, tblk, part_off(1, 0);
  std::vector<long long> tpair_b;
  std::vector<uint16_t> bmat;
  for (int h = 0; h < nparts; ++h) {
    for (int j = 0; j < 4; ++j) {
      const JobTabs& J = jt[j];
      for (int64_t p = 0; p < J.npk; ++p) {
        const int ca = J.pk[p] & 255, cb = (J.pk[p] >> 8) & 255;
        const int nz = J.bo[cb + 1] - J.bo[cb];
        const int kpad = ((J.ao[ca + 1] - J.ao[ca]) * nz + 15) / 16 * 16;
        const size_t bbytes = (size_t)slot_w * kpad * 2;
        // entry key: empty = readout-gated rules, else the segment bits
        std::map<std::vector<int>, std::map<int, std::vector<int>>> groups;  // key -> slot -> rules
        std::map<std::vector<int>, std::vector<int>> gate_of;
        for (int b = J.pbk[p]; b < J.pbk[p + 1]; ++b) {
          const std::vector<int> bits(J.sb + (size_t)J.bs[b] * ms, J.sb + (size_t)(J.bs[b] + 1) * ms);
          for (int r = J.bp[b]; r < J.bp[b + 1]; ++r) {
            const int t = (int)((unsigned)J.pr[r] >> 16), parent = ntc[t];
            if (part_of[parent] != h) continue;
            const std::vector<int> key = incons[t] ? bits : std::vector<int>();
            groups[key][slot_of[parent]].push_back(r);
            std::vector<int>& g = gate_of[key];
            if (g.empty()) g.assign(ms, 0);
            for (int w = 0; w < ms; ++w) g[w] |= bits[w];
          }
        }
        for (auto& kv : groups) {
          std::vector<std::pair<int, const std::vector<int>*>> tiles;
          for (auto& sv : kv.second) tiles.emplace_back(sv.first, &sv.second);
          const std::vector<int>& gate = gate_of[kv.first];
          for (size_t i0 = 0; i0 < tiles.size();) {
            const size_t take = std::min(tiles.size() - i0, bcap / bbytes);
            int4 e;
            e.x = j | (int)(p << 2);
            e.y = kpad;
            e.z = (int)tblk.size();
            e.w = e.z + (int)take;
            tpair.push_back(e);
            tpair_b.push_back((long long)bmat.size() * 2);
            tpair_gate.insert(tpair_gate.end(), gate.begin(), gate.end());
            for (size_t i = i0; i < i0 + take; ++i) {
              tblk.push_back(tiles[i].first);
              const size_t base = bmat.size();
              bmat.resize(base + bbytes / 2, 0);
              for (int r : *tiles[i].second) {
                const int jj = J.pr[r] & 255, kk = (J.pr[r] >> 8) & 255, t = (int)((unsigned)J.pr[r] >> 16);
                bmat[base + tile_offset_host(memidx[t], jj * nz + kk, kpad) / 2] = bf16_bits(J.pw[r]);
              }
            }
            i0 += take;
          }
        }
      }
    }
    part_off.push_back((int)tpair.size());
  }
  puck::DevTc& T = D.tc;
  T.nparts = nparts;
  T.slot_w = slot_w;
  T.ncols = ncols;
  T.max_kpad = max_kpad;
  T.bcap = (int)bcap;
  T.part_off = static_cast<const int*>(D.upload(part_off.data(), part_off.size() * sizeof(int)));
  T.tpair = static_cast<const int4*>(D.upload(tpair.data(), tpair.size() * sizeof(int4)));
  T.tpair_gate = static_cast<const int*>(D.upload(tpair_gate.data(), tpair_gate.size() * sizeof(int)));
  T.tblk = static_cast<const int*>(D.upload(tblk.data(), tblk.size() * sizeof(int)));
  T.tpair_b = static_cast<const long long*>(D.upload(tpair_b.data(), tpair_b.size() * sizeof(long long)));
  T.bmat = static_cast<const unsigned char*>(D.upload(bmat.data(), bmat.size() * 2));
  T.col_tgt = static_cast<const int*>(D.upload(col_tgt.data(), col_tgt.size() * sizeof(int)));
  T.tgt_gate = static_cast<const int*>(D.upload(tgt_gate.data(), tgt_gate.size() * sizeof(int)));
  T.uncovered = static_cast<const int*>(D.upload(uncovered.data(), uncovered.size() * sizeof(int)));
  T.n_uncovered = (int)uncovered.size();
  const int zero = 0;
  T.err = static_cast<int*>(D.upload(&zero, sizeof(int)));
  return true;
}

namespace {

long long tri(int n) { return (long long)n * (n + 1) / 2; }

enum Mode { MODE_PARSE = 0, MODE_PARTITIONS = 1, MODE_INSIDE_OUTSIDE = 2 };

struct LevelBufs {
  DevBuf inside, outside, masks, iscale, oscale, part, decode, live_in, live_out;
};

}  // namespace

constexpr int kNoFlat = 1 << 30;  // flat_from of a level that never runs the flat-tile form

struct puck_parser {
  const puck_grammar* g = nullptr;
  puck_options opt{};
  cudaStream_t stream = nullptr;
  std::vector<std::unique_ptr<LevelDev>> levels;
  std::vector<LevelBufs> bufs;
  DevBuf b_len, b_cell_off, b_word_off, b_words, b_work, b_node_off,
      b_mbr_off, b_nodes, b_status, b_logz, b_scratch, b_counters, b_parts, b_cell_cnt;
  int sms = 1;
  puck::DevBatch last_batch{};
  int64_t last_num_cells = 0;
  int last_batches = 0;
  puck_stats stats{};
  int64_t budget_bytes = 0;
  cudaEvent_t ev_batch[2] = {nullptr, nullptr};
  std::vector<std::array<cudaEvent_t, 5>> ev_level;   // per level: in0, in1, out1, mask1, dec1
  std::vector<std::array<double, 4>> pass_ms;
  std::vector<std::array<int64_t, 4>> pass_launches;
  std::vector<std::array<int64_t, 2>> level_work;  // per level: work units, +0.0 partials (last call)
  // use_graphs: per level, the executable graphs of the inside and outside
  // span sequences, updated in place while a new batch keeps their shape
  std::vector<std::array<cudaGraphExec_t, 2>> graphs;
  int64_t graph_updates = 0, graph_instantiations = 0;
  // autotuned policy: per level the gather form (-1: the archive's choice,
  // 0 target-major, 2 pair-factored), the first span whose inside launch
  // runs the flat-tile form (kNoFlat: none), and the waves of CTAs that long
  // cells are split to fill
  std::vector<int> tuned_mode;
  std::vector<int> flat_from;
  double waves = 2.0;
};

namespace {

int64_t bytes_per_cell(const puck_parser* P, Mode mode) {
  int64_t b = 0;
  const int nl = (int)P->g->levels.size();
  for (int l = 0; l < nl; ++l) {
    const HostLevel& L = P->g->levels[l];
    const bool last = l == nl - 1;
    const bool need_out = !last || mode == MODE_INSIDE_OUTSIDE || (mode == MODE_PARSE && L.semiring != 0 &&
                                                                    P->opt.decode != PUCK_DECODE_VITERBI);
    b += (int64_t)(L.cell_size + L.mask_size) * 4 * (need_out ? 2 : 1);  // chart + liveness
    if (!last) b += (int64_t)L.mask_size * 4 + 8;
    else b += 8;
  }
  return b;
}

// Runs `issue` (which enqueues kernels on st) directly, or, with use_graphs,
// captures it into a graph and launches that graph.  The executable graph of
// (level, pass) is kept and updated in place when the next batch has the
// same launch sequence; grid sizes and kernel arguments may differ.
template <class F>
void launch_sequence(puck_parser* P, int level, int pass, cudaStream_t st, F&& issue) {
  if (!P->opt.use_graphs) {
    issue();
    return;
  }
  cudaGraph_t g = nullptr;
  CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
  try {
    issue();
  } catch (...) {
    cudaStreamEndCapture(st, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  CUDA_TRY(cudaStreamEndCapture(st, &g));
  cudaGraphExec_t& ex = P->graphs[level][pass];
  bool updated = false;
  if (ex) {
    cudaGraphExecUpdateResultInfo info{};
    updated = cudaGraphExecUpdate(ex, g, &info) == cudaSuccess;
    if (!updated) {
      cudaGetLastError();  // clear the failed update
      cudaGraphExecDestroy(ex);
      ex = nullptr;
    }
  }
  if (!ex) {
    const cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
    if (e != cudaSuccess) {
      cudaGraphDestroy(g);
      ex = nullptr;
      CUDA_TRY(e);
    }
    ++P->graph_instantiations;
  } else {
    ++P->graph_updates;
  }
  cudaGraphDestroy(g);
  CUDA_TRY(cudaGraphLaunch(ex, st));
}

struct BatchPlan {
  std::vector<int> sent;  // global sentence ids
};

void run_batch(puck_parser* P, Mode mode, const BatchPlan& plan, const int32_t* word_ids, const int64_t* offsets,
               puck_tree_node* nodes_out, const std::vector<int64_t>& node_off_global, float* log_z,
               int32_t* sent_status) {
  const int nl = (int)P->g->levels.size();
  cudaStream_t st = P->stream;
  const int ns = (int)plan.sent.size();
  // host batch arrays
  std::vector<int> len(ns);
  std::vector<long long> cell_off(ns + 1, 0), word_off(ns + 1, 0), node_off(ns + 1, 0), mbr_off(ns + 1, 0);
  std::vector<int> words;
  int max_len = 0;
  for (int i = 0; i < ns; ++i) {
    const int s = plan.sent[i];
    len[i] = (int)(offsets[s + 1] - offsets[s]);
    max_len = std::max(max_len, len[i]);
    cell_off[i + 1] = cell_off[i] + 2 * tri(len[i]);
    word_off[i + 1] = word_off[i] + len[i];
    node_off[i + 1] = node_off[i] + 2 * len[i] - 1;
    mbr_off[i + 1] = mbr_off[i] + 3LL * (len[i] + 1) * (len[i] + 1);
    words.insert(words.end(), word_ids + offsets[s], word_ids + offsets[s + 1]);
  }
  // Work lists, concatenated into one upload.  Span launches take the
  // sentences that have cells of that span, longest first; the lexicon, the
  // per-cell kernels and the per-sentence kernels take every sentence.
  std::vector<int> order(ns);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return len[a] > len[b]; });
  std::vector<int> wl;
  struct ListAt { size_t sent, pref; int nent; long long nunits; };
  auto add_list = [&](int nent, auto sent_of, auto units_of) {
    ListAt at{wl.size(), 0, nent, 0};
    for (int k = 0; k < nent; ++k) wl.push_back(sent_of(k));
    at.pref = wl.size();
    long long acc = 0;
    wl.push_back(0);
    for (int k = 0; k < nent; ++k) {
      acc += units_of(k);
      wl.push_back((int)acc);
    }
    at.nunits = acc;
    return at;
  };
  std::vector<ListAt> span_list(max_len + 1);
  std::vector<int> ways(max_len + 1, 1);
  long long part_units = 0;
  for (int L = 1; L <= max_len; ++L) {
    int k = 0;
    long long cells = 0;
    while (k < ns && len[order[k]] >= L) cells += len[order[k++]] - L + 1;
    const int G = puck::cell_ways(L, puck::part_target((double)cells * (L - 1), P->sms, P->waves));
    ways[L] = G;
    if (G > 1) part_units = std::max(part_units, cells * G);
    span_list[L] = add_list(k, [&](int j) { return order[j]; }, [&](int j) { return (len[order[j]] - L + 1) * G; });
  }
  // tensor-core inside passes: per span, the (sentence, begin) pairs of its
  // cells in tiles, and a one-CTA-per-cell list for finishing the cells
  const bool any_tc = std::any_of(P->levels.begin(), P->levels.end(), [](const auto& x) { return x->tc_ok; });
  std::vector<ListAt> span_list1;
  std::vector<std::pair<size_t, int>> tc_cells(max_len + 1, {0, 0});
  if (any_tc) {
    span_list1.resize(max_len + 1);
    for (int L = 1; L <= max_len; ++L) {
      int k = 0;
      while (k < ns && len[order[k]] >= L) ++k;
      span_list1[L] = add_list(k, [&](int j) { return order[j]; }, [&](int j) { return len[order[j]] - L + 1; });
      tc_cells[L].first = wl.size();
      for (int j = 0; j < k; ++j)
        for (int b = 0; b + L <= len[order[j]]; ++b) {
          wl.push_back(order[j]);
          wl.push_back(b);
        }
      tc_cells[L].second = (int)((wl.size() - tc_cells[L].first) / 2);
    }
  }
  const ListAt tok_list = add_list(ns, [](int j) { return j; }, [&](int j) { return len[j]; });
  const ListAt cell_list = add_list(ns, [](int j) { return j; }, [&](int j) { return 2 * tri(len[j]); });
  const long long num_cells = cell_off[ns];
  auto h2d = [&](DevBuf& b, const void* src, size_t bytes) {
    b.ensure(std::max<size_t>(bytes, 16));
    if (bytes) CUDA_TRY(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, st));
    P->stats.h2d_bytes += (int64_t)bytes;
  };
  h2d(P->b_len, len.data(), ns * sizeof(int));
  h2d(P->b_cell_off, cell_off.data(), (ns + 1) * sizeof(long long));
  h2d(P->b_word_off, word_off.data(), (ns + 1) * sizeof(long long));
  h2d(P->b_words, words.data(), words.size() * sizeof(int));
  h2d(P->b_work, wl.data(), wl.size() * sizeof(int));
  h2d(P->b_node_off, node_off.data(), (ns + 1) * sizeof(long long));
  puck::DevBatch B{};
  B.nsent = ns;
  B.len = P->b_len.as<int>();
  B.cell_off = P->b_cell_off.as<long long>();
  B.word_off = P->b_word_off.as<long long>();
  B.words = P->b_words.as<int>();
  B.node_off = P->b_node_off.as<long long>();
  const int* wdev = P->b_work.as<int>();
  auto work = [&](const ListAt& a, int span) {
    puck::DevWork W{};
    W.nent = a.nent;
    W.nunits = a.nunits;
    W.sent = wdev + a.sent;
    W.span = nullptr;
    W.span_all = span;
    W.pref = wdev + a.pref;
    W.ways = nullptr;
    W.ways_all = span >= 1 && span <= max_len ? ways[span] : 1;
    W.part_rows = P->b_parts.as<float>();
    W.cell_cnt = P->b_cell_cnt.as<int>();
    W.one_word_batch = max_len == 1;
    return W;
  };
  const puck::DevWork Wtok = work(tok_list, 1), Wcell = work(cell_list, 0);
  puck::DevWork Wsent = Wcell;
  Wsent.pref = nullptr;
  Wsent.nunits = ns;
  P->b_status.ensure(ns * sizeof(int) + 16);
  CUDA_TRY(cudaMemsetAsync(P->b_status.p, 0, ns * sizeof(int), st));
  // per level: binary partials >= +0.0 written, (rule, split) work units;
  // then the cells the last coarse level prunes entirely
  const size_t ctr_bytes = (2 * nl + 1) * sizeof(unsigned long long);
  P->b_counters.ensure(ctr_bytes);
  CUDA_TRY(cudaMemsetAsync(P->b_counters.p, 0, ctr_bytes, st));
  if (part_units > 0) {
    int max_cs = 0;
    for (const HostLevel& HL : P->g->levels) max_cs = std::max(max_cs, HL.cell_size);
    P->b_parts.ensure(part_units * max_cs * sizeof(float));
  }
  P->b_cell_cnt.ensure(num_cells * sizeof(int) + 16);
  CUDA_TRY(cudaMemsetAsync(P->b_cell_cnt.p, 0, num_cells * sizeof(int), st));

  auto rec = [&](cudaEvent_t e) { CUDA_TRY(cudaEventRecord(e, st)); };
  std::vector<std::array<int64_t, 4>> launches_l(nl, std::array<int64_t, 4>{0, 0, 0, 0});
  rec(P->ev_batch[0]);
  puck::DevMask M{nullptr, 0, nullptr, nullptr};
  for (int l = 0; l < nl; ++l) {
    puck::DevLevel D = P->levels[l]->d;
    if (P->tuned_mode[l] >= 0) D.mode = P->tuned_mode[l];
    const bool tc = P->levels[l]->tc_ok && D.mode == 2 && num_cells < INT32_MAX;
    D.tc_binary = tc ? 1 : 0;
    if (tc) CUDA_TRY(cudaMemsetAsync(P->levels[l]->tc.err, 0, sizeof(int), st));
    const HostLevel& HL = P->g->levels[l];
    LevelBufs& lb = P->bufs[l];
    const bool last = l == nl - 1;
    const bool need_out = !last || mode == MODE_INSIDE_OUTSIDE ||
                          (mode == MODE_PARSE && HL.semiring != 0 && P->opt.decode != PUCK_DECODE_VITERBI);
    lb.inside.ensure(num_cells * D.cell_size * sizeof(float));
    if (need_out) lb.outside.ensure(num_cells * D.cell_size * sizeof(float));
    lb.part.ensure(ns * sizeof(double) + 16);
    CUDA_TRY(cudaMemsetAsync(lb.part.p, 0, ns * sizeof(double), st));
    float* inside = lb.inside.as<float>();
    float* outside = need_out ? lb.outside.as<float>() : nullptr;
    lb.live_in.ensure(num_cells * D.mask_size * sizeof(int));
    if (need_out) lb.live_out.ensure(num_cells * D.mask_size * sizeof(int));
    const puck::DevLive V{lb.live_in.as<int>(), need_out ? lb.live_out.as<int>() : nullptr};
    puck::DevMask MM = M;
    if (D.semiring != puck::SEMI_REAL) { MM.iscale = nullptr; MM.oscale = nullptr; }
    auto& EV = P->ev_level[l];
    auto& LC = launches_l[l];
    rec(EV[0]);
    const puck::Counters C{P->b_counters.as<unsigned long long>() + 2 * l,
                           P->b_counters.as<unsigned long long>() + 2 * l + 1, P->b_status.as<int>()};
    launch_sequence(P, l, 0, st, [&] {
      CUDA_TRY(puck::launch_lexicon(D, B, Wtok, MM, inside, lb.part.as<double>(), V, C, st));
      ++LC[0];
      for (int span = 1; span <= max_len; ++span) {
        if (tc && span >= 2) {
          CUDA_TRY(puck::launch_inside_tc(D, P->levels[l]->tc, B, span, wdev + tc_cells[span].first,
                                          tc_cells[span].second, MM, inside, V, C, st));
          ++LC[0];
          puck::DevWork W1 = work(span_list1[span], span);
          W1.ways_all = 1;
          CUDA_TRY(puck::launch_inside_span(D, B, W1, MM, max_len, inside, V, C, st));
        } else {
          // the flat-tile form from the level's chosen span on
          puck::DevLevel Ds = D;
          Ds.flat_inside = P->levels[l]->flat_ready_in && span >= P->flat_from[l];
          CUDA_TRY(puck::launch_inside_span(Ds, B, work(span_list[span], span), MM, max_len, inside, V, C, st));
        }
        ++LC[0];
      }
    });
    rec(EV[1]);
    if (need_out) {
      launch_sequence(P, l, 1, st, [&] {
        for (int span = max_len; span >= 1; --span) {
          puck::DevLevel Ds = D;
          Ds.flat_outside = P->levels[l]->flat_ready_out && span >= P->flat_from[l];
          CUDA_TRY(puck::launch_outside_span(Ds, B, work(span_list[span], span), MM, max_len, inside, outside, V,
                                             C, st));
          ++LC[1];
        }
      });
    }
    rec(EV[2]);
    if (!last) {
      lb.masks.ensure(num_cells * D.mask_size * sizeof(int));
      CUDA_TRY(puck::launch_masks(D, B, Wcell, inside, outside, P->opt.prune_threshold, lb.masks.as<int>(), st,
                                  l == nl - 2 ? P->b_counters.as<unsigned long long>() + 2 * nl : nullptr));
      ++LC[2];
      lb.iscale.ensure(num_cells * sizeof(float));
      lb.oscale.ensure(num_cells * sizeof(float));
      const bool next_real = P->g->levels[l + 1].semiring == puck::SEMI_REAL;
      if (next_real) {
        CUDA_TRY(puck::launch_scaling(D.cell_size, B, Wcell, inside, lb.iscale.as<float>(), st));
        CUDA_TRY(puck::launch_scaling(D.cell_size, B, Wcell, outside, lb.oscale.as<float>(), st));
        LC[2] += 2;
      } else {
        CUDA_TRY(cudaMemsetAsync(lb.iscale.p, 0, num_cells * sizeof(float), st));
        CUDA_TRY(cudaMemsetAsync(lb.oscale.p, 0, num_cells * sizeof(float), st));
      }
      rec(EV[3]);
      rec(EV[4]);
      M.bits = lb.masks.as<int>();
      M.mask_size = D.mask_size;
      M.iscale = lb.iscale.as<float>();
      M.oscale = lb.oscale.as<float>();
      continue;
    }
    // last level
    rec(EV[3]);
    if (mode == MODE_PARTITIONS) {
      P->b_logz.ensure(ns * sizeof(float) + 16);
      CUDA_TRY(puck::launch_root_scores(D, B, Wsent, MM, inside, lb.part.as<double>(), P->b_logz.as<float>(), st));
      ++LC[3];
      rec(EV[4]);
      rec(P->ev_batch[1]);
      std::vector<float> lz(ns);
      CUDA_TRY(cudaMemcpyAsync(lz.data(), P->b_logz.p, ns * sizeof(float), cudaMemcpyDeviceToHost, st));
      P->stats.d2h_bytes += (int64_t)(ns * sizeof(float));
      CUDA_TRY(cudaStreamSynchronize(st));
      for (int i = 0; i < ns; ++i) log_z[plan.sent[i]] = lz[i];
    } else if (mode == MODE_PARSE) {
      P->b_nodes.ensure(node_off[ns] * sizeof(puck::DevNode) + 16);
      const bool vit = P->opt.decode == PUCK_DECODE_VITERBI ||
                       (P->opt.decode == PUCK_DECODE_AUTO && D.semiring == puck::SEMI_VITERBI);
      if (vit) {
        if (D.semiring != puck::SEMI_VITERBI)
          throw PuckError{PUCK_ERR_INVALID_ARG, "Viterbi decoding needs a Viterbi fine level"};
        CUDA_TRY(puck::launch_viterbi(D, B, Wsent, max_len, inside, P->b_nodes.as<puck::DevNode>(), st));
        ++LC[3];
      } else {
        if (!M.bits) throw PuckError{PUCK_ERR_INVALID_ARG, "Can't use null pruning mask for parse extraction!"};
        if (D.semiring == puck::SEMI_VITERBI)
          throw PuckError{PUCK_ERR_INVALID_ARG, "MBR decoding needs a sum-product fine level"};
        lb.decode.ensure(num_cells * sizeof(float2));
        CUDA_TRY(puck::launch_mbr_cells(D, B, Wcell, inside, outside, lb.decode.as<float2>(), st));
        h2d(P->b_mbr_off, mbr_off.data(), (ns + 1) * sizeof(long long));
        P->b_scratch.ensure(mbr_off[ns] * sizeof(float) + 16);
        CUDA_TRY(puck::launch_mbr_decode(B, Wsent, M, D.semiring == puck::SEMI_REAL ? 1 : 0, lb.decode.as<float2>(),
                                         P->b_mbr_off.as<long long>(), P->b_scratch.as<float>(),
                                         P->b_nodes.as<puck::DevNode>(), st));
        LC[3] += 2;
      }
      rec(EV[4]);
      rec(P->ev_batch[1]);
      std::vector<puck::DevNode> hn(node_off[ns]);
      CUDA_TRY(cudaMemcpyAsync(hn.data(), P->b_nodes.p, hn.size() * sizeof(puck::DevNode), cudaMemcpyDeviceToHost, st));
      P->stats.d2h_bytes += (int64_t)(hn.size() * sizeof(puck::DevNode));
      CUDA_TRY(cudaStreamSynchronize(st));
      for (int i = 0; i < ns; ++i) {
        const int s = plan.sent[i];
        std::memcpy(nodes_out + node_off_global[s], hn.data() + node_off[i],
                    (2 * len[i] - 1) * sizeof(puck_tree_node));
      }
    } else {
      // insideOutside: the decode kernels run, nothing is extracted (CLParser.scala:171-182)
      if (D.semiring == puck::SEMI_VITERBI) {
        P->b_nodes.ensure(node_off[ns] * sizeof(puck::DevNode) + 16);
        CUDA_TRY(puck::launch_viterbi(D, B, Wsent, max_len, inside, P->b_nodes.as<puck::DevNode>(), st));
      } else {
        lb.decode.ensure(num_cells * sizeof(float2));
        CUDA_TRY(puck::launch_mbr_cells(D, B, Wcell, inside, outside, lb.decode.as<float2>(), st));
      }
      ++LC[3];
      rec(EV[4]);
      rec(P->ev_batch[1]);
    }
  }
  std::vector<int> status(ns);
  std::vector<unsigned long long> ctr(2 * nl + 1, 0);
  CUDA_TRY(cudaMemcpyAsync(status.data(), P->b_status.p, ns * sizeof(int), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(ctr.data(), P->b_counters.p, ctr_bytes, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (sent_status)
    for (int i = 0; i < ns; ++i)
      if (status[i]) sent_status[plan.sent[i]] = status[i];
  auto ms_between = [](cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&ms, a, b));
    return (double)ms;
  };
  int64_t launches = 0;
  for (int l = 0; l < nl; ++l) {
    auto& EV = P->ev_level[l];
    const double t[4] = {ms_between(EV[0], EV[1]), ms_between(EV[1], EV[2]), ms_between(EV[2], EV[3]),
                         ms_between(EV[3], EV[4])};
    for (int k = 0; k < 4; ++k) {
      P->pass_ms[l][k] += t[k];
      P->pass_launches[l][k] += launches_l[l][k];
      launches += launches_l[l][k];
    }
    P->stats.ms_inside += t[0];
    P->stats.ms_outside += t[1];
    P->stats.ms_masks += t[2];
    P->stats.ms_decode += t[3];
  }
  P->stats.ms_device += ms_between(P->ev_batch[0], P->ev_batch[1]);
  P->stats.cells += num_cells;
  P->stats.cells_pruned += (int64_t)ctr[2 * nl];
  for (int l = 0; l < nl; ++l) {
    P->stats.binary_work += (int64_t)ctr[2 * l + 1];
    P->level_work[l][0] += (int64_t)ctr[2 * l + 1];
    P->level_work[l][1] += (int64_t)ctr[2 * l];
  }
  P->stats.kernel_launches += launches;
  P->stats.batches += 1;
  P->last_batch = B;
  P->last_num_cells = num_cells;
}

puck_status run_call(puck_parser* P, Mode mode, const int32_t* word_ids, const int64_t* offsets, int32_t nsent,
                     puck_tree_node* nodes_out, float* log_z, int32_t* sent_status) {
  try {
    if (!P || (nsent > 0 && (!word_ids || !offsets))) throw PuckError{PUCK_ERR_INVALID_ARG, "null argument"};
    if (nsent < 0) throw PuckError{PUCK_ERR_INVALID_ARG, "negative sentence count"};
    CUDA_TRY(cudaSetDevice(P->opt.device));
    const auto t0 = std::chrono::steady_clock::now();
    P->stats = puck_stats{};
    for (auto& a : P->pass_ms) a = {0, 0, 0, 0};
    for (auto& a : P->pass_launches) a = {0, 0, 0, 0};
    for (auto& a : P->level_work) a = {0, 0};
    const int nwords = P->g->levels.back().n_words;
    std::vector<int64_t> node_off(nsent + 1, 0);
    std::vector<int> valid;
    int first_bad = PUCK_OK;
    for (int s = 0; s < nsent; ++s) {
      const int64_t n = offsets[s + 1] - offsets[s];
      node_off[s + 1] = node_off[s] + std::max<int64_t>(2 * n - 1, 0);
      int st = PUCK_OK;
      if (n <= 0) st = PUCK_ERR_EMPTY;
      else if (n > P->opt.max_length) st = PUCK_ERR_SENT_TOO_LONG;
      else
        for (int64_t k = offsets[s]; k < offsets[s + 1]; ++k)
          if (word_ids[k] < 0 || word_ids[k] >= nwords) { st = PUCK_ERR_OOV; break; }
      if (sent_status) sent_status[s] = st;
      if (st == PUCK_OK) valid.push_back(s);
      else if (first_bad == PUCK_OK) first_bad = st;
    }
    if (nodes_out && mode == MODE_PARSE) std::memset(nodes_out, 0, node_off[nsent] * sizeof(puck_tree_node));
    if (log_z && mode == MODE_PARTITIONS)
      for (int s = 0; s < nsent; ++s) log_z[s] = std::nanf("");
    const int64_t per_cell = bytes_per_cell(P, mode);
    // work-list prefixes are 32-bit: a batch holds fewer than 2^31 cells
    const int64_t cap_cells = std::min<int64_t>(
        std::max<int64_t>(P->budget_bytes / std::max<int64_t>(per_cell, 1), 1), (int64_t)INT32_MAX);
    std::vector<BatchPlan> plans;
    BatchPlan cur;
    int64_t cur_cells = 0;
    for (int s : valid) {
      const int64_t c = 2 * tri((int)(offsets[s + 1] - offsets[s]));
      if (c > cap_cells) {
        if (sent_status) sent_status[s] = PUCK_ERR_OOM;
        continue;
      }
      if (!cur.sent.empty() && (cur_cells + c > cap_cells ||
                                (P->opt.max_batch_sentences > 0 && (int)cur.sent.size() >= P->opt.max_batch_sentences))) {
        plans.push_back(std::move(cur));
        cur = BatchPlan();
        cur_cells = 0;
      }
      cur.sent.push_back(s);
      cur_cells += c;
    }
    if (!cur.sent.empty()) plans.push_back(std::move(cur));
    for (auto& pl : plans) run_batch(P, mode, pl, word_ids, offsets, nodes_out, node_off, log_z, sent_status);
    P->last_batches = (int)plans.size();
    P->stats.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    (void)first_bad;
    return PUCK_OK;
  } catch (const PuckError& e) {
    set_error(e.msg);
    return e.status;
  } catch (const std::exception& e) {
    set_error(e.what());
    return PUCK_ERR_INTERNAL;
  }
}

}  // namespace

extern "C" {

void puck_default_options(puck_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->mem_bytes = 0;
  o->device = 0;
  o->profile = 0;
  o->decode = PUCK_DECODE_AUTO;
  o->max_length = 100;
  o->max_batch_sentences = 0;
  o->prune_threshold = -9.0f;
  o->use_graphs = 0;
  o->tensor_cores = 0;
  o->server_lanes = 0;
}

puck_grammar* puck_grammar_load(const char* path, puck_status* status) {
  auto* g = new puck_grammar();
  try {
    if (!path) throw PuckError{PUCK_ERR_INVALID_ARG, "null path"};
    load_grammar(g, path);
    if (status) *status = PUCK_OK;
    return g;
  } catch (const PuckError& e) {
    set_error(e.msg);
    if (status) *status = e.status;
  } catch (const std::exception& e) {
    set_error(std::string("grammar load failed: ") + e.what());
    if (status) *status = PUCK_ERR_BAD_GRAMMAR;
  }
  delete g;
  return nullptr;
}

void puck_grammar_free(puck_grammar* g) { delete g; }

int32_t puck_grammar_num_levels(const puck_grammar* g) { return g ? (int32_t)g->levels.size() : 0; }

puck_status puck_grammar_level_info(const puck_grammar* g, int32_t level, int32_t out[8]) {
  if (!g || level < 0 || level >= (int)g->levels.size() || !out) {
    set_error("bad level");
    return PUCK_ERR_INVALID_ARG;
  }
  const HostLevel& L = g->levels[level];
  int32_t v[8] = {L.semiring, L.n_nt, L.n_t, L.cell_size, L.mask_size, L.n_coarse, L.root, L.n_words};
  std::memcpy(out, v, sizeof(v));
  return PUCK_OK;
}

int32_t puck_grammar_word_id(const puck_grammar* g, const char* word) {
  if (!g || !word) return -1;
  auto it = g->word_index.find(word);
  return it == g->word_index.end() ? -1 : it->second;
}

int32_t puck_grammar_word_id_at(const puck_grammar* g, const char* word, int32_t position) {
  if (!g || !word || !*word) return -1;
  auto it = g->word_index.find(word);
  if (it != g->word_index.end()) return it->second;
  // the unknown-word class, then ever shorter prefixes of it ("UNK" last)
  std::string sig = unknown_word_class(word, position, g->word_index);
  for (;;) {
    auto s = g->word_index.find(sig);
    if (s != g->word_index.end()) return s->second;
    const size_t cut = sig.rfind('-');
    if (cut == std::string::npos) return -1;
    sig.resize(cut);
  }
}

puck_parser* puck_parser_create(const puck_grammar* g, const puck_options* opts, puck_status* status) {
  auto* P = new puck_parser();
  try {
    if (!g) throw PuckError{PUCK_ERR_INVALID_ARG, "null grammar"};
    P->g = g;
    if (opts) P->opt = *opts;
    else puck_default_options(&P->opt);
    if (P->opt.max_length <= 0) P->opt.max_length = 100;
    if (P->opt.max_length > puck::kMaxLen)
      throw PuckError{PUCK_ERR_INVALID_ARG, "max_length above " + std::to_string(puck::kMaxLen)};
    int ndev = 0;
    CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (P->opt.device < 0 || P->opt.device >= ndev) throw PuckError{PUCK_ERR_INVALID_ARG, "no such CUDA device"};
    CUDA_TRY(cudaSetDevice(P->opt.device));
    CUDA_TRY(cudaDeviceGetAttribute(&P->sms, cudaDevAttrMultiProcessorCount, P->opt.device));
    CUDA_TRY(cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking));
    const int nl = (int)g->levels.size();
    for (auto& e : P->ev_batch) CUDA_TRY(cudaEventCreate(&e));
    P->ev_level.resize(nl);
    for (auto& a : P->ev_level)
      for (auto& e : a) CUDA_TRY(cudaEventCreate(&e));
    P->pass_ms.assign(nl, std::array<double, 4>{0, 0, 0, 0});
    P->pass_launches.assign(nl, std::array<int64_t, 4>{0, 0, 0, 0});
    P->level_work.assign(nl, std::array<int64_t, 2>{0, 0});
    P->graphs.assign(nl, std::array<cudaGraphExec_t, 2>{nullptr, nullptr});
    P->tuned_mode.assign(nl, -1);
    P->flat_from.assign(nl, kNoFlat);
    for (int l = 0; l < nl; ++l) {
      P->levels.emplace_back(new LevelDev());
      LevelDev& LD = *P->levels.back();
      build_level(LD, g->levels[l], l < nl - 1 && nl != 1);
      // by default the flat-tile passes run at every span of the
      // pair-factored levels that have them
      if (LD.d.flat_inside || LD.d.flat_outside) P->flat_from[l] = 2;
      if (P->opt.tensor_cores) {
        if (l == nl - 1) LD.tc_ok = build_tc(LD, g->levels[l], &LD.tc_why);
        else LD.tc_why = "a coarse level of the cascade (it only makes masks)";
      }
    }
    P->bufs.resize(nl);
    size_t free_b = 0, total_b = 0;
    CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    const int64_t cap = (int64_t)(free_b * 0.8);
    P->budget_bytes = P->opt.mem_bytes > 0 ? std::min<int64_t>(P->opt.mem_bytes, cap) : cap;
    if (status) *status = PUCK_OK;
    return P;
  } catch (const PuckError& e) {
    set_error(e.msg);
    if (status) *status = e.status;
  }
  puck_parser_destroy(P);
  return nullptr;
}

void puck_parser_destroy(puck_parser* P) {
  if (!P) return;
  cudaSetDevice(P->opt.device);
  for (auto& b : P->bufs) {
    b.inside.release(); b.outside.release(); b.masks.release(); b.iscale.release(); b.oscale.release();
    b.part.release(); b.decode.release(); b.live_in.release(); b.live_out.release();
  }
  for (DevBuf* b : {&P->b_len, &P->b_cell_off, &P->b_word_off, &P->b_words, &P->b_work, &P->b_node_off, &P->b_mbr_off, &P->b_nodes, &P->b_status,
                    &P->b_logz, &P->b_scratch, &P->b_counters, &P->b_parts, &P->b_cell_cnt})
    b->release();
  for (auto& a : P->graphs)
    for (auto& ex : a)
      if (ex) cudaGraphExecDestroy(ex);
  P->levels.clear();
  for (auto& e : P->ev_batch)
    if (e) cudaEventDestroy(e);
  for (auto& a : P->ev_level)
    for (auto& e : a)
      if (e) cudaEventDestroy(e);
  if (P->stream) cudaStreamDestroy(P->stream);
  delete P;
}

puck_status puck_parse(puck_parser* p, const int32_t* word_ids, const int64_t* offsets, int32_t nsent,
                       puck_tree_node* nodes_out, int32_t* sent_status) {
  if (!nodes_out && nsent > 0) {
    set_error("null nodes_out");
    return PUCK_ERR_INVALID_ARG;
  }
  return run_call(p, MODE_PARSE, word_ids, offsets, nsent, nodes_out, nullptr, sent_status);
}

puck_status puck_partitions(puck_parser* p, const int32_t* word_ids, const int64_t* offsets, int32_t nsent,
                            float* log_z, int32_t* sent_status) {
  if (!log_z && nsent > 0) {
    set_error("null log_z");
    return PUCK_ERR_INVALID_ARG;
  }
  return run_call(p, MODE_PARTITIONS, word_ids, offsets, nsent, nullptr, log_z, sent_status);
}

puck_status puck_inside_outside(puck_parser* p, const int32_t* word_ids, const int64_t* offsets, int32_t nsent) {
  return run_call(p, MODE_INSIDE_OUTSIDE, word_ids, offsets, nsent, nullptr, nullptr, nullptr);
}

int64_t puck_debug_num_cells(const puck_parser* p) { return p ? p->last_num_cells : 0; }

puck_status puck_debug_copy(puck_parser* P, int32_t level, int32_t which, void* host_out, size_t bytes) {
  try {
    if (!P || level < 0 || level >= (int)P->bufs.size() || !host_out)
      throw PuckError{PUCK_ERR_INVALID_ARG, "bad debug copy arguments"};
    if (P->last_batches != 1) throw PuckError{PUCK_ERR_INVALID_ARG, "last call did not run as one batch"};
    const HostLevel& L = P->g->levels[level];
    LevelBufs& b = P->bufs[level];
    const int64_t nc = P->last_num_cells;
    const void* src = nullptr;
    size_t need = 0;
    switch (which) {
      case 0: src = b.inside.p; need = nc * L.cell_size * 4; break;
      case 1: src = b.outside.p; need = nc * L.cell_size * 4; break;
      case 2: src = b.masks.p; need = nc * L.mask_size * 4; break;
      case 3: src = b.iscale.p; need = nc * 4; break;
      case 4: src = b.oscale.p; need = nc * 4; break;
      case 5: src = b.decode.p; need = nc * 8; break;
      default: throw PuckError{PUCK_ERR_INVALID_ARG, "bad 'which'"};
    }
    if (!src) throw PuckError{PUCK_ERR_INVALID_ARG, "buffer not computed by the last call"};
    if (bytes < need) throw PuckError{PUCK_ERR_INVALID_ARG, "host buffer too small"};
    CUDA_TRY(cudaSetDevice(P->opt.device));
    CUDA_TRY(cudaMemcpyAsync(host_out, src, need, cudaMemcpyDeviceToHost, P->stream));
    CUDA_TRY(cudaStreamSynchronize(P->stream));
    return PUCK_OK;
  } catch (const PuckError& e) {
    set_error(e.msg);
    return e.status;
  }
}

puck_status puck_parser_stats(const puck_parser* p, puck_stats* out) {
  if (!p || !out) return PUCK_ERR_INVALID_ARG;
  *out = p->stats;
  return PUCK_OK;
}

puck_status puck_parser_autotune(puck_parser* P, const int32_t* word_ids, const int64_t* offsets, int32_t nsent,
                                 int32_t* chosen) {
  if (!P || nsent <= 0 || !word_ids || !offsets) {
    set_error("puck_parser_autotune: needs a non-empty sample");
    return PUCK_ERR_INVALID_ARG;
  }
  const int nl = (int)P->levels.size();
  std::vector<int32_t> st(nsent, 0);
  std::vector<puck_tree_node> nodes;
  int64_t total_nodes = 0;
  for (int i = 0; i < nsent; ++i) total_nodes += std::max<int64_t>(2 * (offsets[i + 1] - offsets[i]) - 1, 0);
  nodes.resize(std::max<int64_t>(total_nodes, 1));
  // one parse of the sample; the device time of `level`'s passes, or of the
  // whole parse with level < 0
  auto run = [&](int level) -> double {
    const puck_status r = run_call(P, MODE_PARSE, word_ids, offsets, nsent, nodes.data(), nullptr, st.data());
    if (r != PUCK_OK) return -1.0;
    if (level < 0) return P->stats.ms_device;
    return P->pass_ms[level][0] + P->pass_ms[level][1];
  };
  if (run(-1) < 0) return PUCK_ERR_CUDA;  // warm-up
  // the gather form stays the archive's choice per level (target-major or
  // pair-factored); the tuned knob is how many waves of CTAs long cells are
  // split to fill
  for (int l = 0; l < nl; ++l) P->tuned_mode[l] = P->levels[l]->d.mode;
  // waves of CTAs that split long cells
  double best = -1.0, best_w = 2.0;
  for (double w : {1.0, 2.0, 4.0}) {
    P->waves = w;
    const double t = run(-1);
    if (t < 0) return PUCK_ERR_CUDA;
    if (best < 0 || t < best) { best = t; best_w = w; }
  }
  P->waves = best_w;
  // per level with the flat-tile layout, the span band that runs it (the
  // 16 x 16 tiles: the sub-tiles of the level's pairs, or groups of 16
  // coarse ids) and the band that keeps the level's own form (the whole
  // pairs' tiles, or one rule at a time): from span 2, 8, 16 or never
  for (int l = 0; l < nl; ++l) {
    if (!P->levels[l]->flat_ready_in && !P->levels[l]->flat_ready_out) continue;
    double best_t = -1.0;
    int best_f = P->flat_from[l];
    for (int f : {2, 8, 16, kNoFlat}) {
      P->flat_from[l] = f;
      const double t = run(-1);
      if (t < 0) return PUCK_ERR_CUDA;
      if (best_t < 0 || t < best_t) { best_t = t; best_f = f; }
    }
    P->flat_from[l] = best_f;
  }
  if (chosen) {
    for (int l = 0; l < nl; ++l) chosen[l] = P->tuned_mode[l];
    chosen[nl] = (int32_t)(best_w * 100);
  }
  return PUCK_OK;
}

puck_status puck_parser_set_flat_from(puck_parser* p, int32_t level, int32_t span) {
  if (!p || level < 0 || level >= (int)p->levels.size() || span < 0 || span == 1 ||
      (span > 0 && !p->levels[level]->flat_ready_in && !p->levels[level]->flat_ready_out)) {
    set_error("puck_parser_set_flat_from: bad level or span, or a level without the flat-tile layout");
    return PUCK_ERR_INVALID_ARG;
  }
  p->flat_from[level] = span == 0 ? kNoFlat : span;
  return PUCK_OK;
}

int32_t puck_debug_flat_check(const puck_grammar* g, int32_t level, int32_t job, int32_t form, int64_t out[4]) {
  try {
    if (!g || level < 0 || level >= (int)g->levels.size() || job < 0 || job >= puck::NJOBS || form < 0 ||
        form > 2 || (form == 1 && job > 3))
      return -3;
    static const bool a_t[puck::NJOBS] = {false, false, true, true, false, false, false, false, false, true, false, true};
    static const bool b_t[puck::NJOBS] = {false, true, false, true, false, false, true, false, false, false, true, false};
    const HostLevel& L = g->levels[level];
    const std::string n = kJobNames[job];
    const float pad_w = L.semiring == puck::SEMI_REAL ? 0.f : -INFINITY;
    int64_t nseg = 0;
    L.get<int>(n + "/seg_bits", "i4", &nseg);
    nseg /= std::max(1, L.mask_size);
    int64_t nrow = 0;
    const int* rowptr = L.get<int>(n + "/rowptr", "i4", &nrow);
    const int* ab = L.get<int>(n + "/ab", "i4", nullptr);
    const float* wr = L.get<float>(n + "/w", "f4", nullptr);
    using R = std::array<int64_t, 4>;
    std::vector<R> got, want;
    for (int t = 0; t + 1 < nrow; ++t)
      for (int r = rowptr[t]; r < rowptr[t + 1]; ++r) {
        uint32_t bits;
        std::memcpy(&bits, &wr[r], 4);
        want.push_back(R{t, ab[r] & 0xffff, (int64_t)((unsigned)ab[r] >> 16), bits});
      }
    std::sort(want.begin(), want.end());
    if (form == 2) {  // the pair-major tables: every pair's rules, pairs distinct
      std::vector<int> pab, poff;
      std::vector<int2> prule;
      if (!pm_tables_host(L, job, pab, poff, prule)) return -1;
      for (size_t p = 0; p < pab.size(); ++p) {
        if (p > 0 && pab[p] == pab[p - 1]) return -2;
        for (int r = poff[p]; r < poff[p + 1]; ++r)
          got.push_back(R{prule[r].x, pab[p] & 0xffff, (int64_t)((unsigned)pab[p] >> 16), (uint32_t)prule[r].y});
      }
      std::sort(got.begin(), got.end());
      if (out) {
        out[0] = (int64_t)got.size();
        out[1] = (int64_t)pab.size();
        out[2] = out[3] = 0;
      }
      return got == want ? 0 : -2;
    }
    FlatHost F;
    bool ok;
    if (form == 1) {
      ok = group_tiles_host(F, L, job, (int)nseg, false);
    } else {
      int64_t npk = 0;
      const int* pk = L.get<int>(n + "/pair_key", "i4", &npk);
      ok = flat_tiles_host(F, (int)(nrow - 1), npk, pk, L.get<int>(n + "/pair_blk", "i4", nullptr),
                           L.get<int>(n + "/blk_seg", "i4", nullptr), L.get<int>(n + "/blk_ptr", "i4", nullptr),
                           L.get<int>(n + "/pair_rule", "i4", nullptr), L.get<float>(n + "/pair_w", "f4", nullptr),
                           L.get<int>(n + "/seg_bits", "i4", nullptr), (int)nseg, L.mask_size,
                           L.get<int>(a_t[job] ? "t_mem_off" : "nt_mem_off", "i4", nullptr),
                           L.get<int>(a_t[job] ? "t_mem" : "nt_mem", "i4", nullptr),
                           L.get<int>(b_t[job] ? "t_mem_off" : "nt_mem_off", "i4", nullptr),
                           L.get<int>(b_t[job] ? "t_mem" : "nt_mem", "i4", nullptr), pad_w);
    }
    if (!ok) return -1;
    // every rule the tables hold, as (target, a, b, weight bits), against the
    // job's target-major rule table
    int64_t records = 0;
    for (const int4& D : F.desc) {
      const int a_first = D.x & 0xffff, b_first = (int)((unsigned)D.x >> 16);
      const int sy = D.z & 255, sz = (D.z >> 8) & 255, nb = (int)((unsigned)D.z >> 16);
      for (int q = D.y; q < D.y + nb; ++q) {
        const int4 B = F.blk[q];
        std::vector<int> tg;
        for (int g0 = B.y; g0 < B.z; ++g0) {
          ++records;
          const int lane = (g0 - B.y) % 32, t = F.tgt[(size_t)q * 32 + lane];
          for (int c = 0; c < 4; ++c) {
            const float wt = (&F.w[g0].x)[c];
            if (wt == pad_w || (std::isinf(pad_w) && std::isinf(wt) && wt < 0)) continue;
            const int e = (int)((F.idx[g0] >> (8 * c)) & 255u);
            if (t < 0 || e >= sy * sz) return -2;
            uint32_t bits;
            std::memcpy(&bits, &wt, 4);
            got.push_back(R{t, a_first + e / sz, b_first + e % sz, bits});
            tg.push_back(t);
          }
        }
        std::sort(tg.begin(), tg.end());
        if (std::unique(tg.begin(), tg.end()) - tg.begin() > 32) return -2;
      }
    }
    std::sort(got.begin(), got.end());
    if (out) {
      out[0] = (int64_t)got.size();
      out[1] = (int64_t)F.desc.size();
      out[2] = (int64_t)F.blk.size();
      out[3] = records;
    }
    return got == want ? 0 : -2;
  } catch (const PuckError& e) {
    set_error(e.msg);
    return -3;
  }
}

int32_t puck_parser_flat_from(const puck_parser* p, int32_t level) {
  if (!p || level < 0 || level >= (int)p->levels.size()) return -1;
  const LevelDev& L = *p->levels[level];
  return (L.flat_ready_in || L.flat_ready_out) && p->flat_from[level] < kNoFlat ? p->flat_from[level] : 0;
}

int32_t puck_parser_tensor_cores(const puck_parser* p, int32_t level, char* why, size_t len) {
  if (!p || level < 0 || level >= (int)p->levels.size()) return -1;
  const LevelDev& L = *p->levels[level];
  if (why && len) {
    const std::string m = L.tc_ok ? std::string() : (p->opt.tensor_cores ? L.tc_why : "tensor cores not requested");
    const size_t k = std::min(len - 1, m.size());
    std::memcpy(why, m.data(), k);
    why[k] = 0;
  }
  return L.tc_ok ? 1 : 0;
}

puck_status puck_parser_level_work(const puck_parser* p, int32_t level, int64_t out[2]) {
  if (!p || !out || level < 0 || level >= (int)p->level_work.size()) {
    set_error("bad level");
    return PUCK_ERR_INVALID_ARG;
  }
  out[0] = p->level_work[level][0];
  out[1] = p->level_work[level][1];
  return PUCK_OK;
}

puck_status puck_parser_pass_ms(const puck_parser* p, int32_t level, double out[4], int64_t launches[4]) {
  if (!p || level < 0 || level >= (int)p->pass_ms.size()) {
    set_error("bad level");
    return PUCK_ERR_INVALID_ARG;
  }
  for (int k = 0; k < 4; ++k) {
    if (out) out[k] = p->pass_ms[level][k];
    if (launches) launches[k] = p->pass_launches[level][k];
  }
  return PUCK_OK;
}

size_t puck_last_error(char* buf, size_t len) {
  if (buf && len) {
    size_t n = std::min(len - 1, g_last_error.size());
    std::memcpy(buf, g_last_error.data(), n);
    buf[n] = 0;
  }
  return g_last_error.size();
}

}  // extern "C"
