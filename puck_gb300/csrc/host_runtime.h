// Host-side pieces shared by the batch runtime and the serving loop: error
// type, grammar levels as loaded from grammar.grz, device buffers and the
// per-level device tables.
#pragma once

#include "puck_internal.h"
#include "../../include/puck_gpu.h"

#include <algorithm>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

namespace puck_host {

struct PuckError {
  puck_status status;
  std::string msg;
};

#define CUDA_TRY(expr)                                                                          \
  do {                                                                                          \
    cudaError_t _e = (expr);                                                                    \
    if (_e != cudaSuccess)                                                                      \
      throw PuckError{_e == cudaErrorMemoryAllocation ? PUCK_ERR_OOM : PUCK_ERR_CUDA,           \
                      std::string(#expr) + ": " + cudaGetErrorString(_e)};                      \
  } while (0)

struct Array {
  char tag[5] = {0};
  std::vector<char> bytes;
  int64_t count = 0;
};

struct HostLevel {
  int semiring = 0, n_nt = 0, n_t = 0, cell_size = 0, mask_size = 0, n_coarse = 0, root = 0, n_words = 0;
  std::map<std::string, Array> arrays;
  std::vector<std::string> words;

  template <class T>
  const T* get(const std::string& name, const char* tag, int64_t* count) const {
    auto it = arrays.find(name);
    if (it == arrays.end()) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "missing array " + name};
    if (std::strncmp(it->second.tag, tag, 2) != 0) throw PuckError{PUCK_ERR_BAD_GRAMMAR, "bad dtype for " + name};
    if (count) *count = it->second.count;
    return reinterpret_cast<const T*>(it->second.bytes.data());
  }
};

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  void ensure(size_t bytes) {
    if (bytes <= cap) return;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = std::max<size_t>(bytes + bytes / 8, 256);
    CUDA_TRY(cudaMalloc(&p, want));
    cap = want;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <class T> T* as() const { return reinterpret_cast<T*>(p); }
};

struct LevelDev {
  std::vector<void*> allocs;
  puck::DevLevel d{};
  puck::DevTc tc{};
  bool tc_ok = false;     // the tensor-core tables were built
  bool flat_ready_in = false;   // every inside job with rules has the flat-tile layout (DevJob::flat)
  bool flat_ready_out = false;  // every outside job with rules has it
  std::string tc_why;     // else why not
  void* upload(const void* src, size_t bytes) {
    void* p = nullptr;
    CUDA_TRY(cudaMalloc(&p, std::max<size_t>(bytes, 16)));
    allocs.push_back(p);
    if (bytes) CUDA_TRY(cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice));
    return p;
  }
  ~LevelDev() {
    for (void* p : allocs) cudaFree(p);
  }
};

// Uploads a level's tables (rule CSR, pair tables, lexicon, Viterbi tables).
void build_level(LevelDev& D, const HostLevel& L, bool merged);
// Uploads a sum-product level's tensor-core tables (DevTc) after build_level;
// false, with the reason, if the level's structure is not covered.
bool build_tc(LevelDev& D, const HostLevel& L, std::string* why);

}  // namespace puck_host

struct puck_grammar {
  std::vector<puck_host::HostLevel> levels;
  std::unordered_map<std::string, int> word_index;
};
