// Per-sentence max-constituent (MBR) decode shared by the MBR kernels:
// the host CKY of the reference's extractMBRParses (dlwh/puck,
// src/main/scala/puck/parser/CLParser.scala:589-696), run by one thread per
// sentence over the per-cell best coarse marginals {score, symbol}.
#pragma once

#include "device_common.cuh"

namespace puck {
namespace dev {

// Scratch per sentence of length n: 3 * (n+1)^2 floats (best scores, best
// splits, unary flags).  Cells are laid out as a bot half then a top half
// starting at `off`; the 2n-1 preorder nodes go to `out`.
__device__ inline void mbr_decode_sentence(int n, long long off, const float2* decode, const float* iscale,
                                           const float* oscale, int scaling, float* scratch, DevNode* out) {
  const long long toff = off + tri(n);
  float* bs = scratch;
  int* bsplit = reinterpret_cast<int*>(bs + (n + 1) * (n + 1));
  int* uu = bsplit + (n + 1) * (n + 1);
  auto idx = [n](int x, int y) { return x * (n + 1) + y; };
  const float root_i = scaling ? iscale[toff + chart_index(0, n, n)] : 0.f;
  for (int span = 1; span <= n; ++span) {
    for (int bg = 0; bg + span <= n; ++bg) {
      const int en = bg + span;
      const long long ct = toff + chart_index(bg, en, n), cb = off + chart_index(bg, en, n);
      float topS = decode[ct].x, botS = decode[cb].x;
      if (scaling) {
        // CLParser.scala:613-614: the scales are summed in FP32 (Scala Float
        // arithmetic), exponentiated with math.exp in FP64 and rounded to
        // FP32; the one FP64 exp per cell reproduces that factor
        const float at = (iscale[ct] + oscale[ct]) - root_i, ab = (iscale[cb] + oscale[cb]) - root_i;
        topS *= (float)exp((double)at);
        botS *= (float)exp((double)ab);
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
  int stack_b[kMaxLen + 1], stack_e[kMaxLen + 1];
  int top = 1, p = 0;
  stack_b[0] = 0;
  stack_e[0] = n;
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
      stack_b[top] = sp;
      stack_e[top] = en;
      ++top;
      stack_b[top] = bg;
      stack_e[top] = sp;
      ++top;
    }
  }
}

}  // namespace dev
}  // namespace puck
