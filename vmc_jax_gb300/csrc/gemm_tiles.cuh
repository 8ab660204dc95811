// Tile order of the tcgen05 GEMM (gemm_tc.cu), shared with the host so the
// grid size and the block -> tile map come from one definition.  Plain C++
// when compiled without nvcc.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define VMC_TILE_FN __host__ __device__
#else
#define VMC_TILE_FN
#endif

namespace vmc {

// Tile order.  Column tiles are taken in groups of TC_GROUP; inside a group
// the tiles run row by row (tm outer, tn inner), so the CTAs resident at one
// time cover about 19 row tiles x 8 column tiles and share their operand
// panels through L2 (a column-at-a-time order streams ~150 distinct A panels
// per wave from DRAM).
//
// Symmetric product (mode 0): only tiles touching the upper triangle,
// column tile tn holds the row tiles tm < 2 tn + 2 (BN = 2 BM), capped at
// tilesM; equivalently row tm meets the column tiles tn >= tm / 2.  A group
// [c0, c1) has full rows tm < min(R, 2 c0) (all w = c1 - c0 tiles) and at
// most 2 w ragged rows after them, R = min(tilesM, 2 c1).
constexpr int TC_GROUP = 8;

VMC_TILE_FN inline int sym_group_size(int c0, int c1, int tilesM, int& full) {
  const int R = tilesM < 2 * c1 ? tilesM : 2 * c1;
  full = R < 2 * c0 ? R : 2 * c0;
  int n = (c1 - c0) * full;
  for (int tm = full; tm < R; ++tm) n += c1 - tm / 2;
  return n;
}

VMC_TILE_FN inline void tile_of(int b, int mode, int tilesM, int tilesN, int& tm, int& tn) {
  if (mode != 0) {
    const int per = TC_GROUP * tilesM;
    const int g = b / per, o = b - g * per;
    const int c0 = g * TC_GROUP;
    const int w = tilesN - c0 < TC_GROUP ? tilesN - c0 : TC_GROUP;
    tm = o / w;
    tn = c0 + (o - tm * w);
    return;
  }
  int o = b;
  for (int c0 = 0; c0 < tilesN; c0 += TC_GROUP) {
    const int c1 = c0 + TC_GROUP < tilesN ? c0 + TC_GROUP : tilesN;
    int full;
    const int n = sym_group_size(c0, c1, tilesM, full);
    if (o >= n) {
      o -= n;
      continue;
    }
    const int w = c1 - c0;
    if (o < w * full) {
      tm = o / w;
      tn = c0 + (o - tm * w);
      return;
    }
    o -= w * full;
    for (int r = full;; ++r) {
      const int cnt = c1 - r / 2;
      if (o < cnt) {
        tm = r;
        tn = r / 2 + o;
        return;
      }
      o -= cnt;
    }
  }
  tm = tn = 0;  // not reached for b < number of tiles
}

inline int64_t tile_count(int mode, int tilesM, int tilesN) {
  if (mode != 0) return (int64_t)tilesM * tilesN;
  int64_t n = 0;
  for (int tn = 0; tn < tilesN; ++tn) n += tilesM < 2 * tn + 2 ? tilesM : 2 * tn + 2;
  return n;
}

}  // namespace vmc
