// Application of one branch-free operator string to one configuration
// (operator/branch_free.py:443-487).
#pragma once

#include "vmc_common.cuh"

namespace vmc {

// Result of applying one string: matrix element and the sites whose local
// state was written (with their final values).  Strings are at most
// VMC_BF_MAX_LEN operators long, so at most that many distinct sites change.
struct bf_string_result {
  cpx<double> m;
  int nmod;
  int site[VMC_BF_MAX_LEN];
  int val[VMC_BF_MAX_LEN];
};

// cfg: the configuration's local states (shared memory), occ: bitmask of
// sites with state 1 (used only by fermionic strings), L sites.
// The string's operators are applied in table order (the tables hold the
// string right-to-left): m *= mat_els[current] * fermion_sign, then
// state = map[current].  The fermion sign is (-1)^(number of occupied sites
// j > idx) of the current configuration (branch_free.py:463-466).
__device__ __forceinline__ void bf_apply_string(const vmc_bf_operator& op, int o, const int8_t* cfg,
                                                const uint32_t* occ, int L, bf_string_result& r) {
  const double2* me = reinterpret_cast<const double2*>(op.mat_els);
  const double2 pf = reinterpret_cast<const double2*>(op.prefactor)[o];
  cpx<double> m = mk(pf.x, pf.y);
  int nmod = 0;
  const int ml = op.max_len, ld = op.local_dim;
  for (int k = 0; k < ml; ++k) {
    const int e = o * ml + k;
    const int i = op.idx[e];
    if (i < 0 || i >= L) {  // malformed table: poison the element, touch nothing
      m = mk(nan(""), nan(""));
      continue;
    }
    int cur = cfg[i];
    int slot = -1;
    for (int q = 0; q < nmod; ++q)
      if (r.site[q] == i) {
        cur = r.val[q];
        slot = q;
      }
    double sign = 1.0;
    if (op.fermi[e]) {
      // occupied sites above i in the original configuration ...
      int cnt = 0;
      int w0 = (i + 1) >> 5;
      int nw = (L + 31) >> 5;
      if (w0 < nw) {
        uint32_t first = occ[w0] & (0xffffffffu << ((i + 1) & 31));
        cnt += __popc(first);
        for (int w = w0 + 1; w < nw; ++w) cnt += __popc(occ[w]);
      }
      // ... corrected by the sites this string already changed
      for (int q = 0; q < nmod; ++q)
        if (r.site[q] > i) cnt += r.val[q] - cfg[r.site[q]];
      if (cnt & 1) sign = -1.0;
    }
    if (cur < 0 || cur >= ld) {  // local state outside [0, lDim)
      m = mk(nan(""), nan(""));
      continue;
    }
    double2 x = me[e * ld + cur];
    m = m * mk(x.x, x.y);
    m = mk(m.re * sign, m.im * sign);
    int nv = op.map[e * ld + cur];
    if (slot >= 0) {
      r.val[slot] = nv;
    } else {
      r.site[nmod] = i;
      r.val[nmod] = nv;
      ++nmod;
    }
  }
  r.m = m;
  r.nmod = nmod;
}

// Load one configuration (int32) into shared int8 storage and its
// occupancy bitmask; executed by one warp.
__device__ __forceinline__ void warp_load_config(const int32_t* __restrict__ src, int L, int8_t* cfg, uint32_t* occ,
                                                 int lane) {
  for (int i = lane; i < L; i += 32) cfg[i] = (int8_t)src[i];
  int nw = (L + 31) >> 5;
  for (int w = 0; w < nw; ++w) {
    int i = w * 32 + lane;
    unsigned b = __ballot_sync(0xffffffffu, i < L && src[i] == 1);
    if (lane == 0) occ[w] = b;
  }
  __syncwarp();
}

}  // namespace vmc
