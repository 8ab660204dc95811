// FP64-accurate complex products on the BF16 tensor cores (included by
// gemm_tc.cu, which defines the tcgen05 / TMA / mbarrier helpers and the
// wait-limit variable these kernels share).
//
// C = P^H Q for complex P (K x M) and Q (K x N) given in FP64.  Written as
// real products: with P = Pr + i Pi and Q = Qr + i Qi,
//   Re C = [Pr; Pi]^T [Qr; Qi],   Im C = [Pr; Pi]^T [Qi; -Qr],
// i.e. one real product of an M x 2K operand ("A rows") with a 2N x 2K
// operand ("B rows", the Re C columns first, then the Im C columns).
//
// Ozaki splitting (Ozaki, Ogita, Oishi, Rump, Numer. Algorithms 59 (2012)):
// every operand row is scaled by a power of two 2^e (e per row) so that its
// entries lie in (-1, 1) and cut into s slices of 7 bits,
//   x = 2^e sum_i n_i 2^(-7(i+1)),  n_0 in [-128, 128], |n_i| <= 64 (i > 0),
// each slice stored as the bf16 value n_i 2^(-7(i+1)) (exact: 8 significant
// bits).  The product is the sum over slice pairs (i, j) of A_i B_j^T; pairs
// of one level d = i + j share the unit 2^(-7(d+2)).  Products of slices are
// exact in the tensor core and a level's sum over a K range of length
// chunk(d) stays below 2^24 units, so the FP32 TMEM accumulator holds it
// exactly.  After each such group the epilogue converts the accumulator to an
// int32 count of level units (exact) and adds it to per-element int64 sums
// held in registers, in units of 2^-lsb with lsb the largest for which
// 1.02 K2 2^lsb < 2^63 (47 for K2 = 33,280): shifted left (exact) for the
// levels with 7 (d + 2) <= lsb, shifted right with rounding below.  Levels
// above maxLevel are dropped (their sum is below 2^(-7(maxLevel+1)) relative
// to the row and column scales).
//
// Kernel: persistent, 128 x 128 output tiles, one tcgen05.mma M=128 N=128
// K=16 per 16 columns of a stage; stage = one 64-column block of one A slice
// and one B slice (2 x 16 KB), 6-stage TMA ring.  Warp 0: TMA producer;
// warp 1: TMEM owner and MMA issuer (two 128-column accumulators, so the
// epilogue of one group overlaps the MMAs of the next); warps 2..9:
// epilogue, warp w reading TMEM lanes 32 (w % 4) .. +31 and columns
// 64 ((w - 2) / 4) .. +63.  Tiles are taken in groups of OZ_GROUP complex
// column blocks, row by row inside a group, so the CTAs resident at one time
// share their operand panels through L2.
#pragma once

namespace vmc {

constexpr int OZ_BM = 128, OZ_BN = 128, OZ_BK = 64, OZ_STAGES = 6, OZ_GROUP = 12;
constexpr int OZ_TILE_BYTES = OZ_BM * OZ_BK * 2;   // 16 KB, A and B tiles alike
constexpr int OZ_STAGE_BYTES = 2 * OZ_TILE_BYTES;
constexpr int OZ_EPI_WARPS = 8;
constexpr int OZ_THREADS = 64 + 32 * OZ_EPI_WARPS;
constexpr int OZ_SMEM = OZ_STAGES * OZ_STAGE_BYTES + 1024 + 256;
constexpr uint32_t OZ_TMEM_COLS = 256;
constexpr int OZ_BITS = 7;
constexpr int OZ_MAX_SLICES = 8;

// K columns of one exactly accumulated group of level d (a multiple of the
// 64-column stage): (d + 1) * chunk * 2^14 <= 2^24.
__host__ __device__ constexpr int oz_chunk(int d) { return (1024 / (d + 1)) & ~63; }

struct oz_args {
  int M, K2;               // output rows; reduction length (2K, padded to 64)
  int halfTiles;           // 128-column tiles per half (Re C | Im C) of the output
  int tilesM;
  int slicesA, slicesB, maxLevel;
  int hermitian;           // 1: only tiles whose complex column block >= the row block
  int numTiles;
  int lsb;                 // int64 sums count units of 2^-lsb
  const int* ea;           // per output row: scale exponent
  const int* eb;           // per complex output column
  double* out;             // M x (2 * halfTiles * 128) FP64, row-major, ld = ldo
  int64_t ldo;
  int* status;
};

// Tile t of the launch -> (row block, column tile).  Column tiles come in
// groups of OZ_GROUP complex column blocks (both halves of each); inside a
// group, row by row.
__host__ __device__ inline void oz_tile(int t, const oz_args& a, int& tm, int& tn) {
  for (int c0 = 0; c0 < a.halfTiles; c0 += OZ_GROUP) {
    const int c1 = c0 + OZ_GROUP < a.halfTiles ? c0 + OZ_GROUP : a.halfTiles;
    for (int r = 0; r < a.tilesM; ++r) {
      int lo = c0;
      if (a.hermitian && r > lo) lo = r;
      const int w = c1 > lo ? c1 - lo : 0;
      if (t < 2 * w) {
        tm = r;
        const int c = lo + (t >> 1);
        tn = (t & 1) ? a.halfTiles + c : c;
        return;
      }
      t -= 2 * w;
    }
  }
  tm = tn = 0;
}

inline int oz_tile_count(int tilesM, int halfTiles, int hermitian) {
  int n = 0;
  for (int r = 0; r < tilesM; ++r) {
    const int lo = hermitian ? r : 0;
    if (halfTiles > lo) n += 2 * (halfTiles - lo);
  }
  return n;
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(dst),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
      : "memory");
}

// Slice pairs (i, d - i) of level d: i in [oz_pair_lo, oz_pair_hi].  Every
// role of the kernel walks the same sequence: tiles, levels, K ranges of
// oz_chunk(d) columns, pairs, 64-column stages.
__device__ __forceinline__ int oz_pair_lo(const oz_args& a, int d) {
  const int lo = d - (a.slicesB - 1);
  return lo > 0 ? lo : 0;
}
__device__ __forceinline__ int oz_pair_hi(const oz_args& a, int d) {
  return d < a.slicesA - 1 ? d : a.slicesA - 1;
}

__global__ void __launch_bounds__(OZ_THREADS, 1)
    oz_gemm_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, oz_args a) {
  extern __shared__ __align__(1024) unsigned char oz_smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(oz_smem_raw) + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + OZ_STAGES * OZ_STAGE_BYTES);
  // bars[0..S): stage full, [S..2S): stage empty, [2S..2S+2): accumulator
  // full, [2S+2..2S+4): accumulator empty, [2S+4]: all MMAs done (teardown)
  uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(bars + 2 * OZ_STAGES + 5);
  volatile int* abortFlag = reinterpret_cast<volatile int*>(tmemSlot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint64_t* full = bars;
  uint64_t* empty = bars + OZ_STAGES;
  uint64_t* accFull = bars + 2 * OZ_STAGES;
  uint64_t* accEmpty = accFull + 2;
  uint64_t* mmaDone = accFull + 4;

  if (threadIdx.x == 0) {
    for (int s = 0; s < OZ_STAGES; ++s) {
      mbar_init(smem_u32(&full[s]), 1);
      mbar_init(smem_u32(&empty[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&accFull[b]), 1);
      mbar_init(smem_u32(&accEmpty[b]), OZ_EPI_WARPS);
    }
    mbar_init(smem_u32(mmaDone), 1);
    *abortFlag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmemSlot)),
                 "r"(OZ_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmemSlot;

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      uint32_t it = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < a.numTiles && ok; t += gridDim.x) {
        int tm, tn;
        oz_tile(t, a, tm, tn);
        for (int d = 0; d <= a.maxLevel && ok; ++d) {
          const int ilo = oz_pair_lo(a, d), ihi = oz_pair_hi(a, d);
          if (ilo > ihi) continue;
          const int ch = oz_chunk(d);
          for (int k0 = 0; k0 < a.K2 && ok; k0 += ch) {
            const int k1 = k0 + ch < a.K2 ? k0 + ch : a.K2;
            for (int i = ilo; i <= ihi && ok; ++i) {
              for (int k = k0; k < k1; k += OZ_BK, ++it) {
                const int s = it % OZ_STAGES;
                const uint32_t ph = (it / OZ_STAGES) & 1u;
                if (*abortFlag || !mbar_wait(smem_u32(&empty[s]), ph ^ 1u, 11, a.status)) {
                  ok = false;
                  break;
                }
                const uint32_t fb = smem_u32(&full[s]);
                mbar_expect_tx(fb, OZ_STAGE_BYTES);
                unsigned char* st = smem + s * OZ_STAGE_BYTES;
                tma_load_3d(smem_u32(st), &mapA, k, tm * OZ_BM, i, fb);
                tma_load_3d(smem_u32(st + OZ_TILE_BYTES), &mapB, k, tn * OZ_BN, d - i, fb);
              }
            }
          }
        }
      }
      if (!ok) {
        *abortFlag = 1;
        // the copies issued last may still be in flight: let them land
        const uint32_t first = it > (uint32_t)OZ_STAGES ? it - OZ_STAGES : 0u;
        for (uint32_t j = first; j < it; ++j)
          mbar_wait_for(smem_u32(&full[j % OZ_STAGES]), (j / OZ_STAGES) & 1u, 12, a.status, TC_DRAIN_NS);
      }
    }
  } else if (warp == 1) {
    // ----------------------------------------------------------- MMA issue
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_bf16_f32(OZ_BM, OZ_BN);
      uint32_t it = 0, g = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < a.numTiles && ok; t += gridDim.x) {
        for (int d = 0; d <= a.maxLevel && ok; ++d) {
          const int ilo = oz_pair_lo(a, d), ihi = oz_pair_hi(a, d);
          if (ilo > ihi) continue;
          const int ch = oz_chunk(d);
          for (int k0 = 0; k0 < a.K2 && ok; k0 += ch, ++g) {
            const int k1 = k0 + ch < a.K2 ? k0 + ch : a.K2;
            const uint32_t b = g & 1u;
            if (*abortFlag || !mbar_wait(smem_u32(&accEmpty[b]), ((g >> 1) & 1u) ^ 1u, 13, a.status)) {
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t acc = tmem + b * OZ_BN;
            bool first = true;
            for (int i = ilo; i <= ihi && ok; ++i) {
              for (int k = k0; k < k1; k += OZ_BK, ++it) {
                const int s = it % OZ_STAGES;
                const uint32_t ph = (it / OZ_STAGES) & 1u;
                if (*abortFlag || !mbar_wait(smem_u32(&full[s]), ph, 14, a.status)) {
                  ok = false;
                  break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                unsigned char* st = smem + s * OZ_STAGE_BYTES;
                const uint64_t da = smem_desc_sw128(smem_u32(st));
                const uint64_t db = smem_desc_sw128(smem_u32(st + OZ_TILE_BYTES));
#pragma unroll
                for (int kk = 0; kk < OZ_BK / 16; ++kk) {
                  const uint64_t o = (uint64_t)(2 * kk);
                  mma_bf16(acc, da + o, db + o, idesc, first ? 0u : 1u);
                  first = false;
                }
                mma_commit(smem_u32(&empty[s]));
              }
            }
            if (ok) mma_commit(smem_u32(&accFull[b]));
          }
        }
      }
      if (!ok) *abortFlag = 1;
      // completes once every MMA issued above has finished
      mma_commit(smem_u32(mmaDone));
      mbar_wait_for(smem_u32(mmaDone), 0u, 15, a.status, TC_DRAIN_NS);
    }
  } else {
    // ------------------------------------------------------------ epilogue
    const int ew = warp - 2;
    const int q = warp & 3;           // TMEM lane quadrant of this warp
    const int half = ew >> 2;         // 64-column half of the tile
    const int row = q * 32 + lane;
    long long sum[64];
    uint32_t g = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < a.numTiles && ok; t += gridDim.x) {
      int tm, tn;
      oz_tile(t, a, tm, tn);
#pragma unroll
      for (int c = 0; c < 64; ++c) sum[c] = 0;
      for (int d = 0; d <= a.maxLevel && ok; ++d) {
        const int ilo = oz_pair_lo(a, d), ihi = oz_pair_hi(a, d);
        if (ilo > ihi) continue;
        const int ch = oz_chunk(d);
        // the group's sum is q 2^(-7(d+2)) with q an integer, |q| <= 2^24:
        // q converts exactly to int32 and enters the 2^-lsb sums shifted left
        // (exact) or, for the levels below 2^-lsb, shifted right with rounding
        const float toUnits = __int_as_float((127 + OZ_BITS * (d + 2)) << 23);
        const int sh = a.lsb - OZ_BITS * (d + 2);
        for (int k0 = 0; k0 < a.K2 && ok; k0 += ch, ++g) {
          const uint32_t b = g & 1u;
          if (*abortFlag || !mbar_wait(smem_u32(&accFull[b]), (g >> 1) & 1u, 16, a.status)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t base = tmem + ((uint32_t)(q * 32) << 16) + b * OZ_BN + half * 64;
#pragma unroll
          for (int c0 = 0; c0 < 64; c0 += 16) {
            float v[16];
            tmem_ld16(base + c0, v);
            if (sh >= 0) {
#pragma unroll
              for (int c = 0; c < 16; ++c) sum[c0 + c] += (long long)__float2int_rn(v[c] * toUnits) << sh;
            } else {
              const int rs = -sh, hf = 1 << (rs - 1);
#pragma unroll
              for (int c = 0; c < 16; ++c) sum[c0 + c] += (long long)((__float2int_rn(v[c] * toUnits) + hf) >> rs);
            }
          }
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&accEmpty[b])) : "memory");
        }
      }
      if (!ok) break;
      const int gr = tm * OZ_BM + row;
      if (gr < a.M) {
        const int colBase = tn * OZ_BN + half * 64;
        const int cc = (tn >= a.halfTiles ? tn - a.halfTiles : tn) * OZ_BN + half * 64;  // complex column
        const int er = a.ea[gr];
        double* dst = a.out + (int64_t)gr * a.ldo + colBase;
#pragma unroll
        for (int c = 0; c < 64; c += 2) {
          const double v0 = ldexp((double)sum[c], er + a.eb[cc + c] - a.lsb);
          const double v1 = ldexp((double)sum[c + 1], er + a.eb[cc + c + 1] - a.lsb);
          *reinterpret_cast<double2*>(dst + c) = make_double2(v0, v1);
        }
      }
    }
    if (!ok) *abortFlag = 1;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(OZ_TMEM_COLS) : "memory");
  }
}

}  // namespace vmc
