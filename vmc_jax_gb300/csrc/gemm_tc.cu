// Split-precision BF16 GEMMs on the 5th-generation tensor cores (tcgen05,
// TMEM accumulators, TMA operand staging) for the two dense contractions of
// the TDVP step:
//
//   S build  (stats.py:52-58 via tdvp.py:142):  G = R R^T with R the
//            transposed real representation [Re X | Im X]^T (2P x N) of the
//            centred, weighted log-derivatives; only tiles touching the upper
//            triangle are computed.
//   SNR      (stats.py:75-83 via tdvp.py:175-179): colsq_c = sum_n D_nc^2
//            with D = A B^T, A the SNR data (N x 2P), B^T the real
//            representation of the eigenvectors; D is never stored.
//
// Every operand x is given as two BF16 planes x ~ hi + lo and the product is
// formed as hi.hi + hi.lo + lo.hi accumulating into the same FP32 TMEM tile:
// about 16 significant bits per operand instead of 8 (products = 3), or as
// hi.hi alone with the lo planes not read (products = 1: plain BF16).
//
// Tile: 128 x 256 x 64 (one tcgen05.mma M=128 N=256 per 16-wide K slice).
// A pipeline stage holds all four operand tiles of one 64-wide K block
// (A hi, A lo, B hi, B lo: 96 KB), so each plane is read from L2 once per K
// block and the stage feeds 12 MMAs (3 products x 4 slices); 2-stage TMA ->
// shared memory ring (128-byte swizzle, K-major).  Warp 0: TMA producer;
// warp 1: TMEM owner and MMA issuer; warps 2-5: epilogue (tcgen05.ld of the
// 128 x 256 FP32 accumulator).  Every mbarrier wait is bounded by
// vmc_tc_wait_limit_ns of %globaltimer time (host-settable, 2 s by default);
// a wait that runs out writes its code to the call's status word (or to the
// library-wide flag when the caller passed none) and the CTA unwinds.  The
// unwinding itself first lets every TMA copy and MMA already issued finish
// (waits bounded by a fixed 2 s, independent of the settable limit), so
// shared memory and TMEM are never released under asynchronous writes.
#include <cuda.h>
#include <cuda_bf16.h>

#include <atomic>
#include <cmath>

#include "gemm_tiles.cuh"
#include "vmc_common.cuh"

namespace vmc {

constexpr int TC_BM = 128, TC_BN = 256, TC_BK = 64, TC_STAGES = 2;
constexpr int TC_A_BYTES = TC_BM * TC_BK * 2;                 // 16 KB per plane
constexpr int TC_B_BYTES = TC_BN * TC_BK * 2;                 // 32 KB per plane
constexpr int TC_STAGE_BYTES = 2 * TC_A_BYTES + 2 * TC_B_BYTES;  // 96 KB: A hi, A lo, B hi, B lo
constexpr int TC_SMEM = TC_STAGES * TC_STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
constexpr int TC_THREADS = 192;
constexpr uint32_t TC_TMEM_COLS = 256;
constexpr unsigned long long TC_DRAIN_NS = 2000000000ull;  // waits on work already issued, when unwinding

__device__ int vmc_tc_error = 0;
__device__ unsigned long long vmc_tc_wait_limit_ns = 2000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void tc_record(int* status, int code) {
  atomicExch(status ? status : &vmc_tc_error, code);
}

// Wait until the barrier's phase with the given parity has completed.
// Returns false (and records `code`) once `limit_ns` of wall-clock time
// (%globaltimer) have passed, however long each try_wait suspends.
__device__ __forceinline__ bool mbar_wait_for(uint32_t bar, uint32_t parity, int code, int* status,
                                              unsigned long long limit_ns) {
  const unsigned long long t0 = global_ns();
  for (;;) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.b32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (global_ns() - t0 > limit_ns) break;
  }
  tc_record(status, code);
  return false;
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int code, int* status) {
  return mbar_wait_for(bar, parity, code, status, vmc_tc_wait_limit_ns);
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(map), "r"(c0), "r"(c1), "r"(bar)
      : "memory");
}

// Shared-memory matrix descriptor of a K-major, 128-byte-swizzled tile whose
// rows are 128 bytes (64 bf16) and whose 8-row groups are 1024 bytes apart.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);  // start address
  d |= (uint64_t)(16u >> 4) << 16;          // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024u >> 4) << 32;        // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;                   // descriptor version (sm_100 family)
  d |= (uint64_t)2 << 61;                   // 128-byte swizzle
  return d;
}

// Instruction descriptor of tcgen05.mma.kind::f16: BF16 x BF16 -> FP32,
// both operands K-major, M = 128, N = 256.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
  return (1u << 4)                      // D format FP32
         | (1u << 7)                    // A format BF16
         | (1u << 10)                   // B format BF16
         | ((uint32_t)(N >> 3) << 17)   // N / 8
         | ((uint32_t)(M >> 4) << 24);  // M / 16
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

struct tc_args {
  int M, N, K;        // D is M x N, reduction over K (operand rows are K-contiguous)
  int mode;           // 0: store upper tiles of a symmetric product, 1: column sums of squares
  int tilesM, tilesN;
  float* out;         // mode 0: D (row-major, ld = ldOut); mode 1: partial column sums (tilesM * 4, N)
  int64_t ldOut;
  int* status;        // receives the code of a wait that ran out (NULL: the library-wide flag)
  int products;       // 3: hi.hi + hi.lo + lo.hi; 1: hi.hi only (lo planes not read)
};

__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap mapAhi, const __grid_constant__ CUtensorMap mapAlo,
                   const __grid_constant__ CUtensorMap mapBhi, const __grid_constant__ CUtensorMap mapBlo,
                   tc_args a) {
  extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + TC_STAGES * TC_STAGE_BYTES);
  // bars[0..S): full, bars[S..2S): empty, bars[2S]: accumulator ready
  uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(bars + 2 * TC_STAGES + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  int tm, tn;
  tile_of(blockIdx.x, a.mode, a.tilesM, a.tilesN, tm, tn);

  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(smem_u32(&bars[s]), 1);
      mbar_init(smem_u32(&bars[TC_STAGES + s]), 1);
    }
    mbar_init(smem_u32(&bars[2 * TC_STAGES]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmemSlot)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmemSlot;

  const int nkb = (a.K + TC_BK - 1) / TC_BK;
  const int iters = nkb;  // one stage per K block, all three products
  bool ok = true;

  if (warp == 0) {
    if (lane == 0) {
      int issued = 0;
      for (int it = 0; it < iters && ok; ++it) {
        const int s = it % TC_STAGES;
        const uint32_t ph = (uint32_t)(it / TC_STAGES) & 1u;
        ok = mbar_wait(smem_u32(&bars[TC_STAGES + s]), ph ^ 1u, 1, a.status);
        if (!ok) break;
        const uint32_t full = smem_u32(&bars[s]);
        mbar_expect_tx(full, a.products == 1 ? TC_A_BYTES + TC_B_BYTES : TC_STAGE_BYTES);
        const int kb = it;
        unsigned char* st = smem + s * TC_STAGE_BYTES;
        tma_load_2d(smem_u32(st), &mapAhi, kb * TC_BK, tm * TC_BM, full);
        tma_load_2d(smem_u32(st + 2 * TC_A_BYTES), &mapBhi, kb * TC_BK, tn * TC_BN, full);
        if (a.products != 1) {
          tma_load_2d(smem_u32(st + TC_A_BYTES), &mapAlo, kb * TC_BK, tm * TC_BM, full);
          tma_load_2d(smem_u32(st + 2 * TC_A_BYTES + TC_B_BYTES), &mapBlo, kb * TC_BK, tn * TC_BN, full);
        }
        ++issued;
      }
      if (!ok) {
        // drain: let the copies already issued land before the CTA unwinds
        for (int j = issued > TC_STAGES ? issued - TC_STAGES : 0; j < issued; ++j)
          mbar_wait_for(smem_u32(&bars[j % TC_STAGES]), (uint32_t)(j / TC_STAGES) & 1u, 4, a.status, TC_DRAIN_NS);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_bf16_f32(TC_BM, TC_BN);
      for (int it = 0; it < iters && ok; ++it) {
        const int s = it % TC_STAGES;
        const uint32_t ph = (uint32_t)(it / TC_STAGES) & 1u;
        ok = mbar_wait(smem_u32(&bars[s]), ph, 2, a.status);
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        unsigned char* st = smem + s * TC_STAGE_BYTES;
        const uint64_t dah = smem_desc_sw128(smem_u32(st));
        const uint64_t dal = smem_desc_sw128(smem_u32(st + TC_A_BYTES));
        const uint64_t dbh = smem_desc_sw128(smem_u32(st + 2 * TC_A_BYTES));
        const uint64_t dbl = smem_desc_sw128(smem_u32(st + 2 * TC_A_BYTES + TC_B_BYTES));
#pragma unroll
        for (int k = 0; k < TC_BK / 16; ++k) {
          // advance the start address by k * 16 bf16 = 32 bytes inside the swizzle atom
          const uint64_t o = (uint64_t)(2 * k);
          mma_bf16(tmem, dah + o, dbh + o, idesc, (it > 0 || k > 0) ? 1u : 0u);
          if (a.products != 1) {
            mma_bf16(tmem, dah + o, dbl + o, idesc, 1u);
            mma_bf16(tmem, dal + o, dbh + o, idesc, 1u);
          }
        }
        mma_commit(smem_u32(&bars[TC_STAGES + s]));
      }
      // always signal the accumulator barrier: it completes only after every
      // MMA issued above has finished, so TMEM is idle before it is freed
      mma_commit(smem_u32(&bars[2 * TC_STAGES]));
    }
  } else {
    // epilogue: warps 2..5 -> TMEM lane quadrant (warp % 4)
    const int q = warp & 3;
    const int row = q * 32 + lane;
    ok = mbar_wait(smem_u32(&bars[2 * TC_STAGES]), 0u, 3, a.status);
    if (ok) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int gr = tm * TC_BM + row;
      for (int c0 = 0; c0 < TC_BN; c0 += 16) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, v);
        const int gc = tn * TC_BN + c0;
        if (a.mode == 0) {
          if (gr < a.M) {
            float* dst = a.out + (int64_t)gr * a.ldOut + gc;
            if (gc + 16 <= a.N) {
#pragma unroll
              for (int i = 0; i < 16; i += 4)
                *reinterpret_cast<float4*>(dst + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
            } else {
              for (int i = 0; i < 16; ++i)
                if (gc + i < a.N) dst[i] = v[i];
            }
          }
        } else {
          // per-(row tile, warp) partial column sums, reduced later in a
          // fixed order (bitwise reproducible, no atomics)
          float* part = a.out + ((int64_t)tm * 4 + q) * a.N;
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            float s2 = gr < a.M ? v[i] * v[i] : 0.f;
            s2 = warp_sum(s2);
            if (lane == 0 && gc + i < a.N) part[gc + i] = s2;
          }
        }
      }
    }
  }
  // before TMEM is released, every MMA issued above must have finished: the
  // accumulator barrier completes only then (its wait returns at once when
  // the epilogue already saw it complete)
  if (warp == 1 && lane == 0) mbar_wait_for(smem_u32(&bars[2 * TC_STAGES]), 0u, 5, a.status, TC_DRAIN_NS);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
  }
}

// One thread waits on an mbarrier that nothing ever arrives on, with the
// given limit: the wait runs out and records code 6 in *status.  Lets the
// host check the timeout path of the waits above without a stalled GEMM.
__global__ void tc_wait_check_kernel(unsigned long long limit_ns, int* status) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(&bar), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) mbar_wait_for(smem_u32(&bar), 0u, 6, status, limit_ns);
}

// ---------------------------------------------------------------- host side
typedef CUresult (*encode_fn_t)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// The driver entry point is looked up once per process (host threads of the
// serving loop call in concurrently); the kernel's shared-memory attribute
// is per device and is set on every launch.
static encode_fn_t get_encode() {
  static std::atomic<encode_fn_t> fn{nullptr};
  encode_fn_t f = fn.load(std::memory_order_acquire);
  if (!f) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess) {
      f = reinterpret_cast<encode_fn_t>(p);
      fn.store(f, std::memory_order_release);
    }
  }
  return f;
}

// 2-D bf16 tensor (rows x cols, cols contiguous, leading dimension ld
// elements); box = box_rows x 64 columns, 128-byte swizzle, zero fill.
static int make_map(CUtensorMap* m, const void* base, int64_t rows, int64_t cols, int64_t ld, int box_rows) {
  encode_fn_t enc = get_encode();
  VMC_REQUIRE(enc, VMC_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  VMC_REQUIRE(((uintptr_t)base & 15) == 0, VMC_ERR_INVALID_ARGUMENT, "tensor base not 16-byte aligned");
  VMC_REQUIRE((ld * 2) % 16 == 0 && ld >= cols, VMC_ERR_INVALID_ARGUMENT,
              "leading dimension %lld must be a multiple of 8 elements and >= %lld", (long long)ld,
              (long long)cols);
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * 2)};
  cuuint32_t box[2] = {(cuuint32_t)TC_BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  VMC_REQUIRE(r == CUDA_SUCCESS, VMC_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return VMC_OK;
}

static int launch_tc(const CUtensorMap& ah, const CUtensorMap& al, const CUtensorMap& bh, const CUtensorMap& bl,
                     tc_args a, int grid, cudaStream_t st) {
  VMC_ALLOW_SMEM(tc_gemm_kernel, TC_SMEM, "tc_gemm");
  tc_gemm_kernel<<<grid, TC_THREADS, TC_SMEM, st>>>(ah, al, bh, bl, a);
  return check_launch("tc_gemm");
}

}  // namespace vmc

using namespace vmc;

extern "C" int vmc_gram_bf16x3(const void* hi, const void* lo, int32_t rows, int32_t k, int64_t ld, float* gram,
                               int64_t ld_gram, int32_t products, int32_t* status, vmc_stream_t stream) {
  VMC_REQUIRE(products == 1 || products == 3, VMC_ERR_INVALID_ARGUMENT,
              "vmc_gram_bf16x3: products must be 1 or 3, not %d", products);
  VMC_REQUIRE(hi && lo && gram && rows > 0 && k > 0 && ld_gram >= rows, VMC_ERR_INVALID_ARGUMENT,
              "vmc_gram_bf16x3: bad arguments");
  VMC_REQUIRE(ld_gram % 4 == 0 && ((uintptr_t)gram & 15) == 0, VMC_ERR_INVALID_ARGUMENT,
              "vmc_gram_bf16x3: the Gram matrix must start on 16 bytes and ld_gram (%lld) be a multiple of 4",
              (long long)ld_gram);
  CUtensorMap mh, ml, nh, nl;
  int rc;
  if ((rc = make_map(&mh, hi, rows, k, ld, TC_BM))) return rc;
  if ((rc = make_map(&ml, lo, rows, k, ld, TC_BM))) return rc;
  if ((rc = make_map(&nh, hi, rows, k, ld, TC_BN))) return rc;
  if ((rc = make_map(&nl, lo, rows, k, ld, TC_BN))) return rc;
  tc_args a;
  a.M = rows;
  a.N = rows;
  a.K = k;
  a.mode = 0;
  a.tilesM = (rows + TC_BM - 1) / TC_BM;
  a.tilesN = (rows + TC_BN - 1) / TC_BN;
  a.out = gram;
  a.ldOut = ld_gram;
  a.status = status;
  a.products = products;
  return launch_tc(mh, ml, nh, nl, a, (int)tile_count(0, a.tilesM, a.tilesN), as_stream(stream));
}

namespace vmc {
// colsq[c] = sum over (row tile, warp) partials in a fixed order, FP64 accumulation
__global__ void colsq_reduce_kernel(const float* __restrict__ part, int nparts, int n, float* __restrict__ colsq) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int r = 0; r < nparts; ++r) s += (double)part[(int64_t)r * n + c];
    colsq[c] = (float)s;
  }
}
}  // namespace vmc

extern "C" size_t vmc_gemm_bf16x3_colsq_workspace_bytes(int32_t m, int32_t n) {
  return (size_t)((m + TC_BM - 1) / TC_BM) * 4 * (size_t)n * sizeof(float) + 256;
}

extern "C" int vmc_gemm_bf16x3_colsq(const void* a_hi, const void* a_lo, int32_t m, int64_t lda, const void* b_hi,
                                     const void* b_lo, int32_t n, int64_t ldb, int32_t k, float* colsq,
                                     void* workspace, size_t workspace_bytes, int32_t products, int32_t* status,
                                     vmc_stream_t stream) {
  VMC_REQUIRE(products == 1 || products == 3, VMC_ERR_INVALID_ARGUMENT,
              "vmc_gemm_bf16x3_colsq: products must be 1 or 3, not %d", products);
  VMC_REQUIRE(a_hi && a_lo && b_hi && b_lo && colsq && m > 0 && n > 0 && k > 0, VMC_ERR_INVALID_ARGUMENT,
              "vmc_gemm_bf16x3_colsq: bad arguments");
  VMC_REQUIRE(workspace && workspace_bytes >= vmc_gemm_bf16x3_colsq_workspace_bytes(m, n), VMC_ERR_WORKSPACE,
              "vmc_gemm_bf16x3_colsq: workspace of %zu bytes needed", vmc_gemm_bf16x3_colsq_workspace_bytes(m, n));
  CUtensorMap ah, al, bh, bl;
  int rc;
  if ((rc = make_map(&ah, a_hi, m, k, lda, TC_BM))) return rc;
  if ((rc = make_map(&al, a_lo, m, k, lda, TC_BM))) return rc;
  if ((rc = make_map(&bh, b_hi, n, k, ldb, TC_BN))) return rc;
  if ((rc = make_map(&bl, b_lo, n, k, ldb, TC_BN))) return rc;
  tc_args a;
  a.M = m;
  a.N = n;
  a.K = k;
  a.mode = 1;
  a.tilesM = (m + TC_BM - 1) / TC_BM;
  a.tilesN = (n + TC_BN - 1) / TC_BN;
  a.out = reinterpret_cast<float*>(workspace);
  a.ldOut = 0;
  a.status = status;
  a.products = products;
  int rc2 = launch_tc(ah, al, bh, bl, a, (int)tile_count(1, a.tilesM, a.tilesN), as_stream(stream));
  if (rc2) return rc2;
  colsq_reduce_kernel<<<(n + 255) / 256, 256, 0, as_stream(stream)>>>(reinterpret_cast<const float*>(workspace),
                                                                       a.tilesM * 4, n, colsq);
  return check_launch("vmc_gemm_bf16x3_colsq(reduce)");
}

extern "C" int vmc_tc_set_wait_limit(uint64_t limit_ns) {
  VMC_REQUIRE(limit_ns > 0, VMC_ERR_INVALID_ARGUMENT, "vmc_tc_set_wait_limit: the limit must be positive");
  unsigned long long v = (unsigned long long)limit_ns;
  cudaError_t e = cudaMemcpyToSymbol(vmc_tc_wait_limit_ns, &v, sizeof(v));
  VMC_REQUIRE(e == cudaSuccess, VMC_ERR_CUDA, "vmc_tc_set_wait_limit: %s", cudaGetErrorString(e));
  return VMC_OK;
}

extern "C" int vmc_tc_wait_check(uint64_t limit_ns, int32_t* status, vmc_stream_t stream) {
  VMC_REQUIRE(status && limit_ns > 0 && limit_ns <= 1000000000ull, VMC_ERR_INVALID_ARGUMENT,
              "vmc_tc_wait_check: needs a status word and a limit in (0, 1 s]");
  tc_wait_check_kernel<<<1, 32, 0, as_stream(stream)>>>((unsigned long long)limit_ns, status);
  return check_launch("vmc_tc_wait_check");
}

extern "C" int vmc_tc_error_flag(int32_t reset) {
  int v = 0;
  cudaMemcpyFromSymbol(&v, vmc_tc_error, sizeof(int));
  if (reset) {
    int z = 0;
    cudaMemcpyToSymbol(vmc_tc_error, &z, sizeof(int));
  }
  return v;
}

// ===================================================================
// FP64-accurate complex products (Ozaki split, tcgen05): kernel in
// oz_gemm.cuh, operand slicing and output assembly below.
// ===================================================================
#include "oz_gemm.cuh"
#include "oz_host.h"

namespace vmc {

constexpr int OZ_MAX_K2 = 61440;  // keeps the int64 tile sums below 2^63

__host__ __device__ inline int64_t oz_pad(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

// Scale exponent of every operand row m (a column of P, P[k][m] = Z[k sk + m sm]):
// the smallest e with max_k max(|Re|, |Im|) < 2^e (0 for a zero row).
// One warp per row when the row is contiguous (sk == 1), else lanes along m.
__global__ void oz_row_exponent_kernel(const double2* __restrict__ Z, int64_t sk, int64_t sm, int K, int M,
                                       int* __restrict__ e) {
  if (sk == 1) {
    const int warpsPerBlock = blockDim.x >> 5;
    const int m = blockIdx.x * warpsPerBlock + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (m >= M) return;
    double mx = 0.0;
    for (int k = lane; k < K; k += 32) {
      const double2 v = Z[(int64_t)k + (int64_t)m * sm];
      mx = fmax(mx, fmax(fabs(v.x), fabs(v.y)));
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) {
      int ex = 0;
      if (mx > 0.0) frexp(mx, &ex);
      e[m] = ex;
    }
  } else {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    double mx = 0.0;
    for (int k = 0; k < K; ++k) {
      const double2 v = Z[(int64_t)k * sk + (int64_t)m * sm];
      mx = fmax(mx, fmax(fabs(v.x), fabs(v.y)));
    }
    int ex = 0;
    if (mx > 0.0) frexp(mx, &ex);
    e[m] = ex;
  }
}

// Slices of the operand rows: plane i, row m holds n_i 2^(-7(i+1)) of
// [Re P[:, m] 2^-e_m | Im P[:, m] 2^-e_m] (columns [0, K) and [K, 2K));
// with bRole, row rowsHalf + m holds the slices of [Im | -Re].  Rows >= M
// are written as zeros.  32 x 32 tiles through shared memory so that both
// the reads (either layout of Z) and the writes are coalesced.
__global__ void oz_slice_kernel(const double2* __restrict__ Z, int64_t sk, int64_t sm, int conj, int K, int M,
                                int rowsP, int rowsHalf, int bRole, int slices, int64_t K2p,
                                const int* __restrict__ e, __nv_bfloat16* __restrict__ planes) {
  __shared__ double2 tile[32][33];
  const int k0 = blockIdx.x * 32, m0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  if (sk == 1) {
#pragma unroll
    for (int j = 0; j < 32; j += 8) {
      const int k = k0 + tx, m = m0 + ty + j;
      double2 v = make_double2(0.0, 0.0);
      if (k < K && m < M) v = Z[(int64_t)k + (int64_t)m * sm];
      tile[tx][ty + j] = v;
    }
  } else {
#pragma unroll
    for (int j = 0; j < 32; j += 8) {
      const int m = m0 + tx, k = k0 + ty + j;
      double2 v = make_double2(0.0, 0.0);
      if (k < K && m < M) v = Z[(int64_t)k * sk + (int64_t)m * sm];
      tile[ty + j][tx] = v;
    }
  }
  __syncthreads();
  const int64_t planeStride = (int64_t)rowsP * K2p;
#pragma unroll
  for (int j = 0; j < 32; j += 8) {
    const int k = k0 + tx, m = m0 + ty + j;
    if (k >= K || m >= rowsHalf) continue;
    double2 v = tile[tx][ty + j];
    if (conj) v.y = -v.y;
    const int ex = m < M ? e[m] : 0;
    double re = ldexp(v.x, -ex), im = ldexp(v.y, -ex);
    __nv_bfloat16* rowA = planes + (int64_t)m * K2p;
    __nv_bfloat16* rowB = planes + (int64_t)(rowsHalf + m) * K2p;
    for (int i = 0; i < slices; ++i) {
      const double sr = rint(re * 128.0), si = rint(im * 128.0);
      re = re * 128.0 - sr;
      im = im * 128.0 - si;
      const float scale = __int_as_float((127 - OZ_BITS * (i + 1)) << 23);
      const __nv_bfloat16 br = __float2bfloat16_rn((float)sr * scale), bi = __float2bfloat16_rn((float)si * scale);
      __nv_bfloat16* pa = rowA + i * planeStride;
      pa[k] = br;
      pa[K + k] = bi;
      if (bRole) {
        __nv_bfloat16* pb = rowB + i * planeStride;
        pb[k] = bi;
        pb[K + k] = __hneg(br);
      }
    }
  }
}

// Zero the padding columns [2K, K2p) of every row of every plane.
__global__ void oz_pad_kernel(__nv_bfloat16* planes, int64_t rows, int64_t K2p, int K2) {
  const int w = (int)(K2p - K2);
  const int64_t n = rows * w;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / w;
    planes[r * K2p + K2 + (t - r * w)] = __float2bfloat16_rn(0.0f);
  }
}

// C (column-major, ldc) = alpha product (+ C), the product read from the
// kernel's row-major [Re | Im] output; with hermitian, entries below the
// diagonal come from the mirrored entry, conjugated, and the diagonal is real.
__global__ void oz_finish_kernel(const double* __restrict__ out, int64_t ldo, int M, int N, int Np, int hermitian,
                                 double2* __restrict__ C, int64_t ldc, int accumulate, double alpha) {
  __shared__ double2 tile[32][33];
  const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  // Hermitian output: every entry below the diagonal is the conjugate of its
  // mirror (computed by the kernel, whose blocks on and above the diagonal
  // cover it), so the result is exactly Hermitian
  const bool mirror = hermitian && j0 < i0;
  if (!mirror) {
#pragma unroll
    for (int r = 0; r < 32; r += 8) {
      const int i = i0 + ty + r, j = j0 + tx;
      double2 v = make_double2(0.0, 0.0);
      if (i < M && j < N) v = make_double2(out[(int64_t)i * ldo + j], out[(int64_t)i * ldo + Np + j]);
      tile[ty + r][tx] = v;
    }
  } else {
#pragma unroll
    for (int r = 0; r < 32; r += 8) {
      const int j = j0 + ty + r, i = i0 + tx;
      double2 v = make_double2(0.0, 0.0);
      if (i < M && j < N) v = make_double2(out[(int64_t)j * ldo + i], -out[(int64_t)j * ldo + Np + i]);
      tile[tx][ty + r] = v;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < 32; r += 8) {
    const int j = j0 + ty + r, i = i0 + tx;
    if (i < M && j < N) {
      double2 v = tile[tx][ty + r];
      if (hermitian && i0 == j0 && j <= i) {  // diagonal tile: lower part from the upper one
        const double2 u = tile[ty + r][tx];
        v = j < i ? make_double2(u.x, -u.y) : make_double2(v.x, 0.0);
      }
      v.x *= alpha;
      v.y *= alpha;
      double2* dst = C + (int64_t)j * ldc + i;
      if (accumulate) {
        const double2 c = *dst;
        v.x += c.x;
        v.y += c.y;
      }
      *dst = v;
    }
  }
}

size_t oz_operand_bytes(int rows, int K, int slices, bool bRole) {
  const int64_t half = oz_pad(rows, OZ_BM);
  const int64_t rowsP = bRole ? 2 * half : half;
  return (size_t)(slices * rowsP * oz_pad(2 * (int64_t)K, OZ_BK) * 2) + (size_t)oz_pad(half * 4, 256);
}

int oz_make_operand(void* buf, int rows, int K, int slices, bool bRole, oz_operand& op) {
  op.rows = rows;
  op.rowsHalf = (int)oz_pad(rows, OZ_BM);
  op.rowsP = bRole ? 2 * op.rowsHalf : op.rowsHalf;
  op.K = K;
  op.slices = slices;
  op.K2p = oz_pad(2 * (int64_t)K, OZ_BK);
  op.planes = reinterpret_cast<__nv_bfloat16*>(buf);
  op.exps = reinterpret_cast<int*>(reinterpret_cast<char*>(buf) + (size_t)slices * op.rowsP * op.K2p * 2);
  return VMC_OK;
}

int oz_slice(const double* Z, int64_t sk, int64_t sm, int conj, oz_operand& op, bool bRole, cudaStream_t st) {
  const double2* z = reinterpret_cast<const double2*>(Z);
  if (sk == 1)
    oz_row_exponent_kernel<<<(op.rows + 7) / 8, 256, 0, st>>>(z, sk, sm, op.K, op.rows, op.exps);
  else
    oz_row_exponent_kernel<<<(op.rows + 127) / 128, 128, 0, st>>>(z, sk, sm, op.K, op.rows, op.exps);
  if (op.rowsHalf > op.rows)
    cudaMemsetAsync(op.exps + op.rows, 0, (size_t)(op.rowsHalf - op.rows) * sizeof(int), st);
  dim3 grid((unsigned)((op.K + 31) / 32), (unsigned)(op.rowsHalf / 32));
  oz_slice_kernel<<<grid, dim3(32, 8), 0, st>>>(z, sk, sm, conj, op.K, op.rows, op.rowsP, op.rowsHalf,
                                                bRole ? 1 : 0, op.slices, op.K2p, op.exps, op.planes);
  if (op.K2p > 2 * (int64_t)op.K)
    oz_pad_kernel<<<1024, 256, 0, st>>>(op.planes, (int64_t)op.slices * op.rowsP, op.K2p, 2 * op.K);
  return check_launch("oz_slice");
}

static int make_map_3d(CUtensorMap* m, const void* base, int64_t cols, int64_t rows, int64_t planes) {
  encode_fn_t enc = get_encode();
  VMC_REQUIRE(enc, VMC_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  VMC_REQUIRE(((uintptr_t)base & 15) == 0 && (cols * 2) % 16 == 0, VMC_ERR_INVALID_ARGUMENT,
              "sliced operand not 16-byte aligned");
  cuuint64_t dims[3] = {(cuuint64_t)cols, (cuuint64_t)rows, (cuuint64_t)planes};
  cuuint64_t strides[2] = {(cuuint64_t)(cols * 2), (cuuint64_t)(cols * rows * 2)};
  cuuint32_t box[3] = {(cuuint32_t)OZ_BK, (cuuint32_t)OZ_BM, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  VMC_REQUIRE(r == CUDA_SUCCESS, VMC_ERR_CUDA, "cuTensorMapEncodeTiled (3-d) failed (%d)", (int)r);
  return VMC_OK;
}

static int oz_sms() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 148;
}

int oz_multiply(const oz_operand& A, const oz_operand& B, int maxLevel, bool hermitian, double* out, int* status,
                cudaStream_t st) {
  VMC_REQUIRE(A.K == B.K && A.K2p == B.K2p, VMC_ERR_INVALID_ARGUMENT, "oz_multiply: reduction lengths differ");
  VMC_REQUIRE(A.K2p <= OZ_MAX_K2, VMC_ERR_UNSUPPORTED, "oz_multiply: reduction length %d above %d",
              (int)A.K2p / 2, OZ_MAX_K2 / 2);
  VMC_REQUIRE(!hermitian || A.rowsHalf == B.rowsHalf, VMC_ERR_INVALID_ARGUMENT,
              "oz_multiply: a Hermitian product needs a square output");
  CUtensorMap ma, mb;
  int rc;
  if ((rc = make_map_3d(&ma, A.planes, A.K2p, A.rowsP, A.slices))) return rc;
  if ((rc = make_map_3d(&mb, B.planes, B.K2p, B.rowsP, B.slices))) return rc;
  oz_args a;
  a.M = A.rows;
  a.K2 = (int)A.K2p;
  a.halfTiles = B.rowsHalf / OZ_BN;
  a.tilesM = A.rowsHalf / OZ_BM;
  a.slicesA = A.slices;
  a.slicesB = B.slices;
  a.maxLevel = maxLevel;
  a.hermitian = hermitian ? 1 : 0;
  a.numTiles = oz_tile_count(a.tilesM, a.halfTiles, a.hermitian);
  a.lsb = 0;
  while (1.02 * (double)A.K2p * std::ldexp(1.0, a.lsb + 1) < std::ldexp(1.0, 63)) ++a.lsb;
  a.ea = A.exps;
  a.eb = B.exps;
  a.out = out;
  a.ldo = 2 * (int64_t)B.rowsHalf;
  a.status = status;
  VMC_ALLOW_SMEM(oz_gemm_kernel, OZ_SMEM, "oz_gemm");
  const int grid = a.numTiles < oz_sms() ? a.numTiles : oz_sms();
  oz_gemm_kernel<<<grid, OZ_THREADS, OZ_SMEM, st>>>(ma, mb, a);
  return check_launch("oz_gemm");
}

int oz_finish(const double* out, const oz_operand& A, const oz_operand& B, bool hermitian, double* C, int64_t ldc,
              bool accumulate, cudaStream_t st, double alpha) {
  dim3 grid((unsigned)((A.rows + 31) / 32), (unsigned)((B.rows + 31) / 32));
  oz_finish_kernel<<<grid, dim3(32, 8), 0, st>>>(out, 2 * (int64_t)B.rowsHalf, A.rows, B.rows, B.rowsHalf,
                                                  hermitian ? 1 : 0, reinterpret_cast<double2*>(C), ldc,
                                                  accumulate ? 1 : 0, alpha);
  return check_launch("oz_finish");
}

}  // namespace vmc

static size_t zgemm_ozaki_ws(int32_t m, int32_t n, int32_t k, int32_t slices) {
  return oz_operand_bytes(m, k, slices, false) + oz_operand_bytes(n, k, slices, true) +
         (size_t)oz_pad(m, OZ_BM) * 2 * (size_t)oz_pad(n, OZ_BN) * 8 + 1024;
}

extern "C" size_t vmc_zgemm_ozaki_workspace_bytes(int32_t m, int32_t n, int32_t k, int32_t slices) {
  if (m <= 0 || n <= 0 || k <= 0 || slices < 1 || slices > OZ_MAX_SLICES) return 0;
  return zgemm_ozaki_ws(m, n, k, slices);
}

extern "C" int vmc_zgemm_ozaki(int32_t trans_a, int32_t trans_b, int32_t m, int32_t n, int32_t k, const double* A,
                               int64_t lda, const double* B, int64_t ldb, double* C, int64_t ldc, int32_t hermitian,
                               int32_t accumulate, int32_t slices, int32_t max_level, void* workspace,
                               size_t workspace_bytes, int32_t* status, vmc_stream_t stream) {
  VMC_REQUIRE((trans_a == 'N' || trans_a == 'C') && (trans_b == 'N' || trans_b == 'C'), VMC_ERR_INVALID_ARGUMENT,
              "vmc_zgemm_ozaki: trans_a and trans_b must be 'N' or 'C'");
  VMC_REQUIRE(A && B && C && m > 0 && n > 0 && k > 0, VMC_ERR_INVALID_ARGUMENT, "vmc_zgemm_ozaki: bad arguments");
  VMC_REQUIRE(lda >= (trans_a == 'N' ? m : k) && ldb >= (trans_b == 'N' ? k : n) && ldc >= m,
              VMC_ERR_INVALID_ARGUMENT,
              "vmc_zgemm_ozaki: leading dimension too small");
  VMC_REQUIRE(!hermitian || m == n, VMC_ERR_INVALID_ARGUMENT, "vmc_zgemm_ozaki: a Hermitian product is square");
  VMC_REQUIRE(slices >= 1 && slices <= OZ_MAX_SLICES && max_level >= 0 && max_level <= 2 * (slices - 1),
              VMC_ERR_INVALID_ARGUMENT, "vmc_zgemm_ozaki: %d slices, level %d", slices, max_level);
  VMC_REQUIRE(2 * (int64_t)k <= OZ_MAX_K2, VMC_ERR_UNSUPPORTED, "vmc_zgemm_ozaki: k = %d above %d", k,
              OZ_MAX_K2 / 2);
  VMC_REQUIRE(((uintptr_t)A & 15) == 0 && ((uintptr_t)B & 15) == 0 && ((uintptr_t)C & 15) == 0,
              VMC_ERR_INVALID_ARGUMENT, "vmc_zgemm_ozaki: complex128 arrays must be 16-byte aligned");
  const size_t need = zgemm_ozaki_ws(m, n, k, slices);
  VMC_REQUIRE(workspace && workspace_bytes >= need && ((uintptr_t)workspace & 255) == 0, VMC_ERR_WORKSPACE,
              "vmc_zgemm_ozaki: workspace of %zu bytes (256-byte aligned) needed", need);
  cudaStream_t st = as_stream(stream);
  char* ws = reinterpret_cast<char*>(workspace);
  oz_operand oa, ob;
  oz_make_operand(ws, m, k, slices, false, oa);
  ws += oz_operand_bytes(m, k, slices, false);
  oz_make_operand(ws, n, k, slices, true, ob);
  ws += oz_operand_bytes(n, k, slices, true);
  double* out = reinterpret_cast<double*>(ws);
  int rc;
  // C = P^H Q with P = op(A)^H: 'C' -> P[kk][mm] = A[kk + mm lda]; 'N' -> P[kk][mm] = conj(A[mm + kk lda])
  if (trans_a == 'C')
    rc = oz_slice(A, 1, lda, 0, oa, false, st);
  else
    rc = oz_slice(A, lda, 1, 1, oa, false, st);
  if (rc) return rc;
  // Q[kk][nn] = op(B)[kk][nn]: 'N' -> B[kk + nn ldb]; 'C' -> conj(B[nn + kk ldb])
  if (trans_b == 'N')
    rc = oz_slice(B, 1, ldb, 0, ob, true, st);
  else
    rc = oz_slice(B, ldb, 1, 1, ob, true, st);
  if (rc) return rc;
  if ((rc = oz_multiply(oa, ob, max_level, hermitian != 0, out, status, st))) return rc;
  return oz_finish(out, oa, ob, hermitian != 0, C, ldc, accumulate != 0, st, 1.0);
}
