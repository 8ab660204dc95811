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
// about 16 significant bits per operand instead of 8.
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
        mbar_expect_tx(full, TC_STAGE_BYTES);
        const int kb = it;
        unsigned char* st = smem + s * TC_STAGE_BYTES;
        tma_load_2d(smem_u32(st), &mapAhi, kb * TC_BK, tm * TC_BM, full);
        tma_load_2d(smem_u32(st + TC_A_BYTES), &mapAlo, kb * TC_BK, tm * TC_BM, full);
        tma_load_2d(smem_u32(st + 2 * TC_A_BYTES), &mapBhi, kb * TC_BK, tn * TC_BN, full);
        tma_load_2d(smem_u32(st + 2 * TC_A_BYTES + TC_B_BYTES), &mapBlo, kb * TC_BK, tn * TC_BN, full);
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
          mma_bf16(tmem, dah + o, dbl + o, idesc, 1u);
          mma_bf16(tmem, dal + o, dbh + o, idesc, 1u);
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
                               int64_t ld_gram, int32_t* status, vmc_stream_t stream) {
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
                                     void* workspace, size_t workspace_bytes, int32_t* status,
                                     vmc_stream_t stream) {
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
