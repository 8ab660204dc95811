// Branch-free operator expansion in the reference layout
// (operator/branch_free.py:443-487, operator/base.py:91-164).
#include "bf_apply.cuh"
#include "vmc_common.cuh"

namespace vmc {

constexpr int kBfWarps = 8;

// One warp per configuration: matrix elements of every string (lanes own
// strings), diagonal merge into diag[0], ascending compaction of |m| > 1e-6.
__global__ void bf_matels_kernel(const int32_t* __restrict__ configs, int64_t N, int L, vmc_bf_operator op,
                                 double2* __restrict__ mfull, int32_t* __restrict__ nzIndex,
                                 int32_t* __restrict__ nzCount, int32_t* __restrict__ maxCount) {
  extern __shared__ unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = (L + 31) >> 5;
  const size_t perWarp = (((size_t)nw * 4 + ((L + 15) & ~15)) + 15) & ~(size_t)15;
  uint32_t* occ = reinterpret_cast<uint32_t*>(smem + warp * perWarp);
  int8_t* cfg = reinterpret_cast<int8_t*>(occ + nw);
  const int K = op.num_ops;
  for (int64_t n = (int64_t)blockIdx.x * kBfWarps + warp; n < N; n += (int64_t)gridDim.x * kBfWarps) {
    warp_load_config(configs + n * L, L, cfg, occ, lane);
    double2* row = mfull + n * K;
    bf_string_result r;
    for (int o = lane; o < K; o += 32) {
      bf_apply_string(op, o, cfg, occ, L, r);
      row[o] = make_double2(r.m.re, r.m.im);
    }
    __syncwarp();
    if (op.num_diag > 1 && lane == 0) {
      double sr = 0.0, si = 0.0;
      for (int d = 0; d < op.num_diag; ++d) {
        double2 v = row[op.diag[d]];
        sr += v.x;
        si += v.y;
      }
      row[op.diag[0]] = make_double2(sr, si);
      for (int d = 1; d < op.num_diag; ++d) row[op.diag[d]] = make_double2(0.0, 0.0);
    }
    __syncwarp();
    int cnt = 0;
    int32_t* idxRow = nzIndex + n * K;
    for (int o0 = 0; o0 < K; o0 += 32) {
      int o = o0 + lane;
      bool nz = false;
      if (o < K) {
        double2 v = row[o];
        nz = hypot(v.x, v.y) > 1e-6;
      }
      unsigned b = __ballot_sync(0xffffffffu, nz);
      if (nz) idxRow[cnt + __popc(b & ((1u << lane) - 1u))] = o;
      cnt += __popc(b);
    }
    if (lane == 0) {
      nzCount[n] = cnt;
      atomicMax(maxCount, cnt);
    }
    __syncwarp();
  }
}

// One warp per configuration: K output rows, each the s' of string
// nz_index[k] (k < count) or of the last string (padding), written coalesced.
__global__ void bf_gather_kernel(const int32_t* __restrict__ configs, int64_t N, int L, vmc_bf_operator op,
                                 const double2* __restrict__ mfull, const int32_t* __restrict__ nzIndex,
                                 const int32_t* __restrict__ nzCount, int K, int32_t* __restrict__ sp,
                                 double2* __restrict__ mat) {
  extern __shared__ unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = (L + 31) >> 5;
  const size_t perWarp = (((size_t)nw * 4 + ((L + 15) & ~15)) + 15) & ~(size_t)15;
  uint32_t* occ = reinterpret_cast<uint32_t*>(smem + warp * perWarp);
  int8_t* cfg = reinterpret_cast<int8_t*>(occ + nw);
  const int numOps = op.num_ops;
  for (int64_t n = (int64_t)blockIdx.x * kBfWarps + warp; n < N; n += (int64_t)gridDim.x * kBfWarps) {
    warp_load_config(configs + n * L, L, cfg, occ, lane);
    const int cnt = nzCount[n];
    bf_string_result r;
    for (int k = 0; k < K; ++k) {
      const int o = k < cnt ? nzIndex[n * numOps + k] : numOps - 1;
      bf_apply_string(op, o, cfg, occ, L, r);
      int32_t* out = sp + (n * K + k) * (int64_t)L;
      for (int i = lane; i < L; i += 32) {
        int v = cfg[i];
        for (int q = 0; q < r.nmod; ++q)
          if (r.site[q] == i) v = r.val[q];
        out[i] = v;
      }
      if (lane == 0) mat[n * K + k] = k < cnt ? mfull[n * numOps + o] : make_double2(0.0, 0.0);
    }
    __syncwarp();
  }
}

__global__ void oloc_kernel(const double2* __restrict__ mat, const double2* __restrict__ lps,
                            const double2* __restrict__ lpsp, int64_t N, int K, double2* __restrict__ out) {
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
    const double2 y = lps[n];
    cpx<double> acc = mk(0.0, 0.0);
    for (int k = 0; k < K; ++k) {
      const double2 z = lpsp[n * K + k];
      const double2 m = mat[n * K + k];
      cpx<double> e = cexp_(mk(z.x - y.x, z.y - y.y));
      acc = acc + mk(m.x, m.y) * e;
    }
    out[n] = make_double2(acc.re, acc.im);
  }
}

size_t bf_smem(int L) {
  const int nw = (L + 31) >> 5;
  const size_t perWarp = (((size_t)nw * 4 + ((L + 15) & ~15)) + 15) & ~(size_t)15;
  return perWarp * kBfWarps;
}

int bf_grid(int64_t N) {
  int64_t b = (N + kBfWarps - 1) / kBfWarps;
  if (b > 152 * 16) b = 152 * 16;
  return b < 1 ? 1 : (int)b;
}

}  // namespace vmc

using namespace vmc;

extern "C" int vmc_bf_matrix_elements(const int32_t* configs, int64_t num_configs, int32_t num_sites,
                                      const vmc_bf_operator* op, double* mat_el_full, int32_t* nz_index,
                                      int32_t* nz_count, int32_t* max_count, vmc_stream_t stream) {
  int rc = check_op("vmc_bf_matrix_elements", op, num_sites);
  if (rc) return rc;
  VMC_REQUIRE(num_sites > 0 && num_sites <= 8192 && num_configs >= 0, VMC_ERR_UNSUPPORTED,
              "vmc_bf_matrix_elements: L=%d", num_sites);
  VMC_REQUIRE((configs && mat_el_full && nz_index && nz_count) || num_configs == 0, VMC_ERR_INVALID_ARGUMENT,
              "vmc_bf_matrix_elements: null argument");
  VMC_REQUIRE(max_count, VMC_ERR_INVALID_ARGUMENT, "vmc_bf_matrix_elements: null max_count");
  cudaStream_t st = as_stream(stream);
  cudaError_t e = cudaMemsetAsync(max_count, 0, sizeof(int32_t), st);
  VMC_REQUIRE(e == cudaSuccess, VMC_ERR_CUDA, "vmc_bf_matrix_elements: %s", cudaGetErrorString(e));
  if (num_configs == 0) return VMC_OK;
  size_t smem = bf_smem(num_sites);
  bf_matels_kernel<<<bf_grid(num_configs), 32 * kBfWarps, smem, st>>>(
      configs, num_configs, num_sites, *op, reinterpret_cast<double2*>(mat_el_full), nz_index, nz_count, max_count);
  return check_launch("vmc_bf_matrix_elements");
}

extern "C" int vmc_bf_gather(const int32_t* configs, int64_t num_configs, int32_t num_sites, const vmc_bf_operator* op,
                             const double* mat_el_full, const int32_t* nz_index, const int32_t* nz_count, int32_t K,
                             int32_t* s_primes, double* mat_el, vmc_stream_t stream) {
  int rc = check_op("vmc_bf_gather", op, num_sites);
  if (rc) return rc;
  VMC_REQUIRE(K >= 0 && K <= op->num_ops, VMC_ERR_INVALID_ARGUMENT, "vmc_bf_gather: K=%d outside [0, %d]", K,
              op->num_ops);
  VMC_REQUIRE(num_sites > 0 && num_sites <= 8192, VMC_ERR_UNSUPPORTED, "vmc_bf_gather: L=%d", num_sites);
  if (num_configs == 0 || K == 0) return VMC_OK;
  VMC_REQUIRE(configs && mat_el_full && nz_index && nz_count && s_primes && mat_el, VMC_ERR_INVALID_ARGUMENT,
              "vmc_bf_gather: null argument");
  size_t smem = bf_smem(num_sites);
  bf_gather_kernel<<<bf_grid(num_configs), 32 * kBfWarps, smem, as_stream(stream)>>>(
      configs, num_configs, num_sites, *op, reinterpret_cast<const double2*>(mat_el_full), nz_index, nz_count, K,
      s_primes, reinterpret_cast<double2*>(mat_el));
  return check_launch("vmc_bf_gather");
}

extern "C" int vmc_oloc_from_sprimes(const double* mat_el, const double* log_psi_s, const double* log_psi_sp,
                                     int64_t num_configs, int32_t K, double* oloc, vmc_stream_t stream) {
  VMC_REQUIRE(num_configs >= 0 && K >= 0, VMC_ERR_INVALID_ARGUMENT, "vmc_oloc_from_sprimes: bad sizes");
  if (num_configs == 0) return VMC_OK;
  VMC_REQUIRE(log_psi_s && oloc && (K == 0 || (mat_el && log_psi_sp)), VMC_ERR_INVALID_ARGUMENT,
              "vmc_oloc_from_sprimes: null argument");
  int64_t blocks = (num_configs + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  oloc_kernel<<<(int)blocks, 256, 0, as_stream(stream)>>>(reinterpret_cast<const double2*>(mat_el),
                                                          reinterpret_cast<const double2*>(log_psi_s),
                                                          reinterpret_cast<const double2*>(log_psi_sp), num_configs,
                                                          K, reinterpret_cast<double2*>(oloc));
  return check_launch("vmc_oloc_from_sprimes");
}
