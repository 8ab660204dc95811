// ExactSampler basis enumeration and Born weights.
#include "vmc_common.cuh"
#include "reduce.cuh"

namespace vmc {

// One thread per (state, site).  local_dim 2: site i = bit i of the state
// index (sampler.py:442-455); otherwise base-local_dim digits, most
// significant first (sampler.py:457-472).
__global__ void exact_basis_kernel(int32_t* __restrict__ basis, int64_t first, int64_t count, int L, int ldim) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t total = count * (int64_t)L;
  for (; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = t / L;
    int i = (int)(t - r * L);
    int64_t v = first + r;
    int32_t out;
    if (ldim == 2) {
      out = (int32_t)((v >> i) & 1);
    } else {
      // digit k (least significant first) sits at position L-1-k
      int k = L - 1 - i;
      for (int q = 0; q < k; ++q) v /= ldim;
      out = (int32_t)(v % ldim);
    }
    basis[t] = out;
  }
}

// p_r = exp((Re logpsi_r - last_norm)/lpf) (0 past num_valid); block partial sums.
__global__ void exact_prob_kernel(const double* __restrict__ logpsi, int64_t n, int64_t nvalid,
                                  const double* __restrict__ lastNorm, double lpf, double* __restrict__ p,
                                  double* __restrict__ partial) {
  const double last_norm = *lastNorm;
  double acc = 0.0;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double v = r < nvalid ? exp((logpsi[2 * r] - last_norm) / lpf) : 0.0;
    p[r] = v;
    acc += v;
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

__global__ void exact_norm_kernel(double* __restrict__ p, int64_t n, const double* __restrict__ partial, int nparts,
                                  double* __restrict__ norm_out, double* __restrict__ lastNorm, double lpf) {
  // every block sums the partials in the same fixed order
  __shared__ double s_nrm;
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < nparts; ++b) s += partial[b];
    s_nrm = s;
    if (blockIdx.x == 0) {
      if (norm_out) *norm_out = s;
      *lastNorm += lpf * log(s);  // sampler.py:524
    }
  }
  __syncthreads();
  double nrm = s_nrm;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
    p[r] = p[r] / nrm;
}

}  // namespace vmc

using namespace vmc;

extern "C" int vmc_exact_basis(int32_t* basis, int64_t first_state, int64_t num_states, int32_t num_sites,
                               int32_t local_dim, vmc_stream_t stream) {
  VMC_REQUIRE(basis || num_states == 0, VMC_ERR_INVALID_ARGUMENT, "vmc_exact_basis: null output");
  VMC_REQUIRE(num_sites > 0 && local_dim >= 2 && num_states >= 0 && first_state >= 0, VMC_ERR_INVALID_ARGUMENT,
              "vmc_exact_basis: invalid sizes (L=%d, lDim=%d)", num_sites, local_dim);
  VMC_REQUIRE(local_dim != 2 || num_sites <= 62, VMC_ERR_UNSUPPORTED, "vmc_exact_basis: L=%d > 62", num_sites);
  if (num_states == 0) return VMC_OK;
  int64_t total = num_states * (int64_t)num_sites;
  int threads = 256;
  int64_t blocks = (total + threads - 1) / threads;
  if (blocks > 152 * 64) blocks = 152 * 64;
  exact_basis_kernel<<<(unsigned)blocks, threads, 0, as_stream(stream)>>>(basis, first_state, num_states, num_sites,
                                                                         local_dim);
  return check_launch("vmc_exact_basis");
}

extern "C" int vmc_exact_probabilities(const double* log_psi, int64_t num_states, int64_t num_valid, double* last_norm,
                                       double log_prob_factor, double* p, double* norm_out, void* workspace,
                                       size_t workspace_bytes, vmc_stream_t stream) {
  VMC_REQUIRE(log_psi && p && last_norm && num_states > 0, VMC_ERR_INVALID_ARGUMENT,
              "vmc_exact_probabilities: bad arguments");
  VMC_REQUIRE(workspace && workspace_bytes >= vmc_reduce_workspace_bytes(1), VMC_ERR_WORKSPACE,
              "vmc_exact_probabilities: workspace of %zu bytes needed", vmc_reduce_workspace_bytes(1));
  double* partial = reinterpret_cast<double*>(workspace);
  exact_prob_kernel<<<kReduceBlocks, 256, 0, as_stream(stream)>>>(log_psi, num_states, num_valid, last_norm,
                                                                  log_prob_factor, p, partial);
  int rc = check_launch("vmc_exact_probabilities");
  if (rc) return rc;
  exact_norm_kernel<<<kReduceBlocks, 256, 0, as_stream(stream)>>>(p, num_states, partial, kReduceBlocks, norm_out,
                                                                   last_norm, log_prob_factor);
  return check_launch("vmc_exact_probabilities(normalise)");
}

namespace vmc {
__global__ void mc_prob_kernel(const double* __restrict__ logpsi, int64_t n, double factor, double* __restrict__ p,
                               double* __restrict__ partial) {
  double acc = 0.0;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double v = exp(factor * logpsi[2 * r]);
    p[r] = v;
    acc += v;
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

__global__ void normalise_kernel(double* __restrict__ p, int64_t n, const double* __restrict__ partial, int nparts) {
  __shared__ double s_nrm;
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < nparts; ++b) s += partial[b];
    s_nrm = s;
  }
  __syncthreads();
  const double nrm = s_nrm;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
    p[r] = p[r] / nrm;
}
}  // namespace vmc

extern "C" int vmc_mc_probabilities(const double* log_psi, int64_t num_samples, double factor, double* p,
                                    void* workspace, size_t workspace_bytes, vmc_stream_t stream) {
  VMC_REQUIRE(log_psi && p && num_samples > 0, VMC_ERR_INVALID_ARGUMENT, "vmc_mc_probabilities: bad arguments");
  VMC_REQUIRE(workspace && workspace_bytes >= vmc_reduce_workspace_bytes(1), VMC_ERR_WORKSPACE,
              "vmc_mc_probabilities: workspace of %zu bytes needed", vmc_reduce_workspace_bytes(1));
  double* partial = reinterpret_cast<double*>(workspace);
  mc_prob_kernel<<<kReduceBlocks, 256, 0, as_stream(stream)>>>(log_psi, num_samples, factor, p, partial);
  int rc = check_launch("vmc_mc_probabilities");
  if (rc) return rc;
  normalise_kernel<<<kReduceBlocks, 256, 0, as_stream(stream)>>>(p, num_samples, partial, kReduceBlocks);
  return check_launch("vmc_mc_probabilities(normalise)");
}
