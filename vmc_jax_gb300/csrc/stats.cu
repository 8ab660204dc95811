// FP64 sample statistics: weighted means and variances
// (stats.py:197-252, mpi_wrapper.py:114-217).
#include "reduce.cuh"
#include "vmc_common.cuh"

namespace vmc {

__global__ void wmean_partial_kernel(const double2* __restrict__ x, const double* __restrict__ w, int64_t n,
                                     double2* __restrict__ partial) {
  double re = 0.0, im = 0.0;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double2 v = x[r];
    double ww = w[r];
    re = fma(ww, v.x, re);
    im = fma(ww, v.y, im);
  }
  re = block_sum(re);
  im = block_sum(im);
  if (threadIdx.x == 0) partial[blockIdx.x] = make_double2(re, im);
}

__global__ void wvar_partial_kernel(const double2* __restrict__ x, const double* __restrict__ w, int64_t n,
                                    const double2* __restrict__ partial_mean, int nparts, double2* __restrict__ mean_out,
                                    double* __restrict__ partial) {
  __shared__ double2 s_mean;
  if (threadIdx.x == 0) {
    double re = 0.0, im = 0.0;
    for (int b = 0; b < nparts; ++b) {
      re += partial_mean[b].x;
      im += partial_mean[b].y;
    }
    s_mean = make_double2(re, im);
    if (blockIdx.x == 0) *mean_out = s_mean;
  }
  __syncthreads();
  double2 m = s_mean;
  double acc = 0.0;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double2 v = x[r];
    double sw = sqrt(w[r]);
    double a = sw * (v.x - m.x), b = sw * (v.y - m.y);
    acc += a * a + b * b;
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

__global__ void sum_partials_kernel(const double* __restrict__ partial, int nparts, double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < nparts; ++b) s += partial[b];
    *out = s;
  }
}

}  // namespace vmc

using namespace vmc;

extern "C" size_t vmc_reduce_workspace_bytes(int64_t num_outputs) {
  return (size_t)kReduceBlocks * (size_t)(num_outputs > 0 ? num_outputs : 1) * 16 + 256;
}

extern "C" int vmc_weighted_mean_var(const double* x, const double* w, int64_t n, double* mean, double* var,
                                     void* workspace, size_t workspace_bytes, vmc_stream_t stream) {
  VMC_REQUIRE(x && w && mean && var && n > 0, VMC_ERR_INVALID_ARGUMENT, "vmc_weighted_mean_var: bad arguments");
  VMC_REQUIRE(workspace && workspace_bytes >= vmc_reduce_workspace_bytes(2), VMC_ERR_WORKSPACE,
              "vmc_weighted_mean_var: workspace of %zu bytes needed", vmc_reduce_workspace_bytes(2));
  double2* pm = reinterpret_cast<double2*>(workspace);
  double* pv = reinterpret_cast<double*>(pm + kReduceBlocks);
  cudaStream_t st = as_stream(stream);
  wmean_partial_kernel<<<kReduceBlocks, 256, 0, st>>>(reinterpret_cast<const double2*>(x), w, n, pm);
  int rc = check_launch("vmc_weighted_mean_var(mean)");
  if (rc) return rc;
  wvar_partial_kernel<<<kReduceBlocks, 256, 0, st>>>(reinterpret_cast<const double2*>(x), w, n, pm, kReduceBlocks,
                                                    reinterpret_cast<double2*>(mean), pv);
  rc = check_launch("vmc_weighted_mean_var(var)");
  if (rc) return rc;
  sum_partials_kernel<<<1, 32, 0, st>>>(pv, kReduceBlocks, var);
  return check_launch("vmc_weighted_mean_var(final)");
}
