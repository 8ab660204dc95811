// Complex RBM parameter view and host helpers shared by the plain and the
// symmetrised RBM kernels.
#pragma once

#include "vmc_common.cuh"

namespace vmc {

constexpr int kWarpsPerBlock = 8;
constexpr int kMaxSites = 4096;
constexpr int kMaxHidden = 4096;

template <typename T>
struct rbm_params {
  const cpx<T>* W;  // (L, M)
  const cpx<T>* b;  // (M) or null
  int L, M;
};

template <typename T>
rbm_params<T> make_params(const void* kernel, const void* bias, int L, int M) {
  rbm_params<T> p;
  p.W = reinterpret_cast<const cpx<T>*>(kernel);
  p.b = reinterpret_cast<const cpx<T>*>(bias);
  p.L = L;
  p.M = M;
  return p;
}

// grid of a one-warp-per-configuration kernel over N configurations
int grid_for(int64_t N);
// precision, pointers and size limits of an RBM entry point
int check_rbm_args(const char* fn, int32_t precision, const int32_t* configs, int64_t N, int32_t L, int32_t M,
                   const void* kernel);
// raise the dynamic shared-memory limit of `fn` when above 48 KB

}  // namespace vmc
