// Eigendecomposition of the Hermitian S matrix of the TDVP solve
// (tdvp.py:153-171, jnp.linalg.eigh), GB300 form:
//
//   1. vmc_eigh_fp32: complex64 eigendecomposition by cuSOLVER (the O(n^3)
//      tridiagonal reduction and back-transformation at FP32 rates), vectors
//      and values returned widened to complex128 / FP64.
//   2. vmc_eigh_refine_top: the k eigenpairs of largest eigenvalue made
//      FP64-accurate, the rest made orthogonal to them:
//        X = top-k FP32 vectors;  q times X <- A X diag(1/lambda)   (the
//        components of X along the other n - k eigenvectors shrink by
//        |lambda_{n-k-1} / lambda_j| per step);
//        Rayleigh-Ritz in FP64: G = X^H X, H = X^H A X, H c = theta G c
//        (cuSOLVER zhegvd on k x k);  V_top = X C, ev_top = theta;
//        V_rest <- V_rest - V_top (V_top^H V_rest), columns renormalised
//        (orthogonal to V_top to ~1e-12: V_top^H V_rest from 6 slices).
//      Every O(n^2 k) product runs as an FP64-accurate Ozaki-split product
//      on the BF16 tensor cores (oz_host.h).  The n - k other eigenvalues
//      keep their FP32 values (absolute error ~1e-7 of the largest); the
//      caller picks k so that the part of the solve they carry is negligible
//      (util/tdvp.py: the largest spectral gap above the FP32 noise floor,
//      and after step 2 the share of the update left on the unrefined
//      eigenpairs, which must be below 1e-6).
//
// cuSOLVER is called through handles leased from a per-process pool (one
// per concurrent call and device); its device workspace comes from the
// caller's workspace, its small host workspace from a per-thread buffer.
#include <cusolverDn.h>

#include <cstddef>
#include <mutex>
#include <vector>

#include "oz_host.h"
#include "vmc_common.cuh"

namespace vmc {

namespace {

struct solver_slot {
  cusolverDnHandle_t h = nullptr;
  cusolverDnParams_t p = nullptr;
  int dev = -1;
};

// cuSOLVER handles are created on demand and reused: a call leases a free
// handle of its device for its duration and gives it back, so host threads
// that come and go (one per serving step) share a few handles instead of
// each leaving one behind.  The handles live until the process ends.
std::mutex& pool_mutex() {
  static std::mutex m;
  return m;
}
std::vector<solver_slot*>& pool_free() {
  static std::vector<solver_slot*> v;
  return v;
}

class solver_lease {
 public:
  solver_lease() = default;
  solver_lease(const solver_lease&) = delete;
  solver_lease& operator=(const solver_lease&) = delete;
  ~solver_lease() {
    if (s_) {
      std::lock_guard<std::mutex> g(pool_mutex());
      pool_free().push_back(s_);
    }
  }
  // A handle of the current device bound to st.
  int acquire(cudaStream_t st) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    VMC_REQUIRE(e == cudaSuccess, VMC_ERR_CUDA, "eigh: %s", cudaGetErrorString(e));
    {
      std::lock_guard<std::mutex> g(pool_mutex());
      std::vector<solver_slot*>& v = pool_free();
      for (size_t i = 0; i < v.size(); ++i) {
        if (v[i]->dev == dev) {
          s_ = v[i];
          v.erase(v.begin() + (std::ptrdiff_t)i);
          break;
        }
      }
    }
    if (!s_) {
      solver_slot* n = new solver_slot;
      n->dev = dev;
      if (cusolverDnCreate(&n->h) != CUSOLVER_STATUS_SUCCESS) {
        delete n;
        VMC_REQUIRE(false, VMC_ERR_CUDA, "eigh: cusolverDnCreate failed");
      }
      if (cusolverDnCreateParams(&n->p) != CUSOLVER_STATUS_SUCCESS) {
        cusolverDnDestroy(n->h);
        delete n;
        VMC_REQUIRE(false, VMC_ERR_CUDA, "eigh: cusolverDnCreateParams failed");
      }
      s_ = n;
    }
    VMC_REQUIRE(cusolverDnSetStream(s_->h, st) == CUSOLVER_STATUS_SUCCESS, VMC_ERR_CUDA, "eigh: cusolverDnSetStream");
    return VMC_OK;
  }
  solver_slot* operator->() const { return s_; }

 private:
  solver_slot* s_ = nullptr;
};

std::vector<char>& host_scratch() {
  static thread_local std::vector<char> buf;
  return buf;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

__global__ void to_c64_kernel(const double2* __restrict__ A, int64_t lda, int n, float2* __restrict__ B) {
  const int64_t total = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t / n, r = t - c * n;
    const double2 v = A[c * lda + r];
    B[t] = make_float2((float)v.x, (float)v.y);
  }
}

__global__ void from_c64_kernel(const float2* __restrict__ B, const float* __restrict__ w, int n,
                                double2* __restrict__ V, int64_t ldv, double* __restrict__ ev) {
  const int64_t total = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t / n, r = t - c * n;
    const float2 v = B[t];
    V[c * ldv + r] = make_double2((double)v.x, (double)v.y);
    if (t < n) ev[t] = (double)w[t];
  }
}

// X[:, j] *= 1 / s[j] (s != 0)
__global__ void scale_columns_kernel(double2* __restrict__ X, int64_t ldx, int n, int k, const double* __restrict__ s) {
  const int64_t total = (int64_t)n * k;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t / n, r = t - c * n;
    const double d = s[c];
    const double f = d != 0.0 ? 1.0 / d : 1.0;
    double2 v = X[c * ldx + r];
    v.x *= f;
    v.y *= f;
    X[c * ldx + r] = v;
  }
}

// Every column of V (n rows, ldv) scaled to unit 2-norm (one block per column,
// FP64 sum in a fixed order).
__global__ void normalise_columns_kernel(double2* __restrict__ V, int64_t ldv, int n) {
  __shared__ double part[32];
  double2* col = V + (int64_t)blockIdx.x * ldv;
  double s = 0.0;
  for (int r = threadIdx.x; r < n; r += blockDim.x) s += col[r].x * col[r].x + col[r].y * col[r].y;
  for (int o = 16; o >= 1; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.0;
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) part[0] = v;
  }
  __syncthreads();
  const double f = part[0] > 0.0 ? 1.0 / sqrt(part[0]) : 1.0;
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    col[r].x *= f;
    col[r].y *= f;
  }
}

int grid_for(int64_t total) {
  int64_t g = (total + 255) / 256;
  return (int)(g < 8192 ? (g > 0 ? g : 1) : 8192);
}

constexpr int kSlices = 8, kLevel = 7;            // FP64-accurate products
constexpr int kEarlySlices = 6, kEarlyLevel = 5;  // power steps before the last (2^-40 relative)
constexpr int kRestSlices = 5, kRestLevel = 4;    // V_top T: T ~ 1e-7, error 2^-33 of |V_top| |T| (negligible)
constexpr int kProjSlices = 6, kProjLevel = 5;    // T = V_top^H V_rest: error 2^-40 of |V_top| |V_rest| = 1
constexpr int kRestChunk = 4096;                  // columns of V_rest per orthogonalisation pass

struct refine_layout {
  size_t opA, opB, opC, out, X, Y, G, H, w, T, solver, total;
};

int hegvd_lwork(int k, int* lwork, cudaStream_t st) {
  solver_lease s;
  int rc = s.acquire(st);
  if (rc) return rc;
  VMC_REQUIRE(cusolverDnZhegvd_bufferSize(s->h, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR,
                                          CUBLAS_FILL_MODE_UPPER, k, nullptr, k, nullptr, k, nullptr,
                                          lwork) == CUSOLVER_STATUS_SUCCESS,
              VMC_ERR_CUDA, "eigh: zhegvd workspace query failed");
  return VMC_OK;
}

int refine_layout_for(int n, int k, refine_layout& L, cudaStream_t st) {
  const int b = n - k;
  const int rc_cols = b < kRestChunk ? b : kRestChunk;
  int lwork = 0;
  int rc = hegvd_lwork(k, &lwork, st);
  if (rc) return rc;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += align256(bytes);
    return o;
  };
  // A-operand buffer: A (n rows, K n), later V_top^H (k, K n)
  const size_t aBytes = oz_operand_bytes(n, n, kSlices, false);
  // B-operand buffer: X, Y (k rows, K n) / C (k, K k) / V_rest chunk (rc, K n) / T chunk (rc, K k)
  size_t bBytes = oz_operand_bytes(k, n, kSlices, true);
  if (rc_cols > 0) {
    const size_t v = oz_operand_bytes(rc_cols, n, kProjSlices, true);
    if (v > bBytes) bBytes = v;
  }
  // second A-operand buffer: X^H (k, K n) for G and H, X (n, K k) for X C, V_top (n, K k)
  size_t cBytes = oz_operand_bytes(k, n, kSlices, false);
  const size_t cN = oz_operand_bytes(n, k, kSlices, false);
  if (cN > cBytes) cBytes = cN;
  size_t outBytes = oz_out_bytes(n, k);
  if (rc_cols > 0) {
    if (oz_out_bytes(k, rc_cols) > outBytes) outBytes = oz_out_bytes(k, rc_cols);
    if (oz_out_bytes(n, rc_cols) > outBytes) outBytes = oz_out_bytes(n, rc_cols);
  }
  L.opA = take(aBytes);
  L.opB = take(bBytes);
  L.opC = take(cBytes);
  L.out = take(outBytes);
  L.X = take((size_t)n * k * 16);
  L.Y = take((size_t)n * k * 16);
  L.G = take((size_t)k * k * 16);
  L.H = take((size_t)k * k * 16);
  L.w = take((size_t)k * 8 + 16);
  L.T = take((size_t)k * (rc_cols > 0 ? rc_cols : 1) * 16);
  L.solver = take((size_t)lwork * 16 + 16);
  L.total = off + 256;
  return VMC_OK;
}

size_t fp32_device_bytes(int n, cudaStream_t st, size_t* hostBytes) {
  solver_lease s;
  if (s.acquire(st)) return 0;
  size_t dev = 0, host = 0;
  if (cusolverDnXsyevd_bufferSize(s->h, s->p, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, CUDA_C_32F,
                                  nullptr, n, CUDA_R_32F, nullptr, CUDA_C_32F, &dev, &host) != CUSOLVER_STATUS_SUCCESS)
    return 0;
  if (hostBytes) *hostBytes = host;
  return dev;
}

}  // namespace

}  // namespace vmc

using namespace vmc;

extern "C" size_t vmc_eigh_fp32_workspace_bytes(int32_t n) {
  if (n <= 0) return 0;
  const size_t dev = fp32_device_bytes(n, 0, nullptr);
  if (!dev) return 0;
  return align256((size_t)n * n * 8) + align256((size_t)n * 4) + align256(dev) + 256;
}

extern "C" int vmc_eigh_fp32(int32_t n, const double* A, int64_t lda, double* ev, double* V, int64_t ldv,
                             void* workspace, size_t workspace_bytes, int32_t* info, vmc_stream_t stream) {
  VMC_REQUIRE(n > 0 && A && ev && V && info && lda >= n && ldv >= n, VMC_ERR_INVALID_ARGUMENT,
              "vmc_eigh_fp32: bad arguments");
  cudaStream_t st = as_stream(stream);
  size_t hostBytes = 0;
  const size_t dev = fp32_device_bytes(n, st, &hostBytes);
  VMC_REQUIRE(dev > 0, VMC_ERR_CUDA, "vmc_eigh_fp32: cuSOLVER workspace query failed");
  const size_t need = align256((size_t)n * n * 8) + align256((size_t)n * 4) + align256(dev) + 256;
  VMC_REQUIRE(workspace && workspace_bytes >= need, VMC_ERR_WORKSPACE, "vmc_eigh_fp32: workspace of %zu bytes needed",
              need);
  char* ws = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~(uintptr_t)255);
  float2* A32 = reinterpret_cast<float2*>(ws);
  float* w32 = reinterpret_cast<float*>(ws + align256((size_t)n * n * 8));
  void* dws = ws + align256((size_t)n * n * 8) + align256((size_t)n * 4);
  const int64_t total = (int64_t)n * n;
  to_c64_kernel<<<grid_for(total), 256, 0, st>>>(reinterpret_cast<const double2*>(A), lda, n, A32);
  int rc = check_launch("vmc_eigh_fp32(convert)");
  if (rc) return rc;
  solver_lease s;
  if ((rc = s.acquire(st))) return rc;
  std::vector<char>& hb = host_scratch();
  if (hb.size() < hostBytes + 1) hb.resize(hostBytes + 1);
  const cusolverStatus_t cs =
      cusolverDnXsyevd(s->h, s->p, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, CUDA_C_32F, A32, n,
                       CUDA_R_32F, w32, CUDA_C_32F, dws, dev, hb.data(), hostBytes, info);
  VMC_REQUIRE(cs == CUSOLVER_STATUS_SUCCESS, VMC_ERR_CUDA, "vmc_eigh_fp32: cusolverDnXsyevd failed (%d)", (int)cs);
  from_c64_kernel<<<grid_for(total), 256, 0, st>>>(A32, w32, n, reinterpret_cast<double2*>(V), ldv, ev);
  return check_launch("vmc_eigh_fp32(widen)");
}

extern "C" size_t vmc_eigh_refine_workspace_bytes(int32_t n, int32_t k) {
  if (n <= 0 || k <= 0 || k > n) return 0;
  refine_layout L;
  if (refine_layout_for(n, k, L, 0)) return 0;
  return L.total;
}

extern "C" int vmc_eigh_refine_top(int32_t n, const double* A, int64_t lda, int32_t k, int32_t power_steps,
                                   double* ev, double* V, int64_t ldv, void* workspace, size_t workspace_bytes,
                                   int32_t* status, int32_t* info, vmc_stream_t stream) {
  VMC_REQUIRE(n > 0 && k > 0 && k <= n && A && ev && V && info && lda >= n && ldv >= n, VMC_ERR_INVALID_ARGUMENT,
              "vmc_eigh_refine_top: bad arguments");
  VMC_REQUIRE(power_steps >= 0 && power_steps <= 32, VMC_ERR_INVALID_ARGUMENT,
              "vmc_eigh_refine_top: power_steps %d outside [0, 32]", power_steps);
  VMC_REQUIRE(2 * (int64_t)n <= 61440, VMC_ERR_UNSUPPORTED, "vmc_eigh_refine_top: n = %d above 30720", n);
  VMC_REQUIRE(((uintptr_t)A & 15) == 0 && ((uintptr_t)V & 15) == 0, VMC_ERR_INVALID_ARGUMENT,
              "vmc_eigh_refine_top: complex128 arrays must be 16-byte aligned");
  cudaStream_t st = as_stream(stream);
  refine_layout L;
  int rc = refine_layout_for(n, k, L, st);
  if (rc) return rc;
  VMC_REQUIRE(workspace && workspace_bytes >= L.total, VMC_ERR_WORKSPACE,
              "vmc_eigh_refine_top: workspace of %zu bytes needed", L.total);
  char* ws = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~(uintptr_t)255);
  void* bufA = ws + L.opA;
  void* bufB = ws + L.opB;
  void* bufC = ws + L.opC;
  double* out = reinterpret_cast<double*>(ws + L.out);
  double* X = reinterpret_cast<double*>(ws + L.X);
  double* Y = reinterpret_cast<double*>(ws + L.Y);
  double* G = reinterpret_cast<double*>(ws + L.G);
  double* H = reinterpret_cast<double*>(ws + L.H);
  double* w = reinterpret_cast<double*>(ws + L.w);
  double* T = reinterpret_cast<double*>(ws + L.T);
  const int b = n - k;
  double* Vtop = V + 2 * (int64_t)b * ldv;

  // A as the A operand of A X (A Hermitian: A X = A^H X), sliced once
  oz_operand opA, opB, opC;
  oz_make_operand(bufA, n, n, kSlices, false, opA);
  if ((rc = oz_slice(A, 1, lda, 0, opA, false, st))) return rc;

  // X = top-k FP32 vectors
  cudaError_t e = cudaMemcpy2DAsync(X, (size_t)n * 16, Vtop, (size_t)ldv * 16, (size_t)n * 16, k,
                                    cudaMemcpyDeviceToDevice, st);
  VMC_REQUIRE(e == cudaSuccess, VMC_ERR_CUDA, "vmc_eigh_refine_top: %s", cudaGetErrorString(e));

  // power steps X <- A X diag(1 / lambda).  An error of the products is
  // damped like the FP32 error by every later step, so the steps before the
  // last use 6 slices and levels <= 5 (2^-40 relative): after one more step
  // it is below 2^-40 rho.
  for (int step = 0; step < power_steps; ++step) {
    const bool last = step == power_steps - 1;
    oz_make_operand(bufB, k, n, last ? kSlices : kEarlySlices, true, opB);
    if ((rc = oz_slice(X, 1, n, 0, opB, true, st))) return rc;
    if ((rc = oz_multiply(opA, opB, last ? kLevel : kEarlyLevel, false, out, status, st))) return rc;
    if ((rc = oz_finish(out, opA, opB, false, X, n, false, st, 1.0))) return rc;
    scale_columns_kernel<<<grid_for((int64_t)n * k), 256, 0, st>>>(reinterpret_cast<double2*>(X), n, n, k, ev + b);
    if ((rc = check_launch("vmc_eigh_refine_top(scale)"))) return rc;
  }

  // Rayleigh-Ritz: Y = A X, G = X^H X, H = X^H Y
  oz_make_operand(bufB, k, n, kSlices, true, opB);
  if ((rc = oz_slice(X, 1, n, 0, opB, true, st))) return rc;
  if ((rc = oz_multiply(opA, opB, kLevel, false, out, status, st))) return rc;
  if ((rc = oz_finish(out, opA, opB, false, Y, n, false, st, 1.0))) return rc;
  oz_make_operand(bufC, k, n, kSlices, false, opC);
  if ((rc = oz_slice(X, 1, n, 0, opC, false, st))) return rc;
  if ((rc = oz_multiply(opC, opB, kLevel, true, out, status, st))) return rc;
  if ((rc = oz_finish(out, opC, opB, true, G, k, false, st, 1.0))) return rc;
  if ((rc = oz_slice(Y, 1, n, 0, opB, true, st))) return rc;
  if ((rc = oz_multiply(opC, opB, kLevel, true, out, status, st))) return rc;
  if ((rc = oz_finish(out, opC, opB, true, H, k, false, st, 1.0))) return rc;

  // H c = theta G c in FP64
  solver_lease s;
  if ((rc = s.acquire(st))) return rc;
  int lwork = 0;
  if ((rc = hegvd_lwork(k, &lwork, st))) return rc;
  const cusolverStatus_t cs = cusolverDnZhegvd(
      s->h, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, k,
      reinterpret_cast<cuDoubleComplex*>(H), k, reinterpret_cast<cuDoubleComplex*>(G), k, w,
      reinterpret_cast<cuDoubleComplex*>(ws + L.solver), lwork, info);
  VMC_REQUIRE(cs == CUSOLVER_STATUS_SUCCESS, VMC_ERR_CUDA, "vmc_eigh_refine_top: cusolverDnZhegvd failed (%d)",
              (int)cs);

  // V_top = X C (op = X: P[kk][m] = conj(X[m + kk n])), ev_top = theta
  oz_make_operand(bufC, n, k, kSlices, false, opC);
  if ((rc = oz_slice(X, n, 1, 1, opC, false, st))) return rc;
  oz_make_operand(bufB, k, k, kSlices, true, opB);
  if ((rc = oz_slice(H, 1, k, 0, opB, true, st))) return rc;
  if ((rc = oz_multiply(opC, opB, kLevel, false, out, status, st))) return rc;
  if ((rc = oz_finish(out, opC, opB, false, Vtop, ldv, false, st, 1.0))) return rc;
  e = cudaMemcpyAsync(ev + b, w, (size_t)k * 8, cudaMemcpyDeviceToDevice, st);
  VMC_REQUIRE(e == cudaSuccess, VMC_ERR_CUDA, "vmc_eigh_refine_top: %s", cudaGetErrorString(e));

  // V_rest <- V_rest - V_top (V_top^H V_rest), in column chunks
  if (b > 0) {
    oz_operand opVtH, opVtN;
    // V_top^H as A operand (rows k, K n) in bufA (A no longer needed), V_top as A operand (rows n, K k) in bufC
    oz_make_operand(bufA, k, n, kProjSlices, false, opVtH);
    if ((rc = oz_slice(Vtop, 1, ldv, 0, opVtH, false, st))) return rc;
    oz_make_operand(bufC, n, k, kRestSlices, false, opVtN);
    if ((rc = oz_slice(Vtop, ldv, 1, 1, opVtN, false, st))) return rc;
    for (int c0 = 0; c0 < b; c0 += kRestChunk) {
      const int cols = b - c0 < kRestChunk ? b - c0 : kRestChunk;
      double* Vc = V + 2 * (int64_t)c0 * ldv;
      oz_make_operand(bufB, cols, n, kProjSlices, true, opB);
      if ((rc = oz_slice(Vc, 1, ldv, 0, opB, true, st))) return rc;
      if ((rc = oz_multiply(opVtH, opB, kProjLevel, false, out, status, st))) return rc;
      if ((rc = oz_finish(out, opVtH, opB, false, T, k, false, st, 1.0))) return rc;
      oz_make_operand(bufB, cols, k, kRestSlices, true, opB);
      if ((rc = oz_slice(T, 1, k, 0, opB, true, st))) return rc;
      if ((rc = oz_multiply(opVtN, opB, kRestLevel, false, out, status, st))) return rc;
      if ((rc = oz_finish(out, opVtN, opB, false, Vc, ldv, true, st, -1.0))) return rc;
    }
    normalise_columns_kernel<<<b, 256, 0, st>>>(reinterpret_cast<double2*>(V), ldv, n);
    if ((rc = check_launch("vmc_eigh_refine_top(normalise)"))) return rc;
  }
  return VMC_OK;
}

// ---------------------------------------------------------------------------
// FP64 eigendecomposition by cuSOLVER (the reference's jnp.linalg.eigh in
// FP64, tdvp.py:157): complex Hermitian or real symmetric A (column-major);
// ev ascending, eigenvectors overwrite V (A is copied into V first, so A may
// alias V).
// ---------------------------------------------------------------------------
namespace vmc {
namespace {
size_t fp64_device_bytes(int n, int cplx, cudaStream_t st, size_t* hostBytes) {
  solver_lease s;
  if (s.acquire(st)) return 0;
  size_t dev = 0, host = 0;
  const cudaDataType ta = cplx ? CUDA_C_64F : CUDA_R_64F;
  if (cusolverDnXsyevd_bufferSize(s->h, s->p, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, ta, nullptr, n,
                                  CUDA_R_64F, nullptr, ta, &dev, &host) != CUSOLVER_STATUS_SUCCESS)
    return 0;
  if (hostBytes) *hostBytes = host;
  return dev > 0 ? dev : 1;
}
}  // namespace
}  // namespace vmc

extern "C" size_t vmc_eigh_fp64_workspace_bytes(int32_t n, int32_t is_complex) {
  if (n <= 0) return 0;
  const size_t dev = fp64_device_bytes(n, is_complex != 0, 0, nullptr);
  return dev ? align256(dev) + 256 : 0;
}

extern "C" int vmc_eigh_fp64(int32_t n, int32_t is_complex, const double* A, int64_t lda, double* ev, double* V,
                             int64_t ldv, void* workspace, size_t workspace_bytes, int32_t* info,
                             vmc_stream_t stream) {
  VMC_REQUIRE(n > 0 && A && ev && V && info && lda >= n && ldv >= n, VMC_ERR_INVALID_ARGUMENT,
              "vmc_eigh_fp64: bad arguments");
  cudaStream_t st = as_stream(stream);
  const int cplx = is_complex != 0;
  size_t hostBytes = 0;
  const size_t dev = fp64_device_bytes(n, cplx, st, &hostBytes);
  VMC_REQUIRE(dev > 0, VMC_ERR_CUDA, "vmc_eigh_fp64: cuSOLVER workspace query failed");
  VMC_REQUIRE(workspace && workspace_bytes >= align256(dev) + 256, VMC_ERR_WORKSPACE,
              "vmc_eigh_fp64: workspace of %zu bytes needed", align256(dev) + 256);
  void* dws = reinterpret_cast<void*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~(uintptr_t)255);
  const size_t el = cplx ? 16 : 8;
  if (A != V) {
    cudaError_t e = cudaMemcpy2DAsync(V, (size_t)ldv * el, A, (size_t)lda * el, (size_t)n * el, n,
                                      cudaMemcpyDeviceToDevice, st);
    VMC_REQUIRE(e == cudaSuccess, VMC_ERR_CUDA, "vmc_eigh_fp64: %s", cudaGetErrorString(e));
  }
  solver_lease s;
  int rc = s.acquire(st);
  if (rc) return rc;
  std::vector<char>& hb = host_scratch();
  if (hb.size() < hostBytes + 1) hb.resize(hostBytes + 1);
  const cudaDataType ta = cplx ? CUDA_C_64F : CUDA_R_64F;
  const cusolverStatus_t cs = cusolverDnXsyevd(s->h, s->p, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, ta, V,
                                               ldv, CUDA_R_64F, ev, ta, dws, dev, hb.data(), hostBytes, info);
  VMC_REQUIRE(cs == CUSOLVER_STATUS_SUCCESS, VMC_ERR_CUDA, "vmc_eigh_fp64: cusolverDnXsyevd failed (%d)", (int)cs);
  return VMC_OK;
}
