// FP64 pieces of the SNR-regularised TDVP solve (util/tdvp.py:134-213),
// in the complex P-dimensional form of a holomorphic ansatz (the reference's
// 2P real representation has the same eigenvalues, each paired, and the
// same solution; see vmc_tdvp_regularize).
#include <algorithm>

#include "reduce.cuh"
#include "vmc_common.cuh"

namespace vmc {

// A[a][b] = (G[a][b] + G[P+a][P+b]) + i (G[a][P+b] - G[b][P+a]) from the Gram
// matrix G = R^T R of the real representation R = [Re X | Im X], reading only
// entries with row <= col (upper tiles), with A[b][a] = conj(A[a][b]) and
// the diagonal shift A[a][a] *= 1 + shift (tdvp.py:144-145).
// 32 x 32 output tiles (a0 <= b0 tile pairs): the G blocks a tile needs are
// read row-wise (coalesced), the transposed one through shared memory, and
// A[a][b] (a <= b), A[b][a] = conj(A[a][b]) are both written row-wise.  In a
// diagonal tile only a <= b is formed from G (the Gram kernel leaves some
// entries below the diagonal unwritten) and mirrored.
template <typename T>
__global__ void gram_to_hermitian_kernel(const T* __restrict__ G, int64_t ldg, int P, double shift,
                                         double2* __restrict__ A) {
  __shared__ double sRe[32][33];
  __shared__ double sIm[32][33];
  __shared__ double sT[32][33];
  const int nt = (P + 31) / 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
  for (int tile = blockIdx.x; tile < nt * nt; tile += gridDim.x) {
    const int ti = tile / nt, tj = tile - (tile / nt) * nt;
    if (ti > tj) continue;
    const int a0 = ti * 32, b0 = tj * 32;
    // sT[b - b0][a - a0] = G[b][P + a]   (row b, contiguous in a)
    for (int r = ty; r < 32; r += 8) {
      const int b = b0 + r, a = a0 + tx;
      sT[r][tx] = (b < P && a < P) ? (double)G[(int64_t)b * ldg + P + a] : 0.0;
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
      const int a = a0 + r, b = b0 + tx;
      double re = 0.0, im = 0.0;
      if (a < P && b < P && (ti != tj || a <= b)) {
        // row a, columns b: G[a][b], G[P+a][P+b], G[a][P+b] (all contiguous in b)
        re = (double)G[(int64_t)a * ldg + b] + (double)G[(int64_t)(P + a) * ldg + P + b];
        im = (double)G[(int64_t)a * ldg + P + b] - sT[tx][r];
        if (a == b) {
          im = 0.0;
          re *= (1.0 + shift);
        }
        A[(int64_t)a * P + b] = make_double2(re, im);
      }
      sRe[r][tx] = re;
      sIm[r][tx] = im;
    }
    __syncthreads();
    // mirrored entries: A[b][a] = conj(A[a][b]), written row-wise in a
    for (int r = ty; r < 32; r += 8) {
      const int b = b0 + r, a = a0 + tx;
      if (a < P && b < P && (ti != tj || a < b)) A[(int64_t)b * P + a] = make_double2(sRe[tx][r], -sIm[tx][r]);
    }
    __syncthreads();
  }
}

// y_k = sum_j conj(U_jk) x_j ; U column-major (U_jk at k*ld + j): warp per k.
__global__ void gemv_adjoint_kernel(const double2* __restrict__ U, int64_t ld, int n, const double2* __restrict__ x,
                                    double2* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t k = wid; k < n; k += nw) {
    const double2* col = U + k * ld;
    double re = 0.0, im = 0.0;
    for (int j = lane; j < n; j += 32) {
      double2 u = col[j], v = x[j];
      re += u.x * v.x + u.y * v.y;
      im += u.x * v.y - u.y * v.x;
    }
    re = warp_sum(re);
    im = warp_sum(im);
    if (lane == 0) y[k] = make_double2(re, im);
  }
}

// y_j = sum_k U_jk x_k ; U column-major.  Grid (j blocks of 256, k chunks):
// each block sums its k chunk for 256 consecutive j (coalesced), partial
// results are added in a fixed order by gemv_reduce_kernel.
constexpr int kGemvChunk = 256;
__global__ void gemv_partial_kernel(const double2* __restrict__ U, int64_t ld, int n, const double2* __restrict__ x,
                                    double2* __restrict__ part) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int k0 = blockIdx.y * kGemvChunk;
  const int k1 = min(n, k0 + kGemvChunk);
  double re = 0.0, im = 0.0;
  if (j < n) {
    for (int k = k0; k < k1; ++k) {
      const double2 u = U[(int64_t)k * ld + j], v = x[k];
      re += u.x * v.x - u.y * v.y;
      im += u.x * v.y + u.y * v.x;
    }
    part[(int64_t)blockIdx.y * n + j] = make_double2(re, im);
  }
}

__global__ void gemv_reduce_kernel(const double2* __restrict__ part, int chunks, int n, double2* __restrict__ y) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    double re = 0.0, im = 0.0;
    for (int c = 0; c < chunks; ++c) {
      const double2 v = part[(int64_t)c * n + j];
      re += v.x;
      im += v.y;
    }
    y[j] = make_double2(re, im);
  }
}

// The cutoff loop of TDVP.solve (tdvp.py:191-213) on the device, one block.
// Eigen-pairs (ev_k, u_k) of the complex P x P matrix A stand for the 2P
// real-representation pairs of the reference: the two members of a pair
// share |ev/ev_max|, the SNR and |pinv*ev - 1|, and together carry |u^H f|^2
// of the reference's |V^T F|^2, so the residual sums over k are identical.
//   invEv = 1/ev where |ev/ev_max| > 1e-14 else 0
//   cutoff = 1e-2; while residual > pinvTol and cutoff > pinvCutoff:
//     cutoff *= 0.8; reg = 1/(1 + (max(cutoff,pinvCutoff)/|ev/ev_max|)^6) [* 1/(1+(snrTol/snr)^6)]
//     pinvEv = invEv * reg; residual = ||(pinvEv ev - 1) VtF|| / ||F||
// out: pinv (n), result[0] = residual, result[1] = max(cutoff, pinvCutoff).
// The loop's iterations are independent given their cutoff, so every
// candidate cutoff c_m = 1e-2 * 0.8^m (formed by the same repeated products)
// is evaluated at once: blocks (element chunk, m) write partial sums of
// d^2 |VtF|^2, one block picks the first m whose residual <= pinvTol (or the
// last), and a third kernel writes pinv for that m.  The partial sums are
// added in a fixed order.
constexpr int kRegChunk = 2048;
constexpr int kRegMaxIter = 4096;

__device__ __forceinline__ double reg_cutoff(int m) {
  double c = 1e-2;
  for (int q = 0; q < m; ++q) c *= 0.8;
  return c;
}

__device__ __forceinline__ double reg_pinv(double e, double evMax, double c, const double* snr, double snrTol,
                                           int k) {
  const double rel = fabs(e / evMax);
  const double inv = rel > 1e-14 ? 1.0 / e : 0.0;
  const double q = c / rel;
  const double q2 = q * q;
  double reg = 1.0 / (1.0 + q2 * q2 * q2);
  if (snr) {
    const double sq = snrTol / snr[k];
    const double s2 = sq * sq;
    reg *= 1.0 / (1.0 + s2 * s2 * s2);
  }
  return inv * reg;
}

__global__ void __launch_bounds__(256) tdvp_reg_partial_kernel(const double* __restrict__ ev,
                                                               const double2* __restrict__ vtf,
                                                               const double* __restrict__ snr, int n,
                                                               double pinvCutoff, double snrTol,
                                                               double* __restrict__ part, int chunks) {
  const int chunk = blockIdx.x, m = blockIdx.y + 1;
  const double c0 = reg_cutoff(m);
  const double c = c0 > pinvCutoff ? c0 : pinvCutoff;
  const double evMax = ev[n - 1];  // ev ascending: ev[-1] of the reference
  double acc = 0.0;
  const int k1 = min(n, (chunk + 1) * kRegChunk);
  for (int k = chunk * kRegChunk + threadIdx.x; k < k1; k += blockDim.x) {
    const double e = ev[k];
    const double d = reg_pinv(e, evMax, c, snr, snrTol, k) * e - 1.0;
    acc += d * d * abs2(mk(vtf[k].x, vtf[k].y));
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) part[(size_t)(m - 1) * chunks + chunk] = acc;
}

// scalars: [0] chosen m (as double), [1] its cutoff
__global__ void tdvp_reg_select_kernel(const double2* __restrict__ vtf, int n, const double* __restrict__ part,
                                       int chunks, int M, double pinvCutoff, double pinvTol,
                                       double* __restrict__ result, double* __restrict__ scal) {
  double fn = 0.0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) fn += abs2(mk(vtf[k].x, vtf[k].y));
  // ||F||^2 = sum_k |u_k^H f|^2 (U unitary)
  fn = block_sum(fn);
  if (threadIdx.x != 0) return;
  const double Fnorm = sqrt(fn);
  double residual = 1.0, cutoff = 1e-2;
  int m = 0;
  // the reference loop: while residual > pinvTol and cutoff > pinvCutoff
  while (residual > pinvTol && cutoff > pinvCutoff && m < M) {
    ++m;
    cutoff *= 0.8;
    double acc = 0.0;
    for (int q = 0; q < chunks; ++q) acc += part[(size_t)(m - 1) * chunks + q];
    residual = sqrt(acc) / Fnorm;
  }
  const double c = cutoff > pinvCutoff ? cutoff : pinvCutoff;
  result[0] = residual;
  result[1] = c;
  result[2] = (double)m;
  scal[0] = (double)m;
  scal[1] = c;
}

__global__ void tdvp_reg_write_kernel(const double* __restrict__ ev, const double* __restrict__ snr, int n,
                                      double snrTol, const double* __restrict__ scal, double* __restrict__ pinv) {
  const double c = scal[1];
  const double evMax = ev[n - 1];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    pinv[k] = reg_pinv(ev[k], evMax, c, snr, snrTol, k);
}

// iterations the loop can run for pinvCutoff (host side, same products)
static int reg_iterations(double pinvCutoff) {
  double c = 1e-2;
  int m = 0;
  while (c > pinvCutoff && m < kRegMaxIter) {
    c *= 0.8;
    ++m;
  }
  return m;
}

// snr_k = sqrt(|N |VtF_k|^2 / rhoVar_k|) with rhoVar_k = colsq[k] + colsq[P+k]
// (the two real components of the complex projection, tdvp.py:173-181).
template <typename T>
__global__ void snr_kernel(const double2* __restrict__ vtf, const T* __restrict__ colsq, int n, int realRep,
                           double numSamples, double* __restrict__ snr, double* __restrict__ rhoVar) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    double rv = realRep ? (double)colsq[k] + (double)colsq[n + k] : (double)colsq[k];
    if (rhoVar) rhoVar[k] = rv;
    snr[k] = sqrt(fabs(numSamples * abs2(mk(vtf[k].x, vtf[k].y)) / rv));
  }
}

}  // namespace vmc

using namespace vmc;

extern "C" int vmc_gram_to_hermitian(int32_t gram_precision, const void* gram, int64_t ld_gram, int32_t num_params,
                                     double diag_shift, double* A, vmc_stream_t stream) {
  VMC_REQUIRE(gram && A && num_params > 0 && ld_gram >= 2 * (int64_t)num_params, VMC_ERR_INVALID_ARGUMENT,
              "vmc_gram_to_hermitian: bad arguments");
  const int64_t nt = ((int64_t)num_params + 31) / 32;
  int blocks = (int)std::min<int64_t>(nt * nt, 152 * 16);
  if (gram_precision == VMC_F64)
    gram_to_hermitian_kernel<double><<<blocks, 256, 0, as_stream(stream)>>>(
        reinterpret_cast<const double*>(gram), ld_gram, num_params, diag_shift, reinterpret_cast<double2*>(A));
  else
    gram_to_hermitian_kernel<float><<<blocks, 256, 0, as_stream(stream)>>>(
        reinterpret_cast<const float*>(gram), ld_gram, num_params, diag_shift, reinterpret_cast<double2*>(A));
  return check_launch("vmc_gram_to_hermitian");
}

extern "C" size_t vmc_zgemv_workspace_bytes(int32_t n) {
  return (size_t)((n + kGemvChunk - 1) / kGemvChunk) * (size_t)n * 16 + 256;
}

extern "C" int vmc_zgemv(int32_t adjoint, const double* U, int64_t ld, int32_t n, const double* x, double* y,
                         void* workspace, size_t workspace_bytes, vmc_stream_t stream) {
  VMC_REQUIRE(U && x && y && n > 0 && ld >= n, VMC_ERR_INVALID_ARGUMENT, "vmc_zgemv: bad arguments");
  if (adjoint) {
    int blocks = (int)std::min<int64_t>(((int64_t)n * 32 + 255) / 256, 152 * 16);
    gemv_adjoint_kernel<<<blocks, 256, 0, as_stream(stream)>>>(reinterpret_cast<const double2*>(U), ld, n,
                                                               reinterpret_cast<const double2*>(x),
                                                               reinterpret_cast<double2*>(y));
  } else {
    VMC_REQUIRE(workspace && workspace_bytes >= vmc_zgemv_workspace_bytes(n), VMC_ERR_WORKSPACE,
                "vmc_zgemv: workspace of %zu bytes needed", vmc_zgemv_workspace_bytes(n));
    const int chunks = (n + kGemvChunk - 1) / kGemvChunk;
    dim3 grid((n + 255) / 256, chunks);
    double2* part = reinterpret_cast<double2*>(workspace);
    gemv_partial_kernel<<<grid, 256, 0, as_stream(stream)>>>(reinterpret_cast<const double2*>(U), ld, n,
                                                            reinterpret_cast<const double2*>(x), part);
    int rc = check_launch("vmc_zgemv(partial)");
    if (rc) return rc;
    gemv_reduce_kernel<<<(n + 255) / 256, 256, 0, as_stream(stream)>>>(part, chunks, n,
                                                                      reinterpret_cast<double2*>(y));
  }
  return check_launch("vmc_zgemv");
}

extern "C" size_t vmc_tdvp_regularize_workspace_bytes(int32_t n, double pinv_cutoff) {
  const int chunks = (n + kRegChunk - 1) / kRegChunk;
  const int M = reg_iterations(pinv_cutoff);
  return ((size_t)(M > 0 ? M : 1) * chunks + 2) * sizeof(double) + 256;
}

extern "C" int vmc_tdvp_regularize(const double* ev, const double* vtf, const double* snr, int32_t n,
                                   double pinv_cutoff, double pinv_tol, double snr_tol, double* pinv, double* result,
                                   void* workspace, size_t workspace_bytes, vmc_stream_t stream) {
  VMC_REQUIRE(ev && vtf && pinv && result && n > 0, VMC_ERR_INVALID_ARGUMENT, "vmc_tdvp_regularize: bad arguments");
  const size_t need = vmc_tdvp_regularize_workspace_bytes(n, pinv_cutoff);
  VMC_REQUIRE(workspace && workspace_bytes >= need, VMC_ERR_WORKSPACE,
              "vmc_tdvp_regularize: workspace of %zu bytes needed", need);
  const int chunks = (n + kRegChunk - 1) / kRegChunk;
  const int M = reg_iterations(pinv_cutoff);
  double* part = reinterpret_cast<double*>(workspace);
  double* scal = part + (size_t)(M > 0 ? M : 1) * chunks;
  cudaStream_t st = as_stream(stream);
  const double2* v2 = reinterpret_cast<const double2*>(vtf);
  if (M > 0) {
    tdvp_reg_partial_kernel<<<dim3(chunks, M), 256, 0, st>>>(ev, v2, snr, n, pinv_cutoff, snr_tol, part, chunks);
    int rc = check_launch("vmc_tdvp_regularize(partial)");
    if (rc) return rc;
  }
  tdvp_reg_select_kernel<<<1, 1024, 0, st>>>(v2, n, part, chunks, M, pinv_cutoff, pinv_tol, result, scal);
  int rc = check_launch("vmc_tdvp_regularize(select)");
  if (rc) return rc;
  tdvp_reg_write_kernel<<<(n + 255) / 256, 256, 0, st>>>(ev, snr, n, snr_tol, scal, pinv);
  return check_launch("vmc_tdvp_regularize");
}

extern "C" int vmc_tdvp_snr(const double* vtf, int32_t colsq_precision, const void* colsq, int32_t n,
                            int32_t real_rep, double num_samples, double* snr, double* rho_var, vmc_stream_t stream) {
  VMC_REQUIRE(vtf && colsq && snr && n > 0, VMC_ERR_INVALID_ARGUMENT, "vmc_tdvp_snr: bad arguments");
  int blocks = (n + 255) / 256;
  if (colsq_precision == VMC_F64)
    snr_kernel<double><<<blocks, 256, 0, as_stream(stream)>>>(reinterpret_cast<const double2*>(vtf),
                                                              reinterpret_cast<const double*>(colsq), n, real_rep,
                                                              num_samples, snr, rho_var);
  else
    snr_kernel<float><<<blocks, 256, 0, as_stream(stream)>>>(reinterpret_cast<const double2*>(vtf),
                                                             reinterpret_cast<const float*>(colsq), n, real_rep,
                                                             num_samples, snr, rho_var);
  return check_launch("vmc_tdvp_snr");
}

#include <cuda_bf16.h>

namespace vmc {
// Bt[c][k] = B[k][c] with B = [[Ur, -Ui], [Ui, Ur]] (U column-major: U_jk at k*ldu + j).
__global__ void eigvec_bf16x2_kernel(const double2* __restrict__ U, int64_t ldu, int P, __nv_bfloat16* __restrict__ hi,
                                     __nv_bfloat16* __restrict__ lo, int64_t ld) {
  const int64_t n2 = 2 * (int64_t)P;
  const int64_t total = n2 * n2;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(t / n2), k = (int)(t - (t / n2) * n2);
    const int cc = c < P ? c : c - P, kk = k < P ? k : k - P;
    const double2 u = U[(int64_t)cc * ldu + kk];
    double v;
    if (c < P) v = k < P ? u.x : u.y;
    else v = k < P ? -u.y : u.x;
    const float f = (float)v;
    const __nv_bfloat16 h = __float2bfloat16_rn(f);
    hi[(int64_t)c * ld + k] = h;
    lo[(int64_t)c * ld + k] = __float2bfloat16_rn(f - __bfloat162float(h));
  }
}
}  // namespace vmc

extern "C" int vmc_eigvec_bf16x2(const double* U, int64_t ldu, int32_t num_params, void* bt_hi, void* bt_lo,
                                 int64_t ld, vmc_stream_t stream) {
  VMC_REQUIRE(U && bt_hi && bt_lo && num_params > 0 && ldu >= num_params && ld >= 2 * (int64_t)num_params,
              VMC_ERR_INVALID_ARGUMENT, "vmc_eigvec_bf16x2: bad arguments");
  const int64_t total = 4 * (int64_t)num_params * num_params;
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, 152 * 32);
  eigvec_bf16x2_kernel<<<blocks, 256, 0, as_stream(stream)>>>(reinterpret_cast<const double2*>(U), ldu, num_params,
                                                              reinterpret_cast<__nv_bfloat16*>(bt_hi),
                                                              reinterpret_cast<__nv_bfloat16*>(bt_lo), ld);
  return check_launch("vmc_eigvec_bf16x2");
}
