// Statistics and centred data of materialised log-derivatives O (N, P)
// complex128 (row stride ld_o elements) of any holomorphic network, for the
// same S/F build and SNR transform as the CpxRBM producers of rbm_gram.cu
// (stats.py:50-58, 197-205, 255-292 via tdvp.py:134-181):
//   ok_mean_k = sum_n w_n O_nk
//   covOE_k   = sum_n w_n conj(O_nk - ok_mean_k) (E_n - Ebar)
//   X_nk = sqrt(w_n) (O_nk - ok_mean_k)
//   H_nk = sqrt(w_n) ((-x) (E_n - Ebar) conj(O_nk - ok_mean_k) - f_k)
// The statistics are fixed-order reductions (per-chunk partial sums, then a
// per-column sum over the chunks in order).
#include <cuda_bf16.h>

#include <algorithm>

#include "reduce.cuh"
#include "vmc_common.cuh"

namespace vmc {

constexpr int kDenseChunks = 64;
constexpr int kDenseCols = 256;

// partial sums of w O and w conj(O) dE over the rows of chunk blockIdx.y,
// one column per thread; chunk sums of w dE from the first column block
__global__ void __launch_bounds__(kDenseCols) dense_stats_partial_kernel(
    const double2* __restrict__ O, int64_t ld, int64_t N, int64_t P, const double* __restrict__ w,
    const double2* __restrict__ E, const double2* __restrict__ Ebar, double2* __restrict__ pm,
    double2* __restrict__ pc, double2* __restrict__ pe) {
  const int64_t k = (int64_t)blockIdx.x * kDenseCols + threadIdx.x;
  const int c = blockIdx.y;
  const int64_t rows = (N + kDenseChunks - 1) / kDenseChunks;
  const int64_t r0 = c * rows, r1 = min(N, r0 + rows);
  const double2 eb = *Ebar;
  cpx<double> sm = mk(0.0, 0.0), sc = mk(0.0, 0.0), se = mk(0.0, 0.0);
  for (int64_t n = r0; n < r1; ++n) {
    const double wn = w[n];
    const double2 e = E[n];
    const cpx<double> de = mk(wn * (e.x - eb.x), wn * (e.y - eb.y));
    if (k < P) {
      const double2 o = O[n * ld + k];
      sm = sm + mk(wn * o.x, wn * o.y);
      sc = sc + mk(o.x, -o.y) * de;
    }
    se = se + de;
  }
  if (k < P) {
    pm[(size_t)c * P + k] = make_double2(sm.re, sm.im);
    pc[(size_t)c * P + k] = make_double2(sc.re, sc.im);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) pe[c] = make_double2(se.re, se.im);
}

__global__ void dense_stats_final_kernel(const double2* __restrict__ pm, const double2* __restrict__ pc,
                                         const double2* __restrict__ pe, int64_t P, double2* __restrict__ okMean,
                                         double2* __restrict__ covOE) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= P) return;
  cpx<double> m = mk(0.0, 0.0), c = mk(0.0, 0.0), e = mk(0.0, 0.0);
  for (int q = 0; q < kDenseChunks; ++q) {
    const double2 a = pm[(size_t)q * P + k], b = pc[(size_t)q * P + k], d = pe[q];
    m = m + mk(a.x, a.y);
    c = c + mk(b.x, b.y);
    e = e + mk(d.x, d.y);
  }
  // sum w conj(O - m) dE = sum w conj(O) dE - conj(m) sum w dE
  c = c - conjg(m) * e;
  okMean[k] = make_double2(m.re, m.im);
  covOE[k] = make_double2(c.re, c.im);
}

struct dense_args {
  const double2* O;
  int64_t ldo, N, P;
  const double* w;
  const double2* okMean;
  const double2* eloc;      // null: gradient data
  const double2* elocMean;
  double2 xfac;             // -x
  int realPart;             // SNR data of a real-parameter net (makeReal = Re)
  const double2* force;
  int format;
  int64_t ld;
  void* out;
  void* out2;
};

__device__ __forceinline__ cpx<double> dense_value(const dense_args& a, int64_t n, int64_t k) {
  const double2 o = a.O[n * a.ldo + k], mu = a.okMean[k];
  cpx<double> d = mk(o.x - mu.x, o.y - mu.y);
  if (a.eloc) {
    const double2 e = a.eloc[n], em = *a.elocMean;
    const cpx<double> h = mk(a.xfac.x, a.xfac.y) * (mk(e.x - em.x, e.y - em.y) * conjg(d));
    const double2 f = a.force[k];
    d = a.realPart ? mk(h.re - f.x, 0.0) : mk(h.re - f.x, h.im - f.y);
  }
  const double sw = sqrt(a.w[n]);
  return mk(sw * d.re, sw * d.im);
}

__device__ __forceinline__ void split_bf16(float v, __nv_bfloat16& h, __nv_bfloat16& l) {
  h = __float2bfloat16_rn(v);
  l = __float2bfloat16_rn(v - __bfloat162float(h));
}

// 32 x 32 tiles (samples x columns), 32 x 8 threads; the transposed BF16X2
// gradient planes go through shared memory so that both the O reads
// (along k) and the plane writes (along n) are coalesced.
__global__ void __launch_bounds__(256) dense_data_kernel(dense_args a) {
  __shared__ float2 tile[32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int64_t n0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * 32;
  const bool transposed = a.format == VMC_DATA_BF16X2 && a.eloc == nullptr;
  for (int r = ty; r < 32; r += 8) {
    const int64_t n = n0 + r, k = k0 + tx;
    if (n >= a.N || k >= a.P) continue;
    const cpx<double> v = dense_value(a, n, k);
    if (transposed) {
      tile[r][tx] = make_float2((float)v.re, (float)v.im);
    } else if (a.format == VMC_DATA_C128) {
      reinterpret_cast<double2*>(a.out)[n * a.ld + k] = make_double2(v.re, v.im);
    } else if (a.format == VMC_DATA_C64) {
      reinterpret_cast<float2*>(a.out)[n * a.ld + k] = make_float2((float)v.re, (float)v.im);
    } else {  // BF16X2 row-major (N, 2P)
      __nv_bfloat16* hi = reinterpret_cast<__nv_bfloat16*>(a.out);
      __nv_bfloat16* lo = reinterpret_cast<__nv_bfloat16*>(a.out2);
      __nv_bfloat16 h, l;
      split_bf16((float)v.re, h, l);
      hi[n * a.ld + k] = h;
      lo[n * a.ld + k] = l;
      split_bf16((float)v.im, h, l);
      hi[n * a.ld + a.P + k] = h;
      lo[n * a.ld + a.P + k] = l;
    }
  }
  if (!transposed) return;
  __syncthreads();
  __nv_bfloat16* hi = reinterpret_cast<__nv_bfloat16*>(a.out);
  __nv_bfloat16* lo = reinterpret_cast<__nv_bfloat16*>(a.out2);
  for (int c = ty; c < 32; c += 8) {
    const int64_t k = k0 + c, n = n0 + tx;
    if (n >= a.N || k >= a.P) continue;
    const float2 v = tile[tx][c];
    __nv_bfloat16 h, l;
    split_bf16(v.x, h, l);
    hi[(size_t)k * a.ld + n] = h;
    lo[(size_t)k * a.ld + n] = l;
    split_bf16(v.y, h, l);
    hi[(size_t)(a.P + k) * a.ld + n] = h;
    lo[(size_t)(a.P + k) * a.ld + n] = l;
  }
}

int launch_dense(dense_args a, vmc_stream_t stream, const char* fn) {
  VMC_REQUIRE(a.format == VMC_DATA_C128 || a.format == VMC_DATA_C64 || a.format == VMC_DATA_BF16X2,
              VMC_ERR_INVALID_ARGUMENT, "%s: unknown format %d", fn, a.format);
  VMC_REQUIRE(a.out && (a.format != VMC_DATA_BF16X2 || a.out2), VMC_ERR_INVALID_ARGUMENT, "%s: null output", fn);
  VMC_REQUIRE(a.N > 0 && a.P > 0 && a.O && a.ldo >= a.P && a.w && a.okMean, VMC_ERR_INVALID_ARGUMENT,
              "%s: bad arguments", fn);
  const int64_t need = a.format == VMC_DATA_BF16X2 ? (a.eloc ? 2 * a.P : a.N) : a.P;
  VMC_REQUIRE(a.ld >= need, VMC_ERR_INVALID_ARGUMENT, "%s: leading dimension %lld < %lld", fn, (long long)a.ld,
              (long long)need);
  VMC_REQUIRE((a.N + 31) / 32 <= 65535, VMC_ERR_UNSUPPORTED, "%s: N=%lld too large", fn, (long long)a.N);
  dim3 grid((unsigned)((a.P + 31) / 32), (unsigned)((a.N + 31) / 32));
  dense_data_kernel<<<grid, 256, 0, as_stream(stream)>>>(a);
  return check_launch(fn);
}

}  // namespace vmc

using namespace vmc;

extern "C" size_t vmc_dense_grad_stats_workspace_bytes(int64_t num_configs, int64_t num_params) {
  (void)num_configs;
  return (size_t)kDenseChunks * ((size_t)num_params * 32 + 16) + 256;
}

extern "C" int vmc_dense_grad_stats(const double* gradients, int64_t ld_gradients, int64_t num_configs,
                                    int64_t num_params, const double* weights, const double* eloc,
                                    const double* eloc_mean, double* ok_mean, double* force, void* workspace,
                                    size_t workspace_bytes, vmc_stream_t stream) {
  VMC_REQUIRE(gradients && weights && eloc && eloc_mean && ok_mean && force && num_configs > 0 && num_params > 0 &&
                  ld_gradients >= num_params,
              VMC_ERR_INVALID_ARGUMENT, "vmc_dense_grad_stats: bad arguments");
  const size_t need = vmc_dense_grad_stats_workspace_bytes(num_configs, num_params);
  VMC_REQUIRE(workspace && workspace_bytes >= need, VMC_ERR_WORKSPACE,
              "vmc_dense_grad_stats: workspace of %zu bytes needed", need);
  double2* pm = reinterpret_cast<double2*>(workspace);
  double2* pc = pm + (size_t)kDenseChunks * num_params;
  double2* pe = pc + (size_t)kDenseChunks * num_params;
  cudaStream_t st = as_stream(stream);
  dim3 grid((unsigned)((num_params + kDenseCols - 1) / kDenseCols), kDenseChunks);
  dense_stats_partial_kernel<<<grid, kDenseCols, 0, st>>>(
      reinterpret_cast<const double2*>(gradients), ld_gradients, num_configs, num_params, weights,
      reinterpret_cast<const double2*>(eloc), reinterpret_cast<const double2*>(eloc_mean), pm, pc, pe);
  int rc = check_launch("vmc_dense_grad_stats(partial)");
  if (rc) return rc;
  dense_stats_final_kernel<<<(unsigned)((num_params + 255) / 256), 256, 0, st>>>(
      pm, pc, pe, num_params, reinterpret_cast<double2*>(ok_mean), reinterpret_cast<double2*>(force));
  return check_launch("vmc_dense_grad_stats(final)");
}

extern "C" int vmc_dense_centered_gradients(const double* gradients, int64_t ld_gradients, int64_t num_configs,
                                            int64_t num_params, const double* weights, const double* ok_mean,
                                            int32_t format, void* out, void* out_lo, int64_t ld_out,
                                            vmc_stream_t stream) {
  dense_args a;
  a.O = reinterpret_cast<const double2*>(gradients);
  a.ldo = ld_gradients;
  a.N = num_configs;
  a.P = num_params;
  a.w = weights;
  a.okMean = reinterpret_cast<const double2*>(ok_mean);
  a.eloc = nullptr;
  a.elocMean = nullptr;
  a.xfac = make_double2(0, 0);
  a.realPart = 0;
  a.force = nullptr;
  a.format = format;
  a.ld = ld_out;
  a.out = out;
  a.out2 = out_lo;
  return launch_dense(a, stream, "vmc_dense_centered_gradients");
}

extern "C" int vmc_dense_snr_data(const double* gradients, int64_t ld_gradients, int64_t num_configs,
                                  int64_t num_params, const double* weights, const double* ok_mean, const double* eloc,
                                  const double* eloc_mean, double neg_rhs_re, double neg_rhs_im, const double* force,
                                  int32_t real_part, int32_t format, void* out, void* out_lo, int64_t ld_out,
                                  vmc_stream_t stream) {
  VMC_REQUIRE(eloc && eloc_mean && force, VMC_ERR_INVALID_ARGUMENT, "vmc_dense_snr_data: null argument");
  dense_args a;
  a.O = reinterpret_cast<const double2*>(gradients);
  a.ldo = ld_gradients;
  a.N = num_configs;
  a.P = num_params;
  a.w = weights;
  a.okMean = reinterpret_cast<const double2*>(ok_mean);
  a.eloc = reinterpret_cast<const double2*>(eloc);
  a.elocMean = reinterpret_cast<const double2*>(eloc_mean);
  a.xfac = make_double2(neg_rhs_re, neg_rhs_im);
  a.realPart = real_part ? 1 : 0;
  a.force = reinterpret_cast<const double2*>(force);
  a.format = format;
  a.ld = ld_out;
  a.out = out;
  a.out2 = out_lo;
  return launch_dense(a, stream, "vmc_dense_snr_data");
}
