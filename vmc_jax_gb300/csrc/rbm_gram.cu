// Producers of the centred, weighted log-derivative data that the S/F build
// and the SNR transform contract (stats.py:197-205, 255-292 via
// tdvp.py:134-181), for a CpxRBM, in three storage formats:
//   VMC_DATA_C128   (N, P) complex128
//   VMC_DATA_C64    (N, P) complex64
//   VMC_DATA_BF16X2 bf16 hi/lo planes of the real representation
//                   [Re X | Im X]: transposed (2P, N) for the Gram operand
//                   (sample index contiguous), row-major (N, 2P) for the
//                   SNR operand.
// X_nk = sqrt(w_n) (O_nk - mean_k)            (gradients)
// H_nk = sqrt(w_n) (-x dE_n conj(O_nk - mean_k) - f_k)   (SNR data; dE_n = E_n - Ebar)
#include <cuda_bf16.h>

#include <algorithm>

#include "vmc_common.cuh"

namespace vmc {


// tanh(theta) of the tile's kTileN (<= 32) samples into shared memory (as T).
// Thread -> hidden unit j; every W_ij is loaded once per pass of S samples
// and applied to S accumulators in registers, the signs taken from a per-site
// bit mask of the tile's configurations (bit r = s_i of sample r).  Each
// theta is summed in the order b_j, then i = 0 .. L-1, as in rbm_logpsi.
template <typename T, int S>
__device__ void tile_tanh(const int32_t* __restrict__ configs, int64_t n0, int64_t N, int L, int M,
                          const cpx<T>* __restrict__ W, const cpx<T>* __restrict__ b, cpx<T>* tt, int8_t* sg,
                          uint32_t* sbits, int kTileN) {
  const int tid = threadIdx.x;
  for (int idx = tid; idx < kTileN * L; idx += blockDim.x) {
    const int r = idx / L, i = idx - r * L;
    const int64_t n = n0 + r;
    sg[r * (L + 1) + i] = n < N ? (int8_t)(configs[n * L + i] != 0) : (int8_t)0;
  }
  __syncthreads();
  for (int i = tid; i < L; i += blockDim.x) {
    uint32_t m = 0;
    for (int r = 0; r < kTileN; ++r) m |= (uint32_t)sg[r * (L + 1) + i] << r;
    sbits[i] = m;
  }
  __syncthreads();
  for (int s0 = 0; s0 < kTileN; s0 += S) {
    for (int j = tid; j < M; j += blockDim.x) {
      const cpx<T> bj = b ? b[j] : mk(T(0), T(0));
      T ar[S], ai[S];
#pragma unroll
      for (int s = 0; s < S; ++s) {
        ar[s] = bj.re;
        ai[s] = bj.im;
      }
#pragma unroll 4
      for (int i = 0; i < L; ++i) {
        const cpx<T> x = W[(size_t)i * M + j];
        const uint32_t m = sbits[i] >> s0;
#pragma unroll
        for (int s = 0; s < S; ++s) {
          const bool up = (m >> s) & 1u;
          ar[s] += up ? x.re : -x.re;
          ai[s] += up ? x.im : -x.im;
        }
      }
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const int r = s0 + s;
        if (r < kTileN) tt[(size_t)r * (M + 1) + j] = n0 + r < N ? ctanh_(mk(ar[s], ai[s])) : mk(T(0), T(0));
      }
    }
  }
  __syncthreads();
}

struct data_args {
  int64_t N;
  int L, M;
  bool hasBias;
  const double* w;         // (N) weights
  const double2* okMean;   // (P) c128
  const double2* eloc;     // (N) c128 or null (gradients)
  const double2* elocMean; // (1) c128
  double2 xfac;            // -x (rhs prefactor, negated)
  const double2* force;    // (P) f_k = -x * covar(O,E)_k (SNR data) or null
  int format;
  int tileN;  // samples per block
  int colChunk;  // columns per block (grid y)
  int64_t ld; // leading dimension of the output (elements)
  void* out;
  void* out2;              // lo plane for BF16X2
};

// Column k of the (bias | kernel) layout as (in bias, row i, hidden unit j),
// advanced by a fixed stride without integer division per element.
struct col_pos {
  bool bias;
  int i, j;
  __device__ __forceinline__ void set(int k, int M, bool hasBias) {
    const int P0 = hasBias ? M : 0;
    bias = k < P0;
    if (bias) {
      i = 0;
      j = k;
    } else {
      i = (k - P0) / M;
      j = (k - P0) - i * M;
    }
  }
  __device__ __forceinline__ void advance(int step, int M) {
    j += step;
    if (bias && j >= M) {
      bias = false;
      j -= M;
      i = 0;
    }
    while (j >= M) {
      j -= M;
      ++i;
    }
  }
};

// value of column k (position c) for tile row r
template <typename T>
__device__ __forceinline__ cpx<double> data_value(const data_args& a, const cpx<T>* tt, const int8_t* sg, int r,
                                                  int64_t n, int k, const col_pos& c, double sw) {
  cpx<T> o = tt[(size_t)r * (a.M + 1) + c.j];
  if (!c.bias && !sg[r * (a.L + 1) + c.i]) o = mk(-o.re, -o.im);
  const double2 mu = a.okMean[k];
  cpx<double> d = mk((double)o.re - mu.x, (double)o.im - mu.y);
  if (a.eloc) {
    const double2 e = a.eloc[n], em = *a.elocMean;
    cpx<double> de = mk(e.x - em.x, e.y - em.y);
    cpx<double> h = mk(a.xfac.x, a.xfac.y) * (de * conjg(d));
    const double2 f = a.force[k];
    d = mk(h.re - f.x, h.im - f.y);
  }
  return mk(sw * d.re, sw * d.im);
}

// The same value in FP32 for the BF16 hi/lo and complex64 formats, from
// per-block staged column means / forces and per-sample sqrt(w) and
// (-x)(E_n - Ebar): their precision is far below FP32's, and GB300's FP64
// rate would otherwise bound this HBM-streaming kernel.
template <typename T>
__device__ __forceinline__ cpx<float> data_value_f(const data_args& a, const cpx<T>* tt, const int8_t* sg, int r,
                                                  const col_pos& c, float2 mu, float2 f, float sw, float2 xde) {
  cpx<T> o = tt[(size_t)r * (a.M + 1) + c.j];
  if (!c.bias && !sg[r * (a.L + 1) + c.i]) o = mk(-o.re, -o.im);
  cpx<float> d = mk((float)o.re - mu.x, (float)o.im - mu.y);
  if (a.eloc) {
    const cpx<float> h = mk(xde.x, xde.y) * conjg(d);
    d = mk(h.re - f.x, h.im - f.y);
  }
  return mk(sw * d.re, sw * d.im);
}

__device__ __forceinline__ void store_split(__nv_bfloat16* hi, __nv_bfloat16* lo, size_t idx, float v) {
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  hi[idx] = h;
  lo[idx] = __float2bfloat16_rn(v - __bfloat162float(h));
}

// two adjacent elements (idx even) with one 4-byte store per plane; the same
// values as two store_split calls
__device__ __forceinline__ void store_split2(__nv_bfloat16* hi, __nv_bfloat16* lo, size_t idx, float v0, float v1) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(v0, v1);
  const float2 hf = __bfloat1622float2(h);
  *reinterpret_cast<__nv_bfloat162*>(hi + idx) = h;
  *reinterpret_cast<__nv_bfloat162*>(lo + idx) = __floats2bfloat162_rn(v0 - hf.x, v1 - hf.y);
}

template <typename T>
__global__ void __launch_bounds__(256) rbm_data_kernel(const int32_t* __restrict__ configs, const cpx<T>* __restrict__ W,
                                                       const cpx<T>* __restrict__ b, data_args a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int kTileN = a.tileN;
  cpx<T>* tt = reinterpret_cast<cpx<T>*>(smem);
  // rows padded by one element: lanes of the transposed store loop read
  // different rows, which would otherwise fall into the same bank
  int8_t* sg = reinterpret_cast<int8_t*>(smem + (size_t)kTileN * (a.M + 1) * sizeof(cpx<T>));
  const size_t stOff = ((size_t)kTileN * (a.M + 1) * sizeof(cpx<T>) + (size_t)kTileN * (a.L + 1) + 15) & ~(size_t)15;
  float2* cmean = reinterpret_cast<float2*>(smem + stOff);
  float2* cforce = cmean + a.colChunk;
  float2* sxde = cforce + a.colChunk;
  float* ssw = reinterpret_cast<float*>(sxde + kTileN);
  uint32_t* sbits = reinterpret_cast<uint32_t*>(ssw + kTileN);
  const int64_t n0 = (int64_t)blockIdx.x * kTileN;
  const int P = a.M * a.L + (a.hasBias ? a.M : 0);
  const int k0 = blockIdx.y * a.colChunk, k1 = min(P, k0 + a.colChunk);
  const int tid = threadIdx.x;
  const bool lowp = a.format != VMC_DATA_C128;
  if (lowp) {
    for (int k = k0 + tid; k < k1; k += blockDim.x) {
      const double2 mu = a.okMean[k];
      cmean[k - k0] = make_float2((float)mu.x, (float)mu.y);
      if (a.eloc) {
        const double2 f = a.force[k];
        cforce[k - k0] = make_float2((float)f.x, (float)f.y);
      }
    }
    for (int r = tid; r < kTileN; r += blockDim.x) {
      const int64_t n = n0 + r;
      ssw[r] = n < a.N ? (float)sqrt(a.w[n]) : 0.f;
      if (a.eloc && n < a.N) {
        const double2 e = a.eloc[n], em = *a.elocMean;
        const cpx<double> xde = mk(a.xfac.x, a.xfac.y) * mk(e.x - em.x, e.y - em.y);
        sxde[r] = make_float2((float)xde.re, (float)xde.im);
      }
    }
  }
  // ends with __syncthreads; S accumulators per pass: 16 FP32 or 8 FP64 complex
  tile_tanh<T, sizeof(T) == 4 ? 16 : 8>(configs, n0, a.N, a.L, a.M, W, b, tt, sg, sbits, kTileN);
  const float2 zero2 = make_float2(0.f, 0.f);
  // BF16 planes whose leading dimension and bases allow 4-byte stores of
  // element pairs
  const bool pairs = a.format == VMC_DATA_BF16X2 && (a.ld & 1) == 0 &&
                     ((reinterpret_cast<uintptr_t>(a.out) | reinterpret_cast<uintptr_t>(a.out2)) & 3) == 0;
  if (a.format == VMC_DATA_BF16X2 && a.eloc == nullptr) {
    // transposed planes (2P, N)
    __nv_bfloat16* hi = reinterpret_cast<__nv_bfloat16*>(a.out);
    __nv_bfloat16* lo = reinterpret_cast<__nv_bfloat16*>(a.out2);
    if (pairs) {
      // thread -> (sample pair r, r + 1; column group): samples are adjacent
      // in a plane row, so one store carries both
      const int half = kTileN / 2;
      const int r = 2 * (tid % half);
      const int cg = tid / half, ncg = blockDim.x / half;
      const int64_t n = n0 + r;
      if (n < a.N) {
        const bool two = n + 1 < a.N;
        const float sw0 = ssw[r], sw1 = ssw[r + 1];
        col_pos c;
        c.set(k0 + cg, a.M, a.hasBias);
        for (int k = k0 + cg; k < k1; k += ncg, c.advance(ncg, a.M)) {
          const float2 mu = cmean[k - k0];
          const cpx<float> v0 = data_value_f<T>(a, tt, sg, r, c, mu, zero2, sw0, zero2);
          if (two) {
            const cpx<float> v1 = data_value_f<T>(a, tt, sg, r + 1, c, mu, zero2, sw1, zero2);
            store_split2(hi, lo, (size_t)k * a.ld + n, v0.re, v1.re);
            store_split2(hi, lo, (size_t)(P + k) * a.ld + n, v0.im, v1.im);
          } else {
            store_split(hi, lo, (size_t)k * a.ld + n, v0.re);
            store_split(hi, lo, (size_t)(P + k) * a.ld + n, v0.im);
          }
        }
      }
      return;
    }
    // thread -> (sample lane r, column group)
    const int r = tid % kTileN;
    const int cg = tid / kTileN, ncg = blockDim.x / kTileN;
    const int64_t n = n0 + r;
    if (n < a.N) {
      const float sw = ssw[r];
      col_pos c;
      c.set(k0 + cg, a.M, a.hasBias);
      for (int k = k0 + cg; k < k1; k += ncg, c.advance(ncg, a.M)) {
        const cpx<float> v = data_value_f<T>(a, tt, sg, r, c, cmean[k - k0], zero2, sw, zero2);
        store_split(hi, lo, (size_t)k * a.ld + n, v.re);
        store_split(hi, lo, (size_t)(P + k) * a.ld + n, v.im);
      }
    }
    return;
  }
  // row-major formats: thread -> column, loop over the tile's samples
  for (int r = 0; r < kTileN; ++r) {
    const int64_t n = n0 + r;
    if (n >= a.N) break;
    col_pos c;
    c.set(k0 + tid, a.M, a.hasBias);
    if (!lowp) {
      const double sw = sqrt(a.w[n]);
      for (int k = k0 + tid; k < k1; k += blockDim.x, c.advance(blockDim.x, a.M)) {
        const cpx<double> v = data_value<T>(a, tt, sg, r, n, k, c, sw);
        reinterpret_cast<double2*>(a.out)[n * a.ld + k] = make_double2(v.re, v.im);
      }
      continue;
    }
    const float sw = ssw[r];
    const float2 xde = a.eloc ? sxde[r] : zero2;
    if (pairs && (P & 1) == 0) {
      // BF16X2 row-major (N, 2P): thread -> column pair k, k + 1 (k0 and P
      // even, so both halves of the row start on an even element)
      __nv_bfloat16* hi = reinterpret_cast<__nv_bfloat16*>(a.out);
      __nv_bfloat16* lo = reinterpret_cast<__nv_bfloat16*>(a.out2);
      c.set(k0 + 2 * tid, a.M, a.hasBias);
      for (int k = k0 + 2 * tid; k < k1; k += 2 * blockDim.x, c.advance(2 * blockDim.x, a.M)) {
        const cpx<float> v0 =
            data_value_f<T>(a, tt, sg, r, c, cmean[k - k0], a.eloc ? cforce[k - k0] : zero2, sw, xde);
        if (k + 1 < k1) {
          col_pos c1 = c;
          c1.advance(1, a.M);
          const cpx<float> v1 = data_value_f<T>(a, tt, sg, r, c1, cmean[k + 1 - k0],
                                                a.eloc ? cforce[k + 1 - k0] : zero2, sw, xde);
          store_split2(hi, lo, n * a.ld + k, v0.re, v1.re);
          store_split2(hi, lo, n * a.ld + P + k, v0.im, v1.im);
        } else {
          store_split(hi, lo, n * a.ld + k, v0.re);
          store_split(hi, lo, n * a.ld + P + k, v0.im);
        }
      }
      continue;
    }
    for (int k = k0 + tid; k < k1; k += blockDim.x, c.advance(blockDim.x, a.M)) {
      const cpx<float> v =
          data_value_f<T>(a, tt, sg, r, c, cmean[k - k0], a.eloc ? cforce[k - k0] : zero2, sw, xde);
      if (a.format == VMC_DATA_C64) {
        reinterpret_cast<float2*>(a.out)[n * a.ld + k] = make_float2(v.re, v.im);
      } else {  // BF16X2 row-major (N, 2P)
        __nv_bfloat16* hi = reinterpret_cast<__nv_bfloat16*>(a.out);
        __nv_bfloat16* lo = reinterpret_cast<__nv_bfloat16*>(a.out2);
        store_split(hi, lo, n * a.ld + k, v.re);
        store_split(hi, lo, n * a.ld + P + k, v.im);
      }
    }
  }
}

}  // namespace vmc

using namespace vmc;

static int launch_data(int32_t precision, const int32_t* configs, const void* kernel, const void* bias, data_args a,
                       vmc_stream_t stream, const char* fn) {
  VMC_REQUIRE(precision == VMC_F64 || precision == VMC_F32, VMC_ERR_UNSUPPORTED, "%s: precision %d", fn, precision);
  VMC_REQUIRE(a.format == VMC_DATA_C128 || a.format == VMC_DATA_C64 || a.format == VMC_DATA_BF16X2,
              VMC_ERR_INVALID_ARGUMENT, "%s: unknown format %d", fn, a.format);
  VMC_REQUIRE(a.out && (a.format != VMC_DATA_BF16X2 || a.out2), VMC_ERR_INVALID_ARGUMENT, "%s: null output", fn);
  VMC_REQUIRE(a.N > 0 && a.L > 0 && a.M > 0 && configs && kernel && a.w && a.okMean, VMC_ERR_INVALID_ARGUMENT,
              "%s: bad arguments", fn);
  {
    const int64_t P = (int64_t)a.M * a.L + (a.hasBias ? a.M : 0);
    const int64_t need = a.format == VMC_DATA_BF16X2 ? (a.eloc ? 2 * P : a.N) : P;
    VMC_REQUIRE(a.ld >= need, VMC_ERR_INVALID_ARGUMENT, "%s: leading dimension %lld < %lld", fn, (long long)a.ld,
                (long long)need);
  }
  const size_t el = precision == VMC_F64 ? 16 : 8;
  // at most 32 samples per tile (one bit each in the per-site sign masks);
  // fewer when the tile's tanh values would not leave room for two blocks
  int kTileN = 32;
  while (kTileN > 8 && (size_t)kTileN * ((a.M + 1) * el + a.L + 1) > 96 * 1024) kTileN /= 2;
  a.tileN = kTileN;
  a.colChunk = 2048;
  const size_t tileBytes = ((size_t)kTileN * (a.M + 1) * el + (size_t)kTileN * (a.L + 1) + 15) & ~(size_t)15;
  const size_t smem = tileBytes + (size_t)a.colChunk * 16 + (size_t)kTileN * 12 + (size_t)a.L * 4;
  VMC_REQUIRE(smem <= 227 * 1024, VMC_ERR_UNSUPPORTED, "%s: M=%d, L=%d too large for one tile", fn, a.M, a.L);
  // columns split over grid y so that enough blocks are resident; each block
  // recomputes tanh(theta) of its samples (L M per sample, small next to the
  // column loop)
  const int64_t P = (int64_t)a.M * a.L + (a.hasBias ? a.M : 0);
  const dim3 grid((unsigned)((a.N + kTileN - 1) / kTileN), (unsigned)((P + a.colChunk - 1) / a.colChunk));
  VMC_REQUIRE(grid.y <= 65535, VMC_ERR_UNSUPPORTED, "%s: %lld columns", fn, (long long)P);
  cudaStream_t st = as_stream(stream);
  if (precision == VMC_F64) {
    VMC_ALLOW_SMEM(rbm_data_kernel<double>, smem, fn);
    rbm_data_kernel<double><<<grid, 256, smem, st>>>(configs, reinterpret_cast<const cpx<double>*>(kernel),
                                                    reinterpret_cast<const cpx<double>*>(bias), a);
  } else {
    VMC_ALLOW_SMEM(rbm_data_kernel<float>, smem, fn);
    rbm_data_kernel<float><<<grid, 256, smem, st>>>(configs, reinterpret_cast<const cpx<float>*>(kernel),
                                                   reinterpret_cast<const cpx<float>*>(bias), a);
  }
  return check_launch(fn);
}

extern "C" int vmc_rbm_centered_gradients(int32_t precision, const int32_t* configs, int64_t num_configs,
                                          int32_t num_sites, int32_t num_hidden, const void* kernel, const void* bias,
                                          const double* weights, const double* ok_mean, int32_t format, void* out,
                                          void* out_lo, int64_t ld_out, vmc_stream_t stream) {
  data_args a;
  a.N = num_configs;
  a.L = num_sites;
  a.M = num_hidden;
  a.hasBias = bias != nullptr;
  a.w = weights;
  a.okMean = reinterpret_cast<const double2*>(ok_mean);
  a.eloc = nullptr;
  a.elocMean = nullptr;
  a.xfac = make_double2(0, 0);
  a.force = nullptr;
  a.format = format;
  a.out = out;
  a.out2 = out_lo;
  a.ld = ld_out;
  return launch_data(precision, configs, kernel, bias, a, stream, "vmc_rbm_centered_gradients");
}

extern "C" int vmc_rbm_snr_data(int32_t precision, const int32_t* configs, int64_t num_configs, int32_t num_sites,
                                int32_t num_hidden, const void* kernel, const void* bias, const double* weights,
                                const double* ok_mean, const double* eloc, const double* eloc_mean,
                                double neg_rhs_re, double neg_rhs_im, const double* force, int32_t format, void* out,
                                void* out_lo, int64_t ld_out, vmc_stream_t stream) {
  VMC_REQUIRE(eloc && eloc_mean && force, VMC_ERR_INVALID_ARGUMENT, "vmc_rbm_snr_data: null argument");
  data_args a;
  a.N = num_configs;
  a.L = num_sites;
  a.M = num_hidden;
  a.hasBias = bias != nullptr;
  a.w = weights;
  a.okMean = reinterpret_cast<const double2*>(ok_mean);
  a.eloc = reinterpret_cast<const double2*>(eloc);
  a.elocMean = reinterpret_cast<const double2*>(eloc_mean);
  a.xfac = make_double2(neg_rhs_re, neg_rhs_im);
  a.force = reinterpret_cast<const double2*>(force);
  a.format = format;
  a.out = out;
  a.out2 = out_lo;
  a.ld = ld_out;
  return launch_data(precision, configs, kernel, bias, a, stream, "vmc_rbm_snr_data");
}
