// Shared device helpers for the VMC hot-path kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/vmc_gb300.h"

namespace vmc {

// ---------------------------------------------------------------------------
// error reporting (host side)
// ---------------------------------------------------------------------------
void set_error(const char* fmt, ...);
int check_launch(const char* what);
// Validate a branch-free operator descriptor (host side).
int check_op(const char* fn, const vmc_bf_operator* op, int L);
// Allow `bytes` of dynamic shared memory for kernel `fn` on the current
// device (needed above 48 KB; the attribute is per device, so it is set on
// every call).  Returns VMC_OK or VMC_ERR_CUDA with the kernel and the size
// in the error string.
int allow_smem(const void* fn, size_t bytes, const char* what);

#define VMC_ALLOW_SMEM(fn, bytes, what)                                              \
  do {                                                                               \
    int vmc_rc_ = ::vmc::allow_smem((const void*)(fn), (size_t)(bytes), (what));    \
    if (vmc_rc_) return vmc_rc_;                                                     \
  } while (0)

#define VMC_REQUIRE(cond, code, ...)      \
  do {                                     \
    if (!(cond)) {                         \
      ::vmc::set_error(__VA_ARGS__);       \
      return (code);                       \
    }                                      \
  } while (0)

// ---------------------------------------------------------------------------
// complex arithmetic on a plain (re, im) pair; T = float or double
// ---------------------------------------------------------------------------
template <typename T>
struct cpx {
  T re, im;
};

template <typename T>
__host__ __device__ __forceinline__ cpx<T> mk(T r, T i) {
  cpx<T> z;
  z.re = r;
  z.im = i;
  return z;
}
template <typename T>
__device__ __forceinline__ cpx<T> operator+(cpx<T> a, cpx<T> b) { return mk(a.re + b.re, a.im + b.im); }
template <typename T>
__device__ __forceinline__ cpx<T> operator-(cpx<T> a, cpx<T> b) { return mk(a.re - b.re, a.im - b.im); }
template <typename T>
__device__ __forceinline__ cpx<T> operator*(cpx<T> a, cpx<T> b) {
  return mk(fma(a.re, b.re, -a.im * b.im), fma(a.re, b.im, a.im * b.re));
}
template <typename T>
__device__ __forceinline__ cpx<T> operator*(T s, cpx<T> a) { return mk(s * a.re, s * a.im); }
template <typename T>
__device__ __forceinline__ cpx<T> conjg(cpx<T> a) { return mk(a.re, -a.im); }
template <typename T>
__device__ __forceinline__ T abs2(cpx<T> a) { return a.re * a.re + a.im * a.im; }

__device__ __forceinline__ float fexp(float x) { return expf(x); }
__device__ __forceinline__ double fexp(double x) { return exp(x); }
__device__ __forceinline__ float fexpm1(float x) { return expm1f(x); }
__device__ __forceinline__ double fexpm1(double x) { return expm1(x); }
__device__ __forceinline__ float flog1p(float x) { return log1pf(x); }
__device__ __forceinline__ double flog1p(double x) { return log1p(x); }
__device__ __forceinline__ float flog(float x) { return logf(x); }
__device__ __forceinline__ double flog(double x) { return log(x); }
__device__ __forceinline__ float fatan2(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ double fatan2(double y, double x) { return atan2(y, x); }
__device__ __forceinline__ void fsincos(float x, float* s, float* c) { sincosf(x, s, c); }
__device__ __forceinline__ void fsincos(double x, double* s, double* c) { sincos(x, s, c); }
__device__ __forceinline__ float fhypot(float x, float y) { return hypotf(x, y); }
__device__ __forceinline__ double fhypot(double x, double y) { return hypot(x, y); }

template <typename T>
__device__ __forceinline__ cpx<T> cexp_(cpx<T> z) {
  T e = fexp(z.re), s, c;
  fsincos(z.im, &s, &c);
  return mk(e * c, e * s);
}

// log(1 + w) for complex w: log|1+w| + i arg(1+w); the modulus is formed
// with log1p on |w|^2 + 2 Re w so that small w keeps full precision.
template <typename T>
__device__ __forceinline__ cpx<T> clog1p_(cpx<T> w) {
  T a = w.re, b = w.im;
  T m = a * (a + T(2)) + b * b;  // |1+w|^2 - 1
  return mk(T(0.5) * flog1p(m), fatan2(b, T(1) + a));
}

// Complex log(cosh(x)) in the form used by jVMC's activation
// (activation_functions.py:19-22): flip x to Re x >= 0, then
// x + log1p(exp(-2x)) - log 2.
template <typename T>
__device__ __forceinline__ cpx<T> log_cosh(cpx<T> x) {
  if (signbit(x.re)) x = mk(-x.re, -x.im);
  cpx<T> e = cexp_(mk(T(-2) * x.re, T(-2) * x.im));
  cpx<T> l = clog1p_(e);
  const T ln2 = T(0.69314718055994530941723212145818);
  return mk(x.re + l.re - ln2, x.im + l.im);
}

// tanh of a complex argument via exp(-2|Re x|) (no overflow for large |Re|).
template <typename T>
__device__ __forceinline__ cpx<T> ctanh_(cpx<T> x) {
  bool neg = signbit(x.re);
  T a = neg ? -x.re : x.re;
  // tanh(a + ib) = (1 - e^2 + 2 i e sin 2b) / (1 + e^2 + 2 e cos 2b), e = exp(-2a);
  // 1 - e^2 = -em (2 + em) with em = expm1(-2a) keeps full precision for small a
  T em = fexpm1(T(-2) * a);
  T e = T(1) + em;
  T s2, c2;
  fsincos(T(2) * x.im, &s2, &c2);
  T den = T(1) + e * e + T(2) * e * c2;
  T re = -em * (T(2) + em) / den;
  T im = T(2) * e * s2 / den;
  return mk(neg ? -re : re, im);
}

// ---------------------------------------------------------------------------
// Products of many complex factors: mantissa/exponent pair to stay inside
// the range of T.  The exponent is the power of two removed from the
// mantissa (value = mant * 2^ex).
// ---------------------------------------------------------------------------
template <typename T>
struct scaled_cpx {
  cpx<T> m;
  int ex;
};

__device__ __forceinline__ int exponent_of(double x) {
  long long b = __double_as_longlong(x);
  return (int)((b >> 52) & 0x7ff) - 1023;
}
__device__ __forceinline__ int exponent_of(float x) {
  int b = __float_as_int(x);
  return ((b >> 23) & 0xff) - 127;
}

template <typename T>
__device__ __forceinline__ void renorm(scaled_cpx<T>& z) {
  T mx = fmax(fabs(z.m.re), fabs(z.m.im));
  if (mx == T(0) || !isfinite(mx)) return;
  int e = exponent_of(mx);
  z.m.re = ldexp(z.m.re, -e);
  z.m.im = ldexp(z.m.im, -e);
  z.ex += e;
}

template <typename T>
__device__ __forceinline__ scaled_cpx<T> mul(scaled_cpx<T> a, scaled_cpx<T> b) {
  scaled_cpx<T> r;
  r.m = a.m * b.m;
  r.ex = a.ex + b.ex;
  renorm(r);
  return r;
}

template <typename T>
__device__ __forceinline__ cpx<T> to_cpx(scaled_cpx<T> z) {
  int e = z.ex;
  if (e > 4000) e = 4000;
  if (e < -4000) e = -4000;
  return mk(ldexp(z.m.re, e), ldexp(z.m.im, e));
}

template <typename T>
__device__ __forceinline__ cpx<T> shfl_xor(cpx<T> v, int m) {
  return mk(__shfl_xor_sync(0xffffffffu, v.re, m), __shfl_xor_sync(0xffffffffu, v.im, m));
}

template <typename T>
__device__ __forceinline__ scaled_cpx<T> warp_prod(scaled_cpx<T> v) {
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) {
    scaled_cpx<T> o;
    o.m = shfl_xor(v.m, m);
    o.ex = __shfl_xor_sync(0xffffffffu, v.ex, m);
    v = mul(v, o);
  }
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
  return v;
}

template <typename T>
__device__ __forceinline__ cpx<T> warp_sum(cpx<T> v) {
  return mk(warp_sum(v.re), warp_sum(v.im));
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), written from the
// published round function.
// ---------------------------------------------------------------------------
struct u32x4 {
  uint32_t x, y, z, w;
};

__host__ __device__ __forceinline__ u32x4 philox4x32_10(u32x4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)M0 * c.x;
    uint64_t p1 = (uint64_t)M1 * c.z;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    u32x4 n;
    n.x = hi1 ^ c.y ^ k0;
    n.y = lo1;
    n.z = hi0 ^ c.w ^ k1;
    n.w = lo0;
    c = n;
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// One Metropolis draw: flip site in [0, L) and the acceptance uniform,
// as a 53-bit double ((r1>>5) 2^26 + (r2>>6)) / 2^53 (FP64 kernels) or a
// 24-bit float (r1>>8) / 2^24 (FP32 kernels).
struct mc_draw {
  int site;
  uint32_t r1, r2;
  __device__ __forceinline__ double u64() const {
    return ((double)(r1 >> 5) * 67108864.0 + (double)(r2 >> 6)) * (1.0 / 9007199254740992.0);
  }
  __device__ __forceinline__ float u32() const { return (float)(r1 >> 8) * (1.0f / 16777216.0f); }
};

__device__ __forceinline__ mc_draw metropolis_draw(uint64_t seed, uint32_t call, uint32_t step, uint32_t chain,
                                                   int L) {
  u32x4 c;
  c.x = step;
  c.y = chain;
  c.z = call;
  c.w = 0x5EEDu;
  u32x4 r = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  mc_draw d;
  d.site = (int)(((uint64_t)r.x * (uint64_t)L) >> 32);
  d.r1 = r.y;
  d.r2 = r.z;
  return d;
}

inline cudaStream_t as_stream(vmc_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

}  // namespace vmc
