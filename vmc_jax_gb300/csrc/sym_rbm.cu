// Symmetrised complex RBM (nets/sym_wrapper.py:22-64 over nets/rbm.py:17-38):
//   log psi(s) = avg_tau log psi_RBM(tau(s)),
// avg = log sum_tau f_tau exp(.) (avgFun_Coefficients_Exp, sym_wrapper.py:7-9)
// or the mean (avgFun_Coefficients_Log, 12-13).  One block per configuration
// (or per chain); log psi and gradients take one warp per orbit element at a
// time, the per-proposal / per-string ratio products G threads per orbit
// element (a power of two <= 32) with a butterfly over the group.
//
// The orbit arrives as codes (S, L): code = 2 src + flip, tau(s)_i =
// s_src xor flip, and its inverse (S, L): inv[tau][j] = the position i with
// src(tau, i) = j, so that flipping site j of s flips position inv[tau][j]
// of tau(s).  Codes outside [0, 2L) and inverse entries outside [0, L) are
// never dereferenced: the affected result becomes NaN.
#include <algorithm>
#include <math.h>

#include "bf_apply.cuh"
#include "rbm.cuh"
#include "reduce.cuh"
#include "vmc_common.cuh"

namespace vmc {

constexpr int kSymThreads = 256;
constexpr int kSymWarps = kSymThreads / 32;
constexpr int kMaxSym = 4096;
constexpr int kSymChunk = kSymThreads;  // operator strings applied per pass of the fused estimator
constexpr size_t kSmemLimit = 227 * 1024;

struct sym_params {
  int S, avg;
  const int32_t* code;    // (S, L)
  const int32_t* inv;     // (S, L)
  const double2* factor;  // (S)
};

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, m));
  return v;
}

template <typename T>
__device__ __forceinline__ cpx<T> cdiv(cpx<T> a, cpx<T> b) {
  const T d = T(1) / abs2(b);
  return mk((a.re * b.re + a.im * b.im) * d, (a.im * b.re - a.re * b.im) * d);
}

// tau(s) (local states 0/1) into a warp's buffer; false if a code is
// malformed (that position is then written as 0).
__device__ __forceinline__ bool sym_transform(const int32_t* __restrict__ code, const int8_t* cfg, int L, int8_t* out,
                                              int lane) {
  bool ok = true;
  for (int i = lane; i < L; i += 32) {
    const int c = code[i];
    const int src = c >> 1;
    if ((unsigned)src < (unsigned)L) {
      out[i] = (int8_t)(cfg[src] ^ (c & 1));
    } else {
      out[i] = 0;
      ok = false;
    }
  }
  ok = __all_sync(0xffffffffu, ok);
  __syncwarp();
  return ok;
}

template <typename T>
__device__ __forceinline__ cpx<T> theta_of(const rbm_params<T>& p, const int8_t* c, int j) {
  cpx<T> th = p.b ? p.b[j] : mk(T(0), T(0));
  const cpx<T>* w = p.W + j;
  for (int i = 0; i < p.L; ++i) {
    const cpx<T> x = w[(size_t)i * p.M];
    if (c[i]) {
      th.re += x.re;
      th.im += x.im;
    } else {
      th.re -= x.re;
      th.im -= x.im;
    }
  }
  return th;
}

// The average over the orbit of the per-element log psi `lp` (executed by
// one warp; every lane returns the result).  Exp: jax's logsumexp with
// b = factor for complex input: elements with factor 0 are dropped, the
// largest real part m is taken out, result = m + principal log(sum).
// U: the arithmetic (double, or float inside the FP32 sampler).
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, m));
  return v;
}

template <typename U>
__device__ __forceinline__ cpx<U> sym_average(const sym_params& sp, const cpx<U>* lp, int lane) {
  if (sp.avg == VMC_SYM_LOG) {
    cpx<U> s = mk(U(0), U(0));
    for (int t = lane; t < sp.S; t += 32) s = s + lp[t];
    s = warp_sum(s);
    return mk(s.re / U(sp.S), s.im / U(sp.S));
  }
  U mx = -INFINITY;
  for (int t = lane; t < sp.S; t += 32) {
    const double2 f = sp.factor[t];
    if (f.x != 0.0 || f.y != 0.0) mx = fmax(mx, lp[t].re);
  }
  mx = warp_max(mx);
  if (!isfinite(mx)) mx = U(0);
  cpx<U> z = mk(U(0), U(0));
  for (int t = lane; t < sp.S; t += 32) {
    const double2 f = sp.factor[t];
    if (f.x != 0.0 || f.y != 0.0) z = z + mk((U)f.x, (U)f.y) * cexp_(mk(lp[t].re - mx, lp[t].im));
  }
  z = warp_sum(z);
  return mk(mx + flog(fhypot(z.re, z.im)), fatan2(z.im, z.re));
}

// weight of element t in d log psi: f_t exp(lp_t - log psi) (Exp) or 1/S (Log)
template <typename U>
__device__ __forceinline__ cpx<U> sym_weight(const sym_params& sp, const cpx<U>* lp, cpx<U> lsym, int t) {
  if (sp.avg == VMC_SYM_LOG) return mk(U(1) / U(sp.S), U(0));
  const double2 f = sp.factor[t];
  if (f.x == 0.0 && f.y == 0.0) return mk(U(0), U(0));
  return mk((U)f.x, (U)f.y) * cexp_(mk(lp[t].re - lsym.re, lp[t].im - lsym.im));
}

// log psi of every orbit element of cfg into lp (all warps; ends synchronised)
template <typename T>
__device__ __forceinline__ void sym_element_logpsi(const rbm_params<T>& p, const sym_params& sp, const int8_t* cfg,
                                                   int8_t* tcfg, cpx<double>* lp, int warp, int lane) {
  for (int t = warp; t < sp.S; t += kSymWarps) {
    const bool ok = sym_transform(sp.code + (size_t)t * p.L, cfg, p.L, tcfg, lane);
    cpx<T> acc = mk(T(0), T(0));
    for (int j = lane; j < p.M; j += 32) acc = acc + log_cosh(theta_of(p, tcfg, j));
    acc = warp_sum(acc);
    if (lane == 0) lp[t] = ok ? mk((double)acc.re, (double)acc.im) : mk(nan(""), nan(""));
    __syncwarp();
  }
  __syncthreads();
}

// ------------------------------------------------------------------ log psi
template <typename T>
__global__ void __launch_bounds__(kSymThreads) sym_rbm_logpsi_kernel(const int32_t* __restrict__ configs, int64_t N,
                                                                    rbm_params<T> p, sym_params sp,
                                                                    double2* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int Lp = (p.L + 15) & ~15;
  cpx<double>* lp = reinterpret_cast<cpx<double>*>(smem);
  int8_t* cfg = reinterpret_cast<int8_t*>(lp + sp.S);
  int8_t* tcfg = cfg + Lp + warp * Lp;
  for (int64_t n = blockIdx.x; n < N; n += gridDim.x) {
    for (int i = threadIdx.x; i < p.L; i += blockDim.x) cfg[i] = (int8_t)configs[n * p.L + i];
    __syncthreads();
    sym_element_logpsi(p, sp, cfg, tcfg, lp, warp, lane);
    if (warp == 0) {
      const cpx<double> r = sym_average(sp, lp, lane);
      if (lane == 0) out[n] = make_double2(r.re, r.im);
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------ gradients
// d log psi / d theta = sum_tau w_tau d log psi_RBM(tau s) / d theta:
//   bias_j   : sum_tau a_tau,j
//   W_ij     : sum_tau sigma_tau,i a_tau,j,   a_tau,j = w_tau tanh(theta_tau,j)
// The orbit is processed in chunks of TC elements whose a and tau(s) are
// staged in shared memory; each thread owns output entries (coalesced) and
// adds a chunk's contribution to the row in global memory.
template <typename T>
__global__ void __launch_bounds__(kSymThreads) sym_rbm_grad_kernel(const int32_t* __restrict__ configs, int64_t N,
                                                                  rbm_params<T> p, sym_params sp, int layout,
                                                                  int TC, double2* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int Lp = (p.L + 15) & ~15;
  cpx<double>* lp = reinterpret_cast<cpx<double>*>(smem);
  cpx<double>* wt = lp + sp.S;
  cpx<T>* a = reinterpret_cast<cpx<T>*>(wt + sp.S);
  int8_t* sig = reinterpret_cast<int8_t*>(a + (size_t)TC * p.M);
  int8_t* cfg = sig + (size_t)TC * Lp;
  int8_t* tcfg = cfg + Lp + warp * Lp;
  const bool hasBias = p.b != nullptr;
  const int64_t LM = (int64_t)p.L * p.M;
  const int64_t P = LM + (hasBias ? p.M : 0);
  for (int64_t n = blockIdx.x; n < N; n += gridDim.x) {
    for (int i = threadIdx.x; i < p.L; i += blockDim.x) cfg[i] = (int8_t)configs[n * p.L + i];
    __syncthreads();
    sym_element_logpsi(p, sp, cfg, tcfg, lp, warp, lane);
    if (warp == 0) {
      const cpx<double> lsym = sym_average(sp, lp, lane);
      for (int t = lane; t < sp.S; t += 32) wt[t] = sym_weight(sp, lp, lsym, t);
    }
    __syncthreads();
    for (int c0 = 0; c0 < sp.S; c0 += TC) {
      const int tc = min(TC, sp.S - c0);
      for (int k = warp; k < tc; k += kSymWarps) {
        int8_t* sk = sig + (size_t)k * Lp;
        const bool ok = sym_transform(sp.code + (size_t)(c0 + k) * p.L, cfg, p.L, sk, lane);
        const cpx<double> w = wt[c0 + k];
        const cpx<T> wk = ok ? mk((T)w.re, (T)w.im) : mk(T(nan("")), T(nan("")));
        for (int j = lane; j < p.M; j += 32) a[(size_t)k * p.M + j] = wk * ctanh_(theta_of(p, sk, j));
        __syncwarp();
      }
      __syncthreads();
      for (int64_t e = threadIdx.x; e < P; e += blockDim.x) {
        const int r = (int)(e / p.M);
        const int j = (int)(e - (int64_t)r * p.M);
        cpx<T> acc = mk(T(0), T(0));
        if (hasBias && r == 0) {
          for (int k = 0; k < tc; ++k) acc = acc + a[(size_t)k * p.M + j];
        } else {
          const int i = r - (hasBias ? 1 : 0);
          for (int k = 0; k < tc; ++k) {
            const cpx<T> v = a[(size_t)k * p.M + j];
            if (sig[(size_t)k * Lp + i]) acc = acc + v;
            else acc = acc - v;
          }
        }
        double gr = (double)acc.re, gi = (double)acc.im;
        if (layout == VMC_GRAD_COMPACT) {
          double2* o = out + n * P + e;
          if (c0) {
            const double2 prev = *o;
            gr += prev.x;
            gi += prev.y;
          }
          *o = make_double2(gr, gi);
        } else {
          // per leaf [g, i g]; leaves in Flax order: bias (if any), kernel
          double2* row = out + n * 2 * P;
          int64_t ig, ii;
          if (hasBias && r == 0) {
            ig = j;
            ii = p.M + j;
          } else {
            const int64_t off = hasBias ? 2 * (int64_t)p.M : 0;
            const int64_t ek = e - (hasBias ? p.M : 0);
            ig = off + ek;
            ii = off + LM + ek;
          }
          if (c0) {
            const double2 prev = row[ig];
            gr += prev.x;
            gi += prev.y;
          }
          row[ig] = make_double2(gr, gi);
          row[ii] = make_double2(-gi, gr);
        }
      }
      __syncthreads();
    }
  }
}

// ------------------------------------------------------- fused O_loc (Exp)
// O_loc(s) = sum_k m_k psi(s'_k)/psi(s) with
//   psi(s'_k)/psi(s) = sum_tau w_tau r_tau,k,  w_tau = f_tau psi_RBM(tau s)/psi(s),
// r_tau,k = psi_RBM(tau s'_k)/psi_RBM(tau s) the product over hidden units of
// the plain kernel's one-flip / several-flip factors, at the positions of
// tau(s) that the string's flipped sites map to.  Per pass every thread
// applies one string; the nonzero flipping strings are compacted in string
// order (ballots, so the summation order is fixed).  Then G threads per
// orbit element (JPT hidden units each, tanh(theta) in registers) form
// sum_k m_k r_tau,k, the product over the G threads by a butterfly.
template <typename T, int JPT>
__global__ void __launch_bounds__(kSymThreads) sym_rbm_oloc_fused_kernel(
    const int32_t* __restrict__ configs, int64_t N, rbm_params<T> p, sym_params sp, const cpx<T>* __restrict__ tab,
    vmc_bf_operator op, int G, const double2* __restrict__ logPsiS, double2* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gid = threadIdx.x / G, sub = threadIdx.x - gid * G, nGroups = kSymThreads / G;
  const int L = p.L, M = p.M, Lp = (L + 15) & ~15;
  const int nw = (L + 31) >> 5;
  const int diagWords = (op.num_ops + 31) >> 5;
  cpx<double>* lp = reinterpret_cast<cpx<double>*>(smem);
  cpx<double>* A = lp + sp.S;
  cpx<double>* cm = A + sp.S;
  uint32_t* isdiag = reinterpret_cast<uint32_t*>(cm + kSymChunk);
  uint32_t* occ = isdiag + diagWords;
  int* wcount = reinterpret_cast<int*>(occ + nw);
  int16_t* cfs = reinterpret_cast<int16_t*>(wcount + kSymWarps);
  int8_t* cnf = reinterpret_cast<int8_t*>(cfs + (size_t)kSymChunk * VMC_BF_MAX_LEN);
  int8_t* bad = cnf + kSymChunk;        // per orbit element: malformed orbit tables
  int8_t* cfg = bad + ((sp.S + 15) & ~15);
  int8_t* tcfg = cfg + Lp;              // (S, Lp): tau(s) of every orbit element

  for (int w = threadIdx.x; w < diagWords; w += blockDim.x) isdiag[w] = 0u;
  __syncthreads();
  for (int d = threadIdx.x; d < op.num_diag; d += blockDim.x) {
    const int o = op.diag[d];
    if ((unsigned)o < (unsigned)op.num_ops) atomicOr(&isdiag[o >> 5], 1u << (o & 31));
  }
  __syncthreads();

  const size_t LM = (size_t)L * M;
  const cpx<T>* tC = tab;
  const cpx<T>* tS = tab + LM;
  const cpx<T>* tEp = tab + 2 * LM;
  const cpx<T>* tEm = tab + 3 * LM;

  for (int64_t n = blockIdx.x; n < N; n += gridDim.x) {
    if (warp == 0) warp_load_config(configs + n * L, L, cfg, occ, lane);
    for (int t = threadIdx.x; t < sp.S; t += blockDim.x) {
      A[t] = mk(0.0, 0.0);
      bad[t] = 0;
    }
    __syncthreads();
    for (int t = warp; t < sp.S; t += kSymWarps) {
      const bool ok = sym_transform(sp.code + (size_t)t * L, cfg, L, tcfg + (size_t)t * Lp, lane);
      if (lane == 0 && !ok) bad[t] = 1;
    }
    __syncthreads();
    cpx<double> diagAcc = mk(0.0, 0.0), constAcc = mk(0.0, 0.0);
    // at least one pass: it also forms the per-element log psi
    for (int c0 = 0; c0 < max(op.num_ops, 1); c0 += kSymChunk) {
      const int o = c0 + threadIdx.x;
      bool valid = false;
      int nf = 0;
      cpx<double> m = mk(0.0, 0.0);
      int16_t fsl[VMC_BF_MAX_LEN];
      if (o < op.num_ops) {
        bf_string_result r;
        bf_apply_string(op, o, cfg, occ, L, r);
        if ((isdiag[o >> 5] >> (o & 31)) & 1u) {
          diagAcc = diagAcc + r.m;
        } else if (sqrt(abs2(r.m)) > 1e-6) {  // _find_nonzero threshold (base.py:96)
          for (int q = 0; q < r.nmod; ++q)
            if (r.val[q] != cfg[r.site[q]]) fsl[nf++] = (int16_t)r.site[q];
          if (nf == 0) {
            constAcc = constAcc + r.m;  // flips cancel: psi(s') / psi(s) = 1
          } else {
            valid = true;
            m = r.m;
          }
        }
      }
      const unsigned b = __ballot_sync(0xffffffffu, valid);
      if (lane == 0) wcount[warp] = __popc(b);
      __syncthreads();
      int off = 0, total = 0;
      for (int w = 0; w < kSymWarps; ++w) {
        if (w < warp) off += wcount[w];
        total += wcount[w];
      }
      if (valid) {
        const int pos = off + __popc(b & ((1u << lane) - 1u));
        cm[pos] = m;
        cnf[pos] = (int8_t)nf;
        for (int q = 0; q < nf; ++q) cfs[pos * VMC_BF_MAX_LEN + q] = fsl[q];
      }
      __syncthreads();
      // same trip counts on every thread: the group butterflies see full warps
      for (int t0 = 0; t0 < sp.S; t0 += nGroups) {
        const int t = t0 + gid;
        const bool active = t < sp.S;
        const int tt = active ? t : 0;
        const int8_t* tc = tcfg + (size_t)tt * Lp;
        const int32_t* inv = sp.inv + (size_t)tt * L;
        cpx<T> th[JPT];
        cpx<T> lpt = mk(T(0), T(0));
#pragma unroll
        for (int q = 0; q < JPT; ++q) {
          const int j = sub + q * G;
          if (active && j < M) {
            const cpx<T> x = theta_of(p, tc, j);
            if (c0 == 0) lpt = lpt + log_cosh(x);
            th[q] = ctanh_(x);
          } else {
            th[q] = mk(T(0), T(0));
          }
        }
        if (c0 == 0) {
          for (int mm = 1; mm < G; mm <<= 1) lpt = lpt + shfl_xor(lpt, mm);
          if (active && sub == 0) lp[t] = mk((double)lpt.re, (double)lpt.im);
        }
        cpx<double> acc = mk(0.0, 0.0);
        for (int k = 0; k < total; ++k) {
          const int nfk = cnf[k];
          const int16_t* fs = cfs + k * VMC_BF_MAX_LEN;
          scaled_cpx<T> prod;
          prod.m = mk(T(1), T(0));
          prod.ex = 0;
          bool good = active;
          for (int q = 0; q < nfk; ++q) good = good && (unsigned)inv[fs[q]] < (unsigned)L;
          if (!active) {
          } else if (!good) {
            prod.m = mk(T(nan("")), T(nan("")));
          } else if (nfk == 1) {
            const int pi = inv[fs[0]];
            const T sg = tc[pi] ? T(1) : T(-1);
            const cpx<T>* rc = tC + (size_t)pi * M;
            const cpx<T>* rs = tS + (size_t)pi * M;
#pragma unroll
            for (int q = 0; q < JPT; ++q) {
              const int j = sub + q * G;
              if (j < M) prod.m = prod.m * (rc[j] - sg * (th[q] * rs[j]));
              if ((q & 7) == 7) renorm(prod);
            }
          } else {
#pragma unroll
            for (int q = 0; q < JPT; ++q) {
              const int j = sub + q * G;
              if (j < M) {
                cpx<T> e1 = mk(T(1), T(0)), e2 = mk(T(1), T(0));
                for (int qq = 0; qq < nfk; ++qq) {
                  const int pq = inv[fs[qq]];
                  const cpx<T> ea = tEp[(size_t)pq * M + j], eb = tEm[(size_t)pq * M + j];
                  if (tc[pq]) {
                    e1 = e1 * eb;
                    e2 = e2 * ea;
                  } else {
                    e1 = e1 * ea;
                    e2 = e2 * eb;
                  }
                }
                const cpx<T> tj = th[q];
                const cpx<T> onep = mk(T(1) + tj.re, tj.im), onem = mk(T(1) - tj.re, -tj.im);
                prod.m = prod.m * (T(0.5) * (onep * e1 + onem * e2));
              }
              if ((q & 7) == 7) renorm(prod);
            }
          }
          renorm(prod);
          for (int mm = 1; mm < G; mm <<= 1) {
            scaled_cpx<T> o2;
            o2.m = shfl_xor(prod.m, mm);
            o2.ex = __shfl_xor_sync(0xffffffffu, prod.ex, mm);
            prod = mul(prod, o2);
          }
          const cpx<T> r = to_cpx(prod);
          acc = acc + cm[k] * mk((double)r.re, (double)r.im);
        }
        if (active && sub == 0) A[t] = A[t] + acc;
      }
      __syncthreads();
    }
    const double dr = block_sum(diagAcc.re), di = block_sum(diagAcc.im);
    const double cr = block_sum(constAcc.re), ci = block_sum(constAcc.im);
    if (warp == 0) {
      for (int t = lane; t < sp.S; t += 32)
        if (bad[t]) lp[t] = mk(nan(""), nan(""));
      __syncwarp();
      const cpx<double> lsym = sym_average(sp, lp, lane);
      cpx<double> E = mk(0.0, 0.0);
      for (int t = lane; t < sp.S; t += 32) E = E + sym_weight(sp, lp, lsym, t) * A[t];
      E = warp_sum(E);
      E = E + mk(cr, ci);
      if (op.num_diag > 0 && sqrt(dr * dr + di * di) > 1e-6) E = E + mk(dr, di);
      if (logPsiS) {
        const double2 g = logPsiS[n];
        E = E * cexp_(mk(lsym.re - g.x, lsym.im - g.y));
      }
      if (lane == 0) out[n] = make_double2(E.re, E.im);
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------- Metropolis
// One block per chain.  State: tanh(theta_tau,j) of every orbit element
// (shared memory) and, for Exp, the weights w_tau = f_tau psi_RBM(tau s) /
// psi(s) (sum 1).  A flip of site i changes position p = inv[tau][i] of
// tau(s); r_tau = prod_j (cosh 2W_pj - sigma tanh(theta_tau,j) sinh 2W_pj) and
//   psi(s')/psi(s) = sum_tau w_tau r_tau          (Exp)
//   |psi(s')/psi(s)| = prod_tau |r_tau|^(1/S)      (Log).
// Acceptance iff u < |psi(s')/psi(s)|^mu (sampler.py:335-340).  On acceptance
// tanh(theta + D) = (t - sigma tanh 2W) / (1 - sigma t tanh 2W) and
// w_tau <- w_tau r_tau / R.  Every sweepSteps steps the state is rebuilt from
// the configuration, so rounding does not accumulate.
template <typename T>
__device__ void sym_mc_rebuild(const rbm_params<T>& p, const sym_params& sp, const int8_t* cfg, int8_t* tcfg,
                               cpx<T>* tst, cpx<T>* w, int warp, int lane) {
  for (int t = warp; t < sp.S; t += kSymWarps) {
    const bool ok = sym_transform(sp.code + (size_t)t * p.L, cfg, p.L, tcfg, lane);
    cpx<T> acc = mk(T(0), T(0));
    for (int j = lane; j < p.M; j += 32) {
      const cpx<T> x = theta_of(p, tcfg, j);
      acc = acc + log_cosh(x);
      tst[(size_t)t * p.M + j] = ctanh_(x);
    }
    acc = warp_sum(acc);
    if (lane == 0) w[t] = ok ? acc : mk(T(nan("")), T(nan("")));
    __syncwarp();
  }
  __syncthreads();
  if (warp == 0 && sp.avg == VMC_SYM_EXP) {
    const cpx<T> lsym = sym_average(sp, w, lane);  // every lane holds it before w is overwritten
    for (int t = lane; t < sp.S; t += 32) w[t] = sym_weight(sp, w, lsym, t);
  }
  __syncthreads();
}

// per (orbit element, site): 2 * position + flip bit of that position, or -1
// when the tables are malformed
__device__ __forceinline__ void sym_build_comb(const sym_params& sp, int L, int16_t* comb) {
  for (int e = threadIdx.x; e < sp.S * L; e += blockDim.x) {
    const int t = e / L;
    const int pi = sp.inv[e];
    int v = -1;
    if ((unsigned)pi < (unsigned)L) {
      const int c = sp.code[(size_t)t * L + pi];
      if ((unsigned)(c >> 1) < (unsigned)L) v = 2 * pi + (c & 1);
    }
    comb[e] = (int16_t)v;
  }
}

// r_tau = exp(rowLogC_p) prod_j (1 - sigma tanh(theta_j) tanh(2 W_pj)):
// cosh(theta + D)/cosh(theta) = cosh 2W (1 - sigma t tanh 2W), the row's
// cosh product taken out of the loop.  G threads per orbit element, JPT
// hidden units each (loads hoisted by the unrolled loop), butterfly over G.
template <typename T, int JPT>
__global__ void __launch_bounds__(kSymThreads) sym_rbm_metropolis_kernel(
    int32_t* __restrict__ states, int C, rbm_params<T> p, sym_params sp, const cpx<T>* __restrict__ tab, double mu,
    uint64_t seed, uint32_t call, int64_t thermSteps, int64_t sweepSteps, int64_t samplesPerChain, int G,
    int32_t* __restrict__ configsOut, unsigned long long* __restrict__ counters) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int sAcc;
  __shared__ cpx<T> sR;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gid = threadIdx.x / G, sub = threadIdx.x - gid * G, nGroups = kSymThreads / G;
  const int chain = blockIdx.x;
  const int L = p.L, M = p.M, Lp = (L + 15) & ~15;
  // weights, ratios and the decision in the kernel's arithmetic T (the FP32
  // sampler does no FP64 work per proposal)
  cpx<T>* w = reinterpret_cast<cpx<T>*>(smem);
  cpx<T>* rat = w + sp.S;
  cpx<T>* tst = rat + sp.S;
  int16_t* comb = reinterpret_cast<int16_t*>(tst + (size_t)sp.S * M);
  int8_t* cfg = reinterpret_cast<int8_t*>(comb + (((size_t)sp.S * L + 7) & ~(size_t)7));
  int8_t* tcfg = cfg + Lp + warp * Lp;
  int32_t* st = states + (size_t)chain * L;
  for (int i = threadIdx.x; i < L; i += blockDim.x) cfg[i] = (int8_t)st[i];
  sym_build_comb(sp, L, comb);
  __syncthreads();
  sym_mc_rebuild(p, sp, cfg, tcfg, tst, w, warp, lane);

  const size_t LM = (size_t)L * M;
  const cpx<T>* tT = tab + 4 * LM;
  const cpx<T>* rowLogC = tab + 5 * LM;
  unsigned long long accepted = 0;
  const int64_t total = thermSteps + sweepSteps * samplesPerChain;
  for (int64_t step = 0; step < total; ++step) {
    const mc_draw d = metropolis_draw(seed, call, (uint32_t)step, (uint32_t)chain, L);
    const int i = d.site;
    // same trip counts on every thread: the group butterflies see full warps
    for (int t0 = 0; t0 < sp.S; t0 += nGroups) {
      const int t = t0 + gid;
      const bool active = t < sp.S;
      const int pc = active ? comb[t * L + i] : 0;
      const int pi = pc >> 1;
      const T sg = (cfg[i] ^ (pc & 1)) ? T(1) : T(-1);
      scaled_cpx<T> prod;
      prod.m = mk(T(1), T(0));
      prod.ex = 0;
      if (active && pc >= 0) {
        const cpx<T>* rt = tT + (size_t)pi * M;
        const cpx<T>* tt = tst + (size_t)t * M;
        cpx<T> tv[JPT], rv[JPT];
#pragma unroll
        for (int q = 0; q < JPT; ++q) {
          const int j = sub + q * G;
          tv[q] = j < M ? tt[j] : mk(T(0), T(0));
          rv[q] = j < M ? rt[j] : mk(T(0), T(0));
        }
#pragma unroll
        for (int q = 0; q < JPT; ++q) {
          const cpx<T> f = tv[q] * rv[q];
          prod.m = prod.m * mk(T(1) - sg * f.re, -sg * f.im);
          if ((q & 7) == 7) renorm(prod);
        }
      } else if (active) {
        prod.m = mk(T(nan("")), T(nan("")));
      }
      renorm(prod);
      for (int m = 1; m < G; m <<= 1) {
        scaled_cpx<T> o;
        o.m = shfl_xor(prod.m, m);
        o.ex = __shfl_xor_sync(0xffffffffu, prod.ex, m);
        prod = mul(prod, o);
      }
      if (active && sub == 0) {
        if (pc >= 0) {
          // times exp(rowLogC_p) = 2^e2 * (exp(re - e2 ln 2) (cos im, sin im))
          const cpx<T> lc = rowLogC[pi];
          const T e2 = floor(lc.re * T(1.4426950408889634));
          scaled_cpx<T> cr;
          cr.m = cexp_(mk(lc.re - e2 * T(0.6931471805599453), lc.im));
          cr.ex = (int)e2;
          prod = mul(prod, cr);
        }
        // ratios beyond the float range saturate (they decide acceptance alone)
        const int lim = sizeof(T) == sizeof(double) ? 2000 : 120;
        const int e = max(-lim, min(lim, prod.ex));
        rat[t] = mk(ldexp(prod.m.re, e), ldexp(prod.m.im, e));
      }
    }
    __syncthreads();
    if (warp == 0) {
      T logr2;
      cpx<T> R = mk(T(0), T(0));
      if (sp.avg == VMC_SYM_EXP) {
        for (int t = lane; t < sp.S; t += 32) R = R + w[t] * rat[t];
        R = warp_sum(R);
        logr2 = flog(abs2(R));
      } else {
        T s = T(0);
        for (int t = lane; t < sp.S; t += 32) s += flog(abs2(rat[t]));
        logr2 = warp_sum(s) / T(sp.S);
      }
      // P = |psi(s')/psi(s)|^mu; accept iff u < P (bernoulli, sampler.py:339-340)
      bool acc;
      if (sizeof(T) == sizeof(double)) {
        acc = d.u64() < exp(0.5 * mu * (double)logr2);
      } else {
        acc = d.u32() < expf(0.5f * (float)mu * (float)logr2);
      }
      if (lane == 0) {
        sAcc = acc ? 1 : 0;
        sR = R;
      }
    }
    __syncthreads();
    if (sAcc) {
      const cpx<T> R = sR;
      for (int t = gid; t < sp.S; t += nGroups) {
        const int pc = comb[t * L + i];
        if (pc >= 0) {
          const T sg = (cfg[i] ^ (pc & 1)) ? T(1) : T(-1);
          const cpx<T>* rt = tT + (size_t)(pc >> 1) * M;
          cpx<T>* tt = tst + (size_t)t * M;
          // tanh(theta + D) = (t - sigma tanh 2W) / (1 - sigma t tanh 2W)
          for (int j = sub; j < M; j += G) {
            const cpx<T> tj = tt[j], rj = rt[j];
            const cpx<T> f = tj * rj;
            tt[j] = cdiv(mk(tj.re - sg * rj.re, tj.im - sg * rj.im), mk(T(1) - sg * f.re, -sg * f.im));
          }
        }
        if (sub == 0 && sp.avg == VMC_SYM_EXP) w[t] = cdiv(w[t] * rat[t], R);
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        cfg[i] = cfg[i] ? 0 : 1;
        ++accepted;
      }
      __syncthreads();
    }
    if (step >= thermSteps && ((step - thermSteps + 1) % sweepSteps) == 0) {
      const int64_t s = (step - thermSteps + 1) / sweepSteps - 1;
      int32_t* o = configsOut + ((size_t)s * C + chain) * L;
      for (int k = threadIdx.x; k < L; k += blockDim.x) o[k] = cfg[k];
    }
    if ((step + 1) % sweepSteps == 0 && step + 1 < total) sym_mc_rebuild(p, sp, cfg, tcfg, tst, w, warp, lane);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < L; k += blockDim.x) st[k] = cfg[k];
  if (threadIdx.x == 0) {
    atomicAdd(&counters[0], (unsigned long long)total);
    atomicAdd(&counters[1], accepted);
  }
}

// --------------------------------------------------------------- host side
int check_sym(const char* fn, const vmc_sym_desc* sym) {
  VMC_REQUIRE(sym && sym->orbit && sym->inverse && sym->factor, VMC_ERR_INVALID_ARGUMENT,
              "%s: null symmetry descriptor", fn);
  VMC_REQUIRE(sym->num_sym > 0 && sym->num_sym <= kMaxSym, VMC_ERR_UNSUPPORTED, "%s: orbit of %d elements outside [1, %d]",
              fn, sym->num_sym, kMaxSym);
  VMC_REQUIRE(sym->average == VMC_SYM_EXP || sym->average == VMC_SYM_LOG, VMC_ERR_INVALID_ARGUMENT,
              "%s: unknown average %d", fn, sym->average);
  return VMC_OK;
}

sym_params make_sym(const vmc_sym_desc* s) {
  sym_params sp;
  sp.S = s->num_sym;
  sp.avg = s->average;
  sp.code = s->orbit;
  sp.inv = s->inverse;
  sp.factor = reinterpret_cast<const double2*>(s->factor);
  return sp;
}

// threads per orbit element in the per-proposal kernels: a power of two
// <= 32 that spreads the block's threads over the orbit and keeps at least
// a few hidden units per thread
int group_size(int S, int M) {
  int G = 32;
  while (G > 1 && (G * S > kSymThreads || G * 4 > M)) G >>= 1;
  return G;
}

int sym_grid(int64_t N) { return (int)std::max<int64_t>(1, std::min<int64_t>(N, 152 * 4)); }

size_t lp_bytes(int S) { return (size_t)S * 16; }

}  // namespace vmc

using namespace vmc;

extern "C" int vmc_sym_rbm_logpsi(int32_t precision, const int32_t* configs, int64_t num_configs, int32_t num_sites,
                                  int32_t num_hidden, const void* kernel, const void* bias, const vmc_sym_desc* sym,
                                  double* log_psi, vmc_stream_t stream) {
  int rc = check_rbm_args("vmc_sym_rbm_logpsi", precision, configs, num_configs, num_sites, num_hidden, kernel);
  if (rc) return rc;
  if ((rc = check_sym("vmc_sym_rbm_logpsi", sym))) return rc;
  VMC_REQUIRE(log_psi || num_configs == 0, VMC_ERR_INVALID_ARGUMENT, "vmc_sym_rbm_logpsi: null output");
  if (num_configs == 0) return VMC_OK;
  const int Lp = (num_sites + 15) & ~15;
  const size_t smem = lp_bytes(sym->num_sym) + (size_t)(1 + kSymWarps) * Lp;
  VMC_REQUIRE(smem <= kSmemLimit, VMC_ERR_UNSUPPORTED, "vmc_sym_rbm_logpsi: problem too large");
  cudaStream_t st = as_stream(stream);
  const sym_params sp = make_sym(sym);
  if (precision == VMC_F64) {
    VMC_ALLOW_SMEM(sym_rbm_logpsi_kernel<double>, smem, "vmc_sym_rbm_logpsi");
    sym_rbm_logpsi_kernel<double><<<sym_grid(num_configs), kSymThreads, smem, st>>>(
        configs, num_configs, make_params<double>(kernel, bias, num_sites, num_hidden), sp,
        reinterpret_cast<double2*>(log_psi));
  } else {
    VMC_ALLOW_SMEM(sym_rbm_logpsi_kernel<float>, smem, "vmc_sym_rbm_logpsi");
    sym_rbm_logpsi_kernel<float><<<sym_grid(num_configs), kSymThreads, smem, st>>>(
        configs, num_configs, make_params<float>(kernel, bias, num_sites, num_hidden), sp,
        reinterpret_cast<double2*>(log_psi));
  }
  return check_launch("vmc_sym_rbm_logpsi");
}

extern "C" int vmc_sym_rbm_gradients(int32_t precision, const int32_t* configs, int64_t num_configs,
                                     int32_t num_sites, int32_t num_hidden, const void* kernel, const void* bias,
                                     const vmc_sym_desc* sym, int32_t layout, double* out, vmc_stream_t stream) {
  int rc = check_rbm_args("vmc_sym_rbm_gradients", precision, configs, num_configs, num_sites, num_hidden, kernel);
  if (rc) return rc;
  if ((rc = check_sym("vmc_sym_rbm_gradients", sym))) return rc;
  VMC_REQUIRE(layout == VMC_GRAD_REFERENCE || layout == VMC_GRAD_COMPACT, VMC_ERR_INVALID_ARGUMENT,
              "vmc_sym_rbm_gradients: unknown layout %d", layout);
  VMC_REQUIRE(out || num_configs == 0, VMC_ERR_INVALID_ARGUMENT, "vmc_sym_rbm_gradients: null output");
  if (num_configs == 0) return VMC_OK;
  const int Lp = (num_sites + 15) & ~15;
  const size_t el = precision == VMC_F64 ? 16 : 8;
  const size_t fixed = 2 * lp_bytes(sym->num_sym) + (size_t)(1 + kSymWarps) * Lp;
  const size_t perElem = (size_t)num_hidden * el + Lp;
  VMC_REQUIRE(fixed + perElem <= kSmemLimit, VMC_ERR_UNSUPPORTED, "vmc_sym_rbm_gradients: M=%d too large", num_hidden);
  // orbit chunk: as many elements as fit in about 96 KB, rounded to whole warps
  int TC = (int)std::min<size_t>((size_t)sym->num_sym, std::max<size_t>(1, (96 * 1024) / perElem));
  if (TC > kSymWarps) TC -= TC % kSymWarps;
  const size_t smem = fixed + (size_t)TC * perElem;
  VMC_REQUIRE(smem <= kSmemLimit, VMC_ERR_UNSUPPORTED, "vmc_sym_rbm_gradients: problem too large");
  cudaStream_t st = as_stream(stream);
  const sym_params sp = make_sym(sym);
  if (precision == VMC_F64) {
    VMC_ALLOW_SMEM(sym_rbm_grad_kernel<double>, smem, "vmc_sym_rbm_gradients");
    sym_rbm_grad_kernel<double><<<sym_grid(num_configs), kSymThreads, smem, st>>>(
        configs, num_configs, make_params<double>(kernel, bias, num_sites, num_hidden), sp, layout, TC,
        reinterpret_cast<double2*>(out));
  } else {
    VMC_ALLOW_SMEM(sym_rbm_grad_kernel<float>, smem, "vmc_sym_rbm_gradients");
    sym_rbm_grad_kernel<float><<<sym_grid(num_configs), kSymThreads, smem, st>>>(
        configs, num_configs, make_params<float>(kernel, bias, num_sites, num_hidden), sp, layout, TC,
        reinterpret_cast<double2*>(out));
  }
  return check_launch("vmc_sym_rbm_gradients");
}

template <typename T, int JPT>
static int launch_sym_oloc(int grid, size_t smem, cudaStream_t st, const int32_t* configs, int64_t N,
                            rbm_params<T> p, sym_params sp, const void* tables, const vmc_bf_operator* op, int G,
                            const double* lps, double* out) {
  VMC_ALLOW_SMEM((sym_rbm_oloc_fused_kernel<T, JPT>), smem, "vmc_sym_rbm_oloc_fused");
  sym_rbm_oloc_fused_kernel<T, JPT><<<grid, kSymThreads, smem, st>>>(
      configs, N, p, sp, reinterpret_cast<const cpx<T>*>(tables), *op, G, reinterpret_cast<const double2*>(lps),
      reinterpret_cast<double2*>(out));
  return VMC_OK;
}

template <typename T>
static int dispatch_sym_oloc(int jpt, int grid, size_t smem, cudaStream_t st, const int32_t* configs, int64_t N,
                             rbm_params<T> p, sym_params sp, const void* tables, const vmc_bf_operator* op, int G,
                             const double* lps, double* out) {
  int rc;
  if (jpt <= 2) rc = launch_sym_oloc<T, 2>(grid, smem, st, configs, N, p, sp, tables, op, G, lps, out);
  else if (jpt <= 4) rc = launch_sym_oloc<T, 4>(grid, smem, st, configs, N, p, sp, tables, op, G, lps, out);
  else if (jpt <= 8) rc = launch_sym_oloc<T, 8>(grid, smem, st, configs, N, p, sp, tables, op, G, lps, out);
  else rc = launch_sym_oloc<T, 16>(grid, smem, st, configs, N, p, sp, tables, op, G, lps, out);
  if (rc) return rc;
  return check_launch("vmc_sym_rbm_oloc_fused");
}

extern "C" int vmc_sym_rbm_oloc_fused(int32_t precision, const int32_t* configs, int64_t num_configs,
                                      int32_t num_sites, int32_t num_hidden, const void* kernel, const void* bias,
                                      const void* tables, const vmc_sym_desc* sym, const vmc_bf_operator* op,
                                      const double* log_psi_s, double* oloc, vmc_stream_t stream) {
  int rc = check_rbm_args("vmc_sym_rbm_oloc_fused", precision, configs, num_configs, num_sites, num_hidden, kernel);
  if (rc) return rc;
  if ((rc = check_sym("vmc_sym_rbm_oloc_fused", sym))) return rc;
  if ((rc = check_op("vmc_sym_rbm_oloc_fused", op, num_sites))) return rc;
  VMC_REQUIRE(sym->average == VMC_SYM_EXP, VMC_ERR_UNSUPPORTED,
              "vmc_sym_rbm_oloc_fused: only the Exp average has a fused estimator");
  VMC_REQUIRE(op->local_dim == 2, VMC_ERR_UNSUPPORTED, "vmc_sym_rbm_oloc_fused: local dimension %d (RBM needs 2)",
              op->local_dim);
  VMC_REQUIRE(num_hidden <= 32 * 16, VMC_ERR_UNSUPPORTED, "vmc_sym_rbm_oloc_fused: M=%d > 512", num_hidden);
  VMC_REQUIRE(tables && (oloc || num_configs == 0), VMC_ERR_INVALID_ARGUMENT,
              "vmc_sym_rbm_oloc_fused: null argument");
  if (num_configs == 0) return VMC_OK;
  // threads per orbit element: at most 8 hidden units per thread (16 when
  // M > 256), which keeps tanh(theta) in registers at two blocks per SM
  int G = group_size(sym->num_sym, num_hidden);
  while (G < 32 && (num_hidden + G - 1) / G > 8) G <<= 1;
  const int jpt = (num_hidden + G - 1) / G;
  const int Lp = (num_sites + 15) & ~15;
  const int nw = (num_sites + 31) >> 5;
  const int diagWords = (op->num_ops + 31) >> 5;
  const size_t smem = 2 * lp_bytes(sym->num_sym) + (size_t)kSymChunk * 16 +
                      (size_t)(diagWords + nw + kSymWarps) * 4 + (size_t)kSymChunk * VMC_BF_MAX_LEN * 2 + kSymChunk +
                      (size_t)((sym->num_sym + 15) & ~15) + Lp + (size_t)sym->num_sym * Lp;
  VMC_REQUIRE(smem <= kSmemLimit, VMC_ERR_UNSUPPORTED, "vmc_sym_rbm_oloc_fused: problem too large");
  cudaStream_t st = as_stream(stream);
  const sym_params sp = make_sym(sym);
  const int grid = sym_grid(num_configs);
  if (precision == VMC_F64)
    return dispatch_sym_oloc<double>(jpt, grid, smem, st, configs, num_configs,
                                     make_params<double>(kernel, bias, num_sites, num_hidden), sp, tables, op, G,
                                     log_psi_s, oloc);
  return dispatch_sym_oloc<float>(jpt, grid, smem, st, configs, num_configs,
                                  make_params<float>(kernel, bias, num_sites, num_hidden), sp, tables, op, G, log_psi_s,
                                  oloc);
}

template <typename T, int JPT>
static int launch_sym_mc(int C, size_t smem, cudaStream_t st, int32_t* states, rbm_params<T> p, sym_params sp,
                          const void* tables, double mu, uint64_t seed, uint32_t call, int64_t therm, int64_t sweep,
                          int64_t spc, int G, int32_t* out, void* counters) {
  VMC_ALLOW_SMEM((sym_rbm_metropolis_kernel<T, JPT>), smem, "vmc_sym_rbm_metropolis");
  sym_rbm_metropolis_kernel<T, JPT><<<C, kSymThreads, smem, st>>>(
      states, C, p, sp, reinterpret_cast<const cpx<T>*>(tables), mu, seed, call, therm, sweep, spc, G, out,
      reinterpret_cast<unsigned long long*>(counters));
  return VMC_OK;
}

template <typename T>
static int dispatch_sym_mc(int jpt, int C, size_t smem, cudaStream_t st, int32_t* states, rbm_params<T> p,
                           sym_params sp, const void* tables, double mu, uint64_t seed, uint32_t call, int64_t therm,
                           int64_t sweep, int64_t spc, int G, int32_t* out, void* counters) {
  if (jpt <= 2) return launch_sym_mc<T, 2>(C, smem, st, states, p, sp, tables, mu, seed, call, therm, sweep, spc, G, out, counters);
  if (jpt <= 4) return launch_sym_mc<T, 4>(C, smem, st, states, p, sp, tables, mu, seed, call, therm, sweep, spc, G, out, counters);
  if (jpt <= 8) return launch_sym_mc<T, 8>(C, smem, st, states, p, sp, tables, mu, seed, call, therm, sweep, spc, G, out, counters);
  if (jpt <= 16) return launch_sym_mc<T, 16>(C, smem, st, states, p, sp, tables, mu, seed, call, therm, sweep, spc, G, out, counters);
  return launch_sym_mc<T, 32>(C, smem, st, states, p, sp, tables, mu, seed, call, therm, sweep, spc, G, out, counters);
}

extern "C" int vmc_sym_rbm_metropolis(int32_t precision, int32_t* states, int32_t num_chains, int32_t num_sites,
                                      int32_t num_hidden, const void* kernel, const void* bias, const void* tables,
                                      const vmc_sym_desc* sym, double mu, uint64_t seed, uint32_t call_index,
                                      int64_t therm_steps, int64_t sweep_steps, int64_t samples_per_chain,
                                      int32_t* configs_out, void* counters, vmc_stream_t stream) {
  int rc = check_rbm_args("vmc_sym_rbm_metropolis", precision, states, num_chains, num_sites, num_hidden, kernel);
  if (rc) return rc;
  if ((rc = check_sym("vmc_sym_rbm_metropolis", sym))) return rc;
  VMC_REQUIRE(num_chains > 0 && tables && counters && sweep_steps > 0 && therm_steps >= 0 && samples_per_chain >= 0,
              VMC_ERR_INVALID_ARGUMENT, "vmc_sym_rbm_metropolis: bad arguments");
  VMC_REQUIRE(configs_out || samples_per_chain == 0, VMC_ERR_INVALID_ARGUMENT, "vmc_sym_rbm_metropolis: null output");
  VMC_REQUIRE(therm_steps + sweep_steps * samples_per_chain < (int64_t)0xFFFFFFFF, VMC_ERR_UNSUPPORTED,
              "vmc_sym_rbm_metropolis: more than 2^32 steps in one call");
  VMC_REQUIRE(mu >= 0.0 && mu <= 2.0, VMC_ERR_INVALID_ARGUMENT, "vmc_sym_rbm_metropolis: mu=%g outside [0, 2]", mu);
  const int Lp = (num_sites + 15) & ~15;
  const size_t el = precision == VMC_F64 ? 16 : 8;
  VMC_REQUIRE(num_hidden <= 32 * 32 && num_sites <= 16383, VMC_ERR_UNSUPPORTED,
              "vmc_sym_rbm_metropolis: M=%d > 1024 or L=%d > 16383", num_hidden, num_sites);
  const size_t smem = (2 + (size_t)num_hidden) * sym->num_sym * el + ((((size_t)sym->num_sym * num_sites + 7) & ~(size_t)7) * 2) +
                      (size_t)(1 + kSymWarps) * Lp;
  VMC_REQUIRE(smem <= kSmemLimit, VMC_ERR_UNSUPPORTED,
              "vmc_sym_rbm_metropolis: %d orbit elements x %d hidden units do not fit in shared memory", sym->num_sym,
              num_hidden);
  cudaStream_t st = as_stream(stream);
  const sym_params sp = make_sym(sym);
  int G = group_size(sym->num_sym, num_hidden);
  while (G < 32 && (num_hidden + G - 1) / G > 16) G <<= 1;
  const int jpt = (num_hidden + G - 1) / G;
  if (precision == VMC_F64)
    rc = dispatch_sym_mc<double>(jpt, num_chains, smem, st, states, make_params<double>(kernel, bias, num_sites, num_hidden),
                                 sp, tables, mu, seed, call_index, therm_steps, sweep_steps, samples_per_chain, G,
                                 configs_out, counters);
  else
    rc = dispatch_sym_mc<float>(jpt, num_chains, smem, st, states, make_params<float>(kernel, bias, num_sites, num_hidden),
                                sp, tables, mu, seed, call_index, therm_steps, sweep_steps, samples_per_chain, G,
                                configs_out, counters);
  if (rc) return rc;
  return check_launch("vmc_sym_rbm_metropolis");
}
