// Complex RBM kernels: log psi, fused local estimator, log-derivatives and
// their FP64 statistics (nets/rbm.py:17-38, operator/base.py:162-192,
// vqs.py:66-69, stats.py:50-58).
#include <algorithm>

#include "bf_apply.cuh"
#include "rbm.cuh"
#include "reduce.cuh"
#include "vmc_common.cuh"

namespace vmc {

// theta_j = b_j + sum_i (2 s_i - 1) W_ij for the hidden units j = lane + 32 q,
// written as tanh(theta_j) (want_tanh) or theta_j into `out` (shared).
template <typename T>
__device__ __forceinline__ void warp_theta(const rbm_params<T>& p, const int8_t* cfg, cpx<T>* out, int lane,
                                           bool want_tanh) {
  for (int j = lane; j < p.M; j += 32) {
    cpx<T> th = p.b ? p.b[j] : mk(T(0), T(0));
    const cpx<T>* w = p.W + j;
    for (int i = 0; i < p.L; ++i) {
      cpx<T> x = w[(size_t)i * p.M];
      if (cfg[i]) {
        th.re += x.re;
        th.im += x.im;
      } else {
        th.re -= x.re;
        th.im -= x.im;
      }
    }
    out[j] = want_tanh ? ctanh_(th) : th;
  }
  __syncwarp();
}

// ------------------------------------------------------------------ tables
template <typename T>
__global__ void rbm_prepare_kernel(const cpx<T>* __restrict__ W, int64_t n, cpx<T>* __restrict__ tab) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    cpx<T> w = W[t];
    cpx<T> ep = cexp_(mk(T(2) * w.re, T(2) * w.im));
    cpx<T> em = cexp_(mk(T(-2) * w.re, T(-2) * w.im));
    tab[t] = T(0.5) * (ep + em);          // cosh 2W
    tab[n + t] = T(0.5) * (ep - em);      // sinh 2W
    tab[2 * n + t] = ep;                  // exp 2W
    tab[3 * n + t] = em;                  // exp -2W
    tab[4 * n + t] = ctanh_(mk(T(2) * w.re, T(2) * w.im));  // tanh 2W
  }
}

// row sums sum_j log cosh(2 W_ij) after the five tables (one warp per row i)
template <typename T>
__global__ void rbm_prepare_rows_kernel(const cpx<T>* __restrict__ W, int L, int M, cpx<T>* __restrict__ rows) {
  const int lane = threadIdx.x & 31;
  for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < L; i += gridDim.x * (blockDim.x >> 5)) {
    cpx<T> s = mk(T(0), T(0));
    for (int j = lane; j < M; j += 32) {
      const cpx<T> w = W[(size_t)i * M + j];
      s = s + log_cosh(mk(T(2) * w.re, T(2) * w.im));
    }
    s = warp_sum(s);
    if (lane == 0) rows[i] = s;
  }
}

// ------------------------------------------------------------------ log psi
template <typename T>
__global__ void rbm_logpsi_kernel(const int32_t* __restrict__ configs, int64_t N, rbm_params<T> p,
                                  double2* __restrict__ out) {
  extern __shared__ unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int8_t* cfg = reinterpret_cast<int8_t*>(smem) + warp * ((p.L + 15) & ~15);
  for (int64_t n = (int64_t)blockIdx.x * kWarpsPerBlock + warp; n < N; n += (int64_t)gridDim.x * kWarpsPerBlock) {
    const int32_t* src = configs + n * p.L;
    for (int i = lane; i < p.L; i += 32) cfg[i] = (int8_t)src[i];
    __syncwarp();
    cpx<T> acc = mk(T(0), T(0));
    for (int j = lane; j < p.M; j += 32) {
      cpx<T> th = p.b ? p.b[j] : mk(T(0), T(0));
      const cpx<T>* w = p.W + j;
      for (int i = 0; i < p.L; ++i) {
        cpx<T> x = w[(size_t)i * p.M];
        if (cfg[i]) {
          th.re += x.re;
          th.im += x.im;
        } else {
          th.re -= x.re;
          th.im -= x.im;
        }
      }
      acc = acc + log_cosh(th);
    }
    acc = warp_sum(acc);
    if (lane == 0) out[n] = make_double2((double)acc.re, (double)acc.im);
    __syncwarp();
  }
}

// ------------------------------------------------------------ gradients
// One warp per sample; tanh(theta) staged in shared memory, rows written
// coalesced.
template <typename T>
__global__ void rbm_grad_kernel(const int32_t* __restrict__ configs, int64_t N, rbm_params<T> p, int layout,
                                double2* __restrict__ out) {
  extern __shared__ unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cfgBytes = (p.L + 15) & ~15;
  cpx<T>* th = reinterpret_cast<cpx<T>*>(smem) + warp * p.M;
  int8_t* cfg = reinterpret_cast<int8_t*>(smem + (size_t)kWarpsPerBlock * p.M * sizeof(cpx<T>)) + warp * cfgBytes;
  const bool hasBias = p.b != nullptr;
  const int64_t P = (int64_t)p.L * p.M + (hasBias ? p.M : 0);
  for (int64_t n = (int64_t)blockIdx.x * kWarpsPerBlock + warp; n < N; n += (int64_t)gridDim.x * kWarpsPerBlock) {
    const int32_t* src = configs + n * p.L;
    for (int i = lane; i < p.L; i += 32) cfg[i] = (int8_t)src[i];
    __syncwarp();
    warp_theta(p, cfg, th, lane, true);
    if (layout == VMC_GRAD_COMPACT) {
      double2* row = out + n * P;
      int off = 0;
      if (hasBias) {
        for (int j = lane; j < p.M; j += 32) row[j] = make_double2(th[j].re, th[j].im);
        off = p.M;
      }
      for (int i = 0; i < p.L; ++i) {
        T s = cfg[i] ? T(1) : T(-1);
        for (int j = lane; j < p.M; j += 32) row[off + i * p.M + j] = make_double2(s * th[j].re, s * th[j].im);
      }
    } else {
      // per leaf [g, i g]; leaves in Flax order: bias (if any), kernel
      double2* row = out + n * 2 * P;
      int off = 0;
      if (hasBias) {
        for (int j = lane; j < p.M; j += 32) {
          row[j] = make_double2(th[j].re, th[j].im);
          row[p.M + j] = make_double2(-(double)th[j].im, th[j].re);
        }
        off = 2 * p.M;
      }
      const int64_t LM = (int64_t)p.L * p.M;
      for (int i = 0; i < p.L; ++i) {
        T s = cfg[i] ? T(1) : T(-1);
        for (int j = lane; j < p.M; j += 32) {
          double gr = s * th[j].re, gi = s * th[j].im;
          row[off + i * p.M + j] = make_double2(gr, gi);
          row[off + LM + i * p.M + j] = make_double2(-gi, gr);
        }
      }
    }
    __syncwarp();
  }
}

// ------------------------------------------------------- fused O_loc
// One warp per sample.  For every operator string the warp applies the
// string (redundantly on all lanes), and for strings that flip spins forms
// psi(s')/psi(s) = prod_j cosh(theta_j + D_j)/cosh(theta_j) with
// D_j = -2 sum_{flipped i} (2 s_i - 1) W_ij, each factor being
//   one flip :  cosh(2W_ij) - sigma_i tanh(theta_j) sinh(2W_ij)
//   several  :  [(1 + t_j) e^{D_j} + (1 - t_j) e^{-D_j}] / 2
// with e^{+-D_j} products of exp(+-2W) table entries.  Lanes own hidden
// units j = lane + 32 q; the product is kept as mantissa * 2^exponent.
template <typename T>
__global__ void rbm_oloc_fused_kernel(const int32_t* __restrict__ configs, int64_t N, rbm_params<T> p,
                                      const cpx<T>* __restrict__ tab, vmc_bf_operator op,
                                      const double2* __restrict__ logPsiS, double2* __restrict__ out) {
  extern __shared__ unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = (p.L + 31) >> 5;
  const int cfgBytes = (p.L + 15) & ~15;
  // shared layout: [is_diag bits (num_ops)] [per warp: tanh theta (M) | occ (nw words) | cfg (L bytes)]
  uint32_t* isdiag = reinterpret_cast<uint32_t*>(smem);
  const int diagWords = (op.num_ops + 31) >> 5;
  unsigned char* base = smem + ((diagWords * 4 + 15) & ~15);
  const size_t perWarp = (size_t)p.M * sizeof(cpx<T>) + (size_t)nw * 4 + cfgBytes;
  const size_t perWarpAligned = (perWarp + 15) & ~(size_t)15;
  cpx<T>* th = reinterpret_cast<cpx<T>*>(base + warp * perWarpAligned);
  uint32_t* occ = reinterpret_cast<uint32_t*>(th + p.M);
  int8_t* cfg = reinterpret_cast<int8_t*>(occ + nw);
  int16_t* fsites = reinterpret_cast<int16_t*>(base + kWarpsPerBlock * perWarpAligned);

  for (int w = threadIdx.x; w < diagWords; w += blockDim.x) isdiag[w] = 0u;
  __syncthreads();
  for (int d = threadIdx.x; d < op.num_diag; d += blockDim.x) {
    const int o = op.diag[d];
    if ((unsigned)o < (unsigned)op.num_ops) atomicOr(&isdiag[o >> 5], 1u << (o & 31));
  }
  __syncthreads();

  const size_t LM = (size_t)p.L * p.M;
  const cpx<T>* tC = tab;
  const cpx<T>* tS = tab + LM;
  const cpx<T>* tEp = tab + 2 * LM;
  const cpx<T>* tEm = tab + 3 * LM;

  for (int64_t n = (int64_t)blockIdx.x * kWarpsPerBlock + warp; n < N; n += (int64_t)gridDim.x * kWarpsPerBlock) {
    warp_load_config(configs + n * p.L, p.L, cfg, occ, lane);
    // theta -> tanh(theta) in shared memory; log psi(s) of the network only
    // when the caller supplied its own log psi(s) to divide by
    cpx<T> lpNet = mk(T(0), T(0));
    for (int j = lane; j < p.M; j += 32) {
      cpx<T> t = p.b ? p.b[j] : mk(T(0), T(0));
      const cpx<T>* w = p.W + j;
      for (int i = 0; i < p.L; ++i) {
        cpx<T> x = w[(size_t)i * p.M];
        if (cfg[i]) {
          t.re += x.re;
          t.im += x.im;
        } else {
          t.re -= x.re;
          t.im -= x.im;
        }
      }
      if (logPsiS) lpNet = lpNet + log_cosh(t);
      th[j] = ctanh_(t);
    }
    __syncwarp();

    // Strings are handled 32 at a time, lane k applying string c0 + k (the
    // matrix elements are complex128: one FP64 instruction covers 32
    // strings); then, for each nonzero off-diagonal string of the chunk, the
    // whole warp forms psi(s')/psi(s) over the hidden units.
    cpx<double> diagSum = mk(0.0, 0.0);
    cpx<double> acc = mk(0.0, 0.0);
    int16_t* fsRow = fsites + (size_t)warp * 32 * VMC_BF_MAX_LEN;
    for (int c0 = 0; c0 < op.num_ops; c0 += 32) {
      const int o = c0 + lane;
      bool valid = false;
      int nf = 0;
      cpx<double> m = mk(0.0, 0.0);
      if (o < op.num_ops) {
        bf_string_result r;
        bf_apply_string(op, o, cfg, occ, p.L, r);
        if ((isdiag[o >> 5] >> (o & 31)) & 1u) {
          diagSum = diagSum + r.m;
        } else if (sqrt(abs2(r.m)) > 1e-6) {  // _find_nonzero threshold (base.py:96)
          valid = true;
          m = r.m;
          for (int q = 0; q < r.nmod; ++q)
            if (r.val[q] != cfg[r.site[q]]) fsRow[lane * VMC_BF_MAX_LEN + nf++] = (int16_t)r.site[q];
        }
      }
      __syncwarp();
      unsigned vmask = __ballot_sync(0xffffffffu, valid);
      const int myNf = nf;
      cpx<T> myRatio = mk(T(1), T(0));
      while (vmask) {
        const int k = __ffs(vmask) - 1;
        vmask &= vmask - 1;
        const int nfk = __shfl_sync(0xffffffffu, myNf, k);
        if (nfk == 0) continue;  // flips cancel: psi(s') / psi(s) = 1
        const int16_t* fs = fsRow + k * VMC_BF_MAX_LEN;
        scaled_cpx<T> prod;
        prod.m = mk(T(1), T(0));
        prod.ex = 0;
        int cnt = 0;
        if (nfk == 1) {
          const int i = fs[0];
          const T sg = cfg[i] ? T(1) : T(-1);
          const cpx<T>* rc = tC + (size_t)i * p.M;
          const cpx<T>* rs = tS + (size_t)i * p.M;
          for (int j = lane; j < p.M; j += 32) {
            cpx<T> f = rc[j] - sg * (th[j] * rs[j]);
            prod.m = prod.m * f;
            if (++cnt == 8) {
              renorm(prod);
              cnt = 0;
            }
          }
        } else {
          for (int j = lane; j < p.M; j += 32) {
            cpx<T> e1 = mk(T(1), T(0)), e2 = mk(T(1), T(0));
            for (int q = 0; q < nfk; ++q) {
              const int i = fs[q];
              cpx<T> a = tEp[(size_t)i * p.M + j], b = tEm[(size_t)i * p.M + j];
              if (cfg[i]) {
                e1 = e1 * b;
                e2 = e2 * a;
              } else {
                e1 = e1 * a;
                e2 = e2 * b;
              }
            }
            cpx<T> t = th[j];
            cpx<T> onep = mk(T(1) + t.re, t.im), onem = mk(T(1) - t.re, -t.im);
            cpx<T> f = T(0.5) * (onep * e1 + onem * e2);
            prod.m = prod.m * f;
            if (++cnt == 8) {
              renorm(prod);
              cnt = 0;
            }
          }
        }
        renorm(prod);
        prod = warp_prod(prod);
        if (lane == k) myRatio = to_cpx(prod);
      }
      if (valid) acc = acc + m * mk((double)myRatio.re, (double)myRatio.im);
      __syncwarp();
    }
    acc = warp_sum(acc);
    diagSum = warp_sum(diagSum);
    if (op.num_diag > 0 && sqrt(abs2(diagSum)) > 1e-6) acc = acc + diagSum;
    if (logPsiS) {
      // O_loc = sum_k m_k psi(s'_k)/psi_net(s) * exp(log psi_net(s) - log psi_given(s))
      lpNet = warp_sum(lpNet);
      const double2 g = logPsiS[n];
      acc = acc * cexp_(mk((double)lpNet.re - g.x, (double)lpNet.im - g.y));
    }
    if (lane == 0) out[n] = make_double2(acc.re, acc.im);
    __syncwarp();
  }
}

// ------------------------------------------------------ gradient statistics
// Stage 1: tanh(theta) of every sample in FP64 (computed in T).
template <typename T>
__global__ void rbm_tanh_kernel(const int32_t* __restrict__ configs, int64_t N, rbm_params<T> p,
                                double2* __restrict__ tOut) {
  extern __shared__ unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cfgBytes = (p.L + 15) & ~15;
  cpx<T>* th = reinterpret_cast<cpx<T>*>(smem) + warp * p.M;
  int8_t* cfg = reinterpret_cast<int8_t*>(smem + (size_t)kWarpsPerBlock * p.M * sizeof(cpx<T>)) + warp * cfgBytes;
  for (int64_t n = (int64_t)blockIdx.x * kWarpsPerBlock + warp; n < N; n += (int64_t)gridDim.x * kWarpsPerBlock) {
    const int32_t* src = configs + n * p.L;
    for (int i = lane; i < p.L; i += 32) cfg[i] = (int8_t)src[i];
    __syncwarp();
    warp_theta(p, cfg, th, lane, true);
    for (int j = lane; j < p.M; j += 32) tOut[n * p.M + j] = make_double2(th[j].re, th[j].im);
    __syncwarp();
  }
}

constexpr int kStatSiteGroups = 8;
constexpr int kStatChunks = 32;

// Stage 2: partial sums over a chunk of samples of
//   mean rows : a_n * sigma_ni * t_nj            (a_n = w_n)
//   force rows: c_n * sigma_ni * conj(t_nj)      (c_n = w_n (E_n - Ebar))
// for the bias row (sigma = 1, row 0) and every site row (rows 1..L).
// blockDim = (32 hidden lanes, kStatSiteGroups); grid = (ceil(M/32), chunks).
// acoef (optional): complex per-sample coefficients a_n replacing w_n in the
// mean rows (used by the vector-Jacobian product with a_n = conj(g_n)).
__global__ void rbm_stats_partial_kernel(const int32_t* __restrict__ configs, const double2* __restrict__ tanhT,
                                         const double* __restrict__ w, const double2* __restrict__ eloc,
                                         const double2* __restrict__ emean, int64_t N, int L, int M,
                                         double2* __restrict__ partial /* (chunks, 2, L+1, M) */,
                                         double2* __restrict__ csum_partial /* (chunks) */,
                                         const double2* __restrict__ acoef) {
  const int lane = threadIdx.x, grp = threadIdx.y;
  const int j = blockIdx.x * 32 + lane;
  const int rows = L + 1;
  const int rowsPerGrp = (rows + kStatSiteGroups - 1) / kStatSiteGroups;
  const int r0 = grp * rowsPerGrp;
  const int64_t chunk = (N + gridDim.y - 1) / gridDim.y;
  const int64_t n0 = blockIdx.y * chunk;
  const int64_t n1 = min(N, n0 + chunk);
  const double2 em = eloc ? *emean : make_double2(0.0, 0.0);
  constexpr int RMAX = 12;  // rows per group held in registers per pass
  double2 cs = make_double2(0.0, 0.0);
  for (int rb = r0; rb < min(rows, r0 + rowsPerGrp); rb += RMAX) {
    const int re = min(min(rows, r0 + rowsPerGrp), rb + RMAX);
    double mre[RMAX], mim[RMAX], fre[RMAX], fim[RMAX];
#pragma unroll
    for (int q = 0; q < RMAX; ++q) mre[q] = mim[q] = fre[q] = fim[q] = 0.0;
    for (int64_t n = n0; n < n1; ++n) {
      const double a = acoef ? 0.0 : w[n];
      const double2 e = eloc ? eloc[n] : make_double2(0.0, 0.0);
      const double cr = a * (e.x - em.x), ci = a * (e.y - em.y);
      if (rb == r0 && grp == 0 && lane == 0 && blockIdx.x == 0) {
        cs.x += cr;
        cs.y += ci;
      }
      if (j >= M) continue;
      const double2 t = tanhT[n * M + j];
      double ar = a * t.x, ai = a * t.y;
      if (acoef) {
        const double2 z = acoef[n];
        ar = z.x * t.x - z.y * t.y;
        ai = z.x * t.y + z.y * t.x;
      }
      // c * conj(t)
      const double fr = cr * t.x + ci * t.y, fi = ci * t.x - cr * t.y;
      const int32_t* s = configs + n * L;
#pragma unroll
      for (int q = 0; q < RMAX; ++q) {
        const int row = rb + q;
        if (row < re) {
          const bool up = (row == 0) ? true : (s[row - 1] != 0);
          if (up) {
            mre[q] += ar; mim[q] += ai; fre[q] += fr; fim[q] += fi;
          } else {
            mre[q] -= ar; mim[q] -= ai; fre[q] -= fr; fim[q] -= fi;
          }
        }
      }
    }
    if (j < M) {
      double2* pm = partial + ((size_t)blockIdx.y * 2 * rows) * M;
      double2* pf = pm + (size_t)rows * M;
#pragma unroll
      for (int q = 0; q < RMAX; ++q) {
        const int row = rb + q;
        if (row < re) {
          pm[(size_t)row * M + j] = make_double2(mre[q], mim[q]);
          pf[(size_t)row * M + j] = make_double2(fre[q], fim[q]);
        }
      }
    }
  }
  if (grp == 0 && lane == 0 && blockIdx.x == 0) csum_partial[blockIdx.y] = cs;
}

// Stage 3: fixed-order sum of the chunk partials; force_k = Fraw_k - conj(mean_k) * sum_n c_n.
__global__ void rbm_stats_final_kernel(const double2* __restrict__ partial, const double2* __restrict__ csum_partial,
                                       int chunks, int L, int M, bool hasBias, double2* __restrict__ okMean,
                                       double2* __restrict__ force) {
  const int rows = L + 1;
  double2 cs = make_double2(0.0, 0.0);
  for (int c = 0; c < chunks; ++c) {
    cs.x += csum_partial[c].x;
    cs.y += csum_partial[c].y;
  }
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)rows * M;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int row = (int)(t / M);
    if (row == 0 && !hasBias) continue;
    double mr = 0, mi = 0, fr = 0, fi = 0;
    for (int c = 0; c < chunks; ++c) {
      const double2* pm = partial + ((size_t)c * 2 * rows) * M;
      const double2 a = pm[t];
      const double2 f = pm[(size_t)rows * M + t];
      mr += a.x; mi += a.y; fr += f.x; fi += f.y;
    }
    // conj(mean) * cs
    const double cr = mr * cs.x + mi * cs.y, ci = mr * cs.y - mi * cs.x;
    const int64_t k = hasBias ? t : t - M;
    okMean[k] = make_double2(mr, mi);
    force[k] = make_double2(fr - cr, fi - ci);
  }
}

int grid_for(int64_t N) {
  int64_t b = (N + kWarpsPerBlock - 1) / kWarpsPerBlock;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  return (int)b;
}

int check_rbm_args(const char* fn, int32_t precision, const int32_t* configs, int64_t N, int32_t L, int32_t M,
                   const void* kernel) {
  VMC_REQUIRE(precision == VMC_F64 || precision == VMC_F32, VMC_ERR_UNSUPPORTED, "%s: unknown precision %d", fn,
              precision);
  VMC_REQUIRE(N >= 0 && (configs || N == 0) && kernel, VMC_ERR_INVALID_ARGUMENT, "%s: null argument", fn);
  VMC_REQUIRE(L > 0 && L <= kMaxSites && M > 0 && M <= kMaxHidden, VMC_ERR_UNSUPPORTED,
              "%s: L=%d, M=%d outside [1,%d] x [1,%d]", fn, L, M, kMaxSites, kMaxHidden);
  return VMC_OK;
}

}  // namespace vmc

using namespace vmc;

extern "C" size_t vmc_rbm_tables_bytes(int32_t precision, int32_t num_sites, int32_t num_hidden) {
  size_t el = precision == VMC_F32 ? 8 : 16;
  return (5 * (size_t)num_sites * (size_t)num_hidden + (size_t)num_sites) * el;
}

extern "C" int vmc_rbm_prepare(int32_t precision, int32_t num_sites, int32_t num_hidden, const void* kernel,
                               void* tables, vmc_stream_t stream) {
  int rc = check_rbm_args("vmc_rbm_prepare", precision, nullptr, 0, num_sites, num_hidden, kernel);
  if (rc) return rc;
  VMC_REQUIRE(tables, VMC_ERR_INVALID_ARGUMENT, "vmc_rbm_prepare: null tables");
  int64_t n = (int64_t)num_sites * num_hidden;
  int blocks = (int)std::min<int64_t>((n + 255) / 256, 152 * 8);
  const int rowBlocks = (num_sites + 7) / 8;
  if (precision == VMC_F64) {
    cpx<double>* tab = reinterpret_cast<cpx<double>*>(tables);
    rbm_prepare_kernel<double><<<blocks, 256, 0, as_stream(stream)>>>(reinterpret_cast<const cpx<double>*>(kernel),
                                                                      n, tab);
    rbm_prepare_rows_kernel<double><<<rowBlocks, 256, 0, as_stream(stream)>>>(
        reinterpret_cast<const cpx<double>*>(kernel), num_sites, num_hidden, tab + 5 * n);
  } else {
    cpx<float>* tab = reinterpret_cast<cpx<float>*>(tables);
    rbm_prepare_kernel<float><<<blocks, 256, 0, as_stream(stream)>>>(reinterpret_cast<const cpx<float>*>(kernel), n,
                                                                    tab);
    rbm_prepare_rows_kernel<float><<<rowBlocks, 256, 0, as_stream(stream)>>>(
        reinterpret_cast<const cpx<float>*>(kernel), num_sites, num_hidden, tab + 5 * n);
  }
  return check_launch("vmc_rbm_prepare");
}

extern "C" int vmc_rbm_logpsi(int32_t precision, const int32_t* configs, int64_t num_configs, int32_t num_sites,
                              int32_t num_hidden, const void* kernel, const void* bias, double* log_psi,
                              vmc_stream_t stream) {
  int rc = check_rbm_args("vmc_rbm_logpsi", precision, configs, num_configs, num_sites, num_hidden, kernel);
  if (rc) return rc;
  VMC_REQUIRE(log_psi || num_configs == 0, VMC_ERR_INVALID_ARGUMENT, "vmc_rbm_logpsi: null output");
  if (num_configs == 0) return VMC_OK;
  size_t smem = (size_t)kWarpsPerBlock * ((num_sites + 15) & ~15);
  int grid = grid_for(num_configs);
  cudaStream_t st = as_stream(stream);
  if (precision == VMC_F64) {
    VMC_ALLOW_SMEM(rbm_logpsi_kernel<double>, smem, "vmc_rbm_logpsi");
    rbm_logpsi_kernel<double><<<grid, 32 * kWarpsPerBlock, smem, st>>>(
        configs, num_configs, make_params<double>(kernel, bias, num_sites, num_hidden),
        reinterpret_cast<double2*>(log_psi));
  } else {
    VMC_ALLOW_SMEM(rbm_logpsi_kernel<float>, smem, "vmc_rbm_logpsi");
    rbm_logpsi_kernel<float><<<grid, 32 * kWarpsPerBlock, smem, st>>>(
        configs, num_configs, make_params<float>(kernel, bias, num_sites, num_hidden),
        reinterpret_cast<double2*>(log_psi));
  }
  return check_launch("vmc_rbm_logpsi");
}

extern "C" int vmc_rbm_gradients(int32_t precision, const int32_t* configs, int64_t num_configs, int32_t num_sites,
                                 int32_t num_hidden, const void* kernel, const void* bias, int32_t layout, double* out,
                                 vmc_stream_t stream) {
  int rc = check_rbm_args("vmc_rbm_gradients", precision, configs, num_configs, num_sites, num_hidden, kernel);
  if (rc) return rc;
  VMC_REQUIRE(layout == VMC_GRAD_REFERENCE || layout == VMC_GRAD_COMPACT, VMC_ERR_INVALID_ARGUMENT,
              "vmc_rbm_gradients: unknown layout %d", layout);
  VMC_REQUIRE(out || num_configs == 0, VMC_ERR_INVALID_ARGUMENT, "vmc_rbm_gradients: null output");
  if (num_configs == 0) return VMC_OK;
  const size_t el = precision == VMC_F64 ? 16 : 8;
  size_t smem = (size_t)kWarpsPerBlock * (num_hidden * el + ((num_sites + 15) & ~15));
  VMC_REQUIRE(smem <= 227 * 1024, VMC_ERR_UNSUPPORTED, "vmc_rbm_gradients: M=%d too large", num_hidden);
  int grid = grid_for(num_configs);
  cudaStream_t st = as_stream(stream);
  if (precision == VMC_F64) {
    VMC_ALLOW_SMEM(rbm_grad_kernel<double>, smem, "vmc_rbm_gradients");
    rbm_grad_kernel<double><<<grid, 32 * kWarpsPerBlock, smem, st>>>(
        configs, num_configs, make_params<double>(kernel, bias, num_sites, num_hidden), layout,
        reinterpret_cast<double2*>(out));
  } else {
    VMC_ALLOW_SMEM(rbm_grad_kernel<float>, smem, "vmc_rbm_gradients");
    rbm_grad_kernel<float><<<grid, 32 * kWarpsPerBlock, smem, st>>>(
        configs, num_configs, make_params<float>(kernel, bias, num_sites, num_hidden), layout,
        reinterpret_cast<double2*>(out));
  }
  return check_launch("vmc_rbm_gradients");
}

extern "C" int vmc_rbm_oloc_fused(int32_t precision, const int32_t* configs, int64_t num_configs, int32_t num_sites,
                                  int32_t num_hidden, const void* kernel, const void* bias, const void* tables,
                                  const vmc_bf_operator* op, const double* log_psi_s, double* oloc,
                                  vmc_stream_t stream) {
  int rc = check_rbm_args("vmc_rbm_oloc_fused", precision, configs, num_configs, num_sites, num_hidden, kernel);
  if (rc) return rc;
  rc = check_op("vmc_rbm_oloc_fused", op, num_sites);
  if (rc) return rc;
  VMC_REQUIRE(op->local_dim == 2, VMC_ERR_UNSUPPORTED, "vmc_rbm_oloc_fused: local dimension %d (RBM needs 2)",
              op->local_dim);
  VMC_REQUIRE(tables && (oloc || num_configs == 0), VMC_ERR_INVALID_ARGUMENT, "vmc_rbm_oloc_fused: null argument");
  if (num_configs == 0) return VMC_OK;
  const size_t el = precision == VMC_F64 ? 16 : 8;
  const int nw = (num_sites + 31) >> 5;
  size_t perWarp = (size_t)num_hidden * el + (size_t)nw * 4 + ((num_sites + 15) & ~15);
  perWarp = (perWarp + 15) & ~(size_t)15;
  const size_t diagBytes = ((((op->num_ops + 31) >> 5) * 4) + 15) & ~15;
  size_t smem = diagBytes + kWarpsPerBlock * perWarp + (size_t)kWarpsPerBlock * 32 * VMC_BF_MAX_LEN * 2;
  VMC_REQUIRE(smem <= 227 * 1024, VMC_ERR_UNSUPPORTED, "vmc_rbm_oloc_fused: M=%d, %d strings too large", num_hidden,
              op->num_ops);
  int grid = grid_for(num_configs);
  cudaStream_t st = as_stream(stream);
  if (precision == VMC_F64) {
    VMC_ALLOW_SMEM(rbm_oloc_fused_kernel<double>, smem, "vmc_rbm_oloc_fused");
    rbm_oloc_fused_kernel<double><<<grid, 32 * kWarpsPerBlock, smem, st>>>(
        configs, num_configs, make_params<double>(kernel, bias, num_sites, num_hidden),
        reinterpret_cast<const cpx<double>*>(tables), *op, reinterpret_cast<const double2*>(log_psi_s),
        reinterpret_cast<double2*>(oloc));
  } else {
    VMC_ALLOW_SMEM(rbm_oloc_fused_kernel<float>, smem, "vmc_rbm_oloc_fused");
    rbm_oloc_fused_kernel<float><<<grid, 32 * kWarpsPerBlock, smem, st>>>(
        configs, num_configs, make_params<float>(kernel, bias, num_sites, num_hidden),
        reinterpret_cast<const cpx<float>*>(tables), *op, reinterpret_cast<const double2*>(log_psi_s),
        reinterpret_cast<double2*>(oloc));
  }
  return check_launch("vmc_rbm_oloc_fused");
}

extern "C" size_t vmc_rbm_grad_stats_workspace_bytes(int64_t num_configs, int32_t num_sites, int32_t num_hidden) {
  size_t tanhBytes = (size_t)num_configs * num_hidden * 16;
  size_t partBytes = (size_t)kStatChunks * 2 * (num_sites + 1) * (size_t)num_hidden * 16;
  return ((tanhBytes + 255) & ~(size_t)255) + ((partBytes + 255) & ~(size_t)255) + kStatChunks * 16 + 256;
}

extern "C" int vmc_rbm_grad_stats(int32_t precision, const int32_t* configs, int64_t num_configs, int32_t num_sites,
                                  int32_t num_hidden, const void* kernel, const void* bias, const double* weights,
                                  const double* eloc, const double* eloc_mean, double* ok_mean, double* force,
                                  void* workspace, size_t workspace_bytes, vmc_stream_t stream) {
  int rc = check_rbm_args("vmc_rbm_grad_stats", precision, configs, num_configs, num_sites, num_hidden, kernel);
  if (rc) return rc;
  VMC_REQUIRE(num_configs > 0 && weights && eloc && eloc_mean && ok_mean && force, VMC_ERR_INVALID_ARGUMENT,
              "vmc_rbm_grad_stats: null argument");
  size_t need = vmc_rbm_grad_stats_workspace_bytes(num_configs, num_sites, num_hidden);
  VMC_REQUIRE(workspace && workspace_bytes >= need, VMC_ERR_WORKSPACE, "vmc_rbm_grad_stats: workspace of %zu bytes needed",
              need);
  unsigned char* ws = reinterpret_cast<unsigned char*>(workspace);
  double2* tanhT = reinterpret_cast<double2*>(ws);
  size_t off = ((size_t)num_configs * num_hidden * 16 + 255) & ~(size_t)255;
  double2* partial = reinterpret_cast<double2*>(ws + off);
  off += (((size_t)kStatChunks * 2 * (num_sites + 1) * (size_t)num_hidden * 16) + 255) & ~(size_t)255;
  double2* csum = reinterpret_cast<double2*>(ws + off);

  cudaStream_t st = as_stream(stream);
  const size_t el = precision == VMC_F64 ? 16 : 8;
  size_t smem = (size_t)kWarpsPerBlock * (num_hidden * el + ((num_sites + 15) & ~15));
  VMC_REQUIRE(smem <= 227 * 1024, VMC_ERR_UNSUPPORTED, "vmc_rbm_grad_stats: M=%d too large", num_hidden);
  int grid = grid_for(num_configs);
  if (precision == VMC_F64) {
    VMC_ALLOW_SMEM(rbm_tanh_kernel<double>, smem, "vmc_rbm_grad_stats");
    rbm_tanh_kernel<double><<<grid, 32 * kWarpsPerBlock, smem, st>>>(
        configs, num_configs, make_params<double>(kernel, bias, num_sites, num_hidden), tanhT);
  } else {
    VMC_ALLOW_SMEM(rbm_tanh_kernel<float>, smem, "vmc_rbm_grad_stats");
    rbm_tanh_kernel<float><<<grid, 32 * kWarpsPerBlock, smem, st>>>(
        configs, num_configs, make_params<float>(kernel, bias, num_sites, num_hidden), tanhT);
  }
  rc = check_launch("vmc_rbm_grad_stats(tanh)");
  if (rc) return rc;
  dim3 blk(32, kStatSiteGroups);
  dim3 grd((num_hidden + 31) / 32, kStatChunks);
  rbm_stats_partial_kernel<<<grd, blk, 0, st>>>(configs, tanhT, weights, reinterpret_cast<const double2*>(eloc),
                                                reinterpret_cast<const double2*>(eloc_mean), num_configs, num_sites,
                                                num_hidden, partial, csum, nullptr);
  rc = check_launch("vmc_rbm_grad_stats(partial)");
  if (rc) return rc;
  int64_t outs = (int64_t)(num_sites + 1) * num_hidden;
  int fb = (int)std::min<int64_t>((outs + 255) / 256, 152 * 4);
  rbm_stats_final_kernel<<<fb, 256, 0, st>>>(partial, csum, kStatChunks, num_sites, num_hidden, bias != nullptr,
                                             reinterpret_cast<double2*>(ok_mean), reinterpret_cast<double2*>(force));
  return check_launch("vmc_rbm_grad_stats(final)");
}

// ===================================================================
// Metropolis sampling of |psi|^mu for a CpxRBM (sampler.py:264-367).
// One warp per Markov chain; the chain's configuration lives in shared
// memory, theta_j and tanh(theta_j) of the lane's JPL hidden units in
// registers.  A proposal flips one site i (propose_spin_flip,
// sampler.py:15-19) and is accepted iff u < |psi(s')/psi(s)|^mu with
//   |psi(s')/psi(s)|^2 = prod_j |cosh(2W_ij) - sigma_i tanh(theta_j) sinh(2W_ij)|^2
// (no network re-evaluation), evaluated as |prod_j cosh 2W_ij|^2
// prod_j |1 - sigma_i tanh(theta_j) tanh(2W_ij)|^2 from the tanh(2W) table
// and the row sums of log cosh 2W.  On acceptance theta_j -= 2 sigma_i W_ij.
// Site and u come from the Philox stream metropolis_draw(seed, call, step,
// chain); steps are numbered from 0 within one call.
// ===================================================================
namespace vmc {

template <typename T, int JPL>
__global__ void __launch_bounds__(256) rbm_metropolis_kernel(
    int32_t* __restrict__ states, int C, rbm_params<T> p, const cpx<T>* __restrict__ tab, double mu, uint64_t seed,
    uint32_t callArg, const uint32_t* __restrict__ callPtr, int64_t thermSteps, int64_t sweepSteps,
    int64_t samplesPerChain, int32_t* __restrict__ configsOut, unsigned long long* __restrict__ counters) {
  extern __shared__ unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int chain = blockIdx.x * (blockDim.x >> 5) + warp;
  if (chain >= C) return;  // whole warps exit together
  const uint32_t call = callPtr ? *callPtr : callArg;
  const int L = p.L, M = p.M;
  int8_t* cfg = reinterpret_cast<int8_t*>(smem) + warp * ((L + 15) & ~15);
  int32_t* st = states + (size_t)chain * L;
  for (int i = lane; i < L; i += 32) cfg[i] = (int8_t)st[i];
  __syncwarp();

  cpx<T> th[JPL], tn[JPL];
#pragma unroll
  for (int q = 0; q < JPL; ++q) {
    const int j = lane + 32 * q;
    cpx<T> t = mk(T(0), T(0));
    if (j < M) {
      if (p.b) t = p.b[j];
      for (int i = 0; i < L; ++i) {
        cpx<T> x = p.W[(size_t)i * M + j];
        if (cfg[i]) {
          t.re += x.re;
          t.im += x.im;
        } else {
          t.re -= x.re;
          t.im -= x.im;
        }
      }
    }
    th[q] = t;
    tn[q] = ctanh_(t);
  }
  const size_t LM = (size_t)L * M;
  // cosh(theta + D)/cosh(theta) = cosh 2W (1 - s tanh(theta) tanh 2W): one
  // tanh(2W) row per proposal, the row's |prod_j cosh 2W|^2 =
  // exp(2 Re rowLogC) added to the log-ratio
  const cpx<T>* tT = tab + 4 * LM;
  const cpx<T>* rowLogC = tab + 5 * LM;
  const T halfMu = T(0.5 * mu);
  unsigned long long accepted = 0;
  const int64_t total = thermSteps + sweepSteps * samplesPerChain;
  // the flip site does not depend on the chain state: the next step's table
  // row is loaded while the current step is evaluated
  mc_draw d = metropolis_draw(seed, call, 0u, (uint32_t)chain, L);
  cpx<T> fT[JPL];
  T rowRe = rowLogC[d.site].re;
#pragma unroll
  for (int q = 0; q < JPL; ++q) {
    const int j = lane + 32 * q;
    fT[q] = j < M ? tT[(size_t)d.site * M + j] : mk(T(0), T(0));
  }
  for (int64_t step = 0; step < total; ++step) {
    const int i = d.site;
    const mc_draw dn = metropolis_draw(seed, call, (uint32_t)(step + 1), (uint32_t)chain, L);
    cpx<T> nT[JPL];
    const T nRowRe = rowLogC[dn.site].re;
#pragma unroll
    for (int q = 0; q < JPL; ++q) {
      const int j = lane + 32 * q;
      nT[q] = j < M ? tT[(size_t)dn.site * M + j] : mk(T(0), T(0));
    }
    const T sg = cfg[i] ? T(1) : T(-1);
    // |ratio / prod_j cosh 2W_ij|^2 over this lane's hidden units, as mantissa * 2^ex
    T prod = T(1);
    int ex = 0;
#pragma unroll
    for (int q = 0; q < JPL; ++q) {
      const int j = lane + 32 * q;
      if (j < M) {
        const cpx<T> g = tn[q] * fT[q];
        prod *= abs2(mk(T(1) - sg * g.re, -sg * g.im));
        if ((q & 3) == 3) {
          int e = exponent_of(prod);
          if (prod != T(0) && isfinite(prod)) {
            prod = ldexp(prod, -e);
            ex += e;
          }
        }
      }
    }
    {
      int e = exponent_of(prod);
      if (prod != T(0) && isfinite(prod)) {
        prod = ldexp(prod, -e);
        ex += e;
      }
    }
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) {
      T op = __shfl_xor_sync(0xffffffffu, prod, m);
      int oe = __shfl_xor_sync(0xffffffffu, ex, m);
      prod *= op;
      ex += oe;
      int e = exponent_of(prod);
      if (prod != T(0) && isfinite(prod)) {
        prod = ldexp(prod, -e);
        ex += e;
      }
    }
    // one decision for the whole warp: lane 0's value
    prod = __shfl_sync(0xffffffffu, prod, 0);
    ex = __shfl_sync(0xffffffffu, ex, 0);
    bool acc;
    if (sizeof(T) == sizeof(double)) {
      // P = |ratio|^mu = (prod * 2^ex * exp(2 Re rowLogC))^(mu/2); accept iff
      // u < P (bernoulli, sampler.py:339-340)
      const double logr2 = log((double)prod) + (double)ex * 0.69314718055994530942 + 2.0 * (double)rowRe;
      const double P = exp((double)halfMu * logr2);
      acc = d.u64() < P;
    } else {
      const float lg2 = log2f((float)prod) + (float)ex + 2.8853900817779268f * (float)rowRe;
      const float P = exp2f((float)halfMu * lg2);
      acc = d.u32() < P;
    }
    if (acc) {
#pragma unroll
      for (int q = 0; q < JPL; ++q) {
        const int j = lane + 32 * q;
        if (j < M) {
          cpx<T> w = p.W[(size_t)i * M + j];
          th[q] = th[q] - (T(2) * sg) * w;
          tn[q] = ctanh_(th[q]);
        }
      }
      __syncwarp();
      if (lane == 0) cfg[i] = cfg[i] ? 0 : 1;
      __syncwarp();
      ++accepted;
    }
#pragma unroll
    for (int q = 0; q < JPL; ++q) fT[q] = nT[q];
    rowRe = nRowRe;
    d = dn;
    if (step >= thermSteps && ((step - thermSteps + 1) % sweepSteps) == 0) {
      const int64_t s = (step - thermSteps + 1) / sweepSteps - 1;
      int32_t* out = configsOut + ((size_t)s * C + chain) * L;
      for (int k = lane; k < L; k += 32) out[k] = cfg[k];
    }
  }
  __syncwarp();
  for (int k = lane; k < L; k += 32) st[k] = cfg[k];
  if (lane == 0) {
    atomicAdd(&counters[0], (unsigned long long)total);
    atomicAdd(&counters[1], accepted);
  }
}

template <typename T, int JPL>
int launch_metropolis(int32_t* states, int C, rbm_params<T> p, const void* tables, double mu, uint64_t seed,
                      uint32_t call, const uint32_t* callPtr, int64_t therm, int64_t sweep, int64_t spc,
                      int32_t* out, void* counters, cudaStream_t st) {
  const int warps = 4;
  const size_t smem = (size_t)warps * ((p.L + 15) & ~15);
  const int grid = (C + warps - 1) / warps;
  rbm_metropolis_kernel<T, JPL><<<grid, 32 * warps, smem, st>>>(
      states, C, p, reinterpret_cast<const cpx<T>*>(tables), mu, seed, call, callPtr, therm, sweep, spc, out,
      reinterpret_cast<unsigned long long*>(counters));
  return check_launch("vmc_rbm_metropolis");
}

template <typename T>
int dispatch_metropolis(int32_t* states, int C, rbm_params<T> p, const void* tables, double mu, uint64_t seed,
                        uint32_t call, const uint32_t* cp, int64_t therm, int64_t sweep, int64_t spc, int32_t* out,
                        void* counters, cudaStream_t st) {
  const int jpl = (p.M + 31) / 32;
  if (jpl <= 1) return launch_metropolis<T, 1>(states, C, p, tables, mu, seed, call, cp, therm, sweep, spc, out, counters, st);
  if (jpl <= 2) return launch_metropolis<T, 2>(states, C, p, tables, mu, seed, call, cp, therm, sweep, spc, out, counters, st);
  if (jpl <= 4) return launch_metropolis<T, 4>(states, C, p, tables, mu, seed, call, cp, therm, sweep, spc, out, counters, st);
  if (jpl <= 8) return launch_metropolis<T, 8>(states, C, p, tables, mu, seed, call, cp, therm, sweep, spc, out, counters, st);
  if (jpl <= 16) return launch_metropolis<T, 16>(states, C, p, tables, mu, seed, call, cp, therm, sweep, spc, out, counters, st);
  return launch_metropolis<T, 32>(states, C, p, tables, mu, seed, call, cp, therm, sweep, spc, out, counters, st);
}

// call index read from device memory and advanced by the same stream:
// replaying a captured graph draws fresh random numbers every time
__global__ void counter_add_kernel(uint32_t* c, uint32_t v) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *c += v;
}

}  // namespace vmc

extern "C" int vmc_rbm_metropolis(int32_t precision, int32_t* states, int32_t num_chains, int32_t num_sites,
                                  int32_t num_hidden, const void* kernel, const void* bias, const void* tables,
                                  double mu, uint64_t seed, uint32_t call_index, int64_t therm_steps,
                                  int64_t sweep_steps, int64_t samples_per_chain, int32_t* configs_out,
                                  void* counters, vmc_stream_t stream) {
  int rc = check_rbm_args("vmc_rbm_metropolis", precision, states, num_chains, num_sites, num_hidden, kernel);
  if (rc) return rc;
  VMC_REQUIRE(num_hidden <= 1024, VMC_ERR_UNSUPPORTED, "vmc_rbm_metropolis: M=%d > 1024", num_hidden);
  VMC_REQUIRE(num_chains > 0 && tables && counters && sweep_steps > 0 && therm_steps >= 0 && samples_per_chain >= 0,
              VMC_ERR_INVALID_ARGUMENT, "vmc_rbm_metropolis: bad arguments");
  VMC_REQUIRE(configs_out || samples_per_chain == 0, VMC_ERR_INVALID_ARGUMENT, "vmc_rbm_metropolis: null output");
  VMC_REQUIRE(therm_steps + sweep_steps * samples_per_chain < (int64_t)0xFFFFFFFF, VMC_ERR_UNSUPPORTED,
              "vmc_rbm_metropolis: more than 2^32 steps in one call");
  VMC_REQUIRE(mu >= 0.0 && mu <= 2.0, VMC_ERR_INVALID_ARGUMENT, "vmc_rbm_metropolis: mu=%g outside [0, 2]", mu);
  cudaStream_t st = as_stream(stream);
  if (precision == VMC_F64)
    return dispatch_metropolis<double>(states, num_chains, make_params<double>(kernel, bias, num_sites, num_hidden),
                                       tables, mu, seed, call_index, nullptr, therm_steps, sweep_steps,
                                       samples_per_chain, configs_out, counters, st);
  return dispatch_metropolis<float>(states, num_chains, make_params<float>(kernel, bias, num_sites, num_hidden), tables,
                                    mu, seed, call_index, nullptr, therm_steps, sweep_steps, samples_per_chain,
                                    configs_out, counters, st);
}

extern "C" int vmc_rbm_metropolis_devcall(int32_t precision, int32_t* states, int32_t num_chains, int32_t num_sites,
                                          int32_t num_hidden, const void* kernel, const void* bias,
                                          const void* tables, double mu, uint64_t seed, uint32_t* call_index,
                                          int64_t therm_steps, int64_t sweep_steps, int64_t samples_per_chain,
                                          int32_t* configs_out, void* counters, vmc_stream_t stream) {
  int rc = check_rbm_args("vmc_rbm_metropolis_devcall", precision, states, num_chains, num_sites, num_hidden, kernel);
  if (rc) return rc;
  VMC_REQUIRE(num_hidden <= 1024, VMC_ERR_UNSUPPORTED, "vmc_rbm_metropolis_devcall: M=%d > 1024", num_hidden);
  VMC_REQUIRE(num_chains > 0 && tables && counters && call_index && sweep_steps > 0 && therm_steps >= 0 &&
                  samples_per_chain >= 0 && (configs_out || samples_per_chain == 0),
              VMC_ERR_INVALID_ARGUMENT, "vmc_rbm_metropolis_devcall: bad arguments");
  VMC_REQUIRE(therm_steps + sweep_steps * samples_per_chain < (int64_t)0xFFFFFFFF, VMC_ERR_UNSUPPORTED,
              "vmc_rbm_metropolis_devcall: more than 2^32 steps in one call");
  VMC_REQUIRE(mu >= 0.0 && mu <= 2.0, VMC_ERR_INVALID_ARGUMENT, "vmc_rbm_metropolis_devcall: mu=%g", mu);
  cudaStream_t st = as_stream(stream);
  if (precision == VMC_F64)
    rc = dispatch_metropolis<double>(states, num_chains, make_params<double>(kernel, bias, num_sites, num_hidden),
                                     tables, mu, seed, 0u, call_index, therm_steps, sweep_steps, samples_per_chain,
                                     configs_out, counters, st);
  else
    rc = dispatch_metropolis<float>(states, num_chains, make_params<float>(kernel, bias, num_sites, num_hidden), tables,
                                    mu, seed, 0u, call_index, therm_steps, sweep_steps, samples_per_chain, configs_out,
                                    counters, st);
  if (rc) return rc;
  counter_add_kernel<<<1, 32, 0, st>>>(call_index, 1u);
  return check_launch("vmc_rbm_metropolis_devcall(counter)");
}

namespace vmc {
__global__ void conj_kernel(const double2* __restrict__ g, int64_t n, double2* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = make_double2(g[i].x, -g[i].y);
}

__global__ void vjp_final_kernel(const double2* __restrict__ partial, int chunks, int L, int M, bool hasBias,
                                 double2* __restrict__ out) {
  const int rows = L + 1;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)rows * M;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int row = (int)(t / M);
    if (row == 0 && !hasBias) continue;
    double re = 0, im = 0;
    for (int c = 0; c < chunks; ++c) {
      const double2 a = partial[((size_t)c * 2 * rows) * M + t];
      re += a.x;
      im += a.y;
    }
    out[hasBias ? t : t - M] = make_double2(re, im);
  }
}
}  // namespace vmc

extern "C" size_t vmc_rbm_vjp_workspace_bytes(int64_t num_configs, int32_t num_sites, int32_t num_hidden) {
  return vmc_rbm_grad_stats_workspace_bytes(num_configs, num_sites, num_hidden) + (size_t)num_configs * 16 + 256;
}

extern "C" int vmc_rbm_vjp(int32_t precision, const int32_t* configs, int64_t num_configs, int32_t num_sites,
                           int32_t num_hidden, const void* kernel, const void* bias, const double* cotangent,
                           double* out, void* workspace, size_t workspace_bytes, vmc_stream_t stream) {
  int rc = check_rbm_args("vmc_rbm_vjp", precision, configs, num_configs, num_sites, num_hidden, kernel);
  if (rc) return rc;
  VMC_REQUIRE(num_configs > 0 && cotangent && out, VMC_ERR_INVALID_ARGUMENT, "vmc_rbm_vjp: null argument");
  const size_t need = vmc_rbm_vjp_workspace_bytes(num_configs, num_sites, num_hidden);
  VMC_REQUIRE(workspace && workspace_bytes >= need, VMC_ERR_WORKSPACE, "vmc_rbm_vjp: workspace of %zu bytes needed",
              need);
  unsigned char* ws = reinterpret_cast<unsigned char*>(workspace);
  double2* tanhT = reinterpret_cast<double2*>(ws);
  size_t off = ((size_t)num_configs * num_hidden * 16 + 255) & ~(size_t)255;
  double2* partial = reinterpret_cast<double2*>(ws + off);
  off += (((size_t)kStatChunks * 2 * (num_sites + 1) * (size_t)num_hidden * 16) + 255) & ~(size_t)255;
  double2* csum = reinterpret_cast<double2*>(ws + off);
  off += ((size_t)kStatChunks * 16 + 255) & ~(size_t)255;
  double2* coef = reinterpret_cast<double2*>(ws + off);
  cudaStream_t st = as_stream(stream);
  const size_t el = precision == VMC_F64 ? 16 : 8;
  size_t smem = (size_t)kWarpsPerBlock * (num_hidden * el + ((num_sites + 15) & ~15));
  VMC_REQUIRE(smem <= 227 * 1024, VMC_ERR_UNSUPPORTED, "vmc_rbm_vjp: M=%d too large", num_hidden);
  int grid = grid_for(num_configs);
  if (precision == VMC_F64) {
    VMC_ALLOW_SMEM(rbm_tanh_kernel<double>, smem, "vmc_rbm_vjp");
    rbm_tanh_kernel<double><<<grid, 32 * kWarpsPerBlock, smem, st>>>(
        configs, num_configs, make_params<double>(kernel, bias, num_sites, num_hidden), tanhT);
  } else {
    VMC_ALLOW_SMEM(rbm_tanh_kernel<float>, smem, "vmc_rbm_vjp");
    rbm_tanh_kernel<float><<<grid, 32 * kWarpsPerBlock, smem, st>>>(
        configs, num_configs, make_params<float>(kernel, bias, num_sites, num_hidden), tanhT);
  }
  rc = check_launch("vmc_rbm_vjp(tanh)");
  if (rc) return rc;
  conj_kernel<<<(int)std::min<int64_t>((num_configs + 255) / 256, 1024), 256, 0, st>>>(
      reinterpret_cast<const double2*>(cotangent), num_configs, coef);
  dim3 blk(32, kStatSiteGroups);
  dim3 grd((num_hidden + 31) / 32, kStatChunks);
  rbm_stats_partial_kernel<<<grd, blk, 0, st>>>(configs, tanhT, nullptr, nullptr, nullptr, num_configs, num_sites,
                                                num_hidden, partial, csum, coef);
  rc = check_launch("vmc_rbm_vjp(partial)");
  if (rc) return rc;
  int64_t outs = (int64_t)(num_sites + 1) * num_hidden;
  vjp_final_kernel<<<(int)std::min<int64_t>((outs + 255) / 256, 152 * 4), 256, 0, st>>>(
      partial, kStatChunks, num_sites, num_hidden, bias != nullptr, reinterpret_cast<double2*>(out));
  return check_launch("vmc_rbm_vjp(final)");
}

// ===================================================================
// Allocation-free variant of vmc_rbm_grad_stats.
//
// Some callers cannot call cudaMalloc at the point where they need the
// statistics: a JAX/XLA FFI handler or an inference runtime that owns a
// fixed memory budget, or code running while a stream is being captured
// into a CUDA graph.  This entry point takes the scratch memory of
// vmc_rbm_grad_stats from a file-scope device array instead of a caller
// workspace.  The array (kNoAllocScratchBytes) is part of the library's
// static device memory: every GPU that loads the library holds it until the
// process exits.
// ===================================================================
namespace vmc {

constexpr size_t kNoAllocScratchBytes = 32u << 20;  // 32 MiB per device
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

}  // namespace vmc

#include <mutex>

extern "C" int vmc_rbm_grad_stats_noalloc(int32_t precision, const int32_t* configs, int64_t num_configs,
                                          int32_t num_sites, int32_t num_hidden, const void* kernel, const void* bias,
                                          const double* weights, const double* eloc, const double* eloc_mean,
                                          double* ok_mean, double* force, vmc_stream_t stream) {
  int rc = check_rbm_args("vmc_rbm_grad_stats_noalloc", precision, configs, num_configs, num_sites, num_hidden,
                          kernel);
  if (rc) return rc;
  const size_t need = vmc_rbm_grad_stats_workspace_bytes(num_configs, num_sites, num_hidden);
  VMC_REQUIRE(need <= kNoAllocScratchBytes, VMC_ERR_UNSUPPORTED,
              "vmc_rbm_grad_stats_noalloc: needs %zu bytes of scratch, the static scratch holds %zu "
              "(num_configs * num_hidden * 16 + 1024 * (num_sites + 1) * num_hidden bytes must fit); use "
              "vmc_rbm_grad_stats with a caller workspace",
              need, kNoAllocScratchBytes);
  // Device address of the scratch array, resolved once per device with that
  // device current (host code sees only a stand-in for the symbol).
  static std::mutex mu;
  static void* addr[64] = {nullptr};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  VMC_REQUIRE(e == cudaSuccess && dev >= 0 && dev < 64, VMC_ERR_CUDA, "vmc_rbm_grad_stats_noalloc: %s",
              cudaGetErrorString(e));
  void* scratch;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      VMC_REQUIRE(e == cudaSuccess && p, VMC_ERR_CUDA, "vmc_rbm_grad_stats_noalloc: cudaGetSymbolAddress: %s",
                  cudaGetErrorString(e));
      addr[dev] = p;
    }
    scratch = addr[dev];
  }
  // Every buffer in the scratch is written before it is read (tanh values,
  // per-chunk partial sums), so nothing has to start at zero.
  return vmc_rbm_grad_stats(precision, configs, num_configs, num_sites, num_hidden, kernel, bias, weights, eloc,
                            eloc_mean, ok_mean, force, scratch, kNoAllocScratchBytes, stream);
}
