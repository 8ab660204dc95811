// Real CNN ansatz (nets/cnn.py:18-83): periodic (wrap) padding (0, F-1),
// VALID cross-correlation with HWIO kernels, unit strides, bias per layer,
// polynomial activation after every layer, output sum / sqrt(#elements).
//
// One warp per configuration.  The forward pass keeps every layer's
// pre-activations of that configuration in shared memory; the backward
// kernel (d log psi / d theta, flat_gradient of vqs.py:46-51) recomputes
// them instead of storing activations per sample in HBM.
#include <algorithm>

#include "vmc_common.cuh"

namespace vmc {

constexpr int kCnnMaxLayers = 4;

struct cnn_geom {
  int nd, H, W, FH, FW, layers;
  int ch[kCnnMaxLayers];
  int act[kCnnMaxLayers];
  int bias[kCnnMaxLayers];
  int kOff[kCnnMaxLayers];  // offset of layer kernel in the flat parameter vector
  int bOff[kCnnMaxLayers];  // offset of layer bias (or -1)
  int P;                    // number of parameters
  int sites;
  int maxC;
};

template <typename T>
__device__ __forceinline__ T act_f(int code, T x) {
  T x2 = x * x;
  switch (code) {
    case 0: return T(0.5) * x2 - x2 * x2 / T(12);                                        // x^2/2 - x^4/12
    case 1: return ((T(0.022222222) * x2 - T(0.083333333)) * x2 + T(0.5)) * x2;          // poly6
    case 2: return x2;                                                                   // square
    default: return ((T(0.133333333) * x2 - T(0.333333333)) * x2 + T(1)) * x;            // poly5
  }
}

template <typename T>
__device__ __forceinline__ T act_d(int code, T x) {
  T x2 = x * x;
  switch (code) {
    case 0: return x - x2 * x / T(3);
    case 1: return ((T(6) * T(0.022222222) * x2 - T(4) * T(0.083333333)) * x2 + T(1)) * x;
    case 2: return T(2) * x;
    default: return (T(5) * T(0.133333333) * x2 - T(3) * T(0.333333333)) * x2 + T(1);
  }
}

// z_l[p][c] = b[c] + sum_{dy,dx,ci} a_{l-1}[(y+dy)%H][(x+dx)%W][ci] K[dy][dx][ci][c]
// (cross-correlation of the wrap-padded input; output site p = y*W + x).
template <typename T>
__device__ void warp_forward(const cnn_geom& g, const T* __restrict__ prm, const int8_t* cfg, T* z, int lane) {
  // z holds layers back to back: layer l at z + l * sites * maxC
  const int S = g.sites;
  for (int l = 0; l < g.layers; ++l) {
    const int cin = l == 0 ? 1 : g.ch[l - 1], cout = g.ch[l];
    const T* K = prm + g.kOff[l];
    const T* zin = z + (size_t)(l - 1) * S * g.maxC;
    T* zo = z + (size_t)l * S * g.maxC;
    const int aprev = l == 0 ? 0 : g.act[l - 1];
    for (int o = lane; o < S * cout; o += 32) {
      const int p = o / cout, c = o - (o / cout) * cout;
      const int y = p / g.W, x = p - (p / g.W) * g.W;
      T acc = g.bOff[l] >= 0 ? prm[g.bOff[l] + c] : T(0);
      for (int dy = 0; dy < g.FH; ++dy) {
        int yy = y + dy;
        if (yy >= g.H) yy -= g.H;
        for (int dx = 0; dx < g.FW; ++dx) {
          int xx = x + dx;
          if (xx >= g.W) xx -= g.W;
          const int q = yy * g.W + xx;
          const T* kk = K + ((size_t)(dy * g.FW + dx) * cin) * cout + c;
          if (l == 0) {
            acc += (cfg[q] ? T(1) : T(-1)) * kk[0];
          } else {
            for (int ci = 0; ci < cin; ++ci) acc += act_f(aprev, zin[(size_t)q * g.maxC + ci]) * kk[(size_t)ci * cout];
          }
        }
      }
      zo[(size_t)p * g.maxC + c] = acc;
    }
    __syncwarp();
  }
}

template <typename T>
__device__ T warp_output(const cnn_geom& g, const T* z, int lane) {
  const int l = g.layers - 1, cout = g.ch[l];
  const T* zl = z + (size_t)l * g.sites * g.maxC;
  T s = T(0);
  for (int o = lane; o < g.sites * cout; o += 32) {
    const int p = o / cout, c = o - (o / cout) * cout;
    s += act_f(g.act[l], zl[(size_t)p * g.maxC + c]);
  }
  s = warp_sum(s);
  return s / sqrt(T(g.sites * cout));
}

template <typename T>
__global__ void cnn_logpsi_kernel(const int32_t* __restrict__ configs, int64_t N, cnn_geom g, const T* __restrict__ prm,
                                  int warps, double2* __restrict__ out) {
  extern __shared__ unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t zBytes = (size_t)g.layers * g.sites * g.maxC * sizeof(T);
  const size_t per = (zBytes + g.sites + 15) & ~(size_t)15;
  T* z = reinterpret_cast<T*>(smem + warp * per);
  int8_t* cfg = reinterpret_cast<int8_t*>(smem + warp * per + zBytes);
  for (int64_t n = (int64_t)blockIdx.x * warps + warp; n < N; n += (int64_t)gridDim.x * warps) {
    for (int i = lane; i < g.sites; i += 32) cfg[i] = (int8_t)configs[n * g.sites + i];
    __syncwarp();
    warp_forward(g, prm, cfg, z, lane);
    T v = warp_output(g, z, lane);
    if (lane == 0) out[n] = make_double2((double)v, 0.0);
    __syncwarp();
  }
}

// Backward pass of one configuration: writes d log psi / d theta (P values)
// through the callback-free form `grad[k]`.
template <typename T>
__device__ void warp_backward(const cnn_geom& g, const T* __restrict__ prm, const int8_t* cfg, const T* z, T* da,
                              T* db, double* grad, int gs, int lane) {
  const int S = g.sites;
  const int lastC = g.ch[g.layers - 1];
  const T inv = T(1) / sqrt(T(S * lastC));
  // da <- d out / d a_last = 1/nrm
  for (int o = lane; o < S * lastC; o += 32) {
    const int p = o / lastC, c = o - (o / lastC) * lastC;
    da[(size_t)p * g.maxC + c] = inv;
  }
  __syncwarp();
  for (int l = g.layers - 1; l >= 0; --l) {
    const int cin = l == 0 ? 1 : g.ch[l - 1], cout = g.ch[l];
    const T* zl = z + (size_t)l * S * g.maxC;
    const T* zin = z + (size_t)(l - 1) * S * g.maxC;
    const int aprev = l == 0 ? 0 : g.act[l - 1];
    // dz = da * act'(z)  (in place in da)
    for (int o = lane; o < S * cout; o += 32) {
      const int p = o / cout, c = o - (o / cout) * cout;
      da[(size_t)p * g.maxC + c] *= act_d(g.act[l], zl[(size_t)p * g.maxC + c]);
    }
    __syncwarp();
    if (g.bOff[l] >= 0) {
      for (int c = lane; c < cout; c += 32) {
        T s = T(0);
        for (int p = 0; p < S; ++p) s += da[(size_t)p * g.maxC + c];
        grad[(size_t)(g.bOff[l] + c) * gs] = (double)s;
      }
    }
    // dK[dy][dx][ci][c] = sum_p a_prev[p + off][ci] dz[p][c]
    const int nk = g.FH * g.FW * cin * cout;
    for (int e = lane; e < nk; e += 32) {
      const int c = e % cout;
      const int ci = (e / cout) % cin;
      const int off = e / (cout * cin);
      const int dy = off / g.FW, dx = off - (off / g.FW) * g.FW;
      T s = T(0);
      for (int p = 0; p < S; ++p) {
        const int y = p / g.W, x = p - (p / g.W) * g.W;
        int yy = y + dy, xx = x + dx;
        if (yy >= g.H) yy -= g.H;
        if (xx >= g.W) xx -= g.W;
        const int q = yy * g.W + xx;
        const T a = l == 0 ? (cfg[q] ? T(1) : T(-1)) : act_f(aprev, zin[(size_t)q * g.maxC + ci]);
        s += a * da[(size_t)p * g.maxC + c];
      }
      grad[(size_t)(g.kOff[l] + e) * gs] = (double)s;
    }
    if (l > 0) {
      // da_prev[q][ci] = act-input gradient: sum_{off, c} dz[q - off][c] K[off][ci][c]
      const T* K = prm + g.kOff[l];
      for (int o = lane; o < S * cin; o += 32) {
        const int q = o / cin, ci = o - (o / cin) * cin;
        const int y = q / g.W, x = q - (q / g.W) * g.W;
        T s = T(0);
        for (int dy = 0; dy < g.FH; ++dy) {
          int yy = y - dy;
          if (yy < 0) yy += g.H;
          for (int dx = 0; dx < g.FW; ++dx) {
            int xx = x - dx;
            if (xx < 0) xx += g.W;
            const int p = yy * g.W + xx;
            const T* kk = K + ((size_t)(dy * g.FW + dx) * cin + ci) * cout;
            for (int c = 0; c < cout; ++c) s += da[(size_t)p * g.maxC + c] * kk[c];
          }
        }
        db[(size_t)q * g.maxC + ci] = s;
      }
      __syncwarp();
      for (int o = lane; o < S * cin; o += 32) {
        const int q = o / cin, ci = o - (o / cin) * cin;
        da[(size_t)q * g.maxC + ci] = db[(size_t)q * g.maxC + ci];
      }
    }
    __syncwarp();
  }
}

template <typename T>
__global__ void cnn_grad_kernel(const int32_t* __restrict__ configs, int64_t N, cnn_geom g, const T* __restrict__ prm,
                                int warps, int layout, double* __restrict__ out) {
  extern __shared__ unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t zBytes = (size_t)g.layers * g.sites * g.maxC * sizeof(T);
  const size_t dBytes = (size_t)g.sites * g.maxC * sizeof(T);
  const size_t per = (zBytes + 2 * dBytes + g.sites + 15) & ~(size_t)15;
  unsigned char* base = smem + warp * per;
  T* z = reinterpret_cast<T*>(base);
  T* da = reinterpret_cast<T*>(base + zBytes);
  T* db = reinterpret_cast<T*>(base + zBytes + dBytes);
  int8_t* cfg = reinterpret_cast<int8_t*>(base + zBytes + 2 * dBytes);
  for (int64_t n = (int64_t)blockIdx.x * warps + warp; n < N; n += (int64_t)gridDim.x * warps) {
    for (int i = lane; i < g.sites; i += 32) cfg[i] = (int8_t)configs[n * g.sites + i];
    __syncwarp();
    warp_forward(g, prm, cfg, z, lane);
    if (layout == VMC_GRAD_REFERENCE) {
      // (N, P) complex128, imaginary parts 0 (flat_gradient of a real net)
      double* row = out + n * 2 * (int64_t)g.P;
      warp_backward(g, prm, cfg, z, da, db, row, 2, lane);
      for (int k = lane; k < g.P; k += 32) row[2 * k + 1] = 0.0;
    } else {
      warp_backward(g, prm, cfg, z, da, db, out + n * (int64_t)g.P, 1, lane);
    }
    __syncwarp();
  }
}

}  // namespace vmc

namespace vmc {

// Metropolis for the CNN: one warp per chain, single-flip proposals, full
// re-evaluation of log psi(s') (sampler.py:325-358), same Philox stream and
// decision rule as the RBM sampler.
template <typename T>
__global__ void cnn_metropolis_kernel(int32_t* __restrict__ states, int C, cnn_geom g, const T* __restrict__ prm,
                                      int warps, double mu, uint64_t seed, uint32_t call, int64_t thermSteps,
                                      int64_t sweepSteps, int64_t samplesPerChain, int32_t* __restrict__ configsOut,
                                      unsigned long long* __restrict__ counters) {
  extern __shared__ unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int chain = blockIdx.x * warps + warp;
  if (chain >= C) return;
  const size_t zBytes = (size_t)g.layers * g.sites * g.maxC * sizeof(T);
  const size_t per = (zBytes + 2 * g.sites + 15) & ~(size_t)15;
  T* z = reinterpret_cast<T*>(smem + warp * per);
  int8_t* cfg = reinterpret_cast<int8_t*>(smem + warp * per + zBytes);
  int8_t* prop = cfg + g.sites;
  int32_t* st = states + (size_t)chain * g.sites;
  for (int i = lane; i < g.sites; i += 32) cfg[i] = (int8_t)st[i];
  __syncwarp();
  warp_forward(g, prm, cfg, z, lane);
  double cur = (double)warp_output(g, z, lane);
  cur = __shfl_sync(0xffffffffu, cur, 0);
  unsigned long long accepted = 0;
  const int64_t total = thermSteps + sweepSteps * samplesPerChain;
  for (int64_t step = 0; step < total; ++step) {
    const mc_draw d = metropolis_draw(seed, call, (uint32_t)step, (uint32_t)chain, g.sites);
    for (int i = lane; i < g.sites; i += 32) prop[i] = i == d.site ? (int8_t)(1 - cfg[i]) : cfg[i];
    __syncwarp();
    warp_forward(g, prm, prop, z, lane);
    double nw = (double)warp_output(g, z, lane);
    nw = __shfl_sync(0xffffffffu, nw, 0);
    const double P = exp(mu * nw - mu * cur);
    if (d.u64() < P) {
      if (lane == 0) cfg[d.site] = (int8_t)(1 - cfg[d.site]);
      cur = nw;
      ++accepted;
    }
    __syncwarp();
    if (step >= thermSteps && ((step - thermSteps + 1) % sweepSteps) == 0) {
      const int64_t s = (step - thermSteps + 1) / sweepSteps - 1;
      int32_t* o = configsOut + ((size_t)s * C + chain) * g.sites;
      for (int k = lane; k < g.sites; k += 32) o[k] = cfg[k];
    }
  }
  __syncwarp();
  for (int k = lane; k < g.sites; k += 32) st[k] = cfg[k];
  if (lane == 0) {
    atomicAdd(&counters[0], (unsigned long long)total);
    atomicAdd(&counters[1], accepted);
  }
}

static int make_geom(const vmc_cnn_desc* d, cnn_geom& g) {
  VMC_REQUIRE(d, VMC_ERR_INVALID_ARGUMENT, "cnn: null descriptor");
  VMC_REQUIRE((d->ndim == 1 || d->ndim == 2) && d->num_layers >= 1 && d->num_layers <= kCnnMaxLayers,
              VMC_ERR_UNSUPPORTED, "cnn: %d dimensions, %d layers (1-2 dims, 1-%d layers)", d->ndim, d->num_layers,
              kCnnMaxLayers);
  g.nd = d->ndim;
  g.H = d->ndim == 2 ? d->dims[0] : 1;
  g.W = d->ndim == 2 ? d->dims[1] : d->dims[0];
  g.FH = d->ndim == 2 ? d->filter[0] : 1;
  g.FW = d->ndim == 2 ? d->filter[1] : d->filter[0];
  VMC_REQUIRE(g.H > 0 && g.W > 0 && g.FH > 0 && g.FW > 0 && g.FH <= g.H && g.FW <= g.W, VMC_ERR_INVALID_ARGUMENT,
              "cnn: lattice %dx%d, filter %dx%d", g.H, g.W, g.FH, g.FW);
  g.sites = g.H * g.W;
  VMC_REQUIRE(g.sites <= 4096, VMC_ERR_UNSUPPORTED, "cnn: %d sites > 4096", g.sites);
  g.layers = d->num_layers;
  g.maxC = 1;
  int off = 0, cin = 1;
  for (int l = 0; l < g.layers; ++l) {
    g.ch[l] = d->channels[l];
    g.act[l] = d->activation[l];
    g.bias[l] = d->has_bias[l] ? 1 : 0;
    VMC_REQUIRE(g.ch[l] > 0 && g.ch[l] <= 256 && g.act[l] >= 0 && g.act[l] <= 3, VMC_ERR_UNSUPPORTED,
                "cnn: layer %d: %d channels, activation %d", l, g.ch[l], g.act[l]);
    g.maxC = std::max(g.maxC, g.ch[l]);
    if (g.bias[l]) {  // leaf order: bias before kernel within a layer
      g.bOff[l] = off;
      off += g.ch[l];
    } else {
      g.bOff[l] = -1;
    }
    g.kOff[l] = off;
    off += g.FH * g.FW * cin * g.ch[l];
    cin = g.ch[l];
  }
  for (int l = g.layers; l < kCnnMaxLayers; ++l) {
    g.ch[l] = 0;
    g.bOff[l] = -1;
    g.kOff[l] = 0;
    g.act[l] = 0;
    g.bias[l] = 0;
  }
  g.P = off;
  return VMC_OK;
}

static int pick_warps(size_t perWarp, int maxWarps, const char* fn) {
  int w = maxWarps;
  while (w > 1 && perWarp * w > 200 * 1024) w /= 2;
  VMC_REQUIRE(perWarp * w <= 227 * 1024, VMC_ERR_UNSUPPORTED, "%s: network too large for shared memory", fn);
  return w;
}

template <typename K>
static void allow_smem(K* fn, size_t bytes) {
  if (bytes > 48 * 1024) cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

}  // namespace vmc

using namespace vmc;

extern "C" int vmc_cnn_num_params(const vmc_cnn_desc* desc) {
  cnn_geom g;
  if (make_geom(desc, g)) return -1;
  return g.P;
}

extern "C" int vmc_cnn_logpsi(int32_t precision, const vmc_cnn_desc* desc, const int32_t* configs, int64_t num_configs,
                              const void* params, double* log_psi, vmc_stream_t stream) {
  cnn_geom g;
  int rc = make_geom(desc, g);
  if (rc) return rc;
  VMC_REQUIRE(precision == VMC_F64 || precision == VMC_F32, VMC_ERR_UNSUPPORTED, "vmc_cnn_logpsi: precision");
  if (num_configs == 0) return VMC_OK;
  VMC_REQUIRE(configs && params && log_psi && num_configs > 0, VMC_ERR_INVALID_ARGUMENT, "vmc_cnn_logpsi: null");
  const size_t el = precision == VMC_F64 ? 8 : 4;
  const size_t per = ((size_t)g.layers * g.sites * g.maxC * el + g.sites + 15) & ~(size_t)15;
  int warps = pick_warps(per, 8, "vmc_cnn_logpsi");
  if (!warps) return VMC_ERR_UNSUPPORTED;
  const size_t smem = per * warps;
  int64_t grid = (num_configs + warps - 1) / warps;
  if (grid > 152 * 32) grid = 152 * 32;
  cudaStream_t st = as_stream(stream);
  if (precision == VMC_F64) {
    allow_smem(cnn_logpsi_kernel<double>, smem);
    cnn_logpsi_kernel<double><<<(int)grid, 32 * warps, smem, st>>>(configs, num_configs, g,
                                                                  reinterpret_cast<const double*>(params), warps,
                                                                  reinterpret_cast<double2*>(log_psi));
  } else {
    allow_smem(cnn_logpsi_kernel<float>, smem);
    cnn_logpsi_kernel<float><<<(int)grid, 32 * warps, smem, st>>>(configs, num_configs, g,
                                                                 reinterpret_cast<const float*>(params), warps,
                                                                 reinterpret_cast<double2*>(log_psi));
  }
  return check_launch("vmc_cnn_logpsi");
}

extern "C" int vmc_cnn_gradients(int32_t precision, const vmc_cnn_desc* desc, const int32_t* configs,
                                 int64_t num_configs, const void* params, int32_t layout, double* out,
                                 vmc_stream_t stream) {
  cnn_geom g;
  int rc = make_geom(desc, g);
  if (rc) return rc;
  VMC_REQUIRE(precision == VMC_F64 || precision == VMC_F32, VMC_ERR_UNSUPPORTED, "vmc_cnn_gradients: precision");
  VMC_REQUIRE(layout == VMC_GRAD_REFERENCE || layout == VMC_GRAD_COMPACT, VMC_ERR_INVALID_ARGUMENT,
              "vmc_cnn_gradients: layout %d", layout);
  if (num_configs == 0) return VMC_OK;
  VMC_REQUIRE(configs && params && out && num_configs > 0, VMC_ERR_INVALID_ARGUMENT, "vmc_cnn_gradients: null");
  const size_t el = precision == VMC_F64 ? 8 : 4;
  const size_t per = ((size_t)(g.layers + 2) * g.sites * g.maxC * el + g.sites + 15) & ~(size_t)15;
  int warps = pick_warps(per, 4, "vmc_cnn_gradients");
  if (!warps) return VMC_ERR_UNSUPPORTED;
  const size_t smem = per * warps;
  int64_t grid = (num_configs + warps - 1) / warps;
  if (grid > 152 * 32) grid = 152 * 32;
  cudaStream_t st = as_stream(stream);
  if (precision == VMC_F64) {
    allow_smem(cnn_grad_kernel<double>, smem);
    cnn_grad_kernel<double><<<(int)grid, 32 * warps, smem, st>>>(configs, num_configs, g,
                                                                reinterpret_cast<const double*>(params), warps,
                                                                layout, out);
  } else {
    allow_smem(cnn_grad_kernel<float>, smem);
    cnn_grad_kernel<float><<<(int)grid, 32 * warps, smem, st>>>(configs, num_configs, g,
                                                               reinterpret_cast<const float*>(params), warps, layout,
                                                               out);
  }
  return check_launch("vmc_cnn_gradients");
}

extern "C" int vmc_cnn_metropolis(int32_t precision, const vmc_cnn_desc* desc, int32_t* states, int32_t num_chains,
                                  const void* params, double mu, uint64_t seed, uint32_t call_index,
                                  int64_t therm_steps, int64_t sweep_steps, int64_t samples_per_chain,
                                  int32_t* configs_out, void* counters, vmc_stream_t stream) {
  cnn_geom g;
  int rc = make_geom(desc, g);
  if (rc) return rc;
  VMC_REQUIRE(precision == VMC_F64 || precision == VMC_F32, VMC_ERR_UNSUPPORTED, "vmc_cnn_metropolis: precision");
  VMC_REQUIRE(states && params && counters && num_chains > 0 && sweep_steps > 0 && therm_steps >= 0 &&
                  samples_per_chain >= 0 && (configs_out || samples_per_chain == 0),
              VMC_ERR_INVALID_ARGUMENT, "vmc_cnn_metropolis: bad arguments");
  VMC_REQUIRE(mu >= 0.0 && mu <= 2.0, VMC_ERR_INVALID_ARGUMENT, "vmc_cnn_metropolis: mu=%g outside [0, 2]", mu);
  VMC_REQUIRE(therm_steps + sweep_steps * samples_per_chain < (int64_t)0xFFFFFFFF, VMC_ERR_UNSUPPORTED,
              "vmc_cnn_metropolis: more than 2^32 steps in one call");
  const size_t el = precision == VMC_F64 ? 8 : 4;
  const size_t per = ((size_t)g.layers * g.sites * g.maxC * el + 2 * g.sites + 15) & ~(size_t)15;
  int warps = pick_warps(per, 4, "vmc_cnn_metropolis");
  if (!warps) return VMC_ERR_UNSUPPORTED;
  const size_t smem = per * warps;
  const int grid = (num_chains + warps - 1) / warps;
  cudaStream_t st = as_stream(stream);
  unsigned long long* cnt = reinterpret_cast<unsigned long long*>(counters);
  if (precision == VMC_F64) {
    allow_smem(cnn_metropolis_kernel<double>, smem);
    cnn_metropolis_kernel<double><<<grid, 32 * warps, smem, st>>>(
        states, num_chains, g, reinterpret_cast<const double*>(params), warps, mu, seed, call_index, therm_steps,
        sweep_steps, samples_per_chain, configs_out, cnt);
  } else {
    allow_smem(cnn_metropolis_kernel<float>, smem);
    cnn_metropolis_kernel<float><<<grid, 32 * warps, smem, st>>>(
        states, num_chains, g, reinterpret_cast<const float*>(params), warps, mu, seed, call_index, therm_steps,
        sweep_steps, samples_per_chain, configs_out, cnt);
  }
  return check_launch("vmc_cnn_metropolis");
}
