// Real CNN ansatz (nets/cnn.py:18-83): periodic (wrap) padding (0, F-1),
// VALID cross-correlation with HWIO kernels, unit strides, bias per layer,
// polynomial activation after every layer, output sum / sqrt(#elements).
//
// One warp per configuration.  The forward pass keeps every layer's
// pre-activations of that configuration in shared memory; the backward
// kernel (d log psi / d theta, flat_gradient of vqs.py:46-51) recomputes
// them instead of storing activations per sample in HBM.
#include <algorithm>

#include "bf_apply.cuh"
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

// ------------------------------------------------------------ local updates
// A flip of site q0 changes the outputs of layer l (0-based) only on the
// square of (l+1)(F-1)+1 sites ending at q0 (output p reads p .. p+F-1), so
// a proposal recomputes those regions from the stored activations of the
// layer below (the region of layer l-1 taken from the proposal, the rest
// from the chain's state) and the change of log psi is the sum of the last
// layer's activation changes.  Every region value is formed with the same
// operations in the same order as the full forward pass, so an accepted
// proposal leaves exactly the activations of a full evaluation.
struct cnn_local {
  int h[kCnnMaxLayers], w[kCnnMaxLayers];  // region extents (capped at the lattice)
  int aOff[kCnnMaxLayers];                 // activations of layer l: S x ch[l]
  int newOff[kCnnMaxLayers];               // region values of layer l: h w x ch[l]
  int winOff;                              // input window of the current layer
  int perWarp;                             // elements per warp
};

static cnn_local make_local(const cnn_geom& g) {
  cnn_local lc;
  int off = 0;
  for (int l = 0; l < kCnnMaxLayers; ++l) {
    lc.aOff[l] = 0;
    lc.newOff[l] = 0;
    lc.h[l] = lc.w[l] = 1;
  }
  for (int l = 0; l < g.layers; ++l) {
    lc.aOff[l] = off;
    off += g.sites * g.ch[l];
  }
  int win = 0;
  for (int l = 0; l < g.layers; ++l) {
    lc.h[l] = std::min(g.H, (l + 1) * (g.FH - 1) + 1);
    lc.w[l] = std::min(g.W, (l + 1) * (g.FW - 1) + 1);
    lc.newOff[l] = off;
    off += lc.h[l] * lc.w[l] * g.ch[l];
    if (l > 0) win = std::max(win, (lc.h[l] + g.FH - 1) * (lc.w[l] + g.FW - 1) * g.ch[l - 1]);
  }
  lc.winOff = off;
  off += win;
  lc.perWarp = off;
  return lc;
}

// v mod n for -2n <= v < 3n (every use below stays in that range), without
// an integer division
__device__ __forceinline__ int wrap(int v, int n) {
  v = v >= n ? v - n : v;
  v = v >= n ? v - n : v;
  v = v < 0 ? v + n : v;
  return v < 0 ? v + n : v;
}

// activations of every layer of cfg into a (one warp)
template <typename T>
__device__ T warp_forward_act(const cnn_geom& g, const cnn_local& lc, const T* prm, const int8_t* cfg, T* a,
                              int lane) {
  const int S = g.sites;
  for (int l = 0; l < g.layers; ++l) {
    const int cin = l == 0 ? 1 : g.ch[l - 1], cout = g.ch[l];
    const T* K = prm + g.kOff[l];
    const T* in = a + lc.aOff[l > 0 ? l - 1 : 0];
    T* o_ = a + lc.aOff[l];
    for (int o = lane; o < S * cout; o += 32) {
      const int p = o / cout, c = o - p * cout;
      const int y = p / g.W, x = p - y * g.W;
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
            for (int ci = 0; ci < cin; ++ci) acc += in[(size_t)q * cin + ci] * kk[(size_t)ci * cout];
          }
        }
      }
      o_[o] = act_f(g.act[l], acc);
    }
    __syncwarp();
  }
  const int cl = g.ch[g.layers - 1];
  const T* al = a + lc.aOff[g.layers - 1];
  T s = T(0);
  for (int o = lane; o < S * cl; o += 32) s += al[o];
  s = warp_sum(s);
  return s / sqrt(T(S * cl));
}

__device__ __forceinline__ void region_origin(const cnn_geom& g, const cnn_local& lc, int l, int qy, int qx, int& y0,
                                              int& x0) {
  y0 = lc.h[l] == g.H ? 0 : wrap(qy - (l + 1) * (g.FH - 1), g.H);
  x0 = lc.w[l] == g.W ? 0 : wrap(qx - (l + 1) * (g.FW - 1), g.W);
}

// change of log psi for flipping site q0 of cfg; the region values stay in
// the warp's scratch for warp_local_commit (one warp, all lanes return it)
template <typename T>
__device__ T warp_local_delta(const cnn_geom& g, const cnn_local& lc, const T* prm, const int8_t* cfg, const T* a,
                              T* scr, int q0, int lane) {
  const int qy = q0 / g.W, qx = q0 - (q0 / g.W) * g.W;
  for (int l = 0; l < g.layers; ++l) {
    const int cin = l == 0 ? 1 : g.ch[l - 1], cout = g.ch[l];
    const int h = lc.h[l], w = lc.w[l];
    int y0, x0;
    region_origin(g, lc, l, qy, qx, y0, x0);
    const T* K = prm + g.kOff[l];
    T* nl = scr + lc.newOff[l];
    const int WW = w + g.FW - 1;
    T* win = scr + lc.winOff;
    if (l > 0) {
      // inputs of this layer's region: layer l-1 on the rectangle starting at (y0, x0)
      const int hp = lc.h[l - 1], wp = lc.w[l - 1];
      int y0p, x0p;
      region_origin(g, lc, l - 1, qy, qx, y0p, x0p);
      const int WH = h + g.FH - 1;
      const T* np = scr + lc.newOff[l - 1];
      const T* ap = a + lc.aOff[l - 1];
      for (int o = lane; o < WH * WW * cin; o += 32) {
        const int cell = o / cin, ci = o - cell * cin;
        const int wy = cell / WW, wx = cell - wy * WW;
        const int sy = wrap(y0 + wy, g.H), sx = wrap(x0 + wx, g.W);
        const int dy = wrap(sy - y0p, g.H), dx = wrap(sx - x0p, g.W);
        win[o] = (dy < hp && dx < wp) ? np[(dy * wp + dx) * cin + ci] : ap[(size_t)(sy * g.W + sx) * cin + ci];
      }
      __syncwarp();
    }
    for (int o = lane; o < h * w * cout; o += 32) {
      const int cell = o / cout, c = o - cell * cout;
      const int ry = cell / w, rx = cell - ry * w;
      T acc = g.bOff[l] >= 0 ? prm[g.bOff[l] + c] : T(0);
      if (l == 0) {
        const int py = wrap(y0 + ry, g.H), px = wrap(x0 + rx, g.W);
        for (int dy = 0; dy < g.FH; ++dy) {
          int yy = py + dy;
          if (yy >= g.H) yy -= g.H;
          for (int dx = 0; dx < g.FW; ++dx) {
            int xx = px + dx;
            if (xx >= g.W) xx -= g.W;
            const int q = yy * g.W + xx;
            const int sv = cfg[q] ^ (q == q0 ? 1 : 0);
            acc += (sv ? T(1) : T(-1)) * K[(size_t)(dy * g.FW + dx) * cout + c];
          }
        }
      } else {
        for (int dy = 0; dy < g.FH; ++dy)
          for (int dx = 0; dx < g.FW; ++dx) {
            const T* in = win + (size_t)((ry + dy) * WW + (rx + dx)) * cin;
            const T* kk = K + ((size_t)(dy * g.FW + dx) * cin) * cout + c;
            for (int ci = 0; ci < cin; ++ci) acc += in[ci] * kk[(size_t)ci * cout];
          }
      }
      nl[o] = act_f(g.act[l], acc);
    }
    __syncwarp();
  }
  const int l = g.layers - 1, cout = g.ch[l], w = lc.w[l];
  int y0, x0;
  region_origin(g, lc, l, qy, qx, y0, x0);
  const T* nl = scr + lc.newOff[l];
  const T* al = a + lc.aOff[l];
  T s = T(0);
  for (int o = lane; o < lc.h[l] * w * cout; o += 32) {
    const int cell = o / cout, c = o - cell * cout;
    const int ry = cell / w, rx = cell - ry * w;
    const int site = wrap(y0 + ry, g.H) * g.W + wrap(x0 + rx, g.W);
    s += nl[o] - al[(size_t)site * cout + c];
  }
  s = warp_sum(s);
  return s / sqrt(T(g.sites * cout));
}

// the region values of the last warp_local_delta become the state; cfg[q0]
// flips (one warp)
template <typename T>
__device__ void warp_local_commit(const cnn_geom& g, const cnn_local& lc, int8_t* cfg, T* a, const T* scr, int q0,
                                  int lane) {
  const int qy = q0 / g.W, qx = q0 - (q0 / g.W) * g.W;
  for (int l = 0; l < g.layers; ++l) {
    const int cout = g.ch[l], w = lc.w[l];
    int y0, x0;
    region_origin(g, lc, l, qy, qx, y0, x0);
    const T* nl = scr + lc.newOff[l];
    T* al = a + lc.aOff[l];
    for (int o = lane; o < lc.h[l] * w * cout; o += 32) {
      const int cell = o / cout, c = o - cell * cout;
      const int ry = cell / w, rx = cell - ry * w;
      const int site = wrap(y0 + ry, g.H) * g.W + wrap(x0 + rx, g.W);
      al[(size_t)site * cout + c] = nl[o];
    }
  }
  __syncwarp();
  if (lane == 0) cfg[q0] = (int8_t)(1 - cfg[q0]);
  __syncwarp();
}

// parameters in shared memory when they fit (staged by the whole block)
template <typename T>
__device__ const T* stage_params(const T* __restrict__ prm, int P, T* dst, bool fits) {
  if (!fits) return prm;
  for (int k = threadIdx.x; k < P; k += blockDim.x) dst[k] = prm[k];
  __syncthreads();
  return dst;
}

constexpr int kCnnParamSmem = 32 * 1024;

// Metropolis with local updates: one warp per chain, same Philox stream and
// decision rule (u < exp(mu * delta log psi)) as the RBM sampler.
template <typename T>
__global__ void cnn_metropolis_local_kernel(int32_t* __restrict__ states, int C, const __grid_constant__ cnn_geom g,
                                            const __grid_constant__ cnn_local lc,
                                            const T* __restrict__ prmG, int warps, bool prmInSmem, double mu,
                                            uint64_t seed, uint32_t call, int64_t thermSteps, int64_t sweepSteps,
                                            int64_t samplesPerChain, int32_t* __restrict__ configsOut,
                                            unsigned long long* __restrict__ counters) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t prmBytes = prmInSmem ? (((size_t)g.P * sizeof(T) + 15) & ~(size_t)15) : 0;
  const T* prm = stage_params(prmG, g.P, reinterpret_cast<T*>(smem), prmInSmem);
  const size_t per = ((size_t)lc.perWarp * sizeof(T) + g.sites + 15) & ~(size_t)15;
  T* a = reinterpret_cast<T*>(smem + prmBytes + warp * per);
  T* scr = a;  // scratch offsets follow the activations inside the same per-warp block
  int8_t* cfg = reinterpret_cast<int8_t*>(a + lc.perWarp);
  const int chain = blockIdx.x * warps + warp;
  if (chain >= C) return;  // after the block-wide staging; whole warps exit together
  int32_t* st = states + (size_t)chain * g.sites;
  for (int i = lane; i < g.sites; i += 32) cfg[i] = (int8_t)st[i];
  __syncwarp();
  warp_forward_act(g, lc, prm, cfg, a, lane);
  unsigned long long accepted = 0;
  const int64_t total = thermSteps + sweepSteps * samplesPerChain;
  for (int64_t step = 0; step < total; ++step) {
    const mc_draw d = metropolis_draw(seed, call, (uint32_t)step, (uint32_t)chain, g.sites);
    const T delta = warp_local_delta(g, lc, prm, cfg, a, scr, d.site, lane);
    // accept iff u < exp(mu delta): FP64 rule in the FP64 kernel (replayed by
    // the parity test), FP32 in the FP32 kernel
    bool acc;
    if (sizeof(T) == sizeof(double))
      acc = d.u64() < exp(mu * (double)delta);
    else
      acc = d.u32() < expf((float)mu * (float)delta);
    if (acc) {
      warp_local_commit(g, lc, cfg, a, scr, d.site, lane);
      ++accepted;
    }
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

// O_loc without materialising s' (Operator.get_O_loc, base.py:162-192): one
// warp per configuration; lane k applies string c0 + k; a one-flip string
// costs one local update, a string flipping n sites n local updates applied
// in turn and n more to restore the state.
template <typename T>
__global__ void cnn_oloc_fused_kernel(const int32_t* __restrict__ configs, int64_t N, const __grid_constant__ cnn_geom g,
                                      const __grid_constant__ cnn_local lc,
                                      const T* __restrict__ prmG, int warps, bool prmInSmem,
                                      const __grid_constant__ vmc_bf_operator op,
                                      const double2* __restrict__ logPsiS, double2* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t prmBytes = prmInSmem ? (((size_t)g.P * sizeof(T) + 15) & ~(size_t)15) : 0;
  const T* prm = stage_params(prmG, g.P, reinterpret_cast<T*>(smem), prmInSmem);
  const int diagWords = (op.num_ops + 31) >> 5;
  uint32_t* isdiag = reinterpret_cast<uint32_t*>(smem + prmBytes);
  const size_t diagBytes = ((size_t)diagWords * 4 + 15) & ~(size_t)15;
  const int nw = (g.sites + 31) >> 5;
  const size_t per = ((size_t)lc.perWarp * sizeof(T) + (size_t)nw * 4 + g.sites + 32 * VMC_BF_MAX_LEN * 2 + 15) &
                     ~(size_t)15;
  unsigned char* base = smem + prmBytes + diagBytes + warp * per;
  T* a = reinterpret_cast<T*>(base);
  T* scr = a;
  uint32_t* occ = reinterpret_cast<uint32_t*>(a + lc.perWarp);
  int16_t* fsRow = reinterpret_cast<int16_t*>(occ + nw);
  int8_t* cfg = reinterpret_cast<int8_t*>(fsRow + 32 * VMC_BF_MAX_LEN);
  for (int w = threadIdx.x; w < diagWords; w += blockDim.x) isdiag[w] = 0u;
  __syncthreads();
  for (int d = threadIdx.x; d < op.num_diag; d += blockDim.x) {
    const int o = op.diag[d];
    if ((unsigned)o < (unsigned)op.num_ops) atomicOr(&isdiag[o >> 5], 1u << (o & 31));
  }
  __syncthreads();
  for (int64_t n = (int64_t)blockIdx.x * warps + warp; n < N; n += (int64_t)gridDim.x * warps) {
    warp_load_config(configs + n * g.sites, g.sites, cfg, occ, lane);
    const T lpNet = warp_forward_act(g, lc, prm, cfg, a, lane);
    cpx<double> diagSum = mk(0.0, 0.0), acc = mk(0.0, 0.0);
    for (int c0 = 0; c0 < op.num_ops; c0 += 32) {
      const int o = c0 + lane;
      bool valid = false;
      int nf = 0;
      cpx<double> m = mk(0.0, 0.0);
      if (o < op.num_ops) {
        bf_string_result r;
        bf_apply_string(op, o, cfg, occ, g.sites, r);
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
      double myRatio = 1.0;
      while (vmask) {
        const int k = __ffs(vmask) - 1;
        vmask &= vmask - 1;
        const int nfk = __shfl_sync(0xffffffffu, myNf, k);
        if (nfk == 0) continue;
        const int16_t* fs = fsRow + k * VMC_BF_MAX_LEN;
        T delta;
        if (nfk == 1) {
          delta = warp_local_delta(g, lc, prm, cfg, a, scr, fs[0], lane);
        } else {
          delta = T(0);
          for (int q = 0; q < nfk; ++q) {
            delta += warp_local_delta(g, lc, prm, cfg, a, scr, fs[q], lane);
            warp_local_commit(g, lc, cfg, a, scr, fs[q], lane);
          }
          for (int q = nfk - 1; q >= 0; --q) {
            warp_local_delta(g, lc, prm, cfg, a, scr, fs[q], lane);
            warp_local_commit(g, lc, cfg, a, scr, fs[q], lane);
          }
        }
        if (lane == k) myRatio = exp((double)delta);
      }
      if (valid) acc = acc + mk(m.re * myRatio, m.im * myRatio);
      __syncwarp();
    }
    acc = warp_sum(acc);
    diagSum = warp_sum(diagSum);
    if (op.num_diag > 0 && sqrt(abs2(diagSum)) > 1e-6) acc = acc + diagSum;
    if (logPsiS) {
      const double2 gv = logPsiS[n];
      acc = acc * cexp_(mk((double)lpNet - gv.x, -gv.y));
    }
    if (lane == 0) out[n] = make_double2(acc.re, acc.im);
    __syncwarp();
  }
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
    VMC_ALLOW_SMEM(cnn_logpsi_kernel<double>, smem, "vmc_cnn_logpsi");
    cnn_logpsi_kernel<double><<<(int)grid, 32 * warps, smem, st>>>(configs, num_configs, g,
                                                                  reinterpret_cast<const double*>(params), warps,
                                                                  reinterpret_cast<double2*>(log_psi));
  } else {
    VMC_ALLOW_SMEM(cnn_logpsi_kernel<float>, smem, "vmc_cnn_logpsi");
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
    VMC_ALLOW_SMEM(cnn_grad_kernel<double>, smem, "vmc_cnn_gradients");
    cnn_grad_kernel<double><<<(int)grid, 32 * warps, smem, st>>>(configs, num_configs, g,
                                                                reinterpret_cast<const double*>(params), warps,
                                                                layout, out);
  } else {
    VMC_ALLOW_SMEM(cnn_grad_kernel<float>, smem, "vmc_cnn_gradients");
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
  const cnn_local lc = make_local(g);
  const size_t per = ((size_t)lc.perWarp * el + g.sites + 15) & ~(size_t)15;
  const size_t prmBytes = ((size_t)g.P * el + 15) & ~(size_t)15;
  const bool inSmem = prmBytes <= (size_t)kCnnParamSmem;
  int warps = 4;
  while (warps > 1 && (inSmem ? prmBytes : 0) + per * warps > 200 * 1024) warps /= 2;
  const size_t smem = (inSmem ? prmBytes : 0) + per * warps;
  VMC_REQUIRE(smem <= 227 * 1024, VMC_ERR_UNSUPPORTED, "vmc_cnn_metropolis: network too large for shared memory");
  const int grid = (num_chains + warps - 1) / warps;
  cudaStream_t st = as_stream(stream);
  unsigned long long* cnt = reinterpret_cast<unsigned long long*>(counters);
  if (precision == VMC_F64) {
    VMC_ALLOW_SMEM(cnn_metropolis_local_kernel<double>, smem, "vmc_cnn_metropolis");
    cnn_metropolis_local_kernel<double><<<grid, 32 * warps, smem, st>>>(
        states, num_chains, g, lc, reinterpret_cast<const double*>(params), warps, inSmem, mu, seed, call_index,
        therm_steps, sweep_steps, samples_per_chain, configs_out, cnt);
  } else {
    VMC_ALLOW_SMEM(cnn_metropolis_local_kernel<float>, smem, "vmc_cnn_metropolis");
    cnn_metropolis_local_kernel<float><<<grid, 32 * warps, smem, st>>>(
        states, num_chains, g, lc, reinterpret_cast<const float*>(params), warps, inSmem, mu, seed, call_index,
        therm_steps, sweep_steps, samples_per_chain, configs_out, cnt);
  }
  return check_launch("vmc_cnn_metropolis");
}

extern "C" int vmc_cnn_oloc_fused(int32_t precision, const vmc_cnn_desc* desc, const int32_t* configs,
                                  int64_t num_configs, const void* params, const vmc_bf_operator* op,
                                  const double* log_psi_s, double* oloc, vmc_stream_t stream) {
  cnn_geom g;
  int rc = make_geom(desc, g);
  if (rc) return rc;
  VMC_REQUIRE(precision == VMC_F64 || precision == VMC_F32, VMC_ERR_UNSUPPORTED, "vmc_cnn_oloc_fused: precision");
  if ((rc = check_op("vmc_cnn_oloc_fused", op, g.sites))) return rc;
  VMC_REQUIRE(op->local_dim == 2, VMC_ERR_UNSUPPORTED, "vmc_cnn_oloc_fused: local dimension %d (spins need 2)",
              op->local_dim);
  if (num_configs == 0) return VMC_OK;
  VMC_REQUIRE(configs && params && oloc && num_configs > 0, VMC_ERR_INVALID_ARGUMENT, "vmc_cnn_oloc_fused: null");
  const size_t el = precision == VMC_F64 ? 8 : 4;
  const cnn_local lc = make_local(g);
  const int nw = (g.sites + 31) >> 5;
  const size_t per = ((size_t)lc.perWarp * el + (size_t)nw * 4 + g.sites + 32 * VMC_BF_MAX_LEN * 2 + 15) &
                     ~(size_t)15;
  const size_t prmBytes = ((size_t)g.P * el + 15) & ~(size_t)15;
  const bool inSmem = prmBytes <= (size_t)kCnnParamSmem;
  const size_t diagBytes = ((size_t)((op->num_ops + 31) >> 5) * 4 + 15) & ~(size_t)15;
  int warps = 4;
  while (warps > 1 && (inSmem ? prmBytes : 0) + diagBytes + per * warps > 200 * 1024) warps /= 2;
  const size_t smem = (inSmem ? prmBytes : 0) + diagBytes + per * warps;
  VMC_REQUIRE(smem <= 227 * 1024, VMC_ERR_UNSUPPORTED, "vmc_cnn_oloc_fused: network too large for shared memory");
  int64_t grid = (num_configs + warps - 1) / warps;
  if (grid > 152 * 32) grid = 152 * 32;
  cudaStream_t st = as_stream(stream);
  if (precision == VMC_F64) {
    VMC_ALLOW_SMEM(cnn_oloc_fused_kernel<double>, smem, "vmc_cnn_oloc_fused");
    cnn_oloc_fused_kernel<double><<<(int)grid, 32 * warps, smem, st>>>(
        configs, num_configs, g, lc, reinterpret_cast<const double*>(params), warps, inSmem, *op,
        reinterpret_cast<const double2*>(log_psi_s), reinterpret_cast<double2*>(oloc));
  } else {
    VMC_ALLOW_SMEM(cnn_oloc_fused_kernel<float>, smem, "vmc_cnn_oloc_fused");
    cnn_oloc_fused_kernel<float><<<(int)grid, 32 * warps, smem, st>>>(
        configs, num_configs, g, lc, reinterpret_cast<const float*>(params), warps, inSmem, *op,
        reinterpret_cast<const double2*>(log_psi_s), reinterpret_cast<double2*>(oloc));
  }
  return check_launch("vmc_cnn_oloc_fused");
}
