// Error reporting and version of the C ABI.
#include <cstdarg>
#include <cstdio>

#include "vmc_common.cuh"

namespace vmc {

static thread_local char g_last_error[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return VMC_ERR_CUDA;
  }
  return VMC_OK;
}

int check_op(const char* fn, const vmc_bf_operator* op, int L) {
  VMC_REQUIRE(op, VMC_ERR_INVALID_ARGUMENT, "%s: null operator", fn);
  VMC_REQUIRE(op->num_ops > 0 && op->max_len > 0 && op->max_len <= VMC_BF_MAX_LEN && op->local_dim >= 2 &&
                  op->num_diag >= 0 && op->num_diag <= op->num_ops,
              VMC_ERR_UNSUPPORTED, "%s: operator with %d strings of length %d (max %d), lDim %d", fn, op->num_ops,
              op->max_len, VMC_BF_MAX_LEN, op->local_dim);
  VMC_REQUIRE(op->idx && op->map && op->mat_els && op->fermi && op->prefactor && (op->diag || op->num_diag == 0),
              VMC_ERR_INVALID_ARGUMENT, "%s: null operator table", fn);
  (void)L;
  return VMC_OK;
}

int allow_smem(const void* fn, size_t bytes, const char* what) {
  if (bytes <= 48 * 1024) return VMC_OK;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();  // clear the non-sticky error so the next launch is not blamed
    set_error("%s: cannot allow %zu bytes of dynamic shared memory: %s", what, bytes, cudaGetErrorString(e));
    return VMC_ERR_CUDA;
  }
  return VMC_OK;
}

}  // namespace vmc

extern "C" int vmc_api_version(void) { return VMC_API_VERSION; }

extern "C" const char* vmc_last_error_string(void) { return vmc::g_last_error; }

extern "C" int vmc_metropolis_draws_host(uint64_t seed, uint32_t call_index, uint32_t step, int32_t num_chains,
                                         int32_t num_sites, int32_t* sites, double* uniforms) {
  VMC_REQUIRE(sites && uniforms && num_chains >= 0 && num_sites > 0, VMC_ERR_INVALID_ARGUMENT,
              "vmc_metropolis_draws_host: bad arguments");
  for (int c = 0; c < num_chains; ++c) {
    vmc::u32x4 ctr;
    ctr.x = step;
    ctr.y = (uint32_t)c;
    ctr.z = call_index;
    ctr.w = 0x5EEDu;
    vmc::u32x4 r = vmc::philox4x32_10(ctr, (uint32_t)seed, (uint32_t)(seed >> 32));
    sites[c] = (int32_t)(((uint64_t)r.x * (uint64_t)num_sites) >> 32);
    uniforms[c] = ((double)(r.y >> 5) * 67108864.0 + (double)(r.z >> 6)) * (1.0 / 9007199254740992.0);
  }
  return VMC_OK;
}
