/*
 * vmc_gb300.h -- C ABI of the GB300-native (sm_103a) VMC hot path.
 *
 * Each entry point replaces one stage of jVMC 1.5.8's per-step hot path
 * (the reference file:line it replaces is given with each declaration; paths
 * are relative to the jVMC project root).  The reference is JAX code: these
 * are the functions a jax.ffi / ctypes binding of that path calls.
 *
 * Conventions
 *   - every pointer is a DEVICE pointer unless stated otherwise; the caller
 *     owns every buffer, nothing is allocated inside an entry point;
 *   - complex numbers are interleaved (re, im) pairs: "c128" = 2 doubles
 *     (numpy complex128 / jnp.complex128), "c64" = 2 floats;
 *   - configurations are int32 with values in [0, local_dim), row-major
 *     (num_configs, num_sites), the layout of jVMC's samplers
 *     (sampler.py:118-121, 320-323);
 *   - all work is stream-ordered on `stream` (a cudaStream_t; NULL = legacy
 *     default stream); no entry point synchronises the host except those
 *     that say so;
 *   - return value 0 = success, otherwise a vmc_status code; the message of
 *     the last failure on the calling thread is vmc_last_error_string().
 *     No entry point aborts, traps or hangs.
 */
#ifndef VMC_GB300_H
#define VMC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VMC_API_VERSION 1

typedef void* vmc_stream_t;

typedef enum {
  VMC_OK = 0,
  VMC_ERR_INVALID_ARGUMENT = 1,
  VMC_ERR_UNSUPPORTED = 2,
  VMC_ERR_CUDA = 3,
  VMC_ERR_TIMEOUT = 4,
  VMC_ERR_WORKSPACE = 5
} vmc_status;

/* arithmetic precision of a kernel; parameters are passed in the matching
 * complex type (VMC_F64: c128, VMC_F32: c64) */
typedef enum { VMC_F64 = 0, VMC_F32 = 1 } vmc_precision;

/* layouts of per-sample log-derivatives O_k = d log psi / d theta_k */
typedef enum {
  /* (N, 2P) c128: per parameter leaf [g, i g] -- the holomorphic flat
   * gradient of jVMC (vqs.py:66-69, leaf order of get_parameters) */
  VMC_GRAD_REFERENCE = 0,
  /* (N, P) c128: one complex derivative per complex parameter */
  VMC_GRAD_COMPACT = 1
} vmc_grad_layout;

int vmc_api_version(void);
const char* vmc_last_error_string(void);

/* ------------------------------------------------------------------------
 * ExactSampler basis.  Replaces ExactSampler.get_basis /
 * _get_basis_ldim2 / _get_basis (sampler.py:421-472): state index
 * first_state + r in row r; for local_dim 2 site i holds bit i of the index,
 * otherwise the base-local_dim digits most-significant first.
 * ------------------------------------------------------------------------ */
int vmc_exact_basis(int32_t* basis, int64_t first_state, int64_t num_states, int32_t num_sites,
                    int32_t local_dim, vmc_stream_t stream);

/* Born weights of the exact sampler (sampler.py:474-486, 519-524):
 * p_r = exp((Re log_psi_r - last_norm) / log_prob_factor) for r < num_valid,
 * else 0; nrm = sum(p); p /= nrm; last_norm += log_prob_factor * log(nrm).
 * last_norm is a device f64 read and updated in place (ExactSampler.lastNorm);
 * *norm_out (device f64, optional) receives nrm.
 * workspace: vmc_reduce_workspace_bytes(1) bytes. */
int vmc_exact_probabilities(const double* log_psi, int64_t num_states, int64_t num_valid, double* last_norm,
                            double log_prob_factor, double* p, double* norm_out, void* workspace,
                            size_t workspace_bytes, vmc_stream_t stream);

/* ------------------------------------------------------------------------
 * Complex RBM  log psi(s) = sum_j logcosh(sum_i W_ij (2 s_i - 1) + b_j)
 * (nets/rbm.py:17-38, nets/activation_functions.py:19-22).
 * kernel: (L, M) row-major, bias: (M) or NULL, in the precision's complex type.
 * ------------------------------------------------------------------------ */

/* Size in bytes of the per-parameter tables used by the fused local-energy
 * and Metropolis kernels (5 complex (L, M) tables and L row sums). */
size_t vmc_rbm_tables_bytes(int32_t precision, int32_t num_sites, int32_t num_hidden);

/* Fill the tables: cosh(2W), sinh(2W), exp(2W), exp(-2W), tanh(2W), then
 * sum_j log cosh(2 W_ij) per row i.  Call after every parameter change.
 * No reference counterpart: jVMC re-evaluates rbm.py:29-38 for every s';
 * these factors let the fused E_loc and Metropolis kernels form the ratios
 * psi(s')/psi(s) of that same function. */
int vmc_rbm_prepare(int32_t precision, int32_t num_sites, int32_t num_hidden, const void* kernel, void* tables,
                    vmc_stream_t stream);

/* log psi of num_configs configurations into log_psi (c128).  Replaces
 * NQS.__call__ / _eval (vqs.py:223-251) for a CpxRBM. */
int vmc_rbm_logpsi(int32_t precision, const int32_t* configs, int64_t num_configs, int32_t num_sites,
                   int32_t num_hidden, const void* kernel, const void* bias, double* log_psi, vmc_stream_t stream);

/* Per-sample log-derivatives (holomorphic): d/db_j = tanh(theta_j),
 * d/dW_ij = (2 s_i - 1) tanh(theta_j).  Replaces NQS.gradients with
 * flat_gradient_holo (vqs.py:66-69, 256-287).  out is c128 in `layout`. */
int vmc_rbm_gradients(int32_t precision, const int32_t* configs, int64_t num_configs, int32_t num_sites,
                      int32_t num_hidden, const void* kernel, const void* bias, int32_t layout, double* out,
                      vmc_stream_t stream);

/* Metropolis sampling of |psi|^mu with single spin flips.  Replaces
 * MCSampler._get_samples_mcmc / _get_samples / _sweep with propose_spin_flip
 * (sampler.py:15-19, 264-358).  One warp per chain; states (num_chains, L)
 * are read and written back (the chains persist between calls);
 * therm_steps proposals, then samples_per_chain times sweep_steps proposals
 * followed by a record, into configs_out (samples_per_chain*num_chains, L)
 * with row = sample*num_chains + chain (sampler.py:320-323).
 * Random numbers: Philox4x32-10 with key = seed, counter =
 * (step, chain, call_index, 0x5EED); site = (r0 * L) >> 32, accept iff
 * u < |psi(s')/psi(s)|^mu with u = ((r1>>5) 2^26 + (r2>>6)) / 2^53.
 * counters (device uint64[2]) += {proposed, accepted}.  Needs the tables of
 * vmc_rbm_prepare. */
int vmc_rbm_metropolis(int32_t precision, int32_t* states, int32_t num_chains, int32_t num_sites,
                       int32_t num_hidden, const void* kernel, const void* bias, const void* tables, double mu,
                       uint64_t seed, uint32_t call_index, int64_t therm_steps, int64_t sweep_steps,
                       int64_t samples_per_chain, int32_t* configs_out, void* counters, vmc_stream_t stream);

/* Host-side copy of the Metropolis random stream (no GPU needed): flip sites
 * and acceptance uniforms of `step` for chains 0..num_chains-1 (host arrays).
 * Stands where jVMC draws jax.random.randint / bernoulli (sampler.py:15-19,
 * 330-340); used by tests to replay chains on the host. */
int vmc_metropolis_draws_host(uint64_t seed, uint32_t call_index, uint32_t step, int32_t num_chains,
                              int32_t num_sites, int32_t* sites, double* uniforms);

/* vmc_rbm_metropolis (MCSampler._get_samples_mcmc / _sweep, sampler.py:264-367) with
 * the call index read from device memory
 * (*call_index, uint32) and incremented after the sweep on the same stream:
 * a CUDA graph that captures it draws a fresh random stream on every replay
 * (the serving loop's shared graph launches). */
int vmc_rbm_metropolis_devcall(int32_t precision, int32_t* states, int32_t num_chains, int32_t num_sites,
                               int32_t num_hidden, const void* kernel, const void* bias, const void* tables,
                               double mu, uint64_t seed, uint32_t* call_index, int64_t therm_steps,
                               int64_t sweep_steps, int64_t samples_per_chain, int32_t* configs_out, void* counters,
                               vmc_stream_t stream);

/* Metropolis weights p_r = exp(factor * Re log_psi_r) / sum (sampler.py:234-235,
 * factor = 1/logProbFactor - mu).  workspace: vmc_reduce_workspace_bytes(1). */
int vmc_mc_probabilities(const double* log_psi, int64_t num_samples, double factor, double* p, void* workspace,
                         size_t workspace_bytes, vmc_stream_t stream);

/* Vector-Jacobian product of log psi (the contraction jax.grad forms inside
 * NQS.gradients, vqs.py:66-69, 256-287):
 * out_k = sum_n conj(g_n) O_nk (c128, compact
 * layout) for a cotangent g (N, c128), without materialising O: the
 * activations tanh(theta) are recomputed from the configurations.  The
 * backward of a torch.autograd.Function / jax.custom_vjp over log psi.
 * workspace: vmc_rbm_vjp_workspace_bytes. */
size_t vmc_rbm_vjp_workspace_bytes(int64_t num_configs, int32_t num_sites, int32_t num_hidden);
int vmc_rbm_vjp(int32_t precision, const int32_t* configs, int64_t num_configs, int32_t num_sites,
                int32_t num_hidden, const void* kernel, const void* bias, const double* cotangent, double* out,
                void* workspace, size_t workspace_bytes, vmc_stream_t stream);

/* ------------------------------------------------------------------------
 * Branch-free operators (operator/branch_free.py:311-487).
 * The tables are those of BranchFreeOperator.compile (348-414): every
 * operator string is stored right-to-left and padded with Id(0).
 * ------------------------------------------------------------------------ */
typedef struct {
  int32_t num_ops;       /* number of operator strings                      */
  int32_t max_len;       /* maxOpStrLength                                  */
  int32_t local_dim;     /* lDim                                             */
  int32_t num_diag;      /* number of diagonal strings                       */
  const int32_t* idx;    /* (num_ops, max_len) site index                    */
  const int32_t* map;    /* (num_ops, max_len, local_dim) new local state    */
  const double* mat_els; /* (num_ops, max_len, local_dim) c128               */
  const int32_t* fermi;  /* (num_ops, max_len) 1 = fermionic operator        */
  const double* prefactor; /* (num_ops) c128, arg_fun(*args) (416-438)      */
  const int32_t* diag;   /* (num_diag) indices of the diagonal strings       */
} vmc_bf_operator;

/* Maximum operator-string length the kernels accept. */
#define VMC_BF_MAX_LEN 16

/* Matrix elements of every string for every configuration, the diagonal
 * merge (branch_free.py:483-485) and the nonzero compaction of
 * Operator._find_nonzero (base.py:91-103): mat_el_full (N, num_ops) c128,
 * nz_index (N, num_ops) ascending indices of |m| > 1e-6, nz_count (N),
 * *max_count (device int32) = max nz_count (the value of
 * jnp.max(numNonzero) in base.py:157). */
int vmc_bf_matrix_elements(const int32_t* configs, int64_t num_configs, int32_t num_sites,
                           const vmc_bf_operator* op, double* mat_el_full, int32_t* nz_index, int32_t* nz_count,
                           int32_t* max_count, vmc_stream_t stream);

/* s' and matrix elements in the reference layout of Operator.get_s_primes
 * (base.py:116-160): s_primes (N*K, L) and mat_el (N, K) c128; entries past
 * nz_count are the last string's s' with matrix element 0
 * (set_zero_to_zero, base.py:105-114).  K = the max_count above. */
int vmc_bf_gather(const int32_t* configs, int64_t num_configs, int32_t num_sites, const vmc_bf_operator* op,
                  const double* mat_el_full, const int32_t* nz_index, const int32_t* nz_count, int32_t K,
                  int32_t* s_primes, double* mat_el, vmc_stream_t stream);

/* O_loc(s) = sum_k mat_el_k exp(log psi(s'_k) - log psi(s))
 * (Operator._get_O_loc, base.py:162-164). */
int vmc_oloc_from_sprimes(const double* mat_el, const double* log_psi_s, const double* log_psi_sp,
                          int64_t num_configs, int32_t K, double* oloc, vmc_stream_t stream);

/* Fused local estimator for a CpxRBM: O_loc(s) of a branch-free operator
 * without materialising s' (replaces get_s_primes + psi(s') + _get_O_loc,
 * base.py:166-192).  Uses the tables of vmc_rbm_prepare.  local_dim 2.
 * log_psi_s (c128, optional): the caller's log psi(s); when given the result
 * is sum_k m_k exp(log psi(s'_k) - log_psi_s) exactly as base.py:162-164,
 * when NULL the network's own log psi(s) is used. */
int vmc_rbm_oloc_fused(int32_t precision, const int32_t* configs, int64_t num_configs, int32_t num_sites,
                       int32_t num_hidden, const void* kernel, const void* bias, const void* tables,
                       const vmc_bf_operator* op, const double* log_psi_s, double* oloc, vmc_stream_t stream);

/* ------------------------------------------------------------------------
 * Sample statistics (stats.py:197-265, mpi_wrapper.py:114-217), FP64,
 * fixed-order (bitwise reproducible) reductions.
 * ------------------------------------------------------------------------ */

/* Workspace bytes of a reduction producing `num_outputs` c128 values. */
size_t vmc_reduce_workspace_bytes(int64_t num_outputs);

/* mean = sum_n w_n x_n (c128), var = sum_n w_n |x_n - mean|^2 (f64). */
int vmc_weighted_mean_var(const double* x, const double* w, int64_t n, double* mean, double* var, void* workspace,
                          size_t workspace_bytes, vmc_stream_t stream);

/* Mean of the RBM log-derivatives and the force for the compact layout:
 * ok_mean_k = sum_n w_n O_nk, force_k = sum_n w_n conj(O_nk - ok_mean_k)(E_n - eloc_mean)
 * (stats.py:50-58 via tdvp.py:139-142), without materialising O.  P = M + L*M
 * with bias, L*M without.  workspace: vmc_rbm_grad_stats_workspace_bytes. */
size_t vmc_rbm_grad_stats_workspace_bytes(int64_t num_configs, int32_t num_sites, int32_t num_hidden);
int vmc_rbm_grad_stats(int32_t precision, const int32_t* configs, int64_t num_configs, int32_t num_sites,
                       int32_t num_hidden, const void* kernel, const void* bias, const double* weights,
                       const double* eloc, const double* eloc_mean, double* ok_mean, double* force,
                       void* workspace, size_t workspace_bytes, vmc_stream_t stream);

/* vmc_rbm_grad_stats without a caller workspace, for callers that cannot
 * allocate device memory at the point of the call (an XLA FFI handler, a
 * runtime with a fixed memory budget, code inside a stream capture).  No
 * counterpart in the reference: jVMC allocates through XLA.  The scratch is
 * a 32 MiB static device array inside the library (held by every GPU that
 * loads it until the process exits); problems needing more
 * (vmc_rbm_grad_stats_workspace_bytes > 32 MiB) are rejected with
 * VMC_ERR_UNSUPPORTED.  The first call on a device resolves the array's
 * address (cudaGetSymbolAddress) and should come before any stream capture.
 * All calls share the one array: calls that overlap on the GPU (different
 * streams, or different host threads) race and must be serialised by the
 * caller.  Results equal vmc_rbm_grad_stats's. */
int vmc_rbm_grad_stats_noalloc(int32_t precision, const int32_t* configs, int64_t num_configs, int32_t num_sites,
                               int32_t num_hidden, const void* kernel, const void* bias, const double* weights,
                               const double* eloc, const double* eloc_mean, double* ok_mean, double* force,
                               vmc_stream_t stream);

/* ------------------------------------------------------------------------
 * Centred, weighted data of the S/F build and of the SNR transform
 * (stats.py:197-205, 255-292; tdvp.py:134-181) for a CpxRBM.
 * ------------------------------------------------------------------------ */
typedef enum {
  VMC_DATA_C128 = 0,   /* (N, P) complex128                                   */
  VMC_DATA_C64 = 1,    /* (N, P) complex64                                    */
  VMC_DATA_BF16X2 = 2  /* bf16 hi (out) and lo (out_lo) planes of the real
                        * representation [Re | Im]: (2P, N) for gradients,
                        * (N, 2P) for SNR data; value ~ hi + lo            */
} vmc_data_format;

/* X_nk = sqrt(w_n) (O_nk - ok_mean_k), O in the compact layout; ld_out is
 * the leading dimension (elements) of the output rows (>= P for C128/C64,
 * >= N for the transposed BF16X2 planes). */
int vmc_rbm_centered_gradients(int32_t precision, const int32_t* configs, int64_t num_configs, int32_t num_sites,
                               int32_t num_hidden, const void* kernel, const void* bias, const double* weights,
                               const double* ok_mean, int32_t format, void* out, void* out_lo, int64_t ld_out,
                               vmc_stream_t stream);

/* H_nk = sqrt(w_n) ((neg_rhs) (E_n - Ebar) conj(O_nk - ok_mean_k) - force_k): the
 * per-sample data of covar_data(O, E).transform(makeReal(-x .)) before the
 * eigenbasis projection (tdvp.py:173-181); neg_rhs = -rhsPrefactor, force =
 * -rhsPrefactor * covar(O, E). */
int vmc_rbm_snr_data(int32_t precision, const int32_t* configs, int64_t num_configs, int32_t num_sites,
                     int32_t num_hidden, const void* kernel, const void* bias, const double* weights,
                     const double* ok_mean, const double* eloc, const double* eloc_mean, double neg_rhs_re,
                     double neg_rhs_im, const double* force, int32_t format, void* out, void* out_lo,
                     int64_t ld_out, vmc_stream_t stream);

/* ------------------------------------------------------------------------
 * TDVP solve helpers (util/tdvp.py:134-213), complex P-dimensional form.
 * ------------------------------------------------------------------------ */

/* Hermitian A (P x P, c128, both triangles) from the Gram matrix G of the
 * real representation [Re X | Im X] (2P x 2P, row-major, leading dimension
 * ld_gram, only row <= col read) with A_aa *= 1 + diag_shift. */
int vmc_gram_to_hermitian(int32_t gram_precision, const void* gram, int64_t ld_gram, int32_t num_params,
                          double diag_shift, double* A, vmc_stream_t stream);

/* y = U^H x (adjoint = 1) or y = U x (adjoint = 0); U column-major c128:
 * VtF = V^dagger F (tdvp.py:171) and update = V (pinv VtF)
 * (tdvp.py:211).
 * adjoint = 0 needs vmc_zgemv_workspace_bytes(n) of workspace (partial sums
 * over 256-wide chunks of k, added in a fixed order); adjoint = 1 needs none. */
size_t vmc_zgemv_workspace_bytes(int32_t n);
int vmc_zgemv(int32_t adjoint, const double* U, int64_t ld, int32_t n, const double* x, double* y, void* workspace,
              size_t workspace_bytes, vmc_stream_t stream);

/* The SNR of every eigenvector: snr_k = sqrt(|N |VtF_k|^2 / rhoVar_k|) with
 * rhoVar_k = colsq[k] (+ colsq[n + k] when real_rep), colsq the column sums of
 * |projected SNR data|^2 (tdvp.py:173-181). */
int vmc_tdvp_snr(const double* vtf, int32_t colsq_precision, const void* colsq, int32_t n, int32_t real_rep,
                 double num_samples, double* snr, double* rho_var, vmc_stream_t stream);

/* The regularised pseudo-inverse cutoff loop (tdvp.py:191-209) on the
 * device: pinv (n) and result[3] = {residual, cutoff used, iterations}.
 * snr NULL = exact sampling (no SNR factor). ev ascending.  Every candidate
 * cutoff is evaluated in parallel and the loop's stopping rule applied to
 * the residuals; workspace: vmc_tdvp_regularize_workspace_bytes(n,
 * pinv_cutoff) bytes. */
size_t vmc_tdvp_regularize_workspace_bytes(int32_t n, double pinv_cutoff);
int vmc_tdvp_regularize(const double* ev, const double* vtf, const double* snr, int32_t n, double pinv_cutoff,
                        double pinv_tol, double snr_tol, double* pinv, double* result, void* workspace,
                        size_t workspace_bytes, vmc_stream_t stream);

/* ------------------------------------------------------------------------
 * Split-precision BF16 contractions on the tcgen05 tensor cores (FP32
 * accumulation in TMEM): x ~ hi + lo, products hi.hi + hi.lo + lo.hi.
 * Operand planes are bf16, row-major with leading dimension ld (elements,
 * a multiple of 8, rows 16-byte aligned); the reduction index is contiguous.
 * products = 3 forms hi.hi + hi.lo + lo.hi; products = 1 forms hi.hi only
 * and does not read the lo planes (plain BF16, for accuracy studies).
 * Every wait inside these kernels is bounded (vmc_tc_set_wait_limit); a
 * wait that runs out writes a non-zero code to *status (a device int32 the
 * caller zeroes beforehand; NULL selects the library-wide flag read by
 * vmc_tc_error_flag) and the output is then incomplete.
 * ------------------------------------------------------------------------ */

/* S build (stats.py:52-58 via tdvp.py:142): gram = R R^T for R (rows x k)
 * given as hi/lo planes; fp32 output (rows x rows, leading dimension ld_gram,
 * a multiple of 4); only 128x256 tiles touching the upper triangle
 * (row <= col) are written; gram must be 16-byte aligned. */
int vmc_gram_bf16x3(const void* hi, const void* lo, int32_t rows, int32_t k, int64_t ld, float* gram,
                    int64_t ld_gram, int32_t products, int32_t* status, vmc_stream_t stream);

/* SNR transform (stats.py:75-83 via tdvp.py:175-179): colsq[c] =
 * sum_r (sum_j A[r][j] B[c][j])^2 for A (m x k) and B (n x k) given as hi/lo
 * planes; colsq (n floats) is overwritten; the product is never stored.
 * Partial sums per 128-row tile and warp go to the workspace
 * (vmc_gemm_bf16x3_colsq_workspace_bytes) and are added in a fixed order:
 * the result is bitwise reproducible. */
size_t vmc_gemm_bf16x3_colsq_workspace_bytes(int32_t m, int32_t n);
int vmc_gemm_bf16x3_colsq(const void* a_hi, const void* a_lo, int32_t m, int64_t lda, const void* b_hi,
                          const void* b_lo, int32_t n, int64_t ldb, int32_t k, float* colsq, void* workspace,
                          size_t workspace_bytes, int32_t products, int32_t* status, vmc_stream_t stream);

/* Library-wide error flag of the tensor-core kernels (a bounded wait that
 * ran out in a call given no status word); synchronises the device.
 * reset != 0 clears it.  No reference counterpart (XLA reports kernel
 * failures itself). */
int vmc_tc_error_flag(int32_t reset);

/* Limit (ns of %globaltimer, default 2e9) after which a wait of the
 * tensor-core kernels on the current device gives up; later launches use
 * it.  No reference counterpart. */
int vmc_tc_set_wait_limit(uint64_t limit_ns);

/* Check of the bounded-wait path: one thread waits limit_ns (<= 1 s) on a
 * barrier that nothing completes and writes code 6 to *status.  No
 * reference counterpart (failure detection of this library). */
int vmc_tc_wait_check(uint64_t limit_ns, int32_t* status, vmc_stream_t stream);

/* FP64-accurate complex product on the BF16 tensor cores (Ozaki split):
 * C = op(A) op(B) (+ C when accumulate != 0), A, B, C complex128
 * column-major; trans_a 'C' (67): op(A) = A^H with A k x m; 'N' (78):
 * op(A) = A with A m x k; trans_b 'N': op(B) = B with B k x n; 'C':
 * op(B) = B^H with B n x k.  Every operand column is scaled by a power of two and cut into
 * `slices` (1..8) slices of 7 bits; slice pairs up to level max_level
 * (<= 2 (slices - 1)) are summed exactly (FP32 tensor-core groups that stay
 * below 2^24 units, int64 sums).  slices 8, max_level 7 give entries
 * within ~2^-48 of the row and column scales.  hermitian != 0: the caller
 * asserts C is Hermitian (m == n); only blocks on or above the diagonal
 * are computed and the rest mirrored.  k <= 30720.  Workspace from
 * vmc_zgemm_ozaki_workspace_bytes (256-byte aligned); *status as for the
 * other tensor-core kernels.  Replaces the O(n^3) products of the
 * eigendecomposition behind tdvp.py:157 (jnp.linalg.eigh). */
size_t vmc_zgemm_ozaki_workspace_bytes(int32_t m, int32_t n, int32_t k, int32_t slices);
int vmc_zgemm_ozaki(int32_t trans_a, int32_t trans_b, int32_t m, int32_t n, int32_t k, const double* A,
                    int64_t lda, const double* B, int64_t ldb, double* C, int64_t ldc, int32_t hermitian,
                    int32_t accumulate, int32_t slices, int32_t max_level, void* workspace, size_t workspace_bytes,
                    int32_t* status, vmc_stream_t stream);

/* Eigendecomposition of the Hermitian S of the TDVP solve (tdvp.py:153-171,
 * jnp.linalg.eigh), first stage: the complex64 eigendecomposition of A
 * (n x n complex128, column-major) by cuSOLVER; ev (n, ascending) and V
 * (n x n complex128, column-major, ldv) receive the FP32 values and vectors
 * widened.  *info (device int32) is cuSOLVER's status (0: converged). */
size_t vmc_eigh_fp32_workspace_bytes(int32_t n);
int vmc_eigh_fp32(int32_t n, const double* A, int64_t lda, double* ev, double* V, int64_t ldv, void* workspace,
                  size_t workspace_bytes, int32_t* info, vmc_stream_t stream);

/* FP64 eigendecomposition (tdvp.py:157, jnp.linalg.eigh in FP64; the FP64
 * and plain-FP32 forms, ExactSampler steps, MinSR's pseudo-inverse):
 * cuSOLVER on A (n x n, column-major, complex128 when is_complex != 0, else
 * float64), eigenvalues ascending into ev, eigenvectors into V (A is copied
 * into V first; A may be V).  *info: cuSOLVER's status. */
size_t vmc_eigh_fp64_workspace_bytes(int32_t n, int32_t is_complex);
int vmc_eigh_fp64(int32_t n, int32_t is_complex, const double* A, int64_t lda, double* ev, double* V, int64_t ldv,
                  void* workspace, size_t workspace_bytes, int32_t* info, vmc_stream_t stream);

/* Second stage: on entry ev, V from vmc_eigh_fp32 for the same A.  The k
 * eigenpairs of largest eigenvalue become FP64-accurate: power_steps
 * products X <- A X diag(1/ev) of the top-k vectors, then Rayleigh-Ritz in
 * FP64 (G = X^H X and H = X^H A X as FP64-accurate Ozaki products, the
 * k x k problem H c = theta G c by cuSOLVER zhegvd, V_top = X C).  The other
 * n - k columns of V are made orthogonal to V_top (one Gram-Schmidt pass)
 * and renormalised; their eigenvalues keep the FP32 values.  n <= 30720.
 * *info: zhegvd's status (> k: X^H X not positive definite, when the power
 * steps have made the columns nearly dependent -- the ratio
 * (ev_max / ev_(n-k))^power_steps is too large; the caller then uses
 * vmc_eigh_fp64 and V is not to be used); *status as for the tensor-core
 * kernels.  Replaces the FP64 jnp.linalg.eigh of tdvp.py:157 for the
 * eigenpairs that carry the regularised solve. */
size_t vmc_eigh_refine_workspace_bytes(int32_t n, int32_t k);
int vmc_eigh_refine_top(int32_t n, const double* A, int64_t lda, int32_t k, int32_t power_steps, double* ev,
                        double* V, int64_t ldv, void* workspace, size_t workspace_bytes, int32_t* status,
                        int32_t* info, vmc_stream_t stream);

/* Operand of the SNR transform (tdvp.py:175-179): B^T planes (2P x 2P,
 * leading dimension ld) of the real representation
 * [[Re U, -Im U], [Im U, Re U]] of the eigenvectors U (P x P, column-major
 * c128, leading dimension ldu), split into bf16 hi/lo: the B operand of the
 * SNR contraction. */
int vmc_eigvec_bf16x2(const double* U, int64_t ldu, int32_t num_params, void* bt_hi, void* bt_lo, int64_t ld,
                      vmc_stream_t stream);

/* ------------------------------------------------------------------------
 * Real CNN (nets/cnn.py:18-83): periodic padding (0, F-1), VALID
 * cross-correlation with HWIO kernels, unit strides, activation after every
 * layer (0: x^2/2 - x^4/12, 1: poly6, 2: x^2, 3: poly5), output
 * sum / sqrt(#elements).  Parameters: one flat real array (f64 or f32) in
 * jVMC's leaf order -- per layer Conv_l/bias (if present) then Conv_l/kernel
 * raveled (F..., C_in, C_out).  Configurations: (N, dims...) row-major.
 * ------------------------------------------------------------------------ */
typedef struct {
  int32_t ndim;           /* 1 or 2                                      */
  int32_t dims[2];        /* lattice extent(s)                           */
  int32_t filter[2];      /* filter diameter(s)                          */
  int32_t num_layers;     /* 1..4                                        */
  int32_t channels[4];
  int32_t activation[4];
  int32_t has_bias[4];
} vmc_cnn_desc;

/* Number of real parameters of the network (-1 on an invalid descriptor). */
int vmc_cnn_num_params(const vmc_cnn_desc* desc);

/* log psi (real, returned as c128 with imaginary part 0); replaces
 * NQS._eval for a CNN (vqs.py:242-251, cnn.py:41-81). */
int vmc_cnn_logpsi(int32_t precision, const vmc_cnn_desc* desc, const int32_t* configs, int64_t num_configs,
                   const void* params, double* log_psi, vmc_stream_t stream);

/* d log psi / d theta per configuration by a hand-written backward pass that
 * recomputes the activations of each configuration in shared memory
 * (flat_gradient, vqs.py:46-51).  layout VMC_GRAD_REFERENCE: (N, P) c128
 * with imaginary part 0; VMC_GRAD_COMPACT: (N, P) f64. */
int vmc_cnn_gradients(int32_t precision, const vmc_cnn_desc* desc, const int32_t* configs, int64_t num_configs,
                      const void* params, int32_t layout, double* out, vmc_stream_t stream);

/* Metropolis sampling for the CNN (MCSampler._get_samples / _sweep with
 * propose_spin_flip, sampler.py:264-358): one warp per chain keeps every
 * layer's activations; a proposal recomputes only the region of each layer
 * that the flipped site reaches ((l+1)(F-1)+1 sites per dimension for layer
 * l), with the operations and order of a full evaluation, and accepts iff
 * u < exp(mu delta log psi).  Random stream and arguments as
 * vmc_rbm_metropolis. */
int vmc_cnn_metropolis(int32_t precision, const vmc_cnn_desc* desc, int32_t* states, int32_t num_chains,
                       const void* params, double mu, uint64_t seed, uint32_t call_index, int64_t therm_steps,
                       int64_t sweep_steps, int64_t samples_per_chain, int32_t* configs_out, void* counters,
                       vmc_stream_t stream);

/* O_loc of a branch-free operator for the CNN without forming s'
 * (Operator.get_O_loc, base.py:162-192): psi(s')/psi(s) = exp(delta log psi)
 * from the same local updates (a string flipping n sites: n updates applied
 * in turn, then undone).  log_psi_s as vmc_rbm_oloc_fused. */
int vmc_cnn_oloc_fused(int32_t precision, const vmc_cnn_desc* desc, const int32_t* configs, int64_t num_configs,
                       const void* params, const vmc_bf_operator* op, const double* log_psi_s, double* oloc,
                       vmc_stream_t stream);

/* ---------------------------------------------------------------------------
 * The same statistics and data from materialised log-derivatives O (N, P)
 * complex128 (compact layout, row stride ld_gradients elements) of any
 * holomorphic network (e.g. vmc_sym_rbm_gradients output), so that its S/F
 * build and SNR transform run through the same Gram / eigen / SNR entry
 * points as the CpxRBM's (stats.py:50-58, 197-205, 255-292; tdvp.py:134-181).
 * ------------------------------------------------------------------------- */
size_t vmc_dense_grad_stats_workspace_bytes(int64_t num_configs, int64_t num_params);

/* ok_mean_k = sum_n w_n O_nk, force_k = sum_n w_n conj(O_nk - ok_mean_k)
 * (E_n - Ebar) = covar(O, E) (fixed-order reductions). */
int vmc_dense_grad_stats(const double* gradients, int64_t ld_gradients, int64_t num_configs, int64_t num_params,
                         const double* weights, const double* eloc, const double* eloc_mean, double* ok_mean,
                         double* force, void* workspace, size_t workspace_bytes, vmc_stream_t stream);

/* X as vmc_rbm_centered_gradients, from O. */
int vmc_dense_centered_gradients(const double* gradients, int64_t ld_gradients, int64_t num_configs,
                                 int64_t num_params, const double* weights, const double* ok_mean, int32_t format,
                                 void* out, void* out_lo, int64_t ld_out, vmc_stream_t stream);

/* H as vmc_rbm_snr_data, from O.  real_part != 0 (real-parameter nets,
 * makeReal = Re): H_nk = sqrt(w_n) (Re((-x) (E_n - Ebar) conj(O_nk -
 * ok_mean_k)) - Re force_k), imaginary part 0. */
int vmc_dense_snr_data(const double* gradients, int64_t ld_gradients, int64_t num_configs, int64_t num_params,
                       const double* weights, const double* ok_mean, const double* eloc, const double* eloc_mean,
                       double neg_rhs_re, double neg_rhs_im, const double* force, int32_t real_part, int32_t format,
                       void* out, void* out_lo, int64_t ld_out, vmc_stream_t stream);

/* ---------------------------------------------------------------------------
 * Symmetrised CpxRBM (nets/sym_wrapper.py:22-64 over nets/rbm.py:17-38;
 * orbits of util/symmetries.py).
 *
 * `orbit` (num_sym, L) int32 holds codes 2 * src + flip: site i of the
 * transformed configuration tau(s) is s[src] (flip 0) or 1 - s[src] (flip 1),
 * i.e. row i of the reference's orbit matrix o_tau has its one nonzero entry
 * (+1 or -1) in column src, and tau(s) = (o_tau (2s - 1) + 1) // 2
 * (sym_wrapper.py:51-54).  `inverse` (num_sym, L) int32 holds, for each site
 * j, the position i of tau(s) with src = j; the orbit must consist of signed
 * permutations.  `factor` (num_sym) complex128.
 * VMC_SYM_EXP: log psi = log sum_tau factor_tau exp(log psi_RBM(tau s)), in
 * the form of jax.scipy.special.logsumexp(., b=factor) (avgFun_Coefficients_Exp,
 * sym_wrapper.py:7-9); VMC_SYM_LOG: the mean of log psi_RBM(tau s)
 * (avgFun_Coefficients_Log, sym_wrapper.py:12-13; factor unused).
 * Malformed codes or inverse entries make the affected outputs NaN.
 * ------------------------------------------------------------------------- */
typedef enum { VMC_SYM_EXP = 0, VMC_SYM_LOG = 1 } vmc_sym_average;

typedef struct {
  int32_t num_sym;          /* orbit size, 1..4096 */
  int32_t average;          /* vmc_sym_average */
  const int32_t* orbit;     /* (num_sym, L) codes */
  const int32_t* inverse;   /* (num_sym, L) */
  const double* factor;     /* (num_sym) complex128 */
} vmc_sym_desc;

/* log psi of the symmetrised net; replaces NQS._eval for a SymNet
 * (vqs.py:242-251, sym_wrapper.py:48-60).  Output (N) complex128. */
int vmc_sym_rbm_logpsi(int32_t precision, const int32_t* configs, int64_t num_configs, int32_t num_sites,
                       int32_t num_hidden, const void* kernel, const void* bias, const vmc_sym_desc* sym,
                       double* log_psi, vmc_stream_t stream);

/* d log psi / d theta = sum_tau w_tau O_k(tau s), w_tau = factor_tau
 * psi_RBM(tau s) / psi(s) (Exp) or 1/num_sym (Log); the holomorphic gradient
 * of sym_wrapper.py:48-60 (flat_gradient_holo, vqs.py:66-69).  Layouts as
 * vmc_rbm_gradients. */
int vmc_sym_rbm_gradients(int32_t precision, const int32_t* configs, int64_t num_configs, int32_t num_sites,
                          int32_t num_hidden, const void* kernel, const void* bias, const vmc_sym_desc* sym,
                          int32_t layout, double* out, vmc_stream_t stream);

/* O_loc of a branch-free operator for the symmetrised net without forming s'
 * (Operator.get_O_loc, base.py:162-192): psi(s')/psi(s) = sum_tau w_tau
 * psi_RBM(tau s') / psi_RBM(tau s), each ratio a product over hidden units
 * from the tables of vmc_rbm_prepare.  VMC_SYM_EXP only (VMC_ERR_UNSUPPORTED
 * otherwise).  log_psi_s as vmc_rbm_oloc_fused. */
int vmc_sym_rbm_oloc_fused(int32_t precision, const int32_t* configs, int64_t num_configs, int32_t num_sites,
                           int32_t num_hidden, const void* kernel, const void* bias, const void* tables,
                           const vmc_sym_desc* sym, const vmc_bf_operator* op, const double* log_psi_s,
                           double* oloc, vmc_stream_t stream);

/* Metropolis sampling of |psi_sym|^mu with single spin flips
 * (MCSampler._get_samples / _sweep with propose_spin_flip,
 * sampler.py:264-358); one thread block per chain keeps tanh(theta) of every
 * orbit element in shared memory (num_sym * num_hidden complex values must
 * fit, else VMC_ERR_UNSUPPORTED).  Random stream, arguments and outputs as
 * vmc_rbm_metropolis. */
int vmc_sym_rbm_metropolis(int32_t precision, int32_t* states, int32_t num_chains, int32_t num_sites,
                           int32_t num_hidden, const void* kernel, const void* bias, const void* tables,
                           const vmc_sym_desc* sym, double mu, uint64_t seed, uint32_t call_index,
                           int64_t therm_steps, int64_t sweep_steps, int64_t samples_per_chain, int32_t* configs_out,
                           void* counters, vmc_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* VMC_GB300_H */
