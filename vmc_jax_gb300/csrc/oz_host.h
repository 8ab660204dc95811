// Host interface of the FP64-accurate complex products (gemm_tc.cu), used
// by the eigensolver (eigh.cu).  C = P^H Q for complex P (K x rows of the A
// operand) and Q (K x rows of the B operand), both given in FP64.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace vmc {

// Operand cut into `slices` bf16 planes of 7-bit slices with one power-of-two
// scale per row, in a caller-provided buffer of oz_operand_bytes bytes.
struct oz_operand {
  __nv_bfloat16* planes;
  int* exps;
  int rows;      // rows of the operand (columns of P or Q)
  int rowsHalf;  // rows padded to 128
  int rowsP;     // rows of one plane (2 rowsHalf for the B operand)
  int K, slices;
  int64_t K2p;   // 2K padded to 64
};

size_t oz_operand_bytes(int rows, int K, int slices, bool bRole);
int oz_make_operand(void* buf, int rows, int K, int slices, bool bRole, oz_operand& op);

// Slice P[k][m] = (conj ? conj(z) : z) with z = Z[k sk + m sm] (complex128
// elements), k < op.K, m < op.rows.  bRole: the B operand of a product.
int oz_slice(const double* Z, int64_t sk, int64_t sm, int conj, oz_operand& op, bool bRole, cudaStream_t st);

// Product of two sliced operands, slice pairs of level <= maxLevel; `out`
// holds A.rows x 2 B.rowsHalf doubles (Re | Im).  hermitian: only the blocks
// on or above the diagonal (square products).
int oz_multiply(const oz_operand& A, const oz_operand& B, int maxLevel, bool hermitian, double* out, int* status,
                cudaStream_t st);
inline size_t oz_out_bytes(int rowsA, int rowsB) {
  return (size_t)rowsA * 2 * (((size_t)rowsB + 127) / 128 * 128) * 8;
}

// C (A.rows x B.rows complex128, column-major, ldc) = alpha product
// (+ C when accumulate).
int oz_finish(const double* out, const oz_operand& A, const oz_operand& B, bool hermitian, double* C, int64_t ldc,
              bool accumulate, cudaStream_t st, double alpha);

}  // namespace vmc
