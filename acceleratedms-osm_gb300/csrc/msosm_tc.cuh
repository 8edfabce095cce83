// Tensor-core pieces of the MS-OSM engine (see msosm_tc.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace msosm {

// The 16 KB W_32 operand image of the split-precision transform (hi then lo parts,
// FP16 or BF16 when bf16 != 0) into device memory `dst`.
cudaError_t tc_build_operand(void *dst, int bf16, cudaStream_t st);

// Raise *out (float bits) to the largest |component| of the n complex values at p
// (16-byte aligned, n even).
cudaError_t tc_absmax(const float2 *p, size_t n, unsigned *out, cudaStream_t st);

// Operand-layout self-test: D[m][j] = sum_k A[m][k] * B[b_row0 + j][k] for m < 128,
// j < n (n = 32 or 64), k < 64, with A (128 x 64) and B (64 x 64) row-major 16-bit
// values (FP16, or BF16 when bf16 != 0) in host memory, D in host memory.
cudaError_t tc_selftest_umma(int bf16, int n, int b_row0, const uint16_t *A, const uint16_t *B, float *D,
                             int *timed_out);

} // namespace msosm
