/*
 * frico_gpu_debug.h -- diagnostic entry points of libfrico_gpu, outside the
 * public C-ABI (include/frico_gpu.h). They expose internal kernels so that the
 * tests can check them on their own; a FRICO integration never calls them.
 */
#ifndef FRICO_GPU_DEBUG_H
#define FRICO_GPU_DEBUG_H

#include "frico_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* C -= A B with the LU's complex64 trailing-update kernel (engine
 * FRICO_GEMM_SIMT, FRICO_GEMM_TC: 3xTF32 operands, or FRICO_GEMM_TC_F16:
 * 3xFP16 operands); A m x k (ld m), B k x n (ld k), C m x n (ld m),
 * column-major host buffers. */
int frico_gpu_debug_cgemm(frico_gpu_ctx* ctx, int32_t m, int32_t n, int32_t k, const frico_c64* A,
                          const frico_c64* B, frico_c64* C, int32_t engine);

/* Device address of the resident FP64 Z (n x n complex128, column-major,
 * leading dimension *ld = n), valid until the next call on ctx; ESTATE when no
 * Z is resident (before a fill, or after an FP64 factorisation overwrote it).
 * For checks that multiply with Z on the device without copying it out. */
int frico_gpu_debug_z64(frico_gpu_ctx* ctx, const void** dev_ptr, int64_t* ld);

/* The far-field GEMM form's triangles per launch (kc, a multiple of 16) and k-steps per
 * tensor-core accumulator before its move to double-float sums (group: 1, 2 or 4); 0
 * restores a default. Process-wide, for accuracy and speed studies. */
int frico_gpu_debug_fields_gemm_config(int32_t kc, int32_t group);

#ifdef __cplusplus
}
#endif
#endif /* FRICO_GPU_DEBUG_H */
