/* oracle.h -- CPU oracle for column-major variable-size batched SGEMM.
 * Test infrastructure only (see oracle.c for the restated semantics). */
#ifndef BGEMM_ORACLE_H
#define BGEMM_ORACLE_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { BGO_MODE_SIMT_FP32 = 0, BGO_MODE_TF32 = 1, BGO_MODE_TF32X3 = 2, BGO_MODE_BF16X3 = 3 };

void bgo_sgemm_f32(int M, int N, int K, float alpha, const float* A, int lda,
                   const float* B, int ldb, float beta, float* C, int ldc);
void bgo_sgemm_f64(int M, int N, int K, double alpha, const float* A, int lda,
                   const float* B, int ldb, double beta, const float* C0,
                   int ldc, double* C64, double* absbound);
float bgo_round_tf32(float x);
float bgo_round_bf16(float x);
void bgo_split(int mode, const float* x, size_t n, float* hi, float* lo);
void bgo_sgemm_split_f64(int mode, int M, int N, int K, double alpha,
                         const float* A, int lda, const float* B, int ldb,
                         double beta, const float* C0, int ldc, double* C64);
int bgo_vbatched_f32(int batch, const int* M, const int* N, const int* K,
                     float alpha, const float* const* A, const int* lda,
                     const float* const* B, const int* ldb, float beta,
                     float* const* C, const int* ldc, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
