/*
 * oracle.c -- CPU restatement of the reference's column-major variable-size
 * batched SGEMM.  TEST INFRASTRUCTURE ONLY: the tests, the smoke check and the
 * bench's CPU-baseline leg call it as the checker; the product path never
 * links, loads or falls back to it.
 *
 * What it restates (reference paths are relative to the BatchGEMM project):
 *
 *  - Layout and call convention: cublasSgemm(N, N, M, N, K, alpha, A, M, B, K,
 *    beta, C, M) as issued per matrix by CUDA/default/gemm.cu:84-88, i.e.
 *    column-major, element (m,k) of A at A[m + k*lda], (k,n) of B at
 *    B[k + n*ldb], (m,n) of C at C[m + n*ldc].
 *
 *  - Accumulation order: every tile body of the reference keeps one FP32
 *    register per output element and applies fma(a_mk, b_kn, acc) for
 *    k = 0, 1, ..., K-1 in order (e.g. CUDA/batching/kernel_256.h:37,
 *    CUDA/batching/kernel_256.h:87-90, CUDA/framework/kernel_128_new.h:176-183).
 *
 *  - In-place semantics: the reference kernels load C into the accumulator
 *    before the k-loop and store it back afterwards
 *    (CUDA/framework/kernel_128_new.h:147-148,199-200,
 *    CUDA/batching/kernel_256.h:13,51), i.e. C += A*B (alpha = beta = 1).
 *
 * General alpha/beta are defined so that alpha = beta = 1 is exactly that
 * in-place chain:
 *    alpha == 1 && beta == 1 : acc = C;   acc = fmaf(a, b, acc) over k;  C = acc
 *    otherwise               : acc = 0;   acc = fmaf(a, b, acc) over k;
 *                              C = (beta == 0) ? alpha*acc            (C not read)
 *                                              : fmaf(alpha, acc, beta*C)
 * The CUDA SIMT path implements the same formula, so it is bit-exact with
 * this file.  FP64 variants are the error oracle of the tensor-core modes.
 *
 * Build with -ffp-contract=off: every fused multiply-add below is explicit.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

/* ------------------------------------------------------------------------ */
/* FP32 / FP64 single-matrix kernels                                         */
/* ------------------------------------------------------------------------ */

void bgo_sgemm_f32(int M, int N, int K, float alpha, const float* A, int lda,
                   const float* B, int ldb, float beta, float* C, int ldc) {
  if (M <= 0 || N <= 0) return;
  const int inplace = (alpha == 1.0f && beta == 1.0f);
  float* acc = (float*)malloc(sizeof(float) * (size_t)M);
  for (int n = 0; n < N; ++n) {
    float* c = C + (size_t)n * ldc;
    if (inplace)
      memcpy(acc, c, sizeof(float) * (size_t)M);
    else
      memset(acc, 0, sizeof(float) * (size_t)M);
    /* k outer, m inner: each element still sees its own k-ordered fma chain;
     * the m loop is independent per element and vectorises. */
    for (int k = 0; k < K; ++k) {
      const float b = B[(size_t)n * ldb + k];
      const float* a = A + (size_t)k * lda;
      for (int m = 0; m < M; ++m) acc[m] = fmaf(a[m], b, acc[m]);
    }
    if (inplace) {
      memcpy(c, acc, sizeof(float) * (size_t)M);
    } else if (beta == 0.0f) {
      for (int m = 0; m < M; ++m) c[m] = alpha * acc[m];
    } else {
      for (int m = 0; m < M; ++m) c[m] = fmaf(alpha, acc[m], beta * c[m]);
    }
  }
  free(acc);
}

void bgo_sgemm_f64(int M, int N, int K, double alpha, const float* A, int lda,
                   const float* B, int ldb, double beta, const float* C0,
                   int ldc, double* C64, double* absbound) {
  if (M <= 0 || N <= 0) return;
  double* acc = (double*)malloc(sizeof(double) * (size_t)M);
  double* aab = (double*)malloc(sizeof(double) * (size_t)M);
  for (int n = 0; n < N; ++n) {
    memset(acc, 0, sizeof(double) * (size_t)M);
    memset(aab, 0, sizeof(double) * (size_t)M);
    for (int k = 0; k < K; ++k) {
      const double b = (double)B[(size_t)n * ldb + k];
      const float* a = A + (size_t)k * lda;
      for (int m = 0; m < M; ++m) {
        acc[m] += (double)a[m] * b;
        aab[m] += fabs((double)a[m] * b);
      }
    }
    for (int m = 0; m < M; ++m) {
      const double c0 = (beta != 0.0) ? (double)C0[(size_t)n * ldc + m] : 0.0;
      C64[(size_t)n * M + m] = alpha * acc[m] + beta * c0;
      if (absbound)
        absbound[(size_t)n * M + m] = fabs(alpha) * aab[m] + fabs(beta * c0);
    }
  }
  free(acc);
  free(aab);
}

/* ------------------------------------------------------------------------ */
/* Split-precision operand rounding (tensor-core modes)                      */
/* ------------------------------------------------------------------------ */

static inline uint32_t f2u(float x) { uint32_t u; memcpy(&u, &x, 4); return u; }
static inline float u2f(uint32_t u) { float x; memcpy(&x, &u, 4); return x; }

/* Round to nearest, ties to even, keeping `keep` explicit mantissa bits
 * (TF32: 10, BF16: 7).  Inf and NaN pass through unchanged. */
static inline float round_keep(float x, int drop) {
  uint32_t u = f2u(x);
  if ((u & 0x7f800000u) == 0x7f800000u) return x;
  const uint32_t half = (1u << (drop - 1)) - 1u;
  const uint32_t lsb = (u >> drop) & 1u;
  u += half + lsb;
  u &= ~((1u << drop) - 1u);
  return u2f(u);
}

float bgo_round_tf32(float x) { return round_keep(x, 13); }
float bgo_round_bf16(float x) { return round_keep(x, 16); }

void bgo_split(int mode, const float* x, size_t n, float* hi, float* lo) {
  for (size_t i = 0; i < n; ++i) {
    float h, l;
    if (mode == BGO_MODE_BF16X3) {
      h = bgo_round_bf16(x[i]);
      l = isfinite(x[i]) ? bgo_round_bf16(x[i] - h) : 0.0f;
    } else {
      h = bgo_round_tf32(x[i]);
      l = isfinite(x[i]) ? bgo_round_tf32(x[i] - h) : 0.0f;
    }
    hi[i] = h;
    if (lo) lo[i] = (mode == BGO_MODE_TF32) ? 0.0f : l;
  }
}

/* Exact (FP64) value of the products a tensor-core mode forms:
 *   TF32   : hi(a)*hi(b)
 *   TF32X3 : hi(a)*hi(b) + hi(a)*lo(b) + lo(a)*hi(b), plus lo(a)*lo(b) when
 *            K <= 64 (short inner products, where the split error dominates)
 *   BF16X3 : the same with bfloat16 halves.
 * Every product of two rounded halves is exact in FP64 and K <= 2^20 keeps
 * the FP64 sum far below FP32 resolution, so the only gap left between this
 * and the device result is the tensor core's own FP32 accumulation. */
void bgo_sgemm_split_f64(int mode, int M, int N, int K, double alpha,
                         const float* A, int lda, const float* B, int ldb,
                         double beta, const float* C0, int ldc, double* C64) {
  if (M <= 0 || N <= 0) return;
  float* ah = (float*)malloc(sizeof(float) * (size_t)M * (K > 0 ? K : 1));
  float* al = (float*)malloc(sizeof(float) * (size_t)M * (K > 0 ? K : 1));
  float* bh = (float*)malloc(sizeof(float) * (size_t)(K > 0 ? K : 1));
  float* bl = (float*)malloc(sizeof(float) * (size_t)(K > 0 ? K : 1));
  double* acc = (double*)malloc(sizeof(double) * (size_t)M);
  for (int k = 0; k < K; ++k)
    bgo_split(mode, A + (size_t)k * lda, (size_t)M, ah + (size_t)k * M,
              al + (size_t)k * M);
  for (int n = 0; n < N; ++n) {
    bgo_split(mode, B + (size_t)n * ldb, (size_t)K, bh, bl);
    memset(acc, 0, sizeof(double) * (size_t)M);
    for (int k = 0; k < K; ++k) {
      const double bhk = bh[k], blk = bl[k];
      const float* aH = ah + (size_t)k * M;
      const float* aL = al + (size_t)k * M;
      for (int m = 0; m < M; ++m) {
        double p = (double)aH[m] * bhk;
        if (mode != BGO_MODE_TF32) {
          p += (double)aH[m] * blk + (double)aL[m] * bhk;
          if (K <= 64) p += (double)aL[m] * blk;
        }
        acc[m] += p;
      }
    }
    for (int m = 0; m < M; ++m) {
      const double c0 = (beta != 0.0) ? (double)C0[(size_t)n * ldc + m] : 0.0;
      C64[(size_t)n * M + m] = alpha * acc[m] + beta * c0;
    }
  }
  free(ah); free(al); free(bh); free(bl); free(acc);
}

/* ------------------------------------------------------------------------ */
/* Multi-threaded batched driver (the CPU baseline)                          */
/* ------------------------------------------------------------------------ */

typedef struct {
  int batch;
  const int *M, *N, *K, *lda, *ldb, *ldc;
  float alpha, beta;
  const float* const* A;
  const float* const* B;
  float* const* C;
  const int* order;
  volatile int next;
  pthread_mutex_t mu;
} vb_job;

static void* vb_worker(void* p) {
  vb_job* j = (vb_job*)p;
  for (;;) {
    pthread_mutex_lock(&j->mu);
    const int t = j->next++;
    pthread_mutex_unlock(&j->mu);
    if (t >= j->batch) break;
    const int i = j->order[t];
    bgo_sgemm_f32(j->M[i], j->N[i], j->K[i], j->alpha, j->A[i], j->lda[i],
                  j->B[i], j->ldb[i], j->beta, j->C[i], j->ldc[i]);
  }
  return NULL;
}

static const int* g_sort_M;
static const int* g_sort_N;
static const int* g_sort_K;
static int cmp_flops_desc(const void* x, const void* y) {
  const int a = *(const int*)x, b = *(const int*)y;
  const double fa = (double)g_sort_M[a] * g_sort_N[a] * g_sort_K[a];
  const double fb = (double)g_sort_M[b] * g_sort_N[b] * g_sort_K[b];
  if (fa > fb) return -1;
  if (fa < fb) return 1;
  return a - b;
}

int bgo_vbatched_f32(int batch, const int* M, const int* N, const int* K,
                     float alpha, const float* const* A, const int* lda,
                     const float* const* B, const int* ldb, float beta,
                     float* const* C, const int* ldc, int nthreads) {
  if (batch <= 0) return 0;
  if (nthreads < 1) nthreads = 1;
  int* order = (int*)malloc(sizeof(int) * (size_t)batch);
  for (int i = 0; i < batch; ++i) order[i] = i;
  /* largest first: the same longest-processing-time order the device queue uses */
  g_sort_M = M; g_sort_N = N; g_sort_K = K;
  qsort(order, (size_t)batch, sizeof(int), cmp_flops_desc);
  vb_job job;
  job.batch = batch; job.M = M; job.N = N; job.K = K;
  job.lda = lda; job.ldb = ldb; job.ldc = ldc;
  job.alpha = alpha; job.beta = beta; job.A = A; job.B = B; job.C = C;
  job.order = order; job.next = 0;
  pthread_mutex_init(&job.mu, NULL);
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
  int started = 0;
  for (int t = 1; t < nthreads; ++t) {
    pthread_t tid;
    if (pthread_create(&tid, NULL, vb_worker, &job) == 0) th[started++] = tid;
  }
  vb_worker(&job);
  for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
  pthread_mutex_destroy(&job.mu);
  free(th);
  free(order);
  return started + 1;
}
