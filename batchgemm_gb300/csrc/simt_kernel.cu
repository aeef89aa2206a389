// simt_kernel.cu -- persistent FP32 SIMT kernel for column-major vbatched SGEMM.
//
// Replaces the reference's dense-grid dispatcher (CUDA/framework/kernel.h:11-43,
// launched over (max tiles M, max tiles N, batch) at CUDA/framework/gemm.cu:181-200)
// and its tile bodies (CUDA/framework/kernel_128_new.h, kernel_256_new.h,
// CUDA/batching/kernel_256.h): one wave of persistent CTAs pulls work items
// from a largest-first tile queue with an atomic counter, so no CTA is
// launched for a tile outside its matrix.
//
// Each item is one BM x BN output tile of one matrix.  256 threads form a
// 16 x 16 grid; each owns a TM x TN register tile (the thin 8 x 128 and
// 128 x 8 tiles, simt_thin, give each thread four outputs along the thin
// side instead).  Operands stream through a
// cp.async ring of BK = 16 k-slices (4 stages for 128 x 128 tiles, up to the
// autotuned kSimtRingCap for smaller ones):
//   A slice: [k][BM]     (column of A, 16-byte cp.async when lda % 4 == 0 and
//                         A is 16-byte aligned, 4-byte otherwise)
//   B slice: [k][BN + 4] (transposed on the way in by 4-byte cp.async; the
//                         +4 pad keeps the scattered writes conflict-free)
// Plans with transposed operands run simt_persistent_kernel_t: an operand
// whose slice rows are contiguous in memory (A, or B stored N x K) takes the
// A path above, one contiguous along k (B, or A stored K x M) the B path, and
// the A slice is padded to [k][BM + 4] as well.
// Edges are zero-filled by the cp.async source size, so any M, N, K >= 0 and
// any leading dimension work.  Every output element is a single fma chain
// over k in order (bit-exact with the reference's tile bodies and with the
// oracle).  The epilogue stores float4 columns when C allows it; otherwise a
// warp-shuffle transpose turns each half-warp's 4-element runs into
// contiguous 64-byte stores.
#include <stdint.h>

#include "bgemm_internal.h"
#include "tile_table.h"

namespace bgemm {
namespace {

constexpr int kThreads = 256;
constexpr int kBK = 16;
constexpr int kStages = 4;  // ring stages of the largest (128 x 128) tile
constexpr int kPadB = 4;
constexpr int kMaxStageFloats = kBK * (128 + 128 + kPadB);
constexpr int kSmemBytes = kStages * kMaxStageFloats * 4;
constexpr int kSmemBytesT = kStages * kBK * (128 + kPadB + 128 + kPadB) * 4;  // transposed kernel
static_assert(kSimtRingCap >= kStages && kSimtRingCap <= 32, "SIMT ring cap out of range");

// Stages of the cp.async ring for a tile whose stage holds `stage` floats: as
// many as the kernel's shared memory holds, at most kSimtRingCap (autotuned).
template <bool GEN>
__host__ __device__ constexpr int ring_stages(int stage) {
  return ((GEN ? kSmemBytesT : kSmemBytes) / 4 / stage) < kSimtRingCap
             ? (GEN ? kSmemBytesT : kSmemBytes) / 4 / stage
             : kSimtRingCap;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, int src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src),
               "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async4(uint32_t dst, const void* src, int src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(dst), "l"(src),
               "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <int W>
struct VecLd;
template <>
struct VecLd<1> {
  static __device__ __forceinline__ void ld(const float* p, float* v) { v[0] = p[0]; }
};
template <>
struct VecLd<2> {
  static __device__ __forceinline__ void ld(const float* p, float* v) {
    const float2 t = *reinterpret_cast<const float2*>(p);
    v[0] = t.x; v[1] = t.y;
  }
};
template <>
struct VecLd<4> {
  static __device__ __forceinline__ void ld(const float* p, float* v) {
    const float4 t = *reinterpret_cast<const float4*>(p);
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  }
};

// Slice k0 .. k0+kBK-1 of R operand rows r0 .. r0+R-1 into s[k][LDS] when
// element (r, k) sits at X[r + k*ldx] (rows contiguous).  Out-of-range
// elements are zero-filled through the cp.async source size.
template <int R, int LDS>
__device__ __forceinline__ void load_rows_contig(const float* X, long long ldx, int rows, int r0,
                                                 int k0, int K, float* s, bool vec, int tid) {
  if (vec) {
    constexpr int CH = R * kBK / 4;
#pragma unroll
    for (int c0 = 0; c0 < CH; c0 += kThreads) {
      const int c = c0 + tid;
      if (CH % kThreads == 0 || c < CH) {
        const int rr = (c % (R / 4)) * 4, kk = c / (R / 4);
        const int gr = r0 + rr, gk = k0 + kk;
        const int valid = (gk < K) ? min(max(rows - gr, 0), 4) : 0;
        const float* src = valid ? X + gk * ldx + gr : X;
        cp_async16(smem_u32(s + kk * LDS + rr), src, valid * 4);
      }
    }
  } else {
    constexpr int EL = R * kBK;
#pragma unroll
    for (int e0 = 0; e0 < EL; e0 += kThreads) {
      const int e = e0 + tid;
      if (EL % kThreads == 0 || e < EL) {
        const int rr = e % R, kk = e / R;
        const int gr = r0 + rr, gk = k0 + kk;
        const bool v = (gk < K) && (gr < rows);
        cp_async4(smem_u32(s + kk * LDS + rr), v ? X + gk * ldx + gr : X, v ? 4 : 0);
      }
    }
  }
}

// The same slice when element (r, k) sits at X[k + r*ldx] (k contiguous):
// consecutive threads walk k, so global reads stay in runs of kBK floats.
template <int R, int LDS>
__device__ __forceinline__ void load_k_contig(const float* X, long long ldx, int rows, int r0,
                                              int k0, int K, float* s, int tid) {
  constexpr int EL = R * kBK;
#pragma unroll
  for (int e0 = 0; e0 < EL; e0 += kThreads) {
    const int e = e0 + tid;
    if (EL % kThreads == 0 || e < EL) {
      const int kk = e % kBK, rr = e / kBK;
      const int gk = k0 + kk, gr = r0 + rr;
      const bool v = (gk < K) && (gr < rows);
      cp_async4(smem_u32(s + kk * LDS + rr), v ? X + gr * ldx + gk : X, v ? 4 : 0);
    }
  }
}

// GEN = false: the reference's layout (A and B untransposed), fixed at
// compile time; GEN = true: per-matrix transposition flags.
template <int BM, int BN, int TM, int TN, bool GEN = false>
__device__ __forceinline__ void simt_tile(const MatDesc& d, int tm, int tn,
                                          const float* __restrict__ A,
                                          const float* __restrict__ B, float* __restrict__ C,
                                          float alpha, float beta, float* smem) {
  constexpr int TX = BM / TM;
  constexpr int TY = BN / TN;
  static_assert(TX == 16 && TY == 16, "256 threads as 16 x 16");
  constexpr int TMH = TM > 4 ? 4 : TM;  // contiguous run per half along m
  constexpr int TNH = TN > 4 ? 4 : TN;
  constexpr int HM = TM / TMH;          // halves along m (2 for TM = 8)
  constexpr int HN = TN / TNH;
  constexpr int LDBS = BN + kPadB;
  constexpr int LDAS = GEN ? BM + kPadB : BM;
  constexpr int A_STAGE = kBK * LDAS;
  constexpr int STAGE = A_STAGE + kBK * LDBS;

  const int tid = threadIdx.x;
  const int tx = tid % TX, ty = tid / TX;
  const int M = d.M, N = d.N, K = d.K;
  const long long lda = d.lda, ldb = d.ldb, ldc = d.ldc;
  const int m0 = tm * BM, n0 = tn * BN;
  const bool inplace = (alpha == 1.0f && beta == 1.0f);

  // element (i, j) of the register tile sits at
  //   m = m0 + (i / TMH) * (BM / 2) + tx * TMH + i % TMH
  //   n = n0 + (j / TNH) * (BN / 2) + ty * TNH + j % TNH
  auto row_of = [&](int i) { return m0 + (i / TMH) * (BM / HM) + tx * TMH + (i % TMH); };
  auto col_of = [&](int j) { return n0 + (j / TNH) * (BN / HN) + ty * TNH + (j % TNH); };

  float acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      float v = 0.0f;
      if (inplace) {
        const int m = row_of(i), n = col_of(j);
        if (m < M && n < N) v = C[n * ldc + m];
      }
      acc[i][j] = v;
    }

  if (!inplace && beta != 0.0f) {
#pragma unroll
    for (int j = 0; j < TN; ++j)
#pragma unroll
      for (int h = 0; h < HM; ++h) {
        const int n = col_of(j), mb = m0 + h * (BM / HM) + tx * TMH;
        if (n < N && mb < M)
          asm volatile("prefetch.global.L2 [%0];" ::"l"(C + n * ldc + mb));
      }
  }

  const int nkb = (K + kBK - 1) / kBK;
  const bool a_vec = ((reinterpret_cast<uintptr_t>(A) & 15u) == 0) && ((d.lda & 3) == 0) &&
                     !(GEN && (d.aux & kTransAFlag));

  auto load_stage = [&](int kb, int slot) {
    float* sA = smem + slot * STAGE;
    float* sB = sA + A_STAGE;
    const int k0 = kb * kBK;
    if constexpr (GEN) {
      const bool ta = (d.aux & kTransAFlag) != 0, tb = (d.aux & kTransBFlag) != 0;
      if (!ta)
        load_rows_contig<BM, LDAS>(A, lda, M, m0, k0, K, sA, a_vec, tid);
      else
        load_k_contig<BM, LDAS>(A, lda, M, m0, k0, K, sA, tid);
      if (tb)
        load_rows_contig<BN, LDBS>(B, ldb, N, n0, k0, K, sB,
                                   ((reinterpret_cast<uintptr_t>(B) & 15u) == 0) &&
                                       ((d.ldb & 3) == 0),
                                   tid);
      else
        load_k_contig<BN, LDBS>(B, ldb, N, n0, k0, K, sB, tid);
      return;
    }
    if (a_vec) {
      constexpr int CH = BM * kBK / 4;
#pragma unroll
      for (int c0 = 0; c0 < CH; c0 += kThreads) {
        const int c = c0 + tid;
        if (CH % kThreads == 0 || c < CH) {
          const int mm = (c % (BM / 4)) * 4, kk = c / (BM / 4);
          const int gm = m0 + mm, gk = k0 + kk;
          int valid = (gk < K) ? min(max(M - gm, 0), 4) : 0;
          const float* src = valid ? A + gk * lda + gm : A;
          cp_async16(smem_u32(sA + kk * BM + mm), src, valid * 4);
        }
      }
    } else {
      constexpr int EL = BM * kBK;
#pragma unroll
      for (int e0 = 0; e0 < EL; e0 += kThreads) {
        const int e = e0 + tid;
        if (EL % kThreads == 0 || e < EL) {
          const int mm = e % BM, kk = e / BM;
          const int gm = m0 + mm, gk = k0 + kk;
          const bool v = (gk < K) && (gm < M);
          cp_async4(smem_u32(sA + kk * BM + mm), v ? A + gk * lda + gm : A, v ? 4 : 0);
        }
      }
    }
    constexpr int EB = BN * kBK;
#pragma unroll
    for (int e0 = 0; e0 < EB; e0 += kThreads) {
      const int e = e0 + tid;
      if (EB % kThreads == 0 || e < EB) {
        const int kk = e % kBK, nn = e / kBK;
        const int gk = k0 + kk, gn = n0 + nn;
        const bool v = (gk < K) && (gn < N);
        cp_async4(smem_u32(sB + kk * LDBS + nn), v ? B + gn * ldb + gk : B, v ? 4 : 0);
      }
    }
  };

  constexpr int NS = ring_stages<GEN>(STAGE);
  static_assert(NS >= kStages, "ring of at least kStages stages");
#pragma unroll
  for (int s = 0; s < NS - 1; ++s) {
    if (s < nkb) load_stage(s, s);
    cp_async_commit();
  }

  for (int kb = 0; kb < nkb; ++kb) {
    cp_async_wait<NS - 2>();
    __syncthreads();
    {
      const int nk = kb + NS - 1;
      if (nk < nkb) load_stage(nk, nk % NS);
      cp_async_commit();
    }
    const float* sA = smem + (kb % NS) * STAGE;
    const float* sB = sA + A_STAGE;
#pragma unroll
    for (int k = 0; k < kBK; ++k) {
      float a[TM], b[TN];
#pragma unroll
      for (int h = 0; h < HM; ++h) VecLd<TMH>::ld(sA + k * LDAS + h * (BM / HM) + tx * TMH, a + h * TMH);
#pragma unroll
      for (int h = 0; h < HN; ++h) VecLd<TNH>::ld(sB + k * LDBS + h * (BN / HN) + ty * TNH, b + h * TNH);
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
  }
  cp_async_wait<0>();

  // ---- epilogue ----
  const int lane = tid & 31;
  if (!inplace && beta != 0.0f) {
    // C is read: the lines were prefetched into L2 when the tile started.
    // Columns go two at a time, all reads of a pair before its writes (a
    // write may alias a later read as far as the compiler knows, so
    // interleaving them would serialise one memory round trip per element);
    // rows use the half-warp transpose below so accesses are 64-byte runs.
    constexpr int CJ = TN < 2 ? TN : 2;
#pragma unroll
    for (int jc = 0; jc < TN; jc += CJ) {
      float x[CJ][HM][TMH], cv[CJ][HM][TMH];
#pragma unroll
      for (int jj = 0; jj < CJ; ++jj)
#pragma unroll
        for (int h = 0; h < HM; ++h)
#pragma unroll
          for (int q = 0; q < TMH; ++q) {
            const int ml = q * 16 + tx;
            const int src = (lane & 16) | (ml / TMH);
            const int rsel = ml % TMH;
            float t = 0.0f;
#pragma unroll
            for (int r = 0; r < TMH; ++r) {
              const float u = __shfl_sync(0xffffffffu, acc[h * TMH + r][jc + jj], src);
              if (r == rsel) t = u;
            }
            x[jj][h][q] = t;
          }
#pragma unroll
      for (int jj = 0; jj < CJ; ++jj)
#pragma unroll
        for (int h = 0; h < HM; ++h)
#pragma unroll
          for (int q = 0; q < TMH; ++q) {
            const int n = col_of(jc + jj), m = m0 + h * (BM / HM) + q * 16 + tx;
            cv[jj][h][q] = (n < N && m < M) ? C[n * ldc + m] : 0.0f;
          }
#pragma unroll
      for (int jj = 0; jj < CJ; ++jj)
#pragma unroll
        for (int h = 0; h < HM; ++h)
#pragma unroll
          for (int q = 0; q < TMH; ++q) {
            const int n = col_of(jc + jj), m = m0 + h * (BM / HM) + q * 16 + tx;
            if (n < N && m < M) C[n * ldc + m] = fmaf(alpha, x[jj][h][q], beta * cv[jj][h][q]);
          }
    }
    return;
  }
  const bool c_vec = (TMH == 4) && ((reinterpret_cast<uintptr_t>(C) & 15u) == 0) &&
                     ((d.ldc & 3) == 0);
#pragma unroll
  for (int j = 0; j < TN; ++j) {
    const int n = col_of(j);
    const bool n_ok = n < N;
    float* Ccol = C + n * ldc;
#pragma unroll
    for (int h = 0; h < HM; ++h) {
      const int mb = m0 + h * (BM / HM) + tx * TMH;
      float v[TMH];
#pragma unroll
      for (int r = 0; r < TMH; ++r) v[r] = acc[h * TMH + r][j];
      if (c_vec) {
        if (n_ok) {
          if (mb + TMH <= M) {
            float4* p = reinterpret_cast<float4*>(Ccol + mb);
            float4 o;
            if (inplace) {
              o = make_float4(v[0], v[1], v[2], v[3]);
            } else if (beta == 0.0f) {
              o = make_float4(alpha * v[0], alpha * v[1], alpha * v[2], alpha * v[3]);
            } else {
              const float4 c = *p;
              o = make_float4(fmaf(alpha, v[0], beta * c.x), fmaf(alpha, v[1], beta * c.y),
                              fmaf(alpha, v[2], beta * c.z), fmaf(alpha, v[3], beta * c.w));
            }
            *p = o;
          } else {
#pragma unroll
            for (int r = 0; r < TMH; ++r) {
              const int m = mb + r;
              if (m < M) {
                float* p = Ccol + m;
                *p = inplace ? v[r] : (beta == 0.0f ? alpha * v[r] : fmaf(alpha, v[r], beta * *p));
              }
            }
          }
        }
      } else {
        // Warp-shuffle transpose: in round q, lane tx of each half-warp writes
        // m = base + q*16 + tx, taking it from the lane that owns it.
#pragma unroll
        for (int q = 0; q < TMH; ++q) {
          const int ml = q * 16 + tx;
          const int src = (lane & 16) | (ml / TMH);
          const int rsel = ml % TMH;
          float x = 0.0f;
#pragma unroll
          for (int r = 0; r < TMH; ++r) {
            const float t = __shfl_sync(0xffffffffu, v[r], src);
            if (r == rsel) x = t;
          }
          const int m = m0 + h * (BM / HM) + ml;
          if (n_ok && m < M) {
            float* p = Ccol + m;
            *p = inplace ? x : (beta == 0.0f ? alpha * x : fmaf(alpha, x, beta * *p));
          }
        }
      }
    }
  }
}

// Thin tiles.  THIN_M: an 8 x 128 tile (M <= 8), thread t owns column t % 128
// and rows 4 (t / 128) .. +3; otherwise a 128 x 8 tile (N <= 8), thread t owns
// row t % 128 and columns 4 (t / 128) .. +3.  Same cp.async ring of 16-k
// slices and the same per-element fma chain over k in order as simt_tile, so
// results are bit-identical to every other configuration.
template <bool THIN_M, bool GEN = false>
__device__ __forceinline__ void simt_thin(const MatDesc& d, int tm, int tn,
                                          const float* __restrict__ A,
                                          const float* __restrict__ B, float* __restrict__ C,
                                          float alpha, float beta, float* smem) {
  constexpr int BM = THIN_M ? 8 : 128;
  constexpr int BN = THIN_M ? 128 : 8;
  constexpr int LDAS = BM + kPadB;  // rows of k padded like the transposed loads
  constexpr int LDBS = BN + kPadB;
  // 8 x 128 tiles of the reference layout keep B's slice as [n][k]: each
  // column's 16 k arrive as four 16-byte copies (B is k-contiguous), and each
  // thread reads its own column four k at a time.  Rows of 20 floats keep
  // those float4 reads of eight lanes on distinct banks.
  constexpr bool KMAJ = THIN_M && !GEN;
  constexpr int LDK = kBK + 4;
  constexpr int A_STAGE = kBK * LDAS;
  constexpr int STAGE = A_STAGE + (KMAJ ? BN * LDK : kBK * LDBS);
  constexpr int NS = ring_stages<GEN>(STAGE);
  static_assert(NS >= kStages, "ring of at least kStages stages");
  const int tid = threadIdx.x;
  const int M = d.M, N = d.N, K = d.K;
  const long long lda = d.lda, ldb = d.ldb, ldc = d.ldc;
  const int m0 = tm * BM, n0 = tn * BN;
  const bool inplace = (alpha == 1.0f && beta == 1.0f);
  // this thread's outputs: (m_of(r), n_of(r)) for r = 0..3
  const int own = tid & 127, quad = tid >> 7;
  auto m_of = [&](int r) { return THIN_M ? m0 + 4 * quad + r : m0 + own; };
  auto n_of = [&](int r) { return THIN_M ? n0 + own : n0 + 4 * quad + r; };

  const bool ta = GEN && (d.aux & kTransAFlag), tb = GEN && (d.aux & kTransBFlag);
  const bool a_vec = !ta && ((reinterpret_cast<uintptr_t>(A) & 15u) == 0) && ((d.lda & 3) == 0);
  const bool b_vec = tb && ((reinterpret_cast<uintptr_t>(B) & 15u) == 0) && ((d.ldb & 3) == 0);
  const bool b_vec_k = KMAJ && ((reinterpret_cast<uintptr_t>(B) & 15u) == 0) && ((d.ldb & 3) == 0);
  auto load_stage = [&](int kb, int slot) {
    float* sA = smem + slot * STAGE;
    float* sB = sA + A_STAGE;
    const int k0 = kb * kBK;
    if (!ta)
      load_rows_contig<BM, LDAS>(A, lda, M, m0, k0, K, sA, a_vec, tid);
    else
      load_k_contig<BM, LDAS>(A, lda, M, m0, k0, K, sA, tid);
    if constexpr (KMAJ) {
      if (b_vec_k) {
#pragma unroll
        for (int c0 = 0; c0 < BN * 4; c0 += kThreads) {
          const int c = c0 + tid;
          const int nn = c >> 2, kq = (c & 3) * 4;
          const int gn = n0 + nn, gk = k0 + kq;
          const int valid = (gn < N) ? min(max(K - gk, 0), 4) : 0;
          const float* src = valid ? B + (long long)gn * ldb + gk : B;
          cp_async16(smem_u32(sB + nn * LDK + kq), src, valid * 4);
        }
      } else {
#pragma unroll
        for (int e0 = 0; e0 < BN * kBK; e0 += kThreads) {
          const int e = e0 + tid;
          const int kk = e & (kBK - 1), nn = e / kBK;
          const int gk = k0 + kk, gn = n0 + nn;
          const bool v = (gk < K) && (gn < N);
          cp_async4(smem_u32(sB + nn * LDK + kk), v ? B + (long long)gn * ldb + gk : B, v ? 4 : 0);
        }
      }
      return;
    }
    if (tb)
      load_rows_contig<BN, LDBS>(B, ldb, N, n0, k0, K, sB, b_vec, tid);
    else
      load_k_contig<BN, LDBS>(B, ldb, N, n0, k0, K, sB, tid);
  };
  const int nkb = (K + kBK - 1) / kBK;
#pragma unroll
  for (int s = 0; s < NS - 1; ++s) {
    if (s < nkb) load_stage(s, s);
    cp_async_commit();
  }
  float acc[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    float v = 0.0f;
    if (inplace && m_of(r) < M && n_of(r) < N) v = C[(long long)n_of(r) * ldc + m_of(r)];
    acc[r] = v;
  }
  for (int kb = 0; kb < nkb; ++kb) {
    cp_async_wait<NS - 2>();
    __syncthreads();
    {
      const int nk = kb + NS - 1;
      if (nk < nkb) load_stage(nk, nk % NS);
      cp_async_commit();
    }
    const float* sA = smem + (kb % NS) * STAGE;
    const float* sB = sA + A_STAGE;
    if constexpr (KMAJ) {
#pragma unroll
      for (int k = 0; k < kBK; k += 4) {
        const float4 b4 = *reinterpret_cast<const float4*>(sB + own * LDK + k);
        const float bk[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          const float4 a = *reinterpret_cast<const float4*>(sA + (k + kk) * LDAS + 4 * quad);
          acc[0] = fmaf(a.x, bk[kk], acc[0]);
          acc[1] = fmaf(a.y, bk[kk], acc[1]);
          acc[2] = fmaf(a.z, bk[kk], acc[2]);
          acc[3] = fmaf(a.w, bk[kk], acc[3]);
        }
      }
      continue;
    }
#pragma unroll
    for (int k = 0; k < kBK; ++k) {
      if constexpr (THIN_M) {
        const float b = sB[k * LDBS + own];
        const float4 a = *reinterpret_cast<const float4*>(sA + k * LDAS + 4 * quad);
        acc[0] = fmaf(a.x, b, acc[0]);
        acc[1] = fmaf(a.y, b, acc[1]);
        acc[2] = fmaf(a.z, b, acc[2]);
        acc[3] = fmaf(a.w, b, acc[3]);
      } else {
        const float a = sA[k * LDAS + own];
        const float4 b = *reinterpret_cast<const float4*>(sB + k * LDBS + 4 * quad);
        acc[0] = fmaf(a, b.x, acc[0]);
        acc[1] = fmaf(a, b.y, acc[1]);
        acc[2] = fmaf(a, b.z, acc[2]);
        acc[3] = fmaf(a, b.w, acc[3]);
      }
    }
  }
  cp_async_wait<0>();
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int m = m_of(r), n = n_of(r);
    if (m < M && n < N) {
      float* p = C + (long long)n * ldc + m;
      *p = inplace ? acc[r] : (beta == 0.0f ? alpha * acc[r] : fmaf(alpha, acc[r], beta * *p));
    }
  }
}

__global__ void __launch_bounds__(kThreads, 2) simt_persistent_kernel(const SimtParams p) {
  extern __shared__ __align__(16) float smem[];
  __shared__ int s_item;
  const int n_items = p.n_items_dev ? *p.n_items_dev : p.n_items;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(p.counters, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= n_items) break;
    const TileItem ti = p.items[it];
    const MatDesc d = p.descs[ti.mat];
    const float* A = p.A[ti.mat];
    const float* B = p.B[ti.mat];
    float* C = p.C[ti.mat];
    switch (d.cfg) {
      case 0: simt_tile<16, 16, 1, 1>(d, ti.tm, ti.tn, A, B, C, p.alpha, p.beta, smem); break;
      case 1: simt_tile<32, 32, 2, 2>(d, ti.tm, ti.tn, A, B, C, p.alpha, p.beta, smem); break;
      case 2: simt_tile<64, 32, 4, 2>(d, ti.tm, ti.tn, A, B, C, p.alpha, p.beta, smem); break;
      case 3: simt_tile<32, 64, 2, 4>(d, ti.tm, ti.tn, A, B, C, p.alpha, p.beta, smem); break;
      case 4: simt_tile<64, 64, 4, 4>(d, ti.tm, ti.tn, A, B, C, p.alpha, p.beta, smem); break;
      case 5: simt_tile<128, 64, 8, 4>(d, ti.tm, ti.tn, A, B, C, p.alpha, p.beta, smem); break;
      case 6: simt_tile<64, 128, 4, 8>(d, ti.tm, ti.tn, A, B, C, p.alpha, p.beta, smem); break;
      case 7: simt_tile<128, 128, 8, 8>(d, ti.tm, ti.tn, A, B, C, p.alpha, p.beta, smem); break;
      case 8: simt_thin<true>(d, ti.tm, ti.tn, A, B, C, p.alpha, p.beta, smem); break;
      default: simt_thin<false>(d, ti.tm, ti.tn, A, B, C, p.alpha, p.beta, smem); break;
    }
    __syncthreads();
  }
  // The last CTA to leave resets the queue, so the next launch (or graph
  // replay) starts from item 0 without a memset.
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(reinterpret_cast<unsigned*>(p.counters) + 1, 1u);
    if (prev == gridDim.x - 1) {
      atomicExch(p.counters, 0);
      atomicExch(p.counters + 1, 0);
      __threadfence();
    }
  }
}

// The same persistent loop for plans whose matrices carry kTransAFlag /
// kTransBFlag (kept apart so the untransposed kernel above stays as it is).
__global__ void __launch_bounds__(kThreads, 2) simt_persistent_kernel_t(const SimtParams p) {
  extern __shared__ __align__(16) float smem[];
  __shared__ int s_item;
  const int n_items = p.n_items_dev ? *p.n_items_dev : p.n_items;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(p.counters, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= n_items) break;
    const TileItem ti = p.items[it];
    const MatDesc d = p.descs[ti.mat];
    const float* A = p.A[ti.mat];
    const float* B = p.B[ti.mat];
    float* C = p.C[ti.mat];
    switch (d.cfg) {
      case 0: simt_tile<16, 16, 1, 1, true>(d, ti.tm, ti.tn, A, B, C, p.alpha, p.beta, smem); break;
      case 1: simt_tile<32, 32, 2, 2, true>(d, ti.tm, ti.tn, A, B, C, p.alpha, p.beta, smem); break;
      case 2: simt_tile<64, 32, 4, 2, true>(d, ti.tm, ti.tn, A, B, C, p.alpha, p.beta, smem); break;
      case 3: simt_tile<32, 64, 2, 4, true>(d, ti.tm, ti.tn, A, B, C, p.alpha, p.beta, smem); break;
      case 4: simt_tile<64, 64, 4, 4, true>(d, ti.tm, ti.tn, A, B, C, p.alpha, p.beta, smem); break;
      case 5: simt_tile<128, 64, 8, 4, true>(d, ti.tm, ti.tn, A, B, C, p.alpha, p.beta, smem); break;
      case 6: simt_tile<64, 128, 4, 8, true>(d, ti.tm, ti.tn, A, B, C, p.alpha, p.beta, smem); break;
      case 7: simt_tile<128, 128, 8, 8, true>(d, ti.tm, ti.tn, A, B, C, p.alpha, p.beta, smem); break;
      case 8: simt_thin<true, true>(d, ti.tm, ti.tn, A, B, C, p.alpha, p.beta, smem); break;
      default: simt_thin<false, true>(d, ti.tm, ti.tn, A, B, C, p.alpha, p.beta, smem); break;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(reinterpret_cast<unsigned*>(p.counters) + 1, 1u);
    if (prev == gridDim.x - 1) {
      atomicExch(p.counters, 0);
      atomicExch(p.counters + 1, 0);
      __threadfence();
    }
  }
}

}  // namespace

cudaError_t simt_launch(const SimtParams& p, int grid, cudaStream_t stream, bool transposed) {
  static bool attr_done = false;
  if (!attr_done) {
    cudaError_t e = cudaFuncSetAttribute(simt_persistent_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(simt_persistent_kernel_t,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytesT);
    if (e != cudaSuccess) return e;
    attr_done = true;
  }
  if (transposed)
    simt_persistent_kernel_t<<<grid, kThreads, kSmemBytesT, stream>>>(p);
  else
    simt_persistent_kernel<<<grid, kThreads, kSmemBytes, stream>>>(p);
  return cudaGetLastError();
}

int simt_ctas_per_sm() {
  int n = 0;
  cudaFuncSetAttribute(simt_persistent_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       kSmemBytes);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, simt_persistent_kernel, kThreads,
                                                    kSmemBytes) != cudaSuccess)
    return 1;
  int nt = 0;
  cudaFuncSetAttribute(simt_persistent_kernel_t, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       kSmemBytesT);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nt, simt_persistent_kernel_t, kThreads,
                                                    kSmemBytesT) == cudaSuccess && nt < n)
    n = nt;  // plans size their grid before they know which kernel runs
  return n > 0 ? n : 1;
}

}  // namespace bgemm
