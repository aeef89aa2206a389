// tc_kernel.cu -- tensor-core (tcgen05 / TMEM) form of the variable-size
// batched SGEMM for sm_103a.
//
// Two kernels per execute:
//   tc_pack_kernel  splits every operand element x into hi = round(x) and
//                   lo = round(x - hi) (TF32 or BF16, round to nearest even)
//                   and writes them K-major ("rows of K", 16-byte aligned row
//                   length) into the plan's workspace: A is transposed from
//                   column-major M x K, B (column-major K x N) is already
//                   K-major.  Ragged edges of any shape and leading dimension
//                   are handled here, so the GEMM sees only TMA-legal tiles.
//   tc_gemm_kernel  one persistent CTA per SM pulls output tiles from the
//                   largest-first queue.  Warp 0 (one lane) is the TMA
//                   producer and tile scheduler, warp 1 (one lane) issues
//                   tcgen05.mma into TMEM, warps 2-5 drain TMEM (tcgen05.ld),
//                   apply alpha/beta and store C.  Per 128-byte K slice a
//                   stage holds the hi (and lo) tiles of both sides,
//                   TMA-loaded with 128-byte swizzle through per-matrix
//                   tensor maps.
//
// Accumulation.  The tensor core adds products into its FP32 accumulator
// with truncation, so a long chain of MMAs into one accumulator drifts
// toward zero (measured on GB300: -1.1e-7 of sum|ab| at K = 2048, against
// 2e-8 unbiased for an FP32 fma chain).  The split modes therefore never let
// a chain run long: every group of MMAs (two 128-byte K slices, i.e. 64 k
// for TF32, or one MMA for matrices with K <= 64, which also keep lo*lo)
// accumulates into a fresh buffer of a 4-deep TMEM ring -- the
// small hi*lo and lo*hi products first, hi*hi last -- and the epilogue warps
// add each finished group into FP32 registers with round-to-nearest while
// the MMAs of the next groups run.  The single-product TF32 mode keeps one
// accumulator per tile (double-buffered across tiles); its error is set by
// the TF32 operand rounding anyway.
//
// Every wait on an mbarrier is bounded (global timer); on expiry the kernel
// sets an error flag, lets in-flight copies and MMAs land, frees TMEM and
// returns, and the host reports BGEMM_ERROR_DEVICE_TIMEOUT.
//
// Reference counterpart: the reference's FP32 tile bodies
// (CUDA/framework/kernel_128_new.h, kernel_256_new.h) have no tensor-core
// form; this file is the new precision path that the tile queue drives.
#include <stdint.h>

#include "tc_epilogue.h"
#include "tc_ptx.h"

namespace bgemm {
namespace {

constexpr int kABytes = kTcBM * 128;        // 128 rows x 128 bytes of K
constexpr int kBBytes = kTcMaxBN * 128;     // up to 128 rows x 128 bytes
constexpr int kSchedSlots = 4;
constexpr int kThreads = 64 + 8 * 32;  // producer, MMA, 8 epilogue warps

template <int SPLIT>
struct Geo {
  static constexpr int NP = SPLIT ? 2 : 1;
  static constexpr int STAGE = (kABytes + kBBytes) * NP;
  static constexpr int S = SPLIT ? 3 : 6;
  // TMEM accumulator buffers of 128 columns: a 4-deep group ring (split
  // modes) or 2 tile buffers (single product)
  static constexpr int NACC = SPLIT ? 4 : 2;
  static constexpr int NBAR = 2 * S + 2 * kSchedSlots + 2 * NACC + 1;
  static constexpr int BYTES = S * STAGE + NBAR * 8 + kSchedSlots * 4 + 16 + 1024;
};

// Matrices with K at most this many elements promote every MMA (8 k for
// TF32, 16 k for BF16); larger K promotes every kGroupKB 128-byte slices.
constexpr int kFineK = 64;
constexpr int kGroupKB = 2;
// Epilogue: 8 warps, two per TMEM lane quadrant, each owning half of the
// 128 accumulator columns.
constexpr int kEpiWarps = 8;
constexpr int kEpiCols = kTcMaxBN / 2;

// ---------------------------------------------------- operand splitting --
__device__ __forceinline__ void put(char* hi, char* lo, long long idx, float x, int kind,
                                    int split) {
  if (kind == kKindTF32) {
    const float h = round_keep(x, 13);
    reinterpret_cast<float*>(hi)[idx] = h;
    if (split) {
      const bool fin = (__float_as_uint(x) & 0x7f800000u) != 0x7f800000u;
      reinterpret_cast<float*>(lo)[idx] = fin ? round_keep(x - h, 13) : 0.0f;
    }
  } else {
    const float h = round_keep(x, 16);
    reinterpret_cast<uint16_t*>(hi)[idx] = (uint16_t)(__float_as_uint(h) >> 16);
    if (split) {
      const bool fin = (__float_as_uint(x) & 0x7f800000u) != 0x7f800000u;
      const float l = fin ? round_keep(x - h, 16) : 0.0f;
      reinterpret_cast<uint16_t*>(lo)[idx] = (uint16_t)(__float_as_uint(l) >> 16);
    }
  }
}

// Splits four consecutive k of one packed row and stores hi (and lo) with one
// 16-byte (TF32) or 8-byte (BF16) store each; idx is a multiple of 4.
__device__ __forceinline__ void put4(char* hi, char* lo, long long idx, const float* x, int kind,
                                     int split) {
  float h[4], l[4];
  const int drop = (kind == kKindTF32) ? 13 : 16;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    h[i] = round_keep(x[i], drop);
    const bool fin = (__float_as_uint(x[i]) & 0x7f800000u) != 0x7f800000u;
    l[i] = fin ? round_keep(x[i] - h[i], drop) : 0.0f;
  }
  if (kind == kKindTF32) {
    *reinterpret_cast<float4*>(reinterpret_cast<float*>(hi) + idx) = make_float4(h[0], h[1], h[2], h[3]);
    if (split)
      *reinterpret_cast<float4*>(reinterpret_cast<float*>(lo) + idx) = make_float4(l[0], l[1], l[2], l[3]);
  } else {
    auto pk = [](float a, float b) {
      return (__float_as_uint(a) >> 16) | (__float_as_uint(b) & 0xFFFF0000u);
    };
    *reinterpret_cast<uint2*>(reinterpret_cast<uint16_t*>(hi) + idx) = make_uint2(pk(h[0], h[1]), pk(h[2], h[3]));
    if (split)
      *reinterpret_cast<uint2*>(reinterpret_cast<uint16_t*>(lo) + idx) = make_uint2(pk(l[0], l[1]), pk(l[2], l[3]));
  }
}

// k per chunk of the pre-pass: each thread keeps kPackK / 8 loads in flight.
constexpr int kPackK = 256;

// One job = 32 packed rows of one operand, walked in chunks of kPackK k.  Each
// thread issues all kPackK / 8 of its loads for a chunk before it stores, and
// writes four consecutive k per store (rows are 16-byte aligned, so packed
// writes are full vectors; the K tail and rows past M/N are masked).
__global__ void __launch_bounds__(256) tc_pack_kernel(const TcPackParams p) {
  __shared__ float t[kPackK][33];
  const int tid = threadIdx.x;
  const int n_jobs = p.n_jobs_dev ? *p.n_jobs_dev : p.n_jobs;
  for (int j = blockIdx.x; j < n_jobs; j += gridDim.x) {
    const PackJob job = p.jobs[j];
    const MatDesc d = p.descs[job.mat];
    const PackDesc pd = p.pdescs[job.mat];
    const int K = d.K;
    const long long kpad = pd.kpad;
    // the strip's source: op(A) rows m or op(B)^T rows n, element (r, k) at
    // X[r + k*ldx] ("rows contiguous": A, or B stored transposed) or at
    // X[k + r*ldx] ("k contiguous": B, or A stored transposed)
    const bool is_a = job.op == 0;
    const float* X = is_a ? p.A[job.mat] : p.B[job.mat];
    const long long ldx = is_a ? d.lda : d.ldb;
    const int rows = is_a ? d.M : d.N;
    const bool rows_contig = is_a ? !(d.aux & kTransAFlag) : (d.aux & kTransBFlag) != 0;
    char* hi = p.ws + (is_a ? pd.a_hi : pd.b_hi);
    char* lo = p.ws + (is_a ? pd.a_lo : pd.b_lo);
    if (rows_contig) {
      // transpose through shared memory: loads walk 32 consecutive rows
      const int mm = tid & 31;
      const int m = job.r0 + mm;
      for (int k0 = 0; k0 < K; k0 += kPackK) {
        float v[kPackK / 8];
#pragma unroll
        for (int i = 0; i < kPackK / 8; ++i) {
          const int k = k0 + (tid >> 5) + 8 * i;
          v[i] = (m < rows && k < K) ? X[m + k * ldx] : 0.0f;
        }
#pragma unroll
        for (int i = 0; i < kPackK / 8; ++i) t[(tid >> 5) + 8 * i][mm] = v[i];
        __syncthreads();
        const int wm = tid >> 3;           // packed row within the strip
        const int wk = (tid & 7) * 4;      // first of four k
#pragma unroll
        for (int h2 = 0; h2 < kPackK / 32; ++h2) {
          const int kk = wk + 32 * h2;
          const int k = k0 + kk;
          const int mr = job.r0 + wm;
          if (mr < rows && k < K) {
            float x[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) x[i] = t[kk + i][wm];
            if (k + 4 <= K) {
              put4(hi, lo, mr * kpad + k, x, p.kind, p.split);
            } else {
              for (int i = 0; i < 4 && k + i < K; ++i)
                put(hi, lo, mr * kpad + k + i, x[i], p.kind, p.split);
            }
          }
        }
        __syncthreads();
      }
    } else if (((reinterpret_cast<uintptr_t>(X) | (uintptr_t)(ldx * 4)) & 15u) != 0) {
      // rows of K that do not start on 16 bytes: a warp walks 4 rows, each
      // load covering 32 consecutive k of one row (one coalesced run of 128
      // bytes whatever the alignment; 8 threads per row with 4 scalar loads
      // each would touch every sector of the run four times)
      const int lane = tid & 31;
      const int r_w = job.r0 + (tid >> 5) * 4;  // the warp's first row
      for (int k0 = 0; k0 < K; k0 += kPackK) {
        float x[4][kPackK / 32];
#pragma unroll
        for (int rr = 0; rr < 4; ++rr) {
          const float* row = X + (long long)(r_w + rr) * ldx;
#pragma unroll
          for (int h = 0; h < kPackK / 32; ++h) {
            const int k = k0 + 32 * h + lane;
            x[rr][h] = (r_w + rr < rows && k < K) ? row[k] : 0.0f;
          }
        }
#pragma unroll
        for (int rr = 0; rr < 4; ++rr) {
#pragma unroll
          for (int h = 0; h < kPackK / 32; ++h) {
            const int k = k0 + 32 * h + lane;
            if (r_w + rr < rows && k < K)
              put(hi, lo, (long long)(r_w + rr) * kpad + k, x[rr][h], p.kind, p.split);
          }
        }
      }
    } else {
      // rows of K on 16 bytes: 8 threads per row, four consecutive k each
      const int nn = tid >> 3;
      const int n = job.r0 + nn;
      const int wk = (tid & 7) * 4;
      if (n >= rows) continue;
      const float* col = X + n * ldx;
      const bool vec = ((reinterpret_cast<uintptr_t>(col) & 15u) == 0);
      for (int k0 = 0; k0 < K; k0 += kPackK) {
        float x[kPackK / 32][4];
#pragma unroll
        for (int h2 = 0; h2 < kPackK / 32; ++h2) {
          const int k = k0 + wk + 32 * h2;
          if (vec && k + 4 <= K) {
            const float4 f = *reinterpret_cast<const float4*>(col + k);
            x[h2][0] = f.x; x[h2][1] = f.y; x[h2][2] = f.z; x[h2][3] = f.w;
          } else {
#pragma unroll
            for (int i = 0; i < 4; ++i) x[h2][i] = (k + i < K) ? col[k + i] : 0.0f;
          }
        }
#pragma unroll
        for (int h2 = 0; h2 < kPackK / 32; ++h2) {
          const int k = k0 + wk + 32 * h2;
          if (k + 4 <= K) {
            put4(hi, lo, n * kpad + k, x[h2], p.kind, p.split);
          } else {
            for (int i = 0; i < 4 && k + i < K; ++i)
              put(hi, lo, n * kpad + k + i, x[h2][i], p.kind, p.split);
          }
        }
      }
    }
  }
}

// ------------------------------------------------ per-matrix tensor maps --
// One warp per map: map j of matrix i = j / 4 is part j % 4 (A-side hi, lo,
// B-side hi, lo).  The A side is A unless the matrix's configuration swaps
// the operands; its boxes are 128 rows, the B side's bn rows (bn / 2 per CTA
// of a pair).
__global__ void __launch_bounds__(128) tc_tmap_kernel(const TcTmapParams p) {
  __shared__ __align__(128) CUtensorMap maps[4];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x * 4 + warp;
  if (j >= 4 * p.batch) return;
  const int i = j >> 2, part = j & 3;
  const MatDesc d = p.descs[i];
  if (d.M == 0 || d.N == 0 || d.K == 0) return;  // never loaded
  const PackDesc pd = p.pdescs[i];
  const bool swap = tc_cfg_swap(d.cfg);
  const bool a_side = part < 2, lo = part & 1;
  const bool use_a = a_side != swap;  // which operand's panel this map walks
  const long long off = use_a ? (lo ? pd.a_lo : pd.a_hi) : (lo ? pd.b_lo : pd.b_hi);
  const int rows = use_a ? d.M : d.N;
  const int esz = (p.kind == kKindBF16) ? 2 : 4;
  const int box = a_side ? kTcBM : (p.pair ? tc2_cfg_bn(d.cfg) / 2 : tc_cfg_bn(d.cfg));
  const long long extent = (long long)rows * pd.kpad * esz;
  const CUtensorMap* tpl = p.templ + tmap_template_index(box, extent >= kTmapLargeExtent);
  uint32_t* dst = reinterpret_cast<uint32_t*>(&maps[warp]);
  dst[lane] = reinterpret_cast<const uint32_t*>(tpl)[lane];
  __syncwarp();
  const uint32_t sm = smem_u32(&maps[warp]);
  if (lane == 0) {
    tmap_set_address(sm, p.ws + off);
    tmap_set_dim(sm, 0, (uint32_t)d.K);
    tmap_set_dim(sm, 1, (uint32_t)rows);
    tmap_set_row_stride(sm, (uint64_t)pd.kpad * esz);
  }
  __syncwarp();
  tmap_publish(p.out + j, sm);
}

// ------------------------------------------------------------- the GEMM --
template <int KIND, int SPLIT>
__global__ void __launch_bounds__(kThreads, 1) tc_gemm_kernel(const TcGemmParams p) {
  using G = Geo<SPLIT>;
  constexpr int S = G::S;
  constexpr int KE = (KIND == kKindTF32) ? 32 : 64;  // elements per 128-byte slice
  constexpr int NSUB = 4;                             // MMAs of 32 bytes of K per slice
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t pad = (1024u - (raw & 1023u)) & 1023u;
  uint8_t* smem = smem_raw + pad;
  const uint32_t sbase = raw + pad;

  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + S * G::STAGE);
  const uint32_t bar0 = sbase + S * G::STAGE;
  auto full = [&](int s) { return bar0 + 8u * s; };
  auto empty = [&](int s) { return bar0 + 8u * (S + s); };
  auto sfull = [&](int s) { return bar0 + 8u * (2 * S + s); };
  auto sempty = [&](int s) { return bar0 + 8u * (2 * S + kSchedSlots + s); };
  constexpr int NACC = G::NACC;
  auto tfull = [&](int s) { return bar0 + 8u * (2 * S + 2 * kSchedSlots + s); };
  auto tempty = [&](int s) { return bar0 + 8u * (2 * S + 2 * kSchedSlots + NACC + s); };
  const uint32_t drain = bar0 + 8u * (2 * S + 2 * kSchedSlots + 2 * NACC);
  volatile int* slots = reinterpret_cast<volatile int*>(bars + G::NBAR);
  volatile uint32_t* tmem_slot = reinterpret_cast<volatile uint32_t*>(slots + kSchedSlots);
  volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int n_items = p.n_items_dev ? *p.n_items_dev : p.n_items;
  if (p.cta_times && threadIdx.x == 0) p.cta_times[2 * blockIdx.x] = gtimer();

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(full(s), 1);
      mbar_init(empty(s), 1);
    }
    for (int s = 0; s < kSchedSlots; ++s) {
      mbar_init(sfull(s), 1);
      mbar_init(sempty(s), 1 + kEpiWarps);
    }
    for (int s = 0; s < NACC; ++s) {
      mbar_init(tfull(s), 1);
      mbar_init(tempty(s), kEpiWarps);
    }
    mbar_init(drain, 1);
    *abort = 0;
    fence_mbar_init();
  }
  if (warp == 1) {
    tmem_alloc(smem_u32(const_cast<uint32_t*>(tmem_slot)), 512);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------ producer + scheduler
    if (lane == 0) {
      Ring st, sc;
      int inflight_phase[S];
      bool inflight[S];
      for (int s = 0; s < S; ++s) inflight[s] = false, inflight_phase[s] = 0;
      int last_mat = -1;
      for (;;) {
        const int it = atomicAdd(p.counters, 1);
        if (!wait_bounded(sempty(sc.idx), sc.phase ^ 1u, p.error, abort, p.timeout_ns)) break;
        slots[sc.idx] = (it < n_items) ? it : -1;
        mbar_arrive(sfull(sc.idx));
        sc.next(kSchedSlots);
        if (it >= n_items) break;
        const TileItem ti = p.items[it];
        const MatDesc d = p.descs[ti.mat];
        const int bn = tc_cfg_bn(d.cfg);
        const CUtensorMap* tm = p.tmaps + 4 * ti.mat;
        if (ti.mat != last_mat && d.K > 0) {
          for (int q = 0; q < 4; ++q) tmap_acquire(tm + q);
          prefetch_tmap(tm);
          prefetch_tmap(tm + 2);
          last_mat = ti.mat;
        }
        const int nk = (d.K + KE - 1) / KE;
        const uint32_t tx = (uint32_t)(kABytes + bn * 128) * G::NP;
        const int row_a = ti.tm * kTcBM;
        const int row_b = ti.tn * bn;
        bool ok = true;
        for (int kb = 0; kb < nk; ++kb) {
          if (!wait_bounded(empty(st.idx), st.phase ^ 1u, p.error, abort, p.timeout_ns)) {
            ok = false;
            break;
          }
          const uint32_t sa = sbase + st.idx * G::STAGE;
          const uint32_t sb = sa + kABytes * G::NP;
          mbar_arrive_expect_tx(full(st.idx), tx);
          inflight[st.idx] = true;
          inflight_phase[st.idx] = st.phase;
          tma_load_2d(sa, tm + 0, kb * KE, row_a, full(st.idx));
          tma_load_2d(sb, tm + 2, kb * KE, row_b, full(st.idx));
          if (SPLIT) {
            tma_load_2d(sa + kABytes, tm + 1, kb * KE, row_a, full(st.idx));
            tma_load_2d(sb + kBBytes, tm + 3, kb * KE, row_b, full(st.idx));
          }
          st.next(S);
        }
        if (!ok) break;
      }
      // Let every copy this thread issued land before the CTA can exit.
      for (int s = 0; s < S; ++s)
        if (inflight[s])
          wait_bounded(full(s), (uint32_t)inflight_phase[s], p.error, nullptr, p.timeout_ns);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ----------------------------------------------------------- MMA issue
    if (lane == 0) {
      Ring st, sc, acc;
      for (;;) {
        if (!wait_bounded(sfull(sc.idx), sc.phase, p.error, abort, p.timeout_ns)) break;
        const int it = slots[sc.idx];
        mbar_arrive(sempty(sc.idx));
        sc.next(kSchedSlots);
        if (it < 0) break;
        const TileItem ti = p.items[it];
        const MatDesc d = p.descs[ti.mat];
        const int bn = tc_cfg_bn(d.cfg);
        const uint32_t idesc = make_idesc<KIND>(bn);
        const int nk = (d.K + KE - 1) / KE;
        bool ok = true;
        if constexpr (SPLIT) {
          // group-promoted accumulation (see the file comment)
          const int nsub = (d.K + KE / NSUB - 1) / (KE / NSUB);  // MMAs of K per product
          const bool fine = d.K <= kFineK;
          for (int kb = 0; kb < nk && ok; ++kb) {
            if (!wait_bounded(full(st.idx), st.phase, p.error, abort, p.timeout_ns)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t sa = sbase + st.idx * G::STAGE;
            const uint32_t sb = sa + kABytes * G::NP;
            const int s_end = min(NSUB, nsub - kb * NSUB);
            if (fine) {
              for (int s = 0; s < s_end; ++s) {
                if (!wait_bounded(tempty(acc.idx), acc.phase ^ 1u, p.error, abort,
                                  p.timeout_ns)) {
                  ok = false;
                  break;
                }
                tc_fence_after();
                const uint32_t buf = tmem + acc.idx * 128u;
                const uint64_t ah = sw128_desc(sa + 32u * s), al = sw128_desc(sa + kABytes + 32u * s);
                const uint64_t bh = sw128_desc(sb + 32u * s), bl = sw128_desc(sb + kBBytes + 32u * s);
                // small K: the split error dominates, so lo*lo is kept too
                mma<KIND>(buf, al, bl, idesc, 0u);
                mma<KIND>(buf, al, bh, idesc, 1u);
                mma<KIND>(buf, ah, bl, idesc, 1u);
                mma<KIND>(buf, ah, bh, idesc, 1u);
                mma_commit(tfull(acc.idx));
                acc.next(NACC);
              }
            } else {
              // a group spans kGroupKB slices; small products of each slice first
              const bool first = (kb % kGroupKB) == 0;
              if (first) {
                if (!wait_bounded(tempty(acc.idx), acc.phase ^ 1u, p.error, abort,
                                  p.timeout_ns)) {
                  ok = false;
                  break;
                }
                tc_fence_after();
              }
              const uint32_t buf = tmem + acc.idx * 128u;
              for (int s = 0; s < s_end; ++s) {
                mma<KIND>(buf, sw128_desc(sa + kABytes + 32u * s), sw128_desc(sb + 32u * s), idesc,
                          (first && s == 0) ? 0u : 1u);
                mma<KIND>(buf, sw128_desc(sa + 32u * s), sw128_desc(sb + kBBytes + 32u * s), idesc,
                          1u);
              }
              for (int s = 0; s < s_end; ++s)
                mma<KIND>(buf, sw128_desc(sa + 32u * s), sw128_desc(sb + 32u * s), idesc, 1u);
              if ((kb % kGroupKB) == kGroupKB - 1 || kb == nk - 1) {
                mma_commit(tfull(acc.idx));
                acc.next(NACC);
              }
            }
            mma_commit(empty(st.idx));
            st.next(S);
          }
        } else {
          if (!wait_bounded(tempty(acc.idx), acc.phase ^ 1u, p.error, abort, p.timeout_ns)) break;
          tc_fence_after();
          const uint32_t d_main = tmem + acc.idx * 256u;
          for (int kb = 0; kb < nk; ++kb) {
            if (!wait_bounded(full(st.idx), st.phase, p.error, abort, p.timeout_ns)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t sa = sbase + st.idx * G::STAGE;
            const uint32_t sb = sa + kABytes * G::NP;
#pragma unroll
            for (int s = 0; s < NSUB; ++s)
              mma<KIND>(d_main, sw128_desc(sa + 32u * s), sw128_desc(sb + 32u * s), idesc,
                        (kb > 0 || s > 0) ? 1u : 0u);
            mma_commit(empty(st.idx));
            st.next(S);
          }
          if (ok) {
            mma_commit(tfull(acc.idx));
            acc.next(NACC);
          }
        }
        if (!ok) break;
      }
      // all MMAs issued by this thread complete before TMEM is freed
      mma_commit(drain);
      wait_bounded(drain, 0, p.error, nullptr, p.timeout_ns);
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------ epilogue
    const int q = warp & 3;             // this warp may read TMEM lanes 32q .. 32q+31
    const int half = (warp - 2) >> 2;   // and owns accumulator columns half*64 ..
    Ring sc, acc;
    const float alpha = p.alpha, beta = p.beta;
    for (;;) {
      int ok = 1;
      if (lane == 0) ok = wait_bounded(sfull(sc.idx), sc.phase, p.error, abort, p.timeout_ns);
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) break;
      const int it = slots[sc.idx];
      __syncwarp();
      if (lane == 0) mbar_arrive(sempty(sc.idx));
      sc.next(kSchedSlots);
      if (it < 0) break;
      const TileItem ti = p.items[it];
      const MatDesc d = p.descs[ti.mat];
      float* C = p.C[ti.mat];
      const int bn = tc_cfg_bn(d.cfg);
      const bool swap = tc_cfg_swap(d.cfg);
      const int row0 = ti.tm * kTcBM + q * 32;        // A-side row of lane 0
      const long long ldc = d.ldc;
      const int c_lo = half * kEpiCols;               // first accumulator column owned
      const int ncols = max(0, min(kEpiCols, bn - c_lo));
      const int col_base = ti.tn * bn + c_lo;         // B-side index of owned column 0
      if (beta != 0.0f) c_prefetch<kEpiCols>(C, ldc, d.M, d.N, swap, row0, col_base, ncols, lane);
      float r[kEpiCols];
#pragma unroll
      for (int j = 0; j < kEpiCols; ++j) r[j] = 0.0f;
      if constexpr (SPLIT) {
        // promote every MMA group into FP32 registers (round to nearest)
        const int nk = (d.K + KE - 1) / KE;
        const int nsub = (d.K + KE / NSUB - 1) / (KE / NSUB);
        const int ngroups = (d.K <= kFineK) ? nsub : (nk + kGroupKB - 1) / kGroupKB;
        for (int g = 0; g < ngroups; ++g) {
          if (lane == 0) ok = wait_bounded(tfull(acc.idx), acc.phase, p.error, abort, p.timeout_ns);
          ok = __shfl_sync(0xffffffffu, ok, 0);
          if (!ok) break;
          tc_fence_after();
          const uint32_t tb = tmem + ((uint32_t)(q * 32) << 16) + acc.idx * 128u + c_lo;
          float v[kEpiCols];
#pragma unroll
          for (int c = 0; c < kEpiCols / 16; ++c)
            if (c * 16 < ncols) tmem_ld16(tb + c * 16, v + c * 16);
          tmem_wait_ld();
#pragma unroll
          for (int c = 0; c < kEpiCols / 16; ++c)
            if (c * 16 < ncols) {
#pragma unroll
              for (int j = 0; j < 16; ++j) r[c * 16 + j] += v[c * 16 + j];
            }
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(tempty(acc.idx));
          acc.next(NACC);
        }
        if (!ok) break;
      } else {
        if (lane == 0) ok = wait_bounded(tfull(acc.idx), acc.phase, p.error, abort, p.timeout_ns);
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) break;
        tc_fence_after();
        const uint32_t tb = tmem + ((uint32_t)(q * 32) << 16) + acc.idx * 256u + c_lo;
#pragma unroll
        for (int c = 0; c < kEpiCols / 16; ++c)
          if (c * 16 < ncols) tmem_ld16(tb + c * 16, r + c * 16);
        tmem_wait_ld();
        if (d.K == 0) {
#pragma unroll
          for (int j = 0; j < kEpiCols; ++j) r[j] = 0.0f;
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(tempty(acc.idx));
        acc.next(NACC);
      }
      c_store<kEpiCols>(r, C, ldc, d.M, d.N, swap, row0, col_base, ncols, alpha, beta, lane);
    }
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) tmem_dealloc(tmem, 512);
  if (p.cta_times && threadIdx.x == 0) p.cta_times[2 * blockIdx.x + 1] = gtimer();
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

template <int KIND, int SPLIT>
cudaError_t launch_gemm(const TcGemmParams& p, int grid, cudaStream_t s) {
  static bool attr = false;
  const int bytes = Geo<SPLIT>::BYTES;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(tc_gemm_kernel<KIND, SPLIT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  tc_gemm_kernel<KIND, SPLIT><<<grid, kThreads, bytes, s>>>(p);
  return cudaGetLastError();
}

// Self-test of the bounded mbarrier wait every tensor-core kernel uses: one
// CTA waits on a barrier that nothing will ever arrive on.  The wait must
// give up after limit_ns, set bit 0 of *err, and let the kernel return;
// out[0] = 1 records that the thread got past the wait, out[1] the wait's
// result (0 = gave up).
__global__ void bounded_wait_selftest_kernel(int* err, int* out, unsigned long long limit_ns) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ int abort_flag;
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(&bar), 1);
    abort_flag = 0;
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const bool ok = wait_bounded(smem_u32(&bar), 0, err, &abort_flag, limit_ns);
    out[1] = ok ? 1 : 0;
    out[0] = 1;
  }
}

}  // namespace

cudaError_t tc_wait_selftest_launch(int* err, int* out, unsigned long long limit_ns,
                                    cudaStream_t s) {
  bounded_wait_selftest_kernel<<<1, 32, 0, s>>>(err, out, limit_ns);
  return cudaGetLastError();
}

cudaError_t tc_tmap_launch(const TcTmapParams& p, cudaStream_t s) {
  if (p.batch == 0) return cudaSuccess;
  tc_tmap_kernel<<<p.batch, 128, 0, s>>>(p);  // 4 warps = the 4 maps of one matrix
  return cudaGetLastError();
}

cudaError_t tc_pack_launch(const TcPackParams& p, int grid, cudaStream_t s) {
  if (p.n_jobs == 0 && !p.n_jobs_dev) return cudaSuccess;
  tc_pack_kernel<<<grid, 256, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t tc_gemm_launch(int kind, int split, const TcGemmParams& p, int grid, cudaStream_t s) {
  if (kind == kKindTF32 && !split) return launch_gemm<kKindTF32, 0>(p, grid, s);
  if (kind == kKindTF32 && split) return launch_gemm<kKindTF32, 1>(p, grid, s);
  if (kind == kKindBF16 && split) return launch_gemm<kKindBF16, 1>(p, grid, s);
  return cudaErrorInvalidValue;
}

int tc_smem_bytes(int kind, int split) {
  (void)kind;
  return split ? Geo<1>::BYTES : Geo<0>::BYTES;
}

}  // namespace bgemm
