// tc2s_kernel.cu -- 3xTF32 GEMM on CTA pairs that splits its operands in
// shared memory.
//
// Same tile scheme as tc2_kernel.cu (a cluster of two CTAs per 256 x BN output
// tile, the leader issues cta_group::2 MMAs, group-promoted accumulation into
// FP32 registers), but the operands arrive as raw FP32: the pre-pass only
// transposes/compacts them to K-major rows (4 bytes per element instead of 8
// for a TF32 hi + lo pair), TMA loads raw 128-byte K slices into a 3-deep
// ring, and the eight epilogue warps -- between their promotion duties --
// split each raw slice into the swizzled hi and lo tiles the MMAs read
// (hi = TF32(x), lo = TF32(x - hi), round to nearest even).  The raw and
// hi/lo tiles share the 128-byte-swizzled K-major layout, so the split is an
// elementwise pass over 16-byte chunks at identical offsets.  This halves the
// bytes each SM pulls from L2 per flop and the bytes the pre-pass writes.
//
// Rings and barriers (per CTA unless noted):
//   raw_full[3]   producer's TMA bytes;          raw_empty[3]  8 converter warps
//   hilo_full[2]  leader only: 8 warps x 2 CTAs; hilo_empty[2] multicast commit
//   tfull[2]      multicast commit per group;    tempty[2]     leader only, 16
// The epilogue warps never block on one barrier while the other kind of work
// could proceed: each turn they poll (try_wait) for a raw slice to split and
// for an accumulator group to promote, and do whichever is ready.
#include <stdint.h>

#include "tc_epilogue.h"
#include "tc_ptx.h"

namespace bgemm {
namespace {

constexpr int kRows = 128;
constexpr int kTile = kRows * 128;          // 16 KB: 128 rows x 128 bytes
constexpr int kRawStage = 2 * kTile;        // raw A + raw B (B: up to 128 rows)
constexpr int kHiloStage = 4 * kTile;       // A hi, A lo, B hi, B lo
constexpr int kR = 3;
constexpr int kH = 2;
constexpr int kNAcc = 2;
constexpr int kNBar = 2 * kR + 2 * kH + 2 * kNAcc + 1;
constexpr int kSmem = kR * kRawStage + kH * kHiloStage + kNBar * 8 + 16 + 1024;
constexpr int kEpiWarps = 8;
constexpr int kCols = 128;
constexpr int kThreadsS = 64 + kEpiWarps * 32;
constexpr int kFineK = 64;
constexpr int KE = 32;  // FP32 elements per 128-byte slice

__device__ __forceinline__ int snake(int c, int t, int ncl) {
  const int base = t * ncl;
  return (t & 1) ? base + (ncl - 1 - c) : base + c;
}

__device__ __forceinline__ uint32_t make_idesc_pair_tf32(int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(256 >> 4) << 24);
}

__device__ __forceinline__ float4 split_lo(float4 x, float4 h) {
  auto lo = [](float v, float hv) {
    return ((__float_as_uint(v) & 0x7f800000u) != 0x7f800000u) ? round_keep(v - hv, 13) : 0.0f;
  };
  return make_float4(lo(x.x, h.x), lo(x.y, h.y), lo(x.z, h.z), lo(x.w, h.w));
}

__global__ void __launch_bounds__(kThreadsS, 1) tc2s_gemm_kernel(const TcGemmParams p) {
  constexpr int NSUB = 4;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw0 = smem_u32(smem_raw);
  const uint32_t pad = (1024u - (raw0 & 1023u)) & 1023u;
  uint8_t* smem = smem_raw + pad;
  const uint32_t sbase = raw0 + pad;
  const uint32_t hilo_base = sbase + kR * kRawStage;
  const uint32_t bar0 = hilo_base + kH * kHiloStage;
  auto raw_full = [&](int s) { return bar0 + 8u * s; };
  auto raw_empty = [&](int s) { return bar0 + 8u * (kR + s); };
  auto hilo_full = [&](int s) { return bar0 + 8u * (2 * kR + s); };
  auto hilo_empty = [&](int s) { return bar0 + 8u * (2 * kR + kH + s); };
  auto tfull = [&](int s) { return bar0 + 8u * (2 * kR + 2 * kH + s); };
  auto tempty = [&](int s) { return bar0 + 8u * (2 * kR + 2 * kH + kNAcc + s); };
  const uint32_t drain = bar0 + 8u * (2 * kR + 2 * kH + 2 * kNAcc);
  volatile uint32_t* tmem_slot = reinterpret_cast<volatile uint32_t*>(
      smem + kR * kRawStage + kH * kHiloStage + kNBar * 8);
  volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int n_items = p.n_items_dev ? *p.n_items_dev : p.n_items;
  const uint32_t rank = cluster_ctarank();
  const bool leader = rank == 0;
  const int cl = blockIdx.x >> 1;
  const int ncl = gridDim.x >> 1;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kR; ++s) {
      mbar_init(raw_full(s), 1);
      mbar_init(raw_empty(s), kEpiWarps);
    }
    for (int s = 0; s < kH; ++s) {
      mbar_init(hilo_full(s), 2 * kEpiWarps);
      mbar_init(hilo_empty(s), 1);
    }
    for (int s = 0; s < kNAcc; ++s) {
      mbar_init(tfull(s), 1);
      mbar_init(tempty(s), 2 * kEpiWarps);
    }
    mbar_init(drain, 1);
    *abort = 0;
    fence_mbar_init();
  }
  cluster_sync();
  if (warp == 1) {
    tmem_alloc_pair(smem_u32(const_cast<uint32_t*>(tmem_slot)), 512);
    tmem_relinquish_pair();
  }
  tc_fence_before();
  __syncthreads();
  cluster_sync();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------ producer: raw FP32 slices
    if (lane == 0) {
      Ring st;
      int inflight_phase[kR];
      bool inflight[kR];
      for (int s = 0; s < kR; ++s) inflight[s] = false, inflight_phase[s] = 0;
      bool ok = true;
      int last_mat = -1;
      for (int t = 0; ok; ++t) {
        const int it = snake(cl, t, ncl);
        if (it >= n_items) break;
        const TileItem ti = p.items[it];
        const MatDesc d = p.descs[ti.mat];
        const int bn = tc2_cfg_bn(d.cfg);
        const int hb = bn >> 1;
        const CUtensorMap* tm = p.tmaps + 4 * ti.mat;
        if (ti.mat != last_mat && d.K > 0) {
          tmap_acquire(tm);
          tmap_acquire(tm + 2);
          last_mat = ti.mat;
        }
        const int nk = (d.K + KE - 1) / KE;
        const uint32_t tx = (uint32_t)(kTile + hb * 128);
        const int row_a = ti.tm * 256 + (int)rank * kRows;
        const int row_b = ti.tn * bn + (int)rank * hb;
        for (int kb = 0; kb < nk; ++kb) {
          if (!wait_bounded(raw_empty(st.idx), st.phase ^ 1u, p.error, abort, p.timeout_ns)) {
            ok = false;
            break;
          }
          const uint32_t sa = sbase + st.idx * kRawStage;
          mbar_arrive_expect_tx(raw_full(st.idx), tx);
          inflight[st.idx] = true;
          inflight_phase[st.idx] = st.phase;
          tma_load_2d(sa, tm + 0, kb * KE, row_a, raw_full(st.idx));
          tma_load_2d(sa + kTile, tm + 2, kb * KE, row_b, raw_full(st.idx));
          st.next(kR);
        }
      }
      for (int s = 0; s < kR; ++s)
        if (inflight[s])
          wait_bounded(raw_full(s), (uint32_t)inflight_phase[s], p.error, nullptr, p.timeout_ns);
    }
    __syncwarp();
  } else if (warp == 1) {
    // ------------------------------------------------ MMA issue (leader)
    if (lane == 0 && leader) {
      Ring st, acc;
      bool ok = true;
      for (int t = 0; ok; ++t) {
        const int it = snake(cl, t, ncl);
        if (it >= n_items) break;
        const TileItem ti = p.items[it];
        const MatDesc d = p.descs[ti.mat];
        const int bn = tc2_cfg_bn(d.cfg);
        const uint32_t idesc = make_idesc_pair_tf32(bn);
        const int nk = (d.K + KE - 1) / KE;
        const int nsub = (d.K + KE / NSUB - 1) / (KE / NSUB);
        const bool fine = d.K <= kFineK;
        for (int kb = 0; kb < nk; ++kb) {
          if (!wait_bounded_cluster(hilo_full(st.idx), st.phase, p.error, abort, p.timeout_ns)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t sa = hilo_base + st.idx * kHiloStage;  // A hi | A lo | B hi | B lo
          const uint32_t sb = sa + 2 * kTile;
          const int s_end = min(NSUB, nsub - kb * NSUB);
          if (fine) {
            for (int s = 0; s < s_end && ok; ++s) {
              if (!wait_bounded_cluster(tempty(acc.idx), acc.phase ^ 1u, p.error, abort,
                                        p.timeout_ns)) {
                ok = false;
                break;
              }
              tc_fence_after();
              const uint32_t buf = tmem + acc.idx * 256u;
              // small K: the split error dominates, so lo*lo is kept too
              mma_pair<kKindTF32>(buf, sw128_desc(sa + kTile + 32u * s),
                                  sw128_desc(sb + kTile + 32u * s), idesc, 0u);
              mma_pair<kKindTF32>(buf, sw128_desc(sa + kTile + 32u * s), sw128_desc(sb + 32u * s),
                                  idesc, 1u);
              mma_pair<kKindTF32>(buf, sw128_desc(sa + 32u * s), sw128_desc(sb + kTile + 32u * s),
                                  idesc, 1u);
              mma_pair<kKindTF32>(buf, sw128_desc(sa + 32u * s), sw128_desc(sb + 32u * s), idesc,
                                  1u);
              mma_commit_pair(tfull(acc.idx));
              acc.next(kNAcc);
            }
            if (!ok) break;
          } else {
            if (!wait_bounded_cluster(tempty(acc.idx), acc.phase ^ 1u, p.error, abort,
                                      p.timeout_ns)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t buf = tmem + acc.idx * 256u;
            for (int s = 0; s < s_end; ++s) {
              mma_pair<kKindTF32>(buf, sw128_desc(sa + kTile + 32u * s), sw128_desc(sb + 32u * s),
                                  idesc, s > 0 ? 1u : 0u);
              mma_pair<kKindTF32>(buf, sw128_desc(sa + 32u * s), sw128_desc(sb + kTile + 32u * s),
                                  idesc, 1u);
            }
            for (int s = 0; s < s_end; ++s)
              mma_pair<kKindTF32>(buf, sw128_desc(sa + 32u * s), sw128_desc(sb + 32u * s), idesc,
                                  1u);
            mma_commit_pair(tfull(acc.idx));
            acc.next(kNAcc);
          }
          mma_commit_pair(hilo_empty(st.idx));
          st.next(kH);
        }
      }
      mma_commit_pair(drain);
      wait_bounded(drain, 0, p.error, nullptr, p.timeout_ns);
    }
    __syncwarp();
  } else {
    // ----------------------------- converters + epilogue (both CTAs, 8 warps)
    const int ew = warp - 2;      // 0..7
    const int q = warp & 3;       // TMEM lane quadrant
    const int half = ew >> 2;     // accumulator columns half*128 ..
    const float alpha = p.alpha, beta = p.beta;
    // conversion cursor
    int ct = 0, ckb = 0, c_nk = 0, c_hb = 0;
    bool conv_done = false;
    auto conv_tile = [&]() {  // advance to the next tile that has K > 0
      for (;;) {
        const int it = snake(cl, ct, ncl);
        if (it >= n_items) { conv_done = true; return; }
        const MatDesc d = p.descs[p.items[it].mat];
        c_nk = (d.K + KE - 1) / KE;
        c_hb = tc2_cfg_bn(d.cfg) >> 1;
        ckb = 0;
        if (c_nk > 0) return;
        ++ct;
      }
    };
    conv_tile();
    Ring rr, hh;
    // promotion cursor
    int pt = 0, pg = 0, p_ng = 0;
    bool prom_done = false;
    TileItem pti{};
    MatDesc pd{};
    auto prom_tile = [&]() {
      const int it = snake(cl, pt, ncl);
      if (it >= n_items) { prom_done = true; return; }
      pti = p.items[it];
      pd = p.descs[pti.mat];
      const int nk = (pd.K + KE - 1) / KE;
      const int nsub = (pd.K + KE / NSUB - 1) / (KE / NSUB);
      p_ng = (pd.K <= kFineK) ? nsub : nk;
      pg = 0;
    };
    prom_tile();
    Ring acc;
    float r[kCols];
#pragma unroll
    for (int j = 0; j < kCols; ++j) r[j] = 0.0f;
    uint64_t idle_since = 0;
    for (;;) {
      // a tile with no K (or finished groups) is stored at once
      while (!prom_done && pg == p_ng) {
        const int bn = tc2_cfg_bn(pd.cfg);
        const bool swap = tc_cfg_swap(pd.cfg);
        const int row0 = pti.tm * 256 + (int)rank * kRows + q * 32;
        const int c_lo = half * kCols;
        const int ncols = max(0, min(kCols, bn - c_lo));
        const int col_base = pti.tn * bn + c_lo;
        float* C = p.C[pti.mat];
        const long long ldc = pd.ldc;
        c_store<kCols>(r, C, ldc, pd.M, pd.N, swap, row0, col_base, ncols, alpha, beta, lane);
#pragma unroll
        for (int j = 0; j < kCols; ++j) r[j] = 0.0f;
        ++pt;
        prom_tile();
      }
      if (conv_done && prom_done) break;
      bool did = false;
      if (!conv_done) {
        int ready = 0;
        if (lane == 0)
          ready = mbar_try_wait(raw_full(rr.idx), rr.phase) &&
                  mbar_try_wait_cluster(hilo_empty(hh.idx), hh.phase ^ 1u);
        ready = __shfl_sync(0xffffffffu, ready, 0);
        if (ready) {
          // this warp's share of 16-byte chunks of raw A (128 rows) and raw B
          const int nchunks = 8 * (kRows + c_hb);
          uint8_t* raw = smem + rr.idx * kRawStage;
          uint8_t* hl = smem + kR * kRawStage + hh.idx * kHiloStage;
          for (int c = ew * 32 + lane; c < nchunks; c += kEpiWarps * 32) {
            const int off = c * 16;  // raw A: [0, 16K), raw B: [16K, 32K)
            const float4 x = *reinterpret_cast<const float4*>(raw + off);
            const float4 h = make_float4(round_keep(x.x, 13), round_keep(x.y, 13),
                                         round_keep(x.z, 13), round_keep(x.w, 13));
            const float4 l = split_lo(x, h);
            const int hoff = off < kTile ? off : off + kTile;  // A hi | A lo | B hi | B lo
            *reinterpret_cast<float4*>(hl + hoff) = h;
            *reinterpret_cast<float4*>(hl + hoff + kTile) = l;
          }
          fence_proxy_async_smem();
          __syncwarp();
          if (lane == 0) {
            mbar_arrive(raw_empty(rr.idx));
            mbar_arrive_cluster(mapa_shared(hilo_full(hh.idx), 0));
          }
          rr.next(kR);
          hh.next(kH);
          if (++ckb == c_nk) {
            ++ct;
            conv_tile();
          }
          did = true;
        }
      }
      if (!prom_done && pg < p_ng) {
        int ready = 0;
        if (lane == 0) ready = mbar_try_wait_cluster(tfull(acc.idx), acc.phase);
        ready = __shfl_sync(0xffffffffu, ready, 0);
        if (ready) {
          tc_fence_after();
          const int bn = tc2_cfg_bn(pd.cfg);
          const int c_lo = half * kCols;
          const int ncols = max(0, min(kCols, bn - c_lo));
          const uint32_t tb = tmem + ((uint32_t)(q * 32) << 16) + acc.idx * 256u + c_lo;
#pragma unroll
          for (int c = 0; c < kCols / 16; c += 2) {
            if (c * 16 < ncols) {
              float v0[16], v1[16];
              tmem_ld16(tb + c * 16, v0);
              tmem_ld16(tb + (c + 1) * 16, v1);
              tmem_wait_ld();
#pragma unroll
              for (int j = 0; j < 16; ++j) {
                r[c * 16 + j] += v0[j];
                r[(c + 1) * 16 + j] += v1[j];
              }
            }
          }
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive_cluster(mapa_shared(tempty(acc.idx), 0));
          acc.next(kNAcc);
          ++pg;
          did = true;
        }
      }
      if (did) {
        idle_since = 0;
      } else {
        int stop = 0;
        if (lane == 0) {
          const uint64_t now = gtimer();
          if (idle_since == 0) idle_since = now;
          if (*abort) stop = 1;
          else if (now - idle_since > p.timeout_ns) {
            atomicOr(p.error, 1);
            *abort = 1;
            stop = 1;
          }
        }
        if (__shfl_sync(0xffffffffu, stop, 0)) break;
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  cluster_sync();
  tc_fence_after();
  if (warp == 1) tmem_dealloc_pair(tmem, 512);
}

}  // namespace

cudaError_t tc2s_gemm_launch(const TcGemmParams& p, int grid, cudaStream_t s) {
  if (grid < 2 || (grid & 1)) return cudaErrorInvalidValue;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(tc2s_gemm_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid, 1, 1);
  cfg.blockDim = dim3(kThreadsS, 1, 1);
  cfg.dynamicSmemBytes = kSmem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 2;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, tc2s_gemm_kernel, p);
}

int tc2s_max_clusters() {
  int n = 0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(2, 1, 1);
  cfg.blockDim = dim3(kThreadsS, 1, 1);
  cfg.dynamicSmemBytes = kSmem;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 2;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaFuncSetAttribute(tc2s_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
  if (cudaOccupancyMaxActiveClusters(&n, tc2s_gemm_kernel, &cfg) != cudaSuccess) return 0;
  return n;
}

}  // namespace bgemm
