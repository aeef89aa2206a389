// tc2_kernel.cu -- the split-precision tensor-core GEMM on CTA pairs
// (tcgen05 cta_group::2, two SMs per output tile).
//
// Each cluster of two CTAs owns a 256 x BN output tile (BN = 64, 128 or 256)
// of one matrix: CTA r loads rows [128r, 128r + 128) of the A side and rows
// [r*BN/2, (r+1)*BN/2) of the B side (hi and lo halves) with TMA into its own
// shared memory, the leader CTA issues every cta_group::2 MMA, and each CTA
// receives its 128 x BN slice of the accumulator in its own TMEM.  Per
// 128-byte K slice a CTA loads at most 64 KB for 128 x 256 outputs -- half
// the L2 traffic per flop of the one-SM kernel (tc_kernel.cu), which is what
// bounds that kernel.
//
// Accumulation is group-promoted as in tc_kernel.cu: each group accumulates
// into a fresh 256-column TMEM buffer (2-deep ring) with the small products
// first, and the epilogue warps of both CTAs add it into FP32 registers with
// round-to-nearest.  The group length per bucket of K comes from the launch's
// autotuned TcSchedule (a number of 128-byte K slices, or one MMA with lo*lo
// kept on the small-K path).
//
// Scheduling is dynamic: the leader CTA's producer pulls the next item of
// the largest-first queue with one atomic (fetched a tile ahead, so its
// latency hides behind the current tile's loads) and publishes it in a
// 4-slot ring in the shared memory of both CTAs (a remote store plus a
// release.cluster arrive on the peer's barrier).  The leader's MMA lane, the
// 16 epilogue warps of both CTAs and the peer's producer read each slot and
// acknowledge it on the leader's sempty barrier; -1 ends the walk.  The last
// cluster to finish resets the queue head, so graph replays need no memset.
//
// Synchronisation across the pair:
//   full[s]   leader only: its producer expects the bytes of both CTAs; the
//             peer's TMA completes on the leader's barrier (cta_group::2 TMA);
//   empty[s]  both CTAs: the leader's commit is multicast to the pair;
//   tfull[b]  both CTAs: multicast commit when a group's MMAs finish;
//   tempty[b] leader only: 16 arrivals (8 epilogue warps x 2 CTAs), relaxed:
//             each warp's TMEM loads have completed before it arrives;
//   sfull[j]  both CTAs: the leader's producer published schedule slot j;
//   sempty[j] leader only: 18 arrivals (leader MMA lane, peer producer,
//             8 epilogue warps x 2 CTAs) once slot j has been read.
// All waits are bounded as in tc_kernel.cu.
#include <stdint.h>

#include "tc_epilogue.h"
#include "tc_ptx.h"
#include "tile_table.h"

namespace bgemm {
namespace {

constexpr int kRows = 128;                 // A-side rows per CTA
constexpr int kA = kRows * 128;            // 16 KB per part
constexpr int kB = 128 * 128;              // B-side half: up to 128 rows
constexpr int kNAcc = 2;                   // 256-column accumulator buffers
constexpr int kSched = 4;                  // schedule slots (items published ahead)
// Stage ring of 3 stages of 64 KB, two parts per side: the split modes' hi and
// lo halves of one 128-byte K slice, or two consecutive K slices of the
// single-product TF32 mode (four TMA boxes per stage either way: one thread
// keeps ~150 GB/s per SM in flight with four boxes per stage, ~100 with two).
template <int SPLIT>
struct Geo2 {
  static constexpr int NP = 2;
  static constexpr int STAGE = NP * (kA + kB);
  static constexpr int S = 3;
  static constexpr int NBAR = 2 * S + 2 * kNAcc + 1 + 2 * kSched;
  // barriers | TMEM address, abort flag (16 B) | schedule slots | alignment
  static constexpr int SMEM = S * STAGE + NBAR * 8 + 16 + 4 * kSched + 1024;
};
constexpr int kSmemMax = Geo2<1>::SMEM > Geo2<0>::SMEM ? Geo2<1>::SMEM : Geo2<0>::SMEM;
constexpr int kEpiWarps2 = 8;              // 2 per TMEM lane quadrant
constexpr int kCols = 128;                 // accumulator columns per epilogue warp
// Three warpgroups: warpgroup 0 = producer (warp 0), MMA issuer (warp 1) and
// two idle warps; warpgroups 1 and 2 = the 8 epilogue warps.  At launch every
// thread gets 168 registers (3 warps per SM sub-partition); warpgroup 0 gives
// most of its share to the epilogue warps, whose 128 accumulator columns per
// lane would otherwise spill: 128 x 56 + 256 x 224 = 384 x 168.
constexpr int kThreads2 = 384;
constexpr int kEpiWarp0 = 4;               // first epilogue warp
constexpr uint32_t kRegsCtl = 56, kRegsEpi = 224, kRegsLaunch = 168;
static_assert(128 * kRegsCtl + 256 * kRegsEpi <= kThreads2 * kRegsLaunch, "register split");
// Promotion groups of the split modes come per bucket of K from the launch's
// TcSchedule (autotuned table): group g > 0 = g 128-byte K slices per TMEM
// buffer, g = 0 = the small-K path (promote every MMA, keep lo*lo).
__device__ __forceinline__ int group_slices(const TcGemmParams& p, int K) {
  return p.sched.group(tc_sched_bucket(K));
}
// beta != 0: promotion groups before the tile's end at which C is prefetched
// into L2 (autotuned, tile_table.h; 0 = no prefetch)
constexpr int kCPrefetchLead = kTcCPrefetchLead;
static_assert(kCPrefetchLead >= 0 && kCPrefetchLead <= 16, "C prefetch lead out of range");

// MMA width of a tile along the B side: bn, or for the matrix's last tile
// column its remaining width rounded up to 16 (the pair MMA's N step), so
// that the padding of a ragged edge is not multiplied.  CTA r then loads
// B-side rows [tn*bn + r*n/2, +n/2), the columns stay contiguous.
__device__ __forceinline__ int tile_n(const MatDesc& d, int tn, int bn) {
  const int rem = (tc_cfg_swap(d.cfg) ? d.M : d.N) - tn * bn;
  return min(bn, (rem + 15) & ~15);
}

template <int KIND>
__device__ __forceinline__ uint32_t make_idesc_pair(int n) {
  constexpr uint32_t fmt = (KIND == kKindTF32) ? 2u : 1u;
  return (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(256 >> 4) << 24);
}

// BETA: the launch's beta is nonzero (C is read: late L2 prefetch, 16 reads in
// flight).  The beta = 0 form is a separate instantiation that keeps the
// plain epilogue's code (the read path's registers slowed it by ~4 %).
template <int KIND, int SPLIT, bool BETA>
__global__ void __launch_bounds__(kThreads2, 1) tc2_gemm_kernel(const TcGemmParams p) {
  using G = Geo2<SPLIT>;
  constexpr int kS = G::S;
  constexpr int kStage = G::STAGE;
  constexpr int kNBar = G::NBAR;
  constexpr int KE = (KIND == kKindTF32) ? 32 : 64;  // elements per 128-byte slice
  constexpr int NSUB = 4;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t pad = (1024u - (raw & 1023u)) & 1023u;
  uint8_t* smem = smem_raw + pad;
  const uint32_t sbase = raw + pad;
  const uint32_t bar0 = sbase + kS * kStage;
  auto full = [&](int s) { return bar0 + 8u * s; };
  auto empty = [&](int s) { return bar0 + 8u * (kS + s); };
  auto tfull = [&](int s) { return bar0 + 8u * (2 * kS + s); };
  auto tempty = [&](int s) { return bar0 + 8u * (2 * kS + kNAcc + s); };
  const uint32_t drain = bar0 + 8u * (2 * kS + 2 * kNAcc);
  auto sfull = [&](int j) { return bar0 + 8u * (2 * kS + 2 * kNAcc + 1 + j); };
  auto sempty = [&](int j) { return bar0 + 8u * (2 * kS + 2 * kNAcc + 1 + kSched + j); };
  volatile uint32_t* tmem_slot =
      reinterpret_cast<volatile uint32_t*>(smem + kS * kStage + kNBar * 8);
  volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);
  volatile int* slots = reinterpret_cast<volatile int*>(tmem_slot + 4);
  const uint32_t slots_addr = smem_u32(const_cast<int*>(slots));

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int n_items = p.n_items_dev ? *p.n_items_dev : p.n_items;
  const uint32_t rank = cluster_ctarank();
  const bool leader = rank == 0;
  const int ncl = gridDim.x >> 1;
  if (p.cta_times && threadIdx.x == 0) p.cta_times[2 * blockIdx.x] = gtimer();

  if (threadIdx.x == 0) {
    for (int s = 0; s < kS; ++s) {
      mbar_init(full(s), 1);
      mbar_init(empty(s), 1);
    }
    for (int s = 0; s < kNAcc; ++s) {
      mbar_init(tfull(s), 1);
      mbar_init(tempty(s), 2 * kEpiWarps2);
    }
    for (int j = 0; j < kSched; ++j) {
      mbar_init(sfull(j), 1);
      mbar_init(sempty(j), 2 + 2 * kEpiWarps2);
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

  // Each warpgroup sets its register budget at one point that all four of
  // its warps execute (setmaxnreg is warpgroup-aligned), ahead of the roles'
  // code, so that the compiler allocates every role for its budget.
  if (warp < kEpiWarp0) {
    regs_shrink<kRegsCtl>();
    if (warp == 0) {
      // ------------------------------------------------------------ producer
      if (lane == 0) {
        Ring st, sc;
        // stages with a load in flight, and the phase each was loaded in (bit s)
        uint32_t inflight = 0, inflight_phase = 0;
        bool ok = true;
        int last_mat = -1;
        // The leader publishes each item one tile ahead of its own loads, so
        // the peer's producer and the consumers find the next item ready.
        auto pull = [&]() {
          const int v = atomicAdd(p.counters, 1);
          return v < n_items ? v : -1;
        };
        auto publish = [&](int v) {
          if (!wait_bounded_cluster(sempty(sc.idx), sc.phase ^ 1u, p.error, abort, p.timeout_ns))
            return false;
          slots[sc.idx] = v;
          st_cluster_u32(mapa_shared(slots_addr + 4u * sc.idx, 1), (uint32_t)v);
          mbar_arrive(sfull(sc.idx));
          mbar_arrive_cluster(mapa_shared(sfull(sc.idx), 1));
          sc.next(kSched);
          return true;
        };
        int cur = -1, nxt = -1;
        if (leader) {
          cur = pull();
          ok = publish(cur);
          if (ok && cur >= 0) nxt = pull();
        }
        while (ok) {
          int it;
          if (leader) {
            it = cur;
            if (it < 0) break;
            if (!publish(nxt)) {
              ok = false;
              break;
            }
            const int after = nxt >= 0 ? pull() : -1;
            cur = nxt;
            nxt = after;
          } else {
            if (!wait_bounded_cluster(sfull(sc.idx), sc.phase, p.error, abort, p.timeout_ns)) {
              ok = false;
              break;
            }
            it = slots[sc.idx];
            mbar_arrive_cluster(mapa_shared(sempty(sc.idx), 0));
            sc.next(kSched);
            if (it < 0) break;
          }
          const TileItem ti = p.items[it];
          const MatDesc d = p.descs[ti.mat];
          const int bn = tc2_cfg_bn(d.cfg);
          const int hb = bn >> 1;
          const CUtensorMap* tm = p.tmaps + 4 * ti.mat;
          if (ti.mat != last_mat && d.K > 0) {
            for (int q = 0; q < 4; ++q) tmap_acquire(tm + q);
            last_mat = ti.mat;
          }
          const int nk = (d.K + KE - 1) / KE;           // 128-byte K slices
          const int nst = SPLIT ? nk : (nk + 1) / 2;     // stages
          const int row_a = ti.tm * 256 + (int)rank * kRows;
          const int row_b = ti.tn * bn + (int)rank * (tile_n(d, ti.tn, bn) >> 1);
          for (int kb = 0; kb < nst; ++kb) {
            // single product: slices 2kb and (if it exists) 2kb + 1
            const int parts = SPLIT ? 2 : (2 * kb + 1 < nk ? 2 : 1);
            const uint32_t tx = 2u * parts * (uint32_t)(kA + hb * 128);  // both CTAs
            if (!wait_bounded(empty(st.idx), st.phase ^ 1u, p.error, abort, p.timeout_ns)) {
              ok = false;
              break;
            }
            const uint32_t sa = sbase + st.idx * kStage;
            const uint32_t sb = sa + G::NP * kA;
            const uint32_t fb = mapa_shared(full(st.idx), 0);
            if (leader) {
              mbar_arrive_expect_tx(full(st.idx), tx);
              inflight |= 1u << st.idx;
              inflight_phase = (inflight_phase & ~(1u << st.idx)) | (st.phase << st.idx);
            }
            if (SPLIT) {
              tma_load_2d_pair(sa, tm + 0, kb * KE, row_a, fb);
              tma_load_2d_pair(sb, tm + 2, kb * KE, row_b, fb);
              tma_load_2d_pair(sa + kA, tm + 1, kb * KE, row_a, fb);
              tma_load_2d_pair(sb + kB, tm + 3, kb * KE, row_b, fb);
            } else {
              for (int j = 0; j < parts; ++j) {
                tma_load_2d_pair(sa + j * kA, tm + 0, (2 * kb + j) * KE, row_a, fb);
                tma_load_2d_pair(sb + j * kB, tm + 2, (2 * kb + j) * KE, row_b, fb);
              }
            }
            st.next(kS);
          }
          if (!ok) break;
        }
        // The leader's full barriers count the bytes of both CTAs: once every
        // phase it expected has completed, no copy of either CTA is in flight.
        if (leader) {
          for (int s = 0; s < kS; ++s)
            if ((inflight >> s) & 1u)
              wait_bounded(full(s), (inflight_phase >> s) & 1u, p.error, nullptr, p.timeout_ns);
        }
        if (!ok) {
          const uint64_t t0 = gtimer();  // aborted: give stray copies time to land
          while (gtimer() - t0 < 200000ull) {
          }
        }
      }
      __syncwarp();
    } else if (warp == 1) {
      // -------------------------------------------------- MMA issue (leader)
      if (lane == 0 && leader) {
        Ring st, acc, sc;
        bool ok = true;
        while (ok) {
          if (!wait_bounded(sfull(sc.idx), sc.phase, p.error, abort, p.timeout_ns)) break;
          const int it = slots[sc.idx];
          mbar_arrive(sempty(sc.idx));
          sc.next(kSched);
          if (it < 0) break;
          const TileItem ti = p.items[it];
          const MatDesc d = p.descs[ti.mat];
          const int bn = tc2_cfg_bn(d.cfg);
          const uint32_t idesc = make_idesc_pair<KIND>(tile_n(d, ti.tn, bn));
          const int nk = (d.K + KE - 1) / KE;
          const int nsub = (d.K + KE / NSUB - 1) / (KE / NSUB);
          const int gs = SPLIT ? group_slices(p, d.K) : 1;
          const bool fine = SPLIT && gs == 0;
          int kg = 0;  // slice within the current promotion group
          // A 256-column buffer holds P = 256 / bn promotion groups side by
          // side (sub-accumulators at column stride bn), so narrow tiles run P
          // groups ahead before waiting on the epilogue's drain.
          const int P = 256 / bn;
          int sub = 0;        // promotion group within the current buffer
          uint32_t gbuf = 0;  // TMEM address of the current group
          auto begin_group = [&]() {
            if (sub == 0) {
              if (!wait_bounded(tempty(acc.idx), acc.phase ^ 1u, p.error, abort, p.timeout_ns))
                return false;
              tc_fence_after();
            }
            gbuf = tmem + acc.idx * 256u + (uint32_t)(sub * bn);
            return true;
          };
          auto end_group = [&](bool last) {
            if (++sub == P || last) {
              mma_commit_pair(tfull(acc.idx));
              acc.next(kNAcc);
              sub = 0;
            }
          };
          const int nst = SPLIT ? nk : (nk + 1) / 2;  // stages (the producer's count)
          for (int kb = 0; kb < nst; ++kb) {
            if (!wait_bounded(full(st.idx), st.phase, p.error, abort, p.timeout_ns)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t sa = sbase + st.idx * kStage;
            const uint32_t sb = sa + G::NP * kA;
            const int s_end = min(NSUB, nsub - kb * NSUB);
            if (!SPLIT) {
              // one product: a single accumulator per tile, the 2-deep ring
              // alternating between tiles; the stage holds K slices 2kb, 2kb+1
              if (kb == 0) {
                if (!wait_bounded(tempty(acc.idx), acc.phase ^ 1u, p.error, abort, p.timeout_ns)) {
                  ok = false;
                  break;
                }
                tc_fence_after();
              }
              const uint32_t buf = tmem + acc.idx * 256u;
              for (int j = 0; j < 2 && 2 * kb + j < nk; ++j) {
                const int slice = 2 * kb + j;
                const int se = min(NSUB, nsub - slice * NSUB);
                for (int s = 0; s < se; ++s)
                  mma_pair<KIND>(buf, sw128_desc(sa + j * kA + 32u * s),
                                 sw128_desc(sb + j * kB + 32u * s), idesc,
                                 (slice > 0 || s > 0) ? 1u : 0u);
              }
              if (kb == nst - 1) {
                mma_commit_pair(tfull(acc.idx));
                acc.next(kNAcc);
              }
            } else if (fine) {
              for (int s = 0; s < s_end && ok; ++s) {
                if (!begin_group()) {
                  ok = false;
                  break;
                }
                const uint32_t buf = gbuf;
                // small K: the split error dominates, so lo*lo is kept too
                mma_pair<KIND>(buf, sw128_desc(sa + kA + 32u * s), sw128_desc(sb + kB + 32u * s),
                               idesc, 0u);
                mma_pair<KIND>(buf, sw128_desc(sa + kA + 32u * s), sw128_desc(sb + 32u * s), idesc,
                               1u);
                mma_pair<KIND>(buf, sw128_desc(sa + 32u * s), sw128_desc(sb + kB + 32u * s), idesc,
                               1u);
                mma_pair<KIND>(buf, sw128_desc(sa + 32u * s), sw128_desc(sb + 32u * s), idesc, 1u);
                end_group(kb == nk - 1 && s == s_end - 1);
              }
              if (!ok) break;
            } else {
              // a group spans gs slices; small products of each slice first
              const bool first = kg == 0;
              if (first && !begin_group()) {
                ok = false;
                break;
              }
              const uint32_t buf = gbuf;
              for (int s = 0; s < s_end; ++s) {
                mma_pair<KIND>(buf, sw128_desc(sa + kA + 32u * s), sw128_desc(sb + 32u * s), idesc,
                               (first && s == 0) ? 0u : 1u);
                mma_pair<KIND>(buf, sw128_desc(sa + 32u * s), sw128_desc(sb + kB + 32u * s), idesc,
                               1u);
              }
              for (int s = 0; s < s_end; ++s)
                mma_pair<KIND>(buf, sw128_desc(sa + 32u * s), sw128_desc(sb + 32u * s), idesc, 1u);
              if (++kg == gs || kb == nk - 1) {
                end_group(kb == nk - 1);
                kg = 0;
              }
            }
            mma_commit_pair(empty(st.idx));
            st.next(kS);
          }
        }
        mma_commit_pair(drain);
        wait_bounded(drain, 0, p.error, nullptr, p.timeout_ns);
      }
      __syncwarp();
    }  // warps 2 and 3 are idle
  } else {
    // -------------------------------------------- epilogue (both CTAs)
    regs_grow<kRegsEpi>();
    const int q = warp & 3;  // TMEM lanes 32q .. 32q + 31
    const int half = (warp - kEpiWarp0) >> 2;
    Ring acc, sc;
    const float alpha = p.alpha, beta = p.beta;
    // Reads the next schedule slot (lane 0) and acknowledges it to the
    // leader.  The acknowledgment is a cluster-scope release, which waits for
    // this lane's earlier global stores; so the next item is fetched before a
    // tile's C stores, never right after them.
    auto fetch = [&]() {
      int v = -1;
      if (lane == 0) {
        // the peer's slots are written by the leader's producer (release.cluster)
        const bool got = leader ? wait_bounded(sfull(sc.idx), sc.phase, p.error, abort,
                                               p.timeout_ns)
                                : wait_bounded_cluster(sfull(sc.idx), sc.phase, p.error, abort,
                                                       p.timeout_ns);
        if (got) {
          v = slots[sc.idx];
          mbar_arrive_cluster(mapa_shared(sempty(sc.idx), 0));
        }
      }
      sc.next(kSched);
      return __shfl_sync(0xffffffffu, v, 0);
    };
    int it = fetch();
    while (it >= 0) {
      const TileItem ti = p.items[it];
      const MatDesc d = p.descs[ti.mat];
      float* C = p.C[ti.mat];
      const int bn = tc2_cfg_bn(d.cfg);
      const bool swap = tc_cfg_swap(d.cfg);
      const int row0 = ti.tm * 256 + (int)rank * kRows + q * 32;  // A-side row of lane 0
      const long long ldc = d.ldc;
      const int c_lo = half * kCols;
      const int ncols = max(0, min(kCols, tile_n(d, ti.tn, bn) - c_lo));
      const int col_base = ti.tn * bn + c_lo;
      if constexpr (!BETA) {
        // (never taken: this form is launched with beta = 0; the guarded
        // tile-start prefetch keeps its code as measured fastest)
        if (beta != 0.0f) c_prefetch<kCols>(C, ldc, d.M, d.N, swap, row0, col_base, ncols, lane);
      }
      const int nk = (d.K + KE - 1) / KE;
      const int nsub = (d.K + KE / NSUB - 1) / (KE / NSUB);
      const int gs = SPLIT ? group_slices(p, d.K) : 1;
      const int ngroups = !SPLIT ? (nk > 0 ? 1 : 0) : gs == 0 ? nsub : (nk + gs - 1) / gs;
      float r[kCols];
#pragma unroll
      for (int j = 0; j < kCols; ++j) r[j] = 0.0f;
      int ok = 1;
      // beta != 0: C is pulled into L2 kCPrefetchLead groups before the tile
      // ends (earlier, the operand stream evicts it again before c_store)
      const int g_pf = (BETA && kCPrefetchLead > 0) ? max(0, ngroups - kCPrefetchLead) : -1;
      if (BETA && kCPrefetchLead > 0 && ngroups == 0)
        c_prefetch<kCols>(C, ldc, d.M, d.N, swap, row0, col_base, ncols, lane);
      // buffers of up to P = 256 / bn promotion groups each (see the MMA lane);
      // the groups are added in K order, as if each had a buffer of its own
      const int P = SPLIT ? 256 / bn : 1;
      for (int g0 = 0; g0 < ngroups; g0 += P) {
        if (lane == 0) ok = wait_bounded(tfull(acc.idx), acc.phase, p.error, abort, p.timeout_ns);
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) break;
        tc_fence_after();
        const int nsubs = min(P, ngroups - g0);
        for (int sg = 0; sg < nsubs; ++sg) {
          if (BETA && g0 + sg == g_pf)
            c_prefetch<kCols>(C, ldc, d.M, d.N, swap, row0, col_base, ncols, lane);
          const uint32_t tb =
              tmem + ((uint32_t)(q * 32) << 16) + acc.idx * 256u + (uint32_t)(sg * bn) + c_lo;
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
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive_cluster_relaxed(mapa_shared(tempty(acc.idx), 0));
        acc.next(kNAcc);
      }
      if (!ok) break;
      it = fetch();
      if constexpr (BETA)
        c_store_pipe<kCols, 8>(r, C, ldc, d.M, d.N, swap, row0, col_base, ncols, alpha, beta, lane);
      else
        c_store<kCols>(r, C, ldc, d.M, d.N, swap, row0, col_base, ncols, alpha, beta, lane);
    }
  }

  tc_fence_before();
  __syncthreads();
  cluster_sync();
  tc_fence_after();
  if (warp == 1) tmem_dealloc_pair(tmem, 512);
  if (leader && threadIdx.x == 0) {
    // the last cluster to finish resets the queue for the next launch (every
    // leader has pulled its final item before it gets here)
    __threadfence();
    const unsigned prev = atomicAdd(reinterpret_cast<unsigned*>(p.counters) + 1, 1u);
    if (prev == (unsigned)ncl - 1) {
      atomicExch(p.counters, 0);
      atomicExch(p.counters + 1, 0);
      __threadfence();
    }
  }
  if (p.cta_times && threadIdx.x == 0) p.cta_times[2 * blockIdx.x + 1] = gtimer();
}

template <int KIND, int SPLIT, bool BETA>
cudaError_t launch2(const TcGemmParams& p, int grid, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(tc2_gemm_kernel<KIND, SPLIT, BETA>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         Geo2<SPLIT>::SMEM);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid, 1, 1);
  cfg.blockDim = dim3(kThreads2, 1, 1);
  cfg.dynamicSmemBytes = Geo2<SPLIT>::SMEM;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 2;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, tc2_gemm_kernel<KIND, SPLIT, BETA>, p);
}

template <int KIND, int SPLIT>
cudaError_t launch2b(const TcGemmParams& p, int grid, cudaStream_t s) {
  return p.beta != 0.0f ? launch2<KIND, SPLIT, true>(p, grid, s)
                        : launch2<KIND, SPLIT, false>(p, grid, s);
}

}  // namespace

cudaError_t tc2_gemm_launch(int kind, int split, const TcGemmParams& p, int grid,
                            cudaStream_t s) {
  if (grid < 2 || (grid & 1)) return cudaErrorInvalidValue;
  if (kind == kKindTF32 && !split) return launch2b<kKindTF32, 0>(p, grid, s);
  if (kind == kKindTF32) return launch2b<kKindTF32, 1>(p, grid, s);
  if (kind == kKindBF16 && split) return launch2b<kKindBF16, 1>(p, grid, s);
  return cudaErrorInvalidValue;
}

int tc2_max_clusters() {
  int n = 0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(2, 1, 1);
  cfg.blockDim = dim3(kThreads2, 1, 1);
  cfg.dynamicSmemBytes = kSmemMax;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 2;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaFuncSetAttribute(tc2_gemm_kernel<kKindTF32, 1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       kSmemMax);
  if (cudaOccupancyMaxActiveClusters(&n, tc2_gemm_kernel<kKindTF32, 1, true>, &cfg) != cudaSuccess)
    return 0;
  return n;
}

}  // namespace bgemm
