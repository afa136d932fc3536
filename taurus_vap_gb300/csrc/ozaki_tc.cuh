// The integer-splitting products of ozaki_core.cuh on the 5th-generation
// tensor cores (tcgen05): a warp-specialised pipeline fed by bulk asynchronous
// copies, accumulators in tensor memory, one thread issuing the MMAs.
//
// Every product reaching this path is a REAL product C' = A' B'^T of digit
// planes (complex operands are turned into real ones by the slicing pass:
// the real representation [[Ar, -Ai], [Ai, Ar]] for complex x complex, stacked
// real/imaginary rows otherwise).  The slicing pass writes each digit plane
// already tiled in the tensor cores' canonical no-swizzle K-major layout, so
// that the operands of one k-step (16 k, all 8 digits) of a 128-row A tile and
// of a 64-row B tile are two contiguous blocks of 32 KB and 16 KB, fetched by
// two cp.async.bulk copies that complete on the stage's mbarrier.
//
// Tile layout (bf16 elements) of R rows x 16 k of one digit plane: R/8 row
// groups x 2 k-blocks of 8 x 8 "core matrices" (8 rows x 16 bytes, 128 bytes
// contiguous): element (r, k) at (r / 8) * 128 + (k / 8) * 64 + (r % 8) * 8 +
// k % 8.  Descriptor LBO = 128 B (next k-block), SBO = 256 B (next row group).
// The tiles of one operand are ordered [slot][row tile][k-step][digit].
//
// Persistent CTAs (one per SM) claim output tiles dynamically.  Roles (576 threads):
// warps 0-15 read the accumulators (warp w: TMEM lanes
// 32 (w % 4) .. + 32 = tile rows, columns 16 (w / 4) .. + 16), warp 16 issues
// the copies, warp 17 allocates tensor memory and one of its threads issues
// the MMAs.  The product of every digit pair (s, t) with s + t <= 7 (M128
// N64 K16) accumulates into the TMEM accumulator of weight group g = s + t
// (8 groups x 64 columns = all 512 columns); pairs with the same s and
// adjacent t run as one wider MMA (issue_kstep).  Over a fold interval of 384 k a group sum
// (<= 8 pairs x 2^12 per k) stays below 2^24 and is an exact FP32 integer; at
// the end of an interval the epilogue warps read the accumulators (tcgen05.ld)
// and fold them into 64-bit integer accumulators in registers.
//
// Every wait is bounded: on a timeout the CTA raises its abort flag, stops
// issuing, waits (bounded) for the copies and MMAs it has issued and frees its
// tensor memory; the kernel then reports through the status word.
#pragma once

#include "ozaki_scaled.h"
#include "ozaki_core.cuh"

namespace tvap {
namespace oztc {

using oz::kDigits;
using oz::kKeep;

constexpr int kM = 128;                 // rows of A' per CTA (TMEM lanes)
constexpr int kN = 64;                  // rows of B' (output columns) per tile, at most (48 or 64)
constexpr int kEpiWarps = 16;           // accumulator readers
constexpr int kProducerWarp = 16;       // bulk copies
constexpr int kMmaWarp = 17;            // TMEM allocation + MMA issue
constexpr int kThreads = 32 * (kEpiWarps + 2);
constexpr int kTmemCols = 512;          // 8 groups x 64 columns
constexpr int kStages = 4;
constexpr int kFoldKs = 24;             // k-steps per fold interval: 8 x 2^12 x 384 < 2^24
constexpr long long kSpin = 1LL << 21;  // bounded waits (polls)

constexpr int kATileElems = kM * 16;                // one digit plane of a k-step
constexpr int kBTileElems = kN * 16;
constexpr int kABytes = kDigits * kATileElems * 2;  // 32 KB per k-step
constexpr int kBBytes = kDigits * kBTileElems * 2;  // 16 KB per k-step
constexpr int kStageBytes = kABytes + kBBytes;
constexpr size_t kSmemBytes = size_t(kStages) * kStageBytes;
// B' tile of BN rows: elements of one digit plane of a k-step, bytes of a k-step
__host__ __device__ constexpr int b_tile_elems(int bn) { return bn * 16; }
__host__ __device__ constexpr int b_bytes(int bn) { return kDigits * bn * 16 * 2; }
// one CTA per SM: two CTAs could never hold 512 TMEM columns each
static_assert(2 * kSmemBytes > 228 * 1024, "the tcgen05 kernel must not share an SM with itself");

// element offset of (row r, k) inside the k-step tile of one digit plane
__host__ __device__ __forceinline__ int tile_offset(int r, int k) {
  return (r >> 3) * 128 + ((k >> 3) & 1) * 64 + (r & 7) * 8 + (k & 7);
}

#ifdef __CUDACC__

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t desc(uint32_t addr) {
  // start >> 4, LBO = 128 B, SBO = 256 B, descriptor version 1, no swizzle
  return uint64_t((addr >> 4) & 0x3FFF) | (uint64_t(128 >> 4) << 16) | (uint64_t(256 >> 4) << 32) |
         (uint64_t(1) << 46);
}

// kind::f16, bf16 x bf16 -> f32, both K-major, M = 128, N = n
__host__ __device__ constexpr uint32_t idesc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(n >> 3) << 17) | (uint32_t(kM >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t id, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(ad), "l"(bd), "r"(id), "r"(accumulate));
}

__device__ __forceinline__ void commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smem_u32(mbar))
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(mbar)), "r"(count));
}

__device__ __forceinline__ void mbar_arrive(uint64_t* mbar) {
  asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(smem_u32(mbar))
               : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* mbar, uint32_t bytes) {
  asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}\n" ::"r"(
                   smem_u32(mbar)),
               "r"(bytes)
               : "memory");
}

// bulk global -> shared copy completing `bytes` on an mbarrier (addresses
// 16-byte aligned, size a multiple of 16)
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(mbar))
      : "memory");
}

__device__ __forceinline__ bool try_parity(uint64_t* mbar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(smem_u32(mbar)), "r"(parity)
      : "memory");
  return done != 0;
}

// bounded wait for the completion of phase `parity`; gives up early when the
// CTA's abort flag (if given) is raised.  `sleep` backs off between polls
// (for the many epilogue threads, so that they do not take issue slots from
// the producer and the MMA thread).
__device__ __forceinline__ bool wait_parity(uint64_t* mbar, uint32_t parity, volatile int* abort, bool sleep) {
  for (long long it = 0; it < kSpin; ++it) {
    if (try_parity(mbar, parity)) return true;
    if (abort && *abort) return false;
    if (sleep) __nanosleep(128);
  }
  return false;
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// 16 consecutive 32-bit TMEM columns of the warp's 32 lanes
__device__ __forceinline__ void ld16(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

// integer accumulators of one epilogue thread (16 columns): groups 0-3 (h)
// and 4-7 (l)
struct Acc {
  long long h[16], l[16];
};

constexpr int kRing = 4;  // tile numbers handed from the copy thread to the others

// shared control block
struct Ctl {
  uint64_t full[kStages], empty[kStages];
  uint64_t acc_full, acc_empty, mma_done;
  uint64_t tile_full[kRing], tile_empty[kRing];
  int tile_id[kRing];
  uint32_t tmem;
  int abort;
};

// MMAs of one k-step for all digit pairs (s, t), s + t <= 7.  The B digit
// tiles of a stage lie back to back (digit t at + t * 2 KB, row groups 256 B
// apart), so digits t0 .. t0 + c - 1 form ONE K-major operand of 64 c rows,
// and the accumulators of groups s + t0 .. s + t0 + c - 1 are adjacent TMEM
// column ranges: one MMA of N = 64 c covers c digit pairs.  Per digit s of A
// that is one MMA of N <= 256 (c <= 4) for t = 0..3 and one for t = 4..7-s:
// 12 MMAs per k-step, each A tile read from shared memory once or twice
// instead of 8 - s times.  FIRST = the k-step opens a fold interval (the
// products of s = 0, which reach every group, overwrite the accumulators).
// Every descriptor is the stage's base descriptor plus a constant (the
// start-address field is the low 14 bits and shared addresses stay below
// 2^18, so the addition never carries into the other fields).
template <int BN, bool FIRST>
__device__ __forceinline__ void issue_kstep(uint32_t tmem, const unsigned char* st) {
  const uint64_t da = desc(smem_u32(st)), db = desc(smem_u32(st + kABytes));
  constexpr uint32_t kAT = uint32_t(kATileElems * 2) >> 4, kBT = uint32_t(b_tile_elems(BN) * 2) >> 4;
#pragma unroll
  for (int s = 0; s < kDigits; ++s) {
#pragma unroll
    for (int t0 = 0; t0 <= kKeep - s; t0 += 4) {
      const int c = (kKeep - s - t0 + 1) < 4 ? (kKeep - s - t0 + 1) : 4;
      mma(tmem + uint32_t((s + t0) * BN), da + uint64_t(s * kAT), db + uint64_t(t0 * kBT), idesc(c * BN),
          (FIRST && s == 0) ? 0u : 1u);
    }
  }
}

// fold the accumulators of an interval into the integer accumulators (the
// warps whose 16 columns lie beyond a tile of BN columns read the last 16
// again, and store nothing)
template <int BN>
__device__ __forceinline__ void fold(uint32_t tmem, Acc& o) {
  const int warp = threadIdx.x >> 5;
  const uint32_t lane_base = uint32_t(32 * (warp & 3)) << 16;
  const uint32_t c0 = uint32_t(min((warp >> 2) * 16, BN - 16));
#pragma unroll
  for (int g = 0; g <= kKeep; ++g) {
    uint32_t r[16];
    ld16(tmem + lane_base + uint32_t(g * BN) + c0, r);
    ld_wait();
    const long long w = 1LL << (7 * (3 - (g & 3)));
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      const long long v = (long long)__float2int_rn(__uint_as_float(r[c])) * w;
      if (g < 4)
        o.h[c] += v;
      else
        o.l[c] += v;
    }
  }
}

// Persistent driver, called by every thread of the CTA.  Tiles are claimed
// dynamically: the copy thread takes the next tile number from *counter
// (zero before the launch) and hands it to the MMA thread and the epilogue
// through a ring of kRing entries (mbarriers tile_full / tile_empty), so that
// CTAs that start late -- their SMs held by kernels of other streams -- take
// fewer tiles instead of delaying the product.  A number >= ntiles ends the
// CTA.  tile_ptrs(tile, A, B) gives the tile's first k-step blocks (digit 0;
// nks_of(tile) k-steps of kABytes / b_bytes(BN) each follow contiguously); store(tile, acc)
// is called by the epilogue threads with the tile's integer accumulators,
// after the tensor memory has been handed back to the MMA thread, so that the
// stores of one tile overlap the MMAs of the next.  The copy thread runs
// ahead across tile boundaries.  Returns false on a timeout.
template <int BN, class TilePtrs, class NksOf, class Store>
__device__ bool run_tiles(int* counter, int ntiles, NksOf nks_of, unsigned char* smem, Ctl& ctl, TilePtrs tile_ptrs,
                          Store store) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  volatile int* abort = &ctl.abort;
  if (threadIdx.x == 0) {
    for (int q = 0; q < kStages; ++q) {
      mbar_init(&ctl.full[q], 1);
      mbar_init(&ctl.empty[q], 1);
    }
    for (int q = 0; q < kRing; ++q) {
      mbar_init(&ctl.tile_full[q], 1);
      mbar_init(&ctl.tile_empty[q], 32 * kEpiWarps + 1);
    }
    mbar_init(&ctl.acc_full, 1);
    mbar_init(&ctl.acc_empty, 32 * kEpiWarps);
    mbar_init(&ctl.mma_done, 1);
    ctl.abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&ctl.tmem)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = ctl.tmem;
  bool ok = true;
  long long issued = 0;  // copies issued (copy thread)
  if (warp == kProducerWarp) {
    if (lane == 0) {
      long long it = 0;  // k-steps over all tiles of the CTA
      for (int tt = 0; ok; ++tt) {
        const int slot = tt % kRing;
        if (tt >= kRing && !wait_parity(&ctl.tile_empty[slot], uint32_t((tt / kRing - 1) & 1), abort, false)) {
          ok = false;
          break;
        }
        int tile = atomicAdd(counter, 1);
        if (tile >= ntiles) tile = -1;
        ctl.tile_id[slot] = tile;
        mbar_arrive(&ctl.tile_full[slot]);
        if (tile < 0) break;
        const unsigned char *A, *B;
        tile_ptrs(tile, A, B);
        const int nks = nks_of(tile);
        for (int ks = 0; ks < nks; ++ks, ++it) {
          const int st = int(it % kStages);
          if (it >= kStages && !wait_parity(&ctl.empty[st], uint32_t((it / kStages - 1) & 1), abort, false)) {
            ok = false;
            break;
          }
          unsigned char* dst = smem + size_t(st) * kStageBytes;
          mbar_expect_tx(&ctl.full[st], uint32_t(kABytes + b_bytes(BN)));
          bulk_load(dst, A + size_t(ks) * kABytes, uint32_t(kABytes), &ctl.full[st]);
          bulk_load(dst + kABytes, B + size_t(ks) * b_bytes(BN), uint32_t(b_bytes(BN)), &ctl.full[st]);
          issued = it + 1;
        }
      }
    }
  } else if (warp == kMmaWarp) {
    if (lane == 0) {
      long long it = 0, fc = 0;  // k-steps and fold intervals over all tiles
      for (int tt = 0; ok; ++tt) {
        const int slot = tt % kRing;
        if (!wait_parity(&ctl.tile_full[slot], uint32_t((tt / kRing) & 1), abort, false)) {
          ok = false;
          break;
        }
        const int tile = ctl.tile_id[slot];
        mbar_arrive(&ctl.tile_empty[slot]);
        if (tile < 0) break;
        const int nks = nks_of(tile);
        for (int ks = 0; ks < nks; ++ks, ++it) {
          const int st = int(it % kStages);
          if (!wait_parity(&ctl.full[st], uint32_t((it / kStages) & 1), abort, false)) {
            ok = false;
            break;
          }
          const bool opens = (ks % kFoldKs) == 0;
          // a new interval overwrites the accumulators: the epilogue must have
          // read the previous one
          if (opens && fc > 0 && !wait_parity(&ctl.acc_empty, uint32_t((fc - 1) & 1), abort, false)) {
            ok = false;
            break;
          }
          fence_after();
          const unsigned char* sb = smem + size_t(st) * kStageBytes;
          if (opens)
            issue_kstep<BN, true>(tmem, sb);
          else
            issue_kstep<BN, false>(tmem, sb);
          commit(&ctl.empty[st]);
          if ((ks + 1) % kFoldKs == 0 || ks + 1 == nks) {
            commit(&ctl.acc_full);
            ++fc;
          }
        }
      }
      // every MMA issued by this thread has completed once mma_done flips
      commit(&ctl.mma_done);
      wait_parity(&ctl.mma_done, 0u, nullptr, false);
    }
  } else {
    // the epilogue warps decide as whole warps (a lane that gives up takes its
    // warp with it): the accumulator loads are warp-wide (.sync.aligned) and
    // the paired store shuffles between lanes
    long long fc = 0;
    for (int tt = 0; ok; ++tt) {
      const int slot = tt % kRing;
      if (!__all_sync(0xffffffffu, wait_parity(&ctl.tile_full[slot], uint32_t((tt / kRing) & 1), abort, true))) {
        ok = false;
        break;
      }
      const int tile = ctl.tile_id[slot];
      mbar_arrive(&ctl.tile_empty[slot]);
      if (tile < 0) break;
      const int nfold = (nks_of(tile) + kFoldKs - 1) / kFoldKs;  // fold intervals of the tile
      Acc o;
#pragma unroll
      for (int c = 0; c < 16; ++c) o.h[c] = o.l[c] = 0;
      for (int f = 0; f < nfold; ++f, ++fc) {
        if (!__all_sync(0xffffffffu, wait_parity(&ctl.acc_full, uint32_t(fc & 1), abort, true))) {
          ok = false;
          break;
        }
        fence_after();
        fold<BN>(tmem, o);
        fence_before();
        mbar_arrive(&ctl.acc_empty);
      }
      if (ok) store(tile, o);
    }
  }
  if (!ok) ctl.abort = 1;
  fence_before();
  __syncthreads();
  const bool all_ok = ctl.abort == 0;
  if (!all_ok && warp == kProducerWarp && lane == 0) {
    // the copies in flight land before the shared memory is released: the
    // last phase of each stage's barrier is that of its last copy
    for (long long it = (issued > kStages ? issued - kStages : 0); it < issued; ++it)
      wait_parity(&ctl.full[it % kStages], uint32_t((it / kStages) & 1), nullptr, false);
  }
  if (warp == kMmaWarp) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols));
  }
  return all_ok;
}

// value of column c (0..15 of the thread's quarter) before the exponent scale
__device__ __forceinline__ double value(const Acc& o, int c) { return fma(double(o.h[c]), 0x1p28, double(o.l[c])); }


#endif  // __CUDACC__

}  // namespace oztc
}  // namespace tvap
