// The integer-splitting products of ozaki_core.cuh on the 5th-generation
// tensor cores (tcgen05): accumulators in tensor memory, one thread issuing
// the MMAs, operands in shared memory.
//
// A CTA computes one real component (the real or the imaginary part) of a
// 128 x 64 output tile (MMA shape M128 N64 K16, bf16 x bf16 -> f32; on this
// part an M128 x N x K16 MMA costs the same for every N <= 64, so the widest
// N that tensor memory allows is used).  The component is a sum of one or two
// "segments" of real digit-plane products: real part of complex x complex =
// A_r B_r^T + (-A_i) B_i^T (the minus sign is the MMA's negate-A bit),
// imaginary part = A_r B_i^T + A_i B_r^T; with one real operand one segment.
// For every digit pair (s, t) with s + t <= 7 one MMA accumulates into the
// TMEM accumulator of weight group g = s + t: 8 groups x 64 columns = all 512
// TMEM columns.  Over a fold interval of 384 k (both segments counted) a
// group sum stays below 2^24 and is an exact FP32 integer; at the end of an
// interval the epilogue warps read the accumulators (tcgen05.ld), convert
// them to integers and fold them into 64-bit integer accumulators in
// registers.
//
// Pipeline: two shared-memory stages of two k-steps (32) each; all threads
// fill a stage with cp.async (zero-fill beyond the valid rows / K), a proxy
// fence and a barrier hand it to the MMA thread, whose tcgen05.commit on the
// stage's mbarrier releases it again.  Every wait is bounded: on a timeout
// the CTA stops issuing, waits (bounded) for its MMAs, reports through the
// status word and frees its tensor memory.
//
// Shared-memory operand layout (no swizzle, K-major): a tile of R rows x 16 k
// of one digit plane is R/8 row groups x 2 k-blocks of 8 x 8 "core matrices"
// (8 rows x 16 bytes each, 128 bytes contiguous); descriptor LBO = 128 B
// (next k-block), SBO = 256 B (next row group).
#pragma once

#include "ozaki_core.cuh"

namespace tvap {
namespace oztc {

using oz::kDigits;
using oz::kKeep;

constexpr int kM = 128;          // rows of op(A) per CTA
constexpr int kN = 64;           // columns of op(B) per CTA
constexpr int kThreads = 512;    // 16 warps: loaders, MMA issuer (thread 0), epilogue
constexpr int kTmemCols = 512;   // 8 groups x 64 columns
constexpr int kStages = 2;
constexpr int kKs = 2;           // k-steps (of 16) per stage
constexpr int kFoldSteps = 12;   // stages per fold interval: 8 x 384 x 2^12 < 2^24
constexpr long long kSpin = 1LL << 22;  // bounded waits

constexpr int kATile = kM * 16;  // bf16 per digit tile of a stage
constexpr int kBTile = kN * 16;
constexpr int kKsElems = kDigits * (kATile + kBTile);  // bf16 per k-step of a stage
constexpr int kStage = kKs * kKsElems;                 // bf16 per stage
constexpr size_t kSmemBytes = kStages * sizeof(__nv_bfloat16) * size_t(kStage);

// segments of a component: (A plane, B plane, negate A)
struct Seg {
  int pa, pb;
  bool neg;
};
template <int PA, int PB, int COMP>
struct Segs {
  static constexpr int n = (PA == 2 && PB == 2) ? 2 : 1;
  __host__ __device__ static constexpr Seg get(int i) {
    return (PA == 2 && PB == 2)
               ? (COMP == 0 ? (i == 0 ? Seg{0, 0, false} : Seg{1, 1, true})
                            : (i == 0 ? Seg{0, 1, false} : Seg{1, 0, false}))
               : (PA == 2 ? Seg{COMP, 0, false} : (PB == 2 ? Seg{0, COMP, false} : Seg{0, 0, false}));
  }
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t desc(uint32_t addr) {
  // start >> 4, LBO = 128 B, SBO = 256 B, descriptor version 1, no swizzle
  return uint64_t((addr >> 4) & 0x3FFF) | (uint64_t(128 >> 4) << 16) | (uint64_t(256 >> 4) << 32) |
         (uint64_t(1) << 46);
}

// kind::f16, bf16 x bf16 -> f32, both K-major, M = 128, N = 64
__device__ __forceinline__ uint32_t idesc(bool negate_a) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(negate_a) << 13) | (uint32_t(kN >> 3) << 17) |
         (uint32_t(kM >> 4) << 24);
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

// bounded wait for the completion of phase `parity` of an mbarrier
__device__ __forceinline__ bool wait_parity(uint64_t* mbar, uint32_t parity) {
  uint32_t done = 0;
  for (long long it = 0; it < kSpin && !done; ++it) {
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(mbar)), "r"(parity)
        : "memory");
  }
  return done != 0;
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

// integer accumulators of one epilogue thread: row (warp % 4) * 32 + lane,
// columns (warp / 4) * 16 .. + 16; groups 0-3 (h) and 4-7 (l)
struct Acc {
  long long h[16], l[16];
};

// shared control block
struct Ctl {
  uint64_t mbar[kStages];
  uint32_t tmem;
};

// kKs k-steps of one digit plane of A (128 rows) and of B (64 rows) into a
// stage; digit s at X + s * dstride; a_rows / b_rows valid rows, k >= klen zero
__device__ __forceinline__ void stage_load(const __nv_bfloat16* A, size_t a_dstride, int a_ld, int a_rows,
                                           const __nv_bfloat16* B, size_t b_dstride, int b_ld, int b_rows, int k0,
                                           int klen, __nv_bfloat16* st) {
#pragma unroll
  for (int q = 0; q < kKs; ++q) {
    __nv_bfloat16* sA = st + q * kKsElems;
    __nv_bfloat16* sB = sA + kDigits * kATile;
    const int kq = k0 + 16 * q;
    for (int v = threadIdx.x; v < kDigits * kM * 2; v += kThreads) {
      const int kb = v & 1, r = (v >> 1) & (kM - 1), dg = v >> 8;
      const int k = kq + kb * 8;
      const bool ok = r < a_rows && k < klen;
      __nv_bfloat16* dst = sA + dg * kATile + (((r >> 3) * 2 + kb) * 8 + (r & 7)) * 8;
      oz::cp_async16(dst, ok ? A + dg * a_dstride + size_t(r) * a_ld + k : A, ok);
    }
    for (int v = threadIdx.x; v < kDigits * kN * 2; v += kThreads) {
      const int kb = v & 1, r = (v >> 1) & (kN - 1), dg = v >> 7;
      const int k = kq + kb * 8;
      const bool ok = r < b_rows && k < klen;
      __nv_bfloat16* dst = sB + dg * kBTile + (((r >> 3) * 2 + kb) * 8 + (r & 7)) * 8;
      oz::cp_async16(dst, ok ? B + dg * b_dstride + size_t(r) * b_ld + k : B, ok);
    }
  }
}

// MMAs of one k-step for all digit pairs; FIRST = the k-step opens a fold
// interval (the first product into each group, at s = 0, overwrites it).
// Fully unrolled: every descriptor is the stage's base descriptor plus a
// constant (the start-address field is the low 14 bits and shared addresses
// stay below 2^18, so the addition never carries into the other fields).
template <bool FIRST>
__device__ __forceinline__ void issue_kstep(uint32_t tmem, const __nv_bfloat16* st, uint32_t id) {
  const uint64_t da = desc(smem_u32(st)), db = desc(smem_u32(st + kDigits * kATile));
  constexpr uint32_t kAT = uint32_t(kATile * 2) >> 4, kBT = uint32_t(kBTile * 2) >> 4;
#pragma unroll
  for (int s = 0; s < kDigits; ++s) {
#pragma unroll
    for (int t = 0; t < kDigits; ++t) {
      if (s + t > kKeep) continue;
      mma(tmem + uint32_t((s + t) * kN), da + uint64_t(s * kAT), db + uint64_t(t * kBT), id,
          (FIRST && s == 0) ? 0u : 1u);
    }
  }
}

// fold the accumulators of an interval into the integer accumulators
__device__ __forceinline__ void fold(uint32_t tmem, Acc& o) {
  const int warp = threadIdx.x >> 5;
  const uint32_t lane_base = uint32_t(32 * (warp & 3)) << 16;
  const uint32_t c0 = uint32_t((warp >> 2) * 16);
#pragma unroll
  for (int g = 0; g <= kKeep; ++g) {
    uint32_t r[16];
    ld16(tmem + lane_base + uint32_t(g * kN) + c0, r);
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

// The K loop of one component of a 128 x 64 tile.  A/B point at digit 0,
// plane 0 of the tile's first row; digit s, plane p at + (s * P + p) * plane;
// row r at + r * ld; rows >= a_rows / b_rows and k >= klen read as zero.
// Returns false on a timeout (the accumulators are then incomplete).
template <int PA, int PB, int COMP>
__device__ bool mainloop(const __nv_bfloat16* A, size_t a_plane, int a_ld, int a_rows, const __nv_bfloat16* B,
                         size_t b_plane, int b_ld, int b_rows, int klen, __nv_bfloat16* smem, Ctl& ctl, Acc& o) {
  using SG = Segs<PA, PB, COMP>;
  const int tid = threadIdx.x;
#pragma unroll
  for (int c = 0; c < 16; ++c) o.h[c] = o.l[c] = 0;
  const int nks = (klen + 16 * kKs - 1) / (16 * kKs);  // stages per segment
  const int ksteps = (klen + 15) / 16;                  // k-steps of 16 with data
  const int nsteps = SG::n * nks;
  bool ok = true;
  // commits issued on / completions consumed from each stage's mbarrier
  // (identical in every thread: the control flow is uniform)
  uint32_t committed[kStages] = {}, waited[kStages] = {};
  auto wait_stage = [&](int st) -> bool {
#pragma unroll
    for (int q = 0; q < kStages; ++q)
      if (q == st)
        while (waited[q] < committed[q]) {
          if (!wait_parity(&ctl.mbar[q], waited[q] & 1u)) return false;
          ++waited[q];
        }
    return true;
  };
  auto load = [&](int step) {
    const int seg = step / nks, ks = step - seg * nks;
    const Seg sg = SG::get(seg);
    stage_load(A + sg.pa * a_plane, a_plane * PA, a_ld, a_rows, B + sg.pb * b_plane, b_plane * PB, b_ld, b_rows,
               ks * 16 * kKs, klen, smem + (step % kStages) * kStage);
  };
  for (int j = 0; j < kStages - 1; ++j) {
    if (j < nsteps) load(j);
    oz::cp_async_commit();
  }
  for (int i = 0; i < nsteps; ++i) {
    const int st = i % kStages;
    const int j = i + kStages - 1;  // step to prefetch, into the stage step i - 1 used
    if (j < nsteps) {
      if (__syncthreads_or(!wait_stage(j % kStages))) {
        ok = false;
        break;
      }
      load(j);
    }
    oz::cp_async_commit();
    oz::cp_async_wait<kStages - 1>();
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    fence_before();
    __syncthreads();
    fence_after();
    const bool opens = (i % kFoldSteps) == 0;
    if (tid == 0) {
      const uint32_t id = idesc(SG::get(i / nks).neg);
      const int kchunk = i - (i / nks) * nks;
#pragma unroll
      for (int q = 0; q < kKs; ++q) {
        if (kchunk * kKs + q >= ksteps) break;  // k-steps beyond K hold only zeros
        if (opens && q == 0)
          issue_kstep<true>(ctl.tmem, smem + st * kStage + q * kKsElems, id);
        else
          issue_kstep<false>(ctl.tmem, smem + st * kStage + q * kKsElems, id);
      }
      commit(&ctl.mbar[st]);
    }
#pragma unroll
    for (int q = 0; q < kStages; ++q)
      if (q == st) ++committed[q];
    const bool closes = ((i + 1) % kFoldSteps) == 0 || i + 1 == nsteps;
    if (closes) {
      // every MMA issued so far completes with this step's commit
      if (__syncthreads_or(!wait_stage(st))) {
        ok = false;
        break;
      }
      fence_after();
      fold(ctl.tmem, o);
      fence_before();
      __syncthreads();
      fence_after();
    }
  }
  if (!ok) {
    // let the MMAs in flight finish (bounded) before the tensor memory is freed
    oz::cp_async_wait<0>();
#pragma unroll
    for (int q = 0; q < kStages; ++q) wait_stage(q);
  }
  return ok;
}

// tensor memory and barriers of a CTA (warp 0 allocates)
__device__ __forceinline__ void setup(Ctl& ctl) {
  const int warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    for (int q = 0; q < kStages; ++q)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&ctl.mbar[q])));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&ctl.tmem)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  fence_before();
  __syncthreads();
  fence_after();
}

__device__ __forceinline__ void teardown(Ctl& ctl) {
  fence_before();
  __syncthreads();
  if ((threadIdx.x >> 5) == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(ctl.tmem), "r"(kTmemCols));
}

// value of column c (0..15 of the thread's quarter) before the exponent scale
__device__ __forceinline__ double value(const Acc& o, int c) { return fma(double(o.h[c]), 0x1p28, double(o.l[c])); }

}  // namespace oztc
}  // namespace tvap
