// Core of the FP64-by-integer-splitting products on the bf16 tensor cores,
// shared by the batched GEMM (ozaki.cu) and the dense-block field operator
// (field_blocks.cu).
//
// A real FP64 row x (one row of op(A) or one column of op(B)) is scaled by a
// shared power of two so that every entry is an integer |X| < 2^54, and X is
// written in balanced base 2^7 with 8 digits in [-64, 63] (most significant
// first).  A digit is exact in bf16 and a digit product (<= 2^12) exact in
// FP32.  The tensor cores sum the products of digit pairs (s, t) with
// s + t <= 7 (the dropped pairs sum to at most 7.05 * 2^54 units of
// 2^(e_a + e_b - 106), i.e. 2^-49.2 of 2^(e_a + e_b), which is at most the
// product of the row's and the column's largest entries) into one
// FP32 accumulator per weight group g = s + t; over 64 consecutive k a group
// sum stays below 2^21 (2^23 for the 3M sum products below), so it is an exact
// integer.  Every 64 k the group sums are converted to integers and folded,
// with their weights 2^(7 (7 - g)), into two 64-bit integer accumulators per
// output (groups 0-3 and 4-7); the FP64 value is formed once at the end.
//
// Complex operands carry a real and an imaginary digit plane under one shared
// exponent.  Complex x complex takes three real products per digit pair (3M):
// rr, ii and (r + i)(r + i), the digit sums |d_r + d_i| <= 128 being exact in
// bf16.
#pragma once

#include <cuda_bf16.h>

#include <cstdint>
#include <cstring>

namespace tvap {
namespace oz {

constexpr int kDigits = 8;
constexpr int kKeep = 7;       // digit pairs with s + t <= kKeep are kept
constexpr int kKc = 32;        // K per pipeline stage
constexpr int kLd = kKc + 8;   // staged row (bf16): 80 bytes, conflict-free fragment loads
constexpr int kFoldK = 64;     // K between integer folds (FP32 group sums stay exact)
constexpr int kTile = 32;      // CTA output tile (rows and columns)
constexpr int kThreads = 256;  // 8 warps, one m16n8 sub-tile each
constexpr int kExpZero = -2000;

__host__ __device__ __forceinline__ long long dbits(double x) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(x);
#else
  long long b;
  std::memcpy(&b, &x, sizeof b);
  return b;
#endif
}

// unbiased exponent of a finite non-zero double (subnormals count as zero)
__host__ __device__ __forceinline__ int dexp(double x) {
  const int e = int((dbits(x) >> 52) & 0x7ff);
  return e == 0 ? kExpZero : e - 1023;
}

// integer X with x = X 2^(emax - 53), |X| < 2^54, rounded half up
__host__ __device__ __forceinline__ long long to_fixed(double x, int emax) {
  const long long b = dbits(x);
  const int eb = int((b >> 52) & 0x7ff);
  if (eb == 0) return 0;
  long long m = (b & ((1LL << 52) - 1)) | (1LL << 52);
  const int sh = (eb - 1023) - emax + 1;  // <= 1
  if (sh >= 0) {
    m <<= sh;
  } else if (sh > -60) {
    m = (m + (1LL << (-sh - 1))) >> (-sh);
  } else {
    m = 0;
  }
  return (b < 0) ? -m : m;
}

// balanced base-128 digits, d[0] most significant.  X = hi 2^28 + lo with
// 0 <= lo < 2^28: the low four digits come from lo (leaving a carry of 0 or
// 1), the high four from hi + carry, all in 32-bit arithmetic.
__host__ __device__ __forceinline__ void to_digits(long long X, int* d) {
  int lo = int(X & 0x0FFFFFFFLL);
  int hi = int(X >> 28);
#pragma unroll
  for (int s = kDigits - 1; s >= 4; --s) {
    const int r = ((lo + 64) & 127) - 64;
    d[s] = r;
    lo = (lo - r) >> 7;
  }
  hi += lo;
#pragma unroll
  for (int s = 3; s >= 0; --s) {
    const int r = ((hi + 64) & 127) - 64;
    d[s] = r;
    hi = (hi - r) >> 7;
  }
}

#ifdef __CUDACC__
// bf16 bit patterns of two small integers (|v| < 2^22) packed into one word
// (a in the low half): 1.5 * 2^23 + v is exact in FP32, subtracting
// 1.5 * 2^23 leaves v as an FP32 value whose upper 16 bits are its bf16
// pattern (v has at most 8 significant bits)
__device__ __forceinline__ uint32_t bf16x2_of_ints(int a, int b) {
  const float fa = __int_as_float(0x4B400000 + a) - 12582912.0f;
  const float fb = __int_as_float(0x4B400000 + b) - 12582912.0f;
  return __byte_perm(__float_as_uint(fa), __float_as_uint(fb), 0x7632);
}
#endif

// bf16 bit pattern of a small integer (|v| <= 256: exact)
__host__ __device__ __forceinline__ uint16_t bf16_bits_of_int(int v) {
  const float f = float(v);
#ifdef __CUDA_ARCH__
  return uint16_t(uint32_t(__float_as_uint(f)) >> 16);
#else
  uint32_t u;
  std::memcpy(&u, &f, sizeof u);
  return uint16_t(u >> 16);
#endif
}

#ifdef __CUDACC__

// element-wise sum of two bf16 pairs (exact for the small integers used here)
__device__ __forceinline__ uint32_t bsum(uint32_t a, uint32_t b) {
  __nv_bfloat162 x = *reinterpret_cast<__nv_bfloat162*>(&a), y = *reinterpret_cast<__nv_bfloat162*>(&b);
  __nv_bfloat162 r = __hadd2(x, y);
  return *reinterpret_cast<uint32_t*>(&r);
}

__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// 16-byte asynchronous copy global -> shared; with valid == false nothing is
// read and the destination is zero-filled
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool valid) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  const int nbytes = valid ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(nbytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <int PA, int PB>
struct Shape {
  static constexpr int NC = (PA == 2 && PB == 2) ? 3 : ((PA == 2 || PB == 2) ? 2 : 1);  // products per pair
  static constexpr int PAX = (PA == 2 && PB == 2) ? 3 : PA;  // A fragment planes incl. the r + i sum
  static constexpr int PBX = (PA == 2 && PB == 2) ? 3 : PB;
  static constexpr int kStageElems = kDigits * (PA + PB) * kTile * kLd;
  static constexpr size_t kSmemBytes = 2 * sizeof(__nv_bfloat16) * size_t(kStageElems);
};

// integer accumulators of one thread: outputs q = 0..3 of its m16n8 fragment
struct Acc {
  long long hr[4], lr[4], hi[4], li[4];
};

// Copies K range [kc, kc + kKc) of a 32-row A tile and a 32-column B tile
// (all digit planes) into one stage.  Digit plane dp of row r, element k, sits
// at X + dp * plane + r * ld + k; k >= klen is zero-filled.
template <int PA, int PB>
__device__ __forceinline__ void stage_load(const __nv_bfloat16* A, size_t a_plane, int a_ld, const __nv_bfloat16* B,
                                           size_t b_plane, int b_ld, int kc, int klen, __nv_bfloat16* st) {
  __nv_bfloat16* sA = st;
  __nv_bfloat16* sB = st + kDigits * PA * kTile * kLd;
  constexpr int kVec = kKc / 8;  // 16-byte vectors per staged row
  for (int v = threadIdx.x; v < kDigits * PA * kTile * kVec; v += kThreads) {
    const int kv = v % kVec, r = (v / kVec) % kTile, dp = v / (kVec * kTile);
    const int k = kc + kv * 8;
    const bool ok = k < klen;
    cp_async16(sA + (dp * kTile + r) * kLd + kv * 8, ok ? A + dp * a_plane + size_t(r) * a_ld + k : A, ok);
  }
  for (int v = threadIdx.x; v < kDigits * PB * kTile * kVec; v += kThreads) {
    const int kv = v % kVec, r = (v / kVec) % kTile, dp = v / (kVec * kTile);
    const int k = kc + kv * 8;
    const bool ok = k < klen;
    cp_async16(sB + (dp * kTile + r) * kLd + kv * 8, ok ? B + dp * b_plane + size_t(r) * b_ld + k : B, ok);
  }
}

// 32 x 32 output tile over K = [0, klen) (klen a multiple of 16), two-stage
// cp.async pipeline; smem holds Shape<PA, PB>::kSmemBytes.  Warp w owns rows
// (w / 4) * 16 .. + 16 and columns (w % 4) * 8 .. + 8 of the tile; output q of
// a thread is row gq + 8 (q / 2), column 2 tq + q % 2 of that sub-tile.
template <int PA, int PB>
__device__ __forceinline__ void mainloop(const __nv_bfloat16* A, size_t a_plane, int a_ld, const __nv_bfloat16* B,
                                         size_t b_plane, int b_ld, int klen, __nv_bfloat16* smem, Acc& o) {
  using S = Shape<PA, PB>;
  constexpr int NC = S::NC, PAX = S::PAX, PBX = S::PBX;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gq = lane >> 2, tq = lane & 3;
  const int wm = (warp >> 2) * 16, wn = (warp & 3) * 8;
#pragma unroll
  for (int q = 0; q < 4; ++q) o.hr[q] = o.lr[q] = o.hi[q] = o.li[q] = 0;
  float acc[kKeep + 1][NC][4];
#pragma unroll
  for (int gg = 0; gg <= kKeep; ++gg)
#pragma unroll
    for (int c = 0; c < NC; ++c)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[gg][c][q] = 0.f;
  const int nch = (klen + kKc - 1) / kKc;
  if (nch > 0) {
    stage_load<PA, PB>(A, a_plane, a_ld, B, b_plane, b_ld, 0, klen, smem);
    cp_async_commit();
  }
  for (int ch = 0; ch < nch; ++ch) {
    const __nv_bfloat16* cur = smem + (ch & 1) * S::kStageElems;
    if (ch + 1 < nch) {
      stage_load<PA, PB>(A, a_plane, a_ld, B, b_plane, b_ld, (ch + 1) * kKc, klen,
                         smem + ((ch + 1) & 1) * S::kStageElems);
      cp_async_commit();
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const __nv_bfloat16* sA = cur;
    const __nv_bfloat16* sB = cur + kDigits * PA * kTile * kLd;
    const int kvalid = min(kKc, klen - ch * kKc);
#pragma unroll
    for (int ks = 0; ks < kKc; ks += 16) {
      if (ks >= kvalid) break;
      uint32_t bf[kDigits][PBX][2];
#pragma unroll
      for (int t = 0; t < kDigits; ++t) {
#pragma unroll
        for (int pb = 0; pb < PB; ++pb) {
          const __nv_bfloat16* B0 = sB + ((t * PB + pb) * kTile + wn + gq) * kLd + ks + 2 * tq;
          bf[t][pb][0] = *reinterpret_cast<const uint32_t*>(B0);
          bf[t][pb][1] = *reinterpret_cast<const uint32_t*>(B0 + 8);
        }
        if (PBX == 3) {
          bf[t][PBX - 1][0] = bsum(bf[t][0][0], bf[t][PB - 1][0]);
          bf[t][PBX - 1][1] = bsum(bf[t][0][1], bf[t][PB - 1][1]);
        }
      }
#pragma unroll
      for (int s = 0; s < kDigits; ++s) {
        uint32_t af[PAX][4];
#pragma unroll
        for (int pa = 0; pa < PA; ++pa) {
          const __nv_bfloat16* A0 = sA + ((s * PA + pa) * kTile + wm + gq) * kLd + ks + 2 * tq;
          const __nv_bfloat16* A8 = A0 + 8 * kLd;
          af[pa][0] = *reinterpret_cast<const uint32_t*>(A0);
          af[pa][1] = *reinterpret_cast<const uint32_t*>(A8);
          af[pa][2] = *reinterpret_cast<const uint32_t*>(A0 + 8);
          af[pa][3] = *reinterpret_cast<const uint32_t*>(A8 + 8);
        }
        if (PAX == 3) {
#pragma unroll
          for (int v = 0; v < 4; ++v) af[PAX - 1][v] = bsum(af[0][v], af[PA - 1][v]);
        }
#pragma unroll
        for (int t = 0; t <= kKeep - s; ++t) {
          const int gg = s + t;
          if (PA == 2 && PB == 2) {
            mma16816(acc[gg][0], af[0], bf[t][0]);
            mma16816(acc[gg][1], af[1], bf[t][1]);
            mma16816(acc[gg][2], af[PAX - 1], bf[t][PBX - 1]);
          } else if (PA == 2) {
            mma16816(acc[gg][0], af[0], bf[t][0]);
            mma16816(acc[gg][1], af[1], bf[t][0]);
          } else if (PB == 2) {
            mma16816(acc[gg][0], af[0], bf[t][0]);
            mma16816(acc[gg][1], af[0], bf[t][1]);
          } else {
            mma16816(acc[gg][0], af[0], bf[t][0]);
          }
        }
      }
    }
    if (((ch + 1) * kKc) % kFoldK == 0 || ch + 1 == nch) {
      // the real and imaginary group sums are exact FP32 integers below 2^22
      // (rr - ii and ss - rr - ii included): convert, weight and fold
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        int pr[kKeep + 1], pi[kKeep + 1];
#pragma unroll
        for (int gg = 0; gg <= kKeep; ++gg) {
          float re, im = 0.f;
          if (PA == 2 && PB == 2) {
            re = acc[gg][0][q] - acc[gg][1][q];
            im = acc[gg][2][q] - (acc[gg][0][q] + acc[gg][1][q]);
          } else if (PA == 2 || PB == 2) {
            re = acc[gg][0][q];
            im = acc[gg][1][q];
          } else {
            re = acc[gg][0][q];
          }
          pr[gg] = __float2int_rn(re);
          pi[gg] = __float2int_rn(im);
#pragma unroll
          for (int c = 0; c < NC; ++c) acc[gg][c][q] = 0.f;
        }
        o.hr[q] += ((long long)(pr[0] * 128 + pr[1]) << 14) + (pr[2] * 128 + pr[3]);
        o.lr[q] += ((long long)(pr[4] * 128 + pr[5]) << 14) + (pr[6] * 128 + pr[7]);
        if (NC > 1) {
          o.hi[q] += ((long long)(pi[0] * 128 + pi[1]) << 14) + (pi[2] * 128 + pi[3]);
          o.li[q] += ((long long)(pi[4] * 128 + pi[5]) << 14) + (pi[6] * 128 + pi[7]);
        }
      }
    }
    __syncthreads();
  }
}

// 2^e as a double: built from its bits in the normal range, ldexp outside
__device__ __forceinline__ double pow2(int e) {
  return (e >= -1022 && e <= 1023) ? __longlong_as_double((long long)(e + 1023) << 52) : ldexp(1.0, e);
}

// value of output q, before the exponent scale 2^(ea + eb - 57)
__device__ __forceinline__ double2 acc_value(const Acc& o, int q) {
  return make_double2(fma(double(o.hr[q]), 0x1p28, double(o.lr[q])), fma(double(o.hi[q]), 0x1p28, double(o.li[q])));
}

#endif  // __CUDACC__

}  // namespace oz
}  // namespace tvap
