// FP64 GEMM emulated on the bf16 tensor cores (Ozaki splitting).
//
// GB300's FP64 pipe delivers ~1.2 TFLOP/s while the bf16 tensor path
// (mma.sync) delivers ~600 TFLOP/s.  An FP64 product C = A B is rebuilt
// exactly from integer pieces:
//
//   * every row i of op(A) (column j of op(B)) is scaled by a shared power of
//     two 2^(e_i - 53) so that each entry is an integer |X| < 2^54 (the
//     53-bit mantissa aligned to the row maximum; bits more than 54 binary
//     orders below the row maximum are rounded away);
//   * X is written in balanced base 2^7 with 8 digits d_0 .. d_7 in [-64, 63]
//     (d_0 most significant), using integer operations only;
//   * every digit is exactly representable in bf16, every digit product
//     (|d d'| <= 2^12) exactly in FP32, and the tensor core sums them in FP32;
//     with K split in chunks of 64 a group of digit pairs of equal weight
//     (s + t = g, at most 8 pairs) stays below 2^21, and the complex
//     combination rr - ii below 2^22, so every FP32 group sum is exact;
//   * pairs with s + t <= 7 are kept (the dropped ones weigh < 2^-56 of the
//     leading term); the group sums of each chunk are converted to integers
//     and folded, with their weights 2^(7 (14 - g)), into two 64-bit integer
//     accumulators per output, which are converted to FP64 once at the end and
//     scaled by 2^(e_i + f_j - 106).
//
// The FP64 pipe then does a few operations per output instead of 3-4 per
// multiply-add.  Complex operands carry real and imaginary digit planes with a
// shared exponent per row/column; conjugation flips the imaginary plane; a
// complex x complex product takes three real products per digit pair
// (rr, ii and (r + i)(r + i); digit sums |d_r + d_i| <= 128 stay exact in
// bf16 and their products, summed over a chunk and a group, below 2^23).

#include <cuda_bf16.h>

#include <mutex>

#include "tvap_internal.cuh"

namespace tvap {

namespace {

constexpr int kDigits = 8;
constexpr int kKeep = 7;     // keep digit pairs with s + t <= kKeep

__device__ __forceinline__ int dexp(double x) {
  // unbiased exponent of a finite non-zero double (subnormals treated as 0)
  const long long b = __double_as_longlong(x);
  const int e = int((b >> 52) & 0x7ff);
  return e == 0 ? -2000 : e - 1023;
}

// integer X with x = X 2^(emax - 53), |X| < 2^54 (8 balanced 7-bit digits
// represent |X| < 0.99 2^55)
__device__ __forceinline__ long long to_fixed(double x, int emax) {
  const long long b = __double_as_longlong(x);
  const int eb = int((b >> 52) & 0x7ff);
  if (eb == 0) return 0;  // zero or subnormal
  long long m = (b & ((1LL << 52) - 1)) | (1LL << 52);
  const int sh = (eb - 1023) - emax + 1;  // <= 1
  if (sh >= 0) {
    m <<= sh;
  } else if (sh > -60) {
    m = (m + (1LL << (-sh - 1))) >> (-sh);  // round half up
  } else {
    m = 0;
  }
  return (b < 0) ? -m : m;
}

__device__ __forceinline__ void to_digits(long long X, int* d) {
#pragma unroll
  for (int s = kDigits - 1; s >= 0; --s) {
    const int r = int(((X + 64) & 127)) - 64;
    d[s] = r;
    X = (X - r) >> 7;
  }
}

// Slices of a strided batched operand.  rows = the output dimension of the
// operand (M for A, N for B), K the contraction dimension.  Element (r, k) of
// batch b is at p[r * sr + k * sk + b * bs].  Output layout:
//   sl[((b * kDigits + s) * parts + part) * rows_pad * kpad + r * kpad + k]  (bf16)
//   ex[b * rows_pad + r]
template <bool CPLX>
__global__ void slice_kernel(int rows, int K, int rows_pad, int kpad, const void* __restrict__ p, long long sr,
                             long long sk, long long bs, bool conj, __nv_bfloat16* __restrict__ sl,
                             int* __restrict__ ex) {
  const int lane = threadIdx.x & 31;
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int b = blockIdx.y;
  if (r >= rows_pad) return;
  constexpr int parts = CPLX ? 2 : 1;
  auto val = [&](int k, double& re, double& im) {
    re = 0.0;
    im = 0.0;
    if (r < rows && k < K) {
      const long long off = r * sr + k * sk + b * bs;
      if (CPLX) {
        const double2 v = static_cast<const double2*>(p)[off];
        re = v.x;
        im = conj ? -v.y : v.y;
      } else {
        re = static_cast<const double*>(p)[off];
      }
    }
  };
  int emax = -2000;
  for (int k = lane; k < K; k += 32) {
    double re, im;
    val(k, re, im);
    if (re != 0.0) emax = max(emax, dexp(re));
    if (CPLX && im != 0.0) emax = max(emax, dexp(im));
  }
  for (int off = 16; off > 0; off >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, off));
  if (emax == -2000) emax = 0;
  if (lane == 0) ex[size_t(b) * rows_pad + r] = emax;
  const size_t plane = size_t(rows_pad) * kpad;
  for (int k = lane; k < kpad; k += 32) {
    double re, im;
    val(k, re, im);
    int dr[kDigits], di[kDigits];
    to_digits(to_fixed(re, emax), dr);
    if (CPLX) to_digits(to_fixed(im, emax), di);
#pragma unroll
    for (int s = 0; s < kDigits; ++s) {
      const size_t base = ((size_t(b) * kDigits + s) * parts) * plane + size_t(r) * kpad + k;
      sl[base] = __float2bfloat16_rn(float(dr[s]));
      if (CPLX) sl[base + plane] = __float2bfloat16_rn(float(di[s]));
    }
  }
}

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

// A CTA computes a 32 x 32 output tile with 8 warps, each warp one m16n8
// sub-tile.  K is walked in chunks of 64: the chunk's 8 digit planes of A
// (32 rows) and B (32 columns) are staged in shared memory once, and every
// digit pair of the chunk goes to the tensor cores with the FP32 sums of all
// 8 weight groups held in registers; at the end of each chunk the group sums
// (exact integers) are folded into FP64.  PA / PB: 1 real, 2 complex planes.
constexpr int kKc = 64;        // K chunk staged in shared memory
constexpr int kRowPad = 8;     // bf16 padding per staged row (conflict-free fragment loads)
constexpr int kLd = kKc + kRowPad;

template <int PA, int PB>
__global__ void __launch_bounds__(256, 1)
    ozaki_mma_kernel(int M, int N, int K, int mpad, int npad, int kpad, const __nv_bfloat16* __restrict__ As,
                     const int* __restrict__ ea, const __nv_bfloat16* __restrict__ Bs, const int* __restrict__ eb,
                     GemmArgs g) {
  extern __shared__ __align__(16) __nv_bfloat16 sm[];
  __nv_bfloat16* sA = sm;                                // [kDigits][PA][32][kLd]
  __nv_bfloat16* sB = sm + size_t(kDigits) * PA * 32 * kLd;  // [kDigits][PB][32][kLd]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int gq = lane >> 2, tq = lane & 3;
  const int b = blockIdx.z;
  const int mt0 = blockIdx.y * 32, nt0 = blockIdx.x * 32;
  const int wm = (warp >> 2) * 16, wn = (warp & 3) * 8;  // warp sub-tile inside the CTA tile
  // products per digit pair: 3 (3M) for complex x complex, 2 mixed, 1 real
  constexpr int NC = (PA == 2 && PB == 2) ? 3 : ((PA == 2 || PB == 2) ? 2 : 1);
  constexpr int PAX = (PA == 2 && PB == 2) ? 3 : PA;  // fragment planes incl. the r + i sum
  constexpr int PBX = (PA == 2 && PB == 2) ? 3 : PB;
  const size_t aplane = size_t(mpad) * kpad, bplane = size_t(npad) * kpad;
  long long hre[4], lre[4], him[4], lim[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) hre[q] = lre[q] = him[q] = lim[q] = 0;
  for (int kc = 0; kc < kpad; kc += kKc) {
    // ---- stage the chunk: 16-byte vectors, zero beyond kpad
    {
      const int vecs_per_row = kKc / 8;
      const int totA = kDigits * PA * 32 * vecs_per_row;
      for (int v = tid; v < totA; v += blockDim.x) {
        const int kv = v % vecs_per_row, r = (v / vecs_per_row) % 32, dp = v / (vecs_per_row * 32);
        const int k = kc + kv * 8;
        uint4 val = make_uint4(0, 0, 0, 0);
        if (k < kpad) {
          const int dgt = dp / PA, part = dp % PA;
          val = *reinterpret_cast<const uint4*>(As + ((size_t(b) * kDigits + dgt) * PA + part) * aplane +
                                                size_t(mt0 + r) * kpad + k);
        }
        *reinterpret_cast<uint4*>(sA + (size_t(dp) * 32 + r) * kLd + kv * 8) = val;
      }
      const int totB = kDigits * PB * 32 * vecs_per_row;
      for (int v = tid; v < totB; v += blockDim.x) {
        const int kv = v % vecs_per_row, r = (v / vecs_per_row) % 32, dp = v / (vecs_per_row * 32);
        const int k = kc + kv * 8;
        uint4 val = make_uint4(0, 0, 0, 0);
        if (k < kpad) {
          const int dgt = dp / PB, part = dp % PB;
          val = *reinterpret_cast<const uint4*>(Bs + ((size_t(b) * kDigits + dgt) * PB + part) * bplane +
                                                size_t(nt0 + r) * kpad + k);
        }
        *reinterpret_cast<uint4*>(sB + (size_t(dp) * 32 + r) * kLd + kv * 8) = val;
      }
    }
    __syncthreads();
    float acc[kKeep + 1][NC][4];
#pragma unroll
    for (int gg = 0; gg <= kKeep; ++gg)
#pragma unroll
      for (int c = 0; c < NC; ++c)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[gg][c][q] = 0.f;
    const int kvalid = min(kKc, kpad - kc);
    for (int ks = 0; ks < kvalid; ks += 16) {
      // B fragments of all digits (and, for complex x complex, the digit sums
      // r + i, exact in bf16: |d_r + d_i| <= 128)
      uint32_t bf[kDigits][PBX][2];
#pragma unroll
      for (int t = 0; t < kDigits; ++t) {
#pragma unroll
        for (int pb = 0; pb < PB; ++pb) {
          const __nv_bfloat16* B0 = sB + (size_t(t * PB + pb) * 32 + wn + gq) * kLd + ks + 2 * tq;
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
          const __nv_bfloat16* A0 = sA + (size_t(s * PA + pa) * 32 + wm + gq) * kLd + ks + 2 * tq;
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
            // 3M: rr, ii and (r + i)(r + i)
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
    // ---- fold the exact group sums of this chunk into the integer
    // accumulators: the real and imaginary group sums are exact FP32
    // integers below 2^22 (rr - ii and ss - rr - ii included), so they
    // convert exactly; groups 0-3 go to hi, 4-7 to lo (weights 2^(7 (3 - g))
    // and 2^(7 (7 - g))).
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
      }
      hre[q] += ((long long)(pr[0] * 128 + pr[1]) << 14) + (pr[2] * 128 + pr[3]);
      lre[q] += ((long long)(pr[4] * 128 + pr[5]) << 14) + (pr[6] * 128 + pr[7]);
      if (NC > 1) {
        him[q] += ((long long)(pi[0] * 128 + pi[1]) << 14) + (pi[2] * 128 + pi[3]);
        lim[q] += ((long long)(pi[4] * 128 + pi[5]) << 14) + (pi[6] * 128 + pi[7]);
      }
    }
    __syncthreads();
  }
  double cre[4], cim[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    cre[q] = fma(double(hre[q]), 0x1p28, double(lre[q]));
    cim[q] = fma(double(him[q]), 0x1p28, double(lim[q]));
  }
  // epilogue: scale by 2^(ea + eb - 106), alpha/beta, store
  double2 alpha = g.alpha;
  if (g.alpha_vec) alpha = cmul(alpha, g.alpha_vec[b]);
  const bool cplx_out = !g.c_real;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = mt0 + wm + gq + ((q & 2) ? 8 : 0);
    const int j = nt0 + wn + 2 * tq + (q & 1);
    if (i >= M || j >= N) continue;
    const int sc = ea[size_t(b) * mpad + i] + eb[size_t(b) * npad + j] - 106 + 49;
    const double vr = ldexp(cre[q], sc), vi = ldexp(cim[q], sc);
    const long long idx = i * g.crs + j * g.ccs + b * g.cbs;
    if (cplx_out) {
      double2* C = static_cast<double2*>(g.C);
      double2 v = cmul(alpha, make_double2(vr, vi));
      if (g.beta.x != 0.0 || g.beta.y != 0.0) v = cadd(v, cmul(g.beta, C[idx]));
      C[idx] = v;
    } else {
      double* C = static_cast<double*>(g.C);
      double v = (cmul(alpha, make_double2(vr, vi))).x;
      if (g.beta.x != 0.0) v = fma(g.beta.x, C[idx], v);
      C[idx] = v;
    }
  }
}

template <int PA, int PB>
int launch_ozaki_mma(int M, int N, int K, int mpad, int npad, int kpad, const __nv_bfloat16* As, const int* ea,
                     const __nv_bfloat16* Bs, const int* eb, const GemmArgs& g, cudaStream_t s) {
  const size_t shm = sizeof(__nv_bfloat16) * size_t(kDigits) * (PA + PB) * 32 * kLd;
  static bool attr = false;
  if (!attr) {
    TVAP_CUDA(cudaFuncSetAttribute(ozaki_mma_kernel<PA, PB>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(shm)));
    attr = true;
  }
  dim3 grid(npad / 32, mpad / 32, g.batch);
  ozaki_mma_kernel<PA, PB><<<grid, 256, shm, s>>>(M, N, K, mpad, npad, kpad, As, ea, Bs, eb, g);
  TVAP_CUDA(cudaGetLastError());
  return TVAP_OK;
}

struct OzScratch {
  cudaStream_t stream = nullptr;
  __nv_bfloat16* buf = nullptr;
  size_t bytes = 0;
  int* ex = nullptr;
  size_t ex_count = 0;
};
constexpr int kMaxScratch = 16;
OzScratch g_oz[kMaxScratch];
std::mutex g_oz_mutex;

int oz_reserve(cudaStream_t s, size_t bytes, size_t ex_count, OzScratch** out) {
  std::lock_guard<std::mutex> lock(g_oz_mutex);
  OzScratch* sc = nullptr;
  for (auto& e : g_oz)
    if (e.buf && e.stream == s) sc = &e;
  if (!sc)
    for (auto& e : g_oz)
      if (!e.buf) {
        sc = &e;
        sc->stream = s;
        break;
      }
  if (!sc) {
    set_last_error("too many streams use the emulated GEMM", __FILE__, __LINE__);
    return TVAP_ERR_ARG;
  }
  if (bytes > sc->bytes) {
    if (sc->buf) {
      cudaStreamSynchronize(s);
      cudaFree(sc->buf);
    }
    sc->buf = nullptr;
    TVAP_CUDA(cudaMalloc(&sc->buf, bytes));
    sc->bytes = bytes;
  }
  if (ex_count > sc->ex_count) {
    if (sc->ex) {
      cudaStreamSynchronize(s);
      cudaFree(sc->ex);
    }
    sc->ex = nullptr;
    TVAP_CUDA(cudaMalloc(&sc->ex, ex_count * sizeof(int)));
    sc->ex_count = ex_count;
  }
  *out = sc;
  return TVAP_OK;
}

}  // namespace

// Frees the slice scratch of a stream (called when a context destroys or
// replaces the stream).
void oz_release(cudaStream_t s) {
  std::lock_guard<std::mutex> lock(g_oz_mutex);
  for (auto& e : g_oz)
    if (e.buf && e.stream == s) {
      cudaStreamSynchronize(s);
      cudaFree(e.buf);
      cudaFree(e.ex);
      e = OzScratch();
    }
}

// Returns TVAP_OK after launching, or TVAP_ERR_ARG when the shape is not
// supported (the caller then uses the FP64 pipe).
int gemm_ozaki(const GemmArgs& g, cudaStream_t s) {
  if (g.M <= 0 || g.N <= 0 || g.K <= 0 || g.batch <= 0) return TVAP_OK;
  const int PA = g.a_real ? 1 : 2, PB = g.b_real ? 1 : 2;
  const int mpad = (g.M + 31) / 32 * 32, npad = (g.N + 31) / 32 * 32, kpad = (g.K + 15) / 16 * 16;
  const size_t asz = size_t(g.batch) * kDigits * PA * mpad * kpad;
  const size_t bsz = size_t(g.batch) * kDigits * PB * npad * kpad;
  int rc;
  OzScratch* sc = nullptr;
  if ((rc = oz_reserve(s, sizeof(__nv_bfloat16) * (asz + bsz), size_t(g.batch) * (mpad + npad), &sc))) return rc;
  __nv_bfloat16* As = sc->buf;
  __nv_bfloat16* Bs = sc->buf + asz;
  int* ea = sc->ex;
  int* eb = sc->ex + size_t(g.batch) * mpad;
  // A rows: element (i, k) at A.p[i rs + k cs]; B columns: element (j, k) = B(k, j) at B.p[k rs + j cs]
  {
    dim3 grid((mpad + 7) / 8, g.batch);
    if (PA == 2)
      slice_kernel<true><<<grid, 256, 0, s>>>(g.M, g.K, mpad, kpad, g.A.p, g.A.rs, g.A.cs, g.A.bs, g.conj_a, As, ea);
    else
      slice_kernel<false><<<grid, 256, 0, s>>>(g.M, g.K, mpad, kpad, g.A.p, g.A.rs, g.A.cs, g.A.bs, false, As, ea);
  }
  {
    dim3 grid((npad + 7) / 8, g.batch);
    if (PB == 2)
      slice_kernel<true><<<grid, 256, 0, s>>>(g.N, g.K, npad, kpad, g.B.p, g.B.cs, g.B.rs, g.B.bs, g.conj_b, Bs, eb);
    else
      slice_kernel<false><<<grid, 256, 0, s>>>(g.N, g.K, npad, kpad, g.B.p, g.B.cs, g.B.rs, g.B.bs, false, Bs, eb);
  }
  if (PA == 2 && PB == 2) return launch_ozaki_mma<2, 2>(g.M, g.N, g.K, mpad, npad, kpad, As, ea, Bs, eb, g, s);
  if (PA == 2) return launch_ozaki_mma<2, 1>(g.M, g.N, g.K, mpad, npad, kpad, As, ea, Bs, eb, g, s);
  if (PB == 2) return launch_ozaki_mma<1, 2>(g.M, g.N, g.K, mpad, npad, kpad, As, ea, Bs, eb, g, s);
  return launch_ozaki_mma<1, 1>(g.M, g.N, g.K, mpad, npad, kpad, As, ea, Bs, eb, g, s);
}

}  // namespace tvap
