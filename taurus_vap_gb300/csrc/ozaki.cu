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
//     with K split in chunks of 128 a group of digit pairs of equal weight
//     (s + t = g, at most 8 pairs) stays below 2^22, and the complex
//     combination rr - ii below 2^23, so every FP32 group sum is exact;
//   * pairs with s + t <= 7 are kept (the dropped ones weigh < 2^-56 of the
//     leading term); each group sum is folded into an FP64 accumulator with its
//     weight 2^(7 (14 - g)), and the result is scaled by 2^(e_i + f_j - 106).
//
// The FP64 pipe then does ~4 operations per output and group and K-chunk
// instead of 3-4 per multiply-add.  Complex operands carry real and imaginary
// digit planes with a shared exponent per row/column; conjugation flips the
// imaginary plane.

#include <cuda_bf16.h>

#include <mutex>

#include "tvap_internal.cuh"

namespace tvap {

namespace {

constexpr int kDigits = 8;
constexpr int kKeep = 7;     // keep digit pairs with s + t <= kKeep
constexpr int kChunk = 128;  // K chunk: FP32 group sums stay exact

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

__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// one warp computes a 16 x 16 output tile (two m16n8 sub-tiles); a CTA holds
// 4 warps (32 x 32).  PA / PB: 1 real, 2 complex planes.
template <int PA, int PB>
__global__ void __launch_bounds__(128)
    ozaki_mma_kernel(int M, int N, int K, int mpad, int npad, int kpad, const __nv_bfloat16* __restrict__ As,
                     const int* __restrict__ ea, const __nv_bfloat16* __restrict__ Bs, const int* __restrict__ eb,
                     GemmArgs g) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gq = lane >> 2, tq = lane & 3;
  const int b = blockIdx.z;
  const int m0 = blockIdx.y * 32 + (warp >> 1) * 16;
  const int n0 = blockIdx.x * 32 + (warp & 1) * 16;
  if (m0 >= mpad || n0 >= npad) return;
  constexpr int CRE = (PA == 2 && PB == 2) ? 2 : 1;  // accumulators per output component
  const size_t aplane = size_t(mpad) * kpad, bplane = size_t(npad) * kpad;
  // FP64 accumulators: [sub-tile][element 0..3] for re and im
  double cre[2][4], cim[2][4];
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int q = 0; q < 4; ++q) cre[u][q] = cim[u][q] = 0.0;
  for (int kc = 0; kc < kpad; kc += kChunk) {
    const int kend = min(kpad, kc + kChunk);
    for (int grp = 0; grp <= kKeep; ++grp) {
      // FP32 group sums: [combo][sub-tile][4]
      float acc[2 * CRE][2][4];
#pragma unroll
      for (int c = 0; c < 2 * CRE; ++c)
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[c][u][q] = 0.f;
      for (int s = max(0, grp - (kDigits - 1)); s <= min(grp, kDigits - 1); ++s) {
        const int t = grp - s;
        const __nv_bfloat16* Ab = As + (size_t(b) * kDigits + s) * PA * aplane;
        const __nv_bfloat16* Bb = Bs + (size_t(b) * kDigits + t) * PB * bplane;
        for (int ks = kc; ks < kend; ks += 16) {
          uint32_t af[PA][4], bf[PB][2][2];
#pragma unroll
          for (int pa = 0; pa < PA; ++pa) {
            const __nv_bfloat16* A0 = Ab + pa * aplane + size_t(m0 + gq) * kpad + ks + 2 * tq;
            const __nv_bfloat16* A8 = A0 + size_t(8) * kpad;
            af[pa][0] = *reinterpret_cast<const uint32_t*>(A0);
            af[pa][1] = *reinterpret_cast<const uint32_t*>(A8);
            af[pa][2] = *reinterpret_cast<const uint32_t*>(A0 + 8);
            af[pa][3] = *reinterpret_cast<const uint32_t*>(A8 + 8);
          }
#pragma unroll
          for (int pb = 0; pb < PB; ++pb)
#pragma unroll
            for (int u = 0; u < 2; ++u) {
              const __nv_bfloat16* B0 = Bb + pb * bplane + size_t(n0 + u * 8 + gq) * kpad + ks + 2 * tq;
              bf[pb][u][0] = *reinterpret_cast<const uint32_t*>(B0);
              bf[pb][u][1] = *reinterpret_cast<const uint32_t*>(B0 + 8);
            }
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            if (PA == 2 && PB == 2) {
              mma16816(acc[0][u], af[0], bf[0][u]);  // rr
              mma16816(acc[1][u], af[1], bf[1][u]);  // ii
              mma16816(acc[2][u], af[0], bf[1][u]);  // ri
              mma16816(acc[3][u], af[1], bf[0][u]);  // ir
            } else if (PA == 2) {
              mma16816(acc[0][u], af[0], bf[0][u]);  // re
              mma16816(acc[1][u], af[1], bf[0][u]);  // im
            } else if (PB == 2) {
              mma16816(acc[0][u], af[0], bf[0][u]);
              mma16816(acc[1][u], af[0], bf[1][u]);
            } else {
              mma16816(acc[0][u], af[0], bf[0][u]);
            }
          }
        }
      }
      const double w = ldexp(1.0, 7 * (2 * (kDigits - 1) - grp));
#pragma unroll
      for (int u = 0; u < 2; ++u)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          if (PA == 2 && PB == 2) {
            cre[u][q] = fma(double(acc[0][u][q] - acc[1][u][q]), w, cre[u][q]);
            cim[u][q] = fma(double(acc[2][u][q] + acc[3][u][q]), w, cim[u][q]);
          } else if (PA == 2 || PB == 2) {
            cre[u][q] = fma(double(acc[0][u][q]), w, cre[u][q]);
            cim[u][q] = fma(double(acc[1][u][q]), w, cim[u][q]);
          } else {
            cre[u][q] = fma(double(acc[0][u][q]), w, cre[u][q]);
          }
        }
    }
  }
  // epilogue: scale by 2^(ea + eb - 106), alpha/beta, store
  double2 alpha = g.alpha;
  if (g.alpha_vec) alpha = cmul(alpha, g.alpha_vec[b]);
  const bool cplx_out = !g.c_real;
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = m0 + gq + ((q & 2) ? 8 : 0);
      const int j = n0 + u * 8 + 2 * tq + (q & 1);
      if (i >= M || j >= N) continue;
      const int sc = ea[size_t(b) * mpad + i] + eb[size_t(b) * npad + j] - 106;
      const double vr = ldexp(cre[u][q], sc), vi = ldexp(cim[u][q], sc);
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

// Slice scratch, one per stream (GEMMs on different streams run concurrently);
// grown on demand and kept for the life of the process.
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
  dim3 grid(npad / 32, mpad / 32, g.batch);
  if (PA == 2 && PB == 2)
    ozaki_mma_kernel<2, 2><<<grid, 128, 0, s>>>(g.M, g.N, g.K, mpad, npad, kpad, As, ea, Bs, eb, g);
  else if (PA == 2)
    ozaki_mma_kernel<2, 1><<<grid, 128, 0, s>>>(g.M, g.N, g.K, mpad, npad, kpad, As, ea, Bs, eb, g);
  else if (PB == 2)
    ozaki_mma_kernel<1, 2><<<grid, 128, 0, s>>>(g.M, g.N, g.K, mpad, npad, kpad, As, ea, Bs, eb, g);
  else
    ozaki_mma_kernel<1, 1><<<grid, 128, 0, s>>>(g.M, g.N, g.K, mpad, npad, kpad, As, ea, Bs, eb, g);
  TVAP_CUDA(cudaGetLastError());
  return TVAP_OK;
}

}  // namespace tvap
