// FP64 GEMM emulated on the bf16 tensor cores (integer splitting of the
// operands, exact FP32 group sums, integer folding; the scheme is described in
// ozaki_core.cuh).
//
// GB300's FP64 pipe delivers ~1.2 TFLOP/s while the bf16 tensor path
// (mma.sync) delivers ~600 TFLOP/s.  The product C = op(A) op(B) is rebuilt
// from the digit planes of its operands: a slicing pass writes the planes of
// A (per row of op(A)) and B (per column of op(B)) with one shared exponent
// each, then a 32 x 32-tile kernel runs the digit-pair products and forms
// alpha C + beta C_old in FP64.  Conjugation flips the imaginary plane.

#include <cuda_bf16.h>

#include <mutex>

#include "ozaki_core.cuh"
#include "ozaki_tc.cuh"
#include "tvap_internal.cuh"

namespace tvap {

namespace {

using oz::kDigits;

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
  int emax = oz::kExpZero;
  for (int k = lane; k < K; k += 32) {
    double re, im;
    val(k, re, im);
    if (re != 0.0) emax = max(emax, oz::dexp(re));
    if (CPLX && im != 0.0) emax = max(emax, oz::dexp(im));
  }
  for (int off = 16; off > 0; off >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, off));
  if (emax == oz::kExpZero) emax = 0;
  if (lane == 0) ex[size_t(b) * rows_pad + r] = emax;
  const size_t plane = size_t(rows_pad) * kpad;
  for (int k = lane; k < kpad; k += 32) {
    double re, im;
    val(k, re, im);
    int dr[kDigits], di[kDigits];
    oz::to_digits(oz::to_fixed(re, emax), dr);
    if (CPLX) oz::to_digits(oz::to_fixed(im, emax), di);
#pragma unroll
    for (int s = 0; s < kDigits; ++s) {
      const size_t base = ((size_t(b) * kDigits + s) * parts) * plane + size_t(r) * kpad + k;
      sl[base] = __float2bfloat16_rn(float(dr[s]));
      if (CPLX) sl[base + plane] = __float2bfloat16_rn(float(di[s]));
    }
  }
}

// One CTA per 32 x 32 output tile of one batch entry.
template <int PA, int PB>
__global__ void __launch_bounds__(oz::kThreads, 1)
    ozaki_mma_kernel(int M, int N, int mpad, int npad, int kpad, const __nv_bfloat16* __restrict__ As,
                     const int* __restrict__ ea, const __nv_bfloat16* __restrict__ Bs, const int* __restrict__ eb,
                     GemmArgs g, int a_shared, int b_shared) {
  extern __shared__ __align__(16) __nv_bfloat16 sm[];
  const int b = blockIdx.z;
  const int mt0 = blockIdx.y * oz::kTile, nt0 = blockIdx.x * oz::kTile;
  const size_t aplane = size_t(mpad) * kpad, bplane = size_t(npad) * kpad;
  oz::Acc o;
  // an operand shared by all batch entries (batch stride 0) is split once
  const int ba = a_shared ? 0 : b, bb = b_shared ? 0 : b;
  oz::mainloop<PA, PB>(As + size_t(ba) * kDigits * PA * aplane + size_t(mt0) * kpad, aplane, kpad,
                       Bs + size_t(bb) * kDigits * PB * bplane + size_t(nt0) * kpad, bplane, kpad, kpad, sm, o);
  // epilogue: scale by 2^(ea + eb - 57), alpha/beta, store
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wm = (warp >> 2) * 16, wn = (warp & 3) * 8;
  double2 alpha = g.alpha;
  if (g.alpha_vec) alpha = cmul(alpha, g.alpha_vec[b]);
  const bool cplx_out = !g.c_real;
  const bool alpha_real = alpha.y == 0.0;
  const bool beta_zero = g.beta.x == 0.0 && g.beta.y == 0.0;
  const bool beta_one = g.beta.x == 1.0 && g.beta.y == 0.0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = mt0 + wm + (lane >> 2) + ((q & 2) ? 8 : 0);
    const int j = nt0 + wn + 2 * (lane & 3) + (q & 1);
    if (i >= M || j >= N) continue;
    // the power-of-two scale is exact: folding it into alpha rounds as
    // scaling first would
    const double p2 = oz::pow2(ea[size_t(ba) * mpad + i] + eb[size_t(bb) * npad + j] - 57);
    const double2 v0 = oz::acc_value(o, q);
    const long long idx = i * g.crs + j * g.ccs + b * g.cbs;
    double2 v;
    if (alpha_real) {
      const double f = alpha.x * p2;
      v = make_double2(v0.x * f, v0.y * f);
    } else {
      v = cmul(alpha, make_double2(v0.x * p2, v0.y * p2));
    }
    if (cplx_out) {
      double2* C = static_cast<double2*>(g.C);
      if (beta_one) {
        const double2 c0 = C[idx];
        v = make_double2(v.x + c0.x, v.y + c0.y);
      } else if (!beta_zero) {
        v = cadd(v, cmul(g.beta, C[idx]));
      }
      C[idx] = v;
    } else {
      double* C = static_cast<double*>(g.C);
      double r = v.x;
      if (!beta_zero) r = fma(g.beta.x, C[idx], r);
      C[idx] = r;
    }
  }
}

template <int PA, int PB>
int launch_ozaki_mma(int M, int N, int mpad, int npad, int kpad, const __nv_bfloat16* As, const int* ea,
                     const __nv_bfloat16* Bs, const int* eb, const GemmArgs& g, cudaStream_t s) {
  const int a_shared = g.A.bs == 0 ? 1 : 0, b_shared = g.B.bs == 0 ? 1 : 0;
  const size_t shm = oz::Shape<PA, PB>::kSmemBytes;
  static bool attr = false;
  if (!attr) {
    TVAP_CUDA(cudaFuncSetAttribute(ozaki_mma_kernel<PA, PB>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(shm)));
    attr = true;
  }
  dim3 grid(npad / oz::kTile, mpad / oz::kTile, g.batch);
  ozaki_mma_kernel<PA, PB><<<grid, oz::kThreads, shm, s>>>(M, N, mpad, npad, kpad, As, ea, Bs, eb, g, a_shared,
                                                            b_shared);
  TVAP_CUDA(cudaGetLastError());
  return TVAP_OK;
}

// One CTA per (128 x 64 output tile, component) of one batch entry, tcgen05
// MMAs with tensor-memory accumulators (ozaki_tc.cuh).  alpha and beta are
// real here (the components are then independent).
template <int PA, int PB>
__global__ void __launch_bounds__(oztc::kThreads, 1)
    ozaki_tc_kernel(int M, int N, int mpad, int npad, int kpad, const __nv_bfloat16* __restrict__ As,
                    const int* __restrict__ ea, const __nv_bfloat16* __restrict__ Bs, const int* __restrict__ eb,
                    GemmArgs g, int ncomp, int a_shared, int b_shared, int* flags) {
  extern __shared__ __align__(1024) __nv_bfloat16 tsm[];
  __shared__ oztc::Ctl ctl;
  const int b = blockIdx.z / ncomp, comp = blockIdx.z - b * ncomp;
  const int ba = a_shared ? 0 : b, bb = b_shared ? 0 : b;
  const int mt0 = blockIdx.y * oztc::kM, nt0 = blockIdx.x * oztc::kN;
  const size_t aplane = size_t(mpad) * kpad, bplane = size_t(npad) * kpad;
  const __nv_bfloat16* A = As + size_t(ba) * kDigits * PA * aplane + size_t(mt0) * kpad;
  const __nv_bfloat16* B = Bs + size_t(bb) * kDigits * PB * bplane + size_t(nt0) * kpad;
  oztc::setup(ctl);
  oztc::Acc o;
  bool ok;
  if (comp == 0)
    ok = oztc::mainloop<PA, PB, 0>(A, aplane, kpad, mpad - mt0, B, bplane, kpad, npad - nt0, kpad, tsm, ctl, o);
  else
    ok = oztc::mainloop<PA, PB, 1>(A, aplane, kpad, mpad - mt0, B, bplane, kpad, npad - nt0, kpad, tsm, ctl, o);
  oztc::teardown(ctl);
  if (!ok) {
    if (threadIdx.x == 0 && flags) atomicOr(flags, DEV_TC_TIMEOUT);
    return;
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = mt0 + 32 * (warp & 3) + lane;
  if (i >= M) return;
  const double alpha = g.alpha.x, beta = g.beta.x;
  const int eai = ea[size_t(ba) * mpad + i] - 57;
  double* C = static_cast<double*>(g.C);
  const int cw = g.c_real ? 1 : 2;  // doubles per element
#pragma unroll
  for (int c = 0; c < 16; ++c) {
    const int j = nt0 + 16 * (warp >> 2) + c;
    if (j >= N) continue;
    const double v = oztc::value(o, c) * (alpha * oz::pow2(eai + eb[size_t(bb) * npad + j]));
    const long long idx = (i * g.crs + j * g.ccs + b * g.cbs) * cw + comp;
    C[idx] = (beta == 0.0) ? v : fma(beta, C[idx], v);
  }
}

template <int PA, int PB>
int launch_ozaki_tc(int M, int N, int mpad, int npad, int kpad, const __nv_bfloat16* As, const int* ea,
                    const __nv_bfloat16* Bs, const int* eb, const GemmArgs& g, cudaStream_t s) {
  const size_t shm = oztc::kSmemBytes;
  static bool attr = false;
  if (!attr) {
    TVAP_CUDA(cudaFuncSetAttribute(ozaki_tc_kernel<PA, PB>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(shm)));
    attr = true;
  }
  const int ncomp = (g.c_real || (PA == 1 && PB == 1)) ? 1 : 2;
  const int a_shared = g.A.bs == 0 ? 1 : 0, b_shared = g.B.bs == 0 ? 1 : 0;
  dim3 grid((npad + oztc::kN - 1) / oztc::kN, (mpad + oztc::kM - 1) / oztc::kM, g.batch * ncomp);
  ozaki_tc_kernel<PA, PB><<<grid, oztc::kThreads, shm, s>>>(M, N, mpad, npad, kpad, As, ea, Bs, eb, g, ncomp,
                                                             a_shared, b_shared, g_dev_flags);
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

int oz_scratch(cudaStream_t s, size_t bytes, size_t ex_count, __nv_bfloat16** buf, int** ex) {
  OzScratch* sc = nullptr;
  int rc;
  if ((rc = oz_reserve(s, bytes, ex_count, &sc))) return rc;
  *buf = sc->buf;
  *ex = sc->ex;
  return TVAP_OK;
}

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
  // operands with batch stride 0 are split once for the whole batch
  const int abatch = g.A.bs == 0 ? 1 : g.batch, bbatch = g.B.bs == 0 ? 1 : g.batch;
  const size_t asz = size_t(abatch) * kDigits * PA * mpad * kpad;
  const size_t bsz = size_t(bbatch) * kDigits * PB * npad * kpad;
  int rc;
  OzScratch* sc = nullptr;
  if ((rc = oz_reserve(s, sizeof(__nv_bfloat16) * (asz + bsz), size_t(abatch) * mpad + size_t(bbatch) * npad, &sc)))
    return rc;
  __nv_bfloat16* As = sc->buf;
  __nv_bfloat16* Bs = sc->buf + asz;
  int* ea = sc->ex;
  int* eb = sc->ex + size_t(abatch) * mpad;
  // A rows: element (i, k) at A.p[i rs + k cs]; B columns: element (j, k) = B(k, j) at B.p[k rs + j cs]
  {
    dim3 grid((mpad + 7) / 8, abatch);
    if (PA == 2)
      slice_kernel<true><<<grid, 256, 0, s>>>(g.M, g.K, mpad, kpad, g.A.p, g.A.rs, g.A.cs, g.A.bs, g.conj_a, As, ea);
    else
      slice_kernel<false><<<grid, 256, 0, s>>>(g.M, g.K, mpad, kpad, g.A.p, g.A.rs, g.A.cs, g.A.bs, false, As, ea);
  }
  {
    dim3 grid((npad + 7) / 8, bbatch);
    if (PB == 2)
      slice_kernel<true><<<grid, 256, 0, s>>>(g.N, g.K, npad, kpad, g.B.p, g.B.cs, g.B.rs, g.B.bs, g.conj_b, Bs, eb);
    else
      slice_kernel<false><<<grid, 256, 0, s>>>(g.N, g.K, npad, kpad, g.B.p, g.B.cs, g.B.rs, g.B.bs, false, Bs, eb);
  }
  // tensor-memory path: real alpha / beta (the components are then independent)
  const bool real_scalars = g.alpha.y == 0.0 && g.beta.y == 0.0 && !g.alpha_vec;
  if (g_gemm_mode == 2 && real_scalars && g.batch * 2 <= 65535) {
    if (PA == 2 && PB == 2) return launch_ozaki_tc<2, 2>(g.M, g.N, mpad, npad, kpad, As, ea, Bs, eb, g, s);
    if (PA == 2) return launch_ozaki_tc<2, 1>(g.M, g.N, mpad, npad, kpad, As, ea, Bs, eb, g, s);
    if (PB == 2) return launch_ozaki_tc<1, 2>(g.M, g.N, mpad, npad, kpad, As, ea, Bs, eb, g, s);
    return launch_ozaki_tc<1, 1>(g.M, g.N, mpad, npad, kpad, As, ea, Bs, eb, g, s);
  }
  if (PA == 2 && PB == 2) return launch_ozaki_mma<2, 2>(g.M, g.N, mpad, npad, kpad, As, ea, Bs, eb, g, s);
  if (PA == 2) return launch_ozaki_mma<2, 1>(g.M, g.N, mpad, npad, kpad, As, ea, Bs, eb, g, s);
  if (PB == 2) return launch_ozaki_mma<1, 2>(g.M, g.N, mpad, npad, kpad, As, ea, Bs, eb, g, s);
  return launch_ozaki_mma<1, 1>(g.M, g.N, mpad, npad, kpad, As, ea, Bs, eb, g, s);
}

}  // namespace tvap
