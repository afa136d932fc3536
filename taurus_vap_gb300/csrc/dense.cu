// Dense FP64 building blocks of the per-angle algebra, batched over gauge
// angles: strided batched GEMM (complex/real operands specialised so that no
// FP64 operation is spent on zero imaginary parts), the Thouless solve, the
// Parlett-Reid Pfaffian, the Jacobi eigen-decomposition and the Cholesky
// factorisation with triangular inverse.
//
// On GB300 the FP64 pipe (about 1.25 TFLOP/s for the whole chip) bounds every
// kernel in this file, so each kernel is written to issue the minimum number
// of DFMAs; memory traffic is secondary.

#include <algorithm>
#include <mutex>
#include <utility>
#include <vector>

#include "tvap_internal.cuh"

namespace tvap {

namespace {

// multiply-accumulate specialised on operand types
__device__ __forceinline__ void mac(double2& c, double2 a, double2 b) { cfma(c, a, b); }
__device__ __forceinline__ void mac(double2& c, double a, double2 b) {
  c.x = fma(a, b.x, c.x);
  c.y = fma(a, b.y, c.y);
}
__device__ __forceinline__ void mac(double2& c, double2 a, double b) {
  c.x = fma(a.x, b, c.x);
  c.y = fma(a.y, b, c.y);
}
__device__ __forceinline__ void mac(double& c, double a, double b) { c = fma(a, b, c); }

template <typename T>
__device__ __forceinline__ T load_el(const View& v, long long i, long long j, long long b, bool cj);
template <>
__device__ __forceinline__ double load_el<double>(const View& v, long long i, long long j, long long b, bool) {
  return static_cast<const double*>(v.p)[i * v.rs + j * v.cs + b * v.bs];
}
template <>
__device__ __forceinline__ double2 load_el<double2>(const View& v, long long i, long long j, long long b, bool cj) {
  double2 x = static_cast<const double2*>(v.p)[i * v.rs + j * v.cs + b * v.bs];
  if (cj) x.y = -x.y;
  return x;
}
template <typename T>
__device__ __forceinline__ T zero_of();
template <>
__device__ __forceinline__ double zero_of<double>() {
  return 0.0;
}
template <>
__device__ __forceinline__ double2 zero_of<double2>() {
  return make_double2(0.0, 0.0);
}

template <typename TA, typename TB>
struct AccT {
  typedef double2 type;
};
template <>
struct AccT<double, double> {
  typedef double type;
};

__device__ __forceinline__ void store_out(const GemmArgs& g, long long idx, double acc, double2 alpha) {
  double* C = static_cast<double*>(g.C);
  double v = alpha.x * acc;
  if (g.beta.x != 0.0) v = fma(g.beta.x, C[idx], v);
  C[idx] = v;
}
__device__ __forceinline__ void store_out(const GemmArgs& g, long long idx, double2 acc, double2 alpha) {
  double2* C = static_cast<double2*>(g.C);
  double2 v = cmul(alpha, acc);
  if (g.beta.x != 0.0 || g.beta.y != 0.0) v = cadd(v, cmul(g.beta, C[idx]));
  C[idx] = v;
}
__device__ __forceinline__ void store_out_real_from_complex(const GemmArgs& g, long long idx, double2 acc,
                                                            double2 alpha) {
  double* C = static_cast<double*>(g.C);
  double v = (cmul(alpha, acc)).x;
  if (g.beta.x != 0.0) v = fma(g.beta.x, C[idx], v);
  C[idx] = v;
}

// TM x TN output tile per CTA, 2 x 2 outputs per thread (strided by half the
// tile so that neighbouring threads read neighbouring shared-memory words).
template <int TM, int TN, typename TA, typename TB>
__global__ void __launch_bounds__((TM / 2) * (TN / 2)) gemm_kernel(GemmArgs g) {
  typedef typename AccT<TA, TB>::type TC;
  constexpr int BK = 16;
  constexpr int HM = TM / 2, HN = TN / 2;
  constexpr int NT = HM * HN;
  __shared__ TA As[BK][TM + 1];
  __shared__ TB Bs[BK][TN + 1];
  const long long b = blockIdx.z;
  const int i0 = blockIdx.y * TM, j0 = blockIdx.x * TN;
  const int tid = threadIdx.x;
  const int ty = tid / HN, tx = tid % HN;
  TC acc[2][2];
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int c = 0; c < 2; ++c) acc[r][c] = zero_of<TC>();
  const bool live = (i0 + ty < g.M) && (j0 + tx < g.N);
  for (int k0 = 0; k0 < g.K; k0 += BK) {
    const int kt = min(BK, g.K - k0);
    for (int idx = tid; idx < TM * BK; idx += NT) {
      const int ii = idx % TM, kk = idx / TM;
      TA v = zero_of<TA>();
      if (i0 + ii < g.M && kk < kt) v = load_el<TA>(g.A, i0 + ii, k0 + kk, b, g.conj_a);
      As[kk][ii] = v;
    }
    for (int idx = tid; idx < TN * BK; idx += NT) {
      const int jj = idx % TN, kk = idx / TN;
      TB v = zero_of<TB>();
      if (j0 + jj < g.N && kk < kt) v = load_el<TB>(g.B, k0 + kk, j0 + jj, b, g.conj_b);
      Bs[kk][jj] = v;
    }
    __syncthreads();
    if (live) {
      for (int kk = 0; kk < kt; ++kk) {
        const TA a0 = As[kk][ty], a1 = As[kk][ty + HM];
        const TB b0 = Bs[kk][tx], b1 = Bs[kk][tx + HN];
        mac(acc[0][0], a0, b0);
        mac(acc[0][1], a0, b1);
        mac(acc[1][0], a1, b0);
        mac(acc[1][1], a1, b1);
      }
    }
    __syncthreads();
  }
  double2 alpha = g.alpha;
  if (g.alpha_vec) alpha = cmul(alpha, g.alpha_vec[b]);
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const int i = i0 + ty + r * HM, j = j0 + tx + c * HN;
      if (i < g.M && j < g.N) {
        const long long idx = i * g.crs + j * g.ccs + b * g.cbs;
        if constexpr (sizeof(TC) == sizeof(double)) {
          store_out(g, idx, acc[r][c], alpha);
        } else {
          if (g.c_real)
            store_out_real_from_complex(g, idx, acc[r][c], alpha);
          else
            store_out(g, idx, acc[r][c], alpha);
        }
      }
    }
}

// Complex x complex with three real products per multiply-add (the 3M form):
//   t1 = sum Ar Br,  t2 = sum Ai Bi,  t3 = sum (Ar + Ai)(Br + Bi),
//   Re C = t1 - t2,  Im C = t3 - t1 - t2,
// the sums Ar + Ai, Br + Bi being formed once per element when the tile is
// staged.  3 DFMA instead of 4 per complex multiply-add.
template <int TM, int TN>
__global__ void __launch_bounds__((TM / 2) * (TN / 2)) gemm3m_kernel(GemmArgs g) {
  constexpr int BK = 16;
  constexpr int HM = TM / 2, HN = TN / 2;
  constexpr int NT = HM * HN;
  __shared__ double3 As[BK][TM + 1];
  __shared__ double3 Bs[BK][TN + 1];
  const long long b = blockIdx.z;
  if (g.upper_only && blockIdx.y > blockIdx.x) return;
  const int i0 = blockIdx.y * TM, j0 = blockIdx.x * TN;
  const int tid = threadIdx.x;
  const int ty = tid / HN, tx = tid % HN;
  double t1[2][2], t2[2][2], t3[2][2];
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int c = 0; c < 2; ++c) t1[r][c] = t2[r][c] = t3[r][c] = 0.0;
  const bool live = (i0 + ty < g.M) && (j0 + tx < g.N);
  for (int k0 = 0; k0 < g.K; k0 += BK) {
    const int kt = min(BK, g.K - k0);
    for (int idx = tid; idx < TM * BK; idx += NT) {
      const int ii = idx % TM, kk = idx / TM;
      double2 v = make_double2(0.0, 0.0);
      if (i0 + ii < g.M && kk < kt) v = load_el<double2>(g.A, i0 + ii, k0 + kk, b, g.conj_a);
      As[kk][ii] = make_double3(v.x, v.y, v.x + v.y);
    }
    for (int idx = tid; idx < TN * BK; idx += NT) {
      const int jj = idx % TN, kk = idx / TN;
      double2 v = make_double2(0.0, 0.0);
      if (j0 + jj < g.N && kk < kt) v = load_el<double2>(g.B, k0 + kk, j0 + jj, b, g.conj_b);
      Bs[kk][jj] = make_double3(v.x, v.y, v.x + v.y);
    }
    __syncthreads();
    if (live) {
      for (int kk = 0; kk < kt; ++kk) {
        const double3 a0 = As[kk][ty], a1 = As[kk][ty + HM];
        const double3 b0 = Bs[kk][tx], b1 = Bs[kk][tx + HN];
        t1[0][0] = fma(a0.x, b0.x, t1[0][0]); t2[0][0] = fma(a0.y, b0.y, t2[0][0]); t3[0][0] = fma(a0.z, b0.z, t3[0][0]);
        t1[0][1] = fma(a0.x, b1.x, t1[0][1]); t2[0][1] = fma(a0.y, b1.y, t2[0][1]); t3[0][1] = fma(a0.z, b1.z, t3[0][1]);
        t1[1][0] = fma(a1.x, b0.x, t1[1][0]); t2[1][0] = fma(a1.y, b0.y, t2[1][0]); t3[1][0] = fma(a1.z, b0.z, t3[1][0]);
        t1[1][1] = fma(a1.x, b1.x, t1[1][1]); t2[1][1] = fma(a1.y, b1.y, t2[1][1]); t3[1][1] = fma(a1.z, b1.z, t3[1][1]);
      }
    }
    __syncthreads();
  }
  double2 alpha = g.alpha;
  if (g.alpha_vec) alpha = cmul(alpha, g.alpha_vec[b]);
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const int i = i0 + ty + r * HM, j = j0 + tx + c * HN;
      if (i < g.M && j < g.N) {
        const long long idx = i * g.crs + j * g.ccs + b * g.cbs;
        const double2 acc = make_double2(t1[r][c] - t2[r][c], t3[r][c] - t1[r][c] - t2[r][c]);
        store_out(g, idx, acc, alpha);
      }
    }
}

template <int T, typename TA, typename TB>
void launch_gemm_t(const GemmArgs& g, cudaStream_t s) {
  dim3 grid((g.N + T - 1) / T, (g.M + T - 1) / T, g.batch);
  gemm_kernel<T, T, TA, TB><<<grid, (T / 2) * (T / 2), 0, tvap::counted(s)>>>(g);
}

template <int T>
void launch_gemm_tile(const GemmArgs& g, cudaStream_t s) {
  if (g.a_real && g.b_real)
    launch_gemm_t<T, double, double>(g, s);
  else if (g.a_real)
    launch_gemm_t<T, double, double2>(g, s);
  else if (g.b_real)
    launch_gemm_t<T, double2, double>(g, s);
  else if (g.three_m) {
    dim3 grid((g.N + T - 1) / T, (g.M + T - 1) / T, g.batch);
    gemm3m_kernel<T, T><<<grid, (T / 2) * (T / 2), 0, tvap::counted(s)>>>(g);
  } else
    launch_gemm_t<T, double2, double2>(g, s);
}

// Tile choice: minimise padded FP64 work (the pipe is the bound), then prefer
// larger tiles.  Candidates are compiled instantiations.
const int kTiles[] = {16, 24, 28, 32, 40, 48, 56};

int pick_tile(int M, int N) {
  int best = 32;
  double best_w = 1e30;
  for (int t : kTiles) {
    const double w = double((M + t - 1) / t) * ((N + t - 1) / t) * t * t / (double(M) * N);
    if (w < best_w - 1e-9 || (std::fabs(w - best_w) < 1e-9 && t > best)) {
      best_w = w;
      best = t;
    }
  }
  return best;
}

}  // namespace

thread_local int g_gemm_mode = 2;
thread_local int g_tc_grid_cap = 0;
thread_local int g_tc_bn_policy = 0;
thread_local int g_tc_pairs_min_k = 0;
thread_local int* g_dev_flags = nullptr;
thread_local tvap_ctx* g_tc_timing_ctx = nullptr;
thread_local int g_tc_timing_sec = -1;
thread_local long long g_launch_count = 0;

int gemm_split_k2(const GemmArgs& g, cudaStream_t s) {
  GemmArgs g1 = g;
  g1.K2 = 0;
  int rc;
  if ((rc = gemm(g1, s))) return rc;
  GemmArgs g2 = g;
  g2.K2 = 0;
  g2.reuse_left = false;  // another left operand
  g2.A = g.A2;
  g2.B = g.B2;
  g2.K = g.K2;
  g2.alpha = cscale(g.alpha, g.s2);
  g2.beta = make_double2(1.0, 0.0);
  return gemm(g2, s);
}

int gemm(const GemmArgs& g, cudaStream_t s) {
  if (g.M <= 0 || g.N <= 0 || g.batch <= 0) return TVAP_OK;
  if (g.K2 > 0) {
    const double kk = double(g.K) + g.K2;
    if (g_gemm_mode == 2 && double(g.M) * g.N * kk * g.batch >= 1.0e6) return gemm_ozaki(g, s);
    return gemm_split_k2(g, s);
  }
  // every product of at least 10^6 multiply-adds runs emulated on the tensor
  // cores; the smaller ones (few-column blocks, short K) stay on the FP64 pipe
  if (g_gemm_mode >= 1 && g.K >= 16 && double(g.M) * g.N * g.K * g.batch >= 1.0e6) return gemm_ozaki(g, s);
  // few tiles in all (single small products): the smallest tile, to spread
  // the latency-bound work over more SMs
  const long long t28 = (long long)((g.M + 27) / 28) * ((g.N + 27) / 28) * g.batch;
  const int tile = (t28 < 76) ? 16 : pick_tile(g.M, g.N);
  switch (tile) {
    case 16: launch_gemm_tile<16>(g, s); break;
    case 24: launch_gemm_tile<24>(g, s); break;
    case 28: launch_gemm_tile<28>(g, s); break;
    case 40: launch_gemm_tile<40>(g, s); break;
    case 48: launch_gemm_tile<48>(g, s); break;
    case 56: launch_gemm_tile<56>(g, s); break;
    default: launch_gemm_tile<32>(g, s); break;
  }
  TVAP_CUDA(cudaGetLastError());
  return TVAP_OK;
}

namespace {

__device__ void block_argmax(double v, int idx, double* sv, int* si, int& out_idx, double& out_v) {
  // first index of the maximum, like IZAMAX
  const int tid = threadIdx.x;
  sv[tid] = v;
  si[tid] = idx;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (tid < s) {
      const double a = sv[tid], b = sv[tid + s];
      const int ia = si[tid], ib = si[tid + s];
      if (b > a || (b == a && ib < ia)) {
        sv[tid] = b;
        si[tid] = ib;
      }
    }
    __syncthreads();
  }
  out_idx = si[0];
  out_v = sv[0];
  __syncthreads();
}

}  // namespace

// ---------------------------------------------------------------------------
// Pfaffian: PFAPACK ZSKTF2 (UPLO='U', MODE='P') restated for one CTA per
// matrix (subroutines_pfaffian.f:1694-2017 with the ZSKR2 update :2387-2630):
// pivot = first maximum of |Re|+|Im| over A(1:K-1,K) (IZAMAX), row/column
// exchange, skew rank-2 update of the leading block, and
// Pf = prod A(K-1,K) * (-1)^(#exchanges) (ZSKPFA :193-203).  The product is
// returned as (log|Pf|, phase) to stay finite for large n.
// Output per matrix: pf[b] = (log|Pf|, 0), phase in pf[batch + b]; a zero
// pivot yields log|Pf| = -inf.
// ---------------------------------------------------------------------------
namespace {

constexpr int kPfThreads = 512;

__global__ void __launch_bounds__(kPfThreads) pfaffian_kernel(int N, double2* Aall, double2* pf, int batch,
                                                              int* flags) {
  __shared__ double sv[kPfThreads];
  __shared__ int si[kPfThreads];
  __shared__ double2 xcol[512], ycol[512];
  const int b = blockIdx.x;
  double2* A = Aall + size_t(b) * N * N;
  auto a = [A, N](int i, int j) -> double2& { return A[size_t(i - 1) + size_t(j - 1) * N]; };
  const int tid = threadIdx.x, nt = blockDim.x;
  double logmag = 0.0;
  double2 phase = make_double2(1.0, 0.0);
  bool zero = false;
  for (int K = N; K >= 2; K -= 2) {
    double best = -1.0;
    int bi = N + 1;
    for (int i = 1 + tid; i <= K - 1; i += nt) {
      const double v = cabs1(a(i, K));
      if (v > best) {
        best = v;
        bi = i;
      }
    }
    int KP;
    double pv;
    block_argmax(best, bi, sv, si, KP, pv);
    if (KP > K - 1) KP = 1;  // every |a(i, K)| is NaN: IZAMAX returns the first index
    const int KK = K - 1;
    if (pv == 0.0) {
      zero = true;
      KP = KK;
    }
    if (KP != KK) {
      for (int i = 1 + tid; i <= KP - 1; i += nt) {
        const double2 t = a(i, KK);
        a(i, KK) = a(i, KP);
        a(i, KP) = t;
      }
      for (int t = tid; t < KK - KP - 1; t += nt) {
        const double2 u = a(KP + 1 + t, KK);
        a(KP + 1 + t, KK) = a(KP, KP + 1 + t);
        a(KP, KP + 1 + t) = u;
      }
      for (int j = K + tid; j <= N; j += nt) {
        const double2 u = a(KK, j);
        a(KK, j) = a(KP, j);
        a(KP, j) = u;
      }
      __syncthreads();
      for (int i = KP + tid; i <= KK - 1; i += nt) a(i, KK) = cneg(a(i, KK));
      for (int j = KP + 1 + tid; j <= KK - 1; j += nt) a(KP, j) = cneg(a(KP, j));
      __syncthreads();
    }
    const double2 piv = a(K - 1, K);
    if (!zero) {
      const double m = hypot(piv.x, piv.y);
      logmag += log(m);
      phase = cmul(phase, make_double2(piv.x / m, piv.y / m));
      if (KP != KK) phase = cneg(phase);
      const double2 alpha = crcp(piv);
      const int nn = K - 2;
      for (int i = 1 + tid; i <= nn; i += nt) {
        xcol[i] = a(i, K);
        ycol[i] = a(i, K - 1);
      }
      __syncthreads();
      // A(I,J) += X(I) * (alpha Y(J)) - Y(I) * (alpha X(J)),  I < J <= nn
      // (ZSKR2 skips a column J whose X(J) and Y(J) are both zero);
      // one warp per column J, lanes over I (coalesced, no index division)
      {
        const int warp = tid >> 5, lane = tid & 31, nw = nt >> 5;
        for (int J = 2 + warp; J <= nn; J += nw) {
          const double2 xj = xcol[J], yj = ycol[J];
          if (xj.x == 0.0 && xj.y == 0.0 && yj.x == 0.0 && yj.y == 0.0) continue;
          const double2 t1 = cmul(alpha, yj), t2 = cmul(alpha, xj);
          double2* colJ = A + size_t(J - 1) * N;
          for (int I = 1 + lane; I <= J - 1; I += 32) {
            double2 v = colJ[I - 1];
            cfma(v, xcol[I], t1);
            cfma(v, cneg(ycol[I]), t2);
            colJ[I - 1] = v;
          }
        }
      }
      __syncthreads();
      for (int i = 1 + tid; i <= nn; i += nt) a(i, K) = cmul(alpha, a(i, K));
      __syncthreads();
    }
  }
  if (tid == 0) {
    pf[b] = make_double2(zero ? -INFINITY : logmag, 0.0);
    pf[batch + b] = zero ? make_double2(0.0, 0.0) : phase;
    if (zero) atomicOr(flags, DEV_PFAFF_ZERO);
  }
}

// The same elimination with the packed upper triangle in shared memory
// (N (N + 1) / 2 entries, column-major): every access stays on the SM, the
// pivot search is a warp reduction plus one block step, and the already
// eliminated columns (which no longer enter the Pfaffian) are neither
// exchanged nor scaled.
// The same elimination with the packed upper triangle in shared memory.  Per
// step only the pivot's reciprocal is needed by every thread: one thread
// forms it (an FP64 division costs ~1000 cycles and an FP64 warp instruction
// ~16 cycles of the SM's FP64 pipe, so redundant scalar work in every thread
// costs as much as the rank-2 update), the pivot search compares integer keys,
// and the pivots are kept in shared memory and folded into log|Pf| and its
// phase once, at the end, by a fixed-order warp reduction.
__global__ void __launch_bounds__(kPfThreads) pfaffian_smem_kernel(int N, const double2* __restrict__ Aall,
                                                                   double2* pf, int batch, int* flags) {
  extern __shared__ double2 pf_smem[];
  double2* pk = pf_smem;
  double2* xcol = pk + size_t(N) * (N + 1) / 2;  // 1-based, N + 1 entries
  double2* ycol = xcol + N + 1;
  double2* pivs = ycol + N + 1;                  // N / 2 pivots, then N / 2 signs in .x of the next slots
  double2* tt1 = pivs + N;                       // alpha y_J and alpha x_J, 1-based
  double2* tt2 = tt1 + N + 1;
  __shared__ long long wv[kPfThreads / 32];
  __shared__ int wi[kPfThreads / 32];
  __shared__ int s_kp;
  __shared__ double2 s_alpha;
  const int b = blockIdx.x;
  const double2* A = Aall + size_t(b) * N * N;
  auto a = [pk](int i, int j) -> double2& { return pk[(i - 1) + (size_t(j) * (j - 1)) / 2]; };  // 1 <= i <= j
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  for (int j = 1 + warp; j <= N; j += nw)
    for (int i = 1 + lane; i <= j; i += 32) a(i, j) = A[(i - 1) + size_t(j - 1) * N];
  __syncthreads();
  bool zero = false;
  int steps = 0;
  for (int K = N; K >= 2; K -= 2, ++steps) {
    // |re| + |im| >= 0: its bit pattern orders like its value
    long long best = -1;
    int bi = N + 1;
    for (int i = 1 + tid; i <= K - 1; i += nt) {
      const long long v = __double_as_longlong(cabs1(a(i, K)));
      if (v > best) {
        best = v;
        bi = i;
      }
    }
    for (int off = 16; off > 0; off >>= 1) {
      const long long v2 = __shfl_down_sync(0xffffffffu, best, off);
      const int i2 = __shfl_down_sync(0xffffffffu, bi, off);
      if (v2 > best || (v2 == best && i2 < bi)) {
        best = v2;
        bi = i2;
      }
    }
    if (lane == 0) {
      wv[warp] = best;
      wi[warp] = bi;
    }
    __syncthreads();
    if (warp == 0) {
      long long v = (lane < nw) ? wv[lane] : -1;
      int i = (lane < nw) ? wi[lane] : N + 1;
      for (int off = 16; off > 0; off >>= 1) {
        const long long v2 = __shfl_down_sync(0xffffffffu, v, off);
        const int i2 = __shfl_down_sync(0xffffffffu, i, off);
        if (v2 > v || (v2 == v && i2 < i)) {
          v = v2;
          i = i2;
        }
      }
      if (lane == 0) s_kp = (v <= 0) ? -1 : i;  // -1: the column is zero
    }
    __syncthreads();
    int KP = s_kp;
    const int KK = K - 1;
    if (KP < 0) {
      zero = true;
      KP = KK;
    }
    if (KP != KK) {
      for (int i = 1 + tid; i <= KP - 1; i += nt) {
        const double2 t = a(i, KK);
        a(i, KK) = a(i, KP);
        a(i, KP) = t;
      }
      for (int t = tid; t < KK - KP - 1; t += nt) {
        const double2 u = a(KP + 1 + t, KK);
        a(KP + 1 + t, KK) = a(KP, KP + 1 + t);
        a(KP, KP + 1 + t) = u;
      }
      if (tid == 0) {
        const double2 u = a(KK, K);
        a(KK, K) = a(KP, K);
        a(KP, K) = u;
      }
      __syncthreads();
      for (int i = KP + tid; i <= KK - 1; i += nt) a(i, KK) = cneg(a(i, KK));
      for (int j = KP + 1 + tid; j <= KK - 1; j += nt) a(KP, j) = cneg(a(KP, j));
      __syncthreads();
    }
    if (zero) break;
    const int nn = K - 2;
    if (tid == 0) {
      const double2 piv = a(K - 1, K);
      pivs[steps] = piv;
      pivs[N / 2 + steps] = make_double2(KP != KK ? -1.0 : 1.0, 0.0);
      s_alpha = crcp_newton(piv);
    }
    __syncthreads();
    // the two columns and their products with alpha, once per step (threads
    // over the entries: the FP64 pipe is the bottleneck of this kernel)
    {
      const double2 alpha = s_alpha;
      for (int i = 1 + tid; i <= nn; i += nt) {
        const double2 x = a(i, K), y = a(i, K - 1);
        xcol[i] = x;
        ycol[i] = y;
        tt1[i] = cmul(alpha, y);
        tt2[i] = cmul(alpha, x);
      }
    }
    __syncthreads();
    // A(I,J) += X(I) (alpha Y(J)) - Y(I) (alpha X(J)), I < J <= nn: a warp
    // per pair of columns J1 = 2 + p and J2 = nn - p (about nn entries
    // together), lanes over the pair's entries, two entries in flight
    for (int p = warp; p < nn / 2; p += nw) {
      const int J1 = 2 + p, J2 = nn - p;
      const int L1 = J1 - 1, L = L1 + (J2 > J1 ? J2 - 1 : 0);
      for (int f0 = lane; f0 < L; f0 += 64) {
        int I[2], J[2];
        double2 v[2], x[2], y[2], t1[2], t2[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int f = f0 + 32 * u;
          const bool first = f < L1;
          I[u] = first ? f + 1 : f - L1 + 1;
          J[u] = first ? J1 : J2;
          if (f < L) {
            v[u] = a(I[u], J[u]);
            x[u] = xcol[I[u]];
            y[u] = ycol[I[u]];
            t1[u] = tt1[J[u]];
            t2[u] = tt2[J[u]];
          }
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          if (f0 + 32 * u >= L) continue;
          double2 w = v[u];
          w.x = fma(x[u].x, t1[u].x, w.x);
          w.x = fma(-x[u].y, t1[u].y, w.x);
          w.y = fma(x[u].x, t1[u].y, w.y);
          w.y = fma(x[u].y, t1[u].x, w.y);
          w.x = fma(-y[u].x, t2[u].x, w.x);
          w.x = fma(y[u].y, t2[u].y, w.x);
          w.y = fma(-y[u].x, t2[u].y, w.y);
          w.y = fma(-y[u].y, t2[u].x, w.y);
          a(I[u], J[u]) = w;
        }
      }
    }
    __syncthreads();
  }
  // Pf = prod_k piv_k (times -1 per interchange), as log|Pf| and a unit phase:
  // warp 0, lanes over the pivots, then a fixed shuffle tree
  if (warp == 0) {
    double lm = 0.0;
    double2 ph = make_double2(1.0, 0.0);
    if (!zero) {
      for (int k = lane; k < steps; k += 32) {
        const double2 piv = pivs[k];
        const double m = hypot(piv.x, piv.y);
        lm += log(m);
        ph = cmul(ph, make_double2(piv.x / m, piv.y / m));
        if (pivs[N / 2 + k].x < 0.0) ph = cneg(ph);
      }
    }
    for (int off = 16; off > 0; off >>= 1) {
      const double lm2 = __shfl_down_sync(0xffffffffu, lm, off);
      const double2 ph2 = make_double2(__shfl_down_sync(0xffffffffu, ph.x, off), __shfl_down_sync(0xffffffffu, ph.y, off));
      lm += lm2;
      ph = cmul(ph, ph2);
    }
    if (lane == 0) {
      pf[b] = make_double2(zero ? -INFINITY : lm, 0.0);
      pf[batch + b] = zero ? make_double2(0.0, 0.0) : ph;
      if (zero) atomicOr(flags, DEV_PFAFF_ZERO);
    }
  }
}

// Blocked Parlett-Reid (the reference's ZLASKTRF form of ZSKTRF for large
// N, subroutines_pfaffian.f:1015-1400): a panel of up to kPfNb columns from
// the right is eliminated with delayed updates -- the current value of a
// column is its stored value plus sum_t (p_t q_t[c] - q_t p_t[c]) over the
// panel's earlier steps, with p_t = x (the column K above the pivot row) and
// q_t = y / A(K-1, K) (column K-1) -- and the interchanges act on the stored
// upper triangle and on the rows of the p and q vectors alike.  The leading
// block then takes the whole panel at once, A += P Q^T - Q P^T, as one
// batched product on the tensor cores (pf_trailing in pfaffian_batched).
// The pivots are those of the unblocked elimination; only the order of the
// rounding changes.
constexpr int kPfNb = 32;          // panel width (columns)
constexpr int kPfNs = kPfNb / 2;   // steps per panel

// One panel of every matrix: columns Kstart, Kstart-1, ..., Kstart-width+1
// (0-based).  X = [P | Q], Y = [Q | -P] (n x 2 kPfNs per matrix, unused
// columns zero) for the trailing product X Y^T.  pf[b] = (log|Pf|, 0) and
// pf[batch + b] = phase accumulate over the panels (first: start them).
__global__ void __launch_bounds__(kPfThreads) pf_panel_kernel(int N, int Kstart, int width, double2* __restrict__ Aall,
                                                           double2* __restrict__ Xall, double2* __restrict__ Yall,
                                                           double2* __restrict__ pf, int batch, int* flags,
                                                           int first) {
  __shared__ double sv[kPfThreads];
  __shared__ int si[kPfThreads];
  __shared__ double2 ck[512], ckk[512];
  __shared__ double s_lm;
  __shared__ double2 s_ph;
  __shared__ int s_zero;
  const int b = blockIdx.x;
  double2* A = Aall + size_t(b) * N * N;
  const size_t ldx = size_t(N);
  double2* X = Xall + size_t(b) * N * 2 * kPfNs;
  double2* Y = Yall + size_t(b) * N * 2 * kPfNs;
  auto a = [A, N](int i, int j) -> double2& { return A[i + size_t(j) * N]; };
  auto P = [X, ldx](int i, int t) -> double2& { return X[i + t * ldx]; };
  auto Q = [X, ldx](int i, int t) -> double2& { return X[i + (kPfNs + t) * ldx]; };
  const int tid = threadIdx.x, nt = blockDim.x;
  if (tid == 0) {
    if (first) {
      s_lm = 0.0;
      s_ph = make_double2(1.0, 0.0);
      s_zero = 0;
    } else {
      s_lm = pf[b].x;
      s_ph = pf[batch + b];
      s_zero = isinf(s_lm) && s_lm < 0.0;
    }
  }
  for (size_t idx = tid; idx < ldx * 2 * kPfNs; idx += nt) X[idx] = make_double2(0.0, 0.0);
  __syncthreads();
  if (s_zero) return;  // a zero pivot earlier: Pf = 0
  const int ns = width / 2;
  for (int s = 0; s < ns; ++s) {
    const int K = Kstart - 2 * s, KK = K - 1;
    // the current column K above the diagonal
    double best = -1.0;
    int bi = N + 1;
    for (int i = tid; i < K; i += nt) {
      double2 v = a(i, K);
      for (int t = 0; t < s; ++t) {
        cfma(v, P(i, t), Q(K, t));
        cfma(v, cneg(Q(i, t)), P(K, t));
      }
      ck[i] = v;
      const double m = cabs1(v);
      if (m > best) {
        best = m;
        bi = i;
      }
    }
    int KP;
    double pv;
    block_argmax(best, bi, sv, si, KP, pv);
    if (KP >= K) KP = 0;  // every |a(i, K)| is NaN: IZAMAX returns the first index
    if (pv == 0.0) {
      if (tid == 0) s_zero = 1;
      break;  // uniform: every thread holds the same pv
    }
    if (KP != KK) {
      // symmetric interchange KP <-> KK of the leading block in upper storage
      for (int i = tid; i < KP; i += nt) {
        const double2 t0 = a(i, KK);
        a(i, KK) = a(i, KP);
        a(i, KP) = t0;
      }
      for (int j = KP + 1 + tid; j < KK; j += nt) {
        const double2 t1 = a(j, KK), t2 = a(KP, j);
        a(j, KK) = cneg(t2);
        a(KP, j) = cneg(t1);
      }
      if (tid == 0) {
        a(KP, KK) = cneg(a(KP, KK));
        const double2 t3 = ck[KP];
        ck[KP] = ck[KK];
        ck[KK] = t3;
        s_ph = cneg(s_ph);
      }
      for (int t = tid; t < s; t += nt) {
        double2 u = P(KP, t);
        P(KP, t) = P(KK, t);
        P(KK, t) = u;
        u = Q(KP, t);
        Q(KP, t) = Q(KK, t);
        Q(KK, t) = u;
      }
      __syncthreads();
    }
    const double2 piv = ck[KK];
    const double2 alpha = crcp(piv);
    // the current column KK above the diagonal, then p_s and q_s
    for (int i = tid; i < KK; i += nt) {
      double2 v = a(i, KK);
      for (int t = 0; t < s; ++t) {
        cfma(v, P(i, t), Q(KK, t));
        cfma(v, cneg(Q(i, t)), P(KK, t));
      }
      ckk[i] = v;
    }
    __syncthreads();
    for (int i = tid; i < KK; i += nt) {
      P(i, s) = ck[i];
      Q(i, s) = cmul(alpha, ckk[i]);
    }
    if (tid == 0) {
      const double m = hypot(piv.x, piv.y);
      s_lm += log(m);
      s_ph = cmul(s_ph, make_double2(piv.x / m, piv.y / m));
    }
    __syncthreads();
  }
  // Y = [Q | -P]
  for (size_t idx = tid; idx < ldx * kPfNs; idx += nt) {
    Y[idx] = X[idx + ldx * kPfNs];
    Y[idx + ldx * kPfNs] = cneg(X[idx]);
  }
  if (tid == 0) {
    if (s_zero) {
      pf[b] = make_double2(-INFINITY, 0.0);
      pf[batch + b] = make_double2(0.0, 0.0);
      atomicOr(flags, DEV_PFAFF_ZERO);
    } else {
      pf[b] = make_double2(s_lm, 0.0);
      pf[batch + b] = s_ph;
    }
  }
}

}  // namespace

// blocked: the blocked form also where the packed triangle fits shared
// memory (its CTAs hold 22 KB instead of up to 227 KB, so that products of
// other streams share their SMs)
int pfaffian_batched(int n, int batch, double2* A, double2* pf, int* flags, cudaStream_t s, bool blocked) {
  if (n > 512 || (n & 1)) return TVAP_ERR_ARG;
  const size_t shm = sizeof(double2) * (size_t(n) * (n + 1) / 2 + 4 * size_t(n + 1) + size_t(n));
  if (shm <= jacobi32_smem_limit() && !(blocked && n >= 2)) {
    // the packed upper triangle fits shared memory: the unblocked elimination
    if (int rc = smem_opt_in((const void*)pfaffian_smem_kernel, jacobi32_smem_limit())) return rc;
    pfaffian_smem_kernel<<<batch, kPfThreads, shm, tvap::counted(s)>>>(n, A, pf, batch, flags);
    TVAP_CUDA(cudaGetLastError());
    return TVAP_OK;
  }
  if (n == 0) return TVAP_ERR_ARG;
  // blocked: panels of kPfNb columns, the trailing updates on the tensor cores
  const size_t xy = size_t(batch) * n * 2 * kPfNs;
  double2* XY = nullptr;
  TVAP_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&XY), sizeof(double2) * 2 * xy, s));
  double2 *X = XY, *Y = XY + xy;
  int rc = TVAP_OK;
  for (int Kstart = n - 1, first = 1; Kstart > 0 && rc == TVAP_OK; first = 0) {
    const int width = std::min(kPfNb, Kstart + 1);
    pf_panel_kernel<<<batch, kPfThreads, 0, tvap::counted(s)>>>(n, Kstart, width, A, X, Y, pf, batch, flags, first);
    if (cudaGetLastError() != cudaSuccess) {
      rc = TVAP_ERR_CUDA;
      break;
    }
    const int L = Kstart - width + 1;  // the leading block still to eliminate
    if (L > 1) {
      // A[0:L, 0:L] += X Y^T (upper triangle read later)
      GemmArgs g{};
      g.M = g.N = L;
      g.K = 2 * kPfNs;
      g.batch = batch;
      g.A = View{X, 1, n, (long long)n * 2 * kPfNs};
      g.B = View{Y, n, 1, (long long)n * 2 * kPfNs};  // B(k, j) = Y(j, k)
      g.C = A;
      g.crs = 1;
      g.ccs = n;
      g.cbs = (long long)n * n;
      g.alpha = make_double2(1.0, 0.0);
      g.beta = make_double2(1.0, 0.0);
      g.three_m = true;
      g.upper_only = true;
      rc = gemm(g, s);
    }
    Kstart = L - 1;
  }
  cudaFreeAsync(XY, s);
  if (rc == TVAP_ERR_CUDA) set_last_error("blocked Pfaffian launch failed", __FILE__, __LINE__);
  return rc;
}

// ---------------------------------------------------------------------------
// Symmetric eigen-decomposition by parallel cyclic Jacobi (round-robin pair
// ordering, n/2 disjoint rotations per round), one CTA, FP64.  A (n x n,
// column-major) is destroyed; W receives the eigenvectors as columns and
// evals the eigenvalues, both sorted ascending (the DSYEV convention).
// ---------------------------------------------------------------------------
namespace {

constexpr int kJacThreads = 1024;

template <typename T>
__global__ void __launch_bounds__(kJacThreads) jacobi_kernel(int n, T* A, T* W, double* evals, double* work,
                                                             int* flags, double tolfac, double relrot,
                                                             const double* __restrict__ scale) {
  extern __shared__ double jsh[];
  const int m = (n + 1) & ~1;  // even count incl. a dummy index
  double* cs = jsh;                                    // m/2 cosines
  double* sn = cs + m / 2;                             // m/2 sines
  int* pairs = reinterpret_cast<int*>(sn + m / 2);     // m round-robin slots
  int* pp = pairs + m;                                 // m/2 p indices
  int* qq = pp + m / 2;                                // m/2 q indices
  __shared__ double red[kJacThreads];
  __shared__ int done, nrot;
  const int tid = threadIdx.x, nt = blockDim.x;
  auto Ael = [A, n](int i, int j) -> T& { return A[i + size_t(j) * n]; };
  for (size_t idx = tid; idx < size_t(n) * n; idx += nt) W[idx] = ((idx % n) == (idx / n)) ? T(1) : T(0);
  for (int i = tid; i < m; i += nt) pairs[i] = i;
  double anorm = 0.0;
  for (size_t idx = tid; idx < size_t(n) * n; idx += nt) anorm += double(A[idx]) * double(A[idx]);
  red[tid] = anorm;
  __syncthreads();
  for (int s = nt / 2; s > 0; s >>= 1) {
    if (tid < s) red[tid] += red[tid + s];
    __syncthreads();
  }
  const double fro2 = red[0];
  __syncthreads();
  const double tol2 = fro2 * tolfac;  // converged when off-diagonal^2 <= tolfac ||A||_F^2
  // a block of a larger matrix (scale = that matrix's norm) needs no more
  // than the larger matrix's rounding level
  const double absrot = fmax(0.1 * relrot * sqrt(fro2), scale ? relrot * *scale : 0.0);
  const int kstep = nt / n;
  const int r0 = (tid < kstep * n) ? tid % n : n;
  const int k0 = (tid < kstep * n) ? tid / n : 0;
  int sweep = 0;
  for (sweep = 0; sweep < 60; ++sweep) {
    // off-diagonal norm
    double off = 0.0;
    for (size_t idx = tid; idx < size_t(n) * n; idx += nt) {
      const int i = int(idx % n), j = int(idx / n);
      if (i != j) off += double(A[idx]) * double(A[idx]);
    }
    red[tid] = off;
    __syncthreads();
    for (int s = nt / 2; s > 0; s >>= 1) {
      if (tid < s) red[tid] += red[tid + s];
      __syncthreads();
    }
    // converged: the off-diagonal norm is small, or the last sweep found no
    // entry above the rounding level of its diagonal pair (the off-diagonal
    // norm of a large matrix can stay above tol2 at that level)
    if (tid == 0) done = (red[0] <= tol2 || (sweep > 0 && nrot == 0)) ? 1 : 0;
    __syncthreads();
    if (done) break;
    if (tid == 0) nrot = 0;
    __syncthreads();
    for (int round = 0; round < m - 1; ++round) {
      // pairs (pairs[k], pairs[m-1-k]) for k < m/2
      for (int k = tid; k < m / 2; k += nt) {
        int p, q;
        if (k == 0) {
          p = round;
          q = m - 1;
        } else {
          p = (round + k) % (m - 1);
          q = (round - k + (m - 1)) % (m - 1);
        }
        if (p > q) {
          const int t = p;
          p = q;
          q = t;
        }
        T c = T(1), s = T(0);
        if (q < n) {
          const T apq = Ael(p, q);
          const T app = Ael(p, p), aqq = Ael(q, q);
          // rotate unless apq is at the rounding level of its pair, or below
          // a tenth of it for the whole matrix
          if (apq != T(0) && fabs(double(apq)) > fmax(relrot * sqrt(fabs(double(app) * double(aqq))), absrot)) {
            atomicAdd(&nrot, 1);
            const T theta = (aqq - app) / (T(2) * apq);
            const T t = (theta >= T(0) ? T(1) : T(-1)) / (fabs(theta) + sqrt(theta * theta + T(1)));
            c = T(1) / sqrt(t * t + T(1));
            s = t * c;
          }
        }
        pp[k] = p;
        qq[k] = q;
        cs[k] = c;
        sn[k] = s;
      }
      __syncthreads();
      // columns: A <- A J, W <- W J
      for (int k = k0; k < m / 2; k += kstep) {
        const int r = r0;
        const int p = pp[k], q = qq[k];
        if (r >= n || q >= n || sn[k] == 0.0) continue;
        const T c = T(cs[k]), s = T(sn[k]);
        const T ap = Ael(r, p), aq = Ael(r, q);
        Ael(r, p) = c * ap - s * aq;
        Ael(r, q) = s * ap + c * aq;
        const T wp = W[r + size_t(p) * n], wq = W[r + size_t(q) * n];
        W[r + size_t(p) * n] = c * wp - s * wq;
        W[r + size_t(q) * n] = s * wp + c * wq;
      }
      __syncthreads();
      // rows: A <- J^T A
      for (int k = k0; k < m / 2; k += kstep) {
        const int col = r0;
        const int p = pp[k], q = qq[k];
        if (col >= n || q >= n || sn[k] == 0.0) continue;
        const T c = T(cs[k]), s = T(sn[k]);
        const T ap = Ael(p, col), aq = Ael(q, col);
        Ael(p, col) = c * ap - s * aq;
        Ael(q, col) = s * ap + c * aq;
      }
      __syncthreads();
    }
  }
  if (sweep >= 60 && tid == 0) atomicOr(flags, DEV_EIGEN_NOCONV);
  // sort ascending (selection by rank; ties broken by index)
  for (int i = tid; i < n; i += nt) work[i] = double(Ael(i, i));
  __syncthreads();
  for (int i = tid; i < n; i += nt) {
    const double v = work[i];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const double u = work[j];
      rank += (u < v || (u == v && j < i)) ? 1 : 0;
    }
    evals[rank] = v;
    reinterpret_cast<int*>(work + n)[i] = rank;
  }
  __syncthreads();
  // permute eigenvector columns into A (as scratch) then copy back
  for (size_t idx = tid; idx < size_t(n) * n; idx += nt) {
    const int r = int(idx % n), j = int(idx / n);
    const int dst = reinterpret_cast<int*>(work + n)[j];
    A[r + size_t(dst) * n] = W[idx];
  }
  __syncthreads();
  for (size_t idx = tid; idx < size_t(n) * n; idx += nt) W[idx] = A[idx];
}

}  // namespace

int jacobi_eigen(int n, double* A, double* W, double* evals, double* work, int* flags, cudaStream_t s,
                 const double* scale) {
  const int m = (n + 1) & ~1;
  const size_t shm = sizeof(double) * m + sizeof(int) * 2 * m + 64;
  jacobi_kernel<double><<<1, kJacThreads, shm, tvap::counted(s)>>>(n, A, W, evals, work, flags, 1.0e-30, 1.0e-16,
                                                                    scale);
  TVAP_CUDA(cudaGetLastError());
  return TVAP_OK;
}

int jacobi_eigen_f32(int n, float* A, float* W, double* evals, double* work, int* flags, cudaStream_t s) {
  const int m = (n + 1) & ~1;
  const size_t shm = sizeof(double) * m + sizeof(int) * 2 * m + 64;
  jacobi_kernel<float><<<1, kJacThreads, shm, tvap::counted(s)>>>(n, A, W, evals, work, flags, 1.0e-13, 6.0e-8, nullptr);
  TVAP_CUDA(cudaGetLastError());
  return TVAP_OK;
}


// ---------------------------------------------------------------------------
// FP32 parallel cyclic Jacobi with the matrix and the rotations resident in
// shared memory (n <= 160): the cheap first stage of the canonical-basis
// eigensolver; the FP64 refinement that follows restores full accuracy.
// Writes the (unsorted) eigenvectors as FP64 columns of W.
// ---------------------------------------------------------------------------
namespace {

struct __align__(16) JRot {
  float c, s;
  int p, q;
};

__global__ void __launch_bounds__(1024) jacobi32_smem_kernel(int n, const double* __restrict__ A64,
                                                              const double* __restrict__ W0,
                                                              double* __restrict__ W64, int* sweeps_out) {
  extern __shared__ float js[];
  const int m = (n + 1) & ~1;
  const int h = m / 2;
  const int ld = n | 1;                  // odd leading dimension: conflict-free row access
  float* A = js;                         // n x ld
  float* W = A + size_t(n) * ld;         // n x ld
  JRot* rot = reinterpret_cast<JRot*>(W + size_t(n) * ld);  // 16-byte aligned: n is even
  __shared__ float red[1024];
  __shared__ int done;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  float fro = 0.f;
  for (int idx = tid; idx < n * n; idx += nt) {
    const int i = idx % n, j = idx / n;
    const float a = float(A64[idx]);
    A[i + j * ld] = a;
    W[i + j * ld] = W0 ? float(W0[idx]) : ((i == j) ? 1.f : 0.f);
    fro += a * a;
  }
  red[tid] = fro;
  __syncthreads();
  for (int s = nt / 2; s > 0; s >>= 1) {
    if (tid < s) red[tid] += red[tid + s];
    __syncthreads();
  }
  const float tol2 = red[0] * 1.0e-12f;  // off-diagonal <= 1e-6 ||A||: enough for the FP64 refinement
  // off-norm: thread -> (row, first column) with a fixed stride
  const int kstep = nt / n;
  const int r0 = (tid < kstep * n) ? tid % n : n;
  const int k0 = (tid < kstep * n) ? tid / n : 0;
  __syncthreads();
  int sweep = 0;
  for (; sweep < 40; ++sweep) {
    float off = 0.f;
    if (r0 < n)
      for (int j = k0; j < n; j += kstep)
        if (j != r0) off += A[r0 + j * ld] * A[r0 + j * ld];
    red[tid] = off;
    __syncthreads();
    for (int s = nt / 2; s > 0; s >>= 1) {
      if (tid < s) red[tid] += red[tid + s];
      __syncthreads();
    }
    if (tid == 0) done = (red[0] <= tol2) ? 1 : 0;
    __syncthreads();
    if (done) break;
    for (int round = 0; round < m - 1; ++round) {
      for (int k = tid; k < h; k += nt) {
        // circle method: player m-1 fixed, the others rotate with the round
        int p, q;
        if (k == 0) {
          p = round;
          q = m - 1;
        } else {
          p = (round + k) % (m - 1);
          q = (round - k + (m - 1)) % (m - 1);
        }
        if (p > q) {
          const int t = p;
          p = q;
          q = t;
        }
        float c = 1.f, s = 0.f;
        if (q < n) {
          const float apq = A[p + q * ld];
          if (apq != 0.f) {
            const float theta = (A[q + q * ld] - A[p + p * ld]) / (2.f * apq);
            const float t = (theta >= 0.f ? 1.f : -1.f) / (fabsf(theta) + sqrtf(theta * theta + 1.f));
            c = rsqrtf(t * t + 1.f);
            s = t * c;
          }
        } else {
          q = p;  // padding player: no rotation, keep the indices in range
        }
        rot[k] = JRot{c, s, p, q};
      }
      __syncthreads();
      // A <- J^T A J: warp w takes the row pairs w, w + nw, ..., its lanes the
      // column pairs lane, lane + 32, lane + 64; every 2 x 2 block is read and
      // written once.  W <- W J: warp per pair, lanes over rows.
      {
        JRot r2[3];
        int o2p[3], o2q[3];
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) {
          const int k2 = lane + 32 * jj;
          r2[jj] = (k2 < h) ? rot[k2] : JRot{1.f, 0.f, 0, 0};
          o2p[jj] = r2[jj].p * ld;
          o2q[jj] = r2[jj].q * ld;
        }
        for (int k1 = warp; k1 < h; k1 += nw) {
          const JRot r1 = rot[k1];
#pragma unroll
          for (int jj = 0; jj < 3; ++jj) {
            const int k2 = lane + 32 * jj;
            if (k2 >= h || (r1.s == 0.f && r2[jj].s == 0.f) || r1.p == r1.q || r2[jj].p == r2[jj].q) continue;
            const float c1 = r1.c, s1 = r1.s, c2 = r2[jj].c, s2 = r2[jj].s;
            float* a0 = A + r1.p;
            float* a1 = A + r1.q;
            const float a = a0[o2p[jj]], b = a0[o2q[jj]], cc = a1[o2p[jj]], d = a1[o2q[jj]];
            const float xa = c2 * a - s2 * b, xb = s2 * a + c2 * b;    // row p1 after the column rotation
            const float xc = c2 * cc - s2 * d, xd = s2 * cc + c2 * d;  // row q1
            a0[o2p[jj]] = c1 * xa - s1 * xc;
            a0[o2q[jj]] = c1 * xb - s1 * xd;
            a1[o2p[jj]] = s1 * xa + c1 * xc;
            a1[o2q[jj]] = s1 * xb + c1 * xd;
          }
        }
        for (int k = warp; k < h; k += nw) {
          const JRot r = rot[k];
          if (r.s == 0.f || r.p == r.q) continue;
          float* wp = W + r.p * ld;
          float* wq = W + r.q * ld;
          for (int row = lane; row < n; row += 32) {
            const float x = wp[row], y = wq[row];
            wp[row] = r.c * x - r.s * y;
            wq[row] = r.s * x + r.c * y;
          }
        }
      }
      __syncthreads();
    }
  }
  // no error flag here: the FP64 refinement's final check decides
  for (int idx = tid; idx < n * n; idx += nt) W64[idx] = double(W[(idx % n) + (idx / n) * ld]);
  if (tid == 0 && sweeps_out) *sweeps_out = sweep;
}

}  // namespace

size_t jacobi32_smem_bytes(int n) {
  const int m = (n + 1) & ~1;
  return sizeof(float) * (2 * size_t(n) * (n | 1) + 4) + 16 * size_t(m / 2) + 64;
}

// largest dynamic shared memory the FP32 Jacobi kernel may request on the
// current device (found once per device)
size_t jacobi32_smem_limit() {
  static std::mutex m;
  static std::vector<std::pair<int, size_t>> limits;  // (device, bytes)
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  std::lock_guard<std::mutex> lock(m);
  for (const auto& e : limits)
    if (e.first == dev) return e.second;
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncAttributes fa{};
  cudaFuncGetAttributes(&fa, jacobi32_smem_kernel);
  const size_t lim = (size_t(optin) > fa.sharedSizeBytes) ? size_t(optin) - fa.sharedSizeBytes : 0;
  size_t limit = 1;  // unusable: callers fall back to the FP64 solver
  if (cudaFuncSetAttribute(jacobi32_smem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(lim)) ==
      cudaSuccess)
    limit = lim;
  cudaGetLastError();
  limits.emplace_back(dev, limit);
  return limit;
}

int jacobi32_smem(int n, const double* A, const double* W0, double* W, int* sweeps_out, cudaStream_t s) {
  const size_t shm = jacobi32_smem_bytes(n);
  if (shm > jacobi32_smem_limit()) return TVAP_ERR_ARG;
  jacobi32_smem_kernel<<<1, 1024, shm, tvap::counted(s)>>>(n, A, W0, W, sweeps_out);
  TVAP_CUDA(cudaGetLastError());
  return TVAP_OK;
}

// ---------------------------------------------------------------------------
// Cholesky L L^T = A (lower, right-looking) followed by L^{-1} in place
// (DPBTRF + DTRTRI of cholesky_factorization / evolve_wavefunction,
// module_constraints.f90:497-590).  One CTA.
// ---------------------------------------------------------------------------
namespace {

__global__ void __launch_bounds__(1024) cholesky_inverse_kernel(int n, double* A, int* flags) {
  const int tid = threadIdx.x, nt = blockDim.x;
  auto a = [A, n](int i, int j) -> double& { return A[i + size_t(j) * n]; };
  __shared__ double dkk;
  __shared__ int bad;
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    if (tid == 0) {
      const double d = a(k, k);
      if (!(d > 0.0)) bad = 1;
      dkk = sqrt(fmax(d, 0.0));
      a(k, k) = dkk;
    }
    __syncthreads();
    if (bad) break;
    for (int i = k + 1 + tid; i < n; i += nt) a(i, k) = a(i, k) / dkk;
    __syncthreads();
    {
      const int warp = tid >> 5, lane = tid & 31, nw = nt >> 5;
      for (int j = k + 1 + warp; j < n; j += nw) {
        const double ljk = a(j, k);
        for (int i = j + lane; i < n; i += 32) a(i, j) = fma(-a(i, k), ljk, a(i, j));
      }
    }
    __syncthreads();
  }
  if (bad) {
    if (tid == 0) atomicOr(flags, DEV_CHOLESKY);
    return;
  }
  // zero the strict upper triangle
  for (int j = tid >> 5; j < n; j += nt >> 5)
    for (int i = tid & 31; i < j; i += 32) a(i, j) = 0.0;
  __syncthreads();
  // inverse of lower-triangular L, column by column from the right:
  // for j = n-1..0: L^{-1}(j,j) = 1/L(j,j); L^{-1}(i,j) = -(sum_{k=j+1..i} L^{-1}(i,k) L(k,j)) / L(j,j)
  // done in place with the standard DTRTI2-style update.
  for (int j = n - 1; j >= 0; --j) {
    __shared__ double ajj;
    if (tid == 0) {
      if (a(j, j) == 0.0) bad = 1;
      a(j, j) = 1.0 / a(j, j);
      ajj = -a(j, j);
    }
    __syncthreads();
    if (bad) break;
    // x = A(j+1:n, j); A(j+1:n, j) = T * x with T = A(j+1:n, j+1:n) (already inverted, lower)
    // computed row by row: y_i = sum_{k=j+1..i} T(i,k) x_k
    const int len = n - j - 1;
    for (int r = tid; r < len; r += nt) {
      const int i = j + 1 + r;
      double y = 0.0;
      for (int k = j + 1; k <= i; ++k) y = fma(a(i, k), a(k, j), y);
      A[size_t(n) * n + i] = y;  // scratch row after the matrix
    }
    __syncthreads();
    for (int r = tid; r < len; r += nt) {
      const int i = j + 1 + r;
      a(i, j) = A[size_t(n) * n + i] * ajj;
    }
    __syncthreads();
  }
  if (bad && tid == 0) atomicOr(flags, DEV_TRTRI);
}

}  // namespace

// A must have room for n*n + n doubles (scratch row).
// The same factorisation with the matrix in shared memory (n^2 doubles): the
// right-looking Cholesky with two barriers per column, then L^{-1} one
// column per thread (forward substitution L x = e_j, no barriers), x kept in
// the free upper triangle.
constexpr int kCholThreads = 512;
__global__ void __launch_bounds__(kCholThreads) cholesky_inverse_smem_kernel(int n, double* A, int* flags) {
  extern __shared__ double chol_smem[];  // n x n column-major, then dinv[n]
  double* Ls = chol_smem;
  double* dinv = Ls + size_t(n) * n;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  auto L = [Ls, n](int i, int j) -> double& { return Ls[i + size_t(j) * n]; };
  for (int idx = tid; idx < n * n; idx += nt) Ls[idx] = A[idx];
  __syncthreads();
  bool bad = false;
  for (int k = 0; k < n; ++k) {
    const double d = L(k, k);
    if (!(d > 0.0)) {
      bad = true;  // uniform: every thread read the same value
      break;
    }
    const double dk = sqrt(d);
    const double rdk = 1.0 / dk;  // the column is scaled by the reciprocal, as DPBTF2 does
    for (int i = k + 1 + tid; i < n; i += nt) L(i, k) = L(i, k) * rdk;
    __syncthreads();
    if (tid == 0) L(k, k) = dk;
    for (int j = k + 1 + warp; j < n; j += nw) {
      const double ljk = L(j, k);
      for (int i = j + lane; i < n; i += 32) L(i, j) = fma(-L(i, k), ljk, L(i, j));
    }
    __syncthreads();
  }
  if (bad) {
    if (tid == 0) atomicOr(flags, DEV_CHOLESKY);
    return;
  }
  for (int i = tid; i < n; i += nt) {
    if (L(i, i) == 0.0) atomicOr(flags, DEV_TRTRI);
    dinv[i] = 1.0 / L(i, i);
  }
  __syncthreads();
  // column j of L^{-1}: x_j = 1/L_jj, x_i = -(sum_{k=j..i-1} L_ik x_k) / L_ii,
  // x_i (i > j) stored at the upper-triangle position (j, i)
  for (int j = tid; j < n; j += nt) {
    const double xj = dinv[j];
    for (int i = j + 1; i < n; ++i) {
      double s0 = L(i, j) * xj, s1 = 0.0;
      int k = j + 1;
      for (; k + 1 < i; k += 2) {
        s0 = fma(L(i, k), L(j, k), s0);
        s1 = fma(L(i, k + 1), L(j, k + 1), s1);
      }
      if (k < i) s0 = fma(L(i, k), L(j, k), s0);
      L(j, i) = -(s0 + s1) * dinv[i];
    }
  }
  __syncthreads();
  for (int idx = tid; idx < n * n; idx += nt) {
    const int i = idx % n, j = idx / n;
    A[idx] = (i == j) ? dinv[j] : (i > j ? L(j, i) : 0.0);
  }
}

int cholesky_inverse(int n, double* A, int* flags, cudaStream_t s) {
  const size_t shm = sizeof(double) * (size_t(n) * n + n);
  if (shm <= jacobi32_smem_limit()) {
    if (int rc = smem_opt_in((const void*)cholesky_inverse_smem_kernel, jacobi32_smem_limit())) return rc;
    cholesky_inverse_smem_kernel<<<1, kCholThreads, shm, tvap::counted(s)>>>(n, A, flags);
  } else {
    cholesky_inverse_kernel<<<1, 1024, 0, tvap::counted(s)>>>(n, A, flags);
  }
  TVAP_CUDA(cudaGetLastError());
  return TVAP_OK;
}


// ---------------------------------------------------------------------------
// Cholesky factorisation of S (lower, L L^T = S; S has n x n + n doubles, the
// last n receive 1 / L_jj) and the evolution solves
// X L^T = A for two n x n matrices A (U1 = A1 L^{-T}, V1 = A2 L^{-T}) in one
// cooperative launch.  GB300's FP64 pipe gives one SM about 2 FMAs per clock,
// so the factorisation is spread over the grid: panels of kCoopNb columns; CTA
// 0 factors each diagonal block, all CTAs solve the panel rows below it and
// apply the trailing update (CTA 0 updating and factoring the next diagonal
// block meanwhile); then one warp per row of A1 / A2 runs the forward
// substitution L x = a with L in shared memory.  Grid-wide barriers between
// the phases are bounded spins (all CTAs are co-resident by the cooperative
// launch); a barrier that gives up raises the status word and every CTA
// returns.
// ---------------------------------------------------------------------------
namespace {

constexpr int kCoopThreads = 256;
constexpr int kCoopNb = 16;
constexpr long long kCoopSpin = 1LL << 22;

// bar[0] arrivals, bar[1] generation, bar[2] abort; zeroed before the launch
__device__ bool coop_barrier(unsigned* bar, unsigned nblocks, unsigned& gen, int* flags) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    __threadfence();
    if (atomicAdd(&bar[0], 1u) == nblocks - 1) {
      atomicExch(&bar[0], 0u);
      __threadfence();
      atomicExch(&bar[1], gen + 1);
    } else {
      volatile unsigned* g = &bar[1];
      long long it = 0;
      while (*g == gen) {
        if (++it > kCoopSpin || *(volatile unsigned*)&bar[2]) {
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    if (!ok || *(volatile unsigned*)&bar[2]) {
      if (!*(volatile unsigned*)&bar[2]) atomicOr(flags, DEV_WAIT_TIMEOUT);
      atomicExch(&bar[2], 1u);
      ok = 0;
    }
    __threadfence();
    ok_s = ok;
  }
  ++gen;
  __syncthreads();
  return ok_s != 0;
}

// 1 / sqrt(d) for a positive normal d: an FP32 seed (of d's value with the
// mantissa truncated to 23 bits) refined by two Newton-Raphson steps for the
// reciprocal square root, y <- y (3 - d y^2) / 2 (each step doubles the
// correct bits: 2^-22 -> 2^-44 -> FP64 rounding).  The range test, the seed's
// conversions and d / 2 (an exponent decrement) run on the integer pipe, so
// the 6 Newton instructions are all that occupy the FP64 pipe; outside the
// range of seed_range the library routines are used.
__device__ __forceinline__ double rsqrt_newton(double d) {
  if (!seed_range(d)) return 1.0 / sqrt(d);
  double y = seed_f64(rsqrtf(seed_f32(d)));
  const double h = __longlong_as_double(__double_as_longlong(d) - (1LL << 52));  // d / 2, exact
  y = y * fma(-h, y * y, 1.5);
  y = y * fma(-h, y * y, 1.5);
  return y;
}

// Unblocked Cholesky of the nb x nb diagonal block at (j0, j0) of S by the
// whole CTA (kCoopThreads >= kCoopNb^2 threads, one entry of the block each,
// the block in B): per step the pivot's thread forms 1 / sqrt(d), the column
// is scaled by it (as DPBTF2 does) and the trailing entries take
// A_ij -= L_ik L_jk, each entry in the same order as an unblocked
// elimination.  An FP64 warp instruction holds the FP64 unit of its SM
// sub-partition for about 64 cycles on this part: with the block's entries
// spread over all the CTA's warps, a step's update is one instruction on
// every sub-partition instead of up to 15 on one.  The reciprocals go to
// rd[j0 ..] for the solves; sc (2 doubles of shared memory) carries the
// pivot's reciprocal and the failure flag.  Elements written by other CTAs
// are read through L2.  Every thread of the CTA calls it; the result is
// uniform.
__device__ bool coop_factor_diag(int n, double* S, double* rd, int j0, int nb, double (*B)[kCoopNb + 1],
                                 double* sc) {
  static_assert(kCoopThreads >= kCoopNb * kCoopNb, "one thread per entry of the diagonal block");
  const int t = threadIdx.x;
  const int i = t % kCoopNb, j = t / kCoopNb;
  const bool mine = t < kCoopNb * kCoopNb && i < nb && j < nb && i >= j;
  if (mine) B[i][j] = __ldcg(&S[(j0 + i) + size_t(j0 + j) * n]);
  __syncthreads();
  for (int k = 0; k < nb; ++k) {
    if (t == k * kCoopNb + k) {  // the pivot's thread
      const double d = B[k][k];
      if (d > 0.0) {
        const double y = rsqrt_newton(d);
        B[k][k] = d * y;
        rd[j0 + k] = y;
        sc[0] = y;
        sc[1] = 0.0;
      } else {
        sc[1] = 1.0;
      }
    }
    __syncthreads();
    if (sc[1] != 0.0) return false;  // uniform: read by every thread after the barrier
    if (mine && j == k && i > k) B[i][k] *= sc[0];
    __syncthreads();
    if (mine && j > k) B[i][j] = fma(-B[i][k], B[j][k], B[i][j]);
    __syncthreads();
  }
  if (mine) S[(j0 + i) + size_t(j0 + j) * n] = B[i][j];
  return true;
}

template <int SLOTS>
__global__ void __launch_bounds__(kCoopThreads, 1) cholesky_evolve_kernel(int n, double* S, const double* A,
                                                                       long long a_stride, double* X,
                                                                       long long x_stride, unsigned* bar,
                                                                       int* flags, int skip_cta, int l_smem) {
  // the panel rows; then, in the solve phase, L (n x n, when l_smem) and 1 / L_jj
  extern __shared__ double coop_smem[];
  __shared__ double L11[kCoopNb][kCoopNb + 1];
  __shared__ double rdiag[kCoopNb];
  __shared__ unsigned gen_s;
  const int t = threadIdx.x, G = gridDim.x, cta = blockIdx.x;
  if (t == 0) gen_s = *(volatile unsigned*)&bar[1];
  __syncthreads();
  unsigned gen = gen_s;  // every thread keeps its own copy of the generation
  double* rd = S + size_t(n) * n;  // 1 / L_jj
  if (cta == 0 && !coop_factor_diag(n, S, rd, 0, min(kCoopNb, n), L11, rdiag) && t == 0) {
    atomicOr(flags, DEV_CHOLESKY);
    atomicExch(&bar[2], 1u);
  }
  // test hook: this CTA leaves without arriving, so that the others' bounded
  // waits at the first barrier run out (status DEV_WAIT_TIMEOUT, abort)
  if (cta == skip_cta) return;
  if (!coop_barrier(bar, G, gen, flags)) return;
  for (int j0 = 0;;) {
    const int j1 = min(j0 + kCoopNb, n);
    if (j1 >= n) break;
    const int nbp = j1 - j0, j2 = min(j1 + kCoopNb, n);
    // panel rows below the diagonal block: L21 = S21 L11^{-T}, one warp per
    // row (lane k holds x_k), rows spread over the CTAs so that their FP64
    // work runs on different SMs
    if (j1 + cta < n) {
      for (int idx = t; idx < nbp * nbp; idx += blockDim.x) {
        const int i = idx % nbp, j = idx / nbp;
        if (i >= j) L11[i][j] = __ldcg(&S[(j0 + i) + size_t(j0 + j) * n]);
      }
      if (t < nbp) rdiag[t] = __ldcg(&rd[j0 + t]);
      __syncthreads();
      const int warp = t >> 5, lane = t & 31, warps = blockDim.x >> 5;
      for (int i = j1 + cta + G * warp; i < n; i += G * warps) {
        double xk = (lane < nbp) ? __ldcg(&S[i + size_t(j0 + lane) * n]) : 0.0;
        for (int m = 0; m < nbp; ++m) {
          if (lane == m) xk *= rdiag[m];
          const double xm = __shfl_sync(0xffffffffu, xk, m);
          if (lane > m && lane < nbp) xk = fma(-xm, L11[lane][m], xk);
        }
        if (lane < nbp) S[i + size_t(j0 + lane) * n] = xk;
      }
    }
    if (!coop_barrier(bar, G, gen, flags)) return;
    // trailing update S22 -= L21 L21^T (lower triangle).  CTA 0 takes the
    // next diagonal block (rows and columns j1 .. j2-1) and factors it; the
    // other CTAs take the rest, one column at a time.  The panel rows j1..n-1
    // are staged in shared memory first (independent loads: one L2 round
    // trip instead of one per k).
    double* P = coop_smem;  // (n - j1) x nbp, row-major
    const int prow = n - j1;
    if (cta == 0 || cta - 1 < prow) {
#pragma unroll 4
      for (int idx = t; idx < prow * nbp; idx += blockDim.x) {
        const int k = idx / prow, i = idx - k * prow;
        P[i * kCoopNb + k] = __ldcg(&S[(j1 + i) + size_t(j0 + k) * n]);
      }
      __syncthreads();
    }
    if (cta == 0) {
      const int nb2 = j2 - j1;
      for (int idx = t; idx < nb2 * nb2; idx += blockDim.x) {
        const int i = idx % nb2, j = idx / nb2;
        if (i < j) continue;
        double v = __ldcg(&S[(j1 + i) + size_t(j1 + j) * n]);
        for (int k = 0; k < nbp; ++k) v = fma(-P[i * kCoopNb + k], P[j * kCoopNb + k], v);
        S[(j1 + i) + size_t(j1 + j) * n] = v;
      }
      __syncthreads();
      // (L11 and rdiag are free until the barrier: every CTA reloads them)
      if (!coop_factor_diag(n, S, rd, j1, nb2, L11, rdiag) && t == 0) {
        atomicOr(flags, DEV_CHOLESKY);
        atomicExch(&bar[2], 1u);
      }
    }
    if (cta > 0 || G == 1) {
      const int workers = G > 1 ? G - 1 : 1, w = G > 1 ? cta - 1 : 0;
      for (int j = j1 + w; j < n; j += workers) {
        const double* pj = P + (j - j1) * kCoopNb;
        const int i0 = (j < j2) ? j2 : j;
        for (int i = i0 + t; i < n; i += blockDim.x) {
          const double* pi = P + (i - j1) * kCoopNb;
          double v = __ldcg(&S[i + size_t(j) * n]);
          for (int k = 0; k < nbp; ++k) v = fma(-pi[k], pj[k], v);
          S[i + size_t(j) * n] = v;
        }
      }
    }
    if (!coop_barrier(bar, G, gen, flags)) return;
    j0 = j1;
  }
  // forward substitution L x = a for every row of A1 and A2: one warp per
  // row, rows spread over all CTAs
  const int warps = blockDim.x >> 5, warp = t >> 5, lane = t & 31;
  const int rows = 2 * n;
  if (cta >= rows) return;
  // L from shared memory when it fits (n <= 168), else from L2 (S is
  // written by this grid before the last barrier: read through L2, not L1)
  double* Ls = coop_smem;
  double* dinv = l_smem ? Ls + size_t(n) * n : coop_smem;
  if (l_smem) {
    if ((reinterpret_cast<uintptr_t>(S) & 15) == 0) {
      // 16-byte loads, many in flight
      const int nn2 = (n * n) / 2;
      const double2* S2 = reinterpret_cast<const double2*>(S);
      double2* L2 = reinterpret_cast<double2*>(Ls);
#pragma unroll 16
      for (int idx = t; idx < nn2; idx += blockDim.x) L2[idx] = __ldcg(&S2[idx]);
      if (((n * n) & 1) && t == 0) Ls[n * n - 1] = __ldcg(&S[n * n - 1]);
    } else {
#pragma unroll 16
      for (int idx = t; idx < n * n; idx += blockDim.x) Ls[idx] = __ldcg(&S[idx]);
    }
  }
  __syncthreads();
  for (int j = t; j < n; j += blockDim.x) dinv[j] = __ldcg(&rd[j]);
  __syncthreads();
  constexpr int kMaxPerLane = SLOTS;
  for (int r = cta + G * warp; r < rows; r += G * warps) {
    const int mat = r >= n ? 1 : 0, row = r - mat * n;
    const double* a = A + mat * a_stride;
    double* x = X + mat * x_stride;
    double v[kMaxPerLane];
#pragma unroll
    for (int q = 0; q < kMaxPerLane; ++q) {
      const int j = lane + 32 * q;
      v[q] = (j < n) ? a[row + size_t(j) * n] : 0.0;
    }
    // columns j in slot qj (a compile-time index once unrolled): the slots
    // below qj are finished, the slots above take every lane, slot qj the
    // lanes above j -- only those FMAs are issued (each an FP64 instruction
    // of about 64 cycles on this part), in the order of an unblocked solve
#pragma unroll
    for (int qj = 0; qj < kMaxPerLane; ++qj) {
      if (32 * qj >= n) break;
      const int jend = min(32 * qj + 32, n);
      for (int j = 32 * qj; j < jend; ++j) {
        const int owner = j & 31;
        const double xj = __shfl_sync(0xffffffffu, v[qj], owner) * dinv[j];
        if (lane == owner) v[qj] = xj;
        const double* lc = (l_smem ? Ls : S) + size_t(j) * n;
        {
          const int jj = lane + 32 * qj;
          if (jj > j && jj < n) v[qj] = fma(-xj, l_smem ? lc[jj] : __ldcg(&lc[jj]), v[qj]);
        }
#pragma unroll
        for (int q = qj + 1; q < kMaxPerLane; ++q) {
          if (32 * q >= n) break;
          const int jj = lane + 32 * q;
          if (jj < n) v[q] = fma(-xj, l_smem ? lc[jj] : __ldcg(&lc[jj]), v[q]);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < kMaxPerLane; ++q) {
      const int j = lane + 32 * q;
      if (j < n) x[row + size_t(j) * n] = v[q];
    }
  }
}

}  // namespace

int cholesky_evolve_coop(int n, double* S, const double* A, long long a_stride, double* X, long long x_stride,
                         unsigned* bar, int* flags, cudaStream_t s, int skip_cta) {
  // L in shared memory for the solves when it fits; else the panel rows
  // ((n - 1) x kCoopNb) and 1 / L_jj only, L read from L2
  const size_t shm_full = sizeof(double) * (size_t(n) * n + n);
  const int l_smem = shm_full <= jacobi32_smem_limit() ? 1 : 0;
  const size_t shm = l_smem ? shm_full : sizeof(double) * (size_t(n) * kCoopNb + n);
  if (n > 384 || shm > jacobi32_smem_limit()) return TVAP_ERR_ARG;
  const int slots = (n + 31) / 32;
  const void* kern = slots <= 2    ? (const void*)cholesky_evolve_kernel<2>
                     : slots <= 4  ? (const void*)cholesky_evolve_kernel<4>
                     : slots <= 5  ? (const void*)cholesky_evolve_kernel<5>
                     : slots <= 6  ? (const void*)cholesky_evolve_kernel<6>
                     : slots <= 8  ? (const void*)cholesky_evolve_kernel<8>
                     : slots <= 11 ? (const void*)cholesky_evolve_kernel<11>
                                   : (const void*)cholesky_evolve_kernel<12>;
  // the co-resident grid of this instantiation and shared-memory size, found
  // once per device
  struct GridKey {
    int dev;
    const void* kern;
    size_t shm;
  };
  static std::mutex m;
  static std::vector<std::pair<GridKey, int>> grids;
  int dev = 0;
  TVAP_CUDA(cudaGetDevice(&dev));
  int grid = 0;
  {
    std::lock_guard<std::mutex> lock(m);
    for (const auto& e : grids)
      if (e.first.dev == dev && e.first.kern == kern && e.first.shm == shm) grid = e.second;
    if (grid == 0) {
      if (int rc = smem_opt_in(kern, shm)) return rc;
      int per_sm = 0;
      TVAP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kCoopThreads, shm));
      grid = std::min(per_sm * device_sms(), 128);
      if (grid >= 1) grids.push_back({GridKey{dev, kern, shm}, grid});
    }
  }
  if (grid < 1) return TVAP_ERR_ARG;
  TVAP_CUDA(cudaMemsetAsync(bar, 0, 3 * sizeof(unsigned), s));
  // the hook names the grid's last CTA (never CTA 0, which factors the
  // diagonal blocks); -1 leaves every CTA in
  int skip = (skip_cta >= 0 && grid > 1) ? grid - 1 : -1;
  void* args[] = {&n, &S, &A, &a_stride, &X, &x_stride, &bar, &flags, &skip, const_cast<int*>(&l_smem)};
  ++g_launch_count;
  TVAP_CUDA(cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(kCoopThreads), args,
                                        shm, s));
  return TVAP_OK;
}

}  // namespace tvap
