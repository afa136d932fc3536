// diagonalize_hsp_and_H11 with opt = 0 (module_gradient.f90:158-453): the
// spectra of h^RR and of the quasiparticle Hamiltonian H11 from which the
// gradient types 1 and 2 take their step sizes (calculate_gradient,
// module_gradient.f90:86-119).
//
//   fields of the real densities: calculate_fields_diag(rho^RR, kappa^RR)
//     (the general contraction with kappa^LR = kappa^RL = kappa; for M = 1 the
//     reference reads the projection's phi = 0 fields, equal to these up to
//     rounding because V_phi = V^T U + U^T V vanishes for a Bogoliubov state)
//   H11 = U^T h U - V^T h^T V + (U^T Delta V + (U^T Delta V)^T) factor_delta
//     (calculate_H11_real, module_fields.f90:327-354)
//   constraints: H11 -= f11(sum_m lambda_m C_m) over the non-pair ones (f11 is
//     linear; the reference's constraint_11 of a pair constraint stays zero),
//     h -= sum_m lambda_m C_m over all (module_gradient.f90:189-218)
//   spectra: DSYEV('U') of both (:297, :416; the upper triangles, mirrored
//     before the reduction).  GB300's FP64 pipe makes Jacobi
//     sweeps slow, so the eigenvalues come from an FP64 Householder
//     tridiagonalisation (one CTA per matrix, O(n^3) once) followed by Sturm
//     multisection on the tridiagonal matrix (one warp per eigenvalue, 32
//     points per round).  Both are backward stable: the eigenvalues agree with
//     DSYEV's to a few units of eps ||A||.

#include <cmath>

#include "tvap_internal.cuh"

namespace tvap {

int upload_matrix(const void* src, void* dst, size_t bytes, cudaStream_t s);
int download_matrix(const void* src, void* dst, size_t bytes, cudaStream_t s);
int check_flags(tvap_ctx* c);
int real_product(int M, int N, int K, View A, View B, double* C, int ldc, double alpha, double beta,
                 cudaStream_t s);

namespace {

constexpr int kTdThreads = 1024;
constexpr int kTdMaxN = 512;

__device__ double block_sum(double v, double* red) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    double s = (lane < int(blockDim.x >> 5)) ? red[lane] : 0.0;
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) red[32] = s;
  }
  __syncthreads();
  return red[32];
}

// Householder reduction of the symmetric matrices A_b (n x n, column-major,
// destroyed) to tridiagonal form: diagonal d_b[0..n-1], off-diagonal
// e_b[0..n-2].  Step k reflects x = A[k+1:n, k] onto alpha e_1 with
// H = 1 - tau v v^T and updates the trailing block A22 <- H A22 H =
// A22 - v w^T - w v^T with p = tau A22 v, w = p - (tau/2)(v^T p) v.  A
// non-finite entry sets bad[b].
__global__ void __launch_bounds__(kTdThreads) tridiag_kernel(int n, double* __restrict__ Aall, double* __restrict__ dall,
                                                          double* __restrict__ eall, int* __restrict__ bad) {
  __shared__ double v[kTdMaxN], w[kTdMaxN];
  __shared__ double red[33];
  const int b = blockIdx.x;
  double* A = Aall + size_t(b) * n * n;
  double* d = dall + size_t(b) * n;
  double* e = eall + size_t(b) * n;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  auto a = [A, n](int i, int j) -> double& { return A[i + size_t(j) * n]; };
  int nonfinite = 0;
  for (size_t idx = tid; idx < size_t(n) * n; idx += nt) nonfinite |= !isfinite(A[idx]);
  if (__syncthreads_or(nonfinite)) {
    if (tid == 0) bad[b] = 1;
    return;
  }
  for (int k = 0; k + 2 < n; ++k) {
    const int m = n - k - 1;  // length of x
    const double x0 = a(k + 1, k);
    double s = 0.0;
    for (int i = 1 + tid; i < m; i += nt) s = fma(a(k + 1 + i, k), a(k + 1 + i, k), s);
    const double sigma = block_sum(s, red);
    if (tid == 0) d[k] = a(k, k);
    if (sigma == 0.0) {
      if (tid == 0) e[k] = x0;
      __syncthreads();
      continue;
    }
    const double alpha = -copysign(sqrt(fma(x0, x0, sigma)), x0);
    const double v0 = x0 - alpha;
    const double tau = 2.0 / fma(v0, v0, sigma);
    for (int i = tid; i < m; i += nt) v[i] = (i == 0) ? v0 : a(k + 1 + i, k);
    __syncthreads();
    // p = tau A22 v: row i of A22 is column k+1+i (symmetry), one warp per row
    for (int i = warp; i < m; i += nw) {
      const double* col = A + size_t(k + 1 + i) * n + (k + 1);
      double acc = 0.0;
      for (int j = lane; j < m; j += 32) acc = fma(col[j], v[j], acc);
      for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
      if (lane == 0) w[i] = tau * acc;
    }
    __syncthreads();
    double vp = 0.0;
    for (int i = tid; i < m; i += nt) vp = fma(v[i], w[i], vp);
    const double K = 0.5 * tau * block_sum(vp, red);
    for (int i = tid; i < m; i += nt) w[i] = fma(-K, v[i], w[i]);
    __syncthreads();
    // A22 -= v w^T + w v^T (both triangles)
    for (int j = warp; j < m; j += nw) {
      const double vj = v[j], wj = w[j];
      double* col = A + size_t(k + 1 + j) * n + (k + 1);
      for (int i = lane; i < m; i += 32) col[i] = fma(-v[i], wj, fma(-w[i], vj, col[i]));
    }
    if (tid == 0) e[k] = alpha;
    __syncthreads();
  }
  if (tid == 0) {
    if (n >= 2) {
      d[n - 2] = a(n - 2, n - 2);
      e[n - 2] = a(n - 1, n - 2);
    }
    d[n - 1] = a(n - 1, n - 1);
  }
}

// number of eigenvalues of the tridiagonal (d, e) below x (Sturm sequence)
__device__ __forceinline__ int sturm_count(int n, const double* d, const double* e2, double x) {
  int c = 0;
  double q = d[0] - x;
  if (q < 0.0) ++c;
  for (int i = 1; i < n; ++i) {
    const double qq = (q == 0.0) ? 1.0e-300 : q;
    q = d[i] - x - e2[i - 1] / qq;
    if (q < 0.0) ++c;
  }
  return c;
}

// Eigenvalues of the tridiagonal matrices in ascending order, one warp per
// eigenvalue j: eigenvalue j lies in [lo, hi); each round the 32 lanes count
// at 32 interior points and the interval shrinks to the part that holds
// eigenvalue j (about 5 bits per round).
constexpr int kStThreads = 512;
__global__ void __launch_bounds__(kStThreads) sturm_kernel(int n, const double* __restrict__ dall,
                                                        const double* __restrict__ eall, double* __restrict__ wall) {
  extern __shared__ double st[];  // d[n], e^2[n]
  const int b = blockIdx.y;
  const double* dg = dall + size_t(b) * n;
  const double* eg = eall + size_t(b) * n;
  double* d = st;
  double* e2 = st + n;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < n; i += blockDim.x) {
    d[i] = dg[i];
    e2[i] = (i + 1 < n) ? eg[i] * eg[i] : 0.0;
  }
  __syncthreads();
  const int j = blockIdx.x * (kStThreads / 32) + warp;
  if (j >= n) return;  // whole warps
  // Gershgorin interval, widened
  double lo = 1.0e300, hi = -1.0e300, amax = 0.0;
  for (int i = 0; i < n; ++i) {
    const double r = ((i > 0) ? sqrt(e2[i - 1]) : 0.0) + ((i + 1 < n) ? sqrt(e2[i]) : 0.0);
    lo = fmin(lo, d[i] - r);
    hi = fmax(hi, d[i] + r);
    amax = fmax(amax, fabs(d[i]) + r);
  }
  const double pad = 2.0e-15 * amax + 1.0e-300;
  lo -= pad;
  hi += pad;
  for (int round = 0; round < 40; ++round) {
    if (hi - lo <= 4.0e-16 * fmax(fabs(lo), fabs(hi)) + 1.0e-300) break;
    const double x = lo + (hi - lo) * double(lane + 1) / 33.0;
    const int c = sturm_count(n, d, e2, x);
    // the first point with more than j eigenvalues below it (f is the same in
    // every lane, so the shuffles below run in all lanes or in none)
    const unsigned above = __ballot_sync(0xffffffffu, c > j);
    const int f = above ? __ffs(above) - 1 : 32;
    const double xl = (f == 0) ? lo : __shfl_sync(0xffffffffu, x, max(f - 1, 0));
    const double xh = (f == 32) ? hi : __shfl_sync(0xffffffffu, x, min(f, 31));
    lo = xl;
    hi = xh;
  }
  if (lane == 0) wall[size_t(b) * n + j] = 0.5 * (lo + hi);
}

__global__ void real_part_kernel(size_t nn, const double2* __restrict__ src, double* __restrict__ dst) {
  const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i < nn) dst[i] = src[i].x;
}

__global__ void to_complex_kernel(size_t nn, const double* __restrict__ src, double2* __restrict__ dst) {
  const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i < nn) dst[i] = make_double2(src[i], 0.0);
}

// H11 = A2 - A3 + (A4 + A4^T) fd, then H11 -= Q11 (the constraint term)
__global__ void h11_kernel(int n, const double* __restrict__ A2, const double* __restrict__ A3,
                           const double* __restrict__ A4, const double* __restrict__ Q11, double fd,
                           double* __restrict__ H11) {
  const size_t idx = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (idx >= size_t(n) * n) return;
  const int i = int(idx % n), j = int(idx / n);
  const size_t ji = j + size_t(i) * n;
  double v = A2[idx] - A3[idx] + (A4[idx] + A4[ji]) * fd;
  if (Q11) v -= Q11[idx];
  H11[idx] = v;
}

// C = sum_m lambda_m Cm over m in [m0, m1) (n^2 entries each), times sign;
// added to C when add, else written
__global__ void lincomb_kernel(size_t nn, int m0, int m1, const double* __restrict__ lam,
                               const double* __restrict__ ops, double* __restrict__ C, int add, double sign) {
  const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i >= nn) return;
  double s = 0.0;
  for (int m = m0; m < m1; ++m) s = fma(lam[m], ops[size_t(m) * nn + i], s);
  C[i] = (add ? C[i] : 0.0) + sign * s;
}

// the strict lower triangles of `batch` n x n matrices replaced by the upper
// ones: DSYEV('U', ...) reads only the upper triangle, and h - sum_m lambda_m
// C_m need not be symmetric (a pair operator in the sum)
__global__ void mirror_upper_kernel(int n, int batch, double* __restrict__ A) {
  const size_t nn = size_t(n) * n;
  const size_t idx = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (idx >= nn * batch) return;
  const size_t b = idx / nn, e = idx % nn;
  const int i = int(e % n), j = int(e / n);
  if (i > j) A[idx] = A[b * nn + j + size_t(i) * n];
}

// B = 1/2 (A1 + A1^T) with A1 = A2 - A3 (set_operator_qpbasis 'f11',
// module_operators.f90:49-97)
__global__ void f11_finish_kernel(int n, const double* __restrict__ A2, const double* __restrict__ A3,
                                  double* __restrict__ B) {
  const size_t idx = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (idx >= size_t(n) * n) return;
  const int i = int(idx % n), j = int(idx / n);
  const size_t ji = j + size_t(i) * n;
  B[idx] = 0.5 * ((A2[idx] - A3[idx]) + (A2[ji] - A3[ji]));
}

}  // namespace

// Eigenvalues (ascending) of `batch` symmetric n x n matrices A (destroyed)
// into W (batch x n); bad[b] = 1 for a matrix with a non-finite entry.
int symmetric_eigenvalues(int n, int batch, double* A, double* dtmp, double* etmp, double* W, int* bad,
                          cudaStream_t s) {
  if (n < 1 || n > kTdMaxN) return TVAP_ERR_ARG;
  tridiag_kernel<<<batch, kTdThreads, 0, tvap::counted(s)>>>(n, A, dtmp, etmp, bad);
  dim3 g((n + kStThreads / 32 - 1) / (kStThreads / 32), batch);
  sturm_kernel<<<g, kStThreads, 2 * sizeof(double) * n, tvap::counted(s)>>>(n, dtmp, etmp, W);
  TVAP_CUDA(cudaGetLastError());
  return TVAP_OK;
}

}  // namespace tvap

using namespace tvap;

extern "C" {

int tvap_diagonalize_hsp_and_H11(tvap_ctx* c, const double* U0, const double* V0, int cdim, int cpair,
                                 const double* lambda, const double* constraint_HO, double factor_delta,
                                 double* eigen_hsp, double* eigen_H11, int* info) {
  if (!c || !U0 || !V0 || !eigen_hsp || !eigen_H11 || !info || cdim < 0 || cpair < 0 || cpair > cdim ||
      (cdim > 0 && (!lambda || !constraint_HO)))
    return TVAP_ERR_ARG;
  if (!c->have_ham) return TVAP_ERR_NOT_READY;
  const int n = c->n;
  if (n > kTdMaxN) return TVAP_ERR_ARG;
  LaunchTally tally(c);
  g_gemm_mode = c->gemm_mode;
  g_tc_bn_policy = c->tune_bn;
  g_tc_pairs_min_k = c->tune_pairs_k;
  g_dev_flags = c->d_flags;
  const size_t nn = size_t(n) * n;
  cudaStream_t s = c->stream;
  const int tb = 256;
  const unsigned nb = unsigned((nn + tb - 1) / tb);
  // 6 complex n^2 (rho, kappa, gamma, h, Delta^LR, Delta^RL) first (the
  // buffer's start is aligned for double2); U, V, rho, kappa, h, Delta,
  // A1..A4, Q (real n^2 each); two matrices for the spectra (h, H11); the
  // constraint operators and multipliers; d, e, W, bad
  double* buf = nullptr;
  const size_t tot = 12 * nn + 11 * nn + 2 * nn + size_t(cdim) * nn + cdim + 6 * size_t(n) + 2;
  int rc;
  if ((rc = ctx_scratch(c, tot, &buf))) return rc;
  double2* zc = reinterpret_cast<double2*>(buf);
  double2 *zrho = zc, *zkap = zc + nn, *zgam = zc + 2 * nn, *zh = zc + 3 * nn, *zdl = zc + 4 * nn, *zdr = zc + 5 * nn;
  double* U = reinterpret_cast<double*>(zc + 6 * nn);
  double *V = U + nn, *rho = V + nn, *kap = rho + nn, *h = kap + nn, *D = h + nn, *A1 = D + nn, *A2 = A1 + nn,
         *A3 = A2 + nn, *A4 = A3 + nn, *Q = A4 + nn;
  double* M2 = Q + nn;  // [h | H11] for the spectra
  double* cops = M2 + 2 * nn;
  double* lam = cops + size_t(cdim) * nn;
  double* dt = lam + cdim;
  double* et = dt + 2 * size_t(n);
  double* W = et + 2 * size_t(n);
  int* bad = reinterpret_cast<int*>(W + 2 * size_t(n));
  if ((rc = upload_matrix(U0, U, sizeof(double) * nn, s))) return rc;
  if ((rc = upload_matrix(V0, V, sizeof(double) * nn, s))) return rc;
  if (cdim > 0) {
    if ((rc = upload_matrix(constraint_HO, cops, sizeof(double) * nn * cdim, s))) return rc;
    if ((rc = upload_matrix(lambda, lam, sizeof(double) * cdim, s))) return rc;
  }
  TVAP_CUDA(cudaMemsetAsync(bad, 0, 2 * sizeof(int), s));
  const View Uv = view_cm(U, n, 0), Vv = view_cm(V, n, 0);
  // rho = V V^T, kappa = V U^T (calculate_densities_real)
  if ((rc = real_product(n, n, n, Vv, view_t(Vv), rho, n, 1.0, 0.0, s))) return rc;
  if ((rc = real_product(n, n, n, Vv, view_t(Uv), kap, n, 1.0, 0.0, s))) return rc;
  to_complex_kernel<<<nb, tb, 0, tvap::counted(s)>>>(nn, rho, zrho);
  to_complex_kernel<<<nb, tb, 0, tvap::counted(s)>>>(nn, kap, zkap);
  // the fields of the real densities (one column: the gather kernels)
  if ((rc = fields_batched(c, 1, 1, zrho, zkap, zkap, zgam, zh, zdl, zdr, s))) return rc;
  real_part_kernel<<<nb, tb, 0, tvap::counted(s)>>>(nn, zh, h);
  real_part_kernel<<<nb, tb, 0, tvap::counted(s)>>>(nn, zdr, D);
  // H11 = U^T h U - V^T h^T V + (U^T D V + (U^T D V)^T) fd
  if ((rc = real_product(n, n, n, view_t(Uv), view_cm(h, n, 0), A1, n, 1.0, 0.0, s))) return rc;
  if ((rc = real_product(n, n, n, view_cm(A1, n, 0), Uv, A2, n, 1.0, 0.0, s))) return rc;
  if ((rc = real_product(n, n, n, view_t(Vv), view_t(view_cm(h, n, 0)), A1, n, 1.0, 0.0, s))) return rc;
  if ((rc = real_product(n, n, n, view_cm(A1, n, 0), Vv, A3, n, 1.0, 0.0, s))) return rc;
  if ((rc = real_product(n, n, n, view_t(Uv), view_cm(D, n, 0), A1, n, 1.0, 0.0, s))) return rc;
  if ((rc = real_product(n, n, n, view_cm(A1, n, 0), Vv, A4, n, 1.0, 0.0, s))) return rc;
  const int cnp = cdim - cpair;
  double* Q11 = nullptr;
  if (cnp > 0) {
    // f11 of C = sum over the non-pair constraints of lambda_m C_m
    lincomb_kernel<<<nb, tb, 0, tvap::counted(s)>>>(nn, 0, cnp, lam, cops, Q, 0, 1.0);
    double* B2 = M2;  // free until the spectra
    double* B3 = M2 + nn;
    if ((rc = real_product(n, n, n, view_t(Uv), view_cm(Q, n, 0), A1, n, 1.0, 0.0, s))) return rc;
    if ((rc = real_product(n, n, n, view_cm(A1, n, 0), Uv, B2, n, 1.0, 0.0, s))) return rc;
    if ((rc = real_product(n, n, n, view_t(Vv), view_t(view_cm(Q, n, 0)), A1, n, 1.0, 0.0, s))) return rc;
    if ((rc = real_product(n, n, n, view_cm(A1, n, 0), Vv, B3, n, 1.0, 0.0, s))) return rc;
    f11_finish_kernel<<<nb, tb, 0, tvap::counted(s)>>>(n, B2, B3, Q);
    Q11 = Q;
  }
  // the two matrices of the spectra: h - sum_m lambda_m C_m, H11 - Q11
  TVAP_CUDA(cudaMemcpyAsync(M2, h, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s));
  if (cdim > 0) lincomb_kernel<<<nb, tb, 0, tvap::counted(s)>>>(nn, 0, cdim, lam, cops, M2, 1, -1.0);
  h11_kernel<<<nb, tb, 0, tvap::counted(s)>>>(n, A2, A3, A4, Q11, factor_delta, M2 + nn);
  mirror_upper_kernel<<<(2 * nb), tb, 0, tvap::counted(s)>>>(n, 2, M2);
  TVAP_CUDA(cudaGetLastError());
  if ((rc = symmetric_eigenvalues(n, 2, M2, dt, et, W, bad, s))) return rc;
  if ((rc = download_matrix(W, eigen_hsp, sizeof(double) * n, s))) return rc;
  if ((rc = download_matrix(W + n, eigen_H11, sizeof(double) * n, s))) return rc;
  int hb[2] = {0, 0};
  TVAP_CUDA(cudaMemcpyAsync(hb, bad, sizeof(hb), cudaMemcpyDeviceToHost, s));
  if ((rc = check_flags(c))) return rc;
  info[0] = hb[0];
  info[1] = hb[1];
  return TVAP_OK;
}

int tvap_gradient_parameters(int gradient_type, int n, const double* eigen_hsp, const double* eigen_H11,
                             const int* info, double eta_in, double mu_in, double* eta, double* mu) {
  if (!eta || !mu || n < 1 || gradient_type < 0 || gradient_type > 2) return TVAP_ERR_ARG;
  int opt = gradient_type;
  if (opt == 1 && (!eigen_H11 || (info && info[1] != 0))) opt = 0;
  if (opt == 2 && (!eigen_hsp || (info && info[0] != 0))) opt = 0;
  *eta = eta_in;
  *mu = mu_in;
  if (opt == 0) return TVAP_OK;
  const double* e = (opt == 1) ? eigen_H11 : eigen_hsp;
  double amax = 0.0, amin = 1.0e300;
  for (int i = 0; i < n; ++i) {
    amax = std::fmax(amax, std::fabs(e[i]));
    amin = std::fmin(amin, std::fabs(e[i]));
  }
  const double emax = (opt == 1 ? 4.0 : 2.0) * amax, emin = 2.0 * amin;
  const double cond = emax / emin;
  const double t = 2.0 / (std::sqrt(emax) + std::sqrt(emin));
  const double r = (std::sqrt(cond) - 1.0) / (std::sqrt(cond) + 1.0);
  *eta = t * t;
  *mu = r * r;
  return TVAP_OK;
}

}  // extern "C"
