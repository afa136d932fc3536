// adjust_constraints (module_constraints.f90:270-373) on the device: the
// Newton iteration that moves the Thouless step Z_i until the constraint
// expectation values of the evolved state reach their targets.
//
// Per iteration (at most 100, as in the reference):
//   (U1, V1) = evolve(U0, V0, Z_i)                      cholesky + evolve
//   rho = V1 V1^T, kappa = V1 U1^T                       calculate_densities_real
//   <C_m> = Tr(C_m rho) (one-body), Tr(C_m kappa^T) (pair)  calculate_expectval_*
//   C20_m = f20(C_m) or g20(C_m) at (U1, V1)             set_operator_qpbasis
//   stop when every |target_m - <C_m>| <= eps
//   A_ij = Tr(C20_i^T C20_j); A x = B; Z_i += sum_m x_m C20_m
// Everything but the c x c solve runs on the device; the expectation values
// and the Gram matrix come back in one read per iteration (fixed-order
// reductions, no atomics), the c-vector x goes down.

#include <cmath>
#include <vector>

#include "tvap_internal.cuh"

namespace tvap {

int upload_matrix(const void* src, void* dst, size_t bytes, cudaStream_t s);
int download_matrix(const void* src, void* dst, size_t bytes, cudaStream_t s);
int check_flags(tvap_ctx* c);
int real_product(int M, int N, int K, View A, View B, double* C, int ldc, double alpha, double beta,
                 cudaStream_t s);
int evolve_state(tvap_ctx* c, const double* U0, const double* V0, const double* Z, double* U1, double* V1,
                 double* work);

namespace {

constexpr int kDotThreads = 256;
constexpr int kDotBlocks = 64;

// partial[p * kDotBlocks + b] = sum over block b's share of x_p[i] y_p[i]
// (y_p read transposed when tr_p: the (i, j) entry of y is at j + i n)
struct DotJob {
  const double* x;
  const double* y;
  int tr;
};
__global__ void __launch_bounds__(kDotThreads) dot_partial_kernel(int n, const DotJob* __restrict__ jobs,
                                                               double* __restrict__ partial) {
  __shared__ double red[kDotThreads / 32];
  const DotJob J = jobs[blockIdx.y];
  const size_t nn = size_t(n) * n;
  double s = 0.0;
  for (size_t i = blockIdx.x * size_t(kDotThreads) + threadIdx.x; i < nn; i += size_t(kDotBlocks) * kDotThreads) {
    const size_t iy = J.tr ? (i / n) + (i % n) * size_t(n) : i;
    s = fma(J.x[i], J.y[iy], s);
  }
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kDotThreads / 32; ++w) t += red[w];
    partial[size_t(blockIdx.y) * kDotBlocks + blockIdx.x] = t;
  }
}

__global__ void dot_finish_kernel(int njobs, const double* __restrict__ partial, double* __restrict__ out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= njobs) return;
  double t = 0.0;
  for (int b = 0; b < kDotBlocks; ++b) t += partial[size_t(p) * kDotBlocks + b];
  out[p] = t;
}

// B = 1/2 (A1 - A1^T) with A1 = A2 - A3 (the '20' parts of
// set_operator_qpbasis, factor -1, module_operators.f90:49-97)
__global__ void part20_finish_kernel(int n, const double* __restrict__ A2, const double* __restrict__ A3,
                                     double* __restrict__ B) {
  const size_t idx = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (idx >= size_t(n) * n) return;
  const int i = int(idx % n), j = int(idx / n);
  const size_t ji = j + size_t(i) * n;
  B[idx] = 0.5 * ((A2[idx] - A3[idx]) - (A2[ji] - A3[ji]));
}

// Z += sum_m x_m C_m
__global__ void add_combination_kernel(size_t nn, int c, const double* __restrict__ x, const double* __restrict__ C,
                                       double* __restrict__ Z) {
  const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i >= nn) return;
  double s = Z[i];
  for (int m = 0; m < c; ++m) s = fma(x[m], C[size_t(m) * nn + i], s);
  Z[i] = s;
}

// A x = b for a small symmetric system (the reference's DSYSV): Gaussian
// elimination with partial pivoting; false for a singular A
bool small_solve(int c, std::vector<double> A, std::vector<double>& b) {
  for (int k = 0; k < c; ++k) {
    int p = k;
    for (int i = k + 1; i < c; ++i)
      if (std::fabs(A[i + k * c]) > std::fabs(A[p + k * c])) p = i;
    if (A[p + k * c] == 0.0) return false;
    if (p != k) {
      for (int j = 0; j < c; ++j) std::swap(A[k + j * c], A[p + j * c]);
      std::swap(b[k], b[p]);
    }
    for (int i = k + 1; i < c; ++i) {
      const double f = A[i + k * c] / A[k + k * c];
      for (int j = k; j < c; ++j) A[i + j * c] -= f * A[k + j * c];
      b[i] -= f * b[k];
    }
  }
  for (int k = c - 1; k >= 0; --k) {
    double s = b[k];
    for (int j = k + 1; j < c; ++j) s -= A[k + j * c] * b[j];
    b[k] = s / A[k + k * c];
  }
  return true;
}

}  // namespace

}  // namespace tvap

using namespace tvap;

extern "C" {

int tvap_adjust_constraints(tvap_ctx* c, const double* U0, const double* V0, double* Zi, int cdim, int cpair,
                            const double* constraint_HO, const double* values, double eps, double* U1, double* V1,
                            double* C20, int* iterations) {
  if (!c || !U0 || !V0 || !Zi || !U1 || !V1 || cdim < 0 || cpair < 0 || cpair > cdim ||
      (cdim > 0 && (!constraint_HO || !values)) || cdim > 64)
    return TVAP_ERR_ARG;
  LaunchTally tally(c);
  g_gemm_mode = c->gemm_mode;
  g_tc_bn_policy = c->tune_bn;
  g_tc_pairs_min_k = c->tune_pairs_k;
  g_dev_flags = c->d_flags;
  const int n = c->n;
  const size_t nn = size_t(n) * n;
  cudaStream_t s = c->stream;
  const int njobs = cdim + cdim * (cdim + 1) / 2;
  // U0, V0, Z, U1, V1 (adjacent), rho, kappa, T1, T2, T3, evolution work
  // (3 n^2 + n), the operators, C20, x, partial sums and results, the jobs
  double* buf = nullptr;
  const size_t jobs_doubles = (sizeof(DotJob) * size_t(njobs > 0 ? njobs : 1) + 7) / 8;
  const size_t tot = 13 * nn + n + 2 * size_t(cdim) * nn + cdim + size_t(njobs) * (kDotBlocks + 1) + jobs_doubles + 2;
  int rc;
  if ((rc = ctx_scratch(c, tot, &buf))) return rc;
  double *dU0 = buf, *dV0 = dU0 + nn, *dZ = dV0 + nn, *dU1 = dZ + nn, *dV1 = dU1 + nn, *rho = dV1 + nn,
         *kap = rho + nn, *T1 = kap + nn, *T2 = T1 + nn, *T3 = T2 + nn, *work = T3 + nn;
  double* cops = work + 3 * nn + n;
  double* c20 = cops + size_t(cdim) * nn;
  double* dx = c20 + size_t(cdim) * nn;
  double* partial = dx + cdim;
  double* results = partial + size_t(njobs) * kDotBlocks;
  DotJob* djobs = reinterpret_cast<DotJob*>(results + njobs + (njobs & 1));
  if ((rc = upload_matrix(U0, dU0, sizeof(double) * nn, s))) return rc;
  if ((rc = upload_matrix(V0, dV0, sizeof(double) * nn, s))) return rc;
  if ((rc = upload_matrix(Zi, dZ, sizeof(double) * nn, s))) return rc;
  if (cdim > 0 && (rc = upload_matrix(constraint_HO, cops, sizeof(double) * nn * cdim, s))) return rc;
  // the dot products of one iteration: the expectation values, then the
  // upper triangle of the Gram matrix of the C20
  std::vector<DotJob> jobs;
  for (int m = 0; m < cdim; ++m) {
    if (m < cdim - cpair)
      jobs.push_back({cops + m * nn, rho, 1});  // Tr(C rho) = sum C_ik rho_ki
    else
      jobs.push_back({cops + m * nn, kap, 0});  // Tr(C kappa^T) = sum C_ik kappa_ik
  }
  for (int i = 0; i < cdim; ++i)
    for (int j = i; j < cdim; ++j) jobs.push_back({c20 + i * nn, c20 + j * nn, 0});
  if (njobs > 0) TVAP_CUDA(cudaMemcpyAsync(djobs, jobs.data(), sizeof(DotJob) * njobs, cudaMemcpyHostToDevice, s));
  const View Uv = view_cm(dU1, n, 0), Vv = view_cm(dV1, n, 0);
  const int tb = 256;
  const unsigned nb = unsigned((nn + tb - 1) / tb);
  std::vector<double> res(njobs), x(cdim);
  int iter = 0;
  for (iter = 1; iter <= 100; ++iter) {
    if ((rc = evolve_state(c, dU0, dV0, dZ, dU1, dV1, work))) return rc;
    if (cdim == 0) break;
    if ((rc = real_product(n, n, n, Vv, view_t(Vv), rho, n, 1.0, 0.0, s))) return rc;
    if ((rc = real_product(n, n, n, Vv, view_t(Uv), kap, n, 1.0, 0.0, s))) return rc;
    for (int m = 0; m < cdim; ++m) {
      const View A = view_cm(cops + m * nn, n, 0);
      if (m < cdim - cpair) {
        // f20: U^T A V - V^T A^T U
        if ((rc = real_product(n, n, n, view_t(Uv), A, T1, n, 1.0, 0.0, s))) return rc;
        if ((rc = real_product(n, n, n, view_cm(T1, n, 0), Vv, T2, n, 1.0, 0.0, s))) return rc;
        if ((rc = real_product(n, n, n, view_t(Vv), view_t(A), T1, n, 1.0, 0.0, s))) return rc;
        if ((rc = real_product(n, n, n, view_cm(T1, n, 0), Uv, T3, n, 1.0, 0.0, s))) return rc;
      } else {
        // g20: U^T A U - V^T A V
        if ((rc = real_product(n, n, n, view_t(Uv), A, T1, n, 1.0, 0.0, s))) return rc;
        if ((rc = real_product(n, n, n, view_cm(T1, n, 0), Uv, T2, n, 1.0, 0.0, s))) return rc;
        if ((rc = real_product(n, n, n, view_t(Vv), A, T1, n, 1.0, 0.0, s))) return rc;
        if ((rc = real_product(n, n, n, view_cm(T1, n, 0), Vv, T3, n, 1.0, 0.0, s))) return rc;
      }
      part20_finish_kernel<<<nb, tb, 0, tvap::counted(s)>>>(n, T2, T3, c20 + m * nn);
    }
    dot_partial_kernel<<<dim3(kDotBlocks, njobs), kDotThreads, 0, tvap::counted(s)>>>(n, djobs, partial);
    dot_finish_kernel<<<(njobs + 127) / 128, 128, 0, tvap::counted(s)>>>(njobs, partial, results);
    TVAP_CUDA(cudaGetLastError());
    TVAP_CUDA(cudaMemcpyAsync(res.data(), results, sizeof(double) * njobs, cudaMemcpyDeviceToHost, s));
    TVAP_CUDA(cudaStreamSynchronize(s));
    std::vector<double> B(cdim);
    int ia = 0;
    for (int m = 0; m < cdim; ++m) {
      B[m] = values[m] - res[m];
      if (std::fabs(B[m]) > eps) ++ia;
    }
    if (ia == 0) break;
    std::vector<double> A(size_t(cdim) * cdim);
    int k = cdim;
    for (int i = 0; i < cdim; ++i)
      for (int j = i; j < cdim; ++j, ++k) A[i + j * cdim] = A[j + i * cdim] = res[k];
    if (!small_solve(cdim, A, B)) break;  // the reference's DSYSV leaves B as is on failure; stop adjusting
    x = B;
    TVAP_CUDA(cudaMemcpyAsync(dx, x.data(), sizeof(double) * cdim, cudaMemcpyHostToDevice, s));
    add_combination_kernel<<<nb, tb, 0, tvap::counted(s)>>>(nn, cdim, dx, c20, dZ);
    TVAP_CUDA(cudaGetLastError());
  }
  if (iter > 100) iter = 100;
  if ((rc = download_matrix(dU1, U1, sizeof(double) * nn, s))) return rc;
  if ((rc = download_matrix(dV1, V1, sizeof(double) * nn, s))) return rc;
  if ((rc = download_matrix(dZ, Zi, sizeof(double) * nn, s))) return rc;
  if (C20 && cdim > 0 && (rc = download_matrix(c20, C20, sizeof(double) * nn * cdim, s))) return rc;
  if (iterations) *iterations = iter;
  return check_flags(c);
}

}  // extern "C"
