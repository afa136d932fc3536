// Dense building blocks of the path exported on their own, with the calling
// conventions of the library routines the reference links for them:
//
//   tvap_zskpfa_batched  ZSKPFA('U', 'P', ...) of PFAPACK
//                        (subroutines_pfaffian.f:12-258), called by
//                        calculate_overlap (module_projection.f90:921)
//   tvap_zgemm/dgemm     ZGEMM / DGEMM of BLAS, called throughout
//                        module_projection.f90 and module_fields.f90, in the
//                        arithmetic the context uses for its own products
//                        (tvap_set_gemm_mode)
//
// plus the check of caller matrices for non-finite entries that
// tvap_project runs before it launches any kernel.

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "tvap_internal.cuh"

namespace tvap {

int upload_matrix(const void* src, void* dst, size_t bytes, cudaStream_t s);
int download_matrix(const void* src, void* dst, size_t bytes, cudaStream_t s);
bool is_device_pointer(const void* p);
int check_flags(tvap_ctx* c);

namespace {

__global__ void nonfinite_kernel(size_t count, const double* __restrict__ a, int* __restrict__ found) {
  int bad = 0;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < count; i += size_t(gridDim.x) * blockDim.x)
    bad |= !isfinite(a[i]);
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(found, 1);
}

int op_view(char t, const double* p, int ld, View* v, bool* conj) {
  *conj = false;
  switch (t) {
    case 'N': case 'n': *v = view_cm(p, ld, 0); return TVAP_OK;
    case 'T': case 't': *v = view_t(view_cm(p, ld, 0)); return TVAP_OK;
    case 'C': case 'c': *v = view_t(view_cm(p, ld, 0)); *conj = true; return TVAP_OK;
    default: return TVAP_ERR_ARG;
  }
}

// Shared body of tvap_zgemm / tvap_dgemm: C = alpha op(A) op(B) + beta C
// with column-major operands (host or device memory).
int gemm_abi(tvap_ctx* c, bool cplx, char transa, char transb, int m, int n, int k, const double* alpha,
             const double* A, int lda, const double* B, int ldb, const double* beta, double* C, int ldc) {
  if (!c || !alpha || !beta || m < 0 || n < 0 || k < 0 || ldc < (m > 1 ? m : 1)) return TVAP_ERR_ARG;
  const bool ta = !(transa == 'N' || transa == 'n'), tb = !(transb == 'N' || transb == 'n');
  const int arows = ta ? k : m, acols = ta ? m : k, brows = tb ? n : k, bcols = tb ? k : n;
  if (lda < (arows > 1 ? arows : 1) || ldb < (brows > 1 ? brows : 1)) return TVAP_ERR_ARG;
  if (m == 0 || n == 0) return TVAP_OK;
  if ((k > 0 && (!A || !B)) || !C) return TVAP_ERR_ARG;
  LaunchTally tally(c);
  g_gemm_mode = c->gemm_mode;
  g_tc_bn_policy = c->tune_bn;
  g_tc_pairs_min_k = c->tune_pairs_k;
  g_dev_flags = c->d_flags;
  cudaStream_t s = c->stream;
  const size_t w = cplx ? 2 : 1;  // doubles per element
  const size_t na = size_t(lda) * acols * w, nb = size_t(ldb) * bcols * w, nc = size_t(ldc) * n * w;
  double* buf = nullptr;
  int rc;
  if ((rc = ctx_scratch(c, na + nb + nc, &buf))) return rc;
  double *dA = buf, *dB = buf + na, *dC = buf + na + nb;
  if (k > 0) {
    if ((rc = upload_matrix(A, dA, sizeof(double) * na, s))) return rc;
    if ((rc = upload_matrix(B, dB, sizeof(double) * nb, s))) return rc;
  }
  const bool beta_zero = beta[0] == 0.0 && (!cplx || beta[1] == 0.0);
  if (!beta_zero) {
    if ((rc = upload_matrix(C, dC, sizeof(double) * nc, s))) return rc;
  } else {
    TVAP_CUDA(cudaMemsetAsync(dC, 0, sizeof(double) * nc, s));
  }
  if (k > 0) {
    GemmArgs g{};
    g.M = m;
    g.N = n;
    g.K = k;
    g.batch = 1;
    bool ca = false, cb = false;
    if (op_view(transa, dA, lda, &g.A, &ca) || op_view(transb, dB, ldb, &g.B, &cb)) return TVAP_ERR_ARG;
    g.conj_a = cplx && ca;
    g.conj_b = cplx && cb;
    g.C = dC;
    g.crs = 1;
    g.ccs = ldc;
    g.alpha = make_double2(alpha[0], cplx ? alpha[1] : 0.0);
    g.beta = make_double2(beta[0], cplx ? beta[1] : 0.0);
    g.a_real = g.b_real = g.c_real = !cplx;
    if ((rc = gemm(g, s))) return rc;
  } else if (!beta_zero) {
    // k = 0: C = beta C
    std::vector<double> h(nc);
    TVAP_CUDA(cudaMemcpyAsync(h.data(), dC, sizeof(double) * nc, cudaMemcpyDeviceToHost, s));
    TVAP_CUDA(cudaStreamSynchronize(s));
    for (size_t j = 0; j < size_t(n); ++j)
      for (size_t i = 0; i < size_t(m); ++i) {
        double* e = h.data() + (i + j * ldc) * w;
        if (cplx) {
          const double re = beta[0] * e[0] - beta[1] * e[1], im = beta[0] * e[1] + beta[1] * e[0];
          e[0] = re;
          e[1] = im;
        } else {
          e[0] *= beta[0];
        }
      }
    TVAP_CUDA(cudaMemcpyAsync(dC, h.data(), sizeof(double) * nc, cudaMemcpyHostToDevice, s));
  }
  if ((rc = download_matrix(dC, C, sizeof(double) * nc, s))) return rc;
  return check_flags(c);
}

}  // namespace

// Non-finite entries in `count` caller matrices of `elems` doubles each (host
// or device memory): TVAP_ERR_ARG with a message naming the argument.  Host
// matrices are scanned on the host; device ones by one kernel, read back with
// one synchronisation of the context's stream before anything else is
// launched (a NaN must not reach the pivot searches).
int check_finite(tvap_ctx* c, const double* const* ptrs, const char* const* names, int count, size_t elems) {
  std::vector<int> on_dev(count, 0);
  bool any_dev = false;
  for (int q = 0; q < count; ++q) {
    on_dev[q] = is_device_pointer(ptrs[q]) ? 1 : 0;
    any_dev |= on_dev[q] != 0;
    if (!on_dev[q]) {
      const double* p = ptrs[q];
      for (size_t i = 0; i < elems; ++i)
        if (!std::isfinite(p[i])) {
          set_last_error((std::string(names[q]) + " has a non-finite entry").c_str(), __FILE__, __LINE__);
          return TVAP_ERR_ARG;
        }
    }
  }
  if (!any_dev) return TVAP_OK;
  int* found = c->d_flags + 1;  // the word after the status word: free for this check
  TVAP_CUDA(cudaMemsetAsync(found, 0, sizeof(int) * count, c->stream));
  const int tb = 256;
  const int nb = int(std::min<size_t>((elems + tb - 1) / tb, size_t(4 * device_sms())));
  for (int q = 0; q < count; ++q)
    if (on_dev[q]) nonfinite_kernel<<<nb > 0 ? nb : 1, tb, 0, tvap::counted(c->stream)>>>(elems, ptrs[q], found + q);
  TVAP_CUDA(cudaGetLastError());
  std::vector<int> h(count, 0);
  TVAP_CUDA(cudaMemcpyAsync(h.data(), found, sizeof(int) * count, cudaMemcpyDeviceToHost, c->stream));
  TVAP_CUDA(cudaStreamSynchronize(c->stream));
  for (int q = 0; q < count; ++q)
    if (h[q]) {
      set_last_error((std::string(names[q]) + " has a non-finite entry").c_str(), __FILE__, __LINE__);
      return TVAP_ERR_ARG;
    }
  return TVAP_OK;
}

}  // namespace tvap

using namespace tvap;

extern "C" {

int tvap_zskpfa_batched(tvap_ctx* c, int batch, int64_t n, const double* A, double* pfaff) {
  if (!c || batch < 0 || n < 0 || n > 512 || (batch > 0 && (!A || !pfaff))) return TVAP_ERR_ARG;
  if (batch == 0) return TVAP_OK;
  if (n == 0 || (n & 1)) {
    // ZSKPFA's quick returns: Pf = 1 for N = 0, 0 for odd N (A not referenced)
    for (int b = 0; b < batch; ++b) {
      double v[2] = {n == 0 ? 1.0 : 0.0, 0.0};
      if (is_device_pointer(pfaff)) {
        TVAP_CUDA(cudaMemcpy(pfaff + 2 * b, v, sizeof(v), cudaMemcpyHostToDevice));
      } else {
        pfaff[2 * b] = v[0];
        pfaff[2 * b + 1] = v[1];
      }
    }
    return TVAP_OK;
  }
  LaunchTally tally(c);
  g_gemm_mode = c->gemm_mode;  // the blocked form (n > 164) updates with the context's products
  g_tc_bn_policy = c->tune_bn;
  g_tc_pairs_min_k = c->tune_pairs_k;
  g_dev_flags = c->d_flags;
  cudaStream_t s = c->stream;
  const size_t nn = size_t(n) * n;
  double* buf = nullptr;
  int rc;
  if ((rc = ctx_scratch(c, 2 * nn * batch + 4 * size_t(batch), &buf))) return rc;
  double2* dA = reinterpret_cast<double2*>(buf);
  double2* dpf = dA + nn * batch;  // (log|Pf|, 0) per matrix, then the unit phases
  if ((rc = upload_matrix(A, dA, sizeof(double2) * nn * batch, s))) return rc;
  if ((rc = pfaffian_batched(int(n), batch, dA, dpf, c->d_flags, s))) return rc;
  std::vector<double2> h(2 * size_t(batch));
  TVAP_CUDA(cudaMemcpyAsync(h.data(), dpf, sizeof(double2) * 2 * batch, cudaMemcpyDeviceToHost, s));
  if ((rc = check_flags(c))) return rc;
  std::vector<double> out(2 * size_t(batch));
  for (int b = 0; b < batch; ++b) {
    // a zero pivot (ZSKTRF's INFO > 0) gives Pf = 0, as ZSKPFA does
    const double lm = h[b].x;
    const double2 ph = h[batch + b];
    const double mag = std::isinf(lm) && lm < 0 ? 0.0 : std::exp(lm);
    out[2 * b] = mag * ph.x;
    out[2 * b + 1] = mag * ph.y;
  }
  if (is_device_pointer(pfaff)) {
    TVAP_CUDA(cudaMemcpy(pfaff, out.data(), sizeof(double) * out.size(), cudaMemcpyHostToDevice));
  } else {
    std::memcpy(pfaff, out.data(), sizeof(double) * out.size());
  }
  return TVAP_OK;
}

int tvap_zgemm(tvap_ctx* c, char transa, char transb, int m, int n, int k, const double* alpha, const double* A,
               int lda, const double* B, int ldb, const double* beta, double* C, int ldc) {
  return gemm_abi(c, true, transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

int tvap_dgemm(tvap_ctx* c, char transa, char transb, int m, int n, int k, const double* alpha, const double* A,
               int lda, const double* B, int ldb, const double* beta, double* C, int ldc) {
  if (transa == 'C' || transa == 'c') transa = 'T';
  if (transb == 'C' || transb == 'c') transb = 'T';
  return gemm_abi(c, false, transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

}  // extern "C"
