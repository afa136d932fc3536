// Gradient step, Thouless evolution and the adjoint of the projected energy.
//
//   calculate_gradient (module_gradient.f90:79-143), gradient_type 0
//   cholesky_factorization + evolve_wavefunction (module_constraints.f90:497-590)
//   dE/dZ for E(Z) = projected energy of evolve(U0, V0, Z): with
//     L L^T = 1 + Z^T Z and Phi1 = evolve(U0, V0, Z), a change dZ moves Phi1
//     by the Thouless matrix L^{-1} dZ L^{-T} in Phi1's quasiparticle basis,
//     and the gradient there is field_H20v(Phi1) (the projected H20 of
//     calculate_projected_H20).  Hence dE/dZ = L^{-T} H20v(Phi1) L^{-1}.
//     The per-angle densities are recomputed by the projection at Phi1.

#include <cmath>

#include "tvap_internal.cuh"

namespace tvap {

int upload_matrix(const void* src, void* dst, size_t bytes, cudaStream_t s);
int download_matrix(const void* src, void* dst, size_t bytes, cudaStream_t s);
int project_device(tvap_ctx* c, const tvap_proj_opts& o, tvap_pnp* out, bool sync = true);
int ensure_workspace(tvap_ctx* c, int G);
int angle_count(const tvap_proj_opts& o);
int check_flags(tvap_ctx* c);
bool is_device_pointer_on(const void* p, int device);

namespace {

__global__ void gradient_kernel(size_t nn, int cdim, const double* __restrict__ H20v,
                                const double* __restrict__ lambda, const double* __restrict__ C20,
                                const double* __restrict__ Zim1, double eta, double mu, double* __restrict__ Zi,
                                double* __restrict__ partial) {
  __shared__ double red[256];
  const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  double z2 = 0.0;
  if (i < nn) {
    double sg = 0.0;
    for (int j = 0; j < cdim; ++j) sg += lambda[j] * C20[size_t(j) * nn + i];
    const double z = -eta * (H20v[i] - sg) + mu * Zim1[i];
    Zi[i] = z;
    z2 = z * z;
  }
  red[threadIdx.x] = z2;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void sum_partials_kernel(int m, const double* __restrict__ partial, double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < m; ++i) s += partial[i];
    out[0] = s;
  }
}

__global__ void add_identity_kernel(int n, double* A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) A[i + size_t(i) * n] += 1.0;
}

int rgemm(int M, int N, int K, View A, View B, double* C, int ldc, double alpha, double beta, cudaStream_t s) {
  GemmArgs g{};
  g.M = M;
  g.N = N;
  g.K = K;
  g.batch = 1;
  g.A = A;
  g.B = B;
  g.C = C;
  g.crs = 1;
  g.ccs = ldc;
  g.alpha = make_double2(alpha, 0.0);
  g.beta = make_double2(beta, 0.0);
  g.a_real = g.b_real = g.c_real = true;
  return gemm(g, s);
}

struct EvolveBuf {
  double *Z = nullptr, *L = nullptr, *A1 = nullptr, *A2 = nullptr, *U0 = nullptr, *V0 = nullptr;
};

// U1 = (U0 + V0 Z) L^{-T}, V1 = (V0 + U0 Z) L^{-T} with L L^T = 1 + Z^T Z.
// With want_linv, L^{-1} is left in b.L (cholesky_inverse and two products);
// otherwise one cooperative launch factorises and solves when n allows it.
int evolve_device(tvap_ctx* c, EvolveBuf& b, int n, double* U1, double* V1, bool want_linv) {
  cudaStream_t s = c->stream;
  const size_t nn = size_t(n) * n;
  int rc;
  const View Zv = view_cm(b.Z, n, 0);
  sec_begin(c, SEC_EVOLVE);
  if ((rc = rgemm(n, n, n, view_t(Zv), Zv, b.L, n, 1.0, 0.0, s))) return rc;
  add_identity_kernel<<<(n + 255) / 256, 256, 0, tvap::counted(s)>>>(n, b.L);
  TVAP_CUDA(cudaMemcpyAsync(b.A1, b.U0, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s));
  TVAP_CUDA(cudaMemcpyAsync(b.A2, b.V0, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s));
  const bool coop = !want_linv && c->d_bar;
  if (!coop && (rc = cholesky_inverse(n, b.L, c->d_flags, s))) return rc;
  const View LinvT = view_t(view_cm(b.L, n, 0));
  // A1 = U0 + V0 Z, A2 = V0 + U0 Z as one batch of two when A2 follows A1
  // (then U1 = A1 L^-T, V1 = A2 L^-T likewise when V1 follows U1)
  const bool pair_a = (b.A2 == b.A1 + nn);
  const bool pair_u = pair_a && (V1 == U1 + nn);
  if (pair_a) {
    GemmArgs g{};
    g.M = g.N = g.K = n;
    g.batch = 2;
    g.A = View{b.V0, 1, n, (long long)(b.U0 - b.V0)};
    g.B = View{b.Z, 1, n, 0};
    g.C = b.A1;
    g.crs = 1;
    g.ccs = n;
    g.cbs = (long long)nn;
    g.alpha = make_double2(1.0, 0.0);
    g.beta = make_double2(1.0, 0.0);
    g.a_real = g.b_real = g.c_real = true;
    if ((rc = gemm(g, s))) return rc;
  } else {
    if ((rc = rgemm(n, n, n, view_cm(b.V0, n, 0), Zv, b.A1, n, 1.0, 1.0, s))) return rc;
    if ((rc = rgemm(n, n, n, view_cm(b.U0, n, 0), Zv, b.A2, n, 1.0, 1.0, s))) return rc;
  }
  if (coop) {
    const int skip = c->test_skip_arrival ? 1 : -1;
    c->test_skip_arrival = false;
    rc = cholesky_evolve_coop(n, b.L, b.A1, (long long)(b.A2 - b.A1), U1, (long long)(V1 - U1), c->d_bar,
                              c->d_flags, s, skip);
    if (rc == TVAP_OK) {
      sec_end(c, SEC_EVOLVE);
      return TVAP_OK;
    }
    if (rc != TVAP_ERR_ARG) return rc;
    if ((rc = cholesky_inverse(n, b.L, c->d_flags, s))) return rc;
  }
  if (pair_u) {
    GemmArgs g{};
    g.M = g.N = g.K = n;
    g.batch = 2;
    g.A = View{b.A1, 1, n, (long long)nn};
    g.B = View{LinvT.p, LinvT.rs, LinvT.cs, 0};
    g.C = U1;
    g.crs = 1;
    g.ccs = n;
    g.cbs = (long long)nn;
    g.alpha = make_double2(1.0, 0.0);
    g.beta = make_double2(0.0, 0.0);
    g.a_real = g.b_real = g.c_real = true;
    if ((rc = gemm(g, s))) return rc;
  } else {
    if ((rc = rgemm(n, n, n, view_cm(b.A1, n, 0), LinvT, U1, n, 1.0, 0.0, s))) return rc;
    if ((rc = rgemm(n, n, n, view_cm(b.A2, n, 0), LinvT, V1, n, 1.0, 0.0, s))) return rc;
  }
  sec_end(c, SEC_EVOLVE);
  return TVAP_OK;
}

}  // namespace

// The Thouless evolution of a device state for the other translation units:
// U1 = (U0 + V0 Z) L^-T, V1 = (V0 + U0 Z) L^-T, every matrix on the device;
// work holds 3 n^2 + n doubles.  Runs on the context's stream in the calling
// thread's arithmetic.
int evolve_state(tvap_ctx* c, const double* U0, const double* V0, const double* Z, double* U1, double* V1,
                 double* work) {
  const int n = c->n;
  const size_t nn = size_t(n) * n;
  EvolveBuf b;
  b.Z = const_cast<double*>(Z);
  b.U0 = const_cast<double*>(U0);
  b.V0 = const_cast<double*>(V0);
  b.A1 = work;
  b.A2 = work + nn;
  b.L = work + 2 * nn;
  return evolve_device(c, b, n, U1, V1, false);
}

double* ws_U(tvap_ctx* c);
double* ws_V(tvap_ctx* c);
double* ws_H20v(tvap_ctx* c);
double2* ws_sums(tvap_ctx* c);
int sync_with_flags(tvap_ctx* c, void* dst, const void* src, size_t bytes);
int check_finite(tvap_ctx* c, const double* const* ptrs, const char* const* names, int count, size_t elems);

// ---------------------------------------------------------------------------
// Scratch of tvap_evolve_noalloc: a file-scope device array, so that the
// entry point never allocates.  Layout for a basis of n states:
// L (n*n + n: the Cholesky factor and its scratch row), A1 (n*n), A2 (n*n).
// Every GPU that loads this library holds the array until the process exits.
// ---------------------------------------------------------------------------
constexpr int kNoallocMaxN = 336;
constexpr size_t kNoallocScratchDoubles = 3 * size_t(kNoallocMaxN) * kNoallocMaxN + kNoallocMaxN;
static __device__ __align__(256) double g_noalloc_scratch[kNoallocScratchDoubles];

namespace {

constexpr int kMaxDevices = 64;
double* g_noalloc_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device, looked up once
// per device with that device current (the host-side symbol is only a
// stand-in, not a device address).
int noalloc_scratch(double** out) {
  int dev = 0;
  TVAP_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_last_error("tvap_evolve_noalloc: device ordinal out of range", __FILE__, __LINE__);
    return TVAP_ERR_ARG;
  }
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    TVAP_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return TVAP_OK;
}

}  // namespace

}  // namespace tvap

using namespace tvap;

extern "C" {

int tvap_calculate_gradient(tvap_ctx* c, const double* H20v, int cdim, const double* lambda, const double* C20,
                            const double* Zim1, double eta, double mu, double* Zi, double* gradient_norm) {
  if (!c || !H20v || !Zim1 || !Zi || !gradient_norm || cdim < 0 || (cdim > 0 && (!lambda || !C20)) || eta == 0.0)
    return TVAP_ERR_ARG;
  LaunchTally tally(c);
  const int n = c->n;
  const size_t nn = size_t(n) * n;
  cudaStream_t s = c->stream;
  const int tb = 256;
  const int nblocks = int((nn + tb - 1) / tb);
  double* buf = nullptr;
  const size_t tot = nn * (3 + size_t(cdim)) + cdim + nblocks + 1;
  if (int r0 = ctx_scratch(c, tot, &buf)) return r0;
  double *dH = buf, *dZm = buf + nn, *dZ = buf + 2 * nn, *dC = buf + 3 * nn, *dl = dC + nn * cdim,
         *part = dl + cdim, *sum = part + nblocks;
  int rc = upload_matrix(H20v, dH, sizeof(double) * nn, s);
  if (!rc) rc = upload_matrix(Zim1, dZm, sizeof(double) * nn, s);
  if (!rc && cdim > 0) rc = upload_matrix(C20, dC, sizeof(double) * nn * cdim, s);
  if (!rc && cdim > 0) rc = upload_matrix(lambda, dl, sizeof(double) * cdim, s);
  if (!rc) {
    sec_begin(c, SEC_GRADIENT);
    gradient_kernel<<<nblocks, tb, 0, tvap::counted(s)>>>(nn, cdim, dH, dl, dC, dZm, eta, mu, dZ, part);
    sum_partials_kernel<<<1, 32, 0, tvap::counted(s)>>>(nblocks, part, sum);
    sec_end(c, SEC_GRADIENT);
    double h = 0.0;
    rc = download_matrix(dZ, Zi, sizeof(double) * nn, s);
    if (!rc) {
      cudaMemcpyAsync(&h, sum, sizeof(double), cudaMemcpyDeviceToHost, s);
      if (cudaStreamSynchronize(s) != cudaSuccess) rc = TVAP_ERR_CUDA;
      *gradient_norm = std::sqrt(h) / eta;
    }
  }
  return rc;
}

int tvap_evolve(tvap_ctx* c, const double* U0, const double* V0, const double* Z, double* U1, double* V1) {
  if (!c || !U0 || !V0 || !Z || !U1 || !V1) return TVAP_ERR_ARG;
  LaunchTally tally(c);
  g_gemm_mode = c->gemm_mode;
  g_tc_bn_policy = c->tune_bn;
  g_tc_pairs_min_k = c->tune_pairs_k;
  g_dev_flags = c->d_flags;
  const int n = c->n;
  const size_t nn = size_t(n) * n;
  cudaStream_t s = c->stream;
  double* buf = nullptr;
  if (int r0 = ctx_scratch(c, 8 * nn + n, &buf)) return r0;
  EvolveBuf b;
  b.Z = buf;
  b.U0 = buf + nn;
  b.V0 = buf + 2 * nn;
  b.A1 = buf + 3 * nn;
  b.A2 = buf + 4 * nn;
  double* dU1 = buf + 5 * nn;
  double* dV1 = buf + 6 * nn;
  b.L = buf + 7 * nn;  // n*n + n (scratch row)
  int rc = upload_matrix(Z, b.Z, sizeof(double) * nn, s);
  if (!rc) rc = upload_matrix(U0, b.U0, sizeof(double) * nn, s);
  if (!rc) rc = upload_matrix(V0, b.V0, sizeof(double) * nn, s);
  if (!rc) rc = evolve_device(c, b, n, dU1, dV1, false);
  if (!rc) rc = download_matrix(dU1, U1, sizeof(double) * nn, s);
  if (!rc) rc = download_matrix(dV1, V1, sizeof(double) * nn, s);
  if (!rc) rc = check_flags(c);
  return rc;
}

int tvap_iterate(tvap_ctx* c, const double* U0, const double* V0, const tvap_proj_opts* opts, double eta, double mu,
                 const double* Zim1, double* Zi, double* U1, double* V1, tvap_pnp* out, double* H20v,
                 double* gradient_norm) {
  if (!c || !U0 || !V0 || !opts || !Zim1 || !Zi || !U1 || !V1 || !out || !gradient_norm || eta == 0.0 ||
      opts->Mphip < 1 || opts->Mphin < 1)
    return TVAP_ERR_ARG;
  if (!c->have_ham) return TVAP_ERR_NOT_READY;
  LaunchTally tally(c);
  g_gemm_mode = c->gemm_mode;
  g_tc_bn_policy = c->tune_bn;
  g_tc_pairs_min_k = c->tune_pairs_k;
  g_dev_flags = c->d_flags;
  const int n = c->n;
  const size_t nn = size_t(n) * n;
  cudaStream_t s = c->stream;
  int rc;
  if ((rc = ensure_workspace(c, angle_count(*opts)))) return rc;
  {
    const double* mats[2] = {U0, V0};
    const char* names[2] = {"U0", "V0"};
    if ((rc = check_finite(c, mats, names, 2, nn))) return rc;
  }
  const int tb = 256;
  const int nblocks = int((nn + tb - 1) / tb);
  double* buf = nullptr;
  // Z_{i-1}, Z_i, A1, A2, U1, V1 (adjacent pairs), L (n^2 + n), partial sums
  if ((rc = ctx_scratch(c, 7 * nn + n + nblocks, &buf))) return rc;
  double *dZm = buf, *dZ = buf + nn, *dU1 = buf + 4 * nn, *dV1 = buf + 5 * nn, *part = buf + 7 * nn + n;
  if ((rc = upload_matrix(U0, ws_U(c), sizeof(double) * nn, s))) return rc;
  if ((rc = upload_matrix(V0, ws_V(c), sizeof(double) * nn, s))) return rc;
  if ((rc = upload_matrix(Zim1, dZm, sizeof(double) * nn, s))) return rc;
  // project_wavefunction + calculate_projected_H20, without the final wait
  if ((rc = project_device(c, *opts, out, false))) return rc;
  // calculate_gradient (type 0, no constraints): Z_i = -eta H20v + mu Z_{i-1};
  // |Z_i|^2 into the first free slot after the projected sums
  double* norm2 = reinterpret_cast<double*>(ws_sums(c) + 6);
  sec_begin(c, SEC_GRADIENT);
  gradient_kernel<<<nblocks, tb, 0, tvap::counted(s)>>>(nn, 0, ws_H20v(c), nullptr, nullptr, dZm, eta, mu, dZ, part);
  sum_partials_kernel<<<1, 32, 0, tvap::counted(s)>>>(nblocks, part, norm2);
  TVAP_CUDA(cudaGetLastError());
  sec_end(c, SEC_GRADIENT);
  // cholesky_factorization + evolve_wavefunction of the projected state
  EvolveBuf b;
  b.Z = dZ;
  b.U0 = ws_U(c);
  b.V0 = ws_V(c);
  b.A1 = buf + 2 * nn;
  b.A2 = buf + 3 * nn;
  b.L = buf + 6 * nn;
  if ((rc = evolve_device(c, b, n, dU1, dV1, false))) return rc;
  if ((rc = download_matrix(dZ, Zi, sizeof(double) * nn, s))) return rc;
  if ((rc = download_matrix(dU1, U1, sizeof(double) * nn, s))) return rc;
  if ((rc = download_matrix(dV1, V1, sizeof(double) * nn, s))) return rc;
  if (H20v && (rc = download_matrix(ws_H20v(c), H20v, sizeof(double) * nn, s))) return rc;
  // one round trip: the sums, |Z_i|^2 and the status word
  double2 sc[7];
  rc = sync_with_flags(c, sc, ws_sums(c), sizeof(sc));
  double* dst[6] = {out->over, out->ener, out->prot, out->neut, out->prot2, out->neut2};
  for (int q = 0; q < 6; ++q) {
    dst[q][0] = sc[q].x;
    dst[q][1] = sc[q].y;
  }
  *gradient_norm = std::sqrt(sc[6].x) / eta;
  return rc;
}

int tvap_test_wait_timeout(tvap_ctx* c) {
  if (!c) return TVAP_ERR_ARG;
  c->test_skip_arrival = true;
  return TVAP_OK;
}

int tvap_evolve_noalloc(tvap_ctx* c, const double* U0, const double* V0, const double* Z, double* U1, double* V1) {
  if (!c || !U0 || !V0 || !Z || !U1 || !V1) return TVAP_ERR_ARG;
  const int n = c->n;
  if (n > kNoallocMaxN) {
    set_last_error("tvap_evolve_noalloc: basis larger than the static scratch (n > 336)", __FILE__, __LINE__);
    return TVAP_ERR_ARG;
  }
  int dev = 0;
  TVAP_CUDA(cudaGetDevice(&dev));
  if (dev != c->device) {
    set_last_error("tvap_evolve_noalloc: the context's device must be current", __FILE__, __LINE__);
    return TVAP_ERR_ARG;
  }
  const int d = c->device;
  if (!is_device_pointer_on(U0, d) || !is_device_pointer_on(V0, d) || !is_device_pointer_on(Z, d) ||
      !is_device_pointer_on(U1, d) || !is_device_pointer_on(V1, d)) {
    set_last_error("tvap_evolve_noalloc: all matrices must be device memory of the context's device", __FILE__,
                   __LINE__);
    return TVAP_ERR_ARG;
  }
  double* scratch = nullptr;
  int rc;
  if ((rc = noalloc_scratch(&scratch))) return rc;
  LaunchTally tally(c);
  const size_t nn = size_t(n) * n;
  cudaStream_t s = c->stream;
  double* L = scratch;               // n*n + n
  double* A1 = scratch + nn + n;     // n*n
  double* A2 = A1 + nn;              // n*n
  // dense products on the FP64 pipe: the emulated GEMM would need slice buffers
  const int saved_mode = g_gemm_mode;
  g_gemm_mode = 0;
  const View Zv = view_cm(Z, n, 0);
  rc = rgemm(n, n, n, view_t(Zv), Zv, L, n, 1.0, 0.0, s);  // Z^T Z (every entry written)
  if (!rc) {
    add_identity_kernel<<<(n + 255) / 256, 256, 0, tvap::counted(s)>>>(n, L);
    rc = cholesky_inverse(n, L, c->d_flags, s);
  }
  if (!rc) {
    const cudaError_t e1 = cudaMemcpyAsync(A1, U0, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s);
    const cudaError_t e2 = cudaMemcpyAsync(A2, V0, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s);
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
      set_last_error(cudaGetErrorString(e1 != cudaSuccess ? e1 : e2), __FILE__, __LINE__);
      rc = TVAP_ERR_CUDA;
    }
  }
  if (!rc) rc = rgemm(n, n, n, view_cm(V0, n, 0), Zv, A1, n, 1.0, 1.0, s);
  if (!rc) rc = rgemm(n, n, n, view_cm(U0, n, 0), Zv, A2, n, 1.0, 1.0, s);
  const View LinvT = view_t(view_cm(L, n, 0));
  if (!rc) rc = rgemm(n, n, n, view_cm(A1, n, 0), LinvT, U1, n, 1.0, 0.0, s);
  if (!rc) rc = rgemm(n, n, n, view_cm(A2, n, 0), LinvT, V1, n, 1.0, 0.0, s);
  g_gemm_mode = saved_mode;
  if (rc) return rc;
  return check_flags(c);
}

int tvap_energy_adjoint(tvap_ctx* c, const double* U0, const double* V0, const double* Z,
                        const tvap_proj_opts* opts, double* energy, double* dEdZ) {
  if (!c || !U0 || !V0 || !Z || !opts || !energy || !dEdZ) return TVAP_ERR_ARG;
  if (!c->have_ham) return TVAP_ERR_NOT_READY;
  const int n = c->n;
  const size_t nn = size_t(n) * n;
  cudaStream_t s = c->stream;
  int rc;
  if ((rc = ensure_workspace(c, angle_count(*opts)))) return rc;
  LaunchTally tally(c);
  g_gemm_mode = c->gemm_mode;
  g_tc_bn_policy = c->tune_bn;
  g_tc_pairs_min_k = c->tune_pairs_k;
  g_dev_flags = c->d_flags;
  double* buf = nullptr;
  if ((rc = ctx_scratch(c, 7 * nn + n, &buf))) return rc;
  EvolveBuf b;
  b.Z = buf;
  b.U0 = buf + nn;
  b.V0 = buf + 2 * nn;
  b.A1 = buf + 3 * nn;
  b.A2 = buf + 4 * nn;
  double* G = buf + 5 * nn;
  b.L = buf + 6 * nn;
  rc = upload_matrix(Z, b.Z, sizeof(double) * nn, s);
  if (!rc) rc = upload_matrix(U0, b.U0, sizeof(double) * nn, s);
  if (!rc) rc = upload_matrix(V0, b.V0, sizeof(double) * nn, s);
  if (!rc) rc = evolve_device(c, b, n, ws_U(c), ws_V(c), true);
  if (!rc) rc = check_flags(c);
  tvap_pnp p{};
  if (!rc) rc = project_device(c, *opts, &p);
  if (!rc) {
    // dE/dZ = L^{-T} H20v L^{-1}
    const View Li = view_cm(b.L, n, 0);
    rc = rgemm(n, n, n, view_cm(ws_H20v(c), n, 0), Li, G, n, 1.0, 0.0, s);
    if (!rc) rc = rgemm(n, n, n, view_t(Li), view_cm(G, n, 0), b.A1, n, 1.0, 0.0, s);
    if (!rc) rc = download_matrix(b.A1, dEdZ, sizeof(double) * nn, s);
    if (!rc) {
      if (cudaStreamSynchronize(s) != cudaSuccess) rc = TVAP_ERR_CUDA;
      const double ore = p.over[0], oim = p.over[1], ere = p.ener[0], eim = p.ener[1];
      const double d = ore * ore + oim * oim;
      *energy = (ere * ore + eim * oim) / d;
    }
  }
  return rc;
}

}  // extern "C"
