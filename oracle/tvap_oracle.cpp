// ORACLE -- test infrastructure only.
//
// A CPU restatement of the TAURUS_vap PNVAP gradient path, used as the checker
// of the device implementation and as the timed CPU baseline.  It is loaded
// only by tests/, __graft_entry__.smoke() and bench.py's CPU legs; the product
// never links it.  Each routine follows the reference subroutine named in its
// comment (paths relative to the reference project's src/).
//
// Dense linear algebra goes through the BLAS/LAPACK routines the reference
// calls (ZGEMM, DGEMM, ZGETRF, ZGETRI, DSYEV, DGEES, DPBTRF, DTRTRI, DSYSV).
// Their addresses are handed in at run time by oracle.py, which takes them from
// SciPy's bundled BLAS/LAPACK (scipy.linalg.cython_blas / cython_lapack).  The
// vendored PFAPACK Pfaffian (subroutines_pfaffian.f) is restated here.
//
// Parity pin: tests/test_oracle_golden.py runs the Mg24 / USDB examples of the
// reference (examples/gradient_mg24) and compares the iteration counts and the
// converged projected energies with the reference's stored tables, and reaches
// the HFB minimum of its USDB minima table (examples/minima_usdb) from random
// seeds.

#include <omp.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

typedef std::complex<double> cplx;

// ---------------------------------------------------------------------------
// BLAS / LAPACK entry points (Fortran calling convention via SciPy wrappers)
// ---------------------------------------------------------------------------
typedef void (*zgemm_t)(char*, char*, int*, int*, int*, cplx*, cplx*, int*, cplx*, int*, cplx*, cplx*, int*);
typedef void (*dgemm_t)(char*, char*, int*, int*, int*, double*, double*, int*, double*, int*, double*, double*,
                        int*);
typedef void (*zgetrf_t)(int*, int*, cplx*, int*, int*, int*);
typedef void (*zgetri_t)(int*, cplx*, int*, int*, cplx*, int*, int*);
typedef void (*dsyev_t)(char*, char*, int*, double*, int*, double*, double*, int*, int*);
typedef int (*dselect2_t)(double*, double*);
typedef void (*dgees_t)(char*, char*, dselect2_t, int*, double*, int*, int*, double*, double*, double*, int*,
                        double*, int*, int*, int*);
typedef void (*dpbtrf_t)(char*, int*, int*, double*, int*, int*);
typedef void (*dtrtri_t)(char*, char*, int*, double*, int*, int*);
typedef void (*dsysv_t)(char*, int*, int*, double*, int*, int*, double*, int*, double*, int*, int*);

static zgemm_t p_zgemm;
static dgemm_t p_dgemm;
static zgetrf_t p_zgetrf;
static zgetri_t p_zgetri;
static dsyev_t p_dsyev;
static dgees_t p_dgees;
static dpbtrf_t p_dpbtrf;
static dtrtri_t p_dtrtri;
static dsysv_t p_dsysv;

static void zgemm(char ta, char tb, int m, int n, int k, cplx alpha, const cplx* A, int lda, const cplx* B, int ldb,
                  cplx beta, cplx* C, int ldc) {
  p_zgemm(&ta, &tb, &m, &n, &k, &alpha, const_cast<cplx*>(A), &lda, const_cast<cplx*>(B), &ldb, &beta, C, &ldc);
}
static void dgemm(char ta, char tb, int m, int n, int k, double alpha, const double* A, int lda, const double* B,
                  int ldb, double beta, double* C, int ldc) {
  p_dgemm(&ta, &tb, &m, &n, &k, &alpha, const_cast<double*>(A), &lda, const_cast<double*>(B), &ldb, &beta, C, &ldc);
}
static int lapack_sel(double*, double*) { return 0; }

namespace {

const cplx zone(1.0, 0.0), zzero(0.0, 0.0), zimag(0.0, 1.0);
constexpr double kPi = 3.14159265358979323846;

inline double dsign(double a, double b) { return std::copysign(std::fabs(a), b); }
inline int ipow_m1(long long e) { return (e & 1) ? -1 : 1; }

struct Mat {  // column-major complex n x n helper
  std::vector<cplx> v;
  int n = 0;
  Mat() {}
  explicit Mat(int n_) : v(size_t(n_) * n_, zzero), n(n_) {}
  cplx& operator()(int i, int j) { return v[size_t(i) + size_t(j) * n]; }
  const cplx& operator()(int i, int j) const { return v[size_t(i) + size_t(j) * n]; }
  cplx* p() { return v.data(); }
  const cplx* p() const { return v.data(); }
};

}  // namespace

// ---------------------------------------------------------------------------
// Model: the module-global arrays read by the hot path
// (module_hamiltonian.f90:53-58, module_basis.f90:33-41)
// ---------------------------------------------------------------------------
struct orc_model {
  int n = 0;
  std::vector<int> sp_2mj, sp_tr, sp_l;
  long long S = 0;
  std::vector<int16_t> abcd;
  std::vector<float> h2;
  std::vector<int8_t> trperm;
  Mat H1;
  cplx H0;
};

// find_timerev (module_hamiltonian.f90:1028-1089); indices 1-based.
static inline void find_timerev(const orc_model* m, int p, int& a, int& b, int& c, int& d) {
  const int ta = m->sp_tr[a - 1], tb = m->sp_tr[b - 1], tc = m->sp_tr[c - 1], td = m->sp_tr[d - 1];
  switch (p) {
    case -8: case 0: a = ta; b = tb; c = tc; d = td; break;
    case -7: case 1: a = tb; b = ta; c = tc; d = td; break;
    case -6: case 2: a = ta; b = tb; c = td; d = tc; break;
    case -5: case 3: a = tb; b = ta; c = td; d = tc; break;
    case -4: case 4: a = tc; b = td; c = ta; d = tb; break;
    case -3: case 5: a = tc; b = td; c = tb; d = ta; break;
    case -2: case 6: a = td; b = tc; c = ta; d = tb; break;
    case -1: case 7: a = td; b = tc; c = tb; d = ta; break;
    default: break;
  }
}

// calculate_fields (module_fields.f90:99-189): OpenMP over elements with
// thread-private full-matrix accumulators reduced at the end (the reference's
// FIRSTPRIVATE/REDUCTION(+:) pattern).
static void calculate_fields(const orc_model* m, const cplx* rho, const cplx* kLR, const cplx* kRL, cplx* gamma,
                             cplx* hsp, cplx* dLR, cplx* dRL, int nthreads) {
  const int n = m->n;
  const size_t nn = size_t(n) * n;
  std::fill(gamma, gamma + nn, zzero);
  std::fill(dLR, dLR + nn, zzero);
  std::fill(dRL, dRL + nn, zzero);
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
  {
    std::vector<cplx> g(nn, zzero), dl(nn, zzero), dr(nn, zzero);
    auto IX = [n](int i, int j) { return size_t(i - 1) + size_t(j - 1) * n; };
#pragma omp for schedule(static)
    for (long long kk = 0; kk < m->S; ++kk) {
      int ia = m->abcd[4 * kk], ib = m->abcd[4 * kk + 1], ic = m->abcd[4 * kk + 2], id = m->abcd[4 * kk + 3];
      double h2b = double(m->h2[kk]);
      const int perm = m->trperm[kk];
      for (int it = 1; it <= 2; ++it) {
        if (it == 2) {
          if (m->sp_2mj[ia - 1] + m->sp_2mj[ib - 1] == 0) continue;
          find_timerev(m, perm, ia, ib, ic, id);
          h2b = (perm < 0 ? -1.0 : 1.0) * h2b;
        }
        const double f2b = h2b * (1 - ((ia == ic) ? 1 : 0) * ((ib == id) ? 1 : 0));
        g[IX(ia, ic)] += h2b * rho[IX(id, ib)];
        g[IX(ia, id)] -= h2b * rho[IX(ic, ib)];
        g[IX(ib, ic)] -= h2b * rho[IX(id, ia)];
        g[IX(ib, id)] += h2b * rho[IX(ic, ia)];
        g[IX(ic, ia)] += f2b * rho[IX(ib, id)];
        g[IX(ic, ib)] -= f2b * rho[IX(ia, id)];
        g[IX(id, ia)] -= f2b * rho[IX(ib, ic)];
        g[IX(id, ib)] += f2b * rho[IX(ia, ic)];
        dl[IX(ib, ia)] += h2b * kLR[IX(id, ic)];
        dr[IX(ib, ia)] += h2b * kRL[IX(id, ic)];
        dl[IX(id, ic)] += f2b * kLR[IX(ib, ia)];
        dr[IX(id, ic)] += f2b * kRL[IX(ib, ia)];
      }
    }
#pragma omp critical
    {
      for (size_t i = 0; i < nn; ++i) {
        gamma[i] += g[i];
        dLR[i] += dl[i];
        dRL[i] += dr[i];
      }
    }
  }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) hsp[i + size_t(j) * n] = gamma[i + size_t(j) * n] + m->H1(i, j);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < j; ++i) {
      dLR[i + size_t(j) * n] = -1.0 * dLR[j + size_t(i) * n];
      dRL[i + size_t(j) * n] = -1.0 * dRL[j + size_t(i) * n];
    }
}

// calculate_fields_diag (module_fields.f90:204-317)
static void calculate_fields_diag(const orc_model* m, const cplx* rho, const cplx* kLR, cplx* gamma, cplx* hsp,
                                  cplx* dLR, cplx* dRL, int nthreads) {
  const int n = m->n;
  const size_t nn = size_t(n) * n;
  std::fill(gamma, gamma + nn, zzero);
  std::fill(dLR, dLR + nn, zzero);
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
  {
    std::vector<cplx> g(nn, zzero), dl(nn, zzero);
    auto IX = [n](int i, int j) { return size_t(i - 1) + size_t(j - 1) * n; };
#pragma omp for schedule(static)
    for (long long kk = 0; kk < m->S; ++kk) {
      int ia = m->abcd[4 * kk], ib = m->abcd[4 * kk + 1], ic = m->abcd[4 * kk + 2], id = m->abcd[4 * kk + 3];
      cplx h2b = double(m->h2[kk]);
      const int perm = m->trperm[kk];
      for (int it = 1; it <= 2; ++it) {
        if (it == 2) {
          if (m->sp_2mj[ia - 1] + m->sp_2mj[ib - 1] == 0) continue;
          find_timerev(m, perm, ia, ib, ic, id);
          h2b = (perm < 0 ? -1.0 : 1.0) * h2b;
        }
        g[IX(ia, ic)] += h2b * rho[IX(id, ib)];
        g[IX(ia, id)] -= h2b * rho[IX(ic, ib)];
        if (ic == ia && ib != id) g[IX(ic, ia)] += h2b * rho[IX(ib, id)];
        if (ib <= id) g[IX(ib, id)] += h2b * rho[IX(ic, ia)];
        if (ib <= ic) g[IX(ib, ic)] -= h2b * rho[IX(id, ia)];
        if (ia != ic || ib != id) {
          if (id <= ib) g[IX(id, ib)] += h2b * rho[IX(ia, ic)];
          if (ic <= ib) g[IX(ic, ib)] -= h2b * rho[IX(ia, id)];
        }
        dl[IX(ib, ia)] += h2b * kLR[IX(id, ic)];
        if (ia != ic || ib != id) dl[IX(id, ic)] += h2b * kLR[IX(ib, ia)];
      }
    }
#pragma omp critical
    {
      for (size_t i = 0; i < nn; ++i) {
        gamma[i] += g[i];
        dLR[i] += dl[i];
      }
    }
  }
  for (int j = 0; j < n; ++j)
    for (int i = j + 1; i < n; ++i) gamma[i + size_t(j) * n] = std::conj(gamma[j + size_t(i) * n]);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) hsp[i + size_t(j) * n] = gamma[i + size_t(j) * n] + m->H1(i, j);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < j; ++i) dLR[i + size_t(j) * n] = -1.0 * dLR[j + size_t(i) * n];
  if (dRL)
    for (size_t i = 0; i < nn; ++i) dRL[i] = std::conj(dLR[i]);
}

// ---------------------------------------------------------------------------
// PFAPACK ZSKPFA('U','P') restated: ZSKTF2 (subroutines_pfaffian.f:1694-2017)
// on the whole matrix with ZSKR2 rank-2 updates (:2387-2630), followed by the
// product of the superdiagonal pivots with one sign flip per row exchange
// (:193-203).  The reference switches to the blocked ZLASKTRF path for
// N >= 4*NB (NB from ILAENV('ZHETRF')); the two are the same elimination and
// differ only in rounding order.  Returns info (>0: zero pivot, Pf = 0).
// ---------------------------------------------------------------------------
static inline double dcabs1(cplx z) { return std::fabs(z.real()) + std::fabs(z.imag()); }

static int zsktf2_upper_p(int N, cplx* A, int lda, int* ipiv) {
  auto a = [A, lda](int i, int j) -> cplx& { return A[size_t(i - 1) + size_t(j - 1) * lda]; };
  int info = 0;
  ipiv[N - 1] = N;
  for (int K = N; K >= 2; --K) {
    if (K % 2 == 0) {
      // IZAMAX over A(1:K-1, K)
      int KP = 1;
      double best = dcabs1(a(1, K));
      for (int i = 2; i <= K - 1; ++i) {
        const double v = dcabs1(a(i, K));
        if (v > best) {
          best = v;
          KP = i;
        }
      }
      const double colmax = std::abs(a(KP, K));
      if (colmax == 0.0) {
        if (info == 0) info = K - 1;
        KP = K - 1;
      }
      const int KK = K - 1;
      if (KP != KK) {
        for (int i = 1; i <= KP - 1; ++i) std::swap(a(i, KK), a(i, KP));
        for (int t = 0; t < KK - KP - 1; ++t) std::swap(a(KP + 1 + t, KK), a(KP, KP + 1 + t));
        for (int j = K; j <= N; ++j) std::swap(a(KK, j), a(KP, j));
        for (int i = KP; i <= KK - 1; ++i) a(i, KK) = -zone * a(i, KK);
        for (int j = KP + 1; j <= KK - 1; ++j) a(KP, j) = -zone * a(KP, j);
      }
      if (colmax != 0.0) {
        const cplx alpha = zone / a(K - 1, K);
        const int nn = K - 2;
        // ZSKR2('U', nn, alpha, x = A(1:,K), y = A(1:,K-1), A)
        for (int J = 1; J <= nn; ++J) {
          const cplx xj = a(J, K), yj = a(J, K - 1);
          if (xj != zzero || yj != zzero) {
            const cplx t1 = alpha * yj, t2 = alpha * xj;
            for (int I = 1; I <= J - 1; ++I) a(I, J) = a(I, J) + a(I, K) * t1 - a(I, K - 1) * t2;
            a(J, J) = zzero;
          } else {
            a(J, J) = zzero;
          }
        }
        const cplx s = zone / a(K - 1, K);
        for (int i = 1; i <= nn; ++i) a(i, K) = s * a(i, K);
      }
      ipiv[K - 2] = KP;
    } else {
      ipiv[K - 2] = K - 1;
    }
  }
  return info;
}

static cplx zskpfa_up(int N, cplx* A, int lda, int* info_out) {
  *info_out = 0;
  if (N == 0) return zone;
  if (N % 2 == 1) return zzero;
  std::vector<int> ipiv(N);
  const int info = zsktf2_upper_p(N, A, lda, ipiv.data());
  if (info > 0) return zzero;
  cplx pf = zone;
  for (int I = 1; I <= N - 1; I += 2) {
    pf = pf * A[size_t(I - 1) + size_t(I) * lda];
    if (ipiv[I - 1] != I) pf = -pf;
  }
  return pf;
}

// ---------------------------------------------------------------------------
// construct_canonical_basis (module_wavefunctions.f90:777-945)
// ---------------------------------------------------------------------------
struct Canon {
  int nocc = 0, nemp = 0;
  double ovac = 0.0;
  std::vector<double> D;  // real n x n
  Mat zUc, zVc;
  std::vector<double> voveru;  // length n - nocc
  int info = 0;
};

static void construct_canonical_basis(const double* U, const double* V, int n, double occeps, int allemp,
                                      Canon& cb) {
  const double eps = (occeps < 2.2250738585072014e-308) ? 1.0e-8 : occeps;
  const size_t nn = size_t(n) * n;
  std::vector<double> rho(nn), kappa(nn), Dc(nn), rhoc(nn), kappac(nn), A1(nn), A2(nn), eig(n);
  dgemm('n', 't', n, n, n, 1.0, V, n, V, n, 0.0, rho.data(), n);
  Dc = rho;
  {
    int lwork = 3 * n - 1, info = 0;
    std::vector<double> work(std::max(1, lwork));
    char jv = 'V', up = 'U';
    int nn_ = n;
    p_dsyev(&jv, &up, &nn_, Dc.data(), &nn_, eig.data(), work.data(), &lwork, &info);
    cb.info = info;
  }
  dgemm('t', 'n', n, n, n, 1.0, Dc.data(), n, rho.data(), n, 0.0, A1.data(), n);
  dgemm('n', 'n', n, n, n, 1.0, A1.data(), n, Dc.data(), n, 0.0, rhoc.data(), n);
  auto R = [&](std::vector<double>& X, int i, int j) -> double& { return X[size_t(i - 1) + size_t(j - 1) * n]; };
  int nocc = 0, nemp = 0;
  double ovac = 0.0;
  for (int i = 1; i <= n; ++i) {
    const double v2 = std::fabs(R(rhoc, i, i));
    const double u = std::sqrt(std::fabs(1.0 - v2));
    if (v2 >= 1.0 - eps)
      ++nocc;
    else if (v2 <= eps && allemp == 0)
      ++nemp;
    else
      ovac = ovac + std::log(u);
  }
  dgemm('n', 't', n, n, n, 1.0, V, n, U, n, 0.0, kappa.data(), n);
  dgemm('t', 'n', n, n, n, 1.0, Dc.data(), n, kappa.data(), n, 0.0, A1.data(), n);
  dgemm('n', 'n', n, n, n, 1.0, A1.data(), n, Dc.data(), n, 0.0, kappac.data(), n);
  std::vector<int> submax(n + 2, 0), subdim(n + 2, 0);  // 1-based
  for (int i = 1 + nemp; i <= n - nocc; ++i) {
    submax[i] = i;
    for (int j = i + 1; j <= n - nocc; ++j)
      if (std::fabs(R(kappac, j, i)) > std::sqrt(eps) * 1.0e-2) submax[i] = j;
  }
  int k = 1 + nemp;
  while (k < n - nocc) {
    const int j = submax[k];
    std::fill(subdim.begin(), subdim.end(), 0);
    int mx = 0;
    for (int t = k; t <= j; ++t) {
      subdim[t] = submax[t];
      mx = std::max(mx, subdim[t]);
    }
    for (int t = k; t <= j; ++t) submax[t] = mx;
    if (mx == j) k = j + 1;
  }
  k = 1 + nemp;
  while (k < n - nocc) {
    subdim[k] = submax[k] - k + 1;
    if (subdim[k] > 2 && (subdim[k] % 2) != 0) subdim[k] = 2;
    k = k + subdim[k];
  }
  std::fill(A1.begin(), A1.end(), 0.0);
  for (int i = 1; i <= n; ++i) R(A1, i, i) = 1.0;
  k = 1 + nemp;
  while (k < n - nocc) {
    const int mdim = subdim[k];
    if (mdim > 2) {
      std::vector<double> B1(size_t(mdim) * mdim), wr(mdim), wi(mdim), work(3 * mdim), vs(size_t(mdim) * mdim);
      std::vector<int> bwork(mdim);
      for (int jj = 0; jj < mdim; ++jj)
        for (int ii = 0; ii < mdim; ++ii) B1[ii + size_t(jj) * mdim] = R(kappac, k + ii, k + jj);
      int sdim = 0, info = 0, lwork = 3 * mdim, md = mdim;
      char jv = 'V', srt = 'N';
      p_dgees(&jv, &srt, lapack_sel, &md, B1.data(), &md, &sdim, wr.data(), wi.data(), vs.data(), &md, work.data(),
              &lwork, bwork.data(), &info);
      for (int jj = 0; jj < mdim; ++jj)
        for (int ii = 0; ii < mdim; ++ii) {
          R(A1, k + ii, k + jj) = vs[ii + size_t(jj) * mdim];
          R(kappac, k + ii, k + jj) = B1[ii + size_t(jj) * mdim];
        }
    }
    k = k + mdim;
  }
  int maxsub = 0;
  for (int t = 1; t <= n; ++t) maxsub = std::max(maxsub, subdim[t]);
  if (maxsub > 2) {
    dgemm('n', 'n', n, n, n, 1.0, Dc.data(), n, A1.data(), n, 0.0, A2.data(), n);
    Dc = A2;
  }
  cb.D = Dc;
  cb.zUc = Mat(n);
  cb.zVc = Mat(n);
  k = 0;
  for (int i = 1; i <= n; ++i) {
    const double v2 = std::fabs(R(rhoc, i, i));
    const double v = std::sqrt(v2);
    cb.zUc(i - 1, i - 1) = std::sqrt(std::fabs(1.0 - v2));
    if (v2 > 1.0 - eps) {
      cb.zVc(i - 1, i - 1) = v * zone;
    } else if (v2 <= eps) {
      cb.zVc(i - 1, i - 1) = v * zone;
    } else {
      if (k % 2 == 0) {
        if (i < n) cb.zVc(i - 1, i) = dsign(v, R(kappac, i, i + 1)) * zone;
      } else {
        cb.zVc(i - 1, i - 2) = dsign(v, R(kappac, i, i - 1)) * zone;
      }
      ++k;
    }
  }
  cb.nocc = nocc;
  cb.nemp = nemp;
  cb.ovac = ovac;
}

// v/u in the canonical basis (module_projection.f90:219-234)
static void voveru_from_canon(Canon& cb, int n) {
  cb.voveru.assign(std::max(1, n - cb.nocc), 0.0);
  int j = 1;
  for (int i = 1 + cb.nemp; i <= n - cb.nocc; ++i) {
    if (ipow_m1(j) == -1)
      cb.voveru[i - 1] = (i < n) ? (cb.zVc(i - 1, i) / cb.zUc(i - 1, i - 1)).real() : 0.0;
    else
      cb.voveru[i - 1] = (cb.zVc(i - 1, i - 2) / cb.zUc(i - 1, i - 1)).real();
    ++j;
  }
}

// calculate_overlap (module_projection.f90:782-937), same state left and right
static int calculate_overlap(const Canon& c0, const Canon& c1, const cplx* ROT, int n, cplx* overlap) {
  const int nocc0 = c0.nocc, nemp0 = c0.nemp, nocc1 = c1.nocc, nemp1 = c1.nemp;
  const int nempm = std::min(nemp1, nemp0);
  const int nbloc0 = n - nocc0 - nempm;
  const int nbloc1 = n - nocc1 - nempm;
  const int nreg = nbloc1 + nbloc0;
  const int n0 = n - nocc0, n1 = n - nocc1, n2 = n - nempm;
  const double fac1 = ipow_m1((long long)n2 * (n2 + 1) / 2);
  const double fac2 = ipow_m1((long long)nocc0 * (nocc0 - 1) / 2);
  const double fac3 = ipow_m1((long long)nocc0 * (nocc0 + 1) / 2 + (long long)nocc1 * (nocc1 + 1) / 2 +
                              (long long)nocc0 * (n0 + n2) + (long long)nocc1 * n1);
  const double signfac = fac1 * fac2 * fac3;
  const cplx normvac = zone * (0.5 * (c0.ovac + c1.ovac));
  int isla0 = (n0 - nemp0 == 0) ? 1 : 0;
  int isla1 = (n1 - nemp1 == 0) ? 2 : 0;
  *overlap = zzero;
  switch (isla0 + isla1) {
    case 1:
      if (nocc0 > n - nemp1) return 0;
      break;
    case 2:
      if (nocc1 > n - nemp0) return 0;
      break;
    case 3:
      if (nocc0 == nocc1)
        *overlap = zone;
      else
        return 0;
      break;
    default:
      break;
  }
  Mat D0(n), D1(n), DRc(n), Rn(n);
  for (size_t i = 0; i < size_t(n) * n; ++i) {
    D0.v[i] = c0.D[i] * zone;
    D1.v[i] = c1.D[i] * zone;
  }
  zgemm('n', 'n', n, n, n, zone, ROT, n, D1.p(), n, zzero, DRc.p(), n);
  zgemm('c', 'n', n, n, n, zone, D0.p(), n, DRc.p(), n, zzero, Rn.p(), n);
  std::vector<cplx> Rinv(size_t(n2) * n2);
  for (int j = 0; j < n2; ++j)
    for (int i = 0; i < n2; ++i) Rinv[i + size_t(j) * n2] = Rn(nempm + i, nempm + j);
  std::vector<int> ipiv(std::max(1, n2));
  int info = 0, nn2 = n2;
  if (n2 > 0) p_zgetrf(&nn2, &nn2, Rinv.data(), &nn2, ipiv.data(), &info);
  if (info != 0) return 10;  // reference stops: "got info from zgetrf"
  cplx detR = zone;
  for (int i = 0; i < n2; ++i) detR = detR * Rinv[i + size_t(i) * n2];
  double sgn = 1.0;
  for (int i = 0; i < n2; ++i)
    if (ipiv[i] != i + 1) sgn = -sgn;
  detR = sgn * detR;
  if (n2 > 0) {
    std::vector<cplx> work(std::max(1, n2));
    int lw = n2;
    p_zgetri(&nn2, Rinv.data(), &nn2, ipiv.data(), work.data(), &lw, &info);
    if (info != 0) return 11;
  }
  if (isla0 + isla1 != 3) {
    std::vector<cplx> M(size_t(nreg) * nreg, zzero);
    auto Mr = [&](int i, int j) -> cplx& { return M[size_t(i - 1) + size_t(j - 1) * nreg]; };
    for (int i = 1; i <= nbloc1; ++i) {
      if (ipow_m1(i) == -1)
        Mr(i, i + 1) = c1.voveru[i + nempm - 1];
      else
        Mr(i, i - 1) = c1.voveru[i + nempm - 1];
    }
    for (int j = 1; j <= nbloc0; ++j) {
      const int i = j + nbloc1;
      if (ipow_m1(i) == -1)
        Mr(i, i + 1) = -c0.voveru[j + nempm - 1];
      else
        Mr(i, i - 1) = -c0.voveru[j + nempm - 1];
    }
    for (int j = 1; j <= nbloc0; ++j)
      for (int i = 1; i <= nbloc1; ++i) {
        Mr(i, j + nbloc1) = -Rinv[size_t(i - 1) + size_t(j - 1) * n2];
        Mr(j + nbloc1, i) = Rinv[size_t(i - 1) + size_t(j - 1) * n2];
      }
    int pinfo = 0;
    *overlap = zskpfa_up(nreg, M.data(), nreg, &pinfo);
  }
  if (std::abs(*overlap) > 0.0) {
    const cplx ph = zimag * std::atan2(overlap->imag(), overlap->real());
    const cplx mod = zone * std::log(std::abs(*overlap));
    *overlap = detR * signfac * std::exp(ph + mod + normvac);
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Per-angle quantities and the gauge-angle loop
// ---------------------------------------------------------------------------
struct PNP {  // pnp_* accumulators (module_projection.f90:58-72)
  cplx over, ener, prot, neut, prot2, neut2, pari;
};

extern "C" {
struct orc_angle_out {  // one gauge angle, for component parity tests
  double over[2], ener[2], prot[2], neut[2], prot2[2], neut2[2];
};
}

struct ProjWork {
  int n;
  Mat zU, zV, Ubar, Vbar, Utl, Vtl, A, rho, kLR, kRL, gam, hsp, dLR, dRL, H20, ROTG;
  explicit ProjWork(int n_)
      : n(n_), zU(n_), zV(n_), Ubar(n_), Vbar(n_), Utl(n_), Vtl(n_), A(n_), rho(n_), kLR(n_), kRL(n_), gam(n_),
        hsp(n_), dLR(n_), dRL(n_), H20(n_), ROTG(n_) {}
};

// calculate_thouless (module_projection.f90:684-718)
static int calculate_thouless(const Mat& U, const Mat& V, const Mat& Ubar, const Mat& Vbar, Mat& Aphi, Mat& Utl,
                              Mat& Vtl) {
  const int n = U.n;
  Mat Uphi(n), Vphi(n), Uinv(n), A1(n), A2(n);
  zgemm('t', 'n', n, n, n, zone, V.p(), n, Vbar.p(), n, zzero, Uphi.p(), n);
  zgemm('t', 'n', n, n, n, zone, U.p(), n, Ubar.p(), n, zone, Uphi.p(), n);
  zgemm('t', 'n', n, n, n, zone, V.p(), n, Ubar.p(), n, zzero, Vphi.p(), n);
  zgemm('t', 'n', n, n, n, zone, U.p(), n, Vbar.p(), n, zone, Vphi.p(), n);
  Uinv = Uphi;
  std::vector<int> ipiv(n);
  std::vector<cplx> work(n);
  int info1 = 0, info2 = 0, nn = n, lw = n;
  p_zgetrf(&nn, &nn, Uinv.p(), &nn, ipiv.data(), &info1);
  p_zgetri(&nn, Uinv.p(), &nn, ipiv.data(), work.data(), &lw, &info2);
  zgemm('n', 'n', n, n, n, zone, Vphi.p(), n, Uinv.p(), n, zzero, Aphi.p(), n);
  for (auto& x : Aphi.v) x = std::conj(x);
  zgemm('n', 'n', n, n, n, zone, V.p(), n, Aphi.p(), n, zzero, A1.p(), n);
  zgemm('n', 'n', n, n, n, zone, U.p(), n, Aphi.p(), n, zzero, A2.p(), n);
  for (size_t i = 0; i < Utl.v.size(); ++i) {
    Utl.v[i] = U.v[i] + A1.v[i];
    Vtl.v[i] = V.v[i] + A2.v[i];
  }
  return (info1 != 0 || info2 != 0) ? 20 : 0;
}

// calculate_densities (module_wavefunctions.f90:1073-1087), called with
// UR = conj(Utilde), VR = conj(Vtilde) (module_projection.f90:264-266)
static void calculate_densities_lr(const Mat& UL, const Mat& VL, const Mat& Utl, const Mat& Vtl, Mat& rho, Mat& kLR,
                                   Mat& kRL) {
  const int n = UL.n;
  // URc = conj(conj(Utilde)) = Utilde
  zgemm('n', 't', n, n, n, zone, Vtl.p(), n, VL.p(), n, zzero, rho.p(), n);
  zgemm('n', 't', n, n, n, zone, Vtl.p(), n, UL.p(), n, zzero, kLR.p(), n);
  zgemm('n', 't', n, n, n, zone, VL.p(), n, Utl.p(), n, zzero, kRL.p(), n);
}

// calculate_particle_number io=0 (module_particlenumber.f90:78-143)
static void calculate_particle_number(const Mat& rho, const Mat& kLR, const Mat& kRL, cplx& prot, cplx& neut,
                                      cplx& prot2, cplx& neut2) {
  const int n = rho.n, h = n / 2;
  prot = neut = zzero;
  for (int i = 0; i < h; ++i) {
    prot += rho(i, i);
    neut += rho(i + h, i + h);
  }
  Mat rp(h), rn(h), klp(h), kln(h), krp(h), krn(h), A1(h), A2(h), A3(h), A4(h);
  for (int j = 0; j < h; ++j)
    for (int i = 0; i < h; ++i) {
      rp(i, j) = rho(i, j);
      rn(i, j) = rho(i + h, j + h);
      klp(i, j) = kLR(i, j);
      kln(i, j) = kLR(i + h, j + h);
      krp(i, j) = kRL(i, j);
      krn(i, j) = kRL(i + h, j + h);
    }
  zgemm('n', 'n', h, h, h, zone, rp.p(), h, rp.p(), h, zzero, A1.p(), h);
  zgemm('t', 'n', h, h, h, zone, krp.p(), h, klp.p(), h, zzero, A2.p(), h);
  zgemm('n', 'n', h, h, h, zone, rn.p(), h, rn.p(), h, zzero, A3.p(), h);
  zgemm('t', 'n', h, h, h, zone, krn.p(), h, kln.p(), h, zzero, A4.p(), h);
  cplx t1 = 0, t2 = 0, t3 = 0, t4 = 0;
  for (int i = 0; i < h; ++i) {
    t1 += A1(i, i);
    t2 += A2(i, i);
    t3 += A3(i, i);
    t4 += A4(i, i);
  }
  prot2 = prot + prot * prot - t1 + t2;
  neut2 = neut + neut * neut - t3 + t4;
}

// calculate_expectval_energy (module_hamiltonian.f90:1098-1126)
static cplx calculate_expectval_energy(const orc_model* m, const Mat& rho, const Mat& kRL, const Mat& gam,
                                       const Mat& dLR) {
  const int n = rho.n;
  Mat A1(n), A2(n), A3(n);
  zgemm('n', 'n', n, n, n, zone, m->H1.p(), n, rho.p(), n, zzero, A1.p(), n);
  zgemm('n', 'n', n, n, n, zone, gam.p(), n, rho.p(), n, zzero, A2.p(), n);
  zgemm('n', 't', n, n, n, zone, dLR.p(), n, kRL.p(), n, zzero, A3.p(), n);
  cplx e1 = 0, e2 = 0, e3 = 0;
  for (int i = 0; i < n; ++i) {
    e1 += A1(i, i);
    e2 += A2(i, i);
    e3 += A3(i, i);
  }
  return m->H0 + e1 + 0.5 * (e2 + e3);
}

// calculate_H20 (module_fields.f90:366-391)
static void calculate_H20(const Mat& U, const Mat& V, const Mat& hsp, const Mat& dLR, const Mat& dRL,
                          double factor_delta, Mat& H20) {
  const int n = U.n;
  Mat A1(n), A2(n), A4(n), A5(n);
  zgemm('t', 'n', n, n, n, zone, U.p(), n, hsp.p(), n, zzero, A1.p(), n);
  zgemm('n', 'n', n, n, n, zone, A1.p(), n, V.p(), n, zzero, A2.p(), n);
  zgemm('t', 'n', n, n, n, zone, U.p(), n, dLR.p(), n, zzero, A1.p(), n);
  zgemm('n', 'n', n, n, n, zone, A1.p(), n, U.p(), n, zzero, A4.p(), n);
  zgemm('t', 'n', n, n, n, zone, V.p(), n, dRL.p(), n, zzero, A1.p(), n);
  zgemm('n', 'n', n, n, n, zone, A1.p(), n, V.p(), n, zzero, A5.p(), n);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) H20(i, j) = A2(i, j) - A2(j, i) + (A4(i, j) - A5(i, j)) * factor_delta;
}

// generate_rotation_gauge applied to ROT = identity (module_projection.f90:569-588)
static void rotation_gauge(double php, double phn, int n, Mat& R) {
  const cplx pp = std::exp(zimag * php), pn = std::exp(zimag * phn);
  std::fill(R.v.begin(), R.v.end(), zzero);
  for (int i = 0; i < n / 2; ++i) {
    R(i, i) = pp;
    R(i + n / 2, i + n / 2) = pn;
  }
}

// assign_angles (module_projection.f90:112-185), single process
struct Angles {
  std::vector<double> php, phn;
  std::vector<cplx> wp, wn;
};
static Angles assign_angles(int Mp, int Mn, double facpi, double Z, double N) {
  Angles a;
  for (int jp = 1; jp <= Mp; ++jp)
    for (int jn = 1; jn <= Mn; ++jn) {
      const double php = (Mp % 2 == 1) ? facpi * (jp - 1.0) / Mp : facpi * (jp - 0.5) / Mp;
      const double phn = (Mn % 2 == 1) ? facpi * (jn - 1.0) / Mn : facpi * (jn - 0.5) / Mn;
      a.php.push_back(php);
      a.phn.push_back(phn);
      a.wp.push_back(std::exp(-zimag * php * Z) / double(Mp));
      a.wn.push_back(std::exp(-zimag * phn * N) / double(Mn));
    }
  return a;
}

// ---------------------------------------------------------------------------
// Iteration state (module globals of Wavefunctions, Constraints, Gradient)
// ---------------------------------------------------------------------------
struct orc_vap {
  const orc_model* m = nullptr;
  int n = 0;
  std::vector<double> U0, V0, U1, V1, rhoRR, kapRR;
  int Mp = 1, Mn = 1;
  double facpi = 2 * kPi, Z = 0, N = 0, factor_delta = 1.0, occeps = 0.0;
  int allemp = 0;
  int gtype = 0;
  double eta = 0, mu = 0, geps = 1e-4;
  int cdim = 0, cpair = 0;
  double ceps = 1e-6;
  std::vector<double> cHO, cval, c20, lam0, lam1;
  std::vector<double> Zi, Zim1, H20v, Lchol;
  // diagonalize_hsp_and_H11 (gradient types 1 and 2)
  std::vector<double> eig_hsp, eig_H11;
  int info_hsp = 0, info_H11 = 0;
  double eta_used = 0.0, mu_used = 0.0;
  double gnorm = 0.0;
  PNP pnp;
  std::vector<cplx> pnpA, pnpH20, pnpAH20;
  int nthreads = 0;
  int control_NZ[5] = {0, 0, 0, 0, 0};
};

extern "C" {

struct orc_pnp_out {
  double over[2], ener[2], prot[2], neut[2], prot2[2], neut2[2];
  int nocc, nemp;
};

void orc_set_lapack(void* zg, void* dg, void* zgtrf, void* zgtri, void* dsy, void* dge, void* dpb, void* dtr,
                    void* dsy2) {
  p_zgemm = (zgemm_t)zg;
  p_dgemm = (dgemm_t)dg;
  p_zgetrf = (zgetrf_t)zgtrf;
  p_zgetri = (zgetri_t)zgtri;
  p_dsyev = (dsyev_t)dsy;
  p_dgees = (dgees_t)dge;
  p_dpbtrf = (dpbtrf_t)dpb;
  p_dtrtri = (dtrtri_t)dtr;
  p_dsysv = (dsysv_t)dsy2;
}

orc_model* orc_model_new(int n, const int* sp_2mj, const int* sp_tr, const int* sp_l, long long S,
                         const int16_t* abcd, const float* h2, const int8_t* trperm, const double* H1,
                         const double* H0) {
  auto* m = new orc_model();
  m->n = n;
  m->sp_2mj.assign(sp_2mj, sp_2mj + n);
  m->sp_tr.assign(sp_tr, sp_tr + n);
  m->sp_l.assign(sp_l, sp_l + n);
  m->S = S;
  m->abcd.assign(abcd, abcd + 4 * S);
  m->h2.assign(h2, h2 + S);
  m->trperm.assign(trperm, trperm + S);
  m->H1 = Mat(n);
  std::memcpy(m->H1.p(), H1, sizeof(cplx) * size_t(n) * n);
  m->H0 = cplx(H0[0], H0[1]);
  return m;
}
void orc_model_free(orc_model* m) { delete m; }

void orc_calculate_fields(const orc_model* m, const double* rho, const double* kLR, const double* kRL, double* gamma,
                          double* hsp, double* dLR, double* dRL, int nthreads) {
  calculate_fields(m, (const cplx*)rho, (const cplx*)kLR, (const cplx*)kRL, (cplx*)gamma, (cplx*)hsp, (cplx*)dLR,
                   (cplx*)dRL, nthreads);
}

void orc_calculate_fields_diag(const orc_model* m, const double* rho, const double* kLR, double* gamma, double* hsp,
                               double* dLR, double* dRL, int nthreads) {
  calculate_fields_diag(m, (const cplx*)rho, (const cplx*)kLR, (cplx*)gamma, (cplx*)hsp, (cplx*)dLR, (cplx*)dRL,
                        nthreads);
}

// ZSKPFA('U','P'); A (complex, column-major, n x n) is overwritten.
int orc_pfaffian(int n, double* A, double* pf) {
  int info = 0;
  const cplx r = zskpfa_up(n, (cplx*)A, n, &info);
  pf[0] = r.real();
  pf[1] = r.imag();
  return info;
}

// Canonical basis summary for tests: nocc, nemp, ovac and v/u.
int orc_canonical(const double* U, const double* V, int n, double occeps, int allemp, int* nocc, int* nemp,
                  double* ovac, double* voveru, double* D) {
  Canon cb;
  construct_canonical_basis(U, V, n, occeps, allemp, cb);
  if (n - cb.nocc - cb.nemp == 0) cb.ovac = 0.0;
  voveru_from_canon(cb, n);
  *nocc = cb.nocc;
  *nemp = cb.nemp;
  *ovac = cb.ovac;
  for (int i = 0; i < n - cb.nocc; ++i) voveru[i] = cb.voveru[i];
  if (D) std::memcpy(D, cb.D.data(), sizeof(double) * size_t(n) * n);
  return cb.info;
}

// project_wavefunction(iopt=0, iprint=0) (module_projection.f90:201-373),
// followed by calculate_projected_H20 (:729-759).  Per-angle scalars are
// optionally written to `angles` (G entries).  pnpA/pnpH20/pnpAH20 and H20v may
// be null.
int orc_project(const orc_model* m, const double* U0, const double* V0, int Mp, int Mn, double facpi, double Z,
                double N, double factor_delta, double occeps, int allemp, orc_pnp_out* out, double* H20v,
                double* pnpA_out, double* pnpH20_out, double* pnpAH20_out, orc_angle_out* angles, int nthreads) {
  const int n = m->n;
  const size_t nn = size_t(n) * n;
  Canon cb;
  construct_canonical_basis(U0, V0, n, occeps, allemp, cb);
  if (n - cb.nocc - cb.nemp == 0) cb.ovac = 0.0;
  voveru_from_canon(cb, n);
  ProjWork w(n);
  for (size_t i = 0; i < nn; ++i) {
    w.zU.v[i] = U0[i] * zone;
    w.zV.v[i] = V0[i] * zone;
  }
  Angles an = assign_angles(Mp, Mn, facpi, Z, N);
  PNP p{};
  std::vector<cplx> pA(nn, zzero), pH(nn, zzero), pAH(nn, zzero);
  int status = 0;
  for (size_t g = 0; g < an.php.size(); ++g) {
    rotation_gauge(an.php[g], an.phn[g], n, w.ROTG);
    // rotate_wavefunction: Ubar = R U, Vbar = R^* V (module_projection.f90:641-653)
    Mat Rc(n);
    for (size_t i = 0; i < nn; ++i) Rc.v[i] = std::conj(w.ROTG.v[i]);
    zgemm('n', 'n', n, n, n, zone, w.ROTG.p(), n, w.zU.p(), n, zzero, w.Ubar.p(), n);
    zgemm('n', 'n', n, n, n, zone, Rc.p(), n, w.zV.p(), n, zzero, w.Vbar.p(), n);
    cplx rot_over = zone;
    if (std::max(Mp, Mn) > 1) {
      const int st = calculate_overlap(cb, cb, w.ROTG.p(), n, &rot_over);
      if (st) return st;
    }
    const int st = calculate_thouless(w.zU, w.zV, w.Ubar, w.Vbar, w.A, w.Utl, w.Vtl);
    if (st) status = st;
    calculate_densities_lr(w.zU, w.zV, w.Utl, w.Vtl, w.rho, w.kLR, w.kRL);
    if (std::max(Mp, Mn) > 1)
      calculate_fields(m, w.rho.p(), w.kLR.p(), w.kRL.p(), w.gam.p(), w.hsp.p(), w.dLR.p(), w.dRL.p(), nthreads);
    else
      calculate_fields_diag(m, w.rho.p(), w.kLR.p(), w.gam.p(), w.hsp.p(), w.dLR.p(), w.dRL.p(), nthreads);
    cplx prot, neut, prot2, neut2;
    calculate_particle_number(w.rho, w.kLR, w.kRL, prot, neut, prot2, neut2);
    const cplx ener = calculate_expectval_energy(m, w.rho, w.kRL, w.gam, w.dLR);
    calculate_H20(w.Utl, w.Vtl, w.hsp, w.dLR, w.dRL, factor_delta, w.H20);
    // sum_gauge (module_projection.f90:425-458), iopt = 0
    const cplx weight = an.wp[g] * an.wn[g];
    const cplx f1 = weight * rot_over;
    const cplx f2 = f1 * ener;
    p.over += f1;
    p.ener += ener * f1;
    p.prot += prot * f1;
    p.neut += neut * f1;
    p.prot2 += prot2 * f1;
    p.neut2 += neut2 * f1;
    for (size_t i = 0; i < nn; ++i) {
      pA[i] += w.A.v[i] * f1;
      pH[i] += w.H20.v[i] * f1;
      pAH[i] += w.A.v[i] * f2;
    }
    if (angles) {
      orc_angle_out& a = angles[g];
      a.over[0] = rot_over.real(), a.over[1] = rot_over.imag();
      a.ener[0] = ener.real(), a.ener[1] = ener.imag();
      a.prot[0] = prot.real(), a.prot[1] = prot.imag();
      a.neut[0] = neut.real(), a.neut[1] = neut.imag();
      a.prot2[0] = prot2.real(), a.prot2[1] = prot2.imag();
      a.neut2[0] = neut2.real(), a.neut2[1] = neut2.imag();
    }
  }
  // calculate_projected_H20
  int imag_fail = 0;
  if (H20v) {
    const cplx over = p.over, ener = p.ener / p.over;
    int l = 0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i, ++l) {
        const size_t ij = i + size_t(j) * n, ji = j + size_t(i) * n;
        const cplx A = 0.5 * (pA[ij] - pA[ji]) / over;
        const cplx H = 0.5 * (pH[ij] - pH[ji]) / over;
        const cplx AH = 0.5 * (pAH[ij] - pAH[ji]) / over;
        H20v[l] = (AH - ener * A + H).real();
        const double ig = ((pAH[ij] - ener * pA[ij] + pH[ij]) / over).imag();
        if (ig > 1.0e-8) imag_fail = 1;
      }
  }
  if (out) {
    out->over[0] = p.over.real(), out->over[1] = p.over.imag();
    out->ener[0] = p.ener.real(), out->ener[1] = p.ener.imag();
    out->prot[0] = p.prot.real(), out->prot[1] = p.prot.imag();
    out->neut[0] = p.neut.real(), out->neut[1] = p.neut.imag();
    out->prot2[0] = p.prot2.real(), out->prot2[1] = p.prot2.imag();
    out->neut2[0] = p.neut2.real(), out->neut2[1] = p.neut2.imag();
    out->nocc = cb.nocc;
    out->nemp = cb.nemp;
  }
  if (pnpA_out) std::memcpy(pnpA_out, pA.data(), sizeof(cplx) * nn);
  if (pnpH20_out) std::memcpy(pnpH20_out, pH.data(), sizeof(cplx) * nn);
  if (pnpAH20_out) std::memcpy(pnpAH20_out, pAH.data(), sizeof(cplx) * nn);
  if (imag_fail) return 30;
  return status;
}

// calculate_decompo_energy (module_hamiltonian.f90:1134-1260): ecomp[0..11] =
// 1-body p, n; 2-body PH pp, pn, np, nn; PP pp, pn, np, nn; energy p, n
static void calculate_decompo_energy(const orc_model* m, const Mat& rho, const Mat& kRL, const Mat& gam,
                                     const Mat& dLR, cplx* ecomp) {
  const int n = rho.n, h = n / 2;
  auto blk = [h](const Mat& X, int bi, int bj) {
    Mat B(h);
    for (int j = 0; j < h; ++j)
      for (int i = 0; i < h; ++i) B(i, j) = X(i + bi * h, j + bj * h);
    return B;
  };
  auto tr = [](const Mat& A) {
    cplx t = 0;
    for (int i = 0; i < A.n; ++i) t += A(i, i);
    return t;
  };
  Mat A(h);
  const int pr[4][2] = {{0, 0}, {0, 1}, {1, 0}, {1, 1}};  // pp, pn, np, nn
  for (int q = 0; q < 4; ++q) {
    const int bi = pr[q][0], bj = pr[q][1];
    // APH_xy = gamma_xy rho_yx; APP_xy = delta_xy kappaRL_xy^T
    const Mat g = blk(gam, bi, bj), r = blk(rho, bj, bi), d = blk(dLR, bi, bj), k = blk(kRL, bi, bj);
    zgemm('n', 'n', h, h, h, zone, g.p(), h, r.p(), h, zzero, A.p(), h);
    ecomp[2 + q] = 0.5 * tr(A);
    zgemm('n', 't', h, h, h, zone, d.p(), h, k.p(), h, zzero, A.p(), h);
    ecomp[6 + q] = 0.5 * tr(A);
  }
  Mat A1(n), A2(n), A3(n);
  zgemm('n', 'n', n, n, n, zone, m->H1.p(), n, rho.p(), n, zzero, A1.p(), n);
  zgemm('n', 'n', n, n, n, zone, gam.p(), n, rho.p(), n, zzero, A2.p(), n);
  zgemm('n', 't', n, n, n, zone, dLR.p(), n, kRL.p(), n, zzero, A3.p(), n);
  cplx e1p = 0, e1n = 0, php = 0, phn = 0, ppp = 0, ppn = 0;
  for (int i = 0; i < h; ++i) {
    e1p += A1(i, i);
    e1n += A1(i + h, i + h);
    php += 0.5 * A2(i, i);
    phn += 0.5 * A2(i + h, i + h);
    ppp += 0.5 * A3(i, i);
    ppn += 0.5 * A3(i + h, i + h);
  }
  ecomp[0] = e1p;
  ecomp[1] = e1n;
  ecomp[10] = e1p + php + ppp;
  ecomp[11] = e1n + phn + ppn;
}

// calculate_expectval_obo_cplx (module_operators.f90:146-164): Tr(B rho) over
// the proton and the neutron rows of B rho
static void expectval_obo_cplx(const Mat& rho, const Mat& B, cplx& ep, cplx& en) {
  const int n = rho.n;
  Mat A1(n);
  zgemm('n', 'n', n, n, n, zone, B.p(), n, rho.p(), n, zzero, A1.p(), n);
  ep = en = zzero;
  for (int i = 0; i < n / 2; ++i) {
    ep += A1(i, i);
    en += A1(i + n / 2, i + n / 2);
  }
}

// calculate_expectval_obos_cplx (module_operators.f90:227-257): <O^2>
static cplx expectval_obos_cplx(const Mat& rho, const Mat& kLR, const Mat& kRL, const Mat& O, const Mat& O2) {
  const int n = rho.n;
  Mat A1(n), A2(n), A3(n), A4(n), A5(n), A6(n);
  zgemm('n', 'n', n, n, n, zone, O.p(), n, rho.p(), n, zzero, A1.p(), n);
  zgemm('n', 'n', n, n, n, zone, O2.p(), n, rho.p(), n, zzero, A2.p(), n);
  zgemm('t', 't', n, n, n, zone, O.p(), n, kRL.p(), n, zzero, A3.p(), n);
  zgemm('n', 'n', n, n, n, zone, O.p(), n, kLR.p(), n, zzero, A4.p(), n);
  zgemm('n', 'n', n, n, n, zone, A1.p(), n, A1.p(), n, zzero, A5.p(), n);
  zgemm('n', 'n', n, n, n, zone, A3.p(), n, A4.p(), n, zzero, A6.p(), n);
  cplx t1 = 0, t2 = 0, t5 = 0, t6 = 0;
  for (int i = 0; i < n; ++i) {
    t1 += A1(i, i);
    t2 += A2(i, i);
    t5 += A5(i, i);
    t6 += A6(i, i);
  }
  return t1 * t1 + t2 - t5 + t6;
}

// project_wavefunction with iopt = 1 (module_projection.f90:201-373, the
// branch :298-354) and sum_gauge with iopt = 1 (:425-458): the gauge sums of
// the printed observables.  Angles as assign_angles gives them, unfolded.
// scal (complex): over, ener (the energy of the components: the reference
// leaves rot_ener stale in this mode and prints the components), prot, neut,
// prot2, neut2, pari (sum of weight * rot_pari, the overlap with the parity-
// rotated state, generate_rotation_parity :607-625), ecomp[12]; obo_sum
// (nobo x 2 complex: protons, neutrons); sq_sum (nsq complex); occnum
// (nshell x 2 complex, calculate_occupation_number, module_particlenumber.f90:
// 157-176); rho (n x n complex, pnp_rho).  parity may be null (pari = 0).
int orc_project_observables(const orc_model* m, const double* U0, const double* V0, int Mp, int Mn, double facpi,
                            double Z, double N, double factor_delta, double occeps, int allemp, int nobo,
                            const double* obo, int nsq, const double* sq, const int* parity, int nshell,
                            const int* shell_size, double* scal, double* obo_sum, double* sq_sum, double* occnum,
                            double* rho_sum, int nthreads) {
  const int n = m->n, h = n / 2;
  const size_t nn = size_t(n) * n;
  Canon cb;
  construct_canonical_basis(U0, V0, n, occeps, allemp, cb);
  if (n - cb.nocc - cb.nemp == 0) cb.ovac = 0.0;
  voveru_from_canon(cb, n);
  ProjWork w(n);
  for (size_t i = 0; i < nn; ++i) {
    w.zU.v[i] = U0[i] * zone;
    w.zV.v[i] = V0[i] * zone;
  }
  auto mat = [n, nn](const double* p) {
    Mat M(n);
    std::memcpy(M.p(), p, sizeof(cplx) * nn);
    return M;
  };
  std::vector<Mat> B, O, O2;
  for (int k = 0; k < nobo; ++k) B.push_back(mat(obo + 2 * nn * k));
  for (int k = 0; k < nsq; ++k) {
    O.push_back(mat(sq + 2 * nn * (2 * k)));
    O2.push_back(mat(sq + 2 * nn * (2 * k + 1)));
  }
  Angles an = assign_angles(Mp, Mn, facpi, Z, N);
  std::vector<cplx> S(19, zzero), bs(2 * size_t(nobo), zzero), ss(nsq, zzero), oc(2 * size_t(nshell), zzero),
      rs(nn, zzero);
  int status = 0;
  for (size_t g = 0; g < an.php.size(); ++g) {
    rotation_gauge(an.php[g], an.phn[g], n, w.ROTG);
    Mat Rc(n);
    for (size_t i = 0; i < nn; ++i) Rc.v[i] = std::conj(w.ROTG.v[i]);
    zgemm('n', 'n', n, n, n, zone, w.ROTG.p(), n, w.zU.p(), n, zzero, w.Ubar.p(), n);
    zgemm('n', 'n', n, n, n, zone, Rc.p(), n, w.zV.p(), n, zzero, w.Vbar.p(), n);
    cplx rot_over = zone, rot_pari = zzero;
    if (std::max(Mp, Mn) > 1) {
      const int st = calculate_overlap(cb, cb, w.ROTG.p(), n, &rot_over);
      if (st) return st;
    }
    const int st = calculate_thouless(w.zU, w.zV, w.Ubar, w.Vbar, w.A, w.Utl, w.Vtl);
    if (st) status = st;
    calculate_densities_lr(w.zU, w.zV, w.Utl, w.Vtl, w.rho, w.kLR, w.kRL);
    if (std::max(Mp, Mn) > 1)
      calculate_fields(m, w.rho.p(), w.kLR.p(), w.kRL.p(), w.gam.p(), w.hsp.p(), w.dLR.p(), w.dRL.p(), nthreads);
    else
      calculate_fields_diag(m, w.rho.p(), w.kLR.p(), w.gam.p(), w.hsp.p(), w.dLR.p(), w.dRL.p(), nthreads);
    if (parity) {
      // the parity-rotated gauge rotation P R (module_projection.f90:279-283)
      Mat RP(n);
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) RP(i, j) = double(parity[i]) * w.ROTG(i, j);
      const int stp = calculate_overlap(cb, cb, RP.p(), n, &rot_pari);
      if (stp) return stp;
    }
    cplx prot, neut, prot2, neut2;
    calculate_particle_number(w.rho, w.kLR, w.kRL, prot, neut, prot2, neut2);
    cplx ec[12];
    calculate_decompo_energy(m, w.rho, w.kRL, w.gam, w.dLR, ec);
    const cplx weight = an.wp[g] * an.wn[g];
    const cplx f1 = weight * rot_over;
    S[0] += f1;
    S[1] += (m->H0 + ec[10] + ec[11]) * f1;
    S[2] += prot * f1;
    S[3] += neut * f1;
    S[4] += prot2 * f1;
    S[5] += neut2 * f1;
    S[6] += rot_pari * weight;
    for (int q = 0; q < 12; ++q) S[7 + q] += ec[q] * f1;
    for (int k = 0; k < nobo; ++k) {
      cplx ep, en;
      expectval_obo_cplx(w.rho, B[k], ep, en);
      bs[2 * k] += ep * f1;
      bs[2 * k + 1] += en * f1;
    }
    for (int k = 0; k < nsq; ++k) ss[k] += expectval_obos_cplx(w.rho, w.kLR, w.kRL, O[k], O2[k]) * f1;
    for (int t = 0, k = 0; t < nshell; ++t)
      for (int j = 0; j < shell_size[t]; ++j, ++k) {
        oc[2 * t] += w.rho(k, k) * f1;
        oc[2 * t + 1] += w.rho(k + h, k + h) * f1;
      }
    for (size_t i = 0; i < nn; ++i) rs[i] += w.rho.v[i] * f1;
  }
  std::memcpy(scal, S.data(), sizeof(cplx) * S.size());
  if (obo_sum) std::memcpy(obo_sum, bs.data(), sizeof(cplx) * bs.size());
  if (sq_sum) std::memcpy(sq_sum, ss.data(), sizeof(cplx) * ss.size());
  if (occnum) std::memcpy(occnum, oc.data(), sizeof(cplx) * oc.size());
  if (rho_sum) std::memcpy(rho_sum, rs.data(), sizeof(cplx) * nn);
  return status;
}

// One gauge angle's transition densities (rotation + Thouless + densities),
// for component parity tests of the field kernel and the density kernels.
int orc_angle_densities(const orc_model* m, const double* U0, const double* V0, double php, double phn, double* rho,
                        double* kLR, double* kRL, double* Aphi) {
  const int n = m->n;
  const size_t nn = size_t(n) * n;
  ProjWork w(n);
  for (size_t i = 0; i < nn; ++i) {
    w.zU.v[i] = U0[i] * zone;
    w.zV.v[i] = V0[i] * zone;
  }
  rotation_gauge(php, phn, n, w.ROTG);
  Mat Rc(n);
  for (size_t i = 0; i < nn; ++i) Rc.v[i] = std::conj(w.ROTG.v[i]);
  zgemm('n', 'n', n, n, n, zone, w.ROTG.p(), n, w.zU.p(), n, zzero, w.Ubar.p(), n);
  zgemm('n', 'n', n, n, n, zone, Rc.p(), n, w.zV.p(), n, zzero, w.Vbar.p(), n);
  const int st = calculate_thouless(w.zU, w.zV, w.Ubar, w.Vbar, w.A, w.Utl, w.Vtl);
  calculate_densities_lr(w.zU, w.zV, w.Utl, w.Vtl, w.rho, w.kLR, w.kRL);
  std::memcpy(rho, w.rho.p(), sizeof(cplx) * nn);
  std::memcpy(kLR, w.kLR.p(), sizeof(cplx) * nn);
  std::memcpy(kRL, w.kRL.p(), sizeof(cplx) * nn);
  if (Aphi) std::memcpy(Aphi, w.A.p(), sizeof(cplx) * nn);
  return st;
}

// calculate_overlap for one gauge angle of a state with itself.
int orc_overlap(const double* U0, const double* V0, int n, double php, double phn, double occeps, int allemp,
                double* ov) {
  Canon cb;
  construct_canonical_basis(U0, V0, n, occeps, allemp, cb);
  if (n - cb.nocc - cb.nemp == 0) cb.ovac = 0.0;
  voveru_from_canon(cb, n);
  Mat R(n);
  rotation_gauge(php, phn, n, R);
  cplx o;
  const int st = calculate_overlap(cb, cb, R.p(), n, &o);
  ov[0] = o.real();
  ov[1] = o.imag();
  return st;
}

// ---------------------------------------------------------------------------
// Constraints and gradient (module_constraints.f90, module_gradient.f90,
// module_operators.f90)
// ---------------------------------------------------------------------------

// set_operator_qpbasis (module_operators.f90:49-97)
static void set_operator_qpbasis(const char* part, const double* U, const double* V, const double* A, double* B,
                                 int n) {
  const size_t nn = size_t(n) * n;
  std::vector<double> A1(nn), A2(nn), A3(nn);
  double factor = 1.0;
  if (!std::strcmp(part, "f11")) {
    factor = 1.0;
    dgemm('t', 'n', n, n, n, 1.0, U, n, A, n, 0.0, A1.data(), n);
    dgemm('n', 'n', n, n, n, 1.0, A1.data(), n, U, n, 0.0, A2.data(), n);
    dgemm('t', 't', n, n, n, 1.0, V, n, A, n, 0.0, A1.data(), n);
    dgemm('n', 'n', n, n, n, 1.0, A1.data(), n, V, n, 0.0, A3.data(), n);
  } else if (!std::strcmp(part, "g11")) {
    factor = 1.0;
    dgemm('t', 'n', n, n, n, 1.0, U, n, A, n, 0.0, A1.data(), n);
    dgemm('n', 'n', n, n, n, 1.0, A1.data(), n, V, n, 0.0, A2.data(), n);
    dgemm('t', 'n', n, n, n, 1.0, V, n, A, n, 0.0, A1.data(), n);
    dgemm('n', 'n', n, n, n, 1.0, A1.data(), n, U, n, 0.0, A3.data(), n);
  } else if (!std::strcmp(part, "f20")) {
    factor = -1.0;
    dgemm('t', 'n', n, n, n, 1.0, U, n, A, n, 0.0, A1.data(), n);
    dgemm('n', 'n', n, n, n, 1.0, A1.data(), n, V, n, 0.0, A2.data(), n);
    dgemm('t', 't', n, n, n, 1.0, V, n, A, n, 0.0, A1.data(), n);
    dgemm('n', 'n', n, n, n, 1.0, A1.data(), n, U, n, 0.0, A3.data(), n);
  } else {  // g20
    factor = -1.0;
    dgemm('t', 'n', n, n, n, 1.0, U, n, A, n, 0.0, A1.data(), n);
    dgemm('n', 'n', n, n, n, 1.0, A1.data(), n, U, n, 0.0, A2.data(), n);
    dgemm('t', 'n', n, n, n, 1.0, V, n, A, n, 0.0, A1.data(), n);
    dgemm('n', 'n', n, n, n, 1.0, A1.data(), n, V, n, 0.0, A3.data(), n);
  }
  for (size_t i = 0; i < nn; ++i) A1[i] = A2[i] - A3[i];
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) B[i + size_t(j) * n] = 0.5 * (A1[i + size_t(j) * n] + factor * A1[j + size_t(i) * n]);
}

// calculate_expectval_obo (module_operators.f90:114-135)
static void expectval_obo(const double* rho, const double* B, double& ep, double& en, int n) {
  std::vector<double> A1(size_t(n) * n);
  dgemm('n', 'n', n, n, n, 1.0, B, n, rho, n, 0.0, A1.data(), n);
  ep = en = 0.0;
  for (int i = 0; i < n / 2; ++i) {
    ep += A1[i + size_t(i) * n];
    en += A1[(i + n / 2) + size_t(i + n / 2) * n];
  }
}

// calculate_expectval_pair (module_operators.f90:273-289)
static double expectval_pair(const double* kappa, const double* B, int n) {
  std::vector<double> A(size_t(n) * n);
  dgemm('n', 't', n, n, n, 1.0, B, n, kappa, n, 0.0, A.data(), n);
  double e = 0.0;
  for (int i = 0; i < n; ++i) e += A[i + size_t(i) * n];
  return e;
}

static void densities_real(const double* U, const double* V, double* rho, double* kap, int n) {
  dgemm('n', 't', n, n, n, 1.0, V, n, V, n, 0.0, rho, n);
  dgemm('n', 't', n, n, n, 1.0, V, n, U, n, 0.0, kap, n);
}

// update_constraints_qpbasis (module_constraints.f90:381-397)
static void update_constraints_qpbasis(orc_vap* s, const double* U, const double* V) {
  const size_t n2 = size_t(s->n) * s->n;
  for (int i = 0; i < s->cdim; ++i) {
    const char* part = (i < s->cdim - s->cpair) ? "f20" : "g20";
    set_operator_qpbasis(part, U, V, s->cHO.data() + i * n2, s->c20.data() + i * n2, s->n);
  }
}

// calculate_lagrange_multipliers (module_constraints.f90:413-484)
static void calculate_lagrange_multipliers(orc_vap* s) {
  const int n = s->n, c = s->cdim;
  if (c == 0) return;
  const size_t n2 = size_t(n) * n;
  std::vector<double> A(size_t(c) * c), B(c), T(n2);
  for (int i = 0; i < c; ++i) {
    for (int j = i; j < c; ++j) {
      dgemm('n', 't', n, n, n, 1.0, s->c20.data() + i * n2, n, s->c20.data() + j * n2, n, 0.0, T.data(), n);
      double tr = 0.0;
      for (int mm = 0; mm < n; ++mm) tr += T[mm + size_t(mm) * n];
      A[j + size_t(i) * c] = tr;
      A[i + size_t(j) * c] = tr;
    }
    dgemm('n', 't', n, n, n, 1.0, s->H20v.data(), n, s->c20.data() + i * n2, n, 0.0, T.data(), n);
    double tr = 0.0;
    for (int mm = 0; mm < n; ++mm) tr += T[mm + size_t(mm) * n];
    B[i] = tr;
  }
  std::vector<int> ipiv(c);
  std::vector<double> work(c);
  int info = 0, cc = c, one = 1, lw = c;
  char up = 'U';
  p_dsysv(&up, &cc, &one, A.data(), &cc, ipiv.data(), B.data(), &cc, work.data(), &lw, &info);
  for (int i = 0; i < c; ++i) s->lam1[i] = B[i];
  if (info != 0)
    for (int i = 0; i < c; ++i) s->lam1[i] = s->lam0[i];
  for (int i = 0; i < c; ++i) s->lam0[i] = s->lam1[i];
}

// cholesky_factorization (module_constraints.f90:497-543)
static int cholesky_factorization(const double* Zm, double* L, int n) {
  const size_t nn = size_t(n) * n;
  std::vector<double> A1(nn), A2(nn), A3(size_t(n + 1) * n, 0.0);
  dgemm('t', 'n', n, n, n, 1.0, Zm, n, Zm, n, 0.0, A1.data(), n);
  for (int i = 0; i < n; ++i) {
    for (int j = i + 1; j < n; ++j) {
      A2[i + size_t(j) * n] = A1[i + size_t(j) * n];
      A2[j + size_t(i) * n] = A2[i + size_t(j) * n];
    }
    A2[i + size_t(i) * n] = A1[i + size_t(i) * n] + 1.0;
  }
  for (int i = 1; i <= n; ++i)
    for (int j = 1; j <= i; ++j) {
      const int k = 1 + i - j;
      A3[(k - 1) + size_t(j - 1) * (n + 1)] = A2[(i - 1) + size_t(j - 1) * n];
    }
  int info = 0, nn_ = n, kd = n, ldab = n + 1;
  char lo = 'L';
  p_dpbtrf(&lo, &nn_, &kd, A3.data(), &ldab, &info);
  if (info != 0) return 40;
  std::fill(L, L + nn, 0.0);
  for (int i = 1; i <= n; ++i)
    for (int j = 1; j <= n + 1 - i; ++j) {
      const int k = i - 1 + j, mm = j;
      L[(k - 1) + size_t(mm - 1) * n] = A3[(i - 1) + size_t(j - 1) * (n + 1)];
    }
  return 0;
}

// evolve_wavefunction (module_constraints.f90:559-590)
static int evolve_wavefunction(orc_vap* s, const double* Zm) {
  const int n = s->n;
  const size_t nn = size_t(n) * n;
  int info = 0, nn_ = n;
  char lo = 'L', nd = 'N';
  p_dtrtri(&lo, &nd, &nn_, s->Lchol.data(), &nn_, &info);
  if (info != 0) return 41;
  std::vector<double> A1(nn), A2(nn);
  dgemm('n', 'n', n, n, n, 1.0, s->V0.data(), n, Zm, n, 0.0, A1.data(), n);
  dgemm('n', 'n', n, n, n, 1.0, s->U0.data(), n, Zm, n, 0.0, A2.data(), n);
  for (size_t i = 0; i < nn; ++i) {
    A1[i] += s->U0[i];
    A2[i] += s->V0[i];
  }
  dgemm('n', 't', n, n, n, 1.0, A1.data(), n, s->Lchol.data(), n, 0.0, s->U1.data(), n);
  dgemm('n', 't', n, n, n, 1.0, A2.data(), n, s->Lchol.data(), n, 0.0, s->V1.data(), n);
  return 0;
}

// adjust_constraints (module_constraints.f90:270-373)
static int adjust_constraints(orc_vap* s) {
  const int n = s->n, c = s->cdim;
  const size_t n2 = size_t(n) * n;
  for (int iter = 1; iter <= 100; ++iter) {
    int st = cholesky_factorization(s->Zi.data(), s->Lchol.data(), n);
    if (st) return st;
    st = evolve_wavefunction(s, s->Zi.data());
    if (st) return st;
    densities_real(s->U1.data(), s->V1.data(), s->rhoRR.data(), s->kapRR.data(), n);
    std::vector<double> expec(c), B(c);
    for (int mm = 0; mm < c; ++mm) {
      if (mm < c - s->cpair) {
        double ep, en;
        expectval_obo(s->rhoRR.data(), s->cHO.data() + mm * n2, ep, en, n);
        expec[mm] = ep + en;
      } else {
        expec[mm] = expectval_pair(s->kapRR.data(), s->cHO.data() + mm * n2, n);
      }
    }
    int ia = 0;
    for (int i = 0; i < c; ++i) {
      B[i] = s->cval[i] - expec[i];
      if (std::fabs(B[i]) > s->ceps) ++ia;
      const char* part = (i < c - s->cpair) ? "f20" : "g20";
      set_operator_qpbasis(part, s->U1.data(), s->V1.data(), s->cHO.data() + i * n2, s->c20.data() + i * n2, n);
    }
    if (ia == 0) break;
    std::vector<double> A(size_t(c) * c), T(n2);
    for (int i = 0; i < c; ++i)
      for (int j = i; j < c; ++j) {
        dgemm('t', 'n', n, n, n, 1.0, s->c20.data() + i * n2, n, s->c20.data() + j * n2, n, 0.0, T.data(), n);
        double tr = 0.0;
        for (int mm = 0; mm < n; ++mm) tr += T[mm + size_t(mm) * n];
        A[j + size_t(i) * c] = tr;
      }
    for (int i = 0; i < c; ++i)
      for (int j = i + 1; j < c; ++j) A[i + size_t(j) * c] = A[j + size_t(i) * c];
    std::vector<int> ipiv(c);
    std::vector<double> work(c);
    int info = 0, cc = c, one = 1, lw = c;
    char up = 'U';
    p_dsysv(&up, &cc, &one, A.data(), &cc, ipiv.data(), B.data(), &cc, work.data(), &lw, &info);
    // Zi(k) += B(m) * C20_m(k) with k running row-major over (i,j) in the
    // reference; the vector is traversed linearly, so k is the flat index.
    for (size_t k = 0; k < n2; ++k)
      for (int mm = 0; mm < c; ++mm) s->Zi[k] += B[mm] * s->c20[k + mm * n2];
  }
  s->U0 = s->U1;
  s->V0 = s->V1;
  return 0;
}

int orc_angle_densities(const orc_model* m, const double* U0, const double* V0, double php, double phn, double* rho,
                        double* kLR, double* kRL, double* Aphi);

// diagonalize_hsp_and_H11 with opt = 0 (module_gradient.f90:158-453): the
// eigenvalues of h^RR and of H11 that calculate_gradient's types 1 and 2
// read.  The fields: for M = 1 those of the projection's single angle
// phi = 0 (max(proj_Mphip, proj_Mphip) == 1, :177-179), else those of the
// real densities rho^RR, kappa^RR (calculate_fields_diag, :181-185).  H11
// (calculate_H11_real, module_fields.f90:327-354) = U^T h U - V^T h^T V +
// (U^T Delta V + (U^T Delta V)^T) factor_delta; the constraint terms
// lambda_m f11(C_m) (non-pair constraints only: the pair ones keep
// constraint_11 = 0) and lambda_m C_m are subtracted (:189-218); DSYEV of both
// (:297, :416).
static void diagonalize_hsp_and_H11(orc_vap* s) {
  const int n = s->n;
  const size_t n2 = size_t(n) * n;
  std::vector<cplx> rho(n2), kap(n2), kRL(n2), gam(n2), hsp(n2), dLR(n2);
  if (s->Mp == 1) {
    orc_angle_densities(s->m, s->U0.data(), s->V0.data(), 0.0, 0.0, reinterpret_cast<double*>(rho.data()),
                        reinterpret_cast<double*>(kap.data()), reinterpret_cast<double*>(kRL.data()), nullptr);
  } else {
    for (size_t i = 0; i < n2; ++i) {
      rho[i] = s->rhoRR[i] * zone;
      kap[i] = s->kapRR[i] * zone;
    }
  }
  calculate_fields_diag(s->m, rho.data(), kap.data(), gam.data(), hsp.data(), dLR.data(), nullptr, s->nthreads);
  std::vector<double> h(n2), d(n2), A1(n2), A2(n2), A3(n2), A4(n2), H11(n2);
  for (size_t i = 0; i < n2; ++i) {
    h[i] = hsp[i].real();
    d[i] = dLR[i].real();  // real(Delta^RL) = real(conj(Delta^LR))
  }
  const double* U = s->U0.data();
  const double* V = s->V0.data();
  dgemm('t', 'n', n, n, n, 1.0, U, n, h.data(), n, 0.0, A1.data(), n);
  dgemm('n', 'n', n, n, n, 1.0, A1.data(), n, U, n, 0.0, A2.data(), n);
  dgemm('t', 't', n, n, n, 1.0, V, n, h.data(), n, 0.0, A1.data(), n);
  dgemm('n', 'n', n, n, n, 1.0, A1.data(), n, V, n, 0.0, A3.data(), n);
  dgemm('t', 'n', n, n, n, 1.0, U, n, d.data(), n, 0.0, A1.data(), n);
  dgemm('n', 'n', n, n, n, 1.0, A1.data(), n, V, n, 0.0, A4.data(), n);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      const size_t ij = i + size_t(j) * n, ji = j + size_t(i) * n;
      H11[ij] = A2[ij] - A3[ij] + (A4[ij] + A4[ji]) * s->factor_delta;
    }
  std::vector<double> c11(n2);
  for (int m = 0; m < s->cdim; ++m) {
    const double* cHO = s->cHO.data() + m * n2;
    if (m < s->cdim - s->cpair) {
      set_operator_qpbasis("f11", U, V, cHO, c11.data(), n);
      for (size_t i = 0; i < n2; ++i) H11[i] -= s->lam1[m] * c11[i];
    }
    for (size_t i = 0; i < n2; ++i) h[i] -= s->lam1[m] * cHO[i];
  }
  s->eig_hsp.assign(n, 0.0);
  s->eig_H11.assign(n, 0.0);
  char jv = 'V', up = 'U';
  int nn_ = n, lwork = 3 * n - 1, info = 0;
  std::vector<double> work(lwork);
  p_dsyev(&jv, &up, &nn_, h.data(), &nn_, s->eig_hsp.data(), work.data(), &lwork, &info);
  s->info_hsp = info;
  info = 0;
  p_dsyev(&jv, &up, &nn_, H11.data(), &nn_, s->eig_H11.data(), work.data(), &lwork, &info);
  s->info_H11 = info;
}

// the step sizes of calculate_gradient (module_gradient.f90:86-119): type 0
// the input eta and mu; type 1 from the H11 eigenvalues, type 2 from those
// of h^RR (heavy ball with approximate optimal parameters); a failed
// diagonalisation falls back to type 0
static void gradient_parameters(int type, const double* eig_hsp, const double* eig_H11, int info_hsp, int info_H11,
                                int n, double eta_in, double mu_in, double& eta, double& mu) {
  int opt = type;
  if (info_H11 != 0 && type == 1) opt = 0;
  if (info_hsp != 0 && type == 2) opt = 0;
  eta = eta_in;
  mu = mu_in;
  if (opt == 0) return;
  const double* e = (opt == 1) ? eig_H11 : eig_hsp;
  double amax = 0.0, amin = 1.0e300;
  for (int i = 0; i < n; ++i) {
    amax = std::max(amax, std::fabs(e[i]));
    amin = std::min(amin, std::fabs(e[i]));
  }
  const double emax = (opt == 1 ? 4.0 : 2.0) * amax, emin = 2.0 * amin;
  const double cond = emax / emin;
  const double t = 2.0 / (std::sqrt(emax) + std::sqrt(emin));
  const double r = (std::sqrt(cond) - 1.0) / (std::sqrt(cond) + 1.0);
  eta = t * t;
  mu = r * r;
}

// calculate_gradient (module_gradient.f90:79-143)
static void calculate_gradient(orc_vap* s) {
  const int n = s->n;
  const size_t n2 = size_t(n) * n;
  double eta = s->eta, mu = s->mu;
  if (s->gtype > 0)
    gradient_parameters(s->gtype, s->eig_hsp.data(), s->eig_H11.data(), s->info_hsp, s->info_H11, n, s->eta, s->mu,
                        eta, mu);
  s->eta_used = eta;
  s->mu_used = mu;
  for (size_t i = 0; i < n2; ++i) {
    double sg = 0.0;
    for (int j = 0; j < s->cdim; ++j) sg += s->lam1[j] * s->c20[j * n2 + i];
    s->Zi[i] = -eta * (s->H20v[i] - sg) + mu * s->Zim1[i];
  }
  std::vector<double> Z2(n2);
  dgemm('t', 'n', n, n, n, 1.0, s->Zi.data(), n, s->Zi.data(), n, 0.0, Z2.data(), n);
  double sum = 0.0;
  for (int i = 0; i < n; ++i) sum += Z2[i + size_t(i) * n];
  s->gnorm = std::sqrt(sum) / eta;
}

orc_vap* orc_vap_new(const orc_model* m, const double* U0, const double* V0, int Mp, int Mn, double facpi, double Z,
                     double N, int gtype, double eta, double mu, double geps, int cdim, int cpair,
                     const double* cHO, const double* cval, double ceps, double factor_delta, int nthreads) {
  auto* s = new orc_vap();
  const int n = m->n;
  const size_t n2 = size_t(n) * n;
  s->m = m;
  s->n = n;
  s->U0.assign(U0, U0 + n2);
  s->V0.assign(V0, V0 + n2);
  s->U1.assign(n2, 0.0);
  s->V1.assign(n2, 0.0);
  s->rhoRR.assign(n2, 0.0);
  s->kapRR.assign(n2, 0.0);
  s->Mp = Mp;
  s->Mn = Mn;
  s->facpi = facpi;
  s->Z = Z;
  s->N = N;
  s->gtype = gtype;
  s->eta = eta;
  s->mu = mu;
  s->geps = geps;
  s->cdim = cdim;
  s->cpair = cpair;
  s->cHO.assign(cHO, cHO + size_t(cdim) * n2);
  s->cval.assign(cval, cval + cdim);
  s->ceps = ceps;
  s->factor_delta = factor_delta;
  s->c20.assign(size_t(cdim) * n2, 0.0);
  s->lam0.assign(cdim, 0.0);
  s->lam1.assign(cdim, 0.0);
  s->Zi.assign(n2, 0.0);
  s->Zim1.assign(n2, 0.0);
  s->H20v.assign(n2, 0.0);
  s->Lchol.assign(n2, 0.0);
  s->nthreads = nthreads;
  return s;
}
void orc_vap_free(orc_vap* s) { delete s; }

// The first adjust_constraints call before the loop (taurus_vap.f90:62-66).
int orc_vap_initial_adjust(orc_vap* s) { return adjust_constraints(s); }

// One gradient iteration (taurus_vap.f90:77-123) with gradient_type 0, 1 or 2.
// Returns 0 (continue), 1 (converged), 2 (particle numbers wrong three times
// in the last five iterations: the reference stops), or an error code.
int orc_vap_iterate(orc_vap* s, double* info /* [gnorm, E, Z, varZ, N, varN] */) {
  const int n = s->n;
  std::fill(s->H20v.begin(), s->H20v.end(), 0.0);
  densities_real(s->U0.data(), s->V0.data(), s->rhoRR.data(), s->kapRR.data(), n);
  update_constraints_qpbasis(s, s->U0.data(), s->V0.data());
  orc_pnp_out o;
  int st = orc_project(s->m, s->U0.data(), s->V0.data(), s->Mp, s->Mn, s->facpi, s->Z, s->N, s->factor_delta,
                       s->occeps, s->allemp, &o, s->H20v.data(), nullptr, nullptr, nullptr, nullptr, s->nthreads);
  if (st) return 100 + st;
  calculate_lagrange_multipliers(s);
  if (s->gtype > 0) diagonalize_hsp_and_H11(s);
  calculate_gradient(s);
  const cplx over(o.over[0], o.over[1]);
  const double ener = (cplx(o.ener[0], o.ener[1]) / over).real();
  const double prot = (cplx(o.prot[0], o.prot[1]) / over).real();
  const double neut = (cplx(o.neut[0], o.neut[1]) / over).real();
  double prot2 = (cplx(o.prot2[0], o.prot2[1]) / over).real();
  double neut2 = (cplx(o.neut2[0], o.neut2[1]) / over).real();
  prot2 = std::fabs(prot2 - prot * prot);
  neut2 = std::fabs(neut2 - neut * neut);
  info[0] = s->gnorm;
  info[1] = ener;
  info[2] = prot;
  info[3] = prot2;
  info[4] = neut;
  info[5] = neut2;
  for (int i = 4; i >= 1; --i) s->control_NZ[i] = s->control_NZ[i - 1];
  s->control_NZ[0] = (std::fabs(prot - s->Z) > 0.5 || std::fabs(neut - s->N) > 0.5) ? 1 : 0;
  int sumc = 0;
  for (int i = 0; i < 5; ++i) sumc += s->control_NZ[i];
  if (sumc >= 3) return 2;
  if (s->gnorm <= s->geps) return 1;
  st = adjust_constraints(s);
  if (st) return 100 + st;
  s->Zim1 = s->Zi;
  return 0;
}

void orc_vap_get_state(const orc_vap* s, double* U, double* V, double* Zi, double* H20v) {
  const size_t n2 = size_t(s->n) * s->n;
  if (U) std::memcpy(U, s->U0.data(), sizeof(double) * n2);
  if (V) std::memcpy(V, s->V0.data(), sizeof(double) * n2);
  if (Zi) std::memcpy(Zi, s->Zi.data(), sizeof(double) * n2);
  if (H20v) std::memcpy(H20v, s->H20v.data(), sizeof(double) * n2);
}

void orc_vap_get_multipliers(const orc_vap* s, double* lam) {
  for (int i = 0; i < s->cdim; ++i) lam[i] = s->lam1[i];
}

// The eigenvalues of h^RR and H11, their DSYEV infos and the step sizes
// (eta, mu) of the last iteration (gradient types 1 and 2).
void orc_vap_get_step(const orc_vap* s, double* eig_hsp, double* eig_H11, int* infos, double* eta_mu) {
  for (int i = 0; i < s->n && !s->eig_hsp.empty(); ++i) {
    eig_hsp[i] = s->eig_hsp[i];
    eig_H11[i] = s->eig_H11[i];
  }
  infos[0] = s->info_hsp;
  infos[1] = s->info_H11;
  eta_mu[0] = s->eta_used;
  eta_mu[1] = s->mu_used;
}

// diagonalize_hsp_and_H11(0) for a state (U, V) of a projection with
// Mp angles per proton, with multipliers lam of the constraints cHO (cdim
// operators, the last cpair of them pair operators).
int orc_diagonalize_hsp_and_H11(const orc_model* m, const double* U, const double* V, int Mp, int cdim, int cpair,
                                const double* lam, const double* cHO, double factor_delta, double* eig_hsp,
                                double* eig_H11, int* infos, int nthreads) {
  orc_vap s;
  const int n = m->n;
  const size_t n2 = size_t(n) * n;
  s.m = m;
  s.n = n;
  s.Mp = Mp;
  s.U0.assign(U, U + n2);
  s.V0.assign(V, V + n2);
  s.rhoRR.assign(n2, 0.0);
  s.kapRR.assign(n2, 0.0);
  densities_real(U, V, s.rhoRR.data(), s.kapRR.data(), n);
  s.cdim = cdim;
  s.cpair = cpair;
  s.cHO.assign(cHO, cHO + size_t(cdim) * n2);
  s.lam1.assign(lam, lam + cdim);
  s.factor_delta = factor_delta;
  s.nthreads = nthreads;
  diagonalize_hsp_and_H11(&s);
  std::copy(s.eig_hsp.begin(), s.eig_hsp.end(), eig_hsp);
  std::copy(s.eig_H11.begin(), s.eig_H11.end(), eig_H11);
  infos[0] = s.info_hsp;
  infos[1] = s.info_H11;
  return 0;
}

// Thouless map Z -> (U1, V1) of a state (cholesky_factorization +
// evolve_wavefunction), used by the adjoint checks.
int orc_thouless_evolve(const double* U0, const double* V0, const double* Zm, int n, double* U1, double* V1) {
  orc_vap s;
  const size_t n2 = size_t(n) * n;
  s.n = n;
  s.U0.assign(U0, U0 + n2);
  s.V0.assign(V0, V0 + n2);
  s.U1.assign(n2, 0.0);
  s.V1.assign(n2, 0.0);
  s.Lchol.assign(n2, 0.0);
  int st = cholesky_factorization(Zm, s.Lchol.data(), n);
  if (st) return st;
  st = evolve_wavefunction(&s, Zm);
  if (st) return st;
  std::memcpy(U1, s.U1.data(), sizeof(double) * n2);
  std::memcpy(V1, s.V1.data(), sizeof(double) * n2);
  return 0;
}

}  // extern "C"
