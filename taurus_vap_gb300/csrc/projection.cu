// The gauge-angle loop of project_wavefunction (module_projection.f90:201-373)
// for all angles at once, followed by calculate_projected_H20 (:729-759).
//
// Per call (state U0, V0 real n x n):
//   canonical basis (construct_canonical_basis, module_wavefunctions.f90:777-945)
//   angle-independent real blocks:  V_t^T V_t, U_t^T U_t, V_t^T U_t, U_t^T V_t,
//       D_t^T D_t  for t = protons, neutrons, so that for every angle
//       U_phi = sum_t e^{-i phi_t} V_t^T V_t + e^{i phi_t} U_t^T U_t,
//       V_phi = sum_t e^{i phi_t} V_t^T U_t + e^{-i phi_t} U_t^T V_t,
//       R_n   = sum_t e^{i phi_t} D_t^T D_t
//     replace the rotation and Thouless ZGEMMs (:641-653, :695-700, :847-848)
//     by O(n^2) combinations;
//   per angle, batched:  A_phi (Thouless solve), U~ = U + V A, V~ = V + U A,
//     rho = V~ V^T, kappaLR = V~ U^T, kappaRL = V U~^T, the fields, particle
//     number and energy traces, H20 and the Pfaffian overlap;
//   sum_gauge over angles and the projected gradient.
//
// Angle folding: for proj_facpi = 2 pi and integer particle numbers the angle
// pairs (phi_p, phi_n) and (-phi_p, -phi_n) carry complex-conjugate weights and
// complex-conjugate rotated quantities (U0, V0 are real), so only one member of
// each pair is computed and it enters the sums as 2 Re(w o X).
//
// Overlap: the reference evaluates Pf(M) for the 2 n2 x 2 n2 matrix
//   M = [[A1, -P], [P^T, C0]],  P = leading block of R_n2^{-1}
// after an LU and an inverse of R_n2 (:840-933).  Here the Schur-complement
// identities Pf([[A, B], [-B^T, C]]) = Pf(A) Pf(C + B^T A^{-1} B) and
// Pf(X^T Y X) = det(X) Pf(Y) give the same number as
//   overlap = signfac det(R22) Pf(A1) Pf(A1^{-1} + S^T C0 S) exp(ovac),
//   S = R11 - R12 R22^{-1} R21  (R22: the nocc occupied states),
// which needs one Pfaffian of size n2 - nocc and no inverse of R_n2.

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "tvap_internal.cuh"

namespace tvap {

// ---------------------------------------------------------------------------
// workspace
// ---------------------------------------------------------------------------
struct Workspace {
  int n = 0, G = 0;
  // real n x n (V and U adjacent: VU = [V | U], n x 2n)
  double *VU = nullptr, *U = nullptr, *V = nullptr, *rho = nullptr, *kap = nullptr, *jac = nullptr, *D = nullptr,
         *evals = nullptr, *jwork = nullptr, *rhoc = nullptr, *kapc = nullptr, *tmp = nullptr, *blocks = nullptr;
  // canonical summary (device): ints [nocc, nemp, bad], doubles [ovac, logPfA1, signPfA1], voveru[n]
  int* canon_i = nullptr;
  double* canon_d = nullptr;
  // per angle complex n x n (batch G)
  double2 *Uphi = nullptr, *Vphi = nullptr, *W = nullptr, *A = nullptr, *Ut = nullptr, *Vt = nullptr,
          *X = nullptr, *Y = nullptr, *T = nullptr, *Rn = nullptr, *K = nullptr, *SZ = nullptr;
  // angle-innermost (n*n*G)
  double2 *rhoL = nullptr, *kLR = nullptr, *kRL = nullptr, *gam = nullptr, *hsp = nullptr, *dLR = nullptr,
          *dRL = nullptr;
  // per angle scalars
  double2 *ephase = nullptr;  // [G][2] e^{i phi_p}, e^{i phi_n}
  double2 *weight = nullptr;  // [G] w_p w_n
  double* mult = nullptr;     // [G] 1 or 2 (folded)
  double2 *obs = nullptr;     // [G][8]: over, ener, prot, neut, prot2, neut2, logdet terms
  double2 *pf = nullptr;      // [2G] (log|Pf|, phase)
  double2 *detR22 = nullptr;  // [2G] (log|det|, phase)
  double2 *coefA = nullptr;   // [G] c_b (multiplicity-weighted w*o)
  double2 *coefAE = nullptr;  // [G] c_b E_b
  // sums
  double2 *pA = nullptr, *pH = nullptr, *pAH = nullptr, *pscal = nullptr;
  double* H20v = nullptr;
  // eigenvector refinement (warm start from the previous canonical basis):
  // XB = [X0 | rho X0 | X1 | rho X1], RS = [X^T X | X^T rho X]
  double *XB = nullptr, *Xr = nullptr, *Xn = nullptr, *RS = nullptr, *Rr = nullptr, *Br = nullptr, *Sr = nullptr,
         *Mr = nullptr, *lam = nullptr, *rscal = nullptr;
  // pairing bases of the degenerate subspaces of the canonical basis (Q, then
  // Q^T kappa Q, kSubMax^2 each)
  double* schq = nullptr;
  // overlap chain scratch (runs on the second stream)
  double2 *OW = nullptr, *OX = nullptr, *OY = nullptr;
  int* rflag = nullptr;
  // canonical-basis clusters: cluster of each refined column (its first
  // position in the sorted order of the first refinement step), the
  // columns in cluster order, and (start, size) of the clusters left to
  // the FP64 Jacobi of their block
  int *cid = nullptr, *cperm = nullptr, *bigd = nullptr;
  int* piv = nullptr;  // [G][n] row interchanges of the Thouless LU
  // [G][panel][L11^-1, U11^-1] (kPanelMax^2 each) of the Thouless LU
  double2* Tinv = nullptr;
  // the angle tables in ephase/weight/mult were made for these options
  bool angles_valid = false;
  int ang_Mp = 0, ang_Mn = 0, ang_mode = 0;
  double ang_facpi = 0.0, ang_vz = 0.0, ang_vn = 0.0;
  double2* tpart = nullptr;  // [kTraceChunks][G][9] partial traces
  bool have_basis = false;
  size_t bytes = 0;
};

namespace {

template <typename T>
int dalloc(T** p, size_t count, size_t& total) {
  if (count == 0) count = 1;
  TVAP_CUDA(cudaMalloc(p, sizeof(T) * count));
  total += sizeof(T) * count;
  return TVAP_OK;
}

constexpr int kPanelMax = 32;  // columns per panel of the Thouless solve
constexpr int kSubMax = 64;    // largest degenerate subspace of the canonical basis
constexpr int kCfBigSlots = 16;  // clusters of the refined basis passed to the FP64 Jacobi per attempt

// double2 entries per angle of Workspace::Tinv
size_t tinv_stride(int n) { return size_t((n + kPanelMax - 1) / kPanelMax) * 2 * kPanelMax * kPanelMax; }

void ws_free(Workspace* w) {
  void* ptrs[] = {w->VU,  w->rho,    w->kap,   w->jac,    w->D,     w->evals,  w->jwork, w->rhoc,
                  w->kapc, w->tmp,  w->blocks, w->canon_i, w->canon_d, w->Uphi, w->Vphi,   w->W,     w->A,
                  w->Ut,  w->Vt,    w->X,      w->Y,     w->T,      w->Rn,    w->K,      w->SZ,    w->rhoL,
                  w->kLR, w->kRL,   w->gam,    w->hsp,   w->dLR,    w->dRL,   w->ephase, w->weight, w->mult,
                  w->obs, w->pf,    w->detR22, w->coefA, w->coefAE, w->pA,    w->pH,     w->pAH,   w->pscal,
                  w->H20v,  w->XB,    w->RS,     w->Br,    w->Mr,     w->lam,   w->rscal,
                  w->rflag, w->cid,   w->cperm,  w->bigd,   w->OW,  w->OX,   w->OY,    w->piv,   w->Tinv,
                  w->tpart, w->schq};
  for (void* p : ptrs) cudaFree(p);
  *w = Workspace();
}

int ws_ensure(tvap_ctx* c, int G) {
  Workspace* w = c->ws;
  const int n = c->n;
  if (w && w->n == n && w->G >= G) return TVAP_OK;
  if (!w) {
    w = new Workspace();
    c->ws = w;
  } else {
    ws_free(w);
  }
  w->n = n;
  w->G = G;
  const size_t nn = size_t(n) * n, nG = nn * G;
  size_t& t = w->bytes;
  int rc = TVAP_OK;
#define A_(p, cnt) \
  if ((rc = dalloc(&w->p, (cnt), t)) != TVAP_OK) return rc;
  A_(VU, 2 * nn) A_(rho, nn) A_(kap, nn) A_(jac, nn) A_(D, nn) A_(evals, n) A_(jwork, 2 * n + 2)
  A_(rhoc, nn) A_(kapc, nn) A_(tmp, nn + n) A_(blocks, 12 * nn) A_(canon_i, 8) A_(canon_d, 8 + n)
  A_(Uphi, nG) A_(Vphi, nG) A_(W, 2 * nG) A_(A, nG) A_(Ut, nG) A_(Vt, nG) A_(X, nG) A_(Y, nG) A_(T, nG)
  A_(Rn, nG) A_(K, nG) A_(SZ, nG) A_(rhoL, nG) A_(kLR, nG) A_(kRL, nG) A_(gam, nG) A_(hsp, nG) A_(dLR, nG)
  A_(dRL, nG) A_(ephase, 2 * G) A_(weight, G) A_(mult, G) A_(obs, 8 * G) A_(pf, 2 * G) A_(detR22, 2 * G)
  A_(coefA, G) A_(coefAE, G) A_(pA, nn) A_(pH, nn) A_(pAH, nn) A_(pscal, 8) A_(H20v, nn)
  A_(XB, 4 * nn) A_(RS, 2 * nn) A_(Br, nn) A_(Mr, nn) A_(lam, n) A_(rscal, 8) A_(rflag, 8)
  A_(cid, n) A_(cperm, n) A_(bigd, 2 * kCfBigSlots)
  A_(OW, nG) A_(OX, nG) A_(OY, nG) A_(piv, size_t(n) * G)
  A_(Tinv, size_t(G) * tinv_stride(n)) A_(tpart, size_t(G) * 9 * 256) A_(schq, 2 * kSubMax * kSubMax)
#undef A_
  w->V = w->VU;
  w->U = w->VU + nn;
  w->Xr = w->XB;
  w->Xn = w->XB + 2 * nn;
  w->Rr = w->RS;
  w->Sr = w->RS + nn;
  return TVAP_OK;
}

// ---------------------------------------------------------------------------
// small kernels
// ---------------------------------------------------------------------------

__device__ __forceinline__ double warp_sum_d(double v) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

// One warp: column c of Q (d x d, column-major) orthogonalised against
// columns 0 .. c-1 (twice, classical Gram-Schmidt) and normalised; false if
// nothing of it is left.
__device__ bool pair_orthonormalise(int d, double* Q, int c) {
  const int lane = threadIdx.x & 31;
  for (int pass = 0; pass < 2; ++pass)
    for (int cc = 0; cc < c; ++cc) {
      double dot = 0.0;
      for (int i = lane; i < d; i += 32) dot = fma(Q[i + cc * d], Q[i + c * d], dot);
      dot = warp_sum_d(dot);
      for (int i = lane; i < d; i += 32) Q[i + c * d] = fma(-dot, Q[i + cc * d], Q[i + c * d]);
      __syncwarp();
    }
  double nrm = 0.0;
  for (int i = lane; i < d; i += 32) nrm = fma(Q[i + c * d], Q[i + c * d], nrm);
  nrm = warp_sum_d(nrm);
  if (!(nrm > 1.0e-24)) return false;
  const double r = 1.0 / sqrt(nrm);
  for (int i = lane; i < d; i += 32) Q[i + c * d] *= r;
  __syncwarp();
  return true;
}

// Canonical form of kappa on a degenerate subspace of rho (rows and columns
// k0 .. k0+d-1 of the basis; the reference Schur-reduces it with DGEES,
// module_wavefunctions.f90:873-906).  On such a subspace rho = v^2 1 and, the
// state being a quasiparticle vacuum, kappa^2 = -(v^2 - v^4) 1: kappa = b J
// with J orthogonal and skew.  A pairing basis follows without an eigen
// solver: q1 = a unit vector of the subspace (the basis vector least covered
// by the columns so far), q2 = kappa q1 / |kappa q1|; kappa maps span{q1, q2}
// onto itself, so the next pair starts orthogonal to both.  Q^T kappa Q is
// then block diagonal with 2 x 2 blocks; any remaining coupling (a subspace
// that is not exactly degenerate) larger than 1e-10 of the largest entry is
// reported as a failure.  Kappa's subspace block is replaced by Q^T kappa Q
// and D's columns by D Q (rho's diagonal is left as it is, as in the
// reference).  Whole CTA; Q and T = kappa Q in global scratch (2 kSubMax^2).
__device__ bool pair_subspace(int n, int k0, int d, double* kapc, double* D, double* Q, double* T) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31;
  __shared__ int s_ok;
  __shared__ double s_kmax;
  auto K = [&](int i, int j) -> double& { return kapc[(k0 + i) + size_t(k0 + j) * n]; };
  if (tid < 32) {
    bool ok = true;
    for (int p = 0; p < d / 2 && ok; ++p) {
      const int c0 = 2 * p;
      // the basis vector with the largest part outside the columns so far
      double best = -1.0;
      int bi = d;
      for (int i = lane; i < d; i += 32) {
        double r = 1.0;
        for (int c = 0; c < c0; ++c) r = fma(-Q[i + c * d], Q[i + c * d], r);
        if (r > best) {
          best = r;
          bi = i;
        }
      }
      for (int off = 16; off > 0; off >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, off);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      for (int i = lane; i < d; i += 32) Q[i + c0 * d] = (i == bi) ? 1.0 : 0.0;
      __syncwarp();
      ok = pair_orthonormalise(d, Q, c0);
      if (!ok) break;
      for (int i = lane; i < d; i += 32) {
        double w = 0.0;
        for (int j = 0; j < d; ++j) w = fma(K(i, j), Q[j + c0 * d], w);
        Q[i + (c0 + 1) * d] = w;
      }
      __syncwarp();
      ok = pair_orthonormalise(d, Q, c0 + 1);
    }
    if (lane == 0) s_ok = ok ? 1 : 0;
  }
  __syncthreads();
  if (!s_ok) return false;
  // T = kappa Q, then kappa <- Q^T T on the subspace
  for (int e = tid; e < d * d; e += nt) {
    const int i = e % d, c = e / d;
    double v = 0.0;
    for (int j = 0; j < d; ++j) v = fma(K(i, j), Q[j + c * d], v);
    T[e] = v;
  }
  __syncthreads();
  if (tid == 0) s_kmax = 0.0;
  __syncthreads();
  double kmax = 0.0;
  for (int e = tid; e < d * d; e += nt) {
    const int i = e % d, c = e / d;
    double v = 0.0;
    for (int j = 0; j < d; ++j) v = fma(Q[j + i * d], T[j + c * d], v);
    K(i, c) = v;
    kmax = fmax(kmax, fabs(v));
  }
  // the largest entry (non-negative doubles order as their bit patterns)
  atomicMax(reinterpret_cast<unsigned long long*>(&s_kmax), __double_as_longlong(kmax));
  __syncthreads();
  const double tol = 1.0e-10 * s_kmax;
  int bad = 0;
  for (int e = tid; e < d * d; e += nt) {
    const int i = e % d, c = e / d;
    if ((i >> 1) != (c >> 1) && fabs(K(i, c)) > tol) bad = 1;
  }
  // D's subspace columns: D <- D Q, one row per thread
  for (int r = tid; r < n; r += nt) {
    double row[kSubMax];
    for (int j = 0; j < d; ++j) row[j] = D[r + size_t(k0 + j) * n];
    for (int c = 0; c < d; ++c) {
      double v = 0.0;
      for (int j = 0; j < d; ++j) v = fma(row[j], Q[j + c * d], v);
      D[r + size_t(k0 + c) * n] = v;
    }
  }
  return __syncthreads_or(bad) == 0;
}

// canonical-basis bookkeeping (construct_canonical_basis after the
// diagonalisation, module_wavefunctions.f90:818-945, and the v/u extraction
// of project_wavefunction, module_projection.f90:219-234).  One CTA.
__global__ void canon_kernel(int n, const double* __restrict__ rhoc, double* __restrict__ kapc, double* D,
                             double* sch, double eps, int allemp, int* canon_i, double* canon_d) {
  __shared__ int submax[1024];
  __shared__ double rd[256];
  __shared__ int ri[3][256];
  __shared__ int s_nocc, s_nemp, s_nlow, s_bad, s_nsub;
  __shared__ int s_sub[2][kSubMax];
  const int tid = threadIdx.x, nt = blockDim.x;
  // occupation counts and ovac = sum log u over paired states (parallel)
  double ov = 0.0;
  int cocc = 0, cemp = 0, clow = 0;
  for (int i = tid; i < n; i += nt) {
    const double v2 = fabs(rhoc[i + size_t(i) * n]);
    if (v2 >= 1.0 - eps)
      ++cocc;
    else if (v2 <= eps && allemp == 0)
      ++cemp;
    else
      ov += log(sqrt(fabs(1.0 - v2)));
    if (v2 <= eps) ++clow;
  }
  rd[tid] = ov;
  ri[0][tid] = cocc;
  ri[1][tid] = cemp;
  ri[2][tid] = clow;
  __syncthreads();
  for (int s = nt / 2; s > 0; s >>= 1) {
    if (tid < s) {
      rd[tid] += rd[tid + s];
      for (int q = 0; q < 3; ++q) ri[q][tid] += ri[q][tid + s];
    }
    __syncthreads();
  }
  if (tid == 0) {
    s_nocc = ri[0][0];
    s_nemp = ri[1][0];
    s_nlow = ri[2][0];
    s_bad = 0;
    canon_d[0] = (n - s_nocc - s_nemp == 0) ? 0.0 : rd[0];
  }
  __syncthreads();
  const int nocc = s_nocc, nemp = s_nemp, nlow = s_nlow;
  // submax (1-based indices as in the reference)
  for (int i = 1 + nemp + tid; i <= n - nocc; i += nt) {
    int sm = i;
    for (int j = i + 1; j <= n - nocc; ++j)
      if (fabs(kapc[(j - 1) + size_t(i - 1) * n]) > sqrt(eps) * 1.0e-2) sm = j;
    submax[i] = sm;
  }
  __syncthreads();
  if (tid == 0) {
    // subspace dimensions (the reference merges overlapping ranges)
    int k = 1 + nemp;
    while (k < n - nocc) {
      const int j = submax[k];
      int mx = 0;
      for (int t = k; t <= j; ++t) mx = max(mx, submax[t]);
      for (int t = k; t <= j; ++t) submax[t] = mx;
      if (mx == j) k = j + 1;
    }
    k = 1 + nemp;
    s_nsub = 0;
    while (k < n - nocc) {
      int d = submax[k] - k + 1;
      if (d > 2 && (d % 2) != 0) d = 2;  // as the reference does (with a warning)
      if (d > 2) {
        // a degenerate subspace: put into canonical form below
        if (d <= kSubMax && s_nsub < kSubMax) {
          s_sub[0][s_nsub] = k - 1;
          s_sub[1][s_nsub] = d;
          ++s_nsub;
        } else {
          s_bad = 1;
        }
      }
      k += d;
    }
    if ((n - nocc - nemp) % 2 != 0) s_bad = 1;
  }
  __syncthreads();
  for (int q = 0; q < s_nsub; ++q)
    if (!pair_subspace(n, s_sub[0][q], s_sub[1][q], kapc, D, sch, sch + kSubMax * kSubMax) && tid == 0) s_bad = 1;
  __syncthreads();
  // v/u with the sign of kappa in the canonical basis; the paired states are
  // contiguous after the nlow states with v^2 <= eps, so the reference's
  // running counter k of paired states is i - 1 - nlow
  double* vu = canon_d + 8;
  for (int i = 1 + tid; i <= n; i += nt) {
    const double v2 = fabs(rhoc[(i - 1) + size_t(i - 1) * n]);
    const double v = sqrt(v2), u = sqrt(fabs(1.0 - v2));
    const bool paired = !(v2 > 1.0 - eps) && !(v2 <= eps);
    double val = 0.0;
    if (i >= 1 + nemp && i <= n - nocc) {
      // zVc(i, i+1) / zVc(i, i-1) as construct_canonical_basis places them
      // (running count kk of paired states), read back with the parity of
      // j = i - nemp as project_wavefunction does
      const int kk = i - 1 - nlow;
      const double vplus = (paired && kk % 2 == 0 && i < n) ? copysign(v, kapc[(i - 1) + size_t(i) * n]) : 0.0;
      const double vminus = (paired && kk % 2 == 1) ? copysign(v, kapc[(i - 1) + size_t(i - 2) * n]) : 0.0;
      const int j = i - nemp;
      val = ((j % 2) == 1 ? vplus : vminus) / u;
    }
    vu[i - 1] = val;
  }
  __syncthreads();
  // Pf(A1) = prod over odd i of vu(i + nemp), as (log|.|, sign)
  const int nbloc = n - nocc - nemp;
  double lp = 0.0;
  int neg = 0, zero = 0;
  for (int i = 1 + 2 * tid; i <= nbloc - 1; i += 2 * nt) {
    const double a = vu[i + nemp - 1];
    if (a == 0.0)
      zero = 1;
    else
      lp += log(fabs(a));
    if (a < 0.0) neg ^= 1;
  }
  rd[tid] = lp;
  ri[0][tid] = neg;
  ri[1][tid] = zero;
  __syncthreads();
  for (int s = nt / 2; s > 0; s >>= 1) {
    if (tid < s) {
      rd[tid] += rd[tid + s];
      ri[0][tid] ^= ri[0][tid + s];
      ri[1][tid] |= ri[1][tid + s];
    }
    __syncthreads();
  }
  if (tid == 0) {
    canon_d[1] = rd[0];
    canon_d[2] = ri[0][0] ? -1.0 : 1.0;
    canon_i[0] = nocc;
    canon_i[1] = nemp;
    canon_i[2] = s_bad | ri[1][0];
  }
}

// per angle: U_phi, V_phi from the angle-independent blocks of U and V
__global__ void build_uv_kernel(int n, int G, const double* __restrict__ blk, const double2* __restrict__ eph,
                                double2* __restrict__ Uphi, double2* __restrict__ Vphi) {
  const size_t nn = size_t(n) * n;
  const size_t idx = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (idx >= nn * G) return;
  const int b = int(idx / nn);
  const size_t e = idx % nn;
  const double2 pp = eph[2 * b], pn = eph[2 * b + 1];  // e^{i phi_p}, e^{i phi_n}
  // blocks: the Gram matrices C_t = W_t^T W_t of W_t = [V_t | U_t] (rows of
  // isospin t; 2n x 2n at blk + 4 n^2 t), then D_p^T D_p, D_n^T D_n
  const int i = int(e % n), j = int(e / n);
  const size_t n2 = 2 * size_t(n);
  const double* Cp = blk;
  const double* Cn = blk + 4 * nn;
  const size_t vv = i + j * n2, vu = i + (n + j) * n2, uv = (n + i) + j * n2, uu = (n + i) + (n + j) * n2;
  const double vvp = Cp[vv], vvn = Cn[vv], uup = Cp[uu], uun = Cn[uu];
  const double vup = Cp[vu], vun = Cn[vu], uvp = Cp[uv], uvn = Cn[uv];
  double2 up;
  up.x = (vvp + uup) * pp.x + (vvn + uun) * pn.x;
  up.y = (uup - vvp) * pp.y + (uun - vvn) * pn.y;
  double2 vp;
  vp.x = (vup + uvp) * pp.x + (vun + uvn) * pn.x;
  vp.y = (vup - uvp) * pp.y + (vun - uvn) * pn.y;
  Uphi[idx] = up;
  Vphi[idx] = vp;
}

// per angle: the trailing n2 x n2 block (n2 = n - nemp) of R_n = D^T R D
__global__ void build_rn_kernel(int n, int n2, int G, const double* __restrict__ blk,
                                const double2* __restrict__ eph, double2* __restrict__ Rn) {
  const size_t nn = size_t(n) * n, m2 = size_t(n2) * n2;
  const size_t idx = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (idx >= m2 * G) return;
  const int b = int(idx / m2);
  const size_t e2 = idx % m2;
  const int i2 = int(e2 % n2), j2 = int(e2 / n2);
  const int nemp = n - n2;
  const size_t e = size_t(i2 + nemp) + size_t(j2 + nemp) * n;
  const double2 pp = eph[2 * b], pn = eph[2 * b + 1];
  const double dp = blk[8 * nn + e], dn = blk[9 * nn + e];
  Rn[idx] = make_double2(dp * pp.x + dn * pn.x, dp * pp.y + dn * pn.y);
}

// broadcast a real n x n matrix into a complex batch
__global__ void broadcast_real_kernel(size_t nn, int G, const double* __restrict__ src, double2* __restrict__ dst) {
  const size_t idx = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (idx >= nn * G) return;
  dst[idx] = make_double2(src[idx % nn], 0.0);
}

// K = A1^{-1} (nbloc x nbloc, skew 2x2 blocks) and Y = C0 S, with S the
// (Schur-reduced) nbloc x nbloc block of R_n2 stored with leading dim ldS.
__global__ void overlap_prep_kernel(int n, int G, const int* __restrict__ canon_i, const double* __restrict__ canon_d,
                                    const double2* __restrict__ S, int ldS, long long bsS, double2* __restrict__ K,
                                    double2* __restrict__ Y) {
  const int nocc = canon_i[0], nemp = canon_i[1];
  const int nb = n - nocc - nemp;
  const size_t nb2 = size_t(nb) * nb;
  const size_t idx = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (idx >= nb2 * G) return;
  const int b = int(idx / nb2);
  const size_t e = idx % nb2;
  const int i = int(e % nb), j = int(e / nb);  // 0-based local indices
  const double* vu = canon_d + 8;
  // A1u: upper entries A1(i, i+1) = vu(i + nemp) for odd 1-based i
  double2 kv = make_double2(0.0, 0.0);
  if ((i % 2) == 0 && j == i + 1) kv.x = -1.0 / vu[i + nemp];     // (A1^{-1})(i, i+1) = -1/a
  if ((i % 2) == 1 && j == i - 1) kv.x = 1.0 / vu[i - 1 + nemp];  // (A1^{-1})(i+1, i) = 1/a
  K[size_t(b) * nb2 + e] = kv;
  // C0u upper entries C0(i, i+1) = -vu(i + nemp) for odd 1-based i (self overlap)
  // Y(i, :) = C0(i, i+1) S(i+1, :) for even 0-based i; Y(i, :) = -C0(i-1, i) S(i-1, :) for odd
  double2 y;
  if ((i % 2) == 0) {
    const double g = -vu[i + nemp];
    const double2 s = S[b * bsS + (i + 1) + size_t(j) * ldS];
    y = make_double2(g * s.x, g * s.y);
  } else {
    const double g = -vu[i - 1 + nemp];
    const double2 s = S[b * bsS + (i - 1) + size_t(j) * ldS];
    y = make_double2(-g * s.x, -g * s.y);
  }
  Y[size_t(b) * nb2 + e] = y;
}

// per-angle traces: particle numbers (calculate_particle_number io=0,
// module_particlenumber.f90:78-143) and energy (calculate_expectval_energy,
// module_hamiltonian.f90:1098-1126), from angle-innermost arrays.
// Traces of the densities and fields per angle (particle numbers, their
// squares, energy).  Threads run over the angles -- the contiguous index of
// the angle-innermost arrays, so every load is coalesced -- and a CTA over a
// chunk of the n^2 elements; the partial sums of the chunks are reduced in a
// fixed order by traces_finish_kernel.  Partial layout:
// part[((chunk * G + b) * 9 + q)], q = prot, neut, tr rho_p^2, tr kRL kLR (p),
// tr rho_n^2, tr kRL kLR (n), tr H1 rho, tr gamma rho, tr Delta kRL.
constexpr int kTraceChunks = 256;
static_assert(kTraceChunks == 256, "Workspace::tpart is allocated for 256 chunks");
constexpr int kTraceThreads = 128;
// Partial traces over the pairs (i <= j) of chunk blockIdx.x, threads over the
// angles (angle-innermost layout: coalesced).  A pair takes both entries
// (i, j) and (j, i): Tr(H1 rho) and Tr(Gamma rho) need both products, while
// rho_ij rho_ji, kappaRL kappaLR and Delta kappaRL are equal for the two
// entries (Delta and the kappas are skew), so they are formed once and
// doubled.  The diagonal adds the traces of rho.
__global__ void __launch_bounds__(kTraceThreads)
    traces_partial_kernel(int n, int G, const double2* __restrict__ rho, const double2* __restrict__ kLR,
                          const double2* __restrict__ kRL, const double2* __restrict__ gam,
                          const double2* __restrict__ dLR, const double2* __restrict__ H1,
                          double2* __restrict__ part) {
  const int h = n / 2;
  const long long npairs = (long long)n * (n + 1) / 2;
  const int chunk = blockIdx.x;
  const long long q0 = npairs * chunk / kTraceChunks, q1 = npairs * (chunk + 1) / kTraceChunks;
  // pair q = j (j + 1) / 2 + i, 0 <= i <= j
  int j0 = int((sqrt(8.0 * double(q0) + 1.0) - 1.0) * 0.5);
  while ((long long)(j0 + 1) * (j0 + 2) / 2 <= q0) ++j0;
  while ((long long)j0 * (j0 + 1) / 2 > q0) --j0;
  const int i0 = int(q0 - (long long)j0 * (j0 + 1) / 2);
  for (int b = threadIdx.x; b < G; b += blockDim.x) {
    double2 a[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) a[q] = make_double2(0.0, 0.0);
    auto at = [G, n, b](const double2* X, int i, int j) { return X[(size_t(i) + size_t(j) * n) * G + b]; };
    int i = i0, j = j0;
    for (long long q = q0; q < q1; ++q) {
      const double2 rij = at(rho, i, j);
      if (i == j) {
        if (i < h)
          a[0] = cadd(a[0], rij);
        else
          a[1] = cadd(a[1], rij);
        const double2 kri = at(kRL, i, i), kli = at(kLR, i, i);
        if (i < h) {
          cfma(a[2], rij, rij);
          cfma(a[3], kri, kli);
        } else {
          cfma(a[4], rij, rij);
          cfma(a[5], kri, kli);
        }
        cfma(a[6], H1[i + size_t(i) * n], rij);
        cfma(a[7], at(gam, i, i), rij);
        cfma(a[8], at(dLR, i, i), at(kRL, i, i));
      } else {
        const double2 rji = at(rho, j, i), kr = at(kRL, i, j);
        const bool pblk = (i < h && j < h), nblk = (i >= h && j >= h);
        if (pblk || nblk) {
          const double2 rr = cmul(rij, rji), kk = cmul(kr, at(kLR, i, j));
          if (pblk) {
            a[2] = make_double2(fma(2.0, rr.x, a[2].x), fma(2.0, rr.y, a[2].y));
            a[3] = make_double2(fma(2.0, kk.x, a[3].x), fma(2.0, kk.y, a[3].y));
          } else {
            a[4] = make_double2(fma(2.0, rr.x, a[4].x), fma(2.0, rr.y, a[4].y));
            a[5] = make_double2(fma(2.0, kk.x, a[5].x), fma(2.0, kk.y, a[5].y));
          }
        }
        cfma(a[6], H1[i + size_t(j) * n], rji);
        cfma(a[6], H1[j + size_t(i) * n], rij);
        cfma(a[7], at(gam, i, j), rji);
        cfma(a[7], at(gam, j, i), rij);
        const double2 dk = cmul(at(dLR, i, j), kr);
        a[8] = make_double2(fma(2.0, dk.x, a[8].x), fma(2.0, dk.y, a[8].y));
      }
      if (++i > j) {
        ++j;
        i = 0;
      }
    }
#pragma unroll
    for (int q = 0; q < 9; ++q) part[(size_t(chunk) * G + b) * 9 + q] = a[q];
  }
}

// one CTA per angle, warp q sums partial q over the chunks (lanes over
// chunks, then a shuffle tree: a fixed order)
__global__ void __launch_bounds__(9 * 32) traces_finish_kernel(int G, const double2* __restrict__ part, double2 H0,
                                                               double2* __restrict__ obs) {
  __shared__ double2 r[9];
  const int b = blockIdx.x, q = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double2 s = make_double2(0.0, 0.0);
  for (int c = lane; c < kTraceChunks; c += 32) s = cadd(s, part[(size_t(c) * G + b) * 9 + q]);
  for (int off = 16; off > 0; off >>= 1) {
    s.x += __shfl_down_sync(0xffffffffu, s.x, off);
    s.y += __shfl_down_sync(0xffffffffu, s.y, off);
  }
  if (lane == 0) r[q] = s;
  __syncthreads();
  if (threadIdx.x != 0) return;
  const double2 prot = r[0], neut = r[1];
  const double2 prot2 = cadd(csub(cadd(prot, cmul(prot, prot)), r[2]), r[3]);
  const double2 neut2 = cadd(csub(cadd(neut, cmul(neut, neut)), r[4]), r[5]);
  const double2 ener = cadd(cadd(H0, r[6]), cscale(cadd(r[7], r[8]), 0.5));
  obs[8 * b + 1] = ener;
  obs[8 * b + 2] = prot;
  obs[8 * b + 3] = neut;
  obs[8 * b + 4] = prot2;
  obs[8 * b + 5] = neut2;
}

// overlap per angle and the sum_gauge coefficients
__global__ void overlap_finish_kernel(int n, int G, int have_overlap, const int* __restrict__ canon_i,
                                      const double* __restrict__ canon_d, const double2* __restrict__ pf,
                                      const double2* __restrict__ detR22, const double2* __restrict__ weight,
                                      const double* __restrict__ mult, double2* __restrict__ obs,
                                      double2* __restrict__ coefA, double2* __restrict__ coefAE) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= G) return;
  double2 over = make_double2(1.0, 0.0);
  if (have_overlap) {
    const int nocc = canon_i[0], nemp = canon_i[1];
    const int n2 = n - nemp;
    const int n0 = n - nocc;
    // signfac (module_projection.f90:813-816) with nocc0 = nocc1, nempm = nemp
    const long long e1 = (long long)n2 * (n2 + 1) / 2;
    const long long e2 = (long long)nocc * (nocc - 1) / 2;
    const long long e3 = (long long)nocc * (nocc + 1) + (long long)nocc * (n0 + n2) + (long long)nocc * n0;
    const double signfac = ((e1 + e2 + e3) & 1) ? -1.0 : 1.0;
    const double ovac = canon_d[0];
    const double2 pK = pf[b], phK = pf[G + b];
    const double2 pR = detR22[b], phR = detR22[G + b];
    if (isinf(pK.x) && pK.x < 0) {
      over = make_double2(0.0, 0.0);
    } else {
      const double logm = pK.x + pR.x + canon_d[1] + ovac;
      double2 ph = cmul(phK, phR);
      ph = cscale(ph, canon_d[2] * signfac);
      const double m = exp(logm);
      over = make_double2(m * ph.x, m * ph.y);
    }
  }
  obs[8 * b + 0] = over;
  const double2 f1 = cmul(weight[b], over);
  const double2 f2 = cmul(f1, obs[8 * b + 1]);
  coefA[b] = cscale(f1, 1.0);
  coefAE[b] = f2;
}

// sum_gauge of the scalars (module_projection.f90:425-458), folded pairs as 2 Re
// one warp: lanes over the angles, then a shuffle reduction (order differs
// from the serial sum only by rounding)
__global__ void sum_scalars_kernel(int G, const double2* __restrict__ obs, const double* __restrict__ mult,
                                   const double2* __restrict__ weight, double2* __restrict__ pscal, int accumulate) {
  const int lane = threadIdx.x & 31;
  double2 s[6];
  for (int q = 0; q < 6; ++q) s[q] = make_double2(0.0, 0.0);
  for (int b = lane; b < G; b += 32) {
    const double2 f1 = cmul(weight[b], obs[8 * b]);
    const double2 terms[6] = {f1, cmul(obs[8 * b + 1], f1), cmul(obs[8 * b + 2], f1), cmul(obs[8 * b + 3], f1),
                              cmul(obs[8 * b + 4], f1), cmul(obs[8 * b + 5], f1)};
    const bool folded = mult[b] == 2.0;
    for (int q = 0; q < 6; ++q) {
      if (folded)
        s[q].x += 2.0 * terms[q].x;
      else
        s[q] = cadd(s[q], terms[q]);
    }
  }
  for (int q = 0; q < 6; ++q)
    for (int off = 16; off > 0; off >>= 1) {
      s[q].x += __shfl_down_sync(0xffffffffu, s[q].x, off);
      s[q].y += __shfl_down_sync(0xffffffffu, s[q].y, off);
    }
  if (lane == 0)
    for (int q = 0; q < 6; ++q) pscal[q] = accumulate ? cadd(pscal[q], s[q]) : s[q];
}
// sum_gauge of the matrices: pA = sum_b c_b A_b, pH = sum_b c_b 2 T_b,
// pAH = sum_b c_b E_b A_b.  A warp covers 32 consecutive elements (coalesced
// loads), the warps of a CTA split the angles and are reduced in shared
// memory; a folded angle (multiplicity 2) contributes 2 Re(c_b X_b) only, so
// it costs two FMAs per sum (FP64 throughput is the bound on this part).
constexpr int kSumWarps = 8;
__global__ void __launch_bounds__(32 * kSumWarps)
    sum_matrices_kernel(int n, int G, const double2* __restrict__ A, const double2* __restrict__ T,
                        const double2* __restrict__ coefA, const double2* __restrict__ coefAE,
                        const double* __restrict__ mult, double2* __restrict__ pA, double2* __restrict__ pH,
                        double2* __restrict__ pAH, int accumulate) {
  // H20_b = T_b - T_b^T enters as 2 T_b: the sum is antisymmetrised once, in
  // projected_h20_kernel (1/2 (X - X^T)), which gives sum c_b (T_b - T_b^T)
  extern __shared__ double2 sc[];  // per angle: c_b m_b, 2 c_b m_b, c_b E_b m_b (m_b folded into the scale)
  __shared__ double2 red[3][kSumWarps][32];
  const size_t nn = size_t(n) * n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int b = threadIdx.x; b < G; b += blockDim.x) {
    const double f = mult[b] == 2.0 ? 2.0 : 1.0;
    sc[3 * b] = cscale(coefA[b], f);
    sc[3 * b + 1] = cscale(coefA[b], 2.0 * f);
    sc[3 * b + 2] = cscale(coefAE[b], f);
  }
  __syncthreads();
  const size_t e = blockIdx.x * size_t(32) + lane;
  double2 sa = make_double2(0.0, 0.0), sh = sa, sah = sa;
  if (e < nn) {
    for (int b = warp; b < G; b += kSumWarps) {
      const double2 a = A[size_t(b) * nn + e], tv = T[size_t(b) * nn + e];
      const double2 c1 = sc[3 * b], c2 = sc[3 * b + 1], c3 = sc[3 * b + 2];
      if (mult[b] == 2.0) {
        sa.x = fma(a.x, c1.x, fma(-a.y, c1.y, sa.x));
        sh.x = fma(tv.x, c2.x, fma(-tv.y, c2.y, sh.x));
        sah.x = fma(a.x, c3.x, fma(-a.y, c3.y, sah.x));
      } else {
        sa = cadd(sa, cmul(a, c1));
        sh = cadd(sh, cmul(tv, c2));
        sah = cadd(sah, cmul(a, c3));
      }
    }
  }
  red[0][warp][lane] = sa;
  red[1][warp][lane] = sh;
  red[2][warp][lane] = sah;
  __syncthreads();
  if (warp < 3 && e < nn) {
    double2 s = accumulate ? (warp == 0 ? pA[e] : (warp == 1 ? pH[e] : pAH[e])) : make_double2(0.0, 0.0);
#pragma unroll
    for (int w = 0; w < kSumWarps; ++w) s = cadd(s, red[warp][w][lane]);
    (warp == 0 ? pA : (warp == 1 ? pH : pAH))[e] = s;
  }
}

// calculate_projected_H20 (module_projection.f90:729-759)
__global__ void projected_h20_kernel(int n, const double2* __restrict__ pA, const double2* __restrict__ pH,
                                     const double2* __restrict__ pAH, const double2* __restrict__ pscal,
                                     double* __restrict__ H20v, int* flags) {
  const size_t nn = size_t(n) * n;
  const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (e >= nn) return;
  const int i = int(e % n), j = int(e / n);
  const size_t et = j + size_t(i) * n;
  const double2 over = pscal[0];
  const double2 ener = cdiv(pscal[1], over);
  const double2 rov = crcp(over);
  const double2 A = cmul(cscale(csub(pA[e], pA[et]), 0.5), rov);
  const double2 H = cmul(cscale(csub(pH[e], pH[et]), 0.5), rov);
  const double2 AH = cmul(cscale(csub(pAH[e], pAH[et]), 0.5), rov);
  H20v[e] = (cadd(csub(AH, cmul(ener, A)), H)).x;
  const double2 Hraw = cscale(csub(pH[e], pH[et]), 0.5);  // the antisymmetric sum of the H20_b
  const double ig = cmul(cadd(csub(pAH[e], cmul(ener, pA[e])), Hraw), rov).y;
  if (ig > 1.0e-8) atomicOr(flags, DEV_IMAG_GRAD);
}

// generic batched left solve X = A^{-1} B (A m x m, B m x k) by Gaussian
// elimination with partial pivoting on [A | B]; also returns log|det A| and
// the phase of det A.  Views give element (i,j) of batch b at p[i rs + j cs + b bs].
constexpr int kLsThreads = 512;
__global__ void __launch_bounds__(kLsThreads)
    left_solve_kernel(int m, int k, View Av, View Bv, double2* __restrict__ Wall, double2* __restrict__ X,
                      long long xrs, long long xcs, long long xbs, int conj_out, double2* __restrict__ det, int G,
                      int* flags, int flag_bit) {
  __shared__ double sv[kLsThreads];
  __shared__ int si[kLsThreads];
  __shared__ double2 prow[1024];
  __shared__ double2 mult[512];
  const int b = blockIdx.x;
  const int w = m + k;
  double2* W = Wall + size_t(b) * m * w;
  const int tid = threadIdx.x, nt = blockDim.x;
  const double2* Ap = static_cast<const double2*>(Av.p);
  const double2* Bp = static_cast<const double2*>(Bv.p);
  for (int c = tid >> 5; c < w; c += nt >> 5)
    for (int r = tid & 31; r < m; r += 32)
      W[r + size_t(c) * m] =
          (c < m) ? Ap[r * Av.rs + c * Av.cs + b * Av.bs] : Bp[r * Bv.rs + (c - m) * Bv.cs + b * Bv.bs];
  __syncthreads();
  bool singular = false;
  double logdet = 0.0;
  double2 ph = make_double2(1.0, 0.0);
  for (int kk = 0; kk < m; ++kk) {
    double best = -1.0;
    int bi = m;
    for (int i = kk + tid; i < m; i += nt) {
      const double v = cabs1(W[i + size_t(kk) * m]);
      if (v > best) {
        best = v;
        bi = i;
      }
    }
    sv[tid] = best;
    si[tid] = bi;
    __syncthreads();
    for (int s = nt / 2; s > 0; s >>= 1) {
      if (tid < s) {
        const double a = sv[tid], bb = sv[tid + s];
        const int ia = si[tid], ib = si[tid + s];
        if (bb > a || (bb == a && ib < ia)) {
          sv[tid] = bb;
          si[tid] = ib;
        }
      }
      __syncthreads();
    }
    int p = si[0];
    const double pv = sv[0];
    __syncthreads();
    if (pv == 0.0) {
      singular = true;
      p = kk;
    }
    for (int c = kk + tid; c < w; c += nt) {
      double2 a = W[kk + size_t(c) * m], q = W[p + size_t(c) * m];
      if (p != kk) {
        W[kk + size_t(c) * m] = q;
        W[p + size_t(c) * m] = a;
        a = q;
      }
      prow[c] = a;
    }
    __syncthreads();
    const double2 piv = prow[kk];
    if (!singular) {
      const double mg = hypot(piv.x, piv.y);
      logdet += log(mg);
      ph = cmul(ph, make_double2(piv.x / mg, piv.y / mg));
      if (p != kk) ph = cneg(ph);
    }
    const double2 rp = (pv == 0.0) ? make_double2(0.0, 0.0) : crcp(piv);
    for (int i = kk + 1 + tid; i < m; i += nt) mult[i] = cmul(W[i + size_t(kk) * m], rp);
    __syncthreads();
    // rank-1 update of rows kk+1.. over columns kk+1..w-1: one warp per column,
    // lanes over rows (column-major: coalesced), no index division
    {
      const int warp = tid >> 5, lane = tid & 31, nw = nt >> 5;
      for (int c = kk + 1 + warp; c < w; c += nw) {
        const double2 r = prow[c];
        double2* col = W + size_t(c) * m;
        for (int i = kk + 1 + lane; i < m; i += 32) {
          double2 v = col[i];
          const double2 mu = mult[i];
          v.x = fma(-mu.x, r.x, v.x);
          v.x = fma(mu.y, r.y, v.x);
          v.y = fma(-mu.x, r.y, v.y);
          v.y = fma(-mu.y, r.x, v.y);
          col[i] = v;
        }
      }
    }
    __syncthreads();
  }
  for (int kk = m - 1; kk >= 0; --kk) {
    const double2 rk = crcp(W[kk + size_t(kk) * m]);
    for (int c = tid; c < k; c += nt) {
      const double2 y = cmul(W[kk + size_t(m + c) * m], rk);
      W[kk + size_t(m + c) * m] = y;
      prow[c] = y;
    }
    __syncthreads();
    {
      const int warp = tid >> 5, lane = tid & 31, nw = nt >> 5;
      for (int c = warp; c < k; c += nw) {
        const double2 r = prow[c];
        double2* col = W + size_t(m + c) * m;
        for (int i = lane; i < kk; i += 32) {
          double2 v = col[i];
          const double2 mu = W[i + size_t(kk) * m];
          v.x = fma(-mu.x, r.x, v.x);
          v.x = fma(mu.y, r.y, v.x);
          v.y = fma(-mu.x, r.y, v.y);
          v.y = fma(-mu.y, r.x, v.y);
          col[i] = v;
        }
      }
    }
    __syncthreads();
  }
  if (X) {
    for (int c = tid >> 5; c < k; c += nt >> 5)
      for (int r = tid & 31; r < m; r += 32) {
        double2 v = W[r + size_t(m + c) * m];
        if (conj_out) v.y = -v.y;
        X[r * xrs + c * xcs + b * xbs] = v;
      }
  }
  if (tid == 0) {
    if (det) {
      det[b] = make_double2(singular ? -INFINITY : logdet, 0.0);
      det[G + b] = singular ? make_double2(0.0, 0.0) : ph;
    }
    if (singular) atomicOr(flags, flag_bit);
  }
}

__global__ void fill_det_one_kernel(int G, double2* det) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < G) {
    det[b] = make_double2(0.0, 0.0);
    det[G + b] = make_double2(1.0, 0.0);
  }
}

// S = R11 - R12 Z with Z = R22^{-1} R21 (nb x nb, in place into SZ)
__global__ void schur_kernel(int n2, int nb, int G, const double2* __restrict__ Rn, const double2* __restrict__ Z,
                             double2* __restrict__ S) {
  const size_t nb2 = size_t(nb) * nb;
  const size_t idx = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (idx >= nb2 * G) return;
  const int b = int(idx / nb2);
  const size_t e = idx % nb2;
  const int i = int(e % nb), j = int(e / nb);
  const int no = n2 - nb;
  const double2* R = Rn + size_t(b) * n2 * n2;
  double2 s = R[i + size_t(j) * n2];
  for (int t = 0; t < no; ++t) {
    const double2 r12 = R[i + size_t(nb + t) * n2];
    const double2 z = Z[size_t(b) * no * nb + t + size_t(j) * no];
    s = csub(s, cmul(r12, z));
  }
  S[size_t(b) * nb2 + e] = s;
}

// ---------------------------------------------------------------------------
// Symmetric eigenvector refinement (Ogita & Aishima, Japan J. Indust. Appl.
// Math. 35 (2018) 1007): from approximate eigenvectors X of A,
//   R = I - X^T X,  S = X^T A X,  l_i = S_ii / (1 - R_ii),
//   E_ij = (S_ij + l_j R_ij) / (l_j - l_i)  if |l_i - l_j| > delta,  R_ij / 2 otherwise,
//   X <- X (I + E),  delta = 2 (||S - diag(l)|| + ||A|| ||R||),
// converges quadratically; every step is three GEMMs on all SMs instead of
// a serial Jacobi sweep on one SM.  Near-degenerate clusters are
// diagonalised exactly afterwards (cluster_finish_kernel).
// ---------------------------------------------------------------------------
constexpr int kRlThreads = 1024;
__global__ void __launch_bounds__(kRlThreads)
    refine_lambda_kernel(int n, const double* __restrict__ XtX, const double* __restrict__ S,
                         const double* __restrict__ A, double* __restrict__ lam, double* __restrict__ rscal) {
  __shared__ double red[3][kRlThreads / 32];
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < n; i += nt) lam[i] = S[i + size_t(i) * n] / XtX[i + size_t(i) * n];
  double s_off = 0.0, s_r = 0.0, s_a = 0.0;
  const size_t nn = size_t(n) * n;
  // four elements in flight per thread
  for (size_t e0 = tid; e0 < nn; e0 += 4 * size_t(nt)) {
    double xv[4], sv[4], av[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const size_t e = e0 + size_t(u) * nt;
      xv[u] = e < nn ? XtX[e] : 0.0;
      sv[u] = e < nn ? S[e] : 0.0;
      av[u] = e < nn ? A[e] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const size_t e = e0 + size_t(u) * nt;
      if (e >= nn) continue;
      const int i = int(e % n), j = int(e / n);
      const bool d = (i == j);
      const double r = (d ? 1.0 : 0.0) - xv[u];
      // the diagonal of S - diag(l) with l = S_ii / XtX_ii, formed here from
      // the same operands as lam
      const double so = d ? sv[u] - sv[u] / xv[u] : sv[u];
      s_off += so * so;
      s_r += r * r;
      s_a += av[u] * av[u];
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    s_off += __shfl_xor_sync(0xffffffffu, s_off, o);
    s_r += __shfl_xor_sync(0xffffffffu, s_r, o);
    s_a += __shfl_xor_sync(0xffffffffu, s_a, o);
  }
  if (lane == 0) {
    red[0][warp] = s_off;
    red[1][warp] = s_r;
    red[2][warp] = s_a;
  }
  __syncthreads();
  if (tid == 0) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int w2 = 0; w2 < nt / 32; ++w2) {
      a0 += red[0][w2];
      a1 += red[1][w2];
      a2 += red[2][w2];
    }
    const double nS = sqrt(a0), nR = sqrt(a1), nA = sqrt(a2);
    rscal[0] = 2.0 * (nS + nA * nR);  // delta
    rscal[1] = nA;
    rscal[2] = nS;
    rscal[3] = nR;
  }
}

__global__ void refine_update_kernel(int n, const double* __restrict__ XtX, const double* __restrict__ S,
                                     const double* __restrict__ lam, const double* __restrict__ rscal,
                                     const int* __restrict__ cid, double* __restrict__ M,
                                     double* __restrict__ Fout) {
  const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (e >= size_t(n) * n) return;
  const int i = int(e % n), j = int(e / n);
  const size_t et = j + size_t(i) * n;
  // E = R/2 + F with R = I - X^T X and F antisymmetric (Ogita & Aishima's
  // correction E_ij = (S_ij + l_j R_ij)/(l_j - l_i) split into its symmetric
  // and antisymmetric parts).  Both parts are formed from the symmetrised S
  // and R, so F_ji = -F_ij holds exactly and the orthonormality update R/2
  // carries no rounding amplified by small gaps l_j - l_i.
  const double rb = 0.5 * ((((i == j) ? 1.0 : 0.0) - XtX[e]) + (((i == j) ? 1.0 : 0.0) - XtX[et]));
  const double sb = 0.5 * (S[e] + S[et]);
  const double dl = lam[j] - lam[i];
  // the rotation only between columns of different clusters (fixed at the
  // first step, where the gap dominated the coupling 64-fold); the pairs
  // within a cluster are only re-orthonormalised and diagonalised exactly
  // at the end.  Admitting such a pair later, once its coupling looks small
  // beside the shrinking residual, gives corrections of order one whose
  // second-order terms undo the orthonormality.
  const bool newton = (i != j) && cid[i] != cid[j] && fabs(dl) > 2.0 * fabs(sb) + 1.0e-13 * rscal[1];
  const double F = newton ? (sb + 0.5 * (lam[i] + lam[j]) * rb) / dl : 0.0;
  // M = I + R/2 + F here; the steps that continue a refinement whose check
  // failed add F^2 / 2 (I + F + F^2/2 is orthogonal to O(F^3) where I + F
  // loses O(F^2): from an FP32 start, ||R|| ~ 1e-4, on nearly closed shells
  // that stays above the acceptance test after three steps)
  M[e] = ((i == j) ? 1.0 : 0.0) + 0.5 * rb + F;
  Fout[e] = F;
}

// Cyclic Jacobi of one cluster block a (m x m, m <= M) with its rotations
// accumulated in q, by one thread: sweeps until the off-diagonal part is at
// rounding level (at most 30)
template <int M>
__device__ void cluster_jacobi(int m, double (&a)[M][M], double (&q)[M][M]) {
  for (int sweep = 0; sweep < 30 && m > 1; ++sweep) {
    double off = 0.0, dia = 0.0;
    for (int r = 0; r < m; ++r) {
      dia += a[r][r] * a[r][r];
      for (int t = r + 1; t < m; ++t) off += a[r][t] * a[r][t];
    }
    // converged to rounding: further rotations only move noise
    if (off <= 1.0e-32 * dia) break;
    for (int pp = 0; pp < m; ++pp)
      for (int qq = pp + 1; qq < m; ++qq) {
        if (a[pp][qq] == 0.0) continue;
        const double theta = (a[qq][qq] - a[pp][pp]) / (2.0 * a[pp][qq]);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
        for (int r = 0; r < m; ++r) {
          const double ap = a[r][pp], aq = a[r][qq];
          a[r][pp] = cs * ap - sn * aq;
          a[r][qq] = sn * ap + cs * aq;
        }
        for (int r = 0; r < m; ++r) {
          const double ap = a[pp][r], aq = a[qq][r];
          a[pp][r] = cs * ap - sn * aq;
          a[qq][r] = sn * ap + cs * aq;
        }
        for (int r = 0; r < m; ++r) {
          const double qp = q[r][pp], qv = q[r][qq];
          q[r][pp] = cs * qp - sn * qv;
          q[r][qq] = sn * qp + cs * qv;
        }
      }
  }
}

// One cluster (positions k0 .. k0+m-1 of the sorted order): its block of S,
// Jacobi, the eigenvalues in ascending order to lsh / the source column of
// each to osh, the rotation to qb (m x m, column t of the block at t * m)
template <int M>
__device__ void cluster_solve(int n, int m, int k0, const double* __restrict__ S, const int* perm, double* lsh,
                              int* osh, double* qb) {
  double a[M][M], q[M][M];
  for (int r = 0; r < m; ++r)
    for (int t = 0; t < m; ++t) {
      a[r][t] = S[perm[k0 + r] + size_t(perm[k0 + t]) * n];
      q[r][t] = (r == t) ? 1.0 : 0.0;
    }
  cluster_jacobi<M>(m, a, q);
  int ord[M];
  for (int r = 0; r < m; ++r) ord[r] = r;
  for (int r = 1; r < m; ++r)
    for (int t = r; t > 0 && a[ord[t]][ord[t]] < a[ord[t - 1]][ord[t - 1]]; --t) {
      const int x = ord[t];
      ord[t] = ord[t - 1];
      ord[t - 1] = x;
    }
  for (int r = 0; r < m; ++r) {
    osh[k0 + r] = ord[r];
    lsh[k0 + r] = a[ord[r]][ord[r]];
    for (int t = 0; t < m; ++t) qb[t * m + r] = q[t][r];
  }
}

constexpr int kCfThreads = 512;
constexpr int kCfMaxN = 512;
constexpr int kCfQ = 2048;          // rotation entries of the small clusters (sum of m^2)
constexpr double kCfGate = 64.0;    // Newton step where |l_j - l_i| > kCfGate |S_ij|

// Clusters of the refined basis, fixed at the first refinement step (Ogita
// & Aishima's treatment of clustered eigenvalues): columns i, j whose gap
// is not kCfGate times their coupling, |l_j - l_i| <= kCfGate |S_ij| +
// 1e-13 ||A||, belong to one cluster, and a cluster is the smallest range
// of the sorted Rayleigh quotients that contains every such pair.  cid[i] =
// the first sorted position of column i's cluster.  One CTA.
__global__ void __launch_bounds__(kCfThreads)
    cluster_assign_kernel(int n, const double* __restrict__ S, const double* __restrict__ lam,
                          const double* __restrict__ rscal, int* __restrict__ cid) {
  __shared__ int pos[kCfMaxN], order[kCfMaxN], reach[kCfMaxN];
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int i = tid; i < n; i += nt) {
    const double v = lam[i];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const double u = lam[j];
      rank += (u < v || (u == v && j < i)) ? 1 : 0;
    }
    pos[i] = rank;
    order[rank] = i;
    reach[rank] = rank;
  }
  __syncthreads();
  const double floor = 1.0e-13 * rscal[1];
  for (size_t e = tid; e < size_t(n) * n; e += nt) {
    const int i = int(e % n), j = int(e / n);
    if (i >= j) continue;
    const double sb = 0.5 * (S[e] + S[j + size_t(i) * n]);
    if (fabs(lam[j] - lam[i]) <= kCfGate * fabs(sb) + floor) {
      const int pa = pos[i], pb = pos[j];
      atomicMax(&reach[min(pa, pb)], max(pa, pb));
    }
  }
  __syncthreads();
  if (tid == 0) {
    int k = 0;
    while (k < n) {
      int j = reach[k];
      for (int t = k; t <= j; ++t) j = max(j, reach[t]);
      for (int t = k; t <= j; ++t) cid[order[t]] = k;
      k = j + 1;
    }
  }
}

// The refined columns ordered by cluster (the order of the first step) and,
// within a cluster, by Rayleigh quotient; each cluster diagonalised exactly
// (up to 8 columns: a Jacobi by one thread here; larger ones, or those
// beyond the rotation buffer: listed in bigd for the FP64 Jacobi of their
// block, big_cluster_rotate_kernel); the coupling between clusters and the
// orthonormality verified; D and the eigenvalues written in that order.
// One CTA: the diagonal, the order and the clusters in shared memory, one
// thread per small cluster for its Jacobi, a warp per cluster for the
// rotation of its columns.  rflag[0] = failure bits, rflag[2] = number of
// clusters in bigd, rflag[3] = 0 (the big clusters' Jacobi status).
__global__ void __launch_bounds__(kCfThreads)
    cluster_finish_kernel(int n, const double* __restrict__ S, const double* __restrict__ X,
                          const double* __restrict__ rscal, const int* __restrict__ cidg, double* __restrict__ D,
                          double* __restrict__ evals, int* __restrict__ cperm, int* __restrict__ bigd, int* rflag) {
  constexpr int CM = 8;
  __shared__ double sd[kCfMaxN], lsh[kCfMaxN];
  __shared__ int perm[kCfMaxN], cid[kCfMaxN], osh[kCfMaxN], cl_start[kCfMaxN + 1], qoff[kCfMaxN + 1];
  __shared__ double qbuf[kCfQ];
  __shared__ int ncl, fail, nbig;
  __shared__ double red[kCfThreads / 32];
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
  if (tid == 0) {
    fail = 0;
    nbig = 0;
  }
  for (int i = tid; i < n; i += nt) {
    sd[i] = S[i + size_t(i) * n];
    cid[i] = cidg[i];
  }
  __syncthreads();
  for (int i = tid; i < n; i += nt) {
    const double v = sd[i];
    const int ci = cid[i];
    int rank = 0;
    for (int j = 0; j < n; ++j) {
      const double u = sd[j];
      const int cj = cid[j];
      rank += (cj < ci || (cj == ci && (u < v || (u == v && j < i)))) ? 1 : 0;
    }
    perm[rank] = i;
  }
  __syncthreads();
  for (int k = tid; k < n; k += nt) cperm[k] = perm[k];
  const double nA = rscal[1];
  if (tid == 0) {
    int c = 0;
    cl_start[0] = 0;
    for (int k = 1; k < n; ++k)
      if (cid[perm[k]] != cid[perm[k - 1]]) cl_start[++c] = k;
    ncl = c + 1;
    cl_start[ncl] = n;
    // small clusters take rotation buffer space; the rest go to bigd
    // (qoff = -1), as many as it holds
    int off = 0;
    for (int q = 0; q < ncl; ++q) {
      const int m = cl_start[q + 1] - cl_start[q];
      if (m <= CM && off + m * m <= kCfQ) {
        qoff[q] = off;
        off += m * m;
      } else if (nbig < kCfBigSlots) {
        qoff[q] = -1;
        bigd[2 * nbig] = cl_start[q];
        bigd[2 * nbig + 1] = m;
        ++nbig;
      } else {
        qoff[q] = -1;
        fail |= 4;  // more large clusters than the list holds
      }
    }
  }
  __syncthreads();
  // coupling between different clusters must be negligible
  double mx = 0.0;
  for (size_t e = tid; e < size_t(n) * n; e += nt) {
    const int i = int(e % n), j = int(e / n);
    if (cid[i] != cid[j]) mx = fmax(mx, fabs(S[e]));
  }
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) red[warp] = mx;
  __syncthreads();
  // X orthonormal and X^T A X block diagonal over clusters <=> invariant subspaces
  if (tid == 0) {
    double m2 = 0.0;
    for (int w2 = 0; w2 < nwarp; ++w2) m2 = fmax(m2, red[w2]);
    if (m2 > 1.0e-12 * fmax(nA, 1e-300)) fail |= 1;  // clusters still coupled
    if (rscal[3] > 1.0e-12 * sqrt(double(n))) fail |= 2;  // not orthonormal
  }
  for (int c = tid; c < ncl; c += nt) {
    const int k0 = cl_start[c], m = cl_start[c + 1] - k0;
    if (qoff[c] < 0) continue;
    double* qb = qbuf + qoff[c];
    if (m == 1) {
      osh[k0] = 0;
      lsh[k0] = sd[perm[k0]];
      qb[0] = 1.0;
    } else if (m == 2) {
      cluster_solve<2>(n, m, k0, S, perm, lsh, osh, qb);
    } else if (m <= 4) {
      cluster_solve<4>(n, m, k0, S, perm, lsh, osh, qb);
    } else {
      cluster_solve<CM>(n, m, k0, S, perm, lsh, osh, qb);
    }
  }
  __syncthreads();
  for (int c = warp; c < ncl; c += nwarp) {
    const int k0 = cl_start[c], m = cl_start[c + 1] - k0;
    if (qoff[c] < 0) {
      // left to the FP64 Jacobi of the block (or the attempt fails): the
      // refined columns go to D unrotated, so that D stays an orthonormal
      // basis to start the next attempt from
      for (int r = 0; r < m; ++r) {
        if (lane == 0) evals[k0 + r] = sd[perm[k0 + r]];
        for (int row = lane; row < n; row += 32) D[row + size_t(k0 + r) * n] = X[row + size_t(perm[k0 + r]) * n];
      }
    } else {
      const double* qb = qbuf + qoff[c];
      for (int r = 0; r < m; ++r) {
        const int src = osh[k0 + r];
        if (lane == 0) evals[k0 + r] = lsh[k0 + r];
        for (int row = lane; row < n; row += 32) {
          double v = 0.0;
          for (int t = 0; t < m; ++t) v = fma(X[row + size_t(perm[k0 + t]) * n], qb[t * m + src], v);
          D[row + size_t(k0 + r) * n] = v;
        }
      }
    }
  }
  __syncthreads();
  if (tid == 0) {
    rflag[0] = fail;
    rflag[2] = nbig;
    rflag[3] = 0;
  }
}

// The block S_cc of one large cluster (columns cperm[k0 .. k0+m-1] of the
// refined basis), column-major m x m, for the FP64 Jacobi.
__global__ void big_cluster_extract_kernel(int n, int m, const double* __restrict__ S, const int* __restrict__ cp,
                                           double* __restrict__ Sc) {
  const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (e >= size_t(m) * m) return;
  const int a = int(e % m), b = int(e / m);
  Sc[e] = S[cp[a] + size_t(cp[b]) * n];
}

// D(:, k0 + r) = sum_t X(:, cperm[k0 + t]) W(t, r) and the eigenvalues of
// the cluster (ascending, from the FP64 Jacobi of its block).
__global__ void big_cluster_rotate_kernel(int n, int m, const double* __restrict__ X, const int* __restrict__ cp,
                                          const double* __restrict__ W, const double* __restrict__ ev,
                                          double* __restrict__ Dk, double* __restrict__ evk) {
  const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (e >= size_t(n) * m) return;
  const int row = int(e % n), r = int(e / n);
  double v = 0.0;
  for (int t = 0; t < m; ++t) v = fma(X[row + size_t(cp[t]) * n], W[t + size_t(r) * m], v);
  Dk[row + size_t(r) * n] = v;
  if (row == 0) evk[r] = ev[r];
}

// ---------------------------------------------------------------------------
// Blocked Thouless solve.  X = V_phi U_phi^{-1} is obtained from the
// augmented system W = [U_phi^T | V_phi^T] (n x 2n, one per angle) by a
// right-looking blocked LU with partial pivoting: per panel of nb columns a
// small per-angle kernel factors the panel, applies its row exchanges and
// forms U12 = L11^{-1} A12; the trailing update A22 -= L21 U12 is a batched
// GEMM over all SMs.  The blocked back substitution with U alternates GEMM
// updates and small per-block triangular solves.  Same pivots as the
// unblocked elimination; 10.7 n^3 FP64 flops per angle, mostly in GEMMs.
// With the emulated products the solve is a blocked Gauss-Jordan elimination
// instead (panel_gj_kernel): the same partial pivoting per panel, the block
// row scaled by the inverse of its diagonal block and every other row
// eliminated by one product, so that no back substitution is needed.
// ---------------------------------------------------------------------------
constexpr int kPanelThreads = 512;

// argmax over a warp on integer keys: for non-negative doubles the bit
// pattern orders like the value, and an integer compare avoids the FP64 pipe
// (a dependent FP64 operation takes about 64 cycles on this part)
__device__ __forceinline__ void warp_argmax_key(long long& v, int& i) {
  for (int off = 16; off > 0; off >>= 1) {
    const long long v2 = __shfl_down_sync(0xffffffffu, v, off);
    const int i2 = __shfl_down_sync(0xffffffffu, i, off);
    if (v2 > v || (v2 == v && i2 < i)) {
      v = v2;
      i = i2;
    }
  }
}

__device__ __forceinline__ void warp_argmax(double& v, int& i) {
  for (int off = 16; off > 0; off >>= 1) {
    const double v2 = __shfl_down_sync(0xffffffffu, v, off);
    const int i2 = __shfl_down_sync(0xffffffffu, i, off);
    if (v2 > v || (v2 == v && i2 < i)) {
      v = v2;
      i = i2;
    }
  }
}

__global__ void __launch_bounds__(kPanelThreads)
    build_augmented_kernel(int n, const double2* __restrict__ Uphi, const double2* __restrict__ Vphi,
                           double2* __restrict__ Wall) {
  const int b = blockIdx.y;
  const size_t nn = size_t(n) * n;
  double2* W = Wall + b * 2 * nn;
  const double2* U = Uphi + b * nn;
  const double2* V = Vphi + b * nn;
  // W(r, c) = U(c, r);  W(r, n + c) = V(c, r)
  for (int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < 2 * n; c += gridDim.x * (blockDim.x >> 5))
    for (int r = threadIdx.x & 31; r < n; r += 32)
      W[r + size_t(c) * n] = (c < n) ? U[c + size_t(r) * n] : V[(c - n) + size_t(r) * n];
}

__global__ void __launch_bounds__(kPanelThreads)
    panel_kernel(int n, int j0, int nbp, double2* __restrict__ Wall, int* flags) {
  __shared__ double wv[kPanelThreads / 32];
  __shared__ int wi[kPanelThreads / 32];
  __shared__ int s_piv;
  __shared__ double s_pv;
  const int b = blockIdx.x;
  const int w2 = 2 * n;
  double2* W = Wall + size_t(b) * n * w2;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  const int j1 = j0 + nbp;
  bool singular = false;
  for (int jj = 0; jj < nbp; ++jj) {
    const int j = j0 + jj;
    double best = -1.0;
    int bi = n;
    for (int i = j + tid; i < n; i += nt) {
      const double v = cabs1(W[i + size_t(j) * n]);
      if (v > best) {
        best = v;
        bi = i;
      }
    }
    warp_argmax(best, bi);
    if (lane == 0) {
      wv[warp] = best;
      wi[warp] = bi;
    }
    __syncthreads();
    if (warp == 0) {
      double v = (lane < nw) ? wv[lane] : -1.0;
      int i = (lane < nw) ? wi[lane] : n;
      warp_argmax(v, i);
      if (lane == 0) {
        s_piv = i;
        s_pv = v;
      }
    }
    __syncthreads();
    int p = s_piv;
    const double pv = s_pv;
    if (pv == 0.0) {
      singular = true;
      p = j;
    }
    if (p != j)
      for (int c = j0 + tid; c < w2; c += nt) {
        const double2 t = W[j + size_t(c) * n];
        W[j + size_t(c) * n] = W[p + size_t(c) * n];
        W[p + size_t(c) * n] = t;
      }
    __syncthreads();
    const double2 rp = (pv == 0.0) ? make_double2(0.0, 0.0) : crcp(W[j + size_t(j) * n]);
    for (int i = j + 1 + tid; i < n; i += nt) W[i + size_t(j) * n] = cmul(W[i + size_t(j) * n], rp);
    __syncthreads();
    // rank-1 update of the remaining panel columns
    for (int c = j + 1 + warp; c < j1; c += nw) {
      const double2 r = W[j + size_t(c) * n];
      double2* col = W + size_t(c) * n;
      for (int i = j + 1 + lane; i < n; i += 32) {
        double2 v = col[i];
        const double2 mu = W[i + size_t(j) * n];
        v.x = fma(-mu.x, r.x, v.x);
        v.x = fma(mu.y, r.y, v.x);
        v.y = fma(-mu.x, r.y, v.y);
        v.y = fma(-mu.y, r.x, v.y);
        col[i] = v;
      }
    }
    __syncthreads();
  }
  // U12 = L11^{-1} A12 (unit lower forward substitution on the block row)
  for (int jj = 0; jj < nbp; ++jj) {
    const int r = j0 + jj;
    for (int c = j1 + warp; c < w2; c += nw) {
      const double2 top = W[r + size_t(c) * n];
      double2* col = W + size_t(c) * n;
      for (int r2 = r + 1 + lane; r2 < j1; r2 += 32) {
        double2 v = col[r2];
        const double2 mu = W[r2 + size_t(r) * n];
        v.x = fma(-mu.x, top.x, v.x);
        v.x = fma(mu.y, top.y, v.x);
        v.y = fma(-mu.x, top.y, v.y);
        v.y = fma(-mu.y, top.x, v.y);
        col[r2] = v;
      }
    }
    __syncthreads();
  }
  if (singular && tid == 0) atomicOr(flags, DEV_SINGULAR_UPHI);
}

// X_i = U_ii^{-1} Y_i for the diagonal block rows i0..i0+nbp-1 (right-hand
// sides are the columns n .. 2n-1 of W).
__global__ void __launch_bounds__(kPanelThreads)
    block_backsolve_kernel(int n, int i0, int nbp, double2* __restrict__ Wall) {
  const int b = blockIdx.x;
  double2* W = Wall + size_t(b) * n * 2 * n;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  for (int jj = nbp - 1; jj >= 0; --jj) {
    const int r = i0 + jj;
    const double2 rr = crcp(W[r + size_t(r) * n]);
    for (int c = n + tid; c < 2 * n; c += nt) W[r + size_t(c) * n] = cmul(W[r + size_t(c) * n], rr);
    __syncthreads();
    for (int c = n + warp; c < 2 * n; c += nw) {
      const double2 x = W[r + size_t(c) * n];
      double2* col = W + size_t(c) * n;
      for (int r2 = i0 + lane; r2 < r; r2 += 32) {
        double2 v = col[r2];
        const double2 mu = W[r2 + size_t(r) * n];
        v.x = fma(-mu.x, x.x, v.x);
        v.x = fma(mu.y, x.y, v.x);
        v.y = fma(-mu.x, x.y, v.y);
        v.y = fma(-mu.y, x.x, v.y);
        col[r2] = v;
      }
    }
    __syncthreads();
  }
}

// Panel of at most kPanelMax columns factored in shared memory (one CTA per
// angle): partial pivoting by max |re| + |im| (first row on ties, as izamax),
// multipliers and the updated panel written back, pivots (absolute rows) to
// piv[b * n + j].  The interchanges of the other columns and the block row
// U12 are left to panel_apply_kernel (or panel_swap_kernel and a product with
// L11^{-1}).  With Tinv non-null the inverses of the unit lower L11 and of
// U11 are written to Tinv + b * tstride (nbp x nbp each, column-major, the
// second at + kPanelMax^2), computed right-looking in shared memory: every
// step updates all remaining entries at once, so the dependent FP64 chain is
// one complex update per step.
constexpr int kFactorThreads = 256;
constexpr int kApplyThreads = 32;  // one warp: L11 + the column buffers stay under 48 KB

__global__ void __launch_bounds__(kFactorThreads)
    panel_factor_kernel(int n, int j0, int nbp, double2* __restrict__ Wall, int* __restrict__ piv, int* flags,
                        double2* __restrict__ Tinv, long long tstride) {
  extern __shared__ double2 P[];  // rows j0..n-1 of the panel, column-major, ld m; then L11^-1, U11^-1
  __shared__ int s_piv;
  __shared__ double s_pv;
  __shared__ double2 s_rp;
  const int b = blockIdx.x;
  double2* W = Wall + size_t(b) * 2 * n * n;
  const int m = n - j0;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int idx = tid; idx < m * nbp; idx += blockDim.x) {
    const int r = idx % m, c = idx / m;
    P[c * m + r] = W[(j0 + r) + size_t(j0 + c) * n];
  }
  __syncthreads();
  bool singular = false;
  for (int jj = 0; jj < nbp; ++jj) {
    if (warp == 0) {
      long long best = -1;
      int bi = m;
      for (int r = jj + lane; r < m; r += 32) {
        const long long v = __double_as_longlong(cabs1(P[jj * m + r]));
        if (v > best) {
          best = v;
          bi = r;
        }
      }
      warp_argmax_key(best, bi);
      if (lane == 0) {
        s_piv = bi;
        s_pv = __longlong_as_double(best);
        // the pivot's reciprocal, once (an FP64 division costs ~1000 cycles)
        const double2 pe = P[jj * m + bi];
        s_rp = (s_pv == 0.0) ? make_double2(0.0, 0.0) : crcp(pe);
      }
    }
    __syncthreads();
    int p = s_piv;
    const double pv = s_pv;
    if (pv == 0.0) {
      singular = true;
      p = jj;
    }
    if (tid == 0) piv[size_t(b) * n + j0 + jj] = j0 + p;
    if (p != jj)
      for (int c = tid; c < nbp; c += blockDim.x) {
        const double2 t = P[c * m + jj];
        P[c * m + jj] = P[c * m + p];
        P[c * m + p] = t;
      }
    __syncthreads();
    const double2 rp = s_rp;
    for (int r = jj + 1 + tid; r < m; r += blockDim.x) {
      const double2 mu = cmul(P[jj * m + r], rp);
      P[jj * m + r] = mu;
      for (int c = jj + 1; c < nbp; ++c) {
        const double2 top = P[c * m + jj];
        double2 v = P[c * m + r];
        v.x = fma(-mu.x, top.x, v.x);
        v.x = fma(mu.y, top.y, v.x);
        v.y = fma(-mu.x, top.y, v.y);
        v.y = fma(-mu.y, top.x, v.y);
        P[c * m + r] = v;
      }
    }
    __syncthreads();
  }
  for (int idx = tid; idx < m * nbp; idx += blockDim.x) {
    const int r = idx % m, c = idx / m;
    W[(j0 + r) + size_t(j0 + c) * n] = P[c * m + r];
  }
  if (singular && tid == 0) atomicOr(flags, DEV_SINGULAR_UPHI);
  if (!Tinv) return;
  // X = L11^{-1}: X = I; step k: X[i][j] -= L[i][k] X[k][j] for i > k >= j
  double2* X = P + size_t(m) * nbp;
  double2* Y = X + nbp * nbp;
  __shared__ double2 rdu[kPanelMax];
  for (int idx = tid; idx < nbp * nbp; idx += blockDim.x) {
    const int i = idx % nbp, j = idx / nbp;
    X[idx] = make_double2(i == j ? 1.0 : 0.0, 0.0);
    Y[idx] = X[idx];
  }
  if (tid < nbp) rdu[tid] = singular ? make_double2(0.0, 0.0) : crcp(P[tid * m + tid]);
  __syncthreads();
  for (int k = 0; k + 1 < nbp; ++k) {
    const int rows = nbp - 1 - k;
    for (int idx = tid; idx < rows * (k + 1); idx += blockDim.x) {
      const int i = k + 1 + idx % rows, j = idx / rows;
      const double2 l = P[k * m + i], x = X[k + j * nbp];
      double2 v = X[i + j * nbp];
      v.x = fma(-l.x, x.x, v.x);
      v.x = fma(l.y, x.y, v.x);
      v.y = fma(-l.x, x.y, v.y);
      v.y = fma(-l.y, x.x, v.y);
      X[i + j * nbp] = v;
    }
    __syncthreads();
  }
  // Y = U11^{-1}: Y = I; step k (last to first): row k scaled by 1/U_kk, then
  // Y[i][j] -= U[i][k] Y[k][j] for i < k <= j
  for (int k = nbp - 1; k >= 0; --k) {
    for (int j = k + tid; j < nbp; j += blockDim.x) Y[k + j * nbp] = cmul(Y[k + j * nbp], rdu[k]);
    __syncthreads();
    const int cols = nbp - k;
    for (int idx = tid; idx < k * cols; idx += blockDim.x) {
      const int i = idx % k, j = k + idx / k;
      const double2 u = P[k * m + i], y = Y[k + j * nbp];
      double2 v = Y[i + j * nbp];
      v.x = fma(-u.x, y.x, v.x);
      v.x = fma(u.y, y.y, v.x);
      v.y = fma(-u.x, y.y, v.y);
      v.y = fma(-u.y, y.x, v.y);
      Y[i + j * nbp] = v;
    }
    __syncthreads();
  }
  double2* T = Tinv + size_t(b) * tstride;
  for (int idx = tid; idx < nbp * nbp; idx += blockDim.x) {
    T[idx] = X[idx];
    T[kPanelMax * kPanelMax + idx] = Y[idx];
  }
}

// Panel of the blocked Gauss-Jordan solve (GEMM modes 1 and 2), one CTA per
// angle.  The pivot rows are chosen by a single-precision Crout elimination
// of the panel rows j0 .. n-1 with partial pivoting (first maximum of
// |re| + |im|, as izamax): warp w holds columns w, w + 8, w + 16, w + 24,
// lane l rows l, l + 32, ... (SLOTS rows a lane); one barrier per column
// (before it the pivot column's warp finds and swaps the pivot row and forms
// its reciprocal; after it the other warps swap the rows, every warp scales
// its entries of the pivot row and updates its columns).  Only the choice of
// rows comes from single precision: the block A11 of the chosen rows is then
// inverted in FP64 from the original values by Gauss-Jordan elimination
// without further interchanges (its pivots are the partial-pivoting pivots),
// T = A11^{-1} written to Tinv + b * tstride (nbp x nbp, column-major).  The
// panel columns of W are rewritten for the elimination product: the block
// rows j0 .. j0+nbp-1 as zeros, the rows below with their original values in
// the pivoted order.  The other columns' interchanges are left to
// panel_swap_kernel.
__device__ __forceinline__ float2 shfl_f2(float2 v, int src) {
  return make_float2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

// first maximum over the warp, the result in every lane
__device__ __forceinline__ void warp_argmax_key_all(int& v, int& i) {
  for (int off = 16; off > 0; off >>= 1) {
    const int v2 = __shfl_xor_sync(0xffffffffu, v, off);
    const int i2 = __shfl_xor_sync(0xffffffffu, i, off);
    if (v2 > v || (v2 == v && i2 < i)) {
      v = v2;
      i = i2;
    }
  }
}

template <int SLOTS>
__device__ __forceinline__ float2 slot_get(const float2 (&a)[SLOTS], int s) {
  float2 v = a[0];
#pragma unroll
  for (int k = 1; k < SLOTS; ++k)
    if (k == s) v = a[k];
  return v;
}

template <int SLOTS>
__device__ __forceinline__ void slot_set(float2 (&a)[SLOTS], int s, float2 v) {
#pragma unroll
  for (int k = 0; k < SLOTS; ++k)
    if (k == s) a[k] = v;
}

// exchange rows r1 != r2 of a column held as a[slot] in lanes
template <int SLOTS>
__device__ __forceinline__ void swap_rows(float2 (&a)[SLOTS], int r1, int r2, int lane) {
  const float2 v1 = shfl_f2(slot_get(a, r1 >> 5), r1 & 31);
  const float2 v2 = shfl_f2(slot_get(a, r2 >> 5), r2 & 31);
  if (lane == (r1 & 31)) slot_set(a, r1 >> 5, v2);
  if (lane == (r2 & 31)) slot_set(a, r2 >> 5, v1);
}

__device__ __forceinline__ float2 fcmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

constexpr int kGjMaxSlots = 12;  // panels of up to 384 rows
constexpr int kGjEntries = (kPanelMax * kPanelMax + kFactorThreads - 1) / kFactorThreads;  // block entries per thread

template <int SLOTS>
__global__ void __launch_bounds__(kFactorThreads)
    panel_gj_kernel(int n, int j0, int nbp, double2* __restrict__ Wall, int* __restrict__ piv, int* flags,
                    double2* __restrict__ Tinv, long long tstride) {
  constexpr int kQ = kPanelMax / 8;
  constexpr int kP = kPanelMax + 1;
  static_assert(kFactorThreads == 256 && kPanelMax % 8 == 0, "eight warps hold the panel's columns");
  __shared__ float2 scol[2][32 * SLOTS];
  __shared__ float2 s_rp[2];
  __shared__ int s_piv[2];
  __shared__ int s_sing;
  __shared__ int srow[32 * SLOTS];
  __shared__ double2 A11[kPanelMax * kP];
  __shared__ double2 smu[kPanelMax], srk[kPanelMax];
  __shared__ double2 s_rd[2];
  const int b = blockIdx.x;
  double2* W = Wall + size_t(b) * 2 * n * n;
  const int m = n - j0;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_sing = 0;
  for (int r = tid; r < 32 * SLOTS; r += kFactorThreads) srow[r] = r;
  float2 a[kQ][SLOTS];
#pragma unroll
  for (int q = 0; q < kQ; ++q) {
    const int c = warp + 8 * q;
#pragma unroll
    for (int s = 0; s < SLOTS; ++s) {
      const int r = lane + 32 * s;
      double2 v = make_double2(0.0, 0.0);
      if (c < nbp && r < m) v = W[(j0 + r) + size_t(j0 + c) * n];
      a[q][s] = make_float2(float(v.x), float(v.y));
    }
  }
  __syncthreads();
  for (int jj = 0; jj < nbp; ++jj) {
    const int buf = jj & 1, wj = jj & 7, qj = jj >> 3;
    if (warp == wj) {
      int best = -1, bi = m;
#pragma unroll
      for (int q = 0; q < kQ; ++q)
        if (q == qj) {
#pragma unroll
          for (int s = 0; s < SLOTS; ++s) {
            const int r = lane + 32 * s;
            if (r >= jj && r < m) {
              const int v = __float_as_int(fabsf(a[q][s].x) + fabsf(a[q][s].y));
              if (v > best) {
                best = v;
                bi = r;
              }
            }
          }
        }
      warp_argmax_key_all(best, bi);
      const bool zero = best <= 0;
      const int p = zero ? jj : bi;
      if (p != jj) {
#pragma unroll
        for (int q = 0; q < kQ; ++q) swap_rows(a[q], jj, p, lane);
      }
      float2 pv = make_float2(0.f, 0.f);
#pragma unroll
      for (int q = 0; q < kQ; ++q)
        if (q == qj) {
          pv = shfl_f2(slot_get(a[q], jj >> 5), jj & 31);
#pragma unroll
          for (int s = 0; s < SLOTS; ++s) {
            const int r = lane + 32 * s;
            if (r > jj && r < m) scol[buf][r] = a[q][s];
          }
        }
      if (lane == 0) {
        const float d = fmaf(pv.x, pv.x, pv.y * pv.y);
        const float rd = (zero || !(d > 0.f)) ? 0.f : __frcp_rn(d);
        s_rp[buf] = make_float2(pv.x * rd, -pv.y * rd);
        s_piv[buf] = p;
        piv[size_t(b) * n + j0 + jj] = j0 + p;
        const int t0 = srow[jj];
        srow[jj] = srow[p];
        srow[p] = t0;
        if (zero) s_sing = 1;
      }
    }
    __syncthreads();
    if (warp != wj) {
      const int p = s_piv[buf];
      if (p != jj) {
#pragma unroll
        for (int q = 0; q < kQ; ++q) swap_rows(a[q], jj, p, lane);
      }
    }
    const float2 rp = s_rp[buf];
    float2 mu[SLOTS];
#pragma unroll
    for (int s = 0; s < SLOTS; ++s) {
      const int r = lane + 32 * s;
      mu[s] = (r > jj && r < m) ? scol[buf][r] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
      const int c = warp + 8 * q;
      if (c <= jj || c >= nbp) continue;
      // U' entry of the pivot row, then the column update
      const float2 u = fcmul(shfl_f2(slot_get(a[q], jj >> 5), jj & 31), rp);
      if (lane == (jj & 31)) slot_set(a[q], jj >> 5, u);
#pragma unroll
      for (int s = 0; s < SLOTS; ++s)
        if (32 * s + 31 > jj) {
          a[q][s].x = fmaf(-mu[s].x, u.x, fmaf(mu[s].y, u.y, a[q][s].x));
          a[q][s].y = fmaf(-mu[s].x, u.y, fmaf(-mu[s].y, u.x, a[q][s].y));
        }
    }
  }
  // the original rows in the pivoted order: the block to shared memory, the
  // rows below back to the panel (the block rows as zeros).  A column
  // belongs to one warp, so the permutation in place needs only that warp's
  // reads before its writes (one column of rows in registers at a time).
  __syncthreads();  // srow is complete
#pragma unroll
  for (int q = 0; q < kQ; ++q) {
    const int c = warp + 8 * q;
    if (c >= nbp) continue;
    double2 raw[SLOTS];
#pragma unroll
    for (int s = 0; s < SLOTS; ++s) {
      const int r = lane + 32 * s;
      raw[s] = (r < m) ? W[(j0 + srow[r]) + size_t(j0 + c) * n] : make_double2(0.0, 0.0);
      if (r < nbp) A11[r + c * kP] = raw[s];
    }
    __syncwarp();
#pragma unroll
    for (int s = 0; s < SLOTS; ++s) {
      const int r = lane + 32 * s;
      if (r < m) W[(j0 + r) + size_t(j0 + c) * n] = (r < nbp) ? make_double2(0.0, 0.0) : raw[s];
    }
  }
  __syncthreads();
  if (s_sing && tid == 0) atomicOr(flags, DEV_SINGULAR_UPHI);
  // Gauss-Jordan inverse of the block in place: step k with the reciprocal
  // of the pivot (formed by the owner of that entry at the end of the step
  // before), multipliers and the pivot row staged, then every entry at once
  if (tid == 0) s_rd[0] = crcp_newton(A11[0]);
  // entries of the nbp x nbp block, kGjEntries per thread (ei = nbp: none)
  int ei[kGjEntries], ej[kGjEntries];
#pragma unroll
  for (int e = 0; e < kGjEntries; ++e) {
    const int idx = tid + e * kFactorThreads;
    const bool in = idx < nbp * nbp;
    ei[e] = in ? idx % nbp : nbp;
    ej[e] = in ? idx / nbp : 0;
  }
  __syncthreads();
  for (int k = 0; k < nbp; ++k) {
    const double2 rd = s_rd[k & 1];
    if (tid < nbp) {
      smu[tid] = (tid == k) ? make_double2(0.0, 0.0) : cmul(A11[tid + k * kP], rd);
      srk[tid] = A11[k + tid * kP];
    }
    __syncthreads();
    double2 v[kGjEntries];
#pragma unroll
    for (int e = 0; e < kGjEntries; ++e) v[e] = (ei[e] < nbp) ? A11[ei[e] + ej[e] * kP] : make_double2(0.0, 0.0);
#pragma unroll
    for (int e = 0; e < kGjEntries; ++e) {
      const int i = ei[e], j = ej[e];
      if (i >= nbp) continue;
      if (i != k && j != k) {
        cfma(v[e], cneg(smu[i]), srk[j]);
      } else if (i == k && j != k) {
        v[e] = cmul(srk[j], rd);
      } else if (i != k) {
        v[e] = cneg(smu[i]);
      } else {
        v[e] = rd;
      }
      A11[i + j * kP] = v[e];
      if (i == k + 1 && j == k + 1) s_rd[(k + 1) & 1] = crcp_newton(v[e]);
    }
    __syncthreads();
  }
  double2* T = Tinv + size_t(b) * tstride;
  for (int idx = tid; idx < nbp * nbp; idx += kFactorThreads) T[idx] = A11[(idx % nbp) + (idx / nbp) * kP];
}

// Row interchanges of a factored panel applied to columns j1 .. 2n-1 (one
// thread per column, in the order of the pivots)
__global__ void __launch_bounds__(kApplyThreads)
    panel_swap_kernel(int n, int j0, int nbp, double2* __restrict__ Wall, const int* __restrict__ piv) {
  const int b = blockIdx.y;
  const int j1 = j0 + nbp;
  const int c = j1 + blockIdx.x * kApplyThreads + threadIdx.x;
  if (c >= 2 * n) return;
  double2* col = Wall + size_t(b) * 2 * n * n + size_t(c) * n;
  const int* pv = piv + size_t(b) * n + j0;
  for (int jj = 0; jj < nbp; ++jj) {
    const int p = pv[jj];
    if (p == j0 + jj) continue;
    const double2 tmp = col[j0 + jj];
    col[j0 + jj] = col[p];
    col[p] = tmp;
  }
}

// The same interchanges for 32 columns per CTA: the pivot sequence is first
// composed into a permutation of rows j0 .. n-1 (row r after = row src[r]
// before; at most 2 nbp rows move), then the moved rows are read with
// independent loads and written back, instead of one dependent pair of
// accesses per interchange and column.
constexpr int kPermCols = 32;
constexpr int kPermThreads = 256;
constexpr int kPermMaxRows = 1024;
__global__ void __launch_bounds__(kPermThreads)
    panel_perm_kernel(int n, int j0, int nbp, double2* __restrict__ Wall, const int* __restrict__ piv) {
  __shared__ int src[kPermMaxRows];
  __shared__ int moved[2 * kPanelMax];
  __shared__ int nmoved;
  __shared__ double2 buf[2 * kPanelMax][kPermCols];
  const int b = blockIdx.y, t = threadIdx.x;
  const int m = n - j0, j1 = j0 + nbp;
  double2* W = Wall + size_t(b) * 2 * n * n;
  for (int r = t; r < m; r += kPermThreads) src[r] = r;
  if (t == 0) nmoved = 0;
  __syncthreads();
  if (t == 0) {
    const int* pv = piv + size_t(b) * n + j0;
    for (int jj = 0; jj < nbp; ++jj) {
      const int p = pv[jj] - j0;
      if (p != jj) {
        const int x = src[jj];
        src[jj] = src[p];
        src[p] = x;
      }
    }
  }
  __syncthreads();
  for (int r = t; r < m; r += kPermThreads)
    if (src[r] != r) moved[atomicAdd(&nmoved, 1)] = r;
  __syncthreads();
  const int nm = nmoved;
  const int c0 = j1 + blockIdx.x * kPermCols;
  for (int idx = t; idx < nm * kPermCols; idx += kPermThreads) {
    const int k = idx / kPermCols, cc = idx - k * kPermCols, c = c0 + cc;
    if (c < 2 * n) buf[k][cc] = W[(j0 + src[moved[k]]) + size_t(c) * n];
  }
  __syncthreads();
  for (int idx = t; idx < nm * kPermCols; idx += kPermThreads) {
    const int k = idx / kPermCols, cc = idx - k * kPermCols, c = c0 + cc;
    if (c < 2 * n) W[(j0 + moved[k]) + size_t(c) * n] = buf[k][cc];
  }
}

// Columns j1 .. 2n-1 (one thread each): the panel's row interchanges, then
// U12 = L11^{-1} A12 on the block row j0 .. j1-1.
__global__ void __launch_bounds__(kApplyThreads)
    panel_apply_kernel(int n, int j0, int nbp, double2* __restrict__ Wall, const int* __restrict__ piv) {
  __shared__ double2 L[kPanelMax][kPanelMax + 1];
  __shared__ double2 xb[kPanelMax][kApplyThreads];
  __shared__ int sp[kPanelMax];
  const int b = blockIdx.y;
  double2* W = Wall + size_t(b) * 2 * n * n;
  const int j1 = j0 + nbp;
  for (int idx = threadIdx.x; idx < nbp * nbp; idx += blockDim.x) {
    const int i = idx % nbp, k = idx / nbp;
    L[i][k] = W[(j0 + i) + size_t(j0 + k) * n];
  }
  for (int i = threadIdx.x; i < nbp; i += blockDim.x) sp[i] = piv[size_t(b) * n + j0 + i] - j0;
  __syncthreads();
  const int t = threadIdx.x;
  const int c = j1 + blockIdx.x * kApplyThreads + t;
  if (c >= 2 * n) return;
  double2* col = W + size_t(c) * n;
  for (int i = 0; i < nbp; ++i) xb[i][t] = col[j0 + i];
  for (int jj = 0; jj < nbp; ++jj) {
    const int p = sp[jj];
    if (p == jj) continue;
    if (p < nbp) {
      const double2 tmp = xb[jj][t];
      xb[jj][t] = xb[p][t];
      xb[p][t] = tmp;
    } else {
      const double2 tmp = col[j0 + p];
      col[j0 + p] = xb[jj][t];
      xb[jj][t] = tmp;
    }
  }
  for (int i = 1; i < nbp; ++i) {
    double2 v = xb[i][t];
    for (int k = 0; k < i; ++k) {
      const double2 mu = L[i][k], x = xb[k][t];
      v.x = fma(-mu.x, x.x, v.x);
      v.x = fma(mu.y, x.y, v.x);
      v.y = fma(-mu.x, x.y, v.y);
      v.y = fma(-mu.y, x.x, v.y);
    }
    xb[i][t] = v;
  }
  for (int i = 0; i < nbp; ++i) col[j0 + i] = xb[i][t];
}

// X_i = U_ii^{-1} Y_i on block row i0 .. i0+nbp-1, right-hand sides the
// columns n .. 2n-1 (one thread each)
__global__ void __launch_bounds__(kApplyThreads)
    backsolve_apply_kernel(int n, int i0, int nbp, double2* __restrict__ Wall) {
  __shared__ double2 Us[kPanelMax][kPanelMax + 1];
  __shared__ double2 rd[kPanelMax];
  __shared__ double2 xb[kPanelMax][kApplyThreads];
  const int b = blockIdx.y;
  double2* W = Wall + size_t(b) * 2 * n * n;
  for (int idx = threadIdx.x; idx < nbp * nbp; idx += blockDim.x) {
    const int i = idx % nbp, k = idx / nbp;
    if (k >= i) Us[i][k] = W[(i0 + i) + size_t(i0 + k) * n];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nbp; i += blockDim.x) rd[i] = crcp(Us[i][i]);
  __syncthreads();
  const int t = threadIdx.x;
  const int c = n + blockIdx.x * kApplyThreads + t;
  if (c >= 2 * n) return;
  double2* col = W + size_t(c) * n;
  for (int i = 0; i < nbp; ++i) xb[i][t] = col[i0 + i];
  for (int i = nbp - 1; i >= 0; --i) {
    double2 v = xb[i][t];
    for (int k = i + 1; k < nbp; ++k) {
      const double2 u = Us[i][k], x = xb[k][t];
      v.x = fma(-u.x, x.x, v.x);
      v.x = fma(u.y, x.y, v.x);
      v.y = fma(-u.x, x.y, v.y);
      v.y = fma(-u.y, x.x, v.y);
    }
    xb[i][t] = cmul(v, rd[i]);
  }
  for (int i = 0; i < nbp; ++i) col[i0 + i] = xb[i][t];
}

// A_phi(i, j) = conj(X(i, j)) = conj(Y(j, i)), Y = W(:, n:2n)
__global__ void thouless_out_kernel(int n, int G, const double2* __restrict__ Wall, double2* __restrict__ A) {
  const size_t nn = size_t(n) * n;
  const size_t idx = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (idx >= nn * G) return;
  const int b = int(idx / nn);
  const int e = int(idx - size_t(b) * nn);
  const int j = e / n, i = e - j * n;
  A[idx] = cconj(Wall[size_t(b) * 2 * nn + j + size_t(n + i) * n]);
}

inline unsigned nblk(size_t total, int tb) { return unsigned((total + tb - 1) / tb); }

// host-side angle table (assign_angles, module_projection.f90:112-185)
struct AngleTable {
  std::vector<double> php, phn, mult;
  std::vector<std::complex<double>> w;
};

AngleTable make_angles_uncached(const tvap_proj_opts& o, bool fold);

// the last table per host thread (an iteration asks for the same one twice:
// for the workspace size and for the projection)
const AngleTable& make_angles(const tvap_proj_opts& o, bool fold) {
  struct Key {
    int Mp, Mn;
    double facpi, vz, vn;
    bool fold;
    bool operator==(const Key& k) const {
      return Mp == k.Mp && Mn == k.Mn && facpi == k.facpi && vz == k.vz && vn == k.vn && fold == k.fold;
    }
  };
  static thread_local Key key{-1, -1, 0.0, 0.0, 0.0, false};
  static thread_local AngleTable table;
  const Key k{o.Mphip, o.Mphin, o.facpi, o.valence_Z, o.valence_N, fold};
  if (!(k == key)) {
    table = make_angles_uncached(o, fold);
    key = k;
  }
  return table;
}

AngleTable make_angles_uncached(const tvap_proj_opts& o, bool fold) {
  AngleTable t;
  const int Mp = o.Mphip, Mn = o.Mphin;
  const std::complex<double> I(0.0, 1.0);
  auto phi = [&](int M, int j) { return (M % 2 == 1) ? o.facpi * (j - 1.0) / M : o.facpi * (j - 0.5) / M; };
  auto partner = [](int M, int j) { return (M % 2 == 1) ? ((M - (j - 1)) % M) + 1 : M + 1 - j; };
  std::vector<char> seen(size_t(Mp) * Mn, 0);
  for (int jp = 1; jp <= Mp; ++jp)
    for (int jn = 1; jn <= Mn; ++jn) {
      if (seen[size_t(jp - 1) * Mn + (jn - 1)]) continue;
      seen[size_t(jp - 1) * Mn + (jn - 1)] = 1;
      double mult = 1.0;
      if (fold) {
        const int qp = partner(Mp, jp), qn = partner(Mn, jn);
        if (!(qp == jp && qn == jn)) {
          seen[size_t(qp - 1) * Mn + (qn - 1)] = 1;
          mult = 2.0;
        }
      }
      const double pp = phi(Mp, jp), pn = phi(Mn, jn);
      t.php.push_back(pp);
      t.phn.push_back(pn);
      t.mult.push_back(mult);
      t.w.push_back(std::exp(-I * pp * o.valence_Z) / double(Mp) * std::exp(-I * pn * o.valence_N) / double(Mn));
    }
  return t;
}

bool is_integer(double x) { return std::fabs(x - std::round(x)) < 1e-12; }

int real_gemm(int M, int N, int K, View A, View B, double* C, int ldc, double alpha, double beta, cudaStream_t s) {
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
  g.cbs = 0;
  g.alpha = make_double2(alpha, 0.0);
  g.beta = make_double2(beta, 0.0);
  g.a_real = g.b_real = g.c_real = true;
  return gemm(g, s);
}

}  // namespace


// Gauss-Jordan solve of angles [g0, g0 + gc) on stream s (panels of nb
// columns); ev_first, when given, is recorded after the first panel's
// factorisation.  build_augmented_kernel has filled W.
// sb (may be null): a stream for the look-ahead -- the elimination product
// of panel k splits into the next panel's columns (on s, so that panel k+1 is
// factored right after them) and the rest (on sb, beside that factorisation;
// ev_ready / ev_bulk order the two streams), and the row interchanges of
// panel k+1 wait for the rest.  Panel k+1 writes only its own columns, the
// rest only the columns right of them.
int gj_solve_range(tvap_ctx* c, int g0, int gc, int nb, cudaStream_t s, cudaEvent_t ev_first,
                   cudaStream_t sb = nullptr, cudaEvent_t ev_ready = nullptr, cudaEvent_t ev_bulk = nullptr) {
  Workspace* w = c->ws;
  const int n = c->n;
  const size_t nn = size_t(n) * n;
  const long long bsW = 2LL * n * n;
  const long long tstride = (long long)tinv_stride(n);
  double2* W = w->W + size_t(g0) * 2 * nn;
  int* piv = w->piv + size_t(g0) * n;
  double2* Tinv = w->Tinv + size_t(g0) * tstride;
  int rc, blk = 0;
  for (int j0 = 0; j0 < n; j0 += nb, ++blk) {
    const int nbp = std::min(nb, n - j0);
    const int j1 = j0 + nbp;
    double2* tinv = Tinv + size_t(blk) * 2 * kPanelMax * kPanelMax;
    switch ((n - j0 + 31) / 32) {
#define TVAP_PANEL_GJ(S)                                                                                 \
  case S:                                                                                                \
    panel_gj_kernel<S><<<gc, kFactorThreads, 0, tvap::counted(s)>>>(n, j0, nbp, W, piv, c->d_flags, tinv,\
                                                                     tstride);                           \
    break;
      TVAP_PANEL_GJ(1)
      TVAP_PANEL_GJ(2)
      TVAP_PANEL_GJ(3)
      TVAP_PANEL_GJ(4)
      TVAP_PANEL_GJ(5)
      TVAP_PANEL_GJ(6)
      TVAP_PANEL_GJ(7)
      TVAP_PANEL_GJ(8)
      TVAP_PANEL_GJ(9)
      TVAP_PANEL_GJ(10)
      TVAP_PANEL_GJ(11)
      TVAP_PANEL_GJ(12)
#undef TVAP_PANEL_GJ
      default:
        return TVAP_ERR_ARG;
    }
    if (j0 == 0 && ev_first) TVAP_CUDA(cudaEventRecord(ev_first, s));
    // the bulk of the previous elimination product must be done before the
    // interchanges touch its columns
    if (sb && j0 > 0) TVAP_CUDA(cudaStreamWaitEvent(s, ev_bulk, 0));
    if (j1 < 2 * n) {
      if (n - j0 <= kPermMaxRows) {
        dim3 gp((2 * n - j1 + kPermCols - 1) / kPermCols, gc);
        panel_perm_kernel<<<gp, kPermThreads, 0, tvap::counted(s)>>>(n, j0, nbp, W, piv);
      } else {
        dim3 ga((2 * n - j1 + kApplyThreads - 1) / kApplyThreads, gc);
        panel_swap_kernel<<<ga, kApplyThreads, 0, tvap::counted(s)>>>(n, j0, nbp, W, piv);
      }
    }
    // the block row: R = T [A12 | B1] in place (the operands are split into
    // digit planes before the product is formed)
    {
      GemmArgs g{};
      g.M = nbp;
      g.N = 2 * n - j1;
      g.K = nbp;
      g.batch = gc;
      g.A = View{tinv, 1, nbp, tstride};
      g.B = View{W + j0 + size_t(j1) * n, 1, n, bsW};
      g.C = W + j0 + size_t(j1) * n;
      g.crs = 1;
      g.ccs = n;
      g.cbs = bsW;
      g.alpha = make_double2(1.0, 0.0);
      g.beta = make_double2(0.0, 0.0);
      if ((rc = gemm_ozaki(g, s))) return rc;
    }
    // all other rows: W[:, j1:] -= W[:, j0:j1] R (the block rows' panel
    // entries are zero, so they keep R)
    GemmArgs g{};
    g.M = n;
    g.N = 2 * n - j1;
    g.K = nbp;
    g.batch = gc;
    g.A = View{W + size_t(j0) * n, 1, n, bsW};
    g.B = View{W + j0 + size_t(j1) * n, 1, n, bsW};
    g.C = W + size_t(j1) * n;
    g.crs = 1;
    g.ccs = n;
    g.cbs = bsW;
    g.alpha = make_double2(-1.0, 0.0);
    g.beta = make_double2(1.0, 0.0);
    g.three_m = true;
    const int j2 = j1 + std::min(nb, n - j1);  // the next panel's columns end
    if (sb && j1 < n) {
      // look-ahead: columns j2 .. 2n-1 on sb, then j1 .. j2-1 on s
      TVAP_CUDA(cudaEventRecord(ev_ready, s));
      TVAP_CUDA(cudaStreamWaitEvent(sb, ev_ready, 0));
      GemmArgs gb = g;
      gb.N = 2 * n - j2;
      gb.B = View{W + j0 + size_t(j2) * n, 1, n, bsW};
      gb.C = W + size_t(j2) * n;
      if ((rc = gemm(gb, sb))) return rc;
      TVAP_CUDA(cudaEventRecord(ev_bulk, sb));
      g.N = j2 - j1;
    }
    if ((rc = gemm(g, s))) return rc;
  }
  const size_t tot = nn * gc;
  thouless_out_kernel<<<nblk(tot, 256), 256, 0, tvap::counted(s)>>>(n, gc, W, w->A + size_t(g0) * nn);
  TVAP_CUDA(cudaGetLastError());
  return TVAP_OK;
}

int blocked_thouless_solve(tvap_ctx* c, int G, cudaStream_t s) {
  Workspace* w = c->ws;
  const int n = c->n;
  const long long bsW = 2LL * n * n;
  // panels of at most kPanelMax columns, equal widths; the shared-memory panel
  // (n x nb complex) must fit, else the former wider kernels run from global
  const int npanels = (n + kPanelMax - 1) / kPanelMax;
  const int nb_smem = (n + npanels - 1) / npanels;
  // with the emulated products, the triangular solves of the block rows and
  // of the back substitution run as products with the inverted diagonal
  // blocks (computed by the panel kernel) on the tensor cores; on the FP64
  // pipe they stay one-thread-per-column substitutions
  const bool inv_path = g_gemm_mode >= 1;
  const size_t panel_bytes =
      sizeof(double2) * (size_t(n) * nb_smem + (inv_path ? 2 * size_t(nb_smem) * nb_smem : 0));
  const bool smem_path = panel_bytes <= size_t(jacobi32_smem_limit());
  const bool use_inv = inv_path && smem_path;
  const int nb = smem_path ? nb_smem : ((n <= 64) ? n : 28);
  const long long tstride = (long long)tinv_stride(n);
  int rc;
  if (smem_path && panel_bytes > 48 * 1024) {
    if (int r = smem_opt_in((const void*)panel_factor_kernel, jacobi32_smem_limit())) return r;
  }
  {
    dim3 grid(std::max(1, (2 * n + 15) / 16), G);
    build_augmented_kernel<<<grid, kPanelThreads, 0, tvap::counted(s)>>>(n, w->Uphi, w->Vphi, w->W);
  }
  // product with an inverted diagonal block, in place on a block row:
  // rows r0 .. r0+nbp-1 of columns c0 .. 2n-1 <- T (nbp x nbp) times them
  // (the operands are split into digit planes before the product is formed,
  // so the output may overwrite its input)
  auto block_row_product = [&](int blk, int which, int r0, int nbp, int c0) -> int {
    GemmArgs g{};
    g.M = nbp;
    g.N = 2 * n - c0;
    g.K = nbp;
    g.batch = G;
    g.A = View{w->Tinv + (size_t(blk) * 2 + which) * kPanelMax * kPanelMax, 1, nbp, tstride};
    g.B = View{w->W + r0 + size_t(c0) * n, 1, n, bsW};
    g.C = w->W + r0 + size_t(c0) * n;
    g.crs = 1;
    g.ccs = n;
    g.cbs = bsW;
    g.alpha = make_double2(1.0, 0.0);
    g.beta = make_double2(0.0, 0.0);
    return gemm_ozaki(g, s);
  };
  // Blocked Gauss-Jordan (the emulated products, panels of up to 192 rows):
  // per panel the factor kernel chooses the pivots and forms T = A11^{-1},
  // the block row becomes T [A12 | B1] and one product eliminates the panel
  // columns from all other rows; no back substitution follows.
  if (use_inv && (n + 31) / 32 <= kGjMaxSlots && nb <= kPanelMax) {
    // Two halves of the angles on two streams, the second started after the
    // first half's first panel: a panel factorisation takes the same time
    // for any number of angles (one CTA each, latency-bound), so one half's
    // factorisation runs beside the other half's products.  The products
    // leave SMs for it (their CTAs are capped at the SMs the other half's
    // panels do not hold: a panel CTA and a product CTA do not fit one SM).
    const bool split = c->streamM2 && G >= 32 && c->tune_groups != 1;
    const bool la = c->tune_lookahead != 0;
    if (!split)
      return gj_solve_range(c, 0, G, nb, s, nullptr, la ? c->streamB[0] : nullptr, c->ev_la[0][0], c->ev_la[0][1]);
    const int sms = device_sms();
    const int G1 = (G + 1) / 2, G2 = G - G1;
    TcGridCap cap(c->tune_cap == 2 ? 0 : c->tune_cap == 1 ? sms / 2 : std::max(sms - G1, sms / 2));
    if ((rc = gj_solve_range(c, 0, G1, nb, s, c->ev_stagger, la ? c->streamB[0] : nullptr, c->ev_la[0][0],
                             c->ev_la[0][1])))
      return rc;
    TVAP_CUDA(cudaStreamWaitEvent(c->streamM2, c->ev_stagger, 0));
    if ((rc = gj_solve_range(c, G1, G2, nb, c->streamM2, nullptr, la ? c->streamB[1] : nullptr, c->ev_la[1][0],
                             c->ev_la[1][1])))
      return rc;
    TVAP_CUDA(cudaEventRecord(c->ev_join2, c->streamM2));
    TVAP_CUDA(cudaStreamWaitEvent(s, c->ev_join2, 0));
    return TVAP_OK;
  }
  int blk = 0;
  for (int j0 = 0; j0 < n; j0 += nb, ++blk) {
    const int nbp = std::min(nb, n - j0);
    const int j1 = j0 + nbp;
    if (smem_path) {
      const size_t fac_bytes = sizeof(double2) * (size_t(n - j0) * nbp + (use_inv ? 2 * size_t(nbp) * nbp : 0));
      double2* tinv = use_inv ? w->Tinv + size_t(blk) * 2 * kPanelMax * kPanelMax : nullptr;
      panel_factor_kernel<<<G, kFactorThreads, fac_bytes, tvap::counted(s)>>>(n, j0, nbp, w->W, w->piv, c->d_flags, tinv, tstride);
      dim3 ga((2 * n - j1 + kApplyThreads - 1) / kApplyThreads, G);
      if (use_inv) {
        panel_swap_kernel<<<ga, kApplyThreads, 0, tvap::counted(s)>>>(n, j0, nbp, w->W, w->piv);
        if ((rc = block_row_product(blk, 0, j0, nbp, j1))) return rc;
      } else {
        panel_apply_kernel<<<ga, kApplyThreads, 0, tvap::counted(s)>>>(n, j0, nbp, w->W, w->piv);
      }
    } else {
      panel_kernel<<<G, kPanelThreads, 0, tvap::counted(s)>>>(n, j0, nbp, w->W, c->d_flags);
    }
    if (j1 < n) {
      // A22 -= L21 U12 over columns j1 .. 2n-1
      GemmArgs g{};
      g.M = n - j1;
      g.N = 2 * n - j1;
      g.K = nbp;
      g.batch = G;
      g.A = View{w->W + j1 + size_t(j0) * n, 1, n, bsW};
      g.B = View{w->W + j0 + size_t(j1) * n, 1, n, bsW};
      g.C = w->W + j1 + size_t(j1) * n;
      g.crs = 1;
      g.ccs = n;
      g.cbs = bsW;
      g.alpha = make_double2(-1.0, 0.0);
      g.beta = make_double2(1.0, 0.0);
      g.three_m = true;
      if ((rc = gemm(g, s))) return rc;
    }
  }
  // back substitution, block rows from the last
  const int nblocks = (n + nb - 1) / nb;
  for (int bi = nblocks - 1; bi >= 0; --bi) {
    const int i0 = bi * nb, nbp = std::min(nb, n - i0), i1 = i0 + nbp;
    if (i1 < n) {
      // Y_i -= U_{i, i1:n} X_{i1:n}
      GemmArgs g{};
      g.M = nbp;
      g.N = n;
      g.K = n - i1;
      g.batch = G;
      g.A = View{w->W + i0 + size_t(i1) * n, 1, n, bsW};
      g.B = View{w->W + i1 + size_t(n) * n, 1, n, bsW};
      g.C = w->W + i0 + size_t(n) * n;
      g.crs = 1;
      g.ccs = n;
      g.cbs = bsW;
      g.alpha = make_double2(-1.0, 0.0);
      g.beta = make_double2(1.0, 0.0);
      g.three_m = true;
      if ((rc = gemm(g, s))) return rc;
    }
    if (use_inv) {
      // X_i = U_ii^{-1} Y_i
      if ((rc = block_row_product(bi, 1, i0, nbp, n))) return rc;
    } else if (smem_path) {
      dim3 gb((n + kApplyThreads - 1) / kApplyThreads, G);
      backsolve_apply_kernel<<<gb, kApplyThreads, 0, tvap::counted(s)>>>(n, i0, nbp, w->W);
    } else {
      block_backsolve_kernel<<<G, kPanelThreads, 0, tvap::counted(s)>>>(n, i0, nbp, w->W);
    }
  }
  const size_t tot = size_t(n) * n * G;
  thouless_out_kernel<<<nblk(tot, 256), 256, 0, tvap::counted(s)>>>(n, G, w->W, w->A);
  TVAP_CUDA(cudaGetLastError());
  return TVAP_OK;
}

// Eigenvectors of rho (w->rho) into w->D (ascending): FP32 Jacobi in shared
// memory, three FP64 refinement steps on all SMs, exact diagonalisation of
// degenerate clusters; the exact FP64 Jacobi runs only if the final check
// (orthonormality, decoupled clusters) fails or n is too large for the
// shared-memory stage.
namespace {

// Refinement steps from the approximate eigenvectors in X (Xn scratch), the
// exact treatment of near-degenerate clusters and the final check; *fail is
// the check's verdict (read back on the host) and *Xout the buffer holding
// the refined columns.  assign: fix the clusters at the first step (else
// keep those of the previous call); second_order: add F^2/2 to each step.
int refine_canonical(tvap_ctx* c, double* X, double* Xn, int steps, int* fail, cudaStream_t s, bool assign,
                     bool second_order, double** Xout) {
  Workspace* w = c->ws;
  const int n = c->n;
  const size_t nn = size_t(n) * n;
  const View Rho = view_cm(w->rho, n, 0);
  int rc;
  // R = X^T X and S = X^T rho X in one product X^T [X | rho X] (rho X is kept
  // right after X in its buffer, R and S are adjacent)
  auto gram = [&](double* Xc) -> int {
    int r;
    if ((r = real_gemm(n, n, n, Rho, view_cm(Xc, n, 0), Xc + nn, n, 1.0, 0.0, s))) return r;
    return real_gemm(n, 2 * n, n, view_t(view_cm(Xc, n, 0)), view_cm(Xc, n, 0), w->RS, n, 1.0, 0.0, s);
  };
  for (int step = 0; step < steps; ++step) {
    const View Xv = view_cm(X, n, 0);
    if ((rc = gram(X))) return rc;
    refine_lambda_kernel<<<1, kRlThreads, 0, tvap::counted(s)>>>(n, w->Rr, w->Sr, w->rho, w->lam, w->rscal);
    if (step == 0 && assign)
      cluster_assign_kernel<<<1, kCfThreads, 0, tvap::counted(s)>>>(n, w->Sr, w->lam, w->rscal, w->cid);
    refine_update_kernel<<<nblk(nn, 256), 256, 0, tvap::counted(s)>>>(n, w->Rr, w->Sr, w->lam, w->rscal, w->cid,
                                                                      w->Mr, w->Br);
    if (second_order) {
      const View Fv = view_cm(w->Br, n, 0);
      if ((rc = real_gemm(n, n, n, Fv, Fv, w->Mr, n, 0.5, 1.0, s))) return rc;  // M += F^2 / 2
    }
    if ((rc = real_gemm(n, n, n, Xv, view_cm(w->Mr, n, 0), Xn, n, 1.0, 0.0, s))) return rc;
    std::swap(X, Xn);
  }
  if ((rc = gram(X))) return rc;
  refine_lambda_kernel<<<1, kRlThreads, 0, tvap::counted(s)>>>(n, w->Rr, w->Sr, w->rho, w->lam, w->rscal);
  cluster_finish_kernel<<<1, kCfThreads, 0, tvap::counted(s)>>>(n, w->Sr, X, w->rscal, w->cid, w->D, w->evals,
                                                                 w->cperm, w->bigd, w->rflag);
  TVAP_CUDA(cudaGetLastError());
  int hr[3] = {1, 0, 0};
  int bd[2 * kCfBigSlots];
  TVAP_CUDA(cudaMemcpyAsync(hr, w->rflag, sizeof(hr), cudaMemcpyDeviceToHost, s));
  TVAP_CUDA(cudaMemcpyAsync(bd, w->bigd, sizeof(bd), cudaMemcpyDeviceToHost, s));
  TVAP_CUDA(cudaStreamSynchronize(s));
  *fail = hr[0];
  c->canon_attempts[3] += hr[1];
  if (hr[0] == 0 && hr[2] > 0) {
    // the large clusters: the FP64 Jacobi of each block (it starts close to
    // diagonal: the coupling inside a cluster is that left by the FP32
    // stage), its eigenvectors rotate the cluster's columns.  w->jac, w->Mr,
    // w->lam and w->jwork are free here.
    int nb = 0;
    for (int b = 0; b < hr[2] && b < kCfBigSlots; ++b, ++nb) {
      const int k0 = bd[2 * b], m = bd[2 * b + 1];
      if (k0 < 0 || m < 1 || k0 + m > n) {
        *fail = 4;  // not a cluster of this basis: the attempt fails
        break;
      }
      big_cluster_extract_kernel<<<nblk(size_t(m) * m, 256), 256, 0, tvap::counted(s)>>>(n, m, w->Sr, w->cperm + k0,
                                                                                      w->jac);
      // ||rho||_F (rscal[1] of the last Gram step) sets the rounding level
      if ((rc = jacobi_eigen(m, w->jac, w->Mr, w->lam, w->jwork, w->rflag + 3, s, w->rscal + 1))) return rc;
      big_cluster_rotate_kernel<<<nblk(size_t(n) * m, 256), 256, 0, tvap::counted(s)>>>(
          n, m, X, w->cperm + k0, w->Mr, w->lam, w->D + size_t(k0) * n, w->evals + k0);
      TVAP_CUDA(cudaGetLastError());
    }
    c->canon_attempts[7] += nb;
    int jf = 0;
    TVAP_CUDA(cudaMemcpyAsync(&jf, w->rflag + 3, sizeof(int), cudaMemcpyDeviceToHost, s));
    TVAP_CUDA(cudaStreamSynchronize(s));
    if (jf) *fail = 4;  // a block's Jacobi did not converge
  }
  for (int b = 0; b < 3; ++b)
    if (*fail & (1 << b)) ++c->canon_attempts[4 + b];
  *Xout = X;
  return TVAP_OK;
}

}  // namespace

// Eigenvectors of rho (w->rho) into w->D (ascending): FP32 Jacobi in shared
// memory (on rho rotated into the previous canonical basis when there is
// one), three FP64 refinement steps on all SMs, exact diagonalisation of
// degenerate clusters; the exact FP64 Jacobi runs only if the final check
// (orthonormality, decoupled clusters) fails or n is too large for the
// shared-memory stage.  (Refining the previous basis directly, without the
// Jacobi stage, does not converge when the state moves by a full gradient
// step: couplings exceed the gaps between canonical pairs.)
int eigen_canonical(tvap_ctx* c, cudaStream_t s) {
  Workspace* w = c->ws;
  const int n = c->n;
  const size_t nn = size_t(n) * n;
  int rc, fail = 1;
  // the FP32 stage: the cluster Jacobi (n <= 384), else the single-CTA one
  // when its matrices fit shared memory
  if ((n <= 384 || jacobi32_smem_bytes(n) <= jacobi32_smem_limit()) && n <= kCfMaxN) {
    double* X = w->Xr;
    double* Xn = w->Xn;
    const View Rho = view_cm(w->rho, n, 0);
    // a second attempt starts from the basis the first one refined (left in
    // w->D): the FP32 Jacobi then works on a nearly diagonal matrix whose
    // small entries keep their relative precision, which resolves the pairs
    // whose gaps were too small for the Newton steps
    const View Vn = view_cm(w->V, n, 0);
    for (int attempt = 0; attempt < 2 && fail; ++attempt) {
      const bool warm = w->have_basis || attempt > 0;
      // one-sided Jacobi on M = V^T D (M^T M = D^T rho D) over a cluster of
      // 8 CTAs; the two-sided single-CTA kernel on D^T rho D when n is too
      // large for it
      if (warm) {
        const View Dp = view_cm(w->D, n, 0);
        if ((rc = real_gemm(n, n, n, view_t(Vn), Dp, w->Br, n, 1.0, 0.0, s))) return rc;
        rc = jacobi_cluster(n, w->Br, 0, w->D, X, w->rflag + 1, s);
      } else {
        rc = jacobi_cluster(n, w->V, 1, nullptr, X, w->rflag + 1, s);
      }
      if (rc == TVAP_ERR_ARG) {
        if (jacobi32_smem_bytes(n) > jacobi32_smem_limit()) {
          fail = 1;  // neither FP32 stage runs here: the exact FP64 Jacobi below
          break;
        }
        if (warm) {
          const View Dp = view_cm(w->D, n, 0);
          if ((rc = real_gemm(n, n, n, Rho, Dp, w->Br, n, 1.0, 0.0, s))) return rc;
          if ((rc = real_gemm(n, n, n, view_t(Dp), view_cm(w->Br, n, 0), w->Sr, n, 1.0, 0.0, s))) return rc;
          if ((rc = jacobi32_smem(n, w->Sr, w->D, X, w->rflag + 1, s))) return rc;
        } else {
          if ((rc = jacobi32_smem(n, w->rho, nullptr, X, w->rflag + 1, s))) return rc;
        }
      } else if (rc) {
        return rc;
      }
      ++c->canon_attempts[0];
      double* Xf = X;
      if ((rc = refine_canonical(c, X, Xn, 3, &fail, s, true, false, &Xf))) return rc;
      if (fail && !(fail & 4)) {
        // not yet orthonormal or decoupled (nearly closed shells: an FP32
        // start with ||I - X^T X|| ~ 1e-4 and clusters of levels it could not
        // separate): two second-order steps more from the refined basis,
        // with the same clusters, before anything is recomputed
        ++c->canon_attempts[8];
        if ((rc = refine_canonical(c, Xf, Xf == X ? Xn : X, 2, &fail, s, false, true, &Xf))) return rc;
      }
    }
    if (!fail) {
      ++c->canon_attempts[1];
      w->have_basis = true;
      return TVAP_OK;
    }
  }
  // exact cyclic Jacobi in FP64
  ++c->canon_attempts[2];
  TVAP_CUDA(cudaMemcpyAsync(w->jac, w->rho, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s));
  if ((rc = jacobi_eigen(n, w->jac, w->D, w->evals, w->jwork, c->d_flags, s))) return rc;
  w->have_basis = true;
  return TVAP_OK;
}

// Canonical basis + angle-independent blocks for state (w->U, w->V).
// Angle-independent real blocks of U and V (0..7) on stream s.
int prepare_uv_blocks(tvap_ctx* c, cudaStream_t s) {
  Workspace* w = c->ws;
  const int n = c->n, h = n / 2;
  const size_t nn = size_t(n) * n;
  int rc;
  sec_begin_on(c, SEC_BLOCKS, s);
  // C_t = W_t^T W_t, W_t = rows t h .. t h + h - 1 of W = [V | U] (n x 2n), batch t = p, n
  {
    GemmArgs g{};
    g.M = g.N = 2 * n;
    g.K = h;
    g.batch = 2;
    g.A = View{w->VU, n, 1, h};  // (i, k) = W(t h + k, i)
    g.B = View{w->VU, 1, n, h};  // (k, j) = W(t h + k, j)
    g.C = w->blocks;
    g.crs = 1;
    g.ccs = 2 * n;
    g.cbs = 4 * (long long)nn;
    g.alpha = make_double2(1.0, 0.0);
    g.beta = make_double2(0.0, 0.0);
    g.a_real = g.b_real = g.c_real = true;
    if ((rc = gemm(g, s))) return rc;
  }
  sec_end_on(c, SEC_BLOCKS, s);
  return TVAP_OK;
}

// Canonical basis (construct_canonical_basis) and its blocks (8, 9) on stream
// s; host_canon receives nocc, nemp and the bad-block flag (s is
// synchronised).
int prepare_canonical(tvap_ctx* c, double occeps, double allemp_d, int* host_canon, cudaStream_t s) {
  Workspace* w = c->ws;
  const int n = c->n, h = n / 2;
  const size_t nn = size_t(n) * n;
  int rc;
  const View Vn = view_cm(w->V, n, 0), Un = view_cm(w->U, n, 0);
  sec_begin_on(c, SEC_CANONICAL, s);
  // rho = V V^T, kappa = V U^T (construct_canonical_basis :826, :862)
  if ((rc = real_gemm(n, n, n, Vn, view_t(Vn), w->rho, n, 1.0, 0.0, s))) return rc;
  if ((rc = real_gemm(n, n, n, Vn, view_t(Un), w->kap, n, 1.0, 0.0, s))) return rc;
  if ((rc = eigen_canonical(c, s))) return rc;
  const View Dn = view_cm(w->D, n, 0);
  // rhoc = D^T rho D, kappac = D^T kappa D
  if ((rc = real_gemm(n, n, n, view_t(Dn), view_cm(w->rho, n, 0), w->tmp, n, 1.0, 0.0, s))) return rc;
  if ((rc = real_gemm(n, n, n, view_cm(w->tmp, n, 0), Dn, w->rhoc, n, 1.0, 0.0, s))) return rc;
  if ((rc = real_gemm(n, n, n, view_t(Dn), view_cm(w->kap, n, 0), w->tmp, n, 1.0, 0.0, s))) return rc;
  if ((rc = real_gemm(n, n, n, view_cm(w->tmp, n, 0), Dn, w->kapc, n, 1.0, 0.0, s))) return rc;
  const double eps = (occeps < 2.2250738585072014e-308) ? 1.0e-8 : occeps;
  canon_kernel<<<1, 256, 0, tvap::counted(s)>>>(n, w->rhoc, w->kapc, w->D, w->schq, eps, int(allemp_d), w->canon_i,
                                                w->canon_d);
  TVAP_CUDA(cudaGetLastError());
  {
    // D_t^T D_t over the rows of isospin t, batch t = p, n
    GemmArgs g{};
    g.M = g.N = n;
    g.K = h;
    g.batch = 2;
    g.A = View{w->D, n, 1, h};
    g.B = View{w->D, 1, n, h};
    g.C = w->blocks + 8 * nn;
    g.crs = 1;
    g.ccs = n;
    g.cbs = (long long)nn;
    g.alpha = make_double2(1.0, 0.0);
    g.beta = make_double2(0.0, 0.0);
    g.a_real = g.b_real = g.c_real = true;
    if ((rc = gemm(g, s))) return rc;
  }
  sec_end_on(c, SEC_CANONICAL, s);
  TVAP_CUDA(cudaMemcpyAsync(host_canon, w->canon_i, sizeof(int) * 3, cudaMemcpyDeviceToHost, s));
  TVAP_CUDA(cudaStreamSynchronize(s));
  return TVAP_OK;
}

// Overlap chain of angles [0, G) on stream s2 (needs the canonical basis):
// R_n, Z = R22^{-1} R21 and det R22, the Schur complement S, K = A1^{-1} +
// S^T C0 S and its Pfaffian.
// blk: the angle-independent blocks (blocks 8, 9 of it: D_t^T D_t; the
// parity overlap passes blocks 10, 11 as 8, 9, D_t^T Pi D_t)
int angles_overlap(tvap_ctx* c, int G, const double2* d_ephase, int nocc, int nemp, cudaStream_t s2,
                   const double* blk = nullptr) {
  Workspace* w = c->ws;
  const int n = c->n;
  const int tb = 256;
  int rc;
  const int n2 = n - nemp, nb = n2 - nocc;
  sec_begin_on(c, SEC_OVERLAP, s2);
  build_rn_kernel<<<nblk(size_t(n2) * n2 * G, tb), tb, 0, tvap::counted(s2)>>>(n, n2, G, blk ? blk : w->blocks,
                                                                               d_ephase, w->Rn);
  const double2* S = w->Rn;
  int ldS = n2;
  long long bsS = (long long)n2 * n2;
  if (nocc > 0) {
    // Z = R22^{-1} R21 (nocc x nb), det(R22); S = R11 - R12 Z
    left_solve_kernel<<<G, kLsThreads, 0, tvap::counted(s2)>>>(nocc, nb, View{w->Rn + nb + size_t(nb) * n2, 1, n2, (long long)n2 * n2},
                                                View{w->Rn + nb, 1, n2, (long long)n2 * n2}, w->OW, w->OX, 1, nocc,
                                                (long long)nocc * nb, 0, w->detR22, G, c->d_flags, DEV_SINGULAR_RN);
    // (nb = 0: every state occupied or empty, a Slater determinant; no
    // Schur complement, only det R22)
    if (nb > 0)
      schur_kernel<<<nblk(size_t(nb) * nb * G, tb), tb, 0, tvap::counted(s2)>>>(n2, nb, G, w->Rn, w->OX, w->SZ);
    TVAP_CUDA(cudaGetLastError());
    S = w->SZ;
    ldS = nb;
    bsS = (long long)nb * nb;
  } else {
    fill_det_one_kernel<<<nblk(G, tb), tb, 0, tvap::counted(s2)>>>(G, w->detR22);
  }
  if (nb > 0) {
    overlap_prep_kernel<<<nblk(size_t(nb) * nb * G, tb), tb, 0, tvap::counted(s2)>>>(n, G, w->canon_i, w->canon_d, S, ldS, bsS,
                                                                      w->K, w->OY);
    TVAP_CUDA(cudaGetLastError());
    // K += S^T Y
    GemmArgs g{};
    g.M = g.N = g.K = nb;
    g.batch = G;
    g.A = View{S, (long long)ldS, 1, bsS};
    g.B = view_cm(w->OY, nb, (long long)nb * nb);
    g.C = w->K;
    g.crs = 1;
    g.ccs = nb;
    g.cbs = (long long)nb * nb;
    g.alpha = make_double2(1.0, 0.0);
    g.beta = make_double2(1.0, 0.0);
    g.three_m = true;
    g.upper_only = true;  // the Pfaffian reads the upper triangle only
    if ((rc = gemm(g, s2))) return rc;
    sec_end_on(c, SEC_OVERLAP, s2);
    sec_begin_on(c, SEC_PFAFFIAN, s2);
    if ((rc = pfaffian_batched(nb, G, w->K, w->pf, c->d_flags, s2, c->tune_pf_blocked != 0))) return rc;
    sec_end_on(c, SEC_PFAFFIAN, s2);
  } else {
    fill_det_one_kernel<<<nblk(G, tb), tb, 0, tvap::counted(s2)>>>(G, w->pf);
    sec_end_on(c, SEC_OVERLAP, s2);
  }
  TVAP_CUDA(cudaGetLastError());
  return TVAP_OK;
}

// Thouless chain of angles [0, G) on stream s (needs only U, V and their
// blocks): U_phi, V_phi, A_phi, U~, V~, the transition densities, the fields,
// the traces and H20.
int angles_thouless(tvap_ctx* c, int G, const double2* d_ephase, double factor_delta, cudaStream_t s) {
  Workspace* w = c->ws;
  const int n = c->n;
  const size_t nn = size_t(n) * n;
  const int tb = 256;
  int rc;
  sec_begin_on(c, SEC_SOLVE, s);
  build_uv_kernel<<<nblk(nn * G, tb), tb, 0, tvap::counted(s)>>>(n, G, w->blocks, d_ephase, w->Uphi, w->Vphi);
  TVAP_CUDA(cudaGetLastError());
  // A_phi = conj(V_phi U_phi^{-1}): solve U_phi^T Y = V_phi^T, A = conj(Y^T)
  if ((rc = blocked_thouless_solve(c, G, s))) return rc;
  sec_end_on(c, SEC_SOLVE, s);
  sec_begin_on(c, SEC_UV, s);
  // U~ = U + V A, V~ = V + U A
  broadcast_real_kernel<<<nblk(nn * G, tb), tb, 0, tvap::counted(s)>>>(nn, G, w->U, w->Ut);
  broadcast_real_kernel<<<nblk(nn * G, tb), tb, 0, tvap::counted(s)>>>(nn, G, w->V, w->Vt);
  {
    GemmArgs g{};
    g.M = g.N = g.K = n;
    g.batch = G;
    g.A = view_cm(w->V, n, 0);
    g.B = view_cm(w->A, n, (long long)nn);
    g.C = w->Ut;
    g.crs = 1;
    g.ccs = n;
    g.cbs = (long long)nn;
    g.alpha = make_double2(1.0, 0.0);
    g.beta = make_double2(1.0, 0.0);
    g.a_real = true;
    if ((rc = gemm(g, s))) return rc;
    g.A = view_cm(w->U, n, 0);
    g.C = w->Vt;
    g.reuse_left = true;  // A_phi, the per-angle operand of both products
    if ((rc = gemm(g, s))) return rc;
  }
  sec_end_on(c, SEC_UV, s);
  sec_begin_on(c, SEC_DENSITIES, s);
  // densities in angle-innermost layout: X[(i + j n) G + b]
  {
    GemmArgs g{};
    g.M = g.N = g.K = n;
    g.batch = G;
    g.crs = G;
    g.ccs = (long long)n * G;
    g.cbs = 1;
    g.alpha = make_double2(1.0, 0.0);
    g.beta = make_double2(0.0, 0.0);
    // rho = V~ V^T
    g.A = view_cm(w->Vt, n, (long long)nn);
    g.B = view_t(view_cm(w->V, n, 0));
    g.b_real = true;
    g.C = w->rhoL;
    if ((rc = gemm(g, s))) return rc;
    // kappaLR = V~ U^T (the digit planes of V~ from the product before)
    g.B = view_t(view_cm(w->U, n, 0));
    g.C = w->kLR;
    g.reuse_left = true;
    if ((rc = gemm(g, s))) return rc;
    g.reuse_left = false;
    // kappaRL = V U~^T
    g.A = view_cm(w->V, n, 0);
    g.a_real = true;
    g.b_real = false;
    g.B = view_t(view_cm(w->Ut, n, (long long)nn));
    g.C = w->kRL;
    if ((rc = gemm(g, s))) return rc;
  }
  sec_end_on(c, SEC_DENSITIES, s);
  if ((rc = fields_batched(c, G, G, w->rhoL, w->kLR, w->kRL, w->gam, w->hsp, w->dLR, w->dRL, s))) return rc;
  // the traces feed only the sums: on the second stream of the chain, beside
  // the H20 products, joined before the chain ends
  cudaStream_t st = c->streamM2 ? c->streamM2 : s;
  if (st != s) {
    TVAP_CUDA(cudaEventRecord(c->ev_stagger, s));
    TVAP_CUDA(cudaStreamWaitEvent(st, c->ev_stagger, 0));
  }
  sec_begin_on(c, SEC_TRACES, st);
  traces_partial_kernel<<<kTraceChunks, kTraceThreads, 0, tvap::counted(st)>>>(n, G, w->rhoL, w->kLR, w->kRL, w->gam, w->dLR,
                                                                c->d_H1, w->tpart);
  traces_finish_kernel<<<G, 9 * 32, 0, tvap::counted(st)>>>(G, w->tpart, c->H0, w->obs);
  TVAP_CUDA(cudaGetLastError());
  sec_end_on(c, SEC_TRACES, st);
  sec_begin_on(c, SEC_H20, s);
  // H20: T = U~^T (h V~ + fd/2 DeltaLR U~) - fd/2 V~^T DeltaRL V~, H20 = T - T^T,
  // as three products: X = [h | DeltaLR] [V~; fd/2 U~], Y = DeltaRL V~ and
  // T = [U~^T | V~^T] [X; -fd/2 Y] (the first and the last stacked along K)
  {
    TcTimingScope tc_timing(c, SEC_H20_TC);
    const View hv{w->hsp, (long long)G, (long long)n * G, 1};
    const View dl{w->dLR, (long long)G, (long long)n * G, 1};
    const View dr{w->dRL, (long long)G, (long long)n * G, 1};
    GemmArgs g{};
    g.M = g.N = g.K = n;
    g.batch = G;
    g.crs = 1;
    g.ccs = n;
    g.cbs = (long long)nn;
    g.three_m = true;
    g.alpha = make_double2(1.0, 0.0);
    g.beta = make_double2(0.0, 0.0);
    g.A = hv;
    g.B = view_cm(w->Vt, n, (long long)nn);
    g.K2 = n;
    g.A2 = dl;
    g.B2 = view_cm(w->Ut, n, (long long)nn);
    g.s2 = 0.5 * factor_delta;
    g.C = w->X;
    if ((rc = gemm(g, s))) return rc;
    g.K2 = 0;
    g.A = dr;
    g.B = view_cm(w->Vt, n, (long long)nn);
    g.C = w->Y;
    if ((rc = gemm(g, s))) return rc;
    g.A = view_t(view_cm(w->Ut, n, (long long)nn));
    g.B = view_cm(w->X, n, (long long)nn);
    g.K2 = n;
    g.A2 = view_t(view_cm(w->Vt, n, (long long)nn));
    g.B2 = view_cm(w->Y, n, (long long)nn);
    g.s2 = -0.5 * factor_delta;
    g.C = w->T;
    if ((rc = gemm(g, s))) return rc;
  }
  sec_end_on(c, SEC_H20, s);
  if (st != s) {
    TVAP_CUDA(cudaEventRecord(c->ev_join2, st));
    TVAP_CUDA(cudaStreamWaitEvent(s, c->ev_join2, 0));
  }
  return TVAP_OK;
}

// Contribution of angles [0, G) to the gauge sums (accumulate = 0 starts new
// sums), after both chains.
int angles_sums(tvap_ctx* c, int G, const double2* d_weight, const double* d_mult, bool have_overlap,
                int accumulate, cudaStream_t s) {
  Workspace* w = c->ws;
  const int n = c->n;
  const size_t nn = size_t(n) * n;
  const int tb = 256;
  sec_begin_on(c, SEC_SUMS, s);
  overlap_finish_kernel<<<nblk(G, tb), tb, 0, tvap::counted(s)>>>(n, G, have_overlap ? 1 : 0, w->canon_i, w->canon_d, w->pf,
                                                    w->detR22, d_weight, d_mult, w->obs, w->coefA, w->coefAE);
  sum_scalars_kernel<<<1, 32, 0, tvap::counted(s)>>>(G, w->obs, d_mult, d_weight, w->pscal, accumulate);
  sum_matrices_kernel<<<unsigned((nn + 31) / 32), 32 * kSumWarps, sizeof(double2) * 3 * size_t(G), tvap::counted(s)>>>(
      n, G, w->A, w->T, w->coefA, w->coefAE, d_mult, w->pA, w->pH, w->pAH, accumulate);
  TVAP_CUDA(cudaGetLastError());
  sec_end_on(c, SEC_SUMS, s);
  return TVAP_OK;
}

// Angles [0, G) with the canonical basis already known (nocc/nemp its host
// counts): overlap chain on the second stream, concurrent with the Thouless
// chain, then the sums.
int project_angles(tvap_ctx* c, int G, const double2* d_ephase, const double2* d_weight, const double* d_mult,
                   bool have_overlap, int nocc, int nemp, double factor_delta, int accumulate) {
  cudaStream_t s = c->stream, s2 = c->stream2;
  int rc;
  if (have_overlap) {
    TVAP_CUDA(cudaEventRecord(c->ev_fork, s));
    TVAP_CUDA(cudaStreamWaitEvent(s2, c->ev_fork, 0));
    if ((rc = angles_overlap(c, G, d_ephase, nocc, nemp, s2))) return rc;
    TVAP_CUDA(cudaEventRecord(c->ev_join, s2));
  }
  if ((rc = angles_thouless(c, G, d_ephase, factor_delta, s))) return rc;
  if (have_overlap) TVAP_CUDA(cudaStreamWaitEvent(s, c->ev_join, 0));
  return angles_sums(c, G, d_weight, d_mult, have_overlap, accumulate, s);
}

bool is_device_pointer(const void* p) {
  cudaPointerAttributes at{};
  cudaError_t e = cudaPointerGetAttributes(&at, p);
  if (e != cudaSuccess) cudaGetLastError();
  return e == cudaSuccess && (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged);
}

// Device memory of `device` itself, or managed memory (reachable from every
// device); memory of another GPU is refused.
bool is_device_pointer_on(const void* p, int device) {
  cudaPointerAttributes at{};
  cudaError_t e = cudaPointerGetAttributes(&at, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (at.type == cudaMemoryTypeManaged) return true;
  return at.type == cudaMemoryTypeDevice && at.device == device;
}

int upload_matrix(const void* src, void* dst, size_t bytes, cudaStream_t s) {
  cudaPointerAttributes at{};
  cudaError_t e = cudaPointerGetAttributes(&at, src);
  if (e != cudaSuccess) cudaGetLastError();
  const bool dev = (e == cudaSuccess && (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged));
  TVAP_CUDA(cudaMemcpyAsync(dst, src, bytes, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  return TVAP_OK;
}

int download_matrix(const void* src, void* dst, size_t bytes, cudaStream_t s) {
  cudaPointerAttributes at{};
  cudaError_t e = cudaPointerGetAttributes(&at, dst);
  if (e != cudaSuccess) cudaGetLastError();
  const bool dev = (e == cudaSuccess && (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged));
  TVAP_CUDA(cudaMemcpyAsync(dst, src, bytes, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
  return TVAP_OK;
}

// Waits for the context's stream once, reading the status word and (when
// bytes > 0) bytes of device data at src into dst through the pinned buffer;
// then resets the status word and maps it to a code.
int sync_with_flags(tvap_ctx* c, void* dst, const void* src, size_t bytes) {
  if (bytes > kPinnedBytes - 16) return TVAP_ERR_ARG;
  unsigned char* pin = static_cast<unsigned char*>(c->h_pin);
  if (bytes) TVAP_CUDA(cudaMemcpyAsync(pin + 16, src, bytes, cudaMemcpyDeviceToHost, c->stream));
  TVAP_CUDA(cudaMemcpyAsync(pin, c->d_flags, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  TVAP_CUDA(cudaStreamSynchronize(c->stream));
  TVAP_CUDA(cudaMemsetAsync(c->d_flags, 0, sizeof(int), c->stream));
  int f = 0;
  std::memcpy(&f, pin, sizeof(int));
  if (bytes) std::memcpy(dst, pin + 16, bytes);
  if (f & DEV_SINGULAR_RN) return TVAP_ERR_SINGULAR_RN;
  if (f & DEV_SINGULAR_UPHI) return TVAP_ERR_SINGULAR_UPHI;
  if (f & (DEV_EIGEN_NOCONV | DEV_CANON_BLOCK)) return TVAP_ERR_CANONICAL;
  if (f & DEV_CHOLESKY) return TVAP_ERR_CHOLESKY;
  if (f & DEV_TRTRI) return TVAP_ERR_TRTRI;
  if (f & DEV_IMAG_GRAD) return TVAP_ERR_IMAG_GRADIENT;
  if (f & DEV_WAIT_TIMEOUT) {
    set_last_error("a device kernel ran out of its bounded wait", __FILE__, __LINE__);
    return TVAP_ERR_DEVICE_TIMEOUT;
  }
  return TVAP_OK;
}

int check_flags(tvap_ctx* c) { return sync_with_flags(c, nullptr, nullptr, 0); }

// Full projection of state (w->U, w->V) already on the device.  Leaves the
// sums in w->pscal/pA/pH/pAH and the gradient in w->H20v.
int project_device(tvap_ctx* c, const tvap_proj_opts& o, tvap_pnp* out, bool sync) {
  const int n = c->n;
  const size_t nn = size_t(n) * n;
  cudaStream_t s = c->stream, s2 = c->stream2;
  int canon[3] = {0, 0, 0};
  int rc;
  const bool have_overlap = std::max(o.Mphip, o.Mphin) > 1;
  const bool fold = (o.mode == 0) && std::fabs(o.facpi - 2.0 * M_PI) < 1e-12 && is_integer(o.valence_Z) &&
                    is_integer(o.valence_N);
  const AngleTable& t = make_angles(o, fold);
  const int G = int(t.php.size());
  Workspace* w = c->ws;
  std::vector<double2> eph(2 * G), wt(G);
  for (int b = 0; b < G; ++b) {
    const std::complex<double> I(0.0, 1.0);
    const std::complex<double> ep = std::exp(I * t.php[b]), en = std::exp(I * t.phn[b]);
    eph[2 * b] = make_double2(ep.real(), ep.imag());
    eph[2 * b + 1] = make_double2(en.real(), en.imag());
    wt[b] = make_double2(t.w[b].real(), t.w[b].imag());
  }
  // the tables stay on the device while the options do not change (three
  // copies from pageable memory less per projection)
  if (!(w->angles_valid && w->ang_Mp == o.Mphip && w->ang_Mn == o.Mphin && w->ang_mode == o.mode &&
        w->ang_facpi == o.facpi && w->ang_vz == o.valence_Z && w->ang_vn == o.valence_N)) {
    TVAP_CUDA(cudaMemcpyAsync(w->ephase, eph.data(), sizeof(double2) * 2 * G, cudaMemcpyHostToDevice, s));
    TVAP_CUDA(cudaMemcpyAsync(w->weight, wt.data(), sizeof(double2) * G, cudaMemcpyHostToDevice, s));
    TVAP_CUDA(cudaMemcpyAsync(w->mult, t.mult.data(), sizeof(double) * G, cudaMemcpyHostToDevice, s));
    w->angles_valid = true;
    w->ang_Mp = o.Mphip;
    w->ang_Mn = o.Mphin;
    w->ang_mode = o.mode;
    w->ang_facpi = o.facpi;
    w->ang_vz = o.valence_Z;
    w->ang_vn = o.valence_N;
  }
  auto canon_error = [&]() {
    set_last_error("canonical basis: a degenerate subspace larger than 64 or not reducible to 2 x 2 blocks, an "
                   "odd number of paired states, or a zero v/u",
                   __FILE__, __LINE__);
    return TVAP_ERR_CANONICAL;
  };
  if (o.mode == 0) {
    // The Thouless chain needs only U and V: it is queued first, on streamM
    // (priority between those of the second and third streams); the
    // canonical basis (with its host-side checks) follows on the second
    // stream and the overlap chain on the third, concurrently; the sums join
    // all three on the caller's stream.
    cudaStream_t sm = c->streamM;
    sec_mark(c, s);
    TVAP_CUDA(cudaEventRecord(c->ev_fork, s));
    TVAP_CUDA(cudaStreamWaitEvent(s2, c->ev_fork, 0));
    TVAP_CUDA(cudaStreamWaitEvent(sm, c->ev_fork, 0));
    if ((rc = prepare_uv_blocks(c, sm))) return rc;
    if ((rc = angles_thouless(c, G, w->ephase, o.factor_delta, sm))) return rc;
    TVAP_CUDA(cudaEventRecord(c->ev_main, sm));
    if ((rc = prepare_canonical(c, o.seed_occeps, o.seed_allemp, canon, s2))) return rc;
    if (canon[2] && have_overlap) return canon_error();
    // the overlap chain (wide kernels) at the lowest priority
    cudaStream_t s3 = c->stream3;
    TVAP_CUDA(cudaEventRecord(c->ev_canon, s2));
    TVAP_CUDA(cudaStreamWaitEvent(s3, c->ev_canon, 0));
    if (have_overlap && (rc = angles_overlap(c, G, w->ephase, canon[0], canon[1], s3))) return rc;
    TVAP_CUDA(cudaEventRecord(c->ev_join, s3));
    TVAP_CUDA(cudaStreamWaitEvent(s, c->ev_join, 0));
    TVAP_CUDA(cudaStreamWaitEvent(s, c->ev_main, 0));
    if ((rc = angles_sums(c, G, w->weight, w->mult, have_overlap, 0, s))) return rc;
  } else {
    // plain form: one angle per launch sequence
    sec_mark(c, s);
    if ((rc = prepare_uv_blocks(c, s))) return rc;
    if ((rc = prepare_canonical(c, o.seed_occeps, o.seed_allemp, canon, s))) return rc;
    if (canon[2] && have_overlap) return canon_error();
    for (int b = 0; b < G; ++b)
      if ((rc = project_angles(c, 1, w->ephase + 2 * b, w->weight + b, w->mult + b, have_overlap, canon[0],
                               canon[1], o.factor_delta, b > 0 ? 1 : 0)))
        return rc;
  }
  projected_h20_kernel<<<nblk(nn, 256), 256, 0, tvap::counted(s)>>>(n, w->pA, w->pH, w->pAH, w->pscal, w->H20v, c->d_flags);
  TVAP_CUDA(cudaGetLastError());
  if (!sync) {
    // the caller reads the sums (w->pscal) and the status word later, in
    // its own round trip
    if (out) {
      out->nocc = canon[0];
      out->nemp = canon[1];
    }
    return TVAP_OK;
  }
  if (out) {
    // the sums and the status word in one round trip
    double2 sc[6];
    rc = sync_with_flags(c, sc, w->pscal, sizeof(double2) * 6);
    double* dst[6] = {out->over, out->ener, out->prot, out->neut, out->prot2, out->neut2};
    for (int q = 0; q < 6; ++q) {
      dst[q][0] = sc[q].x;
      dst[q][1] = sc[q].y;
    }
    out->nocc = canon[0];
    out->nemp = canon[1];
    return rc;
  }
  return check_flags(c);
}

// ---------------------------------------------------------------------------
// Observables of the projected state: project_wavefunction with iopt = 1
// (module_projection.f90:201-373, the branch :279-354) and sum_gauge with
// iopt = 1 (:425-458).  Per angle: traces of one-body operators with rho^LR
// over the proton and the neutron rows (calculate_expectval_obo_cplx,
// module_operators.f90:146-164), the isospin blocks of the energy
// decomposition (calculate_decompo_energy, module_hamiltonian.f90:1134-1260),
// <O^2> (calculate_expectval_obos_cplx, module_operators.f90:227-257), the
// shell occupations (module_particlenumber.f90:157-176), the overlap with the
// parity-rotated state (generate_rotation_parity, :607-625), and rho^LR;
// summed with weight x overlap (the parity overlap with the weight alone).
// All angles are computed (no conjugate folding: an operator need not be
// real).  FP64 throughout except the <O^2> products (the context's GEMM
// arithmetic).
// ---------------------------------------------------------------------------
namespace {

constexpr int kObsRows = 8;       // rows per CTA of the trace kernels
constexpr int kObsThreads = 128;  // threads over the angles

// part[((ch * nops + k) * 2 + t) * G + b] = sum over the rows i of chunk ch
// of isospin t of (B_k rho_b)(i, i) = sum_j B_k(i, j) rho_b(j, i)
__global__ void __launch_bounds__(kObsThreads)
    obs_trace_kernel(int n, int G, const double2* __restrict__ ops, const double2* __restrict__ rho,
                     double2* __restrict__ part) {
  const int k = blockIdx.x, nops = gridDim.x, ch = blockIdx.y, h = n / 2;
  const double2* B = ops + size_t(k) * n * n;
  const int b = blockIdx.z * blockDim.x + threadIdx.x;
  if (b >= G) return;
  double2 sp = make_double2(0.0, 0.0), sn = make_double2(0.0, 0.0);
  for (int r = 0; r < kObsRows; ++r) {
    const int i = ch * kObsRows + r;
    if (i >= n) break;
    double2 acc = make_double2(0.0, 0.0);
    for (int j = 0; j < n; ++j) cfma(acc, B[i + size_t(j) * n], rho[(size_t(j) + size_t(i) * n) * G + b]);
    if (i < h)
      sp = cadd(sp, acc);
    else
      sn = cadd(sn, acc);
  }
  part[((size_t(ch) * nops + k) * 2 + 0) * G + b] = sp;
  part[((size_t(ch) * nops + k) * 2 + 1) * G + b] = sn;
}

// part[(ch * 10 + q) * G + b] for the rows i of chunk ch: q = 0..3 PH pp, pn,
// np, nn = 0.5 sum gamma(i, j) rho(j, i); q = 4..7 PP = 0.5 sum delta(i, j)
// kappaRL(i, j) (i, j in the blocks' isospins); q = 8, 9 the <O^2> terms
// sum_j X(i, j) X(j, i) and sum_j Y1(i, j) Y2(i, j) when X is given
__global__ void __launch_bounds__(kObsThreads)
    obs_blocks_kernel(int n, int G, const double2* __restrict__ rho, const double2* __restrict__ kRL,
                      const double2* __restrict__ gam, const double2* __restrict__ dLR,
                      const double2* __restrict__ X, const double2* __restrict__ Y1, const double2* __restrict__ Y2,
                      double2* __restrict__ part) {
  const int ch = blockIdx.x, h = n / 2;
  const int b = blockIdx.y * blockDim.x + threadIdx.x;
  if (b >= G) return;
  auto at = [G, n, b](const double2* A, int i, int j) { return A[(size_t(i) + size_t(j) * n) * G + b]; };
  double2 a[10];
#pragma unroll
  for (int q = 0; q < 10; ++q) a[q] = make_double2(0.0, 0.0);
  for (int r = 0; r < kObsRows; ++r) {
    const int i = ch * kObsRows + r;
    if (i >= n) break;
    const int ti = i >= h ? 2 : 0;
    for (int j = 0; j < n; ++j) {
      const int q = ti + (j >= h ? 1 : 0);
      if (gam) {
        cfma(a[q], at(gam, i, j), at(rho, j, i));
        cfma(a[4 + q], at(dLR, i, j), at(kRL, i, j));
      }
      if (X) {
        cfma(a[8], at(X, i, j), at(X, j, i));
        cfma(a[9], at(Y1, i, j), at(Y2, i, j));
      }
    }
  }
#pragma unroll
  for (int q = 0; q < 10; ++q) part[(size_t(ch) * 10 + q) * G + b] = (q < 8) ? cscale(a[q], 0.5) : a[q];
}

// Q[q * G + b] = sum over the chunks of part[(ch * nq + q) * G + b], in order
__global__ void obs_chunks_kernel(int G, int nq, int nch, const double2* __restrict__ part, double2* __restrict__ Q) {
  const size_t idx = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (idx >= size_t(nq) * G) return;
  const int q = int(idx / G), b = int(idx % G);
  double2 s = make_double2(0.0, 0.0);
  for (int ch = 0; ch < nch; ++ch) s = cadd(s, part[(size_t(ch) * nq + q) * G + b]);
  Q[idx] = s;
}

// the occupation numbers of the shells, Q[(s * 2 + t) * G + b] (shell s holds
// the states off[s] .. off[s+1]-1 of each isospin)
__global__ void obs_occ_kernel(int n, int G, int nshell, const int* __restrict__ off, const double2* __restrict__ rho,
                               double2* __restrict__ Q) {
  const size_t idx = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (idx >= size_t(nshell) * G) return;
  const int sh = int(idx / G), b = int(idx % G), h = n / 2;
  double2 sp = make_double2(0.0, 0.0), sn = make_double2(0.0, 0.0);
  for (int k = off[sh]; k < off[sh + 1]; ++k) {
    sp = cadd(sp, rho[(size_t(k) + size_t(k) * n) * G + b]);
    sn = cadd(sn, rho[(size_t(k + h) + size_t(k + h) * n) * G + b]);
  }
  Q[(size_t(sh) * 2 + 0) * G + b] = sp;
  Q[(size_t(sh) * 2 + 1) * G + b] = sn;
}

// <O^2> per angle: tr1^2 + tr2 - tr5 + tr6 (tr1, tr2 = the traces of O and
// O^2 with rho over both isospins; tr5, tr6 from obs_blocks_kernel)
__global__ void obs_sq_kernel(int G, const double2* __restrict__ t1p, const double2* __restrict__ t2p,
                              const double2* __restrict__ t56, double2* __restrict__ out) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= G) return;
  const double2 t1 = cadd(t1p[b], t1p[G + b]), t2 = cadd(t2p[b], t2p[G + b]);
  double2 v = cmul(t1, t1);
  v = cadd(v, t2);
  v = cadd(v, cneg(t56[b]));
  out[b] = cadd(v, t56[G + b]);
}

// out[q] = sum_b f[b] Q[q * G + b], one warp per q, a fixed-order reduction
__global__ void obs_sum_kernel(int G, int nq, const double2* __restrict__ Q, const double2* __restrict__ f,
                               double2* __restrict__ out) {
  const int q = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (q >= nq) return;
  double2 s = make_double2(0.0, 0.0);
  for (int b = lane; b < G; b += 32) cfma(s, f[b], Q[size_t(q) * G + b]);
  for (int o = 16; o > 0; o >>= 1) {
    s.x += __shfl_down_sync(0xffffffffu, s.x, o);
    s.y += __shfl_down_sync(0xffffffffu, s.y, o);
  }
  if (lane == 0) out[q] = s;
}

// sum_b weight[b] ov[8 b], one warp, a fixed-order reduction
__global__ void obs_pari_kernel(int G, const double2* __restrict__ ov, const double2* __restrict__ weight,
                                double2* __restrict__ out) {
  const int lane = threadIdx.x;
  double2 s = make_double2(0.0, 0.0);
  for (int b = lane; b < G; b += 32) cfma(s, weight[b], ov[8 * size_t(b)]);
  for (int o = 16; o > 0; o >>= 1) {
    s.x += __shfl_down_sync(0xffffffffu, s.x, o);
    s.y += __shfl_down_sync(0xffffffffu, s.y, o);
  }
  if (lane == 0) *out = s;
}

// pnp_rho: R(i, j) = sum_b f[b] rho_b(i, j)
__global__ void obs_rho_kernel(int n, int G, const double2* __restrict__ rho, const double2* __restrict__ f,
                               double2* __restrict__ R) {
  const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (e >= size_t(n) * n) return;
  double2 s = make_double2(0.0, 0.0);
  for (int b = 0; b < G; ++b) cfma(s, f[b], rho[e * G + b]);
  R[e] = s;
}

// D with its rows scaled by the parities
__global__ void scale_rows_kernel(int n, const int* __restrict__ par, const double* __restrict__ D,
                                  double* __restrict__ PD) {
  const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (e >= size_t(n) * n) return;
  PD[e] = double(par[e % n]) * D[e];
}

}  // namespace

// scal: over, ener, prot, neut, prot2, neut2, pari, ecomp[12]; obo_out
// (nobo x (p, n)), sq_out (nsq), occ_out (nshell x (p, n)): host arrays;
// rho_out (n x n complex): host or device, may be null.  obo, sq: host or
// device; parity (may be null), shell_size: host.
int project_observables_device(tvap_ctx* c, const tvap_proj_opts& o, int nobo, const double* obo, int nsq,
                               const double* sq, const int* parity, int nshell, const int* shell_size,
                               double2* scal, double2* obo_out, double2* sq_out, double2* occ_out, double* rho_out,
                               int* nocc_nemp) {
  const int n = c->n, h = n / 2;
  const size_t nn = size_t(n) * n;
  cudaStream_t s = c->stream;
  Workspace* w = c->ws;
  const bool have_overlap = std::max(o.Mphip, o.Mphin) > 1;
  const AngleTable& t = make_angles(o, false);
  const int G = int(t.php.size());
  if (!w || w->G < G) return TVAP_ERR_ARG;
  int rc;
  {
    std::vector<double2> eph(2 * G), wt(G);
    for (int b = 0; b < G; ++b) {
      const std::complex<double> I(0.0, 1.0);
      const std::complex<double> ep = std::exp(I * t.php[b]), en = std::exp(I * t.phn[b]);
      eph[2 * b] = make_double2(ep.real(), ep.imag());
      eph[2 * b + 1] = make_double2(en.real(), en.imag());
      wt[b] = make_double2(t.w[b].real(), t.w[b].imag());
    }
    TVAP_CUDA(cudaMemcpyAsync(w->ephase, eph.data(), sizeof(double2) * 2 * G, cudaMemcpyHostToDevice, s));
    TVAP_CUDA(cudaMemcpyAsync(w->weight, wt.data(), sizeof(double2) * G, cudaMemcpyHostToDevice, s));
    TVAP_CUDA(cudaMemcpyAsync(w->mult, t.mult.data(), sizeof(double) * G, cudaMemcpyHostToDevice, s));
    TVAP_CUDA(cudaStreamSynchronize(s));  // the host tables go out of scope
    w->angles_valid = false;              // the next projection uploads its own
  }
  // the trace operators: obo, H1, then O_k and O2_k of the pairs
  const int ntr = nobo + 1 + 2 * nsq;
  const int nch = (n + kObsRows - 1) / kObsRows;
  // Q: 8 energy blocks, 2 per trace operator, nsq <O^2>, 2 per shell
  const int nq = 8 + 2 * ntr + nsq + 2 * nshell;
  const size_t part_elems = size_t(nch) * std::max(2 * ntr, 10) * G;
  double2 *ops = nullptr, *part = nullptr, *Q = nullptr, *sums = nullptr, *obs2 = nullptr, *rsum = nullptr;
  int *dpar = nullptr, *doff = nullptr;
  const size_t obs2_elems = 10 * size_t(G);
  TVAP_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&ops), sizeof(double2) * nn * ntr, s));
  TVAP_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&part), sizeof(double2) * part_elems, s));
  TVAP_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&Q), sizeof(double2) * size_t(nq) * G, s));
  TVAP_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&sums), sizeof(double2) * (nq + 1), s));
  TVAP_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&obs2), sizeof(double2) * obs2_elems, s));
  TVAP_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&rsum), sizeof(double2) * nn, s));
  TVAP_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&dpar), sizeof(int) * n, s));
  TVAP_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&doff), sizeof(int) * (nshell + 1), s));
  auto release = [&]() {
    void* bufs[] = {ops, part, Q, sums, obs2, rsum, dpar, doff};
    for (void* p : bufs)
      if (p) cudaFreeAsync(p, s);
  };
  auto run = [&]() -> int {
    int r;
    for (int k = 0; k < nobo; ++k)
      if ((r = upload_matrix(obo + 2 * nn * k, ops + nn * k, sizeof(double2) * nn, s))) return r;
    TVAP_CUDA(cudaMemcpyAsync(ops + nn * nobo, c->d_H1, sizeof(double2) * nn, cudaMemcpyDeviceToDevice, s));
    for (int k = 0; k < 2 * nsq; ++k)
      if ((r = upload_matrix(sq + 2 * nn * k, ops + nn * (nobo + 1 + k), sizeof(double2) * nn, s))) return r;
    std::vector<int> off(nshell + 1, 0);
    for (int k = 0; k < nshell; ++k) off[k + 1] = off[k] + shell_size[k];
    if (off[nshell] > h) return TVAP_ERR_ARG;
    TVAP_CUDA(cudaMemcpyAsync(doff, off.data(), sizeof(int) * (nshell + 1), cudaMemcpyHostToDevice, s));
    if (parity) TVAP_CUDA(cudaMemcpyAsync(dpar, parity, sizeof(int) * n, cudaMemcpyHostToDevice, s));
    TVAP_CUDA(cudaStreamSynchronize(s));  // the host vectors go out of scope
    // the projection itself (densities, fields, overlaps, traces, sums) on
    // one stream, then the parity-rotated overlaps
    int canon[3] = {0, 0, 0};
    sec_mark(c, s);
    if ((r = prepare_uv_blocks(c, s))) return r;
    if ((r = prepare_canonical(c, o.seed_occeps, o.seed_allemp, canon, s))) return r;
    if (canon[2]) {
      set_last_error("canonical basis: a degenerate subspace larger than 64 or not reducible to 2 x 2 blocks",
                     __FILE__, __LINE__);
      return TVAP_ERR_CANONICAL;
    }
    if ((r = angles_thouless(c, G, w->ephase, o.factor_delta, s))) return r;
    if (have_overlap && (r = angles_overlap(c, G, w->ephase, canon[0], canon[1], s))) return r;
    if ((r = angles_sums(c, G, w->weight, w->mult, have_overlap, 0, s))) return r;
    nocc_nemp[0] = canon[0];
    nocc_nemp[1] = canon[1];
    const int tb = 256;
    // Q: the energy blocks (and, per pair, the <O^2> terms)
    const dim3 gblk(nch, (G + kObsThreads - 1) / kObsThreads);
    obs_blocks_kernel<<<gblk, kObsThreads, 0, tvap::counted(s)>>>(n, G, w->rhoL, w->kRL, w->gam, w->dLR, nullptr,
                                                                   nullptr, nullptr, part);
    obs_chunks_kernel<<<nblk(size_t(10) * G, tb), tb, 0, tvap::counted(s)>>>(G, 10, nch, part, obs2);
    TVAP_CUDA(cudaMemcpyAsync(Q, obs2, sizeof(double2) * 8 * G, cudaMemcpyDeviceToDevice, s));
    // the traces of the operators
    const dim3 gtr(ntr, nch, (G + kObsThreads - 1) / kObsThreads);
    obs_trace_kernel<<<gtr, kObsThreads, 0, tvap::counted(s)>>>(n, G, ops, w->rhoL, part);
    obs_chunks_kernel<<<nblk(size_t(2 * ntr) * G, tb), tb, 0, tvap::counted(s)>>>(G, 2 * ntr, nch, part,
                                                                                   Q + size_t(8) * G);
    TVAP_CUDA(cudaGetLastError());
    // <O^2>: X = O rho, Y1 = kappaRL O, Y2 = O kappaLR per angle (angle-innermost)
    for (int k = 0; k < nsq; ++k) {
      const double2* Op = ops + nn * (nobo + 1 + 2 * k);
      const View Ov{Op, 1, n, 0};
      const View rhoV{w->rhoL, (long long)G, (long long)n * G, 1};
      GemmArgs g{};
      g.M = g.N = g.K = n;
      g.batch = G;
      g.crs = G;
      g.ccs = (long long)n * G;
      g.cbs = 1;
      g.alpha = make_double2(1.0, 0.0);
      g.beta = make_double2(0.0, 0.0);
      g.A = Ov;
      g.B = rhoV;
      g.C = w->X;
      if ((r = gemm(g, s))) return r;
      g.A = View{w->kRL, (long long)G, (long long)n * G, 1};
      g.B = Ov;
      g.C = w->Y;
      if ((r = gemm(g, s))) return r;
      g.A = Ov;
      g.B = View{w->kLR, (long long)G, (long long)n * G, 1};
      g.C = w->T;
      if ((r = gemm(g, s))) return r;
      obs_blocks_kernel<<<gblk, kObsThreads, 0, tvap::counted(s)>>>(n, G, w->rhoL, w->kRL, nullptr, nullptr, w->X,
                                                                     w->Y, w->T, part);
      obs_chunks_kernel<<<nblk(size_t(10) * G, tb), tb, 0, tvap::counted(s)>>>(G, 10, nch, part, obs2);
      const double2* tr = Q + size_t(8) * G;
      obs_sq_kernel<<<nblk(G, tb), tb, 0, tvap::counted(s)>>>(G, tr + size_t(2 * (nobo + 1 + 2 * k)) * G,
                                                              tr + size_t(2 * (nobo + 2 + 2 * k)) * G,
                                                              obs2 + size_t(8) * G,
                                                              Q + size_t(8 + 2 * ntr + k) * G);
      TVAP_CUDA(cudaGetLastError());
    }
    if (nshell > 0)
      obs_occ_kernel<<<nblk(size_t(nshell) * G, tb), tb, 0, tvap::counted(s)>>>(
          n, G, nshell, doff, w->rhoL, Q + size_t(8 + 2 * ntr + nsq) * G);
    // sums with weight x overlap (coefA of angles_sums), and pnp_rho
    obs_sum_kernel<<<(nq + 3) / 4, 128, 0, tvap::counted(s)>>>(G, nq, Q, w->coefA, sums);
    obs_rho_kernel<<<nblk(nn, tb), tb, 0, tvap::counted(s)>>>(n, G, w->rhoL, w->coefA, rsum);
    TVAP_CUDA(cudaGetLastError());
    // the overlaps with the parity-rotated state: R_n from the blocks
    // D_t^T Pi D_t (10, 11), then the overlap chain once more
    double2 pari = make_double2(0.0, 0.0);
    if (parity) {
      scale_rows_kernel<<<nblk(nn, tb), tb, 0, tvap::counted(s)>>>(n, dpar, w->D, w->tmp);
      GemmArgs g{};
      g.M = g.N = n;
      g.K = h;
      g.batch = 2;
      g.A = View{w->D, n, 1, h};
      g.B = View{w->tmp, 1, n, h};
      g.C = w->blocks + 10 * nn;
      g.crs = 1;
      g.ccs = n;
      g.cbs = (long long)nn;
      g.alpha = make_double2(1.0, 0.0);
      g.beta = make_double2(0.0, 0.0);
      g.a_real = g.b_real = g.c_real = true;
      if ((r = gemm(g, s))) return r;
      if ((r = angles_overlap(c, G, w->ephase, canon[0], canon[1], s, w->blocks + 2 * nn))) return r;
      // the overlap formula into obs2 (8 G), its coefficients into scratch
      double2* o2 = obs2;
      TVAP_CUDA(cudaMemsetAsync(o2, 0, sizeof(double2) * 8 * G, s));
      overlap_finish_kernel<<<nblk(G, tb), tb, 0, tvap::counted(s)>>>(n, G, 1, w->canon_i, w->canon_d, w->pf,
                                                                     w->detR22, w->weight, w->mult, o2, part,
                                                                     part + G);
      // sum_b weight_b rot_pari_b (the overlaps sit at stride 8 in o2)
      obs_pari_kernel<<<1, 32, 0, tvap::counted(s)>>>(G, o2, w->weight, sums + nq);
      TVAP_CUDA(cudaGetLastError());
    }
    // results
    std::vector<double2> hs(nq + 1);
    TVAP_CUDA(cudaMemcpyAsync(hs.data(), sums, sizeof(double2) * (nq + 1), cudaMemcpyDeviceToHost, s));
    double2 sc6[6];
    TVAP_CUDA(cudaMemcpyAsync(sc6, w->pscal, sizeof(double2) * 6, cudaMemcpyDeviceToHost, s));
    if (rho_out && (r = download_matrix(rsum, rho_out, sizeof(double2) * nn, s))) return r;
    if ((r = check_flags(c))) return r;  // synchronises the stream
    if (parity) pari = hs[nq];
    for (int q = 0; q < 6; ++q) scal[q] = sc6[q];
    scal[6] = pari;
    const double2* tr = hs.data() + 8;
    const double2 e1p = tr[2 * nobo], e1n = tr[2 * nobo + 1];
    scal[7] = e1p;
    scal[8] = e1n;
    for (int q = 0; q < 8; ++q) scal[9 + q] = hs[q];
    // energy_p = 1b_p + PH_pp + PH_pn + PP_pp + PP_pn (and n)
    scal[17] = cadd(cadd(e1p, cadd(hs[0], hs[1])), cadd(hs[4], hs[5]));
    scal[18] = cadd(cadd(e1n, cadd(hs[2], hs[3])), cadd(hs[6], hs[7]));
    for (int k = 0; k < nobo; ++k) {
      obo_out[2 * k] = tr[2 * k];
      obo_out[2 * k + 1] = tr[2 * k + 1];
    }
    for (int k = 0; k < nsq; ++k) sq_out[k] = hs[8 + 2 * ntr + k];
    for (int k = 0; k < 2 * nshell; ++k) occ_out[k] = hs[8 + 2 * ntr + nsq + k];
    return TVAP_OK;
  };
  rc = run();
  release();
  if (rc == TVAP_OK) TVAP_CUDA(cudaStreamSynchronize(s));
  return rc;
}

int observables_angle_count(const tvap_proj_opts& o) { return int(make_angles(o, false).php.size()); }

int ensure_workspace(tvap_ctx* c, int G) { return ws_ensure(c, G); }
double* ws_U(tvap_ctx* c) { return c->ws->U; }
double* ws_V(tvap_ctx* c) { return c->ws->V; }
double* ws_H20v(tvap_ctx* c) { return c->ws->H20v; }
// one real product C = alpha op(A) op(B) + beta C in the calling thread's
// arithmetic (for the other translation units)
int real_product(int M, int N, int K, View A, View B, double* C, int ldc, double alpha, double beta,
                 cudaStream_t s) {
  return real_gemm(M, N, K, A, B, C, ldc, alpha, beta, s);
}
// the six projected sums (over, ener, prot, neut, prot2, neut2), then two
// free complex slots
double2* ws_sums(tvap_ctx* c) { return c->ws->pscal; }
int angle_count(const tvap_proj_opts& o) {
  const bool fold = (o.mode == 0) && std::fabs(o.facpi - 2.0 * M_PI) < 1e-12 && is_integer(o.valence_Z) &&
                    is_integer(o.valence_N);
  return int(make_angles(o, fold).php.size());
}
void destroy_workspace(tvap_ctx* c) {
  if (c->ws) {
    ws_free(c->ws);
    delete c->ws;
    c->ws = nullptr;
  }
}

}  // namespace tvap
