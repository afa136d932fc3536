// Host-side model-space setup for the PNVAP hot path.
//
// What lives here is the one-time preparation that the Fortran reference does
// before its gradient loop, restated in C++ so that harnesses and benchmarks
// can build the inputs of the device path without the Fortran program:
//
//   * the spherical HO single-particle basis (protons first, then neutrons;
//     inside a shell 2m runs from +2j down to -2j; HOsp_tr(k) = k + 2m_k),
//     module_basis.f90:73-245;
//   * the two-body interaction in JT-coupled form, read from an ANTOINE file
//     (module_hamiltonian.f90:120-190, 412-459) or drawn from a seeded normal
//     distribution, its 7-fold symmetry reconstruction (:282-319), the
//     m-scheme enumeration with the 1e-16 cutoff (:321-378), the JT
//     uncoupling (:828-885) and the time-reversal permutation codes
//     (:970-1018);
//   * the .red reduced-Hamiltonian stream file (:533-627);
//   * the multipole operators Q_lm (module_multipoles.f90:43-128) used by
//     the quadrupole constraints.
//
// Everything is exported with a plain C ABI (see include/tvap_setup.h).

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <random>
#include <sstream>
#include <string>
#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include "../../../include/tvap_setup.h"

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kHbarc = 197.3269788;
constexpr double kMassMa = (938.27208816 + 939.56542052) / 2.0;
constexpr double kRadiusR0 = 1.2;

// ---------------------------------------------------------------------------
// Clebsch-Gordan coefficient <j1 m1 j2 m2 | j3 m3>; every argument is twice
// the physical value.  Racah's closed form, evaluated with log-factorials.
// Same quantity as ClebschGordan (module_mathmethods.f90:281-342).
// ---------------------------------------------------------------------------
double lfact(int n) { return std::lgamma(double(n) + 1.0); }

double clebsch(int j1, int j2, int j3, int m1, int m2, int m3) {
  if (m1 + m2 != m3) return 0.0;
  if (((j1 + m1) & 1) || ((j2 + m2) & 1) || ((j3 + m3) & 1)) return 0.0;
  if (std::abs(m1) > j1 || std::abs(m2) > j2 || std::abs(m3) > j3) return 0.0;
  if ((j1 + j2 + j3) & 1) return 0.0;
  const int a = (j1 + j2 - j3) / 2, b = (j1 - j2 + j3) / 2, c = (-j1 + j2 + j3) / 2;
  if (a < 0 || b < 0 || c < 0) return 0.0;
  const int J = (j1 + j2 + j3) / 2;
  const int p1 = (j1 + m1) / 2, q1 = (j1 - m1) / 2;
  const int p2 = (j2 + m2) / 2, q2 = (j2 - m2) / 2;
  const int p3 = (j3 + m3) / 2, q3 = (j3 - m3) / 2;
  const double lpre = 0.5 * (lfact(a) + lfact(b) + lfact(c) - lfact(J + 1) + lfact(p1) + lfact(q1) +
                             lfact(p2) + lfact(q2) + lfact(p3) + lfact(q3));
  // summation index k: all factorial arguments non-negative
  const int t1 = (j3 - j2 + m1) / 2;  // (j3 - j2 + m1)
  const int t2 = (j3 - j1 - m2) / 2;  // (j3 - j1 - m2)
  int kmin = 0;
  if (-t1 > kmin) kmin = -t1;
  if (-t2 > kmin) kmin = -t2;
  int kmax = a;
  if (q1 < kmax) kmax = q1;
  if (p2 < kmax) kmax = p2;
  double sum = 0.0;
  for (int k = kmin; k <= kmax; ++k) {
    const double l = lfact(k) + lfact(a - k) + lfact(q1 - k) + lfact(p2 - k) + lfact(t1 + k) + lfact(t2 + k);
    const double term = std::exp(lpre - l);
    sum += (k & 1) ? -term : term;
  }
  return std::sqrt(double(j3) + 1.0) * sum;
}

// Cache of CG values keyed by the doubled arguments (j's <= 31, |m| <= 31).
struct CgCache {
  std::vector<double> val;
  std::vector<uint8_t> have;
  int jm = 0;
  explicit CgCache(int jmax) : jm(jmax + 1) {
    const size_t sz = size_t(jm) * jm * (2 * jm) * (2 * jm + 1) * (2 * jm + 1);
    val.assign(sz, 0.0);
    have.assign(sz, 0);
  }
  double get(int j1, int j2, int j3, int m1, int m2) {
    if (j1 >= jm || j2 >= jm || j3 >= 2 * jm || std::abs(m1) > j1 || std::abs(m2) > j2)
      return clebsch(j1, j2, j3, m1, m2, m1 + m2);
    const size_t idx = ((((size_t(j1) * jm + j2) * (2 * jm) + j3) * (2 * jm + 1) + (m1 + jm)) * (2 * jm + 1)) + (m2 + jm);
    if (!have[idx]) {
      val[idx] = clebsch(j1, j2, j3, m1, m2, m1 + m2);
      have[idx] = 1;
    }
    return val[idx];
  }
};

double factorial_d(int n) {
  double f = 1.0;
  for (int i = 2; i <= n; ++i) f *= i;
  return f;
}

}  // namespace

// ---------------------------------------------------------------------------
// Model object
// ---------------------------------------------------------------------------
struct tvs_model {
  // shells
  int htype = 1;  // 1,2 ANTOINE JT; synthetic models use 2
  int nsh = 0;
  std::vector<int> sh_n, sh_l, sh_2j, sh_na;
  // single-particle states (0-based storage, values as in the reference)
  int n = 0;
  std::vector<int> sp_n, sp_l, sp_2j, sp_2mj, sp_2mt, sp_sh, sp_tr;  // sp_sh, sp_tr 1-based
  double hw = 0.0, b = 0.0;
  double valence_Z = 0, valence_N = 0, core_Z = 0, core_N = 0;
  // interaction
  std::string name;
  double H0re = 0.0, H0im = 0.0;
  std::vector<double> H1;  // complex, column-major n x n, interleaved
  std::vector<int16_t> abcd;
  std::vector<float> h2;
  std::vector<int8_t> trperm;
  double scaling_1b = 1.0, scaling_2b = 1.0;
  // coupled elements H2cpd[T][J][a][b][c][d]
  int jdim = 0;  // HO_2jmax + 1
  std::vector<double> cpd;
  std::string err;

  size_t cidx(int T, int J, int a, int b, int c, int d) const {
    return ((((size_t(T) * jdim + J) * nsh + a) * nsh + b) * nsh + c) * nsh + d;
  }
};

namespace {

void build_basis(tvs_model* m, int facn) {
  m->sh_n.resize(m->nsh);
  m->sh_l.resize(m->nsh);
  m->sh_2j.resize(m->nsh);
  int jmax = 0;
  for (int i = 0; i < m->nsh; ++i) {
    m->sh_n[i] = m->sh_na[i] / facn;
    m->sh_l[i] = (m->sh_na[i] - m->sh_n[i] * facn) / 100;
    m->sh_2j[i] = m->sh_na[i] - m->sh_n[i] * facn - m->sh_l[i] * 100;
    if (m->sh_2j[i] > jmax) jmax = m->sh_2j[i];
  }
  m->jdim = jmax + 1;
  int half = 0;
  for (int i = 0; i < m->nsh; ++i) half += m->sh_2j[i] + 1;
  m->n = 2 * half;
  const int n = m->n;
  m->sp_n.assign(n, 0);
  m->sp_l.assign(n, 0);
  m->sp_2j.assign(n, 0);
  m->sp_2mj.assign(n, 0);
  m->sp_2mt.assign(n, 0);
  m->sp_sh.assign(n, 0);
  m->sp_tr.assign(n, 0);
  int k = 0;
  for (int i = 0; i < m->nsh; ++i) {
    int mjinc = 0;
    for (int j = 0; j <= m->sh_2j[i]; ++j) {
      const int kp = k, kn = k + half;  // 0-based
      for (int t = 0; t < 2; ++t) {
        const int kk = t ? kn : kp;
        m->sp_n[kk] = m->sh_n[i];
        m->sp_l[kk] = m->sh_l[i];
        m->sp_2j[kk] = m->sh_2j[i];
        m->sp_2mj[kk] = m->sh_2j[i] - mjinc;
        m->sp_2mt[kk] = t ? 1 : -1;
        m->sp_sh[kk] = i + 1;
      }
      // time-reversal partner (1-based): k + 2m (module_basis.f90:224,233)
      m->sp_tr[kp] = (kp + 1) + m->sp_2mj[kp];
      m->sp_tr[kn] = (kp + 1) + m->sp_2mj[kp] + half;
      mjinc += 2;
      ++k;
    }
  }
}

void set_hw(tvs_model* m, int opt_hw, double hw_in) {
  const double A = m->core_Z + m->core_N + m->valence_Z + m->valence_N;
  if (opt_hw == 0)
    m->hw = 45.0 * std::pow(A, -1.0 / 3.0) - 25.0 * std::pow(A, -2.0 / 3.0);
  else if (opt_hw == 1)
    m->hw = 41.0 * std::pow(A, -1.0 / 3.0);
  else
    m->hw = hw_in;
  m->b = kHbarc / std::sqrt(kMassMa * m->hw);
}

// 7-fold symmetry reconstruction of the coupled elements
// (module_hamiltonian.f90:282-319), JT scheme (find_iso is the identity).
void reconstruct_coupled(tvs_model* m) {
  const int ns = m->nsh;
  const int tmax = 3;
  for (int a = 0; a < ns; ++a)
    for (int b = 0; b < ns; ++b)
      for (int c = 0; c < ns; ++c)
        for (int d = 0; d < ns; ++d)
          for (int J = 0; J < m->jdim; ++J)
            for (int T = 0; T <= tmax; ++T) {
              const double V = m->cpd[m->cidx(T, J, a, b, c, d)];
              if (!(std::fabs(V) > 1.0e-12)) continue;
              const int xt = (T == 0) ? 0 : 1;
              // (ja + jb + J + T) is an integer for half-integer ja, jb
              const int eab = (m->sh_2j[a] + m->sh_2j[b]) / 2 + J + xt;
              const int ecd = (m->sh_2j[c] + m->sh_2j[d]) / 2 + J + xt;
              const double pab = (eab & 1) ? -1.0 : 1.0;
              const double pcd = (ecd & 1) ? -1.0 : 1.0;
              m->cpd[m->cidx(T, J, a, b, d, c)] = V * pcd;
              m->cpd[m->cidx(T, J, b, a, c, d)] = V * pab;
              m->cpd[m->cidx(T, J, b, a, d, c)] = V * pab * pcd;
              m->cpd[m->cidx(T, J, c, d, a, b)] = V;
              m->cpd[m->cidx(T, J, c, d, b, a)] = V * pab;
              m->cpd[m->cidx(T, J, d, c, a, b)] = V * pcd;
              m->cpd[m->cidx(T, J, d, c, b, a)] = V * pab * pcd;
            }
}

// uncouple_JT (module_hamiltonian.f90:828-885); a..d are 0-based sp indices.
double uncouple_jt(const tvs_model* m, CgCache& cg, int a, int b, int c, int d) {
  const int ja = m->sp_2j[a], jb = m->sp_2j[b], jc = m->sp_2j[c], jd = m->sp_2j[d];
  const int ma = m->sp_2mj[a], mb = m->sp_2mj[b], mc = m->sp_2mj[c], md = m->sp_2mj[d];
  const int MJ = ma + mb;
  const int ta = m->sp_2mt[a], tb = m->sp_2mt[b], tc = m->sp_2mt[c], td = m->sp_2mt[d];
  const int MT = ta + tb;
  const int sa = m->sp_sh[a] - 1, sb = m->sp_sh[b] - 1, sc = m->sp_sh[c] - 1, sd = m->sp_sh[d] - 1;
  const double dab = (sa == sb) ? 1.0 : 0.0;
  const double dcd = (sc == sd) ? 1.0 : 0.0;
  double sum = 0.0;
  const int Jlo = std::abs(MJ) / 2;
  int Jhi = (ja + jb) / 2;
  if ((jc + jd) / 2 < Jhi) Jhi = (jc + jd) / 2;
  for (int J = Jlo; J <= Jhi; ++J) {
    const double cg1 = cg.get(ja, jb, 2 * J, ma, mb);
    const double cg2 = cg.get(jc, jd, 2 * J, mc, md);
    int Tlo = std::abs(ta + tb) / 2;
    for (int T = Tlo; T <= 1; ++T) {
      const int MMT = MT / 2 + 2 * T;
      if (J >= m->jdim) continue;
      const double V = m->cpd[m->cidx(MMT, J, sa, sb, sc, sd)];
      if (std::fabs(V) < 1.0e-12) continue;
      const double ph = ((J + T) & 1) ? -1.0 : 1.0;
      const double NAB = std::sqrt(1.0 - dab * ph) / (1.0 + dab);
      const double NCD = std::sqrt(1.0 - dcd * ph) / (1.0 + dcd);
      if (NAB <= 1.0e-12 || NCD <= 1.0e-12) continue;
      const double NINV = 1.0 / (NAB * NCD);
      const double cg3 = cg.get(1, 1, 2 * T, ta, tb);
      const double cg4 = cg.get(1, 1, 2 * T, tc, td);
      sum = sum + NINV * cg1 * cg2 * cg3 * cg4 * V;
    }
  }
  return sum;
}

// Runs body(i, w) for i in [0, count) on up to `threads` host threads (w =
// the worker, 0 .. threads-1; worker 0 is the calling thread), the indices
// taken in order from a shared counter.
template <class F>
void parallel_for(int count, int threads, F body) {
  std::atomic<int> next{0};
  auto work = [&](int w) {
    for (int i; (i = next.fetch_add(1)) < count;) body(i, w);
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; ++t) pool.emplace_back(work, t);
  work(0);
  for (auto& th : pool) th.join();
}

int host_threads() {
  const unsigned hc = std::thread::hardware_concurrency();
  return int(std::max(1u, std::min(hc, 32u)));
}

// m-scheme enumeration (module_hamiltonian.f90:321-378) and the time-reversal
// permutation codes (reconstruct_2body_timerev, :970-1018).  The elements of
// each first index a are found on the host threads (each with its own
// Clebsch-Gordan cache) and joined in the order of a: the list is the serial
// one, element for element.
void enumerate_mscheme(tvs_model* m) {
  const int n = m->n;
  int jmax = 0;
  for (int i = 0; i < m->nsh; ++i) jmax = std::max(jmax, m->sh_2j[i]);
  m->abcd.clear();
  m->h2.clear();
  const double Vcut = 1.0e-16;
  std::vector<std::vector<int16_t>> abcd_a(n);
  std::vector<std::vector<float>> h2_a(n);
  const int threads = host_threads();
  std::vector<CgCache*> caches(threads, nullptr);
  parallel_for(n, threads, [&](int a, int w) {
    if (!caches[w]) caches[w] = new CgCache(std::max(jmax, 2));
    CgCache& cg = *caches[w];
    auto& out_abcd = abcd_a[a];
    auto& out_h2 = h2_a[a];
    const int la = m->sp_l[a], ma = m->sp_2mj[a], ta = m->sp_2mt[a];
    for (int b = a + 1; b < n; ++b) {
      const int lb = m->sp_l[b], mb = m->sp_2mj[b], tb = m->sp_2mt[b];
      if (ma + mb < 0) continue;
      for (int c = a; c < n; ++c) {
        const int lc = m->sp_l[c], mc = m->sp_2mj[c], tc = m->sp_2mt[c];
        const int dmax = (c == a) ? b : n - 1;
        for (int d = c + 1; d <= dmax; ++d) {
          const int ld = m->sp_l[d], md = m->sp_2mj[d], td = m->sp_2mt[d];
          if (((la + lb) & 1) != ((lc + ld) & 1)) continue;
          if (ta + tb != tc + td) continue;
          if (ma + mb != mc + md) continue;
          double V = uncouple_jt(m, cg, a, b, c, d);
          V = V * m->scaling_2b;
          if (std::fabs(V) > Vcut) {
            out_abcd.push_back(int16_t(a + 1));
            out_abcd.push_back(int16_t(b + 1));
            out_abcd.push_back(int16_t(c + 1));
            out_abcd.push_back(int16_t(d + 1));
            out_h2.push_back(float(V));
          }
        }
      }
    }
  });
  for (CgCache* cgp : caches) delete cgp;
  size_t total = 0;
  for (int a = 0; a < n; ++a) total += h2_a[a].size();
  m->abcd.reserve(4 * total);
  m->h2.reserve(total);
  for (int a = 0; a < n; ++a) {
    m->abcd.insert(m->abcd.end(), abcd_a[a].begin(), abcd_a[a].end());
    m->h2.insert(m->h2.end(), h2_a[a].begin(), h2_a[a].end());
    std::vector<int16_t>().swap(abcd_a[a]);
    std::vector<float>().swap(h2_a[a]);
  }
  const size_t S = m->h2.size();
  m->trperm.assign(S, 0);
  const int chunks = 64 * threads;
  parallel_for(chunks, threads, [&](int ch, int) {
  for (size_t kk = S * ch / chunks; kk < S * (ch + 1) / chunks; ++kk) {
    const int ia = m->abcd[4 * kk] - 1, ib = m->abcd[4 * kk + 1] - 1;
    const int ic = m->abcd[4 * kk + 2] - 1, id = m->abcd[4 * kk + 3] - 1;
    const int e = (m->sp_2j[ia] + m->sp_2j[ib] + m->sp_2j[ic] + m->sp_2j[id]) / 2;
    double phase = (e & 1) ? -1.0 : 1.0;
    int tra = m->sp_tr[ia], trb = m->sp_tr[ib], trc = m->sp_tr[ic], trd = m->sp_tr[id];
    int code = 0;
    if (tra > trb) {
      std::swap(tra, trb);
      phase = -phase;
      code += 1;
    }
    if (trc > trd) {
      std::swap(trc, trd);
      phase = -phase;
      code += 2;
    }
    if (tra > trc || (tra == trc && trb > trd)) code += 4;
    if (phase < 0.0) code -= 8;
    m->trperm[kk] = int8_t(code);
  }
  });
}

// Token reader for list-directed Fortran input.
struct Tokens {
  std::vector<std::string> t;
  size_t p = 0;
  bool more() const { return p < t.size(); }
  std::string next() { return p < t.size() ? t[p++] : std::string(); }
  double dbl() {
    std::string s = next();
    for (auto& ch : s)
      if (ch == 'D' || ch == 'd') ch = 'E';
    return std::strtod(s.c_str(), nullptr);
  }
  long lng() { return std::strtol(next().c_str(), nullptr, 10); }
};

void split_line(const std::string& line, std::vector<std::string>& out) {
  std::istringstream is(line);
  std::string w;
  while (is >> w) out.push_back(w);
}

int shell_index(const tvs_model* m, int label) {
  for (int i = 0; i < m->nsh; ++i)
    if (m->sh_na[i] == label) return i;
  return -1;
}

void fill_h1_spe(tvs_model* m, const std::vector<double>& spe_p, const std::vector<double>& spe_n) {
  const int n = m->n, half = n / 2;
  m->H1.assign(size_t(2) * n * n, 0.0);
  int k = 0;
  for (int i = 0; i < m->nsh; ++i)
    for (int j = 0; j <= m->sh_2j[i]; ++j) {
      m->H1[2 * (size_t(k) + size_t(k) * n)] = spe_p[i] * m->scaling_1b;
      const size_t kn = k + half;
      m->H1[2 * (kn + kn * n)] = spe_n[i] * m->scaling_1b;
      ++k;
    }
}

}  // namespace

extern "C" {

tvs_model* tvs_load_antoine(const char* path, double valence_Z, double valence_N) {
  std::ifstream f(path);
  auto* m = new tvs_model();
  if (!f) {
    m->err = "cannot open file";
    return m;
  }
  m->valence_Z = valence_Z;
  m->valence_N = valence_N;
  std::string line;
  std::getline(f, line);
  m->name = line;
  std::getline(f, line);
  {
    std::vector<std::string> w;
    split_line(line, w);
    m->htype = std::atoi(w[0].c_str());
    m->nsh = std::atoi(w[1].c_str());
    for (int i = 0; i < m->nsh; ++i) m->sh_na.push_back(std::atoi(w[2 + i].c_str()));
  }
  if (m->htype != 1 && m->htype != 2) {
    m->err = "only ANTOINE (hamil_type 1/2) files are supported";
    return m;
  }
  const int qmax = m->htype;
  std::vector<std::vector<double>> zepsi(qmax);
  for (int q = 0; q < qmax; ++q) {
    std::getline(f, line);
    std::vector<std::string> w;
    split_line(line, w);
    for (int i = 0; i < m->nsh; ++i) zepsi[q].push_back(std::strtod(w[i].c_str(), nullptr));
  }
  std::getline(f, line);
  int idens = 0, opt_hw = 0;
  double zmass = 0.0, hw = 0.0;
  {
    std::vector<std::string> w;
    split_line(line, w);
    idens = std::atoi(w[0].c_str());
    m->core_Z = std::atof(w[1].c_str());
    m->core_N = std::atof(w[2].c_str());
    zmass = std::atof(w[3].c_str());
    if (w.size() >= 6) {
      opt_hw = std::atoi(w[4].c_str());
      hw = std::atof(w[5].c_str());
    }
  }
  build_basis(m, 1000);
  set_hw(m, opt_hw, hw);
  const double x1 = m->core_Z + m->core_N + valence_Z + valence_N;
  const double x2 = m->core_Z + m->core_N + 2.0;
  if (idens == 1) {
    m->scaling_1b = 1.0;
    m->scaling_2b = std::pow(x2 / x1, zmass);
  } else if (idens == 2) {
    m->scaling_1b = std::pow(x2 / x1, zmass);
    m->scaling_2b = std::pow(x2 / x1, zmass);
  }
  fill_h1_spe(m, zepsi[0], zepsi[qmax - 1]);
  // two-body part (read_hamiltonian_2body_antoine, :412-459)
  Tokens tk;
  while (std::getline(f, line)) split_line(line, tk.t);
  const int ns = m->nsh;
  m->cpd.assign(size_t(4) * m->jdim * ns * ns * ns * ns, 0.0);
  while (tk.p + 8 <= tk.t.size()) {
    const int tmin = int(tk.lng()), tmax = int(tk.lng());
    int lab[4];
    for (int i = 0; i < 4; ++i) lab[i] = int(tk.lng());
    const int jmin = int(tk.lng()), jmax = int(tk.lng());
    int idx[4];
    for (int i = 0; i < 4; ++i) idx[i] = shell_index(m, lab[i]);
    for (int T = tmin; T <= tmax; ++T) {
      std::vector<double> tmp(m->jdim, 0.0);
      for (int J = jmin; J <= jmax; ++J) {
        const double v = tk.dbl();
        if (J < m->jdim) tmp[J] = v;
      }
      if (idx[0] < 0 || idx[1] < 0 || idx[2] < 0 || idx[3] < 0) continue;
      auto put = [&](int Tix) {
        for (int J = 0; J < m->jdim; ++J) m->cpd[m->cidx(Tix, J, idx[0], idx[1], idx[2], idx[3])] = tmp[J];
      };
      if (T == 0) {
        put(0);
      } else if (T == 1) {
        for (int i = 2; i <= 5 - tmax; ++i) put(i == 4 ? 1 : i);
      } else if (T == 2) {
        put(T + (((tmax + 1) & 1) ? -1 : 1));
      } else if (T == 3) {
        put(1);
      }
    }
  }
  reconstruct_coupled(m);
  enumerate_mscheme(m);
  m->cpd.clear();
  m->cpd.shrink_to_fit();
  return m;
}

// Seeded synthetic rotation- and isospin-invariant interaction in JT form:
// independent reduced elements V_JT(ab,cd) ~ N(0,1) * scale * exp(-(e_a+e_b+e_c+e_d)/damp)
// for canonically ordered shell quadruples; the reference's symmetry
// reconstruction then makes them antisymmetric and hermitian.
tvs_model* tvs_synthetic(int nsh, const int* sh_na, const double* spe_p, const double* spe_n,
                         double hw, double core_Z, double core_N, double valence_Z, double valence_N,
                         unsigned long long seed, double scale, double damp) {
  auto* m = new tvs_model();
  m->htype = 2;
  m->nsh = nsh;
  m->sh_na.assign(sh_na, sh_na + nsh);
  m->core_Z = core_Z;
  m->core_N = core_N;
  m->valence_Z = valence_Z;
  m->valence_N = valence_N;
  m->name = "synthetic JT interaction";
  build_basis(m, 1000);
  set_hw(m, 2, hw);
  std::vector<double> sp(spe_p, spe_p + nsh), sn(spe_n, spe_n + nsh);
  fill_h1_spe(m, sp, sn);
  const int ns = nsh;
  m->cpd.assign(size_t(4) * m->jdim * ns * ns * ns * ns, 0.0);
  std::mt19937_64 rng(seed);
  std::normal_distribution<double> nd(0.0, 1.0);
  auto e_of = [&](int s) { return 2 * m->sh_n[s] + m->sh_l[s]; };
  for (int a = 0; a < ns; ++a)
    for (int b = a; b < ns; ++b)
      for (int c = 0; c < ns; ++c)
        for (int d = c; d < ns; ++d) {
          if (a * ns + b > c * ns + d) continue;
          if (((m->sh_l[a] + m->sh_l[b] + m->sh_l[c] + m->sh_l[d]) & 1) != 0) continue;
          const int jlo = std::max(std::abs(m->sh_2j[a] - m->sh_2j[b]), std::abs(m->sh_2j[c] - m->sh_2j[d])) / 2;
          const int jhi = std::min(m->sh_2j[a] + m->sh_2j[b], m->sh_2j[c] + m->sh_2j[d]) / 2;
          const double damping =
              (damp > 0.0) ? std::exp(-double(e_of(a) + e_of(b) + e_of(c) + e_of(d)) / damp) : 1.0;
          for (int J = jlo; J <= jhi; ++J)
            for (int T = 0; T <= 1; ++T) {
              if (a == b && ((J + T) & 1) == 0) continue;
              if (c == d && ((J + T) & 1) == 0) continue;
              double v = nd(rng) * scale * damping;
              if (a == c && b == d) {
                // diagonal elements of a hermitian real matrix are free
              }
              if (J >= m->jdim) continue;
              if (T == 0) {
                m->cpd[m->cidx(0, J, a, b, c, d)] = v;
              } else {
                for (int t = 1; t <= 3; ++t) m->cpd[m->cidx(t, J, a, b, c, d)] = v;
              }
            }
        }
  reconstruct_coupled(m);
  enumerate_mscheme(m);
  m->cpd.clear();
  m->cpd.shrink_to_fit();
  return m;
}

const char* tvs_error(const tvs_model* m) { return m->err.empty() ? nullptr : m->err.c_str(); }
void tvs_free(tvs_model* m) { delete m; }
int tvs_dim(const tvs_model* m) { return m->n; }
int tvs_nshells(const tvs_model* m) { return m->nsh; }
long long tvs_nelements(const tvs_model* m) { return (long long)m->h2.size(); }
double tvs_hw(const tvs_model* m) { return m->hw; }
double tvs_oscillator_length(const tvs_model* m) { return m->b; }

void tvs_get_basis(const tvs_model* m, int* sp_n, int* sp_l, int* sp_2j, int* sp_2mj, int* sp_2mt,
                   int* sp_sh, int* sp_tr) {
  const int n = m->n;
  std::memcpy(sp_n, m->sp_n.data(), sizeof(int) * n);
  std::memcpy(sp_l, m->sp_l.data(), sizeof(int) * n);
  std::memcpy(sp_2j, m->sp_2j.data(), sizeof(int) * n);
  std::memcpy(sp_2mj, m->sp_2mj.data(), sizeof(int) * n);
  std::memcpy(sp_2mt, m->sp_2mt.data(), sizeof(int) * n);
  std::memcpy(sp_sh, m->sp_sh.data(), sizeof(int) * n);
  std::memcpy(sp_tr, m->sp_tr.data(), sizeof(int) * n);
}

void tvs_get_shells(const tvs_model* m, int* sh_na) { std::memcpy(sh_na, m->sh_na.data(), sizeof(int) * m->nsh); }

void tvs_get_hamiltonian(const tvs_model* m, double* H0, double* H1, int16_t* abcd, float* h2, int8_t* trperm) {
  H0[0] = m->H0re;
  H0[1] = m->H0im;
  std::memcpy(H1, m->H1.data(), sizeof(double) * m->H1.size());
  std::memcpy(abcd, m->abcd.data(), sizeof(int16_t) * m->abcd.size());
  std::memcpy(h2, m->h2.data(), sizeof(float) * m->h2.size());
  std::memcpy(trperm, m->trperm.data(), sizeof(int8_t) * m->trperm.size());
}

// <a| r^lam |b> of the HO radial functions (radial_integral_even,
// module_basis.f90:374-410: Suhonen's closed form).  For la = lb it equals
// the Gauss-Laguerre quadrature of radial_integral (module_basis.f90:329-372),
// which is exact for this polynomial integrand.
static double radial_integral_even(const tvs_model* m, int ia, int ib, int lam) {
  const int na = m->sp_n[ia], nb = m->sp_n[ib], la = m->sp_l[ia], lb = m->sp_l[ib];
  double integral = 0.0;
  if (((la + lb + lam) % 2) == 0) {
    const int taua = (lb - la + lam) / 2, taub = (la - lb + lam) / 2;
    if (taua >= 0 && taub >= 0) {
      const double pre = (((na + nb) & 1) ? -1.0 : 1.0) *
                         std::sqrt((factorial_d(na) * factorial_d(nb)) /
                                   (std::tgamma(na + la + 1.5) * std::tgamma(nb + lb + 1.5))) *
                         factorial_d(taua) * factorial_d(taub);
      const int smin = std::max(0, std::max(na - taua, nb - taub));
      const int smax = std::min(na, nb);
      double s = 0.0;
      for (int sg = smin; sg <= smax; ++sg)
        s += std::tgamma((la + lb + lam) / 2.0 + sg + 1.5) /
             (factorial_d(sg) * factorial_d(na - sg) * factorial_d(nb - sg) * factorial_d(sg + taua - na) *
              factorial_d(sg + taub - nb));
      integral = s * pre * std::pow(m->b, lam);
    }
  }
  return integral;
}

// Q_lm HO matrix elements for lambda = 1..4 (set_multipoles,
// module_multipoles.f90:43-128).  Output layout: q[((lam-1)*2 + t)*5 + mq][incr]
// with incr = ia*n + ib (the reference's vectorised operator, 0-based),
// t = 0 protons / 1 neutrons, mq = |mu| (0..lam).  Each operator has n*n
// entries; the caller provides 4*2*5*n*n doubles.
void tvs_multipoles(const tvs_model* m, double* q) {
  const int n = m->n;
  const size_t n2 = size_t(n) * n;
  std::memset(q, 0, sizeof(double) * 40 * n2);
  auto radial_even = [&](int ia, int ib, int lam) { return radial_integral_even(m, ia, ib, lam); };
  size_t incr = 0;
  for (int ia = 0; ia < n; ++ia) {
    const int la = m->sp_l[ia] * 2, ja = m->sp_2j[ia], mja = m->sp_2mj[ia], mta = m->sp_2mt[ia];
    for (int ib = 0; ib < n; ++ib, ++incr) {
      const int lb = m->sp_l[ib] * 2, jb = m->sp_2j[ib], mjb = m->sp_2mj[ib], mtb = m->sp_2mt[ib];
      if (mta != mtb) continue;
      for (int lambda = 2; lambda <= 8; lambda += 2) {
        if ((la + lb + lambda) % 4 != 0) continue;
        const double cb1 = clebsch(lb, lambda, la, 0, 0, 0);
        const double fac = cb1 * radial_even(ia, ib, lambda / 2) *
                           std::sqrt(double((lb + 1) * (lambda + 1)) / (4.0 * kPi * (la + 1)));
        for (int mu = -lambda; mu <= lambda; mu += 2) {
          double sumcb = 0.0;
          for (int ms = -1; ms <= 1; ms += 2)
            for (int mla = -la; mla <= la; mla += 2)
              for (int mlb = -lb; mlb <= lb; mlb += 2) {
                const double c1 = clebsch(la, 1, ja, mla, ms, mja);
                const double c2 = clebsch(lb, 1, jb, mlb, ms, mjb);
                const double c3 = clebsch(lb, lambda, la, mlb, mu, mla);
                sumcb = sumcb + c1 * c2 * c3;
              }
          sumcb = sumcb * fac;
          if (mu < 0) sumcb = (((mu / 2) & 1) ? -1.0 : 1.0) * sumcb;
          if (mu != 0) sumcb = sumcb * 0.5;
          const int t = (mta + 3) / 2 - 1;
          const int mq = std::abs(mu / 2);
          const int lam = lambda / 2;
          q[(size_t((lam - 1) * 2 + t) * 5 + mq) * n2 + incr] += sumcb;
        }
      }
    }
  }
}

// beta_lm -> Q_lm conversion factors coeff_betalm(i,j) (module_multipoles.f90:58-74),
// out[(i-1)*4 + (j-1)], i = 1 protons, 2 neutrons, 3,4 nucleons.
void tvs_coeff_betalm(const tvs_model* m, double* out) {
  const double Z = m->core_Z + m->valence_Z, N = m->core_N + m->valence_N;
  for (int i = 1; i <= 4; ++i)
    for (int j = 1; j <= 4; ++j) {
      const double np = (i == 1) ? Z : (i == 2) ? N : Z + N;
      const double c1 = (4.0 * kPi) / (3.0 * np);
      const double c2 = 1.0 / (kRadiusR0 * std::pow(np, 1.0 / 3.0));
      out[(i - 1) * 4 + (j - 1)] = c1 * std::pow(c2, j);
    }
}

// The one-body operators of the printed observables, each n*n in the
// reference's vectorised layout (incr = ia*n + ib, 0-based):
//   ops[0..5]  Jx, Jy, Jz, Jx^2, Jy^2, Jz^2 (set_angular_momentum,
//              module_angularmomentum.f90:33-103: Jy is stored real, the
//              operator being i Jy);
//   ops[6]     the spin-orbit l.s factor on the diagonal (:106-119);
//   ops[7..8]  r^2 for protons, neutrons (set_radius, module_radius.f90:30-63).
// parity[i] = (-1)^l_i (generate_rotation_parity, module_projection.f90:607-625).
void tvs_observable_ops(const tvs_model* m, double* ops, int* parity) {
  const int n = m->n;
  const size_t n2 = size_t(n) * n;
  std::memset(ops, 0, sizeof(double) * 9 * n2);
  size_t incr = 0;
  for (int ia = 0; ia < n; ++ia) {
    const int ina = m->sp_n[ia], ila = m->sp_l[ia], ija = m->sp_2j[ia], ima = m->sp_2mj[ia], ita = m->sp_2mt[ia];
    for (int ib = 0; ib < n; ++ib, ++incr) {
      const int inb = m->sp_n[ib], ilb = m->sp_l[ib], ijb = m->sp_2j[ib], imb = m->sp_2mj[ib], itb = m->sp_2mt[ib];
      const double rjb = ijb / 2.0, rmb = imb / 2.0;
      const double fp1 = rjb * (rjb + 1.0) - rmb * (rmb + 1.0);
      const double fm1 = rjb * (rjb + 1.0) - rmb * (rmb - 1.0);
      const double fp1p2 = rjb * (rjb + 1.0) - (rmb + 1.0) * (rmb + 2.0);
      const double fm1m2 = rjb * (rjb + 1.0) - (rmb - 1.0) * (rmb - 2.0);
      const double f02 = rjb * (rjb + 1.0) - rmb * rmb;
      if (ina == inb && ila == ilb && ija == ijb && ita == itb) {
        const double dp2 = (ima == imb + 4), dp1 = (ima == imb + 2), d0 = (ima == imb), dm1 = (ima == imb - 2),
                     dm2 = (ima == imb - 4);
        ops[0 * n2 + incr] = 0.5 * (std::sqrt(fp1) * dp1 + std::sqrt(fm1) * dm1);
        ops[1 * n2 + incr] = 0.5 * (std::sqrt(fp1) * dp1 - std::sqrt(fm1) * dm1);
        ops[2 * n2 + incr] = rmb * d0;
        ops[3 * n2 + incr] = 0.25 * (std::sqrt(fp1 * fp1p2) * dp2 + std::sqrt(fm1 * fm1m2) * dm2 + 2 * f02 * d0);
        ops[4 * n2 + incr] = 0.25 * (std::sqrt(fp1 * fp1p2) * dp2 + std::sqrt(fm1 * fm1m2) * dm2 - 2 * f02 * d0);
        ops[5 * n2 + incr] = (rmb * d0) * (rmb * d0);
      }
      if (ia == ib) {
        const double xja = ija / 2.0;
        ops[6 * n2 + incr] = xja * (xja + 1) - ila * (ila + 1) - 0.75;
      }
      if (ija == ijb && ima == imb && ita == itb && ila == ilb) {
        const int t = (ita + 3) / 2 - 1;
        ops[size_t(7 + t) * n2 + incr] = radial_integral_even(m, ib, ia, 2);
      }
    }
    parity[ia] = (ila & 1) ? -1 : 1;
  }
}

// .red stream file (module_hamiltonian.f90:533-627): name (100 chars),
// hamil_type (i32), H0 (c128), H1 (n*n c128), H2dim (i64), abcd (4*dim i16),
// H2 (dim f32), trperm (dim i8).  No record markers.
int tvs_write_red(const tvs_model* m, const char* path) {
  FILE* f = std::fopen(path, "wb");
  if (!f) return 1;
  char name[100];
  std::memset(name, ' ', 100);
  std::memcpy(name, m->name.data(), std::min<size_t>(100, m->name.size()));
  int32_t ht = m->htype;
  double h0[2] = {m->H0re, m->H0im};
  int64_t dim = (int64_t)m->h2.size();
  std::fwrite(name, 1, 100, f);
  std::fwrite(&ht, 4, 1, f);
  std::fwrite(h0, 8, 2, f);
  std::fwrite(m->H1.data(), 8, m->H1.size(), f);
  std::fwrite(&dim, 8, 1, f);
  std::fwrite(m->abcd.data(), 2, m->abcd.size(), f);
  std::fwrite(m->h2.data(), 4, m->h2.size(), f);
  std::fwrite(m->trperm.data(), 1, m->trperm.size(), f);
  std::fclose(f);
  return 0;
}

// Reads a .red file into an existing model whose basis matches (n states).
int tvs_read_red(tvs_model* m, const char* path) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return 1;
  char name[100];
  int32_t ht = 0;
  double h0[2];
  int64_t dim = 0;
  int ok = 1;
  ok &= std::fread(name, 1, 100, f) == 100;
  ok &= std::fread(&ht, 4, 1, f) == 1;
  ok &= std::fread(h0, 8, 2, f) == 2;
  m->H1.assign(size_t(2) * m->n * m->n, 0.0);
  ok &= std::fread(m->H1.data(), 8, m->H1.size(), f) == m->H1.size();
  ok &= std::fread(&dim, 8, 1, f) == 1;
  if (!ok || dim < 0) {
    std::fclose(f);
    return 2;
  }
  m->abcd.resize(size_t(4) * dim);
  m->h2.resize(dim);
  m->trperm.resize(dim);
  ok &= std::fread(m->abcd.data(), 2, m->abcd.size(), f) == m->abcd.size();
  ok &= std::fread(m->h2.data(), 4, m->h2.size(), f) == m->h2.size();
  ok &= std::fread(m->trperm.data(), 1, m->trperm.size(), f) == m->trperm.size();
  std::fclose(f);
  if (!ok) return 3;
  m->name.assign(name, 100);
  m->htype = ht;
  m->H0re = h0[0];
  m->H0im = h0[1];
  return 0;
}

double tvs_clebsch(int j1, int j2, int j3, int m1, int m2, int m3) { return clebsch(j1, j2, j3, m1, m2, m3); }

}  // extern "C"
