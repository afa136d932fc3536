// Sparse two-body contraction (calculate_fields, module_fields.f90:99-189) on
// sm_103a.
//
// Setup (once per Hamiltonian, tvap_set_hamiltonian): the reference's element
// list -- hamil_abcd (i16, 1-based), hamil_H2 (f32), hamil_trperm (i8) -- is
// decoded on the device exactly as the reference's loop does it: pass 1 with
// the stored indices, pass 2 (skipped when 2m_a + 2m_b = 0) through
// find_timerev (module_hamiltonian.f90:1028-1089) with the phase sign(perm),
// f2b = h2b (1 - delta_ac delta_bd).  Every pass produces the reference's 8
// Gamma and 2 Delta updates; these are regrouped by destination (stable radix
// sort, so entries stay in element order) into CSR rows of a gather operator
// W: Gamma_x = sum_e W_e rho_{src(e)}.
//
// Per iteration: one warp owns one output entry and accumulates it in
// registers for every gauge angle at once; angles are the innermost
// (contiguous) dimension of the density and field arrays, so each gathered
// source row is a coalesced 16*ncol-byte read and there are no atomics.
// The Delta pass writes the strict lower triangle and its skew image,
// h = Gamma + H1 is fused into the Gamma epilogue.

#include <cub/cub.cuh>

#include "tvap_internal.cuh"

namespace tvap {

namespace {

__device__ __forceinline__ void find_timerev_dev(const int* __restrict__ tr, int p, int& a, int& b, int& c,
                                                 int& d) {
  const int ta = tr[a - 1], tb = tr[b - 1], tc = tr[c - 1], td = tr[d - 1];
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

constexpr int kInvalid = 0x7fffffff;

// One thread per (element, pass).  Slot layout: Gamma slots e*16 + pass*8 + s,
// Delta slots e*4 + pass*2 + s.  Invalid slots get key kInvalid.
__global__ void decode_kernel(long long S, int n, const int16_t* __restrict__ abcd, const float* __restrict__ h2,
                              const int8_t* __restrict__ trperm, const int* __restrict__ sp_2mj,
                              const int* __restrict__ sp_tr, int* gkey, int* gsrc, double* gcoef, int* dkey,
                              int* dsrc, double* dcoef, int* bad) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= 2 * S) return;
  const long long e = t >> 1;
  const int pass = int(t & 1);
  int ia = abcd[4 * e], ib = abcd[4 * e + 1], ic = abcd[4 * e + 2], id = abcd[4 * e + 3];
  double h2b = double(h2[e]);
  const int perm = trperm[e];
  bool valid = true;
  if (ia < 1 || ia > n || ib < 1 || ib > n || ic < 1 || ic > n || id < 1 || id > n) {
    valid = false;
    atomicOr(bad, 1);
  } else if (pass == 1) {
    if (sp_2mj[ia - 1] + sp_2mj[ib - 1] == 0) {
      valid = false;
    } else {
      find_timerev_dev(sp_tr, perm, ia, ib, ic, id);
      h2b = (perm < 0 ? -1.0 : 1.0) * h2b;
      if (ia < 1 || ia > n || ib < 1 || ib > n || ic < 1 || ic > n || id < 1 || id > n) {
        valid = false;
        atomicOr(bad, 1);
      }
    }
  }
  const double f2b = h2b * double(1 - ((ia == ic) ? 1 : 0) * ((ib == id) ? 1 : 0));
  auto L = [n](int i, int j) { return (i - 1) + (j - 1) * n; };
  const long long g0 = e * 16 + pass * 8, d0 = e * 4 + pass * 2;
  if (!valid) {
    for (int s = 0; s < 8; ++s) gkey[g0 + s] = kInvalid;
    for (int s = 0; s < 2; ++s) dkey[d0 + s] = kInvalid;
    return;
  }
  const int gdst[8] = {L(ia, ic), L(ia, id), L(ib, ic), L(ib, id), L(ic, ia), L(ic, ib), L(id, ia), L(id, ib)};
  const int gs[8] = {L(id, ib), L(ic, ib), L(id, ia), L(ic, ia), L(ib, id), L(ia, id), L(ib, ic), L(ia, ic)};
  const double gc[8] = {h2b, -h2b, -h2b, h2b, f2b, -f2b, -f2b, f2b};
  for (int s = 0; s < 8; ++s) {
    gkey[g0 + s] = (gc[s] != 0.0) ? gdst[s] : kInvalid;
    gsrc[g0 + s] = gs[s];
    gcoef[g0 + s] = gc[s];
  }
  dkey[d0] = (h2b != 0.0) ? L(ib, ia) : kInvalid;
  dsrc[d0] = L(id, ic);
  dcoef[d0] = h2b;
  dkey[d0 + 1] = (f2b != 0.0) ? L(id, ic) : kInvalid;
  dsrc[d0 + 1] = L(ib, ia);
  dcoef[d0 + 1] = f2b;
}

__global__ void gather_sorted_kernel(long long m, const int* __restrict__ slot, const int* __restrict__ src_in,
                                     const double* __restrict__ coef_in, int* __restrict__ src_out,
                                     double* __restrict__ coef_out) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= m) return;
  const int s = slot[i];
  src_out[i] = src_in[s];
  coef_out[i] = coef_in[s];
}

__global__ void count_rows_kernel(long long m, const int* __restrict__ key, int* __restrict__ counts) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= m) return;
  atomicAdd(&counts[key[i]], 1);
}

__global__ void iota_kernel(long long m, int* v) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < m) v[i] = int(i);
}

// number of valid (key != kInvalid) entries after sorting = first invalid pos
__global__ void count_valid_kernel(long long m, const int* __restrict__ key, long long* out) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= m) return;
  const bool v = key[i] != kInvalid;
  const bool vnext = (i + 1 < m) ? (key[i + 1] != kInvalid) : false;
  if (v && !vnext) *out = i + 1;
  if (i == 0 && !v) *out = 0;
}

int sort_and_compress(long long m, int nrows, int* key, int* src, double* coef, int** rowptr_out, int** src_out,
                      double** coef_out, long long* nnz_out, cudaStream_t s) {
  int *slot_in = nullptr, *slot_out = nullptr, *key_out = nullptr;
  TVAP_CUDA(cudaMalloc(&slot_in, sizeof(int) * m));
  TVAP_CUDA(cudaMalloc(&slot_out, sizeof(int) * m));
  TVAP_CUDA(cudaMalloc(&key_out, sizeof(int) * m));
  const int tb = 256;
  const long long gb = (m + tb - 1) / tb;
  iota_kernel<<<gb, tb, 0, tvap::counted(s)>>>(m, slot_in);
  size_t tmp_bytes = 0;
  int end_bit = 1;
  while ((1LL << end_bit) <= (long long)kInvalid && end_bit < 31) ++end_bit;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, key, key_out, slot_in, slot_out, (int)m, 0, end_bit, s);
  void* tmp = nullptr;
  TVAP_CUDA(cudaMalloc(&tmp, tmp_bytes));
  cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, key, key_out, slot_in, slot_out, (int)m, 0, end_bit, s);
  TVAP_CUDA(cudaGetLastError());
  long long* d_nnz = nullptr;
  TVAP_CUDA(cudaMalloc(&d_nnz, sizeof(long long)));
  TVAP_CUDA(cudaMemsetAsync(d_nnz, 0, sizeof(long long), s));
  count_valid_kernel<<<gb, tb, 0, tvap::counted(s)>>>(m, key_out, d_nnz);
  long long nnz = 0;
  TVAP_CUDA(cudaMemcpyAsync(&nnz, d_nnz, sizeof(long long), cudaMemcpyDeviceToHost, s));
  TVAP_CUDA(cudaStreamSynchronize(s));
  int* counts = nullptr;
  TVAP_CUDA(cudaMalloc(&counts, sizeof(int) * (nrows + 1)));
  TVAP_CUDA(cudaMemsetAsync(counts, 0, sizeof(int) * (nrows + 1), s));
  int* rowptr = nullptr;
  TVAP_CUDA(cudaMalloc(&rowptr, sizeof(int) * (nrows + 1)));
  if (nnz > 0) count_rows_kernel<<<(nnz + tb - 1) / tb, tb, 0, tvap::counted(s)>>>(nnz, key_out, counts);
  size_t scan_bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, counts, rowptr, nrows + 1, s);
  void* scan_tmp = nullptr;
  TVAP_CUDA(cudaMalloc(&scan_tmp, scan_bytes));
  cub::DeviceScan::ExclusiveSum(scan_tmp, scan_bytes, counts, rowptr, nrows + 1, s);
  int* srcs = nullptr;
  double* coefs = nullptr;
  TVAP_CUDA(cudaMalloc(&srcs, sizeof(int) * std::max(1LL, nnz)));
  TVAP_CUDA(cudaMalloc(&coefs, sizeof(double) * std::max(1LL, nnz)));
  if (nnz > 0) gather_sorted_kernel<<<(nnz + tb - 1) / tb, tb, 0, tvap::counted(s)>>>(nnz, slot_out, src, coef, srcs, coefs);
  TVAP_CUDA(cudaGetLastError());
  TVAP_CUDA(cudaStreamSynchronize(s));
  cudaFree(slot_in);
  cudaFree(slot_out);
  cudaFree(key_out);
  cudaFree(tmp);
  cudaFree(d_nnz);
  cudaFree(counts);
  cudaFree(scan_tmp);
  *rowptr_out = rowptr;
  *src_out = srcs;
  *coef_out = coefs;
  *nnz_out = nnz;
  return TVAP_OK;
}

}  // namespace

int build_field_csr(tvap_ctx* c) {
  free_field_csr(c->csr);
  const long long S = c->S;
  const int n = c->n;
  const long long mg = 16 * S, md = 4 * S;
  cudaStream_t s = c->stream;
  int *gkey, *gsrc, *dkey, *dsrc, *bad;
  double *gcoef, *dcoef;
  TVAP_CUDA(cudaMalloc(&gkey, sizeof(int) * std::max(1LL, mg)));
  TVAP_CUDA(cudaMalloc(&gsrc, sizeof(int) * std::max(1LL, mg)));
  TVAP_CUDA(cudaMalloc(&gcoef, sizeof(double) * std::max(1LL, mg)));
  TVAP_CUDA(cudaMalloc(&dkey, sizeof(int) * std::max(1LL, md)));
  TVAP_CUDA(cudaMalloc(&dsrc, sizeof(int) * std::max(1LL, md)));
  TVAP_CUDA(cudaMalloc(&dcoef, sizeof(double) * std::max(1LL, md)));
  TVAP_CUDA(cudaMalloc(&bad, sizeof(int)));
  TVAP_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), s));
  if (S > 0) {
    const int tb = 256;
    decode_kernel<<<(2 * S + tb - 1) / tb, tb, 0, tvap::counted(s)>>>(S, n, c->d_abcd, c->d_h2, c->d_trperm, c->d_sp_2mj,
                                                       c->d_sp_tr, gkey, gsrc, gcoef, dkey, dsrc, dcoef, bad);
    TVAP_CUDA(cudaGetLastError());
  }
  int hbad = 0;
  TVAP_CUDA(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
  TVAP_CUDA(cudaStreamSynchronize(s));
  int rc = TVAP_OK;
  if (hbad) {
    set_last_error("element index outside 1..n in hamil_abcd or after time reversal", __FILE__, __LINE__);
    rc = TVAP_ERR_ARG;
  }
  const int nrows = n * n;
  if (rc == TVAP_OK && mg > 0)
    rc = sort_and_compress(mg, nrows, gkey, gsrc, gcoef, &c->csr.g_rowptr, &c->csr.g_src, &c->csr.g_coef,
                           &c->csr.g_nnz, s);
  if (rc == TVAP_OK && md > 0)
    rc = sort_and_compress(md, nrows, dkey, dsrc, dcoef, &c->csr.d_rowptr, &c->csr.d_src, &c->csr.d_coef,
                           &c->csr.d_nnz, s);
  if (rc == TVAP_OK && mg == 0) {
    TVAP_CUDA(cudaMalloc(&c->csr.g_rowptr, sizeof(int) * (nrows + 1)));
    TVAP_CUDA(cudaMemset(c->csr.g_rowptr, 0, sizeof(int) * (nrows + 1)));
    TVAP_CUDA(cudaMalloc(&c->csr.d_rowptr, sizeof(int) * (nrows + 1)));
    TVAP_CUDA(cudaMemset(c->csr.d_rowptr, 0, sizeof(int) * (nrows + 1)));
  }
  cudaFree(gkey);
  cudaFree(gsrc);
  cudaFree(gcoef);
  cudaFree(dkey);
  cudaFree(dsrc);
  cudaFree(dcoef);
  cudaFree(bad);
  return rc;
}

void free_field_csr(FieldCSR& f) {
  free_field_dense(f.dense_g);
  free_field_dense(f.dense_d);
  cudaFree(f.g_rowptr);
  cudaFree(f.g_src);
  cudaFree(f.g_coef);
  cudaFree(f.d_rows);
  cudaFree(f.d_rowptr);
  cudaFree(f.d_src);
  cudaFree(f.d_coef);
  f = FieldCSR();
}

namespace {

constexpr int kWarpsPerBlock = 8;

// Gamma and h: one warp per output entry r = x + y n, CPL angle columns per lane.
template <int CPL>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    gamma_gather_kernel(int n, int ncol, int ldc, const int* __restrict__ rowptr, const int* __restrict__ srcs,
                        const double* __restrict__ coefs, const double2* __restrict__ rho,
                        const double2* __restrict__ H1, double2* __restrict__ gamma, double2* __restrict__ hsp) {
  const int lane = threadIdx.x & 31;
  const long long r = blockIdx.x * (long long)kWarpsPerBlock + (threadIdx.x >> 5);
  if (r >= (long long)n * n) return;
  double2 acc[CPL];
#pragma unroll
  for (int c = 0; c < CPL; ++c) acc[c] = make_double2(0.0, 0.0);
  const int beg = rowptr[r], end = rowptr[r + 1];
  for (int base = beg; base < end; base += 32) {
    const int cnt = min(32, end - base);
    int my_src = 0;
    double my_coef = 0.0;
    if (lane < cnt) {
      my_src = srcs[base + lane];
      my_coef = coefs[base + lane];
    }
    for (int t = 0; t < cnt; ++t) {
      const int sidx = __shfl_sync(0xffffffffu, my_src, t);
      const double w = __shfl_sync(0xffffffffu, my_coef, t);
      const double2* row = rho + (long long)sidx * ldc;
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        const int col = lane + 32 * c;
        if (col < ncol) {
          const double2 v = row[col];
          acc[c].x = fma(w, v.x, acc[c].x);
          acc[c].y = fma(w, v.y, acc[c].y);
        }
      }
    }
  }
  const double2 h1 = H1[r];
#pragma unroll
  for (int c = 0; c < CPL; ++c) {
    const int col = lane + 32 * c;
    if (col < ncol) {
      gamma[r * ldc + col] = acc[c];
      hsp[r * ldc + col] = cadd(acc[c], h1);
    }
  }
}

// Delta^LR, Delta^RL: one warp per strict-lower entry (b > a); writes the
// entry and its skew image; the diagonal is written as zero.
template <int CPL>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    delta_gather_kernel(int n, int ncol, int ldc, const int* __restrict__ rowptr, const int* __restrict__ srcs,
                        const double* __restrict__ coefs, const double2* __restrict__ kLR,
                        const double2* __restrict__ kRL, double2* __restrict__ dLR, double2* __restrict__ dRL) {
  const int lane = threadIdx.x & 31;
  const long long w = blockIdx.x * (long long)kWarpsPerBlock + (threadIdx.x >> 5);
  // w enumerates (row b, col a) pairs with a <= b, column by column
  const long long tot = (long long)n * (n + 1) / 2;
  if (w >= tot) return;
  // invert w -> (a, b): column a holds entries b = a..n-1; offset(a) = a n - a(a-1)/2
  int a = int((2.0 * n + 1.0 - sqrt((2.0 * n + 1.0) * (2.0 * n + 1.0) - 8.0 * double(w))) / 2.0);
  if (a < 0) a = 0;
  if (a > n - 1) a = n - 1;
  while (a > 0 && (long long)a * n - (long long)a * (a - 1) / 2 > w) --a;
  while (a < n - 1 && (long long)(a + 1) * n - (long long)(a + 1) * a / 2 <= w) ++a;
  const int b = a + int(w - ((long long)a * n - (long long)a * (a - 1) / 2));
  const long long r = b + (long long)a * n;
  if (a == b) {
#pragma unroll
    for (int c = 0; c < CPL; ++c) {
      const int col = lane + 32 * c;
      if (col < ncol) {
        dLR[r * ldc + col] = make_double2(0.0, 0.0);
        dRL[r * ldc + col] = make_double2(0.0, 0.0);
      }
    }
    return;
  }
  double2 al[CPL], ar[CPL];
#pragma unroll
  for (int c = 0; c < CPL; ++c) {
    al[c] = make_double2(0.0, 0.0);
    ar[c] = make_double2(0.0, 0.0);
  }
  const int beg = rowptr[r], end = rowptr[r + 1];
  for (int base = beg; base < end; base += 32) {
    const int cnt = min(32, end - base);
    int my_src = 0;
    double my_coef = 0.0;
    if (lane < cnt) {
      my_src = srcs[base + lane];
      my_coef = coefs[base + lane];
    }
    for (int t = 0; t < cnt; ++t) {
      const int sidx = __shfl_sync(0xffffffffu, my_src, t);
      const double wt = __shfl_sync(0xffffffffu, my_coef, t);
      const double2* rl = kLR + (long long)sidx * ldc;
      const double2* rr = kRL + (long long)sidx * ldc;
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        const int col = lane + 32 * c;
        if (col < ncol) {
          const double2 u = rl[col], v = rr[col];
          al[c].x = fma(wt, u.x, al[c].x);
          al[c].y = fma(wt, u.y, al[c].y);
          ar[c].x = fma(wt, v.x, ar[c].x);
          ar[c].y = fma(wt, v.y, ar[c].y);
        }
      }
    }
  }
  const long long rt = a + (long long)b * n;
#pragma unroll
  for (int c = 0; c < CPL; ++c) {
    const int col = lane + 32 * c;
    if (col < ncol) {
      dLR[r * ldc + col] = al[c];
      dRL[r * ldc + col] = ar[c];
      dLR[rt * ldc + col] = make_double2(-al[c].x, -al[c].y);
      dRL[rt * ldc + col] = make_double2(-ar[c].x, -ar[c].y);
    }
  }
}

template <int CPL>
void launch_fields(tvap_ctx* c, int ncol, int ldc, const double2* rho, const double2* kLR, const double2* kRL,
                   double2* gamma, double2* hsp, double2* dLR, double2* dRL, cudaStream_t s) {
  const int n = c->n;
  const long long rows = (long long)n * n;
  sec_begin_on(c, SEC_FIELDS_GAMMA, s);
  gamma_gather_kernel<CPL><<<(rows + kWarpsPerBlock - 1) / kWarpsPerBlock, 32 * kWarpsPerBlock, 0, tvap::counted(s)>>>(
      n, ncol, ldc, c->csr.g_rowptr, c->csr.g_src, c->csr.g_coef, rho, c->d_H1, gamma, hsp);
  sec_end_on(c, SEC_FIELDS_GAMMA, s);
  sec_begin_on(c, SEC_FIELDS_DELTA, s);
  const long long tri = (long long)n * (n + 1) / 2;
  delta_gather_kernel<CPL><<<(tri + kWarpsPerBlock - 1) / kWarpsPerBlock, 32 * kWarpsPerBlock, 0, tvap::counted(s)>>>(
      n, ncol, ldc, c->csr.d_rowptr, c->csr.d_src, c->csr.d_coef, kLR, kRL, dLR, dRL);
  sec_end_on(c, SEC_FIELDS_DELTA, s);
}

}  // namespace

// below this many columns the 32-wide tiles of the dense path are mostly
// padding and the gather kernels are faster
constexpr int kDenseMinCols = 16;

int fields_batched(tvap_ctx* c, int ncol, int ldc, const double2* rho, const double2* kLR, const double2* kRL,
                   double2* gamma, double2* hsp, double2* dLR, double2* dRL, cudaStream_t s) {
  if (ncol <= 0) return TVAP_OK;
  // many gauge angles at once: dense symmetry blocks on the tensor cores
  if (c->gemm_mode >= 1 && c->csr.dense_ok && ncol >= kDenseMinCols)
    return fields_dense(c, ncol, ldc, rho, kLR, kRL, gamma, hsp, dLR, dRL, s);
  if (ncol <= 32)
    launch_fields<1>(c, ncol, ldc, rho, kLR, kRL, gamma, hsp, dLR, dRL, s);
  else if (ncol <= 64)
    launch_fields<2>(c, ncol, ldc, rho, kLR, kRL, gamma, hsp, dLR, dRL, s);
  else if (ncol <= 128)
    launch_fields<4>(c, ncol, ldc, rho, kLR, kRL, gamma, hsp, dLR, dRL, s);
  else if (ncol <= 256)
    launch_fields<8>(c, ncol, ldc, rho, kLR, kRL, gamma, hsp, dLR, dRL, s);
  else
    return TVAP_ERR_ARG;
  TVAP_CUDA(cudaGetLastError());
  return TVAP_OK;
}

}  // namespace tvap
