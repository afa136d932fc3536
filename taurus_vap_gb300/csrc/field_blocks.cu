// Gamma and Delta fields (calculate_fields, module_fields.f90:99-189) as
// dense symmetry blocks on the bf16 tensor cores.
//
// The gather operator W of a field (Gamma_x = sum_y W_xy rho_y over density
// entries y) decomposes into independent blocks: the connected components of
// its bipartite graph output entry <-> input entry.  For an m-scheme
// interaction these are the symmetry sectors of the pair (m_a - m_c,
// t_a - t_c, parity) for Gamma and (m_a + m_b, t_a + t_b, parity) for Delta,
// and the blocks are ~94 % filled, so the contraction over all gauge angles
// is a set of dense products  W_blk [rows x K] * X_blk [K x angles]  with W
// exactly the reference's FP32 coefficients.  They run as the FP64-by-integer
// splitting of ozaki_core.cuh: W is split into digit planes once, when the
// Hamiltonian is set (one exponent per output entry), the densities on every
// call (one exponent per angle column).  The blocks are found from the gather
// form itself, so any element list works; an operator that is not
// block-dense keeps the gather kernels.
//
// Layout: output rows are permuted block by block (each block padded to 32
// rows), input entries block by block (each padded to 16); digit planes of
// block b: wd[aoff_b + (s * r_pad_b + r) * kb_pad_b + k]; density planes:
// bd[((s * 2 + part) * npad + j) * ktot + k].

#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "ozaki_core.cuh"
#include "ozaki_tc.cuh"
#include "tvap_internal.cuh"

namespace tvap {

namespace {

using oz::kDigits;
using oz::kTile;

constexpr int kExpBias = -oz::kExpZero;  // stored column exponents: e + kExpBias, 0 = all-zero column

__device__ __forceinline__ int col_exp(const int* eb_enc, int j) {
  const int v = eb_enc[j];
  return v == 0 ? 0 : v - kExpBias;
}

// maximum exponent of every column j of the input (j < ncol: X0 column j;
// j >= ncol: X1 column j - ncol), over all n^2 entries
__global__ void colexp_kernel(int nent, int ncol, int ncols_tot, int ldc, const double2* __restrict__ X0,
                              const double2* __restrict__ X1, int* __restrict__ eb_enc) {
  __shared__ int red[8][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int j = blockIdx.x * 32 + lane;
  int e = oz::kExpZero;
  if (j < ncols_tot) {
    const double2* X = j < ncol ? X0 + j : X1 + (j - ncol);
    for (int p = blockIdx.y * 8 + warp; p < nent; p += gridDim.y * 8) {
      const double2 v = X[(long long)p * ldc];
      if (v.x != 0.0) e = max(e, oz::dexp(v.x));
      if (v.y != 0.0) e = max(e, oz::dexp(v.y));
    }
  }
  red[warp][lane] = e;
  __syncthreads();
  if (warp == 0) {
    for (int w = 1; w < 8; ++w) e = max(e, red[w][lane]);
    if (j < ncols_tot && e != oz::kExpZero) atomicMax(&eb_enc[j], e + kExpBias);
  }
}

// digit planes of the permuted density columns: a CTA converts a tile of 32
// input entries x 32 columns (transposed through shared memory)
constexpr int kSlPitch = kTile + 2;  // bf16 per staged row (odd word count: conflict-free)
__global__ void __launch_bounds__(256) slice_cols_kernel(int ktot, int npad, int ncol, int ncols_tot, int ldc,
                                                         const double2* __restrict__ X0,
                                                         const double2* __restrict__ X1,
                                                         const int* __restrict__ colperm,
                                                         const int* __restrict__ eb_enc,
                                                         __nv_bfloat16* __restrict__ bd) {
  __shared__ __align__(16) uint16_t sd[kDigits * 2][kTile][kSlPitch];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int k0 = blockIdx.x * kTile, j0 = blockIdx.y * kTile;
  const int j = j0 + lane;
  const int e = j < ncols_tot ? col_exp(eb_enc, j) : 0;
  for (int kl = warp; kl < kTile; kl += 8) {
    const int k = k0 + kl;
    const int p = k < ktot ? colperm[k] : -1;
    double2 v = make_double2(0.0, 0.0);
    if (p >= 0 && j < ncols_tot) v = (j < ncol ? X0[(long long)p * ldc + j] : X1[(long long)p * ldc + (j - ncol)]);
    int dr[kDigits], di[kDigits];
    oz::to_digits(oz::to_fixed(v.x, e), dr);
    oz::to_digits(oz::to_fixed(v.y, e), di);
#pragma unroll
    for (int s = 0; s < kDigits; ++s) {
      sd[2 * s][lane][kl] = oz::bf16_bits_of_int(dr[s]);
      sd[2 * s + 1][lane][kl] = oz::bf16_bits_of_int(di[s]);
    }
  }
  __syncthreads();
  // write out: 16 planes x 32 columns x 32 entries, as 4 words of 16 bytes per row
  for (int v = threadIdx.x; v < kDigits * 2 * kTile * 4; v += blockDim.x) {
    const int kv = v & 3, jl = (v >> 2) & (kTile - 1), dp = v >> 7;
    const uint32_t* row = reinterpret_cast<const uint32_t*>(&sd[dp][jl][0]);
    uint4 w;
    w.x = row[kv * 4 + 0];
    w.y = row[kv * 4 + 1];
    w.z = row[kv * 4 + 2];
    w.w = row[kv * 4 + 3];
    const int k = k0 + kv * 8;
    if (k < ktot)
      *reinterpret_cast<uint4*>(bd + ((size_t(dp) * npad + (j0 + jl)) * ktot + k)) = w;
  }
}

// One CTA per (32-row tile of a block, 32 columns).  delta = false: Gamma and
// h = Gamma + H1; delta = true: Delta^LR (columns < ncol) and Delta^RL, each
// written with its skew image.
template <bool DELTA>
__global__ void __launch_bounds__(oz::kThreads, 1)
    field_mma_kernel(int n, int ncol, int ncols_tot, int ldc, int npad, int ktot, const FieldBlockDesc* __restrict__ blocks,
                     const int2* __restrict__ tiles, const __nv_bfloat16* __restrict__ wd, const int* __restrict__ ea,
                     const int* __restrict__ rowperm, const __nv_bfloat16* __restrict__ bd,
                     const int* __restrict__ eb_enc, const double2* __restrict__ H1, double2* __restrict__ out0,
                     double2* __restrict__ out1) {
  extern __shared__ __align__(16) __nv_bfloat16 sm[];
  const int2 tile = tiles[blockIdx.y];
  const FieldBlockDesc d = blocks[tile.x];
  const int r0 = tile.y, nt0 = blockIdx.x * kTile;
  oz::Acc o;
  oz::mainloop<1, 2>(wd + d.aoff + size_t(r0) * d.kb_pad, size_t(d.r_pad) * d.kb_pad, d.kb_pad,
                     bd + size_t(nt0) * ktot + d.kbeg, size_t(npad) * ktot, ktot, d.kb_pad, sm, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wm = (warp >> 2) * 16, wn = (warp & 3) * 8;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int rr = d.row_base + r0 + wm + (lane >> 2) + ((q & 2) ? 8 : 0);
    const int j = nt0 + wn + 2 * (lane & 3) + (q & 1);
    const int p = rowperm[rr];
    if (p < 0 || j >= ncols_tot) continue;
    const double p2 = oz::pow2(ea[rr] + col_exp(eb_enc, j) - 57);
    const double2 v0 = oz::acc_value(o, q);
    const double2 v = make_double2(v0.x * p2, v0.y * p2);
    if (!DELTA) {
      out0[(long long)p * ldc + j] = v;
      out1[(long long)p * ldc + j] = cadd(v, H1[p]);
    } else {
      const int g = j < ncol ? j : j - ncol;
      double2* out = j < ncol ? out0 : out1;
      const int pt = p / n + (p % n) * n;
      out[(long long)p * ldc + g] = v;
      if (pt != p) out[(long long)pt * ldc + g] = make_double2(-v.x, -v.y);
    }
  }
}

// ---------------------------------------------------------------------------
// tcgen05 form (GEMM mode 2): per block, C_b = W_b X_b with W_b in 128-row
// tiles (planes tiled once per Hamiltonian) and X_b' = [Re X_b; Im X_b]^T
// (B' rows: the real parts of the ncols_tot columns, then the imaginary
// parts) sliced per call into 64-row tiles, on the persistent kernel of
// ozaki_tc.cuh with one k-step count per block.
// ---------------------------------------------------------------------------

// X' planes: one warp per 8-entry chunk of a block's inputs, lanes over the
// columns (coalesced reads of the angle-innermost densities).  The warps
// after the chunks write the rows without gather entries (zero field; for
// Gamma h = H1), which the products do not cover.
template <bool DELTA>
__global__ void __launch_bounds__(128)
    slice_fields_tc_kernel(int n, int ncol, int ncols_tot, int ntn, int ldc, const double2* __restrict__ X0,
                           const double2* __restrict__ X1, const int* __restrict__ colperm,
                           const FieldBlockDesc* __restrict__ blocks, const FieldTcBlock* __restrict__ tcb,
                           const int2* __restrict__ chunks, int nchunks, const int* __restrict__ empty_rows,
                           int nempty, const int* __restrict__ eb_enc, __nv_bfloat16* __restrict__ xt,
                           const double2* __restrict__ H1, double2* __restrict__ out0, double2* __restrict__ out1) {
  const int lane = threadIdx.x & 31;
  const int ch = blockIdx.x * 4 + (threadIdx.x >> 5);
  if (ch >= nchunks) {
    if (ch - nchunks >= nempty) return;
    const int p = empty_rows[ch - nchunks];
    const double2 z = make_double2(0.0, 0.0);
    if (!DELTA) {
      const double2 h = H1[p];
      for (int j = lane; j < ncols_tot; j += 32) {
        out0[(long long)p * ldc + j] = z;
        out1[(long long)p * ldc + j] = h;
      }
    } else {
      const int pt = p / n + (p % n) * n;
      for (int j = lane; j < ncols_tot; j += 32) {
        const int g = j < ncol ? j : j - ncol;
        double2* out = j < ncol ? out0 : out1;
        out[(long long)p * ldc + g] = z;
        if (pt != p) out[(long long)pt * ldc + g] = z;
      }
    }
    return;
  }
  const int2 c = chunks[ch];
  const FieldBlockDesc d = blocks[c.x];
  const FieldTcBlock q = tcb[c.x];
  const int k0 = c.y;
  int ent[8];
#pragma unroll
  for (int kk = 0; kk < 8; ++kk) ent[kk] = colperm[d.kbeg + k0 + kk];
  for (int j = lane; j < ncols_tot; j += 32) {
    const double2* X = j < ncol ? X0 : X1;
    const int jj = j < ncol ? j : j - ncol;
    const int e = col_exp(eb_enc, j);
    double2 v[8];
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) v[kk] = ent[kk] >= 0 ? X[(long long)ent[kk] * ldc + jj] : make_double2(0.0, 0.0);
#pragma unroll
    for (int part = 0; part < 2; ++part) {
      uint32_t w[kDigits][4];
#pragma unroll
      for (int kk = 0; kk < 8; kk += 2) {
        int d0[kDigits], d1[kDigits];
        oz::to_digits(oz::to_fixed(part ? v[kk].y : v[kk].x, e), d0);
        oz::to_digits(oz::to_fixed(part ? v[kk + 1].y : v[kk + 1].x, e), d1);
#pragma unroll
        for (int s = 0; s < kDigits; ++s) w[s][kk >> 1] = oz::bf16x2_of_ints(d0[s], d1[s]);
      }
      const int jr = part * ncols_tot + j;
      const size_t tb = (size_t(q.kboff) * ntn + size_t(jr / oztc::kN) * q.nks + k0 / 16) * kDigits;
      const int toff = oztc::tile_offset(jr % oztc::kN, k0 % 16);
#pragma unroll
      for (int s = 0; s < kDigits; ++s)
        *reinterpret_cast<uint4*>(xt + (tb + s) * oztc::kBTileElems + toff) =
            make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
    }
  }
}

// One persistent CTA per SM over the (block, 128-row tile, 64-column tile)
// tiles.  DELTA = false: Gamma and h = Gamma + H1; DELTA = true: Delta^LR
// (columns < ncol) and Delta^RL, each written with its skew image.  Every
// thread stores one real or imaginary part per column.
template <bool DELTA>
__global__ void __launch_bounds__(oztc::kThreads, 1)
    field_tc_kernel(int n, int ncol, int ncols_tot, int ntn, int ldc, const FieldBlockDesc* __restrict__ blocks,
                    const FieldTcBlock* __restrict__ tcb, const int2* __restrict__ bm, int nbm,
                    const __nv_bfloat16* __restrict__ wt, const __nv_bfloat16* __restrict__ xt,
                    const int* __restrict__ ea, const int* __restrict__ rowperm, const int* __restrict__ eb_enc,
                    const double2* __restrict__ H1, double2* __restrict__ out0, double2* __restrict__ out1,
                    int* counter, int* flags) {
  extern __shared__ __align__(1024) unsigned char fsm[];
  __shared__ oztc::Ctl ctl;
  const int ntiles = nbm * ntn;
  auto tile_ptrs = [&](int tile, const unsigned char*& A, const unsigned char*& B) {
    const int2 m = bm[tile / ntn];
    const int nt = tile % ntn;
    const FieldTcBlock q = tcb[m.x];
    A = reinterpret_cast<const unsigned char*>(wt) +
        (size_t(q.woff) + size_t(m.y) * q.nks * kDigits * oztc::kATileElems) * sizeof(__nv_bfloat16);
    B = reinterpret_cast<const unsigned char*>(xt) + (size_t(q.kboff) * ntn + size_t(nt) * q.nks) * size_t(oztc::kBBytes);
  };
  auto nks_of = [&](int tile) { return tcb[bm[tile / ntn].x].nks; };
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  auto store = [&](int tile, const oztc::Acc& acc) {
    const int2 m = bm[tile / ntn];
    const int nt = tile % ntn;
    const FieldBlockDesc d = blocks[m.x];
    const int i = m.y * oztc::kM + 32 * (warp & 3) + lane;
    if (i >= d.r_pad) return;
    const int rr = d.row_base + i;
    const int p = rowperm[rr];
    if (p < 0) return;
    const int eai = ea[rr] - 57;
    const int pt = p / n + (p % n) * n;
    const int col0 = nt * oztc::kN + 16 * (warp >> 2);
    double h1[2] = {0.0, 0.0};
    if (!DELTA) {
      const double2 hv = H1[p];
      h1[0] = hv.x;
      h1[1] = hv.y;
    }
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      const int jr = col0 + c;
      if (jr >= 2 * ncols_tot) break;
      const int comp = jr >= ncols_tot ? 1 : 0;
      const int j = jr - comp * ncols_tot;
      double v;
      if (!oztc::scaled(acc.h[c], acc.l[c], eai + col_exp(eb_enc, j), false, v))
        v = oztc::value(acc, c) * oz::pow2(eai + col_exp(eb_enc, j));
      if (!DELTA) {
        reinterpret_cast<double*>(out0)[((long long)p * ldc + j) * 2 + comp] = v;
        reinterpret_cast<double*>(out1)[((long long)p * ldc + j) * 2 + comp] = v + h1[comp];
      } else {
        const int g = j < ncol ? j : j - ncol;
        double* out = reinterpret_cast<double*>(j < ncol ? out0 : out1);
        out[((long long)p * ldc + g) * 2 + comp] = v;
        if (pt != p) out[((long long)pt * ldc + g) * 2 + comp] = -v;
      }
    }
  };
  if (!oztc::run_tiles<oztc::kN>(counter, ntiles, nks_of, fsm, ctl, tile_ptrs, store) && threadIdx.x == 0 && flags)
    atomicOr(flags, DEV_TC_TIMEOUT);
}

// ---------------------------------------------------------------------------
// host: blocks from the gather form
// ---------------------------------------------------------------------------
struct Dsu {
  std::vector<int> p;
  explicit Dsu(int m) : p(m) { std::iota(p.begin(), p.end(), 0); }
  int find(int x) {
    while (p[x] != x) {
      p[x] = p[p[x]];
      x = p[x];
    }
    return x;
  }
  void unite(int a, int b) {
    a = find(a);
    b = find(b);
    if (a != b) p[std::max(a, b)] = std::min(a, b);
  }
};

// rows: output entries that take part (Gamma: all; Delta: x >= y, whose
// strict-lower ones carry the entries); returns false when the operator is
// not block-dense (the gather kernels stay in use)
int build_one(int n, bool delta, const std::vector<int>& rowptr, const std::vector<int>& src,
              const std::vector<double>& coef, FieldDense* f, bool* dense) {
  *dense = false;
  const int nent = n * n;
  auto in_rows = [&](int r) { return !delta || (r % n) >= (r / n); };
  auto carries = [&](int r) { return in_rows(r) && (!delta || (r % n) > (r / n)) && rowptr[r + 1] > rowptr[r]; };
  Dsu dsu(2 * nent);
  long long nnz = 0;
  for (int r = 0; r < nent; ++r) {
    if (!carries(r)) continue;
    for (int e = rowptr[r]; e < rowptr[r + 1]; ++e) dsu.unite(r, nent + src[e]);
    nnz += rowptr[r + 1] - rowptr[r];
  }
  std::vector<int> blk_of_root(2 * nent, -1);
  std::vector<std::vector<int>> brow, bcol;
  std::vector<int> empty_rows;
  for (int r = 0; r < nent; ++r) {
    if (!in_rows(r)) continue;
    if (!carries(r)) {
      empty_rows.push_back(r);
      continue;
    }
    const int root = dsu.find(r);
    if (blk_of_root[root] < 0) {
      blk_of_root[root] = int(brow.size());
      brow.emplace_back();
      bcol.emplace_back();
    }
    brow[blk_of_root[root]].push_back(r);
  }
  std::vector<char> col_used(nent, 0);
  for (int r = 0; r < nent; ++r)
    if (carries(r))
      for (int e = rowptr[r]; e < rowptr[r + 1]; ++e) col_used[src[e]] = 1;
  std::vector<int> col_local(nent, -1);
  for (int y = 0; y < nent; ++y) {
    if (!col_used[y]) continue;
    const int b = blk_of_root[dsu.find(nent + y)];
    col_local[y] = int(bcol[b].size());
    bcol[b].push_back(y);
  }
  const int nb = int(brow.size());
  // dense size check
  std::vector<FieldBlockDesc> desc(nb + 1);
  long long dense_elems = 0, aoff = 0;
  int row_base = 0, kbeg = 0;
  for (int b = 0; b <= nb; ++b) {
    const int rows = b < nb ? int(brow[b].size()) : int(empty_rows.size());
    const int cols = b < nb ? int(bcol[b].size()) : 0;
    FieldBlockDesc& d = desc[b];
    d.r_pad = (rows + kTile - 1) / kTile * kTile;
    d.kb_pad = (cols + 15) / 16 * 16;
    d.aoff = aoff;
    d.kbeg = kbeg;
    d.row_base = row_base;
    aoff += (long long)kDigits * d.r_pad * d.kb_pad;
    dense_elems += (long long)d.r_pad * d.kb_pad;
    row_base += d.r_pad;
    kbeg += d.kb_pad;
  }
  if (nnz == 0 || dense_elems > 3 * nnz + 4096) return TVAP_OK;
  const int ktot = (kbeg + kTile - 1) / kTile * kTile;
  const int nrows = row_base;
  std::vector<uint16_t> wd(size_t(std::max<long long>(aoff, 1)), 0);
  std::vector<int> ea(nrows, 0), rowperm(nrows, -1), colperm(ktot, -1);
  std::vector<int2> tiles;
  std::vector<double> wblk;
  // tcgen05 form of the same planes
  std::vector<FieldTcBlock> tcb(nb + 1);
  long long woff = 0;
  int kboff = 0;
  for (int b = 0; b <= nb; ++b) {
    const FieldBlockDesc& d = desc[b];
    FieldTcBlock& q = tcb[b];
    const int rows = b < nb ? int(brow[b].size()) : int(empty_rows.size());
    q.mtiles = b < nb ? (rows + oztc::kM - 1) / oztc::kM : 0;  // the empty rows need no product
    q.nks = d.kb_pad / 16;
    q.kboff = kboff;
    q.pad = 0;
    q.woff = woff;
    woff += (long long)q.mtiles * q.nks * kDigits * oztc::kATileElems;
    kboff += q.nks;
  }
  std::vector<uint16_t> wt(size_t(std::max<long long>(woff, 1)), 0);
  std::vector<int2> tc_bm, tc_chunks;
  for (int b = 0; b < nb; ++b) {
    for (int mt = 0; mt < tcb[b].mtiles; ++mt) tc_bm.push_back(make_int2(b, mt));
    for (int k0 = 0; k0 < desc[b].kb_pad; k0 += 8) tc_chunks.push_back(make_int2(b, k0));
  }
  for (int b = 0; b <= nb; ++b) {
    const FieldBlockDesc& d = desc[b];
    const std::vector<int>& rows = b < nb ? brow[b] : empty_rows;
    for (size_t i = 0; i < rows.size(); ++i) rowperm[d.row_base + i] = rows[i];
    for (int r0 = 0; r0 < d.r_pad; r0 += kTile) tiles.push_back(make_int2(b, r0));
    if (b == nb) break;
    for (size_t k = 0; k < bcol[b].size(); ++k) colperm[d.kbeg + k] = bcol[b][k];
    wblk.assign(size_t(d.r_pad) * d.kb_pad, 0.0);
    for (size_t i = 0; i < rows.size(); ++i) {
      const int r = rows[i];
      for (int e = rowptr[r]; e < rowptr[r + 1]; ++e) wblk[i * d.kb_pad + col_local[src[e]]] += coef[e];
    }
    for (int i = 0; i < d.r_pad; ++i) {
      const double* wr = &wblk[size_t(i) * d.kb_pad];
      int emax = oz::kExpZero;
      for (int k = 0; k < d.kb_pad; ++k)
        if (wr[k] != 0.0) emax = std::max(emax, oz::dexp(wr[k]));
      if (emax == oz::kExpZero) emax = 0;
      ea[d.row_base + i] = emax;
      const FieldTcBlock& q = tcb[b];
      const int mt = i / oztc::kM, ri = i % oztc::kM;
      for (int k = 0; k < d.kb_pad; ++k) {
        int dg[kDigits];
        oz::to_digits(oz::to_fixed(wr[k], emax), dg);
        for (int s = 0; s < kDigits; ++s) {
          const uint16_t bits = oz::bf16_bits_of_int(dg[s]);
          wd[size_t(d.aoff) + (size_t(s) * d.r_pad + i) * d.kb_pad + k] = bits;
          if (mt < q.mtiles)
            wt[size_t(q.woff) + ((size_t(mt) * q.nks + k / 16) * kDigits + s) * oztc::kATileElems +
               oztc::tile_offset(ri, k % 16)] = bits;
        }
      }
    }
  }
  f->nblk = nb + 1;
  f->ntiles = int(tiles.size());
  f->nrows = nrows;
  f->ktot = ktot;
  TVAP_CUDA(cudaMalloc(&f->wd, sizeof(uint16_t) * wd.size()));
  TVAP_CUDA(cudaMalloc(&f->ea, sizeof(int) * nrows));
  TVAP_CUDA(cudaMalloc(&f->rowperm, sizeof(int) * nrows));
  TVAP_CUDA(cudaMalloc(&f->colperm, sizeof(int) * ktot));
  TVAP_CUDA(cudaMalloc(&f->tiles, sizeof(int2) * tiles.size()));
  TVAP_CUDA(cudaMalloc(&f->blocks, sizeof(FieldBlockDesc) * desc.size()));
  TVAP_CUDA(cudaMemcpy(f->wd, wd.data(), sizeof(uint16_t) * wd.size(), cudaMemcpyHostToDevice));
  TVAP_CUDA(cudaMemcpy(f->ea, ea.data(), sizeof(int) * nrows, cudaMemcpyHostToDevice));
  TVAP_CUDA(cudaMemcpy(f->rowperm, rowperm.data(), sizeof(int) * nrows, cudaMemcpyHostToDevice));
  TVAP_CUDA(cudaMemcpy(f->colperm, colperm.data(), sizeof(int) * ktot, cudaMemcpyHostToDevice));
  TVAP_CUDA(cudaMemcpy(f->tiles, tiles.data(), sizeof(int2) * tiles.size(), cudaMemcpyHostToDevice));
  TVAP_CUDA(cudaMemcpy(f->blocks, desc.data(), sizeof(FieldBlockDesc) * desc.size(), cudaMemcpyHostToDevice));
  TVAP_CUDA(cudaMalloc(&f->wt, sizeof(uint16_t) * wt.size()));
  TVAP_CUDA(cudaMalloc(&f->tcb, sizeof(FieldTcBlock) * tcb.size()));
  TVAP_CUDA(cudaMalloc(&f->tc_bm, sizeof(int2) * std::max<size_t>(tc_bm.size(), 1)));
  TVAP_CUDA(cudaMalloc(&f->tc_chunks, sizeof(int2) * std::max<size_t>(tc_chunks.size(), 1)));
  TVAP_CUDA(cudaMemcpy(f->wt, wt.data(), sizeof(uint16_t) * wt.size(), cudaMemcpyHostToDevice));
  TVAP_CUDA(cudaMemcpy(f->tcb, tcb.data(), sizeof(FieldTcBlock) * tcb.size(), cudaMemcpyHostToDevice));
  if (!tc_bm.empty())
    TVAP_CUDA(cudaMemcpy(f->tc_bm, tc_bm.data(), sizeof(int2) * tc_bm.size(), cudaMemcpyHostToDevice));
  if (!tc_chunks.empty())
    TVAP_CUDA(cudaMemcpy(f->tc_chunks, tc_chunks.data(), sizeof(int2) * tc_chunks.size(), cudaMemcpyHostToDevice));
  f->tc_nbm = int(tc_bm.size());
  f->tc_ksteps = kboff;
  f->tc_nchunks = int(tc_chunks.size());
  f->tc_empty_base = desc[nb].row_base;
  f->tc_nempty = int(empty_rows.size());
  *dense = true;
  return TVAP_OK;
}

int download_csr(int nrows, const int* d_rowptr, const int* d_src, const double* d_coef, long long nnz,
                 std::vector<int>& rowptr, std::vector<int>& src, std::vector<double>& coef) {
  rowptr.resize(nrows + 1);
  src.resize(std::max(1LL, nnz));
  coef.resize(std::max(1LL, nnz));
  TVAP_CUDA(cudaMemcpy(rowptr.data(), d_rowptr, sizeof(int) * (nrows + 1), cudaMemcpyDeviceToHost));
  if (nnz > 0) {
    TVAP_CUDA(cudaMemcpy(src.data(), d_src, sizeof(int) * nnz, cudaMemcpyDeviceToHost));
    TVAP_CUDA(cudaMemcpy(coef.data(), d_coef, sizeof(double) * nnz, cudaMemcpyDeviceToHost));
  }
  return TVAP_OK;
}

template <bool DELTA>
int apply_one_tc(tvap_ctx* c, const FieldDense& f, int ncol, int ldc, const double2* X0, const double2* X1,
                 double2* out0, double2* out1, cudaStream_t s) {
  const int n = c->n, nent = n * n;
  const int ncols_tot = DELTA ? 2 * ncol : ncol;
  const int ntn = (2 * ncols_tot + oztc::kN - 1) / oztc::kN;
  const int npad = (ncols_tot + 31) / 32 * 32;
  __nv_bfloat16* xt = nullptr;
  int* eb = nullptr;
  int rc;
  const size_t xt_elems = size_t(f.tc_ksteps) * ntn * kDigits * oztc::kBTileElems;
  if ((rc = oz_scratch(s, sizeof(__nv_bfloat16) * xt_elems + sizeof(int) * 64, size_t(npad), &xt, &eb))) return rc;
  // the tile counter sits after the planes (256-byte aligned: the planes are multiples of 2 KB)
  int* counter = reinterpret_cast<int*>(xt + xt_elems);
  TVAP_CUDA(cudaMemsetAsync(eb, 0, sizeof(int) * npad, s));
  TVAP_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), s));
  colexp_kernel<<<dim3(npad / 32, 64), 256, 0, tvap::counted(s)>>>(nent, ncol, ncols_tot, ldc, X0, X1, eb);
  slice_fields_tc_kernel<DELTA><<<(f.tc_nchunks + f.tc_nempty + 3) / 4, 128, 0, tvap::counted(s)>>>(
      n, ncol, ncols_tot, ntn, ldc, X0, X1, f.colperm, f.blocks, f.tcb, f.tc_chunks, f.tc_nchunks,
      f.rowperm + f.tc_empty_base, f.tc_nempty, eb, xt, c->d_H1, out0, out1);
  if ((rc = smem_opt_in((const void*)field_tc_kernel<DELTA>, oztc::kSmemBytes))) return rc;
  const int grid = std::min(f.tc_nbm * ntn, device_sms());
  field_tc_kernel<DELTA><<<grid, oztc::kThreads, oztc::kSmemBytes, tvap::counted(s)>>>(
      n, ncol, ncols_tot, ntn, ldc, f.blocks, f.tcb, f.tc_bm, f.tc_nbm, static_cast<const __nv_bfloat16*>(f.wt), xt,
      f.ea, f.rowperm, eb, c->d_H1, out0, out1, counter, g_dev_flags);
  TVAP_CUDA(cudaGetLastError());
  return TVAP_OK;
}

template <bool DELTA>
int apply_one(tvap_ctx* c, const FieldDense& f, int ncol, int ldc, const double2* X0, const double2* X1,
              double2* out0, double2* out1, cudaStream_t s) {
  if (c->gemm_mode == 2 && f.tc_nbm > 0) return apply_one_tc<DELTA>(c, f, ncol, ldc, X0, X1, out0, out1, s);
  const int n = c->n, nent = n * n;
  const int ncols_tot = DELTA ? 2 * ncol : ncol;
  const int npad = (ncols_tot + kTile - 1) / kTile * kTile;
  __nv_bfloat16* bd = nullptr;
  int* eb = nullptr;
  int rc;
  if ((rc = oz_scratch(s, sizeof(__nv_bfloat16) * size_t(kDigits) * 2 * npad * f.ktot, size_t(npad), &bd, &eb)))
    return rc;
  TVAP_CUDA(cudaMemsetAsync(eb, 0, sizeof(int) * npad, s));
  colexp_kernel<<<dim3(npad / 32, 64), 256, 0, tvap::counted(s)>>>(nent, ncol, ncols_tot, ldc, X0, X1, eb);
  slice_cols_kernel<<<dim3(f.ktot / kTile, npad / kTile), 256, 0, tvap::counted(s)>>>(f.ktot, npad, ncol, ncols_tot, ldc, X0, X1,
                                                                       f.colperm, eb, bd);
  const size_t shm = oz::Shape<1, 2>::kSmemBytes;
  if (int r = smem_opt_in((const void*)field_mma_kernel<DELTA>, shm)) return r;
  field_mma_kernel<DELTA><<<dim3(npad / kTile, f.ntiles), oz::kThreads, shm, tvap::counted(s)>>>(
      n, ncol, ncols_tot, ldc, npad, f.ktot, f.blocks, f.tiles, static_cast<const __nv_bfloat16*>(f.wd), f.ea, f.rowperm, bd, eb, c->d_H1, out0, out1);
  TVAP_CUDA(cudaGetLastError());
  return TVAP_OK;
}

}  // namespace

int build_field_dense(tvap_ctx* c) {
  free_field_dense(c->csr.dense_g);
  free_field_dense(c->csr.dense_d);
  c->csr.dense_ok = false;
  const int n = c->n, nent = n * n;
  std::vector<int> rowptr, src;
  std::vector<double> coef;
  bool dg = false, dd = false;
  int rc;
  if ((rc = download_csr(nent, c->csr.g_rowptr, c->csr.g_src, c->csr.g_coef, c->csr.g_nnz, rowptr, src, coef)))
    return rc;
  if ((rc = build_one(n, false, rowptr, src, coef, &c->csr.dense_g, &dg))) return rc;
  if ((rc = download_csr(nent, c->csr.d_rowptr, c->csr.d_src, c->csr.d_coef, c->csr.d_nnz, rowptr, src, coef)))
    return rc;
  if ((rc = build_one(n, true, rowptr, src, coef, &c->csr.dense_d, &dd))) return rc;
  c->csr.dense_ok = dg && dd;
  if (!c->csr.dense_ok) {
    free_field_dense(c->csr.dense_g);
    free_field_dense(c->csr.dense_d);
  }
  return TVAP_OK;
}

void free_field_dense(FieldDense& f) {
  cudaFree(f.wt);
  cudaFree(f.tcb);
  cudaFree(f.tc_bm);
  cudaFree(f.tc_chunks);
  cudaFree(f.wd);
  cudaFree(f.ea);
  cudaFree(f.rowperm);
  cudaFree(f.colperm);
  cudaFree(f.tiles);
  cudaFree(f.blocks);
  f = FieldDense();
}

int fields_dense(tvap_ctx* c, int ncol, int ldc, const double2* rho, const double2* kLR, const double2* kRL,
                 double2* gamma, double2* hsp, double2* dLR, double2* dRL, cudaStream_t s) {
  int rc;
  sec_begin_on(c, SEC_FIELDS_GAMMA, s);
  if ((rc = apply_one<false>(c, c->csr.dense_g, ncol, ldc, rho, rho, gamma, hsp, s))) return rc;
  sec_end_on(c, SEC_FIELDS_GAMMA, s);
  sec_begin_on(c, SEC_FIELDS_DELTA, s);
  if ((rc = apply_one<true>(c, c->csr.dense_d, ncol, ldc, kLR, kRL, dLR, dRL, s))) return rc;
  sec_end_on(c, SEC_FIELDS_DELTA, s);
  return TVAP_OK;
}

}  // namespace tvap
