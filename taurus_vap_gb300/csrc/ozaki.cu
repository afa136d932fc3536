// FP64 GEMM emulated on the bf16 tensor cores (integer splitting of the
// operands, exact FP32 group sums, integer folding; the scheme is described in
// ozaki_core.cuh).
//
// GB300's FP64 pipe delivers ~1.2 TFLOP/s while the bf16 tensor path
// (mma.sync) delivers ~600 TFLOP/s.  The product C = op(A) op(B) is rebuilt
// from the digit planes of its operands: a slicing pass writes the planes of
// A (per row of op(A)) and B (per column of op(B)) with one shared exponent
// each, then a 32 x 32-tile kernel runs the digit-pair products and forms
// alpha C + beta C_old in FP64.  Conjugation flips the imaginary plane.

#include <cuda_bf16.h>

#include <algorithm>
#include <climits>
#include <mutex>
#include <utility>

#include "ozaki_core.cuh"
#include "ozaki_tc.cuh"
#include "tvap_internal.cuh"

namespace tvap {

namespace {

using oz::kDigits;

// Slices of a strided batched operand.  rows = the output dimension of the
// operand (M for A, N for B), K the contraction dimension.  Element (r, k) of
// batch b is at p[r * sr + k * sk + b * bs].  Output layout:
//   sl[((b * kDigits + s) * parts + part) * rows_pad * kpad + r * kpad + k]  (bf16)
//   ex[b * rows_pad + r]
template <bool CPLX>
__global__ void slice_kernel(int rows, int K, int rows_pad, int kpad, const void* __restrict__ p, long long sr,
                             long long sk, long long bs, bool conj, __nv_bfloat16* __restrict__ sl,
                             int* __restrict__ ex) {
  const int lane = threadIdx.x & 31;
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int b = blockIdx.y;
  if (r >= rows_pad) return;
  constexpr int parts = CPLX ? 2 : 1;
  auto val = [&](int k, double& re, double& im) {
    re = 0.0;
    im = 0.0;
    if (r < rows && k < K) {
      const long long off = r * sr + k * sk + b * bs;
      if (CPLX) {
        const double2 v = static_cast<const double2*>(p)[off];
        re = v.x;
        im = conj ? -v.y : v.y;
      } else {
        re = static_cast<const double*>(p)[off];
      }
    }
  };
  int emax = oz::kExpZero;
  for (int k = lane; k < K; k += 32) {
    double re, im;
    val(k, re, im);
    if (re != 0.0) emax = max(emax, oz::dexp(re));
    if (CPLX && im != 0.0) emax = max(emax, oz::dexp(im));
  }
  for (int off = 16; off > 0; off >>= 1) emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, off));
  if (emax == oz::kExpZero) emax = 0;
  if (lane == 0) ex[size_t(b) * rows_pad + r] = emax;
  const size_t plane = size_t(rows_pad) * kpad;
  for (int k = lane; k < kpad; k += 32) {
    double re, im;
    val(k, re, im);
    int dr[kDigits], di[kDigits];
    oz::to_digits(oz::to_fixed(re, emax), dr);
    if (CPLX) oz::to_digits(oz::to_fixed(im, emax), di);
#pragma unroll
    for (int s = 0; s < kDigits; ++s) {
      const size_t base = ((size_t(b) * kDigits + s) * parts) * plane + size_t(r) * kpad + k;
      sl[base] = __float2bfloat16_rn(float(dr[s]));
      if (CPLX) sl[base + plane] = __float2bfloat16_rn(float(di[s]));
    }
  }
}

// One CTA per 32 x 32 output tile of one batch entry.
template <int PA, int PB>
__global__ void __launch_bounds__(oz::kThreads, 1)
    ozaki_mma_kernel(int M, int N, int mpad, int npad, int kpad, const __nv_bfloat16* __restrict__ As,
                     const int* __restrict__ ea, const __nv_bfloat16* __restrict__ Bs, const int* __restrict__ eb,
                     GemmArgs g, int a_shared, int b_shared) {
  extern __shared__ __align__(16) __nv_bfloat16 sm[];
  const int b = blockIdx.z;
  const int mt0 = blockIdx.y * oz::kTile, nt0 = blockIdx.x * oz::kTile;
  const size_t aplane = size_t(mpad) * kpad, bplane = size_t(npad) * kpad;
  oz::Acc o;
  // an operand shared by all batch entries (batch stride 0) is split once
  const int ba = a_shared ? 0 : b, bb = b_shared ? 0 : b;
  oz::mainloop<PA, PB>(As + size_t(ba) * kDigits * PA * aplane + size_t(mt0) * kpad, aplane, kpad,
                       Bs + size_t(bb) * kDigits * PB * bplane + size_t(nt0) * kpad, bplane, kpad, kpad, sm, o);
  // epilogue: scale by 2^(ea + eb - 57), alpha/beta, store
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wm = (warp >> 2) * 16, wn = (warp & 3) * 8;
  double2 alpha = g.alpha;
  if (g.alpha_vec) alpha = cmul(alpha, g.alpha_vec[b]);
  const bool cplx_out = !g.c_real;
  const bool alpha_real = alpha.y == 0.0;
  const bool beta_zero = g.beta.x == 0.0 && g.beta.y == 0.0;
  const bool beta_one = g.beta.x == 1.0 && g.beta.y == 0.0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = mt0 + wm + (lane >> 2) + ((q & 2) ? 8 : 0);
    const int j = nt0 + wn + 2 * (lane & 3) + (q & 1);
    if (i >= M || j >= N) continue;
    // the power-of-two scale is exact: folding it into alpha rounds as
    // scaling first would
    const double p2 = oz::pow2(ea[size_t(ba) * mpad + i] + eb[size_t(bb) * npad + j] - 57);
    const double2 v0 = oz::acc_value(o, q);
    const long long idx = i * g.crs + j * g.ccs + b * g.cbs;
    double2 v;
    if (alpha_real) {
      const double f = alpha.x * p2;
      v = make_double2(v0.x * f, v0.y * f);
    } else {
      v = cmul(alpha, make_double2(v0.x * p2, v0.y * p2));
    }
    if (cplx_out) {
      double2* C = static_cast<double2*>(g.C);
      if (beta_one) {
        const double2 c0 = C[idx];
        v = make_double2(v.x + c0.x, v.y + c0.y);
      } else if (!beta_zero) {
        v = cadd(v, cmul(g.beta, C[idx]));
      }
      C[idx] = v;
    } else {
      double* C = static_cast<double*>(g.C);
      double r = v.x;
      if (!beta_zero) r = fma(g.beta.x, C[idx], r);
      C[idx] = r;
    }
  }
}

template <int PA, int PB>
int launch_ozaki_mma(int M, int N, int mpad, int npad, int kpad, const __nv_bfloat16* As, const int* ea,
                     const __nv_bfloat16* Bs, const int* eb, const GemmArgs& g, cudaStream_t s) {
  const int a_shared = g.A.bs == 0 ? 1 : 0, b_shared = g.B.bs == 0 ? 1 : 0;
  const size_t shm = oz::Shape<PA, PB>::kSmemBytes;
  if (int rc = smem_opt_in((const void*)ozaki_mma_kernel<PA, PB>, shm)) return rc;
  dim3 grid(npad / oz::kTile, mpad / oz::kTile, g.batch);
  ozaki_mma_kernel<PA, PB><<<grid, oz::kThreads, shm, tvap::counted(s)>>>(M, N, mpad, npad, kpad, As, ea, Bs, eb, g, a_shared,
                                                            b_shared);
  TVAP_CUDA(cudaGetLastError());
  return TVAP_OK;
}

// ---------------------------------------------------------------------------
// tensor-memory path (ozaki_tc.cuh): real products of tiled digit planes
// ---------------------------------------------------------------------------

// Real operand X' of a product, built from a strided batched source operand X
// (element (r, k) of batch b at p[r sr + k sk + b bs]; r a row of op(A) or a
// column of op(B), k the contraction index).  Forms:
//   0  real:                        X'(r, k) = X(r, k)                      (rows x K)
//   1  complex, planes stacked:     X' = [Re X; Im X]                       (2 rows x K)
//   2  complex, real representation X' = [[Re X, -Im X], [Im X, Re X]]      (2 rows x 2 kp)
//   3  complex, planes side by side X' = [Re X, Im X]                       (rows x 2 kp)
//   4  complex, rows interleaved:   X'(2r, k) = Re X(r, k), X'(2r+1, k) = Im X(r, k)
//                                                                           (2 rows x K)
// so that A' B'^T of (2, 3) holds [Re C; Im C] of a complex x complex
// product, of (1, 0) [Re C; Im C] and of (0, 1) [Re C, Im C]; of (4, 4) the
// four real products Re/Im A x Re/Im B in 2 x 2 blocks, which the epilogue
// combines.  In forms 2 and 3 each column block is padded with zeros from K
// to kp (a multiple of 16).  Forms 2, 3 and 4 give the real and imaginary part
// of a row one exponent (so that the digits of form 4 are those of forms 2
// and 3); forms 0 and 1 give each part its own.
// nstack > 1 stacks the rows of nstack batch entries (X' row b xrows + r).
struct TcSrc {
  const void* p;
  long long sr, sk, bs;
  int rows, K, form;
  bool conj;
  int xrows, xk, nstack, kp;
  // k >= K1 comes from the second source (k - K1), scaled by scale2
  const void* p2;
  long long sr2, sk2, bs2;
  int K1;
  double scale2;
};

// Digit planes of X' in the tiled layout of ozaki_tc.cuh.  One CTA per 8
// source rows of one slot: the rows are gathered into shared memory
// (independent loads, consecutive threads on the source's contiguous index),
// one warp per row takes the exponents, then every thread converts 8
// consecutive k of one part (real or imaginary) of one row to 8 digits and
// stores one 16-byte core-matrix row per digit at each place of X' that
// holds them (twice in form 2: the imaginary block negated by its sign bits;
// once in form 4, whose left operand is half the size of form 2's).
constexpr int kSliceThreads = 256;
__global__ void __launch_bounds__(kSliceThreads) slice_tc_kernel(TcSrc x, int tile_rows, int rows_pad, int nks,
                                                                  __nv_bfloat16* __restrict__ out,
                                                                  int* __restrict__ ex) {
  // 8 rows of ldk = K | 1 elements (real sources use .x): an odd row stride,
  // so that the 8 rows read by 8 consecutive threads (one 16-byte element
  // each) fall in 8 different groups of 4 banks
  extern __shared__ double2 xs[];
  __shared__ int e_s[8][2];        // exponent of the real / imaginary part
  const int t = threadIdx.x;
  const int K = x.K, form = x.form;
  const int ldk = K | 1;
  const bool cplx = form != 0;
  const int sq0 = blockIdx.x * 8;
  const int slot = blockIdx.y;
  const int nsrc = x.nstack * x.rows;
  auto src_row = [&](int row, int& b, int& i) {
    const int sq = sq0 + row;
    b = x.nstack > 1 ? sq / x.rows : slot;
    i = x.nstack > 1 ? sq - b * x.rows : sq;
  };
  const bool k_fast = (x.sk == 1);
#pragma unroll 4
  for (int idx = t; idx < 8 * K; idx += kSliceThreads) {
    int row, k;
    if (k_fast) {
      row = idx / K;
      k = idx - row * K;
    } else {
      row = idx & 7;
      k = idx >> 3;
    }
    double2 v = make_double2(0.0, 0.0);
    if (sq0 + row < nsrc) {
      int b, i;
      src_row(row, b, i);
      const bool second = k >= x.K1;
      const long long off = second ? b * x.bs2 + i * x.sr2 + (k - x.K1) * x.sk2 : b * x.bs + i * x.sr + k * x.sk;
      const void* P = second ? x.p2 : x.p;
      if (cplx) {
        v = static_cast<const double2*>(P)[off];
        if (x.conj) v.y = -v.y;
      } else {
        v.x = static_cast<const double*>(P)[off];
      }
      if (second) {
        v.x *= x.scale2;
        v.y *= x.scale2;
      }
    }
    xs[row * ldk + k] = v;
  }
  __syncthreads();
  {
    const int w = t >> 5, lane = t & 31;
    int er = oz::kExpZero, ei = oz::kExpZero;
    for (int k = lane; k < K; k += 32) {
      const double2 v = xs[w * ldk + k];
      if (v.x != 0.0) er = max(er, oz::dexp(v.x));
      if (v.y != 0.0) ei = max(ei, oz::dexp(v.y));
    }
    for (int off = 16; off > 0; off >>= 1) {
      er = max(er, __shfl_xor_sync(0xffffffffu, er, off));
      ei = max(ei, __shfl_xor_sync(0xffffffffu, ei, off));
    }
    if (form >= 2) er = ei = max(er, ei);  // one exponent for the real and imaginary part
    if (er == oz::kExpZero) er = 0;
    if (ei == oz::kExpZero) ei = 0;
    if (lane == 0) {
      e_s[w][0] = er;
      e_s[w][1] = ei;
      if (sq0 + w < nsrc) {
        int b, i;
        src_row(w, b, i);
        const size_t qtop = size_t(x.nstack > 1 ? b * x.xrows : 0) + (form == 4 ? 2 * i : i);
        ex[size_t(slot) * rows_pad + qtop] = er;
        if (form == 1 || form == 2) ex[size_t(slot) * rows_pad + qtop + x.rows] = ei;
        if (form == 4) ex[size_t(slot) * rows_pad + qtop + 1] = ei;
      }
    }
  }
  __syncthreads();
  // work items: (row, chunk of 8 k, part), rows fastest so that a half-warp
  // writes whole 256-byte core-matrix row groups
  const int nchunk = (form == 2 || form == 3) ? x.kp / 8 : nks * 2;
  const int nparts = cplx ? 2 : 1;
  const int tiles = rows_pad / tile_rows;
  const size_t tile_elems = size_t(tile_rows) * 16;
  for (int item = t; item < 8 * nchunk * nparts; item += kSliceThreads) {
    const int row = item & 7;
    const int c = (item >> 3) % nchunk, part = (item >> 3) / nchunk;
    if (sq0 + row >= nsrc) continue;
    int b, i;
    src_row(row, b, i);
    const int qtop = (x.nstack > 1 ? b * x.xrows : 0) + (form == 4 ? 2 * i : i);
    const int emax = e_s[row][part];
    const int k0 = 8 * c;
    uint32_t w[kDigits][4];
#pragma unroll
    for (int j = 0; j < 8; j += 2) {
      int d0[kDigits], d1[kDigits];
      const double2 v0 = (k0 + j < K) ? xs[row * ldk + k0 + j] : make_double2(0.0, 0.0);
      const double2 v1 = (k0 + j + 1 < K) ? xs[row * ldk + k0 + j + 1] : make_double2(0.0, 0.0);
      oz::to_digits(oz::to_fixed(part ? v0.y : v0.x, emax), d0);
      oz::to_digits(oz::to_fixed(part ? v1.y : v1.x, emax), d1);
#pragma unroll
      for (int s = 0; s < kDigits; ++s) w[s][j >> 1] = oz::bf16x2_of_ints(d0[s], d1[s]);
    }
    auto put = [&](int q, int kq, uint32_t flip) {
      const size_t tb = (size_t(slot) * tiles + q / tile_rows) * nks + (kq >> 4);
      const int toff = oztc::tile_offset(q % tile_rows, kq);
#pragma unroll
      for (int s = 0; s < kDigits; ++s) {
        __nv_bfloat16* dst = out + (tb * kDigits + s) * tile_elems + toff;
        *reinterpret_cast<uint4*>(dst) = make_uint4(w[s][0] ^ flip, w[s][1] ^ flip, w[s][2] ^ flip, w[s][3] ^ flip);
      }
    };
    switch (form) {
      case 0: put(qtop, k0, 0u); break;
      case 1: put(part ? qtop + x.rows : qtop, k0, 0u); break;
      case 2:
        if (part == 0) {
          put(qtop, k0, 0u);
          put(qtop + x.rows, x.kp + k0, 0u);
        } else {
          put(qtop + x.rows, k0, 0u);
          put(qtop, x.kp + k0, 0x80008000u);
        }
        break;
      case 3: put(qtop, part ? x.kp + k0 : k0, 0u); break;
      default: put(qtop + part, k0, 0u); break;
    }
  }
}

// Output mapping of the tensor-memory product: row q of A' (slot z) and row
// col of B' hold component comp = (r >= a_split) + (col >= b_split) of
// C(i, j) of batch entry b; alpha and beta are real.  In the paired form
// (both operands sliced in form 4) rows 2i, 2i + 1 of A' and 2j, 2j + 1 of B'
// are the real and imaginary parts of row i of op(A) and column j of op(B).
struct TcOut {
  void* C;
  long long crs, ccs, cbs;
  bool c_real;
  double alpha, beta;
  int a_rows, a_split, b_rows, b_split, nstack;
};

// Persistent CTAs over the (128 x 64 tile of A' B'^T, slot) tiles, claimed in
// order from *counter; tile numbers run over the N tiles fastest, then the M
// tiles, then the slots, so that the CTAs working at one time share their A
// and B tiles through L2.  PAIRS: the paired form, whose 2 x 2 blocks
// P(2i .. 2i+1, 2j .. 2j+1) give Re C(i, j) = P(2i, 2j) - P(2i+1, 2j+1) and
// Im C(i, j) = P(2i+1, 2j) + P(2i, 2j+1): the two rows of a block are adjacent
// TMEM lanes (one shuffle per column pair), its two columns adjacent
// accumulator columns of one thread.  The four products of a block share one
// exponent (rows and columns: one per real/imaginary pair), so the
// combination is exact on the integer accumulators and the result is, bit
// for bit, that of the real representation [[Re, -Im], [Im, Re]] x [Re, Im].
template <bool UNIT, int BN, bool PAIRS>
__global__ void __launch_bounds__(oztc::kThreads, 1)
    ozaki_tc_kernel(const __nv_bfloat16* __restrict__ As, const int* __restrict__ ea, int a_rows_pad,
                    const __nv_bfloat16* __restrict__ Bs, const int* __restrict__ eb, int b_rows_pad, int b_shared,
                    int nslots, int nks, TcOut o, int* counter, int* flags) {
  extern __shared__ __align__(1024) unsigned char tsm[];
  __shared__ oztc::Ctl ctl;
  const int a_tiles = a_rows_pad / oztc::kM, b_tiles = b_rows_pad / BN;
  const int ntiles = a_tiles * b_tiles * nslots;
  auto tile_ptrs = [&](int tile, const unsigned char*& A, const unsigned char*& B) {
    const int nt = tile % b_tiles, rest = tile / b_tiles;
    const int mt = rest % a_tiles, z = rest / a_tiles;
    const int bz = b_shared ? 0 : z;
    A = reinterpret_cast<const unsigned char*>(As) + (size_t(z) * a_tiles + mt) * nks * size_t(oztc::kABytes);
    B = reinterpret_cast<const unsigned char*>(Bs) + (size_t(bz) * b_tiles + nt) * nks * size_t(oztc::b_bytes(BN));
  };
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // The stores of a tile overlap the MMAs of the next one: exponents, values
  // and (with beta) the old outputs are fetched with independent loads, all
  // issued before the first store (C is not known not to alias them).
  auto store = [&](int tile, const oztc::Acc& acc) {
    const int nt = tile % b_tiles, rest = tile / b_tiles;
    const int mt = rest % a_tiles, z = rest / a_tiles;
    const int bz = b_shared ? 0 : z;
    const int q = mt * oztc::kM + 32 * (warp & 3) + lane;
    if constexpr (BN < 64) {
      if (16 * (warp >> 2) >= BN) return;  // these warps' columns belong to the next tile
    }
    // a row pair lies within the rows of A' or beyond them (a_rows is even):
    // the paired form returns after its shuffles, which the whole warp takes
    const bool row_ok = q < o.nstack * o.a_rows;
    if (!PAIRS && !row_ok) return;
    const int b = o.nstack > 1 ? q / o.a_rows : z;
    int i = o.nstack > 1 ? q - b * o.a_rows : q;
    int comp_a = 0;
    if (PAIRS) {
      comp_a = i & 1;
      i >>= 1;
    } else if (i >= o.a_split) {
      i -= o.a_split;
      comp_a = 1;
    }
    const int eai = (row_ok ? ea[size_t(z) * a_rows_pad + q] : 0) - 57;
    double* __restrict__ C = static_cast<double*>(o.C);
    const int cw = o.c_real ? 1 : 2;  // doubles per element
    const int col0 = nt * BN + 16 * (warp >> 2);
    const int* __restrict__ ebz = eb + size_t(bz) * b_rows_pad;
    // element index of column c, or -1 (padding, or the imaginary part of a
    // real output)
    auto idx_of = [&](int c) -> long long {
      const int col = col0 + c;
      int j = col, comp = comp_a;
      if (j >= o.b_split) {
        j -= o.b_split;
        comp += 1;
      }
      if (col >= o.b_rows || (comp > 0 && o.c_real)) return -1;
      return (i * o.crs + j * o.ccs + b * o.cbs) * cw + comp;
    };
    // UNIT: alpha = +-1 (every product of the path), a sign of the integer
    // conversion; otherwise one product more (a separate instantiation, so
    // that no FP64 multiply is predicated into the common case)
    const bool neg = o.alpha < 0.0;
    if constexpr (PAIRS) {
      // even lane (real row): P(2i, 2j) - P(2i+1, 2j+1); odd lane (imaginary
      // row): P(2i+1, 2j) + P(2i, 2j+1).  Both take the partner's odd column.
      long long hs[8], ls[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const long long th = __shfl_xor_sync(0xffffffffu, acc.h[2 * c + 1], 1);
        const long long tl = __shfl_xor_sync(0xffffffffu, acc.l[2 * c + 1], 1);
        hs[c] = comp_a ? acc.h[2 * c] + th : acc.h[2 * c] - th;
        ls[c] = comp_a ? acc.l[2 * c] + tl : acc.l[2 * c] - tl;
      }
      if (!row_ok || (comp_a && o.c_real)) return;
      const int j0 = col0 >> 1;
      double w[8];
      long long k[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const bool in = col0 + 2 * c < o.b_rows;
        const int e = in ? ebz[col0 + 2 * c] : 0;
        double x;
        if (oztc::scaled(hs[c], ls[c], eai + e, UNIT && neg, x))
          w[c] = UNIT ? x : x * o.alpha;
        else
          w[c] = fma(double(hs[c]), 0x1p28, double(ls[c])) * (o.alpha * oz::pow2(eai + e));
        k[c] = in ? (i * o.crs + (j0 + c) * o.ccs + b * o.cbs) * cw + comp_a : -1;
      }
      if (o.beta != 0.0) {
        double old[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) old[c] = k[c] >= 0 ? C[k[c]] : 0.0;
#pragma unroll
        for (int c = 0; c < 8; ++c) w[c] = fma(o.beta, old[c], w[c]);
      }
#pragma unroll
      for (int c = 0; c < 8; ++c)
        if (k[c] >= 0) C[k[c]] = w[c];
      return;
    }
    double v[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      const int e = (col0 + c < o.b_rows) ? ebz[col0 + c] : 0;
      double x;
      if (oztc::scaled(acc.h[c], acc.l[c], eai + e, UNIT && neg, x))
        v[c] = UNIT ? x : x * o.alpha;
      else
        v[c] = oztc::value(acc, c) * (o.alpha * oz::pow2(eai + e));
    }
    // two groups of 8: the loads of a group are in flight together
#pragma unroll
    for (int c0 = 0; c0 < 16; c0 += 8) {
      if (o.beta != 0.0) {
        double old[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          const long long k = idx_of(c0 + c);
          old[c] = k >= 0 ? C[k] : 0.0;
        }
#pragma unroll
        for (int c = 0; c < 8; ++c) v[c0 + c] = fma(o.beta, old[c], v[c0 + c]);
      }
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const long long k = idx_of(c0 + c);
        if (k >= 0) C[k] = v[c0 + c];
      }
    }
  };
  auto nks_of = [nks](int) { return nks; };
  if (!oztc::run_tiles<BN>(counter, ntiles, nks_of, tsm, ctl, tile_ptrs, store) && threadIdx.x == 0 && flags)
    atomicOr(flags, DEV_TC_TIMEOUT);
}

// the left operand whose digit planes (at the start of buf) and exponents
// (at the start of ex) the last tcgen05 product left
struct LeftSlice {
  bool valid = false;
  const void* p = nullptr;
  const void* p2 = nullptr;
  long long sr = 0, sk = 0, bs = 0, sr2 = 0, sk2 = 0, bs2 = 0;
  int rows = 0, K = 0, K1 = 0, form = 0, conj = 0, xrows = 0, xk = 0, kp = 0, nstack = 0, slots = 0, rows_pad = 0,
      nks = 0;
  double scale2 = 0.0;
  bool operator==(const LeftSlice& o) const {
    return valid && o.valid && p == o.p && p2 == o.p2 && sr == o.sr && sk == o.sk && bs == o.bs && sr2 == o.sr2 &&
           sk2 == o.sk2 && bs2 == o.bs2 && rows == o.rows && K == o.K && K1 == o.K1 && form == o.form &&
           conj == o.conj && xrows == o.xrows && xk == o.xk && kp == o.kp && nstack == o.nstack && slots == o.slots &&
           rows_pad == o.rows_pad && nks == o.nks && scale2 == o.scale2;
  }
};

struct OzScratch {
  cudaStream_t stream = nullptr;
  __nv_bfloat16* buf = nullptr;
  size_t bytes = 0;
  int* ex = nullptr;
  size_t ex_count = 0;
  int* counter = nullptr;  // tile counter of the tcgen05 kernel
  LeftSlice left;          // what buf / ex hold at their start
};
constexpr int kMaxScratch = 192;  // streams with scratch at once (seven per context)
OzScratch g_oz[kMaxScratch];
std::mutex g_oz_mutex;

int oz_reserve(cudaStream_t s, size_t bytes, size_t ex_count, OzScratch** out) {
  std::lock_guard<std::mutex> lock(g_oz_mutex);
  OzScratch* sc = nullptr;
  for (auto& e : g_oz)
    if (e.buf && e.stream == s) sc = &e;
  if (!sc)
    for (auto& e : g_oz)
      if (!e.buf) {
        sc = &e;
        sc->stream = s;
        break;
      }
  if (!sc) {
    set_last_error("too many streams use the emulated GEMM", __FILE__, __LINE__);
    return TVAP_ERR_ARG;
  }
  if (!sc->counter) TVAP_CUDA(cudaMalloc(&sc->counter, sizeof(int)));
  if (bytes > sc->bytes) {
    if (sc->buf) {
      cudaStreamSynchronize(s);
      cudaFree(sc->buf);
    }
    sc->buf = nullptr;
    TVAP_CUDA(cudaMalloc(&sc->buf, bytes));
    sc->bytes = bytes;
    sc->left.valid = false;
  }
  if (ex_count > sc->ex_count) {
    if (sc->ex) {
      cudaStreamSynchronize(s);
      cudaFree(sc->ex);
    }
    sc->ex = nullptr;
    TVAP_CUDA(cudaMalloc(&sc->ex, ex_count * sizeof(int)));
    sc->ex_count = ex_count;
    sc->left.valid = false;
  }
  *out = sc;
  return TVAP_OK;
}

}  // namespace

int oz_scratch(cudaStream_t s, size_t bytes, size_t ex_count, __nv_bfloat16** buf, int** ex) {
  OzScratch* sc = nullptr;
  int rc;
  if ((rc = oz_reserve(s, bytes, ex_count, &sc))) return rc;
  sc->left.valid = false;  // the caller overwrites the planes
  *buf = sc->buf;
  *ex = sc->ex;
  return TVAP_OK;
}

// Frees the slice scratch of a stream (called when a context destroys or
// replaces the stream).
void oz_release(cudaStream_t s) {
  std::lock_guard<std::mutex> lock(g_oz_mutex);
  for (auto& e : g_oz)
    if (e.buf && e.stream == s) {
      cudaStreamSynchronize(s);
      cudaFree(e.buf);
      cudaFree(e.ex);
      cudaFree(e.counter);
      e = OzScratch();
    }
}

namespace {

constexpr int kTcMinTiles = 152;

inline bool g_alpha_unit(double a) { return a == 1.0 || a == -1.0; }

// The tensor-memory path for one product (mode 2).  Returns TVAP_ERR_ARG
// without launching anything when the product is not of a supported kind.
// With upper_only the whole product is formed (the lower triangle is
// written too; its readers ignore it).
int gemm_tc(const GemmArgs& g, cudaStream_t s) {
  const bool real_scalars = g.alpha.y == 0.0 && g.beta.y == 0.0 && !g.alpha_vec;
  if (!real_scalars || (g.a_real && g.b_real && !g.c_real)) return TVAP_ERR_ARG;
  const bool a_sh = g.A.bs == 0 && g.batch > 1, b_sh = g.B.bs == 0 && g.batch > 1;
  if (a_sh && b_sh) return TVAP_ERR_ARG;
  // rows of op(A): element (i, k) at A.p[i rs + k cs]; rows of op(B)^T:
  // element (j, k) at B.p[k rs + j cs].  With a shared A the transposed
  // product C^T = op(B)^T op(A)^T is formed, so that the per-batch operand is
  // always the left one and can be stacked along the rows.
  struct Side {
    const void* p;
    long long sr, sk, bs;
    int rows;
    bool real, conj;
    const void* p2;
    long long sr2, sk2, bs2;
  };
  if (g.K2 > 0 && ((g.A2.bs == 0) != (g.A.bs == 0) || (g.B2.bs == 0) != (g.B.bs == 0))) return TVAP_ERR_ARG;
  Side L{g.A.p, g.A.rs, g.A.cs, g.A.bs, g.M, g.a_real, g.conj_a, g.A2.p, g.A2.rs, g.A2.cs, g.A2.bs};
  Side R{g.B.p, g.B.cs, g.B.rs, g.B.bs, g.N, g.b_real, g.conj_b, g.B2.p, g.B2.cs, g.B2.rs, g.B2.bs};
  long long crs = g.crs, ccs = g.ccs;
  if (a_sh) {
    std::swap(L, R);
    std::swap(crs, ccs);
  }
  // the second term (K2 > 0) continues the contraction: k >= g.K reads A2 /
  // B2, the B side scaled by s2
  const int K = g.K + (g.K2 > 0 ? g.K2 : 0), kp = (K + 15) / 16 * 16;
  const int K1 = g.K2 > 0 ? g.K : K;
  const bool scale_left = a_sh;  // after the swap the B side is on the left
  TcSrc xa{L.p, L.sr, L.sk, L.bs, L.rows, K, 0, L.conj, L.rows, K, 1, K, L.p2, L.sr2, L.sk2, L.bs2, K1,
           scale_left ? g.s2 : 1.0};
  TcSrc xb{R.p, R.sr, R.sk, R.bs, R.rows, K, 0, R.conj, R.rows, K, 1, K, R.p2, R.sr2, R.sk2, R.bs2, K1,
           scale_left ? 1.0 : g.s2};
  TcOut o{};
  o.a_split = o.b_split = INT_MAX;
  const bool stack = g.batch > 1 && (a_sh || b_sh);
  // complex x complex: the paired form (rows interleaved on both sides, the
  // 2 x 2 blocks combined by the epilogue; half the left operand's digit
  // planes, twice the tiles of half the k-steps, so that it pays where the
  // contraction is long; batches with a shared operand keep the real
  // representation) or the real representation
  const bool pairs = !L.real && !R.real && !stack && g_tc_pairs_min_k > 0 && K >= g_tc_pairs_min_k;
  if (pairs) {
    xa.form = xb.form = 4;
    xa.xrows = 2 * L.rows;
    xb.xrows = 2 * R.rows;
  } else if (!L.real && !R.real) {
    xa.form = 2;
    xa.xrows = 2 * L.rows;
    xa.xk = 2 * kp;
    xa.kp = kp;
    xb.form = 3;
    xb.xk = 2 * kp;
    xb.kp = kp;
    o.a_split = L.rows;
  } else if (!L.real) {
    xa.form = 1;
    xa.xrows = 2 * L.rows;
    o.a_split = L.rows;
  } else if (!R.real) {
    xb.form = 1;
    xb.xrows = 2 * R.rows;
    o.b_split = R.rows;
  }
  xa.nstack = stack ? g.batch : 1;
  const int a_slots = stack ? 1 : g.batch, b_slots = stack ? 1 : g.batch;
  const int a_rows_pad = (xa.nstack * xa.xrows + oztc::kM - 1) / oztc::kM * oztc::kM;
  // B' tiles of 48 or 64 rows, whichever pads the output columns less (140
  // columns: 144 instead of 192)
  const int pad48 = (xb.xrows + 47) / 48 * 48, pad64 = (xb.xrows + 63) / 64 * 64;
  const int bn = g_tc_bn_policy == 1 ? 64 : g_tc_bn_policy == 2 ? 48 : (pad48 < pad64 ? 48 : 64);
  const int b_rows_pad = bn == 48 ? pad48 : pad64;
  const int nks = (xa.xk + 15) / 16;
  const size_t asz = size_t(a_slots) * (a_rows_pad / oztc::kM) * nks * (oztc::kABytes / 2);
  const size_t bsz = size_t(b_slots) * (b_rows_pad / bn) * nks * (oztc::b_bytes(bn) / 2);
  // products of few tiles (the single small products of the canonical basis
  // and the evolution) are latency-bound: the 32 x 32 mma.sync tiles spread
  // them over more SMs.  The paired form has twice the tiles of half the
  // k-steps; it is counted in tiles of the real representation, so that both
  // forms route the same products here.
  if (size_t(a_rows_pad / oztc::kM) * (b_rows_pad / bn) * a_slots / (pairs ? 2 : 1) < size_t(kTcMinTiles))
    return TVAP_ERR_ARG;
  int rc;
  OzScratch* sc = nullptr;
  if ((rc = oz_reserve(s, sizeof(__nv_bfloat16) * (asz + bsz), size_t(a_slots) * a_rows_pad +
                                                                   size_t(b_slots) * b_rows_pad, &sc)))
    return rc;
  __nv_bfloat16* As = sc->buf;
  __nv_bfloat16* Bs = sc->buf + asz;
  int* ea = sc->ex;
  int* eb = sc->ex + size_t(a_slots) * a_rows_pad;
  const size_t slice_shm = sizeof(double2) * 8 * size_t(K | 1);  // slice_tc_kernel's padded rows
  if (slice_shm > 48 * 1024) {
    if (slice_shm > size_t(227) * 1024) return TVAP_ERR_ARG;
    if ((rc = smem_opt_in((const void*)slice_tc_kernel, slice_shm))) return rc;
  }
  LeftSlice left;
  left.valid = true;
  left.p = xa.p;
  left.p2 = xa.p2;
  left.sr = xa.sr;
  left.sk = xa.sk;
  left.bs = xa.bs;
  left.sr2 = xa.sr2;
  left.sk2 = xa.sk2;
  left.bs2 = xa.bs2;
  left.rows = xa.rows;
  left.K = xa.K;
  left.K1 = xa.K1;
  left.form = xa.form;
  left.conj = xa.conj ? 1 : 0;
  left.xrows = xa.xrows;
  left.xk = xa.xk;
  left.kp = xa.kp;
  left.nstack = xa.nstack;
  left.slots = a_slots;
  left.rows_pad = a_rows_pad;
  left.nks = nks;
  left.scale2 = xa.scale2;
  if (!(g.reuse_left && sc->left == left)) {
    slice_tc_kernel<<<dim3((xa.nstack * xa.rows + 7) / 8, a_slots), kSliceThreads, slice_shm, tvap::counted(s)>>>(
        xa, oztc::kM, a_rows_pad, nks, As, ea);
    sc->left = left;
  }
  slice_tc_kernel<<<dim3((xb.rows + 7) / 8, b_slots), kSliceThreads, slice_shm, tvap::counted(s)>>>(xb, bn, b_rows_pad, nks, Bs,
                                                                                     eb);
  o.C = g.C;
  o.crs = crs;
  o.ccs = ccs;
  o.cbs = g.cbs;
  o.c_real = g.c_real;
  o.alpha = g.alpha.x;
  o.beta = g.beta.x;
  o.a_rows = xa.xrows;
  o.b_rows = xb.xrows;
  o.nstack = xa.nstack;
  const int sms = device_sms();
  const long long ntiles = (long long)(a_rows_pad / oztc::kM) * (b_rows_pad / bn) * a_slots;
  const int grid = int(std::min<long long>(ntiles, g_tc_grid_cap > 0 ? std::min(sms, g_tc_grid_cap) : sms));
  // the instantiation: alpha = +-1 (a sign in the integer conversion) or
  // general, the B' tile width and the paired form
  const bool unit_alpha = g_alpha_unit(o.alpha);
  auto kern = pairs ? (unit_alpha ? (bn == 48 ? ozaki_tc_kernel<true, 48, true> : ozaki_tc_kernel<true, 64, true>)
                                  : (bn == 48 ? ozaki_tc_kernel<false, 48, true> : ozaki_tc_kernel<false, 64, true>))
                    : (unit_alpha ? (bn == 48 ? ozaki_tc_kernel<true, 48, false> : ozaki_tc_kernel<true, 64, false>)
                                  : (bn == 48 ? ozaki_tc_kernel<false, 48, false> : ozaki_tc_kernel<false, 64, false>));
  if ((rc = smem_opt_in((const void*)kern, oztc::kSmemBytes))) return rc;
  TVAP_CUDA(cudaMemsetAsync(sc->counter, 0, sizeof(int), s));
  if (g_tc_timing_ctx) sec_begin_on(g_tc_timing_ctx, g_tc_timing_sec, s);
  kern<<<grid, oztc::kThreads, oztc::kSmemBytes, tvap::counted(s)>>>(As, ea, a_rows_pad, Bs, eb, b_rows_pad, b_slots == 1 ? 1 : 0,
                                                      a_slots, nks, o, sc->counter, g_dev_flags);
  if (g_tc_timing_ctx) sec_end_on(g_tc_timing_ctx, g_tc_timing_sec, s);
  TVAP_CUDA(cudaGetLastError());
  return TVAP_OK;
}

}  // namespace

// Returns TVAP_OK after launching, or TVAP_ERR_ARG when the shape is not
// supported (the caller then uses the FP64 pipe).
int gemm_ozaki(const GemmArgs& g, cudaStream_t s) {
  if (g.M <= 0 || g.N <= 0 || g.K <= 0 || g.batch <= 0) return TVAP_OK;
  if (g_gemm_mode == 2 && gemm_tc(g, s) == TVAP_OK) return TVAP_OK;
  if (g.K2 > 0) return gemm_split_k2(g, s);
  const int PA = g.a_real ? 1 : 2, PB = g.b_real ? 1 : 2;
  const int mpad = (g.M + 31) / 32 * 32, npad = (g.N + 31) / 32 * 32, kpad = (g.K + 15) / 16 * 16;
  // operands with batch stride 0 are split once for the whole batch
  const int abatch = g.A.bs == 0 ? 1 : g.batch, bbatch = g.B.bs == 0 ? 1 : g.batch;
  const size_t asz = size_t(abatch) * kDigits * PA * mpad * kpad;
  const size_t bsz = size_t(bbatch) * kDigits * PB * npad * kpad;
  int rc;
  OzScratch* sc = nullptr;
  if ((rc = oz_reserve(s, sizeof(__nv_bfloat16) * (asz + bsz), size_t(abatch) * mpad + size_t(bbatch) * npad, &sc)))
    return rc;
  sc->left.valid = false;  // the mma.sync planes overwrite the tcgen05 ones
  __nv_bfloat16* As = sc->buf;
  __nv_bfloat16* Bs = sc->buf + asz;
  int* ea = sc->ex;
  int* eb = sc->ex + size_t(abatch) * mpad;
  // A rows: element (i, k) at A.p[i rs + k cs]; B columns: element (j, k) = B(k, j) at B.p[k rs + j cs]
  {
    dim3 grid((mpad + 7) / 8, abatch);
    if (PA == 2)
      slice_kernel<true><<<grid, 256, 0, tvap::counted(s)>>>(g.M, g.K, mpad, kpad, g.A.p, g.A.rs, g.A.cs, g.A.bs, g.conj_a, As, ea);
    else
      slice_kernel<false><<<grid, 256, 0, tvap::counted(s)>>>(g.M, g.K, mpad, kpad, g.A.p, g.A.rs, g.A.cs, g.A.bs, false, As, ea);
  }
  {
    dim3 grid((npad + 7) / 8, bbatch);
    if (PB == 2)
      slice_kernel<true><<<grid, 256, 0, tvap::counted(s)>>>(g.N, g.K, npad, kpad, g.B.p, g.B.cs, g.B.rs, g.B.bs, g.conj_b, Bs, eb);
    else
      slice_kernel<false><<<grid, 256, 0, tvap::counted(s)>>>(g.N, g.K, npad, kpad, g.B.p, g.B.cs, g.B.rs, g.B.bs, false, Bs, eb);
  }
  if (PA == 2 && PB == 2) return launch_ozaki_mma<2, 2>(g.M, g.N, mpad, npad, kpad, As, ea, Bs, eb, g, s);
  if (PA == 2) return launch_ozaki_mma<2, 1>(g.M, g.N, mpad, npad, kpad, As, ea, Bs, eb, g, s);
  if (PB == 2) return launch_ozaki_mma<1, 2>(g.M, g.N, mpad, npad, kpad, As, ea, Bs, eb, g, s);
  return launch_ozaki_mma<1, 1>(g.M, g.N, mpad, npad, kpad, As, ea, Bs, eb, g, s);
}

}  // namespace tvap
