// Internal declarations of the sm_103a device path (not part of the C ABI).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <vector>

#include "tvap.h"

namespace tvap {

// ---------------------------------------------------------------------------
// complex helpers (double2 = re, im)
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ double2 cmk(double r, double i) { return make_double2(r, i); }
__host__ __device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__host__ __device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ double2 cneg(double2 a) { return make_double2(-a.x, -a.y); }
// c += a * b
__device__ __forceinline__ void cfma(double2& c, double2 a, double2 b) {
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(-a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y);
  c.y = fma(a.y, b.x, c.y);
}
// 1/z with scaling (Smith)
__host__ __device__ __forceinline__ double2 crcp(double2 z) {
  if (fabs(z.x) >= fabs(z.y)) {
    const double r = z.y / z.x, d = z.x + z.y * r;
    return make_double2(1.0 / d, -r / d);
  } else {
    const double r = z.x / z.y, d = z.y + z.x * r;
    return make_double2(r / d, -1.0 / d);
  }
}
__host__ __device__ __forceinline__ double2 cdiv(double2 a, double2 b) { return cmul(a, crcp(b)); }
#ifdef __CUDACC__
// Helpers of the Newton seeds on the integer pipe (an FP64 instruction, a
// compare or a conversion included, holds its SM sub-partition's FP64 unit
// for about 64 cycles on this part, and the seeds sit on dependent chains):
// d > 0 with 2^-99 <= d < 2^100 (normal, within the FP32 exponent range
// with room), its float value with the mantissa truncated to 23 bits, and
// the double of a positive normal float, all from the bits.
__device__ __forceinline__ bool seed_range(double d) {
  const long long b = __double_as_longlong(d);
  const int e = int((b >> 52) & 0x7ff);  // biased exponent; sign bit set: b < 0
  return b > 0 && e >= 1023 - 99 && e <= 1023 + 99;
}
__device__ __forceinline__ float seed_f32(double d) {
  const long long b = __double_as_longlong(d);
  const unsigned e = unsigned(int((b >> 52) & 0x7ff) - 1023 + 127);
  return __uint_as_float((e << 23) | unsigned((b >> 29) & 0x7fffff));
}
__device__ __forceinline__ double seed_f64(float f) {
  const unsigned u = __float_as_uint(f);
  const long long e = (long long)((u >> 23) & 0xff) - 127 + 1023;
  return __longlong_as_double((e << 52) | ((long long)(u & 0x7fffff) << 29));
}
// 1/z = conj(z) / |z|^2 with |z|^2 inverted by two Newton steps from the
// single-precision reciprocal of its truncated value (22 bits or more, 88
// after the steps: relative error a few units of the last place); outside
// the range of seed_range the scaled division (crcp)
__device__ __forceinline__ double2 crcp_newton(double2 z) {
  const double d = fma(z.x, z.x, z.y * z.y);
  if (!seed_range(d)) return crcp(z);
  double y = seed_f64(__frcp_rn(seed_f32(d)));
  double e = fma(-d, y, 1.0);
  y = fma(y, e, y);
  e = fma(-d, y, 1.0);
  y = fma(y, e, y);
  return make_double2(z.x * y, -z.y * y);
}
#endif
__host__ __device__ __forceinline__ double cabs1(double2 a) { return fabs(a.x) + fabs(a.y); }

// ---------------------------------------------------------------------------
// error handling
// ---------------------------------------------------------------------------
#define TVAP_CUDA(call)                                                                        \
  do {                                                                                         \
    cudaError_t e__ = (call);                                                                  \
    if (e__ != cudaSuccess) {                                                                  \
      tvap::set_last_error(cudaGetErrorString(e__), __FILE__, __LINE__);                       \
      return TVAP_ERR_CUDA;                                                                    \
    }                                                                                          \
  } while (0)

void set_last_error(const char* msg, const char* file, int line);
// Raises a kernel's dynamic shared-memory limit to at least `bytes` on the
// current device (cudaFuncSetAttribute acts per device); once per device and
// kernel, under a lock, so contexts on several threads and devices may call it.
int smem_opt_in(const void* func, size_t bytes);
// Streaming multiprocessors of the current device (cached per device).
int device_sms();
// Kernels this thread launched since its current C-ABI call began.  Every
// launch passes its stream through counted(); the launches that do not take
// a stream argument count themselves.
extern thread_local long long g_launch_count;
inline cudaStream_t counted(cudaStream_t s) {
  ++g_launch_count;
  return s;
}

// device status word bits, written by kernels and read back by the host
enum DevFlag : int {
  DEV_SINGULAR_UPHI = 1,
  DEV_SINGULAR_RN = 2,
  DEV_PFAFF_ZERO = 4,
  DEV_CANON_BLOCK = 8,
  DEV_EIGEN_NOCONV = 16,
  DEV_CHOLESKY = 32,
  DEV_TRTRI = 64,
  DEV_IMAG_GRAD = 128,
  DEV_TC_TIMEOUT = 256,  // a bounded device wait gave up (tensor-core pipeline, grid barrier)
  DEV_WAIT_TIMEOUT = 256,
};

// ---------------------------------------------------------------------------
// strided batched matrix view: element (i,j) of batch b at
//   p[i*rs + j*cs + b*bs]   (units: elements)
// ---------------------------------------------------------------------------
struct View {
  const void* p;
  long long rs, cs, bs;
};
inline View view_cm(const void* p, int ld, long long bs) { return View{p, 1, ld, bs}; }
inline View view_t(View v) { return View{v.p, v.cs, v.rs, v.bs}; }

// Batched GEMM  C_b = alpha_b * op(A_b) op(B_b) + beta * C_b  with complex or
// real operands (A real: ar = true).  alpha_b = alpha * (alpha_vec ? alpha_vec[b] : 1).
// C is complex unless c_real.
struct GemmArgs {
  int M, N, K, batch;
  View A, B;
  void* C;
  long long crs, ccs, cbs;
  double2 alpha, beta;
  const double2* alpha_vec;
  bool a_real, b_real, c_real;
  bool conj_a, conj_b;
  bool three_m;     // complex x complex with three real products (3M)
  bool upper_only;  // only the upper triangle is needed (the mma.sync path skips tiles below it)
  // optional second term along K: C = alpha (op(A) op(B) + s2 op(A2) op(B2))
  // + beta C with A2 (M x K2) and B2 (K2 x N) of the types and conjugations
  // of A and B.  The tcgen05 path forms it as one product over K + K2 (the
  // operands stacked along K); elsewhere it is split into two products.
  int K2;
  View A2, B2;
  double s2;
  // the left operand (after a shared left operand is swapped to the right)
  // is the previous tcgen05 product's on this stream, unchanged since: its
  // digit planes are reused (checked against the recorded operand)
  bool reuse_left;
};
int gemm(const GemmArgs& g, cudaStream_t s);
// the two terms of a product with K2 > 0 as two products
int gemm_split_k2(const GemmArgs& g, cudaStream_t s);
// the same product with the FP64 arithmetic emulated on the bf16 tensor cores
int gemm_ozaki(const GemmArgs& g, cudaStream_t s);
void oz_release(cudaStream_t s);
// per-stream scratch of the emulated products (grown on demand, stream-ordered)
int oz_scratch(cudaStream_t s, size_t bytes, size_t ex_count, __nv_bfloat16** buf, int** ex);
// GEMM arithmetic of the calls in flight: 0 FP64 pipe, 1 emulated with
// mma.sync, 2 emulated with tcgen05 (set by every C-ABI entry point from its
// context), and the status word of that context.  These call-scoped settings
// are per host thread: each thread drives its own context.
extern thread_local int g_gemm_mode;
// upper bound on the CTAs of a tcgen05 product (0: one per SM), set while
// two streams share the SMs with kernels that need their own
extern thread_local int g_tc_grid_cap;
// width of the tcgen05 products' B' tiles: 0 the one that pads the output
// columns less, 1 always 64 rows, 2 always 48 (set by every entry point from
// its context's tuning)
extern thread_local int g_tc_bn_policy;
// the tcgen05 complex x complex products of contraction length >= this take
// the paired form (real and imaginary rows interleaved on both sides), the
// others the real representation [[Re, -Im], [Im, Re]] x [Re, Im]; 0: none
// (set by every entry point from its context)
extern thread_local int g_tc_pairs_min_k;
struct TcGridCap {
  int saved;
  explicit TcGridCap(int cap) : saved(g_tc_grid_cap) { g_tc_grid_cap = cap; }
  ~TcGridCap() { g_tc_grid_cap = saved; }
};
extern thread_local int* g_dev_flags;
// when set, the tensor-memory product launches are timed into this section
// of this context (the H20 products; the host issues them one after the other)
extern thread_local tvap_ctx* g_tc_timing_ctx;
extern thread_local int g_tc_timing_sec;
struct TcTimingScope {
  TcTimingScope(tvap_ctx* c, int sec) {
    g_tc_timing_ctx = c;
    g_tc_timing_sec = sec;
  }
  ~TcTimingScope() {
    g_tc_timing_ctx = nullptr;
    g_tc_timing_sec = -1;
  }
};

// ---------------------------------------------------------------------------
// Hamiltonian in gather form (built once from the reference's element list)
// ---------------------------------------------------------------------------
// One field operator as dense symmetry blocks (field_blocks.cu)
struct FieldBlockDesc {
  long long aoff;  // first digit-plane element of the block
  int r_pad, kb_pad, kbeg, row_base;
};
// per block of the tcgen05 form: 128-row tiles of W, k-steps of 16, first
// k-step of the block (prefix over the blocks), first element of its W planes
struct FieldTcBlock {
  int mtiles, nks, kboff, pad;
  long long woff;
};
struct FieldDense {
  int nblk = 0, ntiles = 0, nrows = 0, ktot = 0;
  // tcgen05 form: W planes tiled [block][m tile][k-step][digit][128 x 16],
  // (block, m tile) list, 8-entry chunks of the blocks' inputs (block, k0)
  void* wt = nullptr;
  FieldTcBlock* tcb = nullptr;
  int2* tc_bm = nullptr;
  int2* tc_chunks = nullptr;
  int tc_nbm = 0, tc_ksteps = 0, tc_nchunks = 0;
  int tc_empty_base = 0, tc_nempty = 0;  // permuted rows of the rows without entries (zero fields)
  void* wd = nullptr;       // bf16 digit planes of W, block by block
  int* ea = nullptr;        // exponent per permuted output row
  int* rowperm = nullptr;   // permuted row -> output entry (-1: padding)
  int* colperm = nullptr;   // permuted input index -> input entry (-1: padding)
  int2* tiles = nullptr;    // (block, first row) of every 32-row tile
  FieldBlockDesc* blocks = nullptr;
};

struct FieldCSR {
  // Gamma: one row per output entry (x + y n), entries: src index (z + w n), coef
  int* g_rowptr = nullptr;
  int* g_src = nullptr;
  double* g_coef = nullptr;
  long long g_nnz = 0;
  // Delta (strict lower triangle rows b > a, output index b + a n)
  int* d_rows = nullptr;  // list of output indices with at least one entry
  int* d_rowptr = nullptr;
  int* d_src = nullptr;
  double* d_coef = nullptr;
  int d_nrows = 0;
  long long d_nnz = 0;
  // the same operators as dense symmetry blocks (when block-dense)
  FieldDense dense_g, dense_d;
  bool dense_ok = false;
};

struct Workspace;

}  // namespace tvap

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
constexpr size_t kPinnedBytes = 256;

struct tvap_ctx {
  int n = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int* d_sp_2mj = nullptr;
  int* d_sp_tr = nullptr;
  int* d_sp_l = nullptr;
  std::vector<int> h_sp_2mj, h_sp_tr, h_sp_l;
  // raw element list as uploaded (the reference's arrays)
  long long S = 0;
  int16_t* d_abcd = nullptr;
  float* d_h2 = nullptr;
  int8_t* d_trperm = nullptr;
  double2* d_H1 = nullptr;
  double2 H0 = {0.0, 0.0};
  bool have_ham = false;
  tvap::FieldCSR csr;
  cudaStream_t stream2 = nullptr;  // canonical basis (high priority), concurrent with the Thouless chain
  cudaStream_t stream3 = nullptr;  // overlap chain and Pfaffians (lowest priority)
  cudaStream_t streamM = nullptr;  // Thouless chain of the projection (priority between the two)
  cudaStream_t streamM2 = nullptr;  // second half of the angles in the Thouless solve (same priority)
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_canon = nullptr, ev_main = nullptr;
  cudaEvent_t ev_stagger = nullptr, ev_join2 = nullptr;  // the two halves of the Thouless solve
  // look-ahead of the Thouless solve, per half: the bulk of each elimination
  // product on its own stream (lowest priority) while the next panel is
  // factored; ev_la[h][0] = the block row is ready, [1] = the bulk is done
  cudaStream_t streamB[2] = {nullptr, nullptr};
  cudaEvent_t ev_la[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  void* h_pin = nullptr;  // pinned host buffer (kPinnedBytes) for the status word and small results
  tvap::Workspace* ws = nullptr;
  int* d_flags = nullptr;  // device status word
  unsigned* d_bar = nullptr;  // grid-barrier state of the cooperative kernels (3 words)
  int kernel_launches = 0;  // launches issued by the last top-level call
  int gemm_mode = 2;        // 0: FP64 pipe, 1/2: FP64 emulated on the bf16 tensor cores (mma.sync / tcgen05)
  // optional section timing with CUDA events on the context's stream
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_open;
  double section_ms[16] = {0};
  long long section_calls[16] = {0};
  // summed start and end offsets of the sections from the last timeline mark
  double section_t0[16] = {0}, section_t1[16] = {0};
  // work buffer of the per-call entry points (gradient, evolution), grown on
  // demand and reused: no allocation (and no device-wide cudaFree) per call
  double* scratch = nullptr;
  size_t scratch_count = 0;
  // canonical bases: [0] FP32 Jacobi + refinement attempts, [1] of them
  // accepted, [2] exact FP64 Jacobi runs, [3] FP32 Jacobi sweeps in total
  long long canon_attempts[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  // test hook (tvap_test_wait_timeout): the next cooperative evolution has
  // its last CTA leave before the first grid barrier; one-shot
  bool test_skip_arrival = false;
  // launch shapes chosen by tvap_autotune: B' tile policy (g_tc_bn_policy),
  // groups of angles in the Thouless solve (2 staggered or 1), and the cap
  // on the tcgen05 CTAs while the second group's panels run (0: the SMs the
  // panels leave, 1: half of the SMs, 2: none)
  int tune_bn = 0;
  int tune_groups = 2;
  int tune_cap = 0;
  int tune_lookahead = 0;  // look-ahead of the Thouless solve's panels (streamB)
  int tune_pf_blocked = 0;  // the blocked Pfaffian also where the shared-memory one fits
  int tune_pairs_k = 0;     // complex x complex tcgen05 products in the paired form from K = this on (0: none)
};

namespace tvap {
// Scope of one C-ABI call: starts the launch count and, on every return,
// records it as the context's tvap_kernel_launches.
struct LaunchTally {
  tvap_ctx* c;
  explicit LaunchTally(tvap_ctx* ctx) : c(ctx) { g_launch_count = 0; }
  ~LaunchTally() { c->kernel_launches = int(g_launch_count); }
  LaunchTally(const LaunchTally&) = delete;
  LaunchTally& operator=(const LaunchTally&) = delete;
};
enum Section : int {
  SEC_CANONICAL = 0, SEC_BLOCKS, SEC_SOLVE, SEC_UV, SEC_DENSITIES, SEC_FIELDS_GAMMA, SEC_FIELDS_DELTA, SEC_TRACES,
  SEC_H20, SEC_OVERLAP, SEC_PFAFFIAN, SEC_SUMS, SEC_GRADIENT, SEC_EVOLVE, SEC_H20_TC, SEC_COUNT
};
// brackets a section with events when timing is on (no-ops otherwise)
void sec_begin(tvap_ctx* c, int sec);
void sec_end(tvap_ctx* c, int sec);
void sec_begin_on(tvap_ctx* c, int sec, cudaStream_t s);
void sec_end_on(tvap_ctx* c, int sec, cudaStream_t s);
// origin of the section offsets that follow (the start of a projection)
void sec_mark(tvap_ctx* c, cudaStream_t s);
}  // namespace tvap

namespace tvap {

int build_field_csr(tvap_ctx* c);
void free_field_csr(FieldCSR& f);
// the context's work buffer with at least count doubles (stream-ordered reuse)
int ctx_scratch(tvap_ctx* c, size_t count, double** out);
int build_field_dense(tvap_ctx* c);
void free_field_dense(FieldDense& f);
// fields of ncol gauge-angle columns through the dense blocks (emulated FP64)
int fields_dense(tvap_ctx* c, int ncol, int ldc, const double2* rho, const double2* kLR, const double2* kRL,
                 double2* gamma, double2* hsp, double2* dLR, double2* dRL, cudaStream_t s);

// Fields for `ncol` columns (angles) in angle-innermost layout:
// X[(i + j n) * ldc + col].  hsp/dLR/dRL outputs in the same layout.
int fields_batched(tvap_ctx* c, int ncol, int ldc, const double2* rho, const double2* kLR, const double2* kRL,
                   double2* gamma, double2* hsp, double2* dLR, double2* dRL, cudaStream_t s);

// ---------------------------------------------------------------------------
// dense per-batch factorizations
// ---------------------------------------------------------------------------
// Pfaffian of `batch` skew matrices (upper triangle of column-major n x n
// blocks, stride n*n), Parlett-Reid with the reference's pivoting.
int pfaffian_batched(int n, int batch, double2* A, double2* pf, int* flags, cudaStream_t s, bool blocked = false);
// symmetric eigen-decomposition by cyclic Jacobi (one matrix), ascending order
// scale (device, may be null): the norm of the matrix A is a block of; the
// sweeps stop at that matrix's rounding level
int jacobi_eigen(int n, double* A, double* W, double* evals, double* work, int* flags, cudaStream_t s,
                 const double* scale = nullptr);
// same in FP32 (cold start of the refinement); tolerance ~1e-6.5 ||A||
int jacobi_eigen_f32(int n, float* A, float* W, double* evals, double* work, int* flags, cudaStream_t s);
// FP32 Jacobi with A and W in shared memory (n <= 160); W64 gets the unsorted
// eigenvectors of A64 as FP64 columns.  With W0 != null the rotations start
// from W0 and A64 must be W0^T A W0 (warm start); W64 = W0 J.
size_t jacobi32_smem_bytes(int n);
size_t jacobi32_smem_limit();
// FP32 Jacobi in shared memory (one CTA); the number of sweeps goes to *sweeps_out (may be null)
int jacobi32_smem(int n, const double* A64, const double* W0, double* W64, int* sweeps_out, cudaStream_t s);
// block one-sided FP32 Jacobi on a cluster of 8 CTAs: the columns of M (of
// M^T when m_transposed) orthogonalised, the rotations applied to W0 (the
// identity when null) and written to W (FP64): the eigenvectors of M^T M.
// TVAP_ERR_ARG when n > 256 (the caller then uses jacobi32_smem).
int jacobi_cluster(int n, const double* M, int m_transposed, const double* W0, double* W, int* sweeps_out,
                   cudaStream_t s);
// Cholesky L L^T = A (lower), then L^{-1} in place
int cholesky_inverse(int n, double* A, int* flags, cudaStream_t s);
// Cholesky L L^T = S (S overwritten by L, lower) and X_m = A_m L^{-T} for
// m = 0, 1 (A_1 at A + a_stride, X_1 at X + x_stride) in one cooperative
// launch; TVAP_ERR_ARG when n is outside its range (the caller then uses
// cholesky_inverse and two products)
int cholesky_evolve_coop(int n, double* S, const double* A, long long a_stride, double* X, long long x_stride,
                         unsigned* bar, int* flags, cudaStream_t s, int skip_cta = -1);

}  // namespace tvap
