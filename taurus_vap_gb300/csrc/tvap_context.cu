// C ABI (include/tvap.h): context, Hamiltonian upload, calculate_fields and
// project_wavefunction entry points.

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "tvap_internal.cuh"

namespace tvap {

static thread_local std::string g_last_error;

void set_last_error(const char* msg, const char* file, int line) {
  g_last_error = std::string(msg) + " (" + file + ":" + std::to_string(line) + ")";
}

namespace {
struct SmemGrant {
  int device;
  const void* func;
  size_t bytes;
};
std::mutex g_smem_mutex;
std::vector<SmemGrant> g_smem_grants;
std::mutex g_sms_mutex;
std::vector<std::pair<int, int>> g_sms;  // (device, SM count)
}  // namespace

int smem_opt_in(const void* func, size_t bytes) {
  int dev = 0;
  TVAP_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(g_smem_mutex);
  SmemGrant* g = nullptr;
  for (auto& e : g_smem_grants)
    if (e.device == dev && e.func == func) g = &e;
  if (g && g->bytes >= bytes) return TVAP_OK;
  TVAP_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
  if (g)
    g->bytes = bytes;
  else
    g_smem_grants.push_back({dev, func, bytes});
  return TVAP_OK;
}

int device_sms() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  std::lock_guard<std::mutex> lock(g_sms_mutex);
  for (const auto& e : g_sms)
    if (e.first == dev) return e.second;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  g_sms.emplace_back(dev, sms);
  return sms;
}

int upload_matrix(const void* src, void* dst, size_t bytes, cudaStream_t s);
int download_matrix(const void* src, void* dst, size_t bytes, cudaStream_t s);
bool is_device_pointer(const void* p);
int check_finite(tvap_ctx* c, const double* const* ptrs, const char* const* names, int count, size_t elems);
int project_device(tvap_ctx* c, const tvap_proj_opts& o, tvap_pnp* out, bool sync = true);
int ensure_workspace(tvap_ctx* c, int G);
void destroy_workspace(tvap_ctx* c);
int angle_count(const tvap_proj_opts& o);
int observables_angle_count(const tvap_proj_opts& o);
int project_observables_device(tvap_ctx* c, const tvap_proj_opts& o, int nobo, const double* obo, int nsq,
                               const double* sq, const int* parity, int nshell, const int* shell_size,
                               double2* scal, double2* obo_out, double2* sq_out, double2* occ_out, double* rho_out,
                               int* nocc_nemp);
int check_flags(tvap_ctx* c);
double* ws_U(tvap_ctx* c);
double* ws_V(tvap_ctx* c);
double* ws_H20v(tvap_ctx* c);

static cudaEvent_t take_event(tvap_ctx* c) {
  if (!c->ev_pool.empty()) {
    cudaEvent_t e = c->ev_pool.back();
    c->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

void sec_begin_on(tvap_ctx* c, int sec, cudaStream_t s) {
  if (!c->timing) return;
  cudaEvent_t a = take_event(c), b = take_event(c);
  cudaEventRecord(a, s);
  c->ev_open.push_back({sec, {a, b}});
}

void sec_end_on(tvap_ctx* c, int sec, cudaStream_t s) {
  if (!c->timing) return;
  for (auto it = c->ev_open.rbegin(); it != c->ev_open.rend(); ++it)
    if (it->first == sec && it->second.second) {
      cudaEventRecord(it->second.second, s);
      it->first = sec + 1000;  // closed
      return;
    }
}

void sec_mark(tvap_ctx* c, cudaStream_t s) {
  if (!c->timing) return;
  cudaEvent_t a = take_event(c);
  cudaEventRecord(a, s);
  c->ev_open.push_back({-1, {a, nullptr}});
}

void sec_begin(tvap_ctx* c, int sec) { sec_begin_on(c, sec, c->stream); }
void sec_end(tvap_ctx* c, int sec) { sec_end_on(c, sec, c->stream); }

static void collect_sections(tvap_ctx* c) {
  if (c->ev_open.empty()) return;
  cudaStreamSynchronize(c->stream);
  cudaEvent_t mark = nullptr;
  for (auto& e : c->ev_open) {
    if (e.first == -1) {
      mark = e.second.first;
    } else if (e.first >= 1000) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e.second.first, e.second.second);
      c->section_ms[e.first - 1000] += ms;
      c->section_calls[e.first - 1000] += 1;
      if (mark) {
        float t0 = 0.f, t1 = 0.f;
        cudaEventElapsedTime(&t0, mark, e.second.first);
        cudaEventElapsedTime(&t1, mark, e.second.second);
        c->section_t0[e.first - 1000] += t0;
        c->section_t1[e.first - 1000] += t1;
      }
    }
    c->ev_pool.push_back(e.second.first);
    if (e.second.second) c->ev_pool.push_back(e.second.second);
  }
  c->ev_open.clear();
}

namespace {

// column-major n x n (ncol matrices) <-> angle-innermost
__global__ void to_inner_kernel(size_t nn, int ncol, const double2* __restrict__ src, double2* __restrict__ dst) {
  const size_t idx = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (idx >= nn * ncol) return;
  const size_t e = idx / ncol;
  const int col = int(idx % ncol);
  dst[idx] = src[size_t(col) * nn + e];
}
__global__ void from_inner_kernel(size_t nn, int ncol, const double2* __restrict__ src, double2* __restrict__ dst) {
  const size_t idx = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (idx >= nn * ncol) return;
  const size_t e = idx % nn;
  const int col = int(idx / nn);
  dst[idx] = src[e * ncol + col];
}

}  // namespace

}  // namespace tvap

using namespace tvap;

namespace tvap {

int ctx_scratch(tvap_ctx* c, size_t count, double** out) {
  if (count > c->scratch_count) {
    if (c->scratch) {
      TVAP_CUDA(cudaStreamSynchronize(c->stream));
      cudaFree(c->scratch);
    }
    c->scratch = nullptr;
    c->scratch_count = 0;
    TVAP_CUDA(cudaMalloc(&c->scratch, sizeof(double) * count));
    c->scratch_count = count;
  }
  *out = c->scratch;
  return TVAP_OK;
}

}  // namespace tvap

extern "C" {

const char* tvap_last_error(void) { return g_last_error.c_str(); }

int tvap_kernel_launches(const tvap_ctx* ctx) { return ctx ? ctx->kernel_launches : 0; }

int tvap_set_timing(tvap_ctx* c, int on) {
  if (!c) return TVAP_ERR_ARG;
  collect_sections(c);
  c->timing = (on != 0);
  for (int i = 0; i < 16; ++i) {
    c->section_ms[i] = 0.0;
    c->section_calls[i] = 0;
    c->section_t0[i] = c->section_t1[i] = 0.0;
  }
  for (long long& v : c->canon_attempts) v = 0;
  return TVAP_OK;
}

int tvap_set_gemm_mode(tvap_ctx* c, int mode) {
  if (!c || mode < 0 || mode > 2) return TVAP_ERR_ARG;
  c->gemm_mode = mode;
  return TVAP_OK;
}

int tvap_get_timing(tvap_ctx* c, double* ms, long long* calls, int nsec) {
  if (!c || !ms) return TVAP_ERR_ARG;
  collect_sections(c);
  for (int i = 0; i < nsec && i < 16; ++i) {
    ms[i] = c->section_ms[i];
    if (calls) calls[i] = c->section_calls[i];
  }
  return TVAP_OK;
}

int tvap_get_timeline(tvap_ctx* c, double* t0, double* t1, int nsec) {
  if (!c || !t0 || !t1) return TVAP_ERR_ARG;
  collect_sections(c);
  for (int i = 0; i < nsec && i < 16; ++i) {
    const double k = c->section_calls[i] ? double(c->section_calls[i]) : 1.0;
    t0[i] = c->section_t0[i] / k;
    t1[i] = c->section_t1[i] / k;
  }
  return TVAP_OK;
}

int tvap_get_counters(tvap_ctx* c, long long* out, int nout) {
  if (!c || !out) return TVAP_ERR_ARG;
  for (int i = 0; i < nout && i < 9; ++i) out[i] = c->canon_attempts[i];
  return TVAP_OK;
}

int tvap_init(tvap_ctx** ctx, int64_t n, const int32_t* sp_2mj, const int32_t* sp_tr, const int32_t* sp_l,
              int device) {
  if (!ctx || n <= 0 || n > 512 || (n % 2) != 0 || !sp_2mj || !sp_tr || !sp_l) {
    g_last_error = "tvap_init: n must be even and in 2..512, tables non-null";
    return TVAP_ERR_ARG;
  }
  auto* c = new tvap_ctx();
  c->n = int(n);
  if (device >= 0) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
      set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
      delete c;
      return TVAP_ERR_CUDA;
    }
  }
  cudaGetDevice(&c->device);
  c->h_sp_2mj.assign(sp_2mj, sp_2mj + n);
  c->h_sp_tr.assign(sp_tr, sp_tr + n);
  c->h_sp_l.assign(sp_l, sp_l + n);
  for (int i = 0; i < n; ++i)
    if (sp_tr[i] < 1 || sp_tr[i] > n) {
      g_last_error = "tvap_init: HOsp_tr out of range";
      delete c;
      return TVAP_ERR_ARG;
    }
  auto fail = [&](cudaError_t e) {
    set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
    tvap_destroy(c);
    return TVAP_ERR_CUDA;
  };
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess) return fail(e);
  c->own_stream = true;
  // the second stream carries the latency-bound chain (canonical basis,
  // Pfaffians): it gets the highest priority so that its few CTAs are
  // scheduled ahead of the wide kernels of the main stream
  int prio_lo = 0, prio_hi = 0;
  if ((e = cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi)) != cudaSuccess) return fail(e);
  if ((e = cudaStreamCreateWithPriority(&c->stream2, cudaStreamNonBlocking, prio_hi)) != cudaSuccess) return fail(e);
  if ((e = cudaStreamCreateWithPriority(&c->stream3, cudaStreamNonBlocking, prio_lo)) != cudaSuccess) return fail(e);
  // the Thouless chain ahead of the overlap chain when they share the SMs
  // (the caller's stream usually has the lowest priority)
  const int prio_mid = prio_hi + (prio_lo - prio_hi) / 2;
  if ((e = cudaStreamCreateWithPriority(&c->streamM, cudaStreamNonBlocking, prio_mid)) != cudaSuccess)
    return fail(e);
  if ((e = cudaStreamCreateWithPriority(&c->streamM2, cudaStreamNonBlocking, prio_mid)) != cudaSuccess)
    return fail(e);
  for (int q = 0; q < 2; ++q) {
    if ((e = cudaStreamCreateWithPriority(&c->streamB[q], cudaStreamNonBlocking, prio_lo)) != cudaSuccess)
      return fail(e);
    for (int r = 0; r < 2; ++r)
      if ((e = cudaEventCreateWithFlags(&c->ev_la[q][r], cudaEventDisableTiming)) != cudaSuccess) return fail(e);
  }
  if ((e = cudaEventCreateWithFlags(&c->ev_main, cudaEventDisableTiming)) != cudaSuccess) return fail(e);
  if ((e = cudaEventCreateWithFlags(&c->ev_stagger, cudaEventDisableTiming)) != cudaSuccess) return fail(e);
  if ((e = cudaMallocHost(&c->h_pin, kPinnedBytes)) != cudaSuccess) return fail(e);
  if ((e = cudaEventCreateWithFlags(&c->ev_join2, cudaEventDisableTiming)) != cudaSuccess) return fail(e);
  if ((e = cudaEventCreateWithFlags(&c->ev_canon, cudaEventDisableTiming)) != cudaSuccess) return fail(e);
  if ((e = cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming)) != cudaSuccess) return fail(e);
  if ((e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&c->d_sp_2mj, sizeof(int) * n)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&c->d_sp_tr, sizeof(int) * n)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&c->d_sp_l, sizeof(int) * n)) != cudaSuccess) return fail(e);
  // the status word, then words for the non-finite check of caller matrices
  if ((e = cudaMalloc(&c->d_flags, 8 * sizeof(int))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&c->d_bar, 4 * sizeof(unsigned))) != cudaSuccess) return fail(e);
  cudaMemset(c->d_bar, 0, 4 * sizeof(unsigned));
  cudaMemcpy(c->d_sp_2mj, sp_2mj, sizeof(int) * n, cudaMemcpyHostToDevice);
  cudaMemcpy(c->d_sp_tr, sp_tr, sizeof(int) * n, cudaMemcpyHostToDevice);
  cudaMemcpy(c->d_sp_l, sp_l, sizeof(int) * n, cudaMemcpyHostToDevice);
  cudaMemset(c->d_flags, 0, 8 * sizeof(int));
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
  *ctx = c;
  return TVAP_OK;
}

void tvap_destroy(tvap_ctx* c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->stream2) cudaStreamSynchronize(c->stream2);
  if (c->stream3) cudaStreamSynchronize(c->stream3);
  if (c->streamM) cudaStreamSynchronize(c->streamM);
  if (c->streamM2) cudaStreamSynchronize(c->streamM2);
  for (auto sb : c->streamB)
    if (sb) cudaStreamSynchronize(sb);
  cudaFree(c->scratch);
  destroy_workspace(c);
  free_field_csr(c->csr);
  cudaFree(c->d_sp_2mj);
  cudaFree(c->d_sp_tr);
  cudaFree(c->d_sp_l);
  cudaFree(c->d_abcd);
  cudaFree(c->d_h2);
  cudaFree(c->d_trperm);
  cudaFree(c->d_H1);
  cudaFree(c->d_flags);
  cudaFree(c->d_bar);
  for (auto& e : c->ev_open) {
    cudaEventDestroy(e.second.first);
    if (e.second.second) cudaEventDestroy(e.second.second);
  }
  for (auto e : c->ev_pool) cudaEventDestroy(e);
  if (c->stream) oz_release(c->stream);
  if (c->stream2) oz_release(c->stream2);
  if (c->stream3) oz_release(c->stream3);
  if (c->streamM) oz_release(c->streamM);
  if (c->streamM2) oz_release(c->streamM2);
  for (auto sb : c->streamB)
    if (sb) {
      oz_release(sb);
      cudaStreamDestroy(sb);
    }
  for (auto& q : c->ev_la)
    for (auto ev : q)
      if (ev) cudaEventDestroy(ev);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  if (c->stream2) cudaStreamDestroy(c->stream2);
  if (c->stream3) cudaStreamDestroy(c->stream3);
  if (c->streamM) cudaStreamDestroy(c->streamM);
  if (c->streamM2) cudaStreamDestroy(c->streamM2);
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_stagger) cudaEventDestroy(c->ev_stagger);
  if (c->h_pin) cudaFreeHost(c->h_pin);
  if (c->ev_join2) cudaEventDestroy(c->ev_join2);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  if (c->ev_main) cudaEventDestroy(c->ev_main);
  if (c->ev_canon) cudaEventDestroy(c->ev_canon);
  delete c;
}

int tvap_set_stream(tvap_ctx* c, void* stream) {
  if (!c) return TVAP_ERR_ARG;
  if (c->stream) oz_release(c->stream);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  c->stream = static_cast<cudaStream_t>(stream);
  c->own_stream = false;
  return TVAP_OK;
}

int tvap_set_hamiltonian(tvap_ctx* c, int64_t S, const int16_t* abcd, const float* h2, const int8_t* trperm,
                         const double* H1, const double* H0) {
  if (!c || S < 0 || (S > 0 && (!abcd || !h2 || !trperm)) || !H1 || !H0) return TVAP_ERR_ARG;
  if (S > (int64_t(1) << 26)) {
    g_last_error = "tvap_set_hamiltonian: element list too long (16 slots per element must fit int32)";
    return TVAP_ERR_ARG;
  }
  LaunchTally tally(c);  // CUB's sort and scan of the element list launch kernels of their own, not counted
  const int n = c->n;
  cudaFree(c->d_abcd);
  cudaFree(c->d_h2);
  cudaFree(c->d_trperm);
  cudaFree(c->d_H1);
  c->d_abcd = nullptr;
  c->d_h2 = nullptr;
  c->d_trperm = nullptr;
  c->S = S;
  TVAP_CUDA(cudaMalloc(&c->d_abcd, sizeof(int16_t) * 4 * std::max<int64_t>(S, 1)));
  TVAP_CUDA(cudaMalloc(&c->d_h2, sizeof(float) * std::max<int64_t>(S, 1)));
  TVAP_CUDA(cudaMalloc(&c->d_trperm, sizeof(int8_t) * std::max<int64_t>(S, 1)));
  TVAP_CUDA(cudaMalloc(&c->d_H1, sizeof(double2) * size_t(n) * n));
  int rc;
  if (S > 0) {
    if ((rc = upload_matrix(abcd, c->d_abcd, sizeof(int16_t) * 4 * S, c->stream))) return rc;
    if ((rc = upload_matrix(h2, c->d_h2, sizeof(float) * S, c->stream))) return rc;
    if ((rc = upload_matrix(trperm, c->d_trperm, sizeof(int8_t) * S, c->stream))) return rc;
  }
  if ((rc = upload_matrix(H1, c->d_H1, sizeof(double2) * size_t(n) * n, c->stream))) return rc;
  c->H0 = make_double2(H0[0], H0[1]);
  TVAP_CUDA(cudaStreamSynchronize(c->stream));
  if ((rc = build_field_csr(c))) return rc;
  if ((rc = build_field_dense(c))) return rc;
  c->have_ham = true;
  return TVAP_OK;
}

int tvap_calculate_fields_batched(tvap_ctx* c, int ncol, const double* rho, const double* kLR, const double* kRL,
                                  double* gamma, double* hsp, double* dLR, double* dRL) {
  if (!c || ncol <= 0 || ncol > 256 || !rho || !kLR || !kRL || !gamma || !hsp || !dLR || !dRL)
    return TVAP_ERR_ARG;
  if (!c->have_ham) return TVAP_ERR_NOT_READY;
  LaunchTally tally(c);
  g_gemm_mode = c->gemm_mode;
  g_tc_bn_policy = c->tune_bn;
  g_tc_pairs_min_k = c->tune_pairs_k;
  g_dev_flags = c->d_flags;
  const int n = c->n;
  const size_t nn = size_t(n) * n, tot = nn * ncol;
  cudaStream_t s = c->stream;
  double2* buf = nullptr;  // 7 * tot: staging (column-major) + 3 inner inputs + 4 inner outputs ... reused
  TVAP_CUDA(cudaMalloc(&buf, sizeof(double2) * tot * 8));
  double2* stage = buf;
  double2* in[3] = {buf + tot, buf + 2 * tot, buf + 3 * tot};
  double2* out[4] = {buf + 4 * tot, buf + 5 * tot, buf + 6 * tot, buf + 7 * tot};
  const double* srcs[3] = {rho, kLR, kRL};
  double* dsts[4] = {gamma, hsp, dLR, dRL};
  int rc = TVAP_OK;
  const int tb = 256;
  const unsigned nb = unsigned((tot + tb - 1) / tb);
  for (int q = 0; q < 3 && rc == TVAP_OK; ++q) {
    rc = upload_matrix(srcs[q], stage, sizeof(double2) * tot, s);
    if (rc == TVAP_OK) to_inner_kernel<<<nb, tb, 0, tvap::counted(s)>>>(nn, ncol, stage, in[q]);
  }
  if (rc == TVAP_OK) rc = fields_batched(c, ncol, ncol, in[0], in[1], in[2], out[0], out[1], out[2], out[3], s);
  for (int q = 0; q < 4 && rc == TVAP_OK; ++q) {
    from_inner_kernel<<<nb, tb, 0, tvap::counted(s)>>>(nn, ncol, out[q], stage);
    rc = download_matrix(stage, dsts[q], sizeof(double2) * tot, s);
    if (rc == TVAP_OK) {
      cudaError_t e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
        rc = TVAP_ERR_CUDA;
      }
    }
  }
  cudaFree(buf);
  // the status word: a bounded wait of the tensor-core field kernels that gave up
  if (rc == TVAP_OK) rc = check_flags(c);
  return rc;
}

int tvap_calculate_fields(tvap_ctx* c, const double* rho, const double* kLR, const double* kRL, double* gamma,
                          double* hsp, double* dLR, double* dRL) {
  return tvap_calculate_fields_batched(c, 1, rho, kLR, kRL, gamma, hsp, dLR, dRL);
}

int tvap_project(tvap_ctx* c, const double* U0, const double* V0, const tvap_proj_opts* opts, tvap_pnp* out,
                 double* H20v) {
  if (!c || !U0 || !V0 || !opts || opts->Mphip < 1 || opts->Mphin < 1) return TVAP_ERR_ARG;
  if (!c->have_ham) return TVAP_ERR_NOT_READY;
  LaunchTally tally(c);
  g_gemm_mode = c->gemm_mode;
  g_tc_bn_policy = c->tune_bn;
  g_tc_pairs_min_k = c->tune_pairs_k;
  g_dev_flags = c->d_flags;
  const int n = c->n;
  const size_t nn = size_t(n) * n;
  int rc;
  {
    const double* mats[2] = {U0, V0};
    const char* names[2] = {"U0", "V0"};
    if ((rc = check_finite(c, mats, names, 2, nn))) return rc;
  }
  if ((rc = ensure_workspace(c, angle_count(*opts)))) return rc;
  if ((rc = upload_matrix(U0, ws_U(c), sizeof(double) * nn, c->stream))) return rc;
  if ((rc = upload_matrix(V0, ws_V(c), sizeof(double) * nn, c->stream))) return rc;
  if ((rc = project_device(c, *opts, out))) return rc;
  if (H20v) {
    if ((rc = download_matrix(ws_H20v(c), H20v, sizeof(double) * nn, c->stream))) return rc;
    // a device destination is written in the order of the context's stream;
    // a host one is complete on return
    if (!is_device_pointer(H20v)) TVAP_CUDA(cudaStreamSynchronize(c->stream));
  }
  return TVAP_OK;
}

int tvap_project_observables(tvap_ctx* c, const double* U0, const double* V0, const tvap_proj_opts* opts, int nobo,
                             const double* obo, int nsq, const double* sq, const int32_t* sp_parity, int nshell,
                             const int32_t* shell_size, tvap_pnp_obs* out, double* obo_sum, double* sq_sum,
                             double* occnum, double* rho) {
  if (!c || !U0 || !V0 || !opts || !out || opts->Mphip < 1 || opts->Mphin < 1 || nobo < 0 || nsq < 0 ||
      nshell < 0 || (nobo > 0 && (!obo || !obo_sum)) || (nsq > 0 && (!sq || !sq_sum)) ||
      (nshell > 0 && (!shell_size || !occnum)))
    return TVAP_ERR_ARG;
  if (sp_parity && is_device_pointer(sp_parity)) return TVAP_ERR_ARG;
  if (shell_size && is_device_pointer(shell_size)) return TVAP_ERR_ARG;
  for (int k = 0; k < nshell; ++k)
    if (shell_size[k] < 0) return TVAP_ERR_ARG;
  if (sp_parity)
    for (int i = 0; i < c->n; ++i)
      if (sp_parity[i] != 1 && sp_parity[i] != -1) return TVAP_ERR_ARG;
  if (!c->have_ham) return TVAP_ERR_NOT_READY;
  LaunchTally tally(c);
  g_gemm_mode = c->gemm_mode;
  g_tc_bn_policy = c->tune_bn;
  g_tc_pairs_min_k = c->tune_pairs_k;
  g_dev_flags = c->d_flags;
  const int n = c->n;
  const size_t nn = size_t(n) * n;
  int rc;
  {
    const double* mats[2] = {U0, V0};
    const char* names[2] = {"U0", "V0"};
    if ((rc = check_finite(c, mats, names, 2, nn))) return rc;
  }
  if ((rc = ensure_workspace(c, observables_angle_count(*opts)))) return rc;
  if ((rc = upload_matrix(U0, ws_U(c), sizeof(double) * nn, c->stream))) return rc;
  if ((rc = upload_matrix(V0, ws_V(c), sizeof(double) * nn, c->stream))) return rc;
  std::vector<double2> scal(19), bo(2 * size_t(nobo)), so(static_cast<size_t>(nsq)), oc(2 * size_t(nshell));
  int nn2[2] = {0, 0};
  if ((rc = project_observables_device(c, *opts, nobo, obo, nsq, sq, sp_parity, nshell, shell_size, scal.data(),
                                       bo.data(), so.data(), oc.data(), rho, nn2)))
    return rc;
  double* dst[7] = {out->over, out->ener, out->prot, out->neut, out->prot2, out->neut2, out->pari};
  for (int q = 0; q < 7; ++q) {
    dst[q][0] = scal[q].x;
    dst[q][1] = scal[q].y;
  }
  for (int q = 0; q < 12; ++q) {
    out->ecomp[q][0] = scal[7 + q].x;
    out->ecomp[q][1] = scal[7 + q].y;
  }
  out->nocc = nn2[0];
  out->nemp = nn2[1];
  if (nobo > 0) std::memcpy(obo_sum, bo.data(), sizeof(double2) * bo.size());
  if (nsq > 0) std::memcpy(sq_sum, so.data(), sizeof(double2) * so.size());
  if (nshell > 0) std::memcpy(occnum, oc.data(), sizeof(double2) * oc.size());
  return TVAP_OK;
}

int tvap_set_tuning(tvap_ctx* c, int bn_policy, int solve_groups, int solve_cap) {
  if (!c || bn_policy < 0 || bn_policy > 2 || solve_groups < 1 || solve_groups > 2 || solve_cap < 0 || solve_cap > 2)
    return TVAP_ERR_ARG;
  c->tune_bn = bn_policy;
  c->tune_groups = solve_groups;
  c->tune_cap = solve_cap;
  return TVAP_OK;
}

int tvap_set_option(tvap_ctx* c, int option, int value) {
  if (!c || value < 0) return TVAP_ERR_ARG;
  if (option == TVAP_OPT_COMPLEX_PAIRS) {
    c->tune_pairs_k = value;
    return TVAP_OK;
  }
  if (value > 1) return TVAP_ERR_ARG;
  switch (option) {
    case TVAP_OPT_SOLVE_LOOKAHEAD: c->tune_lookahead = value; return TVAP_OK;
    case TVAP_OPT_PFAFFIAN_BLOCKED: c->tune_pf_blocked = value; return TVAP_OK;
    default: return TVAP_ERR_ARG;
  }
}

int tvap_get_option(const tvap_ctx* c, int option) {
  if (!c) return -1;
  switch (option) {
    case TVAP_OPT_SOLVE_LOOKAHEAD: return c->tune_lookahead;
    case TVAP_OPT_PFAFFIAN_BLOCKED: return c->tune_pf_blocked;
    case TVAP_OPT_COMPLEX_PAIRS: return c->tune_pairs_k;
    default: return -1;
  }
}

int tvap_get_tuning(const tvap_ctx* c, int* knobs) {
  if (!c || !knobs) return TVAP_ERR_ARG;
  knobs[0] = c->tune_bn;
  knobs[1] = c->tune_groups;
  knobs[2] = c->tune_cap;
  return TVAP_OK;
}

int tvap_autotune(tvap_ctx* c, const double* U0, const double* V0, const tvap_proj_opts* opts, int reps,
                  double* table_ms, int ntable) {
  if (!c || !U0 || !V0 || !opts || reps < 1) return TVAP_ERR_ARG;
  if (!c->have_ham) return TVAP_ERR_NOT_READY;
  struct Cand {
    int bn, groups, cap, la, pf;
  };
  std::vector<Cand> cands;
  for (int pf = 0; pf <= 1; ++pf)
    for (int la = 1; la >= 0; --la)
      for (int groups = 2; groups >= 1; --groups)
        for (int cap = 0; cap < (groups == 2 ? 3 : 1); ++cap)
          for (int bn = 0; bn < 3; ++bn) cands.push_back({bn, groups, cap, la, pf});
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  TVAP_CUDA(cudaEventCreate(&e0));
  TVAP_CUDA(cudaEventCreate(&e1));
  int rc = TVAP_OK;
  double best = 1e300;
  Cand chosen = {c->tune_bn, c->tune_groups, c->tune_cap, c->tune_lookahead, c->tune_pf_blocked};
  tvap_pnp out{};
  for (size_t k = 0; k < cands.size() && rc == TVAP_OK; ++k) {
    c->tune_bn = cands[k].bn;
    c->tune_groups = cands[k].groups;
    c->tune_cap = cands[k].cap;
    c->tune_lookahead = cands[k].la;
    c->tune_pf_blocked = cands[k].pf;
    if ((rc = tvap_project(c, U0, V0, opts, &out, nullptr))) break;  // warm-up (scratch, tables)
    cudaEventRecord(e0, c->stream);
    for (int r = 0; r < reps && rc == TVAP_OK; ++r) rc = tvap_project(c, U0, V0, opts, &out, nullptr);
    cudaEventRecord(e1, c->stream);
    if (cudaEventSynchronize(e1) != cudaSuccess) rc = TVAP_ERR_CUDA;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double per = double(ms) / reps;
    if (table_ms && int(k) < ntable) table_ms[k] = per;
    if (per < best) {
      best = per;
      chosen = cands[k];
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c->tune_bn = chosen.bn;
  c->tune_groups = chosen.groups;
  c->tune_cap = chosen.cap;
  c->tune_lookahead = chosen.la;
  c->tune_pf_blocked = chosen.pf;
  return rc;
}

int tvap_project_batched(tvap_ctx* c, int nstates, const double* U0s, const double* V0s, const tvap_proj_opts* opts,
                         tvap_pnp* outs, double* H20vs) {
  if (!c || nstates < 0 || (nstates > 0 && (!U0s || !V0s || !opts || !outs))) return TVAP_ERR_ARG;
  const size_t nn = size_t(c->n) * c->n;
  int launches = 0;  // each tvap_project records its own launches
  int rc = TVAP_OK;
  for (int s = 0; s < nstates && rc == TVAP_OK; ++s) {
    rc = tvap_project(c, U0s + s * nn, V0s + s * nn, opts + s, outs + s, H20vs ? H20vs + s * nn : nullptr);
    launches += c->kernel_launches;
  }
  c->kernel_launches = launches;
  return rc;
}

}  // extern "C"
