// Many independent states at once: the seeds of a minima search and the
// points of a constraint sweep (uneven basis sizes included) iterate
// concurrently on one device.  Each state names its context; the states of
// one context run in order on one host thread, and distinct contexts run on
// concurrent host threads, so that their streams share the GPU.  A state of
// a small basis leaves most SMs idle and waits on its host round trips; with
// several contexts in flight the device stays busy.

#include <algorithm>
#include <string>
#include <thread>
#include <vector>

#include "tvap_internal.cuh"

using namespace tvap;

extern "C" {

int tvap_iterate(tvap_ctx* c, const double* U0, const double* V0, const tvap_proj_opts* opts, double eta, double mu,
                 const double* Zim1, double* Zi, double* U1, double* V1, tvap_pnp* out, double* H20v,
                 double* gradient_norm);
const char* tvap_last_error(void);

int tvap_iterate_many(int nstates, tvap_ctx* const* ctx, const double* const* U0, const double* const* V0,
                      const tvap_proj_opts* opts, const double* eta, const double* mu, const double* const* Zim1,
                      double* const* Zi, double* const* U1, double* const* V1, tvap_pnp* out,
                      double* gradient_norm, int* status) {
  if (nstates < 0 || (nstates > 0 && (!ctx || !U0 || !V0 || !opts || !eta || !mu || !Zim1 || !Zi || !U1 || !V1 ||
                                      !out || !gradient_norm || !status)))
    return TVAP_ERR_ARG;
  // the distinct contexts, in the order of their first state
  std::vector<tvap_ctx*> uniq;
  for (int s = 0; s < nstates; ++s) {
    if (!ctx[s]) return TVAP_ERR_ARG;
    if (std::find(uniq.begin(), uniq.end(), ctx[s]) == uniq.end()) uniq.push_back(ctx[s]);
  }
  for (int s = 0; s < nstates; ++s) status[s] = -1;
  // the message of each state that failed (the last-error text is kept per
  // host thread; the caller's thread gets the first failing state's)
  std::vector<std::string> msgs(nstates);
  auto run = [&](tvap_ctx* c) {
    // the thread works on the context's device
    if (cudaSetDevice(c->device) != cudaSuccess) {
      cudaGetLastError();
      for (int s = 0; s < nstates; ++s)
        if (ctx[s] == c) status[s] = TVAP_ERR_CUDA;
      return;
    }
    int launches = 0;
    for (int s = 0; s < nstates; ++s) {
      if (ctx[s] != c) continue;
      status[s] = tvap_iterate(c, U0[s], V0[s], opts + s, eta[s], mu[s], Zim1[s], Zi[s], U1[s], V1[s], out + s,
                               nullptr, gradient_norm + s);
      if (status[s] != TVAP_OK) msgs[s] = tvap_last_error();
      launches += c->kernel_launches;
    }
    c->kernel_launches = launches;
  };
  if (uniq.size() <= 1) {
    if (!uniq.empty()) run(uniq[0]);
  } else {
    std::vector<std::thread> threads;
    threads.reserve(uniq.size());
    for (tvap_ctx* c : uniq) threads.emplace_back(run, c);
    for (auto& t : threads) t.join();
  }
  for (int s = 0; s < nstates; ++s)
    if (status[s] != TVAP_OK) {
      if (!msgs[s].empty()) set_last_error(("state " + std::to_string(s) + ": " + msgs[s]).c_str(), __FILE__, __LINE__);
      return status[s];
    }
  return TVAP_OK;
}

}  // extern "C"
