// Autotuner of the launch shapes that have more than one good value (sm_103a).
//
// On the first solve of a handle it times, on the handle's own stream and buffers,
//   - the k-line preconditioner (maps + apply) for every candidate chunk length L
//     (kline::chunk_len_candidates: 2 .. 128 elements, at most 64 chunks), in the
//     precision the handle iterates in;
//   - the mixed form's FP32 xi stencil with 2 and 4 xi cells per thread;
// and keeps the fastest of each.  Both choices change rounding only (the chunked
// k-line sweep is an exact re-association of the element recurrence), so the
// choice is cached per shape (n_el, N_K, Nk, N_xi, precision) for the process:
// every handle of a shape, whatever its batch, runs the same launch shapes and
// gives the same results.  Inputs of the timed launches are scratch vectors
// zeroed first (every solve overwrites them before reading).
#include <cuda_runtime.h>

#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>

#include "kline.cuh"
#include "problem.h"

namespace wg {

namespace {

using TuneKey = std::tuple<int, int, int, int, int>;
struct TuneChoice {
  int kline_L;
  int st_cells;
};

std::mutex& tune_mutex() {
  static std::mutex m;
  return m;
}

std::map<TuneKey, TuneChoice>& tune_cache() {
  static std::map<TuneKey, TuneChoice> c;
  return c;
}

bool autotune_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("WG_AUTOTUNE");
    return !(v && v[0] == '0');
  }();
  return on;
}

// Mean device time [ms] of `fn` over `reps` calls after one warm-up call.
template <typename Fn>
float time_ms(Problem& P, cudaEvent_t a, cudaEvent_t b, Fn fn, int reps, cudaError_t& err) {
  err = fn();
  if (err != cudaSuccess) return 0.f;
  cudaEventRecord(a, P.stream);
  for (int i = 0; i < reps && err == cudaSuccess; ++i) err = fn();
  cudaEventRecord(b, P.stream);
  if (err == cudaSuccess) err = cudaEventSynchronize(b);
  float ms = 0.f;
  if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, a, b);
  return ms / reps;
}

}  // namespace

int autotune(Problem& P) {
  P.tuned = true;
  if (!autotune_enabled()) return WG_OK;
  const bool mixed = P.precision == WG_PREC_MIXED;
  const TuneKey key{P.s.n_el, P.s.nK, P.s.nk, P.s.nxi, P.precision};
  std::lock_guard<std::mutex> lock(tune_mutex());
  auto it = tune_cache().find(key);
  if (it != tune_cache().end()) {
    P.kline_L = it->second.kline_L;
    P.st_cells = it->second.st_cells;
    return WG_OK;
  }
  // the tuning launches are not part of any solve: keep the profiler's counters as they are
  const bool prof_on = P.prof.on;
  long long launches[PROF_N];
  for (int i = 0; i < PROF_N; ++i) launches[i] = P.prof.launches[i];
  P.prof.on = false;
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  const long long N = P.N, n = N * P.batch;
  if (e == cudaSuccess)
    e = mixed ? cudaMemsetAsync(P.mx.d, 0, sizeof(float2) * n, P.stream)
              : cudaMemsetAsync(P.w, 0, sizeof(double2) * n, P.stream);
  const int reps = 5;
  TuneChoice best{P.kline_L, P.st_cells};
  float best_ms = 1e30f;
  for (int L : kline::chunk_len_candidates(P.s.n_el)) {
    if (e != cudaSuccess) break;
    P.kline_L = L;
    const float ms = time_ms(P, a, b, [&]() {
      return mixed ? launch_precondition_mixed(P, P.mx.d, N, P.mx.z, P.mx.zb16, nullptr)
                   : launch_precondition(P, P.w, N, P.z);
    }, reps, e);
    if (e == cudaSuccess && ms < best_ms) {
      best_ms = ms;
      best.kline_L = L;
    }
  }
  if (mixed && e == cudaSuccess) {
    e = cudaMemsetAsync(P.mx.xh, 0, sizeof(float2) * (size_t)P.s.nxi * P.ncols, P.stream);
    best_ms = 1e30f;
    for (int cells : {4, 2}) {
      if (e != cudaSuccess) break;
      P.st_cells = cells;
      const float ms = time_ms(P, a, b, [&]() { return launch_stencil_mixed(P); }, reps, e);
      if (e == cudaSuccess && ms < best_ms) {
        best_ms = ms;
        best.st_cells = cells;
      }
    }
  }
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  for (int i = 0; i < PROF_N; ++i) P.prof.launches[i] = launches[i];
  P.prof.on = prof_on;
  P.kline_L = best.kline_L;
  P.st_cells = best.st_cells;
  if (e != cudaSuccess) {
    P.err = std::string("autotuner: ") + cudaGetErrorString(e);
    return WG_ERR_CUDA;
  }
  tune_cache()[key] = best;
  return WG_OK;
}

}  // namespace wg
