// Serving runtime: continuous batching of self-consistent bias points (host C++).
//
// The reference runs an I-V sweep as one bias after another
// (RTD/solve2D_rtd_self_consistent.m: the bias loop around the Gummel iteration,
// each bias seeded by the previous one).  Here every bias point is a request:
//   - requests of one discretisation shape share a handle of max_slots problems;
//     one worker thread per handle owns it and its CUDA stream;
//   - between two Gummel iterations the worker admits queued requests into free
//     slots (the running slots keep their state and iterate on), and retires each
//     slot the moment its own loop ends: continuous batching, not a queue;
//   - handles of different shapes run concurrently on their own streams;
//   - a handle is created only when its estimated bytes fit the device-memory
//     budget beside the live handles; an idle handle is released when another
//     shape waits for memory;
//   - warm start: the nearest finished bias of the same device seeds the
//     potential (phi_seed + phi0_new - phi0_seed); if that bias' slot is free its
//     Wigner function is still resident and seeds the transport solve too.
// Every slot's computation is independent of the others in its handle, so a
// request run alone and inside a mix gives the same result (warm starts aside).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "problem.h"

namespace {

using Clock = std::chrono::steady_clock;

struct ReqData {
  wg_params prm{};
  int nx = 0;
  std::vector<double> x_nm, m_kg, vc, nd, eps, phi0;
  double me_z = 0, temp = 0, bias = 0, ef_offset = 0, dy_nm = 0;
  long long key = 0;
};

struct Req {
  long long id = 0;
  ReqData d;
  int state = WG_REQ_QUEUED;
  int klass = -1, slot = -1, warm = 0;
  double t_submit = 0, t_admit = 0, t_done = 0;
  wg_gummel_info info{};
  std::string err;
  std::vector<double> phi, n, j;
};

// A finished bias of a device, the seed of later neighbours.
struct Seed {
  double bias = 0;
  std::vector<double> phi, phi0;
  int slot = -1;   // slot still holding its Wigner function, -1 once overwritten
};

struct Slot {
  Req* req = nullptr;  // running request
};

struct Klass {
  int index = 0;
  wg_params prm{};
  int slots = 0;
  double bytes = 0;
  double bytes1 = 0, bytes_per_slot = 0;   // affine byte estimate of a handle: bytes1 + (s - 1) * per_slot
  bool alive = false;        // a worker thread serves this shape
  bool has_handle = false;
  std::deque<Req*> queue;
  std::map<long long, std::vector<Seed>> seeds;   // device_key -> finished biases
};

bool same_shape(const wg_params& a, const wg_params& b) {
  return a.n_el == b.n_el && a.n_local == b.n_local && a.nk == b.nk && a.n_xi == b.n_xi && a.l_xi == b.l_xi &&
         a.m_diff == b.m_diff && a.mpc == b.mpc;
}

}  // namespace

struct wg_server {
  wg_server_opts o{};
  std::mutex mu;
  std::condition_variable cv;
  bool stop = false;
  int live_workers = 0;
  std::map<long long, std::unique_ptr<Req>> reqs;
  std::vector<std::unique_ptr<Klass>> classes;
  long long next_id = 1;
  double bytes = 0, bytes_peak = 0;
  long long n_done = 0, n_failed = 0;
  Clock::time_point t0 = Clock::now();
  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

// Under the lock: a request leaves with an error.
void fail_request(wg_server* S, Req* R, const std::string& msg) {
  R->state = WG_REQ_FAILED;
  R->err = msg;
  R->t_done = S->now();
  ++S->n_failed;
}

void worker(wg_server* S, Klass* K) {
  std::unique_lock<std::mutex> lk(S->mu);
  // 1. a handle within the memory budget: as many slots as fit, waiting for memory if none does
  for (;;) {
    if (K->queue.empty()) {
      K->alive = false;
      --S->live_workers;
      S->cv.notify_all();
      return;
    }
    int slots = 0;
    double need = 0;
    for (int s = S->o.max_slots; s >= 1; --s) {
      const double b = K->bytes1 + (s - 1) * K->bytes_per_slot;
      if (S->bytes + b <= S->o.mem_budget_bytes) {
        slots = s;
        need = b;
        break;
      }
    }
    if (slots > 0) {
      K->slots = slots;
      K->bytes = need;
      S->bytes += need;
      S->bytes_peak = std::max(S->bytes_peak, S->bytes);
      break;
    }
    bool others = false;
    for (auto& k2 : S->classes) others |= k2.get() != K && k2->has_handle;
    if (!others) {
      // not even one slot fits the whole budget
      while (!K->queue.empty()) {
        fail_request(S, K->queue.front(), "a single problem of this shape exceeds the device-memory budget");
        K->queue.pop_front();
      }
      continue;
    }
    S->cv.wait_for(lk, std::chrono::milliseconds(10));
  }
  K->has_handle = true;
  lk.unlock();
  wg_problem* h = nullptr;
  int rc = wg_problem_create(&K->prm, K->slots, &h);
  lk.lock();
  if (rc != WG_OK) {
    const std::string msg = std::string("handle creation failed: ") + wg_global_error();
    while (!K->queue.empty()) {
      fail_request(S, K->queue.front(), msg);
      K->queue.pop_front();
    }
    S->bytes -= K->bytes;
    K->has_handle = false;
    K->alive = false;
    --S->live_workers;
    S->cv.notify_all();
    return;
  }
  wg::Problem& P = h->P;
  std::vector<Slot> slot(K->slots);
  const wg_gummel_opts go = S->o.gummel;
  Clock::time_point idle_since = Clock::now();
  bool broken = false;

  // 2. serve: admit, iterate, retire
  for (;;) {
    struct Admit {
      Req* R;
      int slot;
      int warm;
      std::vector<double> phi0;
    };
    std::vector<Admit> adm;
    while (!broken && !K->queue.empty()) {
      Req* R = K->queue.front();
      Seed* seed = nullptr;
      if (S->o.warm_start) {
        auto it = K->seeds.find(R->d.key);
        if (it != K->seeds.end())
          for (Seed& f : it->second)
            if (!seed || std::fabs(f.bias - R->d.bias) < std::fabs(seed->bias - R->d.bias)) seed = &f;
      }
      int best = -1, warm = 0;
      if (seed && seed->slot >= 0 && !slot[seed->slot].req) {
        best = seed->slot;
        warm = 2;
      } else {
        // a free slot, preferring one whose resident state no seed points at
        for (int b = 0; b < K->slots && best < 0; ++b) {
          if (slot[b].req) continue;
          bool held = false;
          for (auto& kv : K->seeds)
            for (Seed& f : kv.second) held |= f.slot == b;
          if (!held) best = b;
        }
        for (int b = 0; b < K->slots && best < 0; ++b)
          if (!slot[b].req) best = b;
        if (best >= 0 && seed) warm = 1;
      }
      if (best < 0) break;
      K->queue.pop_front();
      std::vector<double> phi0 = R->d.phi0;
      if (warm)
        for (size_t i = 0; i < phi0.size(); ++i) phi0[i] = seed->phi[i] + (R->d.phi0[i] - seed->phi0[i]);
      // the slot's resident state is consumed (warm == 2) or overwritten
      for (auto& kv : K->seeds)
        for (Seed& f : kv.second)
          if (f.slot == best) f.slot = -1;
      slot[best].req = R;
      R->state = WG_REQ_RUNNING;
      R->klass = K->index;
      R->slot = best;
      R->warm = warm;
      R->t_admit = S->now();
      adm.push_back({R, best, warm, std::move(phi0)});
    }
    int running = 0;
    for (const Slot& sl : slot) running += sl.req != nullptr;
    if (running == 0) {
      if (broken || (S->stop && K->queue.empty())) break;
      bool wanted = false;
      for (auto& k2 : S->classes) wanted |= k2.get() != K && !k2->has_handle && !k2->queue.empty();
      const double idle = std::chrono::duration<double>(Clock::now() - idle_since).count();
      if (K->queue.empty() && wanted && idle >= S->o.idle_release_s) break;
      S->cv.wait_for(lk, std::chrono::milliseconds(5));
      continue;
    }
    lk.unlock();
    // device set-up of the admitted requests (only this thread touches the handle)
    std::vector<std::pair<Req*, std::string>> setup_failed;
    for (Admit& a : adm) {
      const ReqData& d = a.R->d;
      wg_device dev{d.nx, d.x_nm.data(), d.m_kg.data(), d.me_z, d.temp};
      wg_rtd_1d rtd{d.vc.data(), d.nd.data(), d.eps.data(), a.phi0.data(), d.bias, d.ef_offset, d.dy_nm};
      int r = wg_gummel_set(h, a.slot, &dev, &rtd);
      if (r == WG_OK) r = wg::gummel_start(P, a.slot, go, /*warm=*/a.warm == 2, /*from_phi0=*/false);
      if (r != WG_OK) {
        setup_failed.push_back({a.R, std::string("request set-up failed: ") + wg_last_error(h)});
        P.gh[a.slot].running = 0;
      }
    }
    int still = 0;
    rc = wg::gummel_iterate(P, go, &still);
    // gather the slots whose loop ended
    struct Done {
      int slot;
      std::vector<double> phi, n, j;
      wg_gummel_info info;
    };
    std::vector<Done> done;
    if (rc == WG_OK) {
      for (int b = 0; b < K->slots; ++b) {
        if (!slot[b].req || P.gh[b].running) continue;
        bool failed_setup = false;
        for (auto& f : setup_failed) failed_setup |= f.first == slot[b].req;
        if (failed_setup) continue;
        Done d;
        d.slot = b;
        d.phi.resize(P.nx);
        d.n.resize((size_t)P.s.n_el * P.s.nK);
        d.j.resize(d.n.size());
        if (wg::gummel_get(P, b, d.phi.data(), d.n.data(), d.j.data()) != WG_OK) {
          rc = WG_ERR_CUDA;
          break;
        }
        d.info = P.gh[b].info;
        done.push_back(std::move(d));
      }
    }
    lk.lock();
    for (auto& f : setup_failed) {
      fail_request(S, f.first, f.second);
      slot[f.first->slot].req = nullptr;
    }
    if (rc != WG_OK) {
      const std::string msg = std::string("device error: ") + P.err;
      for (Slot& sl : slot)
        if (sl.req) {
          fail_request(S, sl.req, msg);
          sl.req = nullptr;
        }
      broken = true;
    } else {
      for (Done& d : done) {
        Req* R = slot[d.slot].req;
        R->info = d.info;
        R->phi = std::move(d.phi);
        R->n = std::move(d.n);
        R->j = std::move(d.j);
        R->state = WG_REQ_DONE;
        R->t_done = S->now();
        ++S->n_done;
        if (d.info.status == WG_GUMMEL_CONVERGED) {
          Seed sd;
          sd.bias = R->d.bias;
          sd.phi = R->phi;
          sd.phi0 = R->d.phi0;
          sd.slot = d.slot;
          K->seeds[R->d.key].push_back(std::move(sd));
        }
        slot[d.slot].req = nullptr;
      }
    }
    S->cv.notify_all();
    bool any = false;
    for (const Slot& sl : slot) any |= sl.req != nullptr;
    if (!any) idle_since = Clock::now();
  }
  // 3. release the handle
  K->has_handle = false;
  K->seeds.clear();
  lk.unlock();
  wg_problem_destroy(h);
  lk.lock();
  S->bytes -= K->bytes;
  // requests that arrived while the handle was being released get a new worker
  if (!K->queue.empty() && !S->stop) {
    std::thread(worker, S, K).detach();   // live_workers stays counted for the new thread
  } else {
    K->alive = false;
    --S->live_workers;
  }
  S->cv.notify_all();
}

}  // namespace

extern "C" {

int wg_server_create(const wg_server_opts* opts, wg_server** out) {
  if (!out) return WG_ERR_ARG;
  *out = nullptr;
  wg_server* S = new (std::nothrow) wg_server();
  if (!S) return WG_ERR_OOM;
  if (opts) S->o = *opts;
  if (S->o.mem_budget_bytes <= 0) S->o.mem_budget_bytes = 150e9;
  if (S->o.max_slots <= 0) S->o.max_slots = 8;
  if (S->o.idle_release_s <= 0) S->o.idle_release_s = 0.5;
  if (S->o.precision != WG_PREC_FP64 && S->o.precision != WG_PREC_MIXED) {
    delete S;
    return WG_ERR_ARG;
  }
  *out = S;
  return WG_OK;
}

int wg_server_submit(wg_server* S, const wg_request* r, long long* id) {
  if (!S || !r || !id) return WG_ERR_ARG;
  const int nx = r->n_el * (r->n_local - 1) + 1;
  if (r->n_el < 1 || r->n_local < 2 || r->dev.nx != nx || !r->dev.x_nm || !r->dev.m_kg || !r->rtd.vc_ev ||
      !r->rtd.nd_m3 || !r->rtd.eps_r || !r->rtd.phi0)
    return WG_ERR_ARG;
  auto R = std::make_unique<Req>();
  ReqData& d = R->d;
  d.prm.n_el = r->n_el;
  d.prm.n_local = r->n_local;
  d.prm.nk = r->nk;
  d.prm.n_xi = r->n_xi;
  d.prm.l_xi = r->l_xi;
  d.prm.m_diff = r->m_diff;
  d.prm.mpc = r->mpc;
  d.prm.precision = S->o.precision;
  d.prm.restart = S->o.restart;
  d.prm.inner_restart = S->o.inner_restart;
  d.prm.inner_tol = S->o.inner_tol;
  d.prm.reorth = S->o.reorth;
  d.prm.inner_reorth = S->o.inner_reorth;
  d.nx = nx;
  d.x_nm.assign(r->dev.x_nm, r->dev.x_nm + nx);
  d.m_kg.assign(r->dev.m_kg, r->dev.m_kg + nx);
  d.vc.assign(r->rtd.vc_ev, r->rtd.vc_ev + nx);
  d.nd.assign(r->rtd.nd_m3, r->rtd.nd_m3 + nx);
  d.eps.assign(r->rtd.eps_r, r->rtd.eps_r + nx);
  d.phi0.assign(r->rtd.phi0, r->rtd.phi0 + nx);
  d.me_z = r->dev.me_z;
  d.temp = r->dev.temp;
  d.bias = r->rtd.bias;
  d.ef_offset = r->rtd.ef_offset;
  d.dy_nm = r->rtd.dy_nm;
  d.key = r->device_key;
  double probe = 0;
  if (wg_problem_bytes(&d.prm, 1, &probe) != WG_OK) return WG_ERR_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->stop) return WG_ERR_ARG;
  R->id = S->next_id++;
  R->t_submit = S->now();
  Req* raw = R.get();
  *id = R->id;
  S->reqs[R->id] = std::move(R);
  Klass* K = nullptr;
  for (auto& k : S->classes)
    if (same_shape(k->prm, d.prm)) K = k.get();
  if (!K) {
    S->classes.push_back(std::make_unique<Klass>());
    K = S->classes.back().get();
    K->index = (int)S->classes.size() - 1;
    K->prm = d.prm;
    double b2 = 0;
    wg_problem_bytes(&d.prm, 2, &b2);
    K->bytes1 = probe;
    K->bytes_per_slot = b2 - probe;
  }
  K->queue.push_back(raw);
  if (!K->alive) {
    K->alive = true;
    ++S->live_workers;
    std::thread(worker, S, K).detach();
  }
  S->cv.notify_all();
  return WG_OK;
}

int wg_server_wait(wg_server* S, long long id, double timeout_s, wg_request_status* st) {
  if (!S || !st) return WG_ERR_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->reqs.find(id);
  if (it == S->reqs.end()) return WG_ERR_ARG;
  Req* R = it->second.get();
  auto finished = [&] { return R->state == WG_REQ_DONE || R->state == WG_REQ_FAILED; };
  if (timeout_s < 0)
    S->cv.wait(lk, finished);
  else
    S->cv.wait_for(lk, std::chrono::duration<double>(timeout_s), finished);
  std::memset(st, 0, sizeof(*st));
  st->state = R->state;
  st->info = R->info;
  st->t_submit = R->t_submit;
  st->t_admit = R->t_admit;
  st->t_done = R->t_done;
  st->handle = R->klass;
  st->slot = R->slot;
  st->warm = R->warm;
  std::strncpy(st->error, R->err.c_str(), sizeof(st->error) - 1);
  return finished() ? WG_OK : WG_ERR_TIMEOUT;
}

int wg_server_result(wg_server* S, long long id, double* phi, double* n_dg, double* j) {
  if (!S) return WG_ERR_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->reqs.find(id);
  if (it == S->reqs.end() || it->second->state != WG_REQ_DONE) return WG_ERR_ARG;
  const Req& R = *it->second;
  if (phi) std::copy(R.phi.begin(), R.phi.end(), phi);
  if (n_dg) std::copy(R.n.begin(), R.n.end(), n_dg);
  if (j) std::copy(R.j.begin(), R.j.end(), j);
  return WG_OK;
}

int wg_server_release(wg_server* S, long long id) {
  if (!S) return WG_ERR_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->reqs.find(id);
  if (it == S->reqs.end()) return WG_ERR_ARG;
  if (it->second->state != WG_REQ_DONE && it->second->state != WG_REQ_FAILED) return WG_ERR_ARG;
  S->reqs.erase(it);
  return WG_OK;
}

int wg_server_stats_get(wg_server* S, wg_server_stats* st) {
  if (!S || !st) return WG_ERR_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  std::memset(st, 0, sizeof(*st));
  for (auto& k : S->classes) st->handles += k->has_handle ? 1 : 0;
  for (auto& kv : S->reqs) {
    st->queued += kv.second->state == WG_REQ_QUEUED;
    st->running += kv.second->state == WG_REQ_RUNNING;
  }
  st->done = S->n_done;
  st->failed = S->n_failed;
  st->device_bytes = S->bytes;
  st->device_bytes_peak = S->bytes_peak;
  return WG_OK;
}

int wg_server_destroy(wg_server* S) {
  if (!S) return WG_ERR_ARG;
  {
    std::unique_lock<std::mutex> lk(S->mu);
    S->stop = true;
    S->cv.notify_all();
    S->cv.wait(lk, [&] { return S->live_workers == 0; });
  }
  delete S;
  return WG_OK;
}

}  // extern "C"
