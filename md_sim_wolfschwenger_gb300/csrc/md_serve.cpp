// md_serve.cpp -- request serving on top of the C ABI: continuous batching of
// independent simulations of different N, field programs and step counts
// under a device-memory budget, plus md_init_system (host-side initial
// systems).  Host code only; every device operation goes through the
// library's own C ABI (md_ctx_*, md_batch_*).
//
// Loop (md_serve_run), two threads:
//   admitting thread: in arrival order, as batch slots and the memory budget
//      allow, build each request's system on the host (prepared ahead on
//      worker threads: sizes, placement, Ewald parameters), create its
//      context, upload the state, set the Ewald parameters, and hand the
//      context over;
//   this thread: wait for the round in flight; systems that have run all
//      their steps are read back (final m_z, state checksum), leave the batch
//      and free their memory; the contexts handed over join the batch (it
//      re-packs its launches) and the next round starts.
// A round runs at most round_steps steps and ends early when a system
// finishes, so no system runs past its own step count.  Creating a context
// costs milliseconds (and waits on the busy GPU in places): on the loop's own
// thread it delayed the next round whenever several requests arrived at once.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <future>
#include <mutex>
#include <map>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/md_gb300.h"
#include "md_err.h"
#include "md_host.h"
#include <nvtx3/nvToolsExt.h>

namespace {

using Clock = std::chrono::steady_clock;

struct Live {
  int64_t req;
  md_ctx* ctx;
  int64_t id;       // batch id (0 until it joined)
  int64_t bytes;    // device bytes held
  double lBox;
};

// Configuration of one request: the base keys with the request's field,
// volume fraction, seed and particle count.
md_config request_config(const md_config& base, const md_request& q) {
  md_config c = base;
  c.numbPartOverride = q.n;
  c.volFrac = q.volFrac;
  c.seed = (int64_t)q.seed;
  c.fieldKind = q.fieldKind;
  if (q.fieldKind == MD_FIELD_SIN) {
    c.fieldAmp = q.fieldAmp;
    c.fieldFreq = q.fieldFreq;
  } else {
    c.magFluxDens = q.fieldAmp;
    c.tMag = 1e300;
  }
  c.noise = MD_NOISE_PHILOX;
  md_config_derive(&c);
  return c;
}

// A request's system on the host, with its Ewald parameters from the error
// model and an upper estimate of the device memory it will hold.
struct HostSys {
  int64_t req = -1;
  md_config cfg{};
  std::vector<double> rMag, pos, mm, ea;
  double L = 0, alpha = 0, rc = 0, est = 0;
  int64_t kc = 0;
};

// Device bytes of a mixed-precision context: per-particle state, stage and
// work arrays (~620 B), phase tables, the neighbour list (uniform-density
// estimate with the allocator's margin), k-space arrays and records.
double estimate_bytes(int64_t n, double rc_box, int64_t kc, int64_t steps) {
  const double pi = 3.141592653589793, N = (double)n;
  const double rl = rc_box * 1.02;
  const double nbr = 4.0 * (1.3 * std::min(N * N * 4.0 / 3.0 * pi * rl * rl * rl, N * (N - 1)) + 64.0 * N);
  const double nk = 2.0 * pi / 3.0 * std::pow((double)kc + 1.0, 3.0) + 64.0;
  const double nchunk = std::max(1.0, std::ceil(N / 512.0)) + 8.0;
  const double cells = 8.0 * std::pow(std::max(1.0, std::ceil(2.0 / rc_box)), 3.0);
  return 1.1 * (620.0 * N + 24.0 * (kc + 1) * N + nbr + nk * (80.0 + 16.0 * nchunk) + cells + 64.0 * (steps + 1024) +
                (1 << 20));
}

int prepare_host(const md_config& base, const md_request& q, int64_t qi, HostSys* h) {
  h->req = qi;
  h->cfg = request_config(base, q);
  const size_t n = (size_t)q.n;
  h->rMag.resize(n);
  h->pos.resize(3 * n);
  h->mm.resize(3 * n);
  h->ea.resize(3 * n);
  int st = md_init_system(&h->cfg, q.n, q.seed, h->rMag.data(), nullptr, h->pos.data(), h->mm.data(), h->ea.data(),
                          &h->L);
  if (st) return st;
  double L2 = 0;
  if ((st = md_ewald_params_host(&h->cfg, q.n, h->rMag.data(), nullptr, 0.0, &h->alpha, &h->rc, &h->kc, nullptr,
                                 nullptr, &L2)))
    return st;
  h->est = estimate_bytes(q.n, h->rc / h->L, h->kc, q.steps);
  return MD_OK;
}

// Context with state and Ewald parameters (not yet batched).
int create_device(const HostSys& h, const md_request& q, int autotune, Live* out) {
  md_ctx* ctx = nullptr;
  int st = md_ctx_create(&h.cfg, q.n, MD_PREC_MIXED, &ctx);
  if (st) return st;
  auto fail = [&](int s) {
    md_ctx_destroy(ctx);
    return s;
  };
  if ((st = md_set_particles(ctx, h.rMag.data(), nullptr))) return fail(st);
  if ((st = md_state_upload(ctx, h.pos.data(), h.mm.data(), h.ea.data(), 1))) return fail(st);
  if (autotune) {
    double alpha = 0, rc = 0;
    int64_t kc = 0;
    int hit = 0;
    if ((st = md_autotune_ewald_cached(ctx, q.volFrac, &alpha, &rc, &kc, &hit))) return fail(st);
  } else if ((st = md_set_ewald(ctx, h.alpha, h.rc, h.kc))) {
    return fail(st);
  }
  if ((st = md_set_noise(ctx, MD_NOISE_PHILOX, q.seed))) return fail(st);
  int64_t bytes = 0;
  md_ctx_device_bytes(ctx, &bytes);
  out->req = h.req;
  out->ctx = ctx;
  out->id = 0;
  out->bytes = bytes + 64 * (q.steps + 1024);  // + the per-step records
  out->lBox = h.L;
  return MD_OK;
}

// Final observables of a finished system.
void harvest(Live& s, const md_request& q, md_request_result* r) {
  const size_t n = (size_t)q.n;
  std::vector<double> pos(3 * n), mm(3 * n), ea(3 * n);
  r->status = md_state_download(s.ctx, pos.data(), mm.data(), ea.data());
  double sum = 0;
  for (size_t i = 0; i < 3 * n; i++) sum += pos[i] / s.lBox + mm[i] + ea[i];
  r->checksum = sum;
  int64_t nrec = 0;
  md_num_records(s.ctx, &nrec);
  double rec[8] = {0};
  if (nrec > 0 && md_records(s.ctx, nrec - 1, 1, rec) == MD_OK) r->mz = rec[1];
  r->steps_done = nrec;
}

}  // namespace

extern "C" {

int md_init_system(const md_config* cfg, int64_t n, uint64_t seed, double* rMag, double* rHydr, double* pos,
                   double* mm, double* ea, double* lBox) {
  if (!cfg || !lBox) return set_err(nullptr, MD_ERR_INVALID, "null argument");
  std::string e;
  const int st = mdh::init_system(*cfg, n, seed, rMag, rHydr, pos, mm, ea, lBox, &e);
  return st ? set_err(nullptr, st, "%s", e.c_str()) : MD_OK;
}

int md_serve_run(const md_config* base, const md_request* reqs, int64_t nreq, const md_serve_opts* opts,
                 md_request_result* results, md_serve_stats* stats) {
  nvtxRangePushA("md_serve_run");
  struct Pop {
    ~Pop() { nvtxRangePop(); }
  } pop;
  if (!base || (!reqs && nreq) || nreq < 0 || !opts || (!results && nreq))
    return set_err(nullptr, MD_ERR_INVALID, "null argument");
  if (opts->max_systems < 1 || opts->round_steps < 1 || !(opts->hbm_budget > 0))
    return set_err(nullptr, MD_ERR_INVALID, "bad serving options");
  for (int64_t i = 0; i < nreq; i++) {
    const md_request& q = reqs[i];
    if (q.n < 2 || q.steps < 1 || !(q.dt > 0) || !(q.volFrac > 0) || !(q.arrival >= 0))
      return set_err(nullptr, MD_ERR_INVALID, "request %lld: bad n, steps, dt, volFrac or arrival", (long long)i);
    results[i] = md_request_result{};
    results[i].status = -1;
  }
  md_serve_stats S{};
  md_batch* b = nullptr;
  int st = md_batch_create(opts->max_systems, &b);
  if (st) return st;
  std::vector<int64_t> order((size_t)nreq);
  for (int64_t i = 0; i < nreq; i++) order[(size_t)i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t c) { return reqs[a].arrival < reqs[c].arrival; });

  const Clock::time_point t0 = Clock::now();
  auto now = [&] { return std::chrono::duration<double>(Clock::now() - t0).count(); };

  // State shared by the admitting thread and this one (under mu): the
  // contexts created and not yet finished hold `used` bytes and `held` batch
  // slots; `ready` hands created contexts over in arrival order.
  std::mutex mu;
  std::condition_variable cv_admit, cv_loop;
  std::deque<Live> ready;
  double used = 0;
  int64_t held = 0, completed = 0;
  bool stop = false;
  double admit_s = 0;

  // Admission on its own thread: host systems (prepared ahead on worker
  // threads), contexts, state upload and Ewald parameters, in arrival order,
  // while this thread keeps the packed rounds going (creating a context costs
  // milliseconds and waits on the busy GPU in places; on the loop's thread it
  // delayed the next round whenever several requests arrived together).
  std::thread admitter([&] {
    using Prep = std::pair<int, HostSys>;
    std::map<int64_t, std::future<Prep>> ahead;
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t nahead = std::min<size_t>(16, std::max<size_t>(1, hw / 2));
    HostSys pend;  // the next request's host system, kept while it waits for memory
    auto reject = [&](int64_t qi, int as) {  // this request cannot run: report it
      std::lock_guard<std::mutex> lk(mu);
      results[qi].status = as;
      results[qi].finished = now();
      results[qi].latency = results[qi].finished - reqs[qi].arrival;
      completed++;
      cv_loop.notify_all();
    };
    for (size_t next = 0; next < order.size();) {
      {
        std::lock_guard<std::mutex> lk(mu);
        if (stop) break;
      }
      const int64_t qi = order[next];
      const md_request& q = reqs[qi];
      if (opts->realtime && q.arrival > now()) {  // wait for the arrival (or the end)
        std::unique_lock<std::mutex> lk(mu);
        cv_admit.wait_for(lk, std::chrono::duration<double>(std::min(q.arrival - now(), 0.05)), [&] { return stop; });
        if (stop) break;
        continue;
      }
      for (size_t k = next; k < order.size() && k < next + nahead; k++) {
        const int64_t qk = order[k];
        if (opts->realtime && reqs[qk].arrival > now()) break;
        if (qk != pend.req && !ahead.count(qk))
          ahead.emplace(qk, std::async(std::launch::async, [base, reqs, qk]() {
            Prep r;
            r.first = prepare_host(*base, reqs[qk], qk, &r.second);
            return r;
          }));
      }
      if (pend.req != qi) {
        pend = HostSys();
        int hs;
        auto it = ahead.find(qi);
        if (it != ahead.end()) {
          Prep r = it->second.get();
          ahead.erase(it);
          hs = r.first;
          pend = std::move(r.second);
        } else {
          hs = prepare_host(*base, q, qi, &pend);
        }
        if (hs) {
          reject(qi, hs);
          pend = HostSys();
          next++;
          continue;
        }
      }
      bool alone;
      {  // a batch slot and room in the budget (a request that would run alone always tries)
        std::unique_lock<std::mutex> lk(mu);
        cv_admit.wait(lk, [&] {
          return stop || (held < opts->max_systems && (used + pend.est <= opts->hbm_budget || held == 0));
        });
        if (stop) break;
        alone = held == 0;
      }
      Live sys{qi, nullptr, 0, 0, 0};
      const double ta = now();
      const int as = create_device(pend, q, opts->autotune, &sys);
      admit_s += now() - ta;
      if (as) {
        reject(qi, as);
        pend = HostSys();
        next++;
        continue;
      }
      bool wait_memory = false;
      {
        std::lock_guard<std::mutex> lk(mu);
        if (used + (double)sys.bytes > opts->hbm_budget && !(alone && held == 0)) {
          wait_memory = true;  // the estimate was low: the actual bytes decide
        } else if (used + (double)sys.bytes > opts->hbm_budget) {
          wait_memory = false;
        } else {
          results[qi].admitted = now();
          used += (double)sys.bytes;
          held++;
          S.peak_bytes = std::max(S.peak_bytes, used);
          ready.push_back(sys);
          cv_loop.notify_all();
          pend = HostSys();
          next++;
          continue;
        }
      }
      md_ctx_destroy(sys.ctx);
      if (!wait_memory) {  // alone and still over the budget
        reject(qi, set_err(nullptr, MD_ERR_NOMEM, "request %lld needs more than the memory budget", (long long)qi));
        pend = HostSys();
        next++;
        continue;
      }
      {  // wait until a finished system frees memory, then create it again
        std::unique_lock<std::mutex> lk(mu);
        const double u0 = used;
        const int64_t h0 = held;
        cv_admit.wait(lk, [&] { return stop || used < u0 || held < h0; });
        if (stop) break;
      }
    }
  });

  std::vector<Live> live, staged;
  bool in_flight = false;
  int fatal = MD_OK;
  auto finish_request = [&](Live& s, int status) {
    md_request_result* r = &results[s.req];
    if (status == MD_OK)
      harvest(s, reqs[s.req], r);  // sets the status of the read-back
    else
      r->status = status;
    r->finished = now();
    r->latency = r->finished - reqs[s.req].arrival;
    r->device_bytes = s.bytes;
    md_ctx_destroy(s.ctx);
    std::lock_guard<std::mutex> lk(mu);
    used -= (double)s.bytes;
    held--;
    completed++;
    cv_admit.notify_all();
  };

  for (;;) {
    {  // 1. contexts the admitting thread has created join at the next round
      std::lock_guard<std::mutex> lk(mu);
      if (completed >= nreq && !in_flight) break;
      while (!ready.empty()) {
        staged.push_back(ready.front());
        ready.pop_front();
      }
    }
    // 2. the round in flight
    if (in_flight) {
      const int ws = md_batch_wait(b);
      in_flight = false;
      double ms = 0;
      md_batch_info(b, nullptr, nullptr, nullptr, &ms);
      S.gpu_ms += ms;
      S.rounds++;
      for (size_t k = 0; k < live.size();) {
        int64_t left = 0;
        int sst = MD_OK;
        md_batch_remaining(b, live[k].id, &left, &sst);
        if (ws != MD_OK && sst == MD_OK && ws != MD_ERR_NONFINITE) sst = ws;
        if (left <= 0 || sst != MD_OK) {
          md_batch_remove(b, live[k].id);
          finish_request(live[k], sst);
          live.erase(live.begin() + (ptrdiff_t)k);
        } else {
          k++;
        }
      }
      if (ws != MD_OK && ws != MD_ERR_NONFINITE) {
        fatal = ws;
        break;
      }
    }
    // 3. newly admitted systems join
    if (!staged.empty()) S.repacks++;
    for (Live& s : staged) {
      const int as = md_batch_add(b, s.ctx, reqs[s.req].steps, reqs[s.req].dt, &s.id);
      if (as) {
        finish_request(s, as);
        continue;
      }
      live.push_back(s);
    }
    staged.clear();
    S.peak_systems = std::max<int64_t>(S.peak_systems, (int64_t)live.size());
    // 4. the next round, or wait for the next admission
    if (!live.empty()) {
      int64_t k = 0;
      const int ls = md_batch_launch(b, opts->round_steps, &k);
      if (ls) {
        fatal = ls;
        break;
      }
      in_flight = k > 0;
    } else {
      std::unique_lock<std::mutex> lk(mu);
      cv_loop.wait_for(lk, std::chrono::milliseconds(50), [&] { return !ready.empty() || completed >= nreq; });
    }
  }
  {
    std::lock_guard<std::mutex> lk(mu);
    stop = true;
    cv_admit.notify_all();
  }
  admitter.join();
  if (in_flight) md_batch_wait(b);
  for (Live& s : live) finish_request(s, fatal ? fatal : MD_ERR_INVALID);
  for (Live& s : staged) finish_request(s, fatal ? fatal : MD_ERR_INVALID);
  for (Live& s : ready) finish_request(s, fatal ? fatal : MD_ERR_INVALID);
  md_batch_destroy(b);
  S.wall = now();
  S.admit_ms = 1e3 * admit_s;
  for (int64_t i = 0; i < nreq; i++)
    if (results[i].status == MD_OK) S.particle_steps += (double)reqs[i].n * (double)reqs[i].steps;
  if (stats) *stats = S;
  return fatal;
}

}  // extern "C"
