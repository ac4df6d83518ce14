// Continuous-batching request server over one or several contexts (C ABI in include/fideslib_gb300.h).
//
// The reference has no serving layer (its API runs one op per call, api/CryptoContext.cpp); this is the
// request loop the engine was shaped for.  Clients submit independent requests from any thread, each to one of
// the server's rings (contexts: for example N = 2^15 and N = 2^16 side by side); one worker thread owns every
// context.  Whenever the GPU can take more work, the worker admits, in arrival order and whatever their ring,
// every pending request that fits the one memory budget (output ciphertext + key-switch workspace, counted per
// request with its ring's shape) up to max_batch, runs each ring's share through fides_eval_batch on that
// ring (one launch per pipeline stage for all of them, at their own levels; the rings' batches overlap on the
// device), and keeps up to max_inflight batches in flight, each on a stream of its own (a lane), so requests that
// arrive while a batch runs are admitted into the next one as soon as a lane and memory free up and run beside
// it on the GPU instead of queueing behind it.  A released result is freed once no pending request and no batch in
// flight reads it (a client may release a result right after submitting requests that take it as an operand), and
// completed batches retire in any order.  Bootstrap requests (FIDES_OP_BOOTSTRAP, with the plan set
// by fides_server_set_bootstrap_plan) admitted together run as one fides_eval_bootstrap_batch.  Each request's
// latency is stamped on the host from submit to the completion of its batch's CUDA event.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/fideslib_gb300.h"

namespace fgb {
int set_last_error(int code, const char* msg);
cudaStream_t swap_ctx_stream(fides_ctx* ctx, cudaStream_t s);
}

namespace {

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Req {
  fides_op op{};
  uint32_t ring = 0;
  double t_submit = 0, t_done = 0;
  size_t footprint = 0;
  int state = 0;  // 0 pending, 1 running, 2 done
  int rc = 0;
};

struct InFlight {
  std::vector<cudaEvent_t> evs;  // one per ring that took part
  std::vector<uint64_t> tickets;
  std::vector<std::pair<uint32_t, uint32_t>> reads;  // (ring, handle) operands of its requests
  size_t footprint;
  uint32_t lane;
};

struct Ring {
  fides_ctx* ctx = nullptr;
  uint32_t N = 0, np = 0, nq = 0, alpha = 1;
  std::vector<cudaStream_t> lanes;  // one stream per in-flight batch (made by the worker)
};

struct DeferredFree {
  uint32_t ring, handle;
};

}  // namespace

struct fides_server {
  std::vector<Ring> rings;
  fides_server_config cfg{};
  bool has_plan = false;
  fides_bootstrap_plan plan{};  // cheb_coeffs points into coeffs
  std::vector<double> coeffs;
  int device = 0;  // current at fides_server_create: the contexts' device
  std::thread worker;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<uint64_t> pending;
  std::unordered_map<uint64_t, Req> reqs;
  std::vector<std::pair<uint32_t, uint32_t>> to_free;  // (ring, handle)
  std::vector<double> latencies;
  uint64_t next_ticket = 1, batches = 0, batched_ops = 0;
  double first_submit = -1, last_done = 0;
  bool stop = false;
  std::string error;

  size_t footprint_of(const Req& r) {
    const fides_op& op = r.op;
    const Ring& g = rings[r.ring];
    fides_ct_meta m{};
    if (fides_ct_meta_get(g.ctx, op.a, &m) != FIDES_OK) return 0;
    const size_t S = (size_t)8 * g.N, t = m.towers, np = g.np, beta = (t + g.alpha - 1) / g.alpha;
    size_t limbs = 2 * t;  // output
    if (op.op == FIDES_OP_ROTATE || op.op == FIDES_OP_AUTOMORPHISM || op.op == FIDES_OP_KEY_SWITCH ||
        op.op == FIDES_OP_MULT || op.op == FIDES_OP_SQUARE)
      limbs += t + beta * (t + np) + 2 * (t + np) + 2 * t;
    if (op.op == FIDES_OP_MULT || op.op == FIDES_OP_SQUARE) limbs += 3 * t;
    if (op.op == FIDES_OP_RESCALE) limbs += 2 * t;
    if (op.op == FIDES_OP_BOOTSTRAP)  // estimate: the largest stage holds about 64 ciphertexts at raise_towers
      limbs = (size_t)64 * 2 * plan.raise_towers;
    return limbs * S;
  }

  // Worker loop: admit -> launch (up to max_inflight batches in flight, one per lane) -> retire completed batches.
  void run() {
    cudaSetDevice(device);  // a new thread starts on device 0; the contexts live on the creator's device
    // Batches run on the server's own lanes.  Work the caller queued on a context before the server started
    // (loads of resident ciphertexts and keys) completes first; while the server runs, its worker is the only
    // thread that touches the contexts.
    for (Ring& g : rings) {
      cudaStreamSynchronize((cudaStream_t)fides_ctx_stream(g.ctx));
      g.lanes.assign(cfg.max_inflight_batches, nullptr);
      for (auto& l : g.lanes) cudaStreamCreateWithFlags(&l, cudaStreamNonBlocking);
    }
    std::deque<InFlight> inflight;
    std::vector<DeferredFree> deferred;
    size_t inflight_bytes = 0;
    // A released result is freed (stream-ordered on its context's own stream, which carries no batches) once no
    // pending request and no batch in flight reads it; until then it stays on the deferred list.
    auto flush_frees = [&] {
      if (deferred.empty()) return;
      std::vector<std::pair<uint32_t, uint32_t>> busy;
      for (const InFlight& f : inflight) busy.insert(busy.end(), f.reads.begin(), f.reads.end());
      {
        std::lock_guard<std::mutex> lk(mu);
        for (uint64_t tk : pending) {
          const Req& r = reqs[tk];
          busy.push_back({r.ring, r.op.a});
          busy.push_back({r.ring, r.op.b});
        }
      }
      std::sort(busy.begin(), busy.end());
      size_t k = 0;
      for (const DeferredFree& d : deferred) {
        if (std::binary_search(busy.begin(), busy.end(), std::make_pair(d.ring, d.handle)))
          deferred[k++] = d;
        else
          fides_ct_free(rings[d.ring].ctx, d.handle);
      }
      deferred.resize(k);
    };
    for (;;) {
      std::vector<uint64_t> take;
      std::vector<std::pair<uint32_t, uint32_t>> frees;
      bool idle_wait = false;
      {
        std::unique_lock<std::mutex> lk(mu);
        if (stop && pending.empty() && inflight.empty() && to_free.empty()) {
          for (const DeferredFree& d : deferred) fides_ct_free(rings[d.ring].ctx, d.handle);
          break;
        }
        frees.swap(to_free);
        if (!pending.empty() && inflight.size() < cfg.max_inflight_batches) {
          size_t budget = inflight_bytes;
          while (!pending.empty() && take.size() < cfg.max_batch) {
            Req& r = reqs[pending.front()];
            if (r.footprint == 0) r.footprint = footprint_of(r);  // contexts are only touched by this thread
            const bool first = take.empty() && inflight.empty();
            if (!first && budget + r.footprint > cfg.mem_budget_bytes) break;
            budget += r.footprint;
            r.state = 1;
            take.push_back(pending.front());
            pending.pop_front();
          }
        }
        idle_wait = take.empty() && frees.empty() && inflight.empty();
        if (idle_wait) cv_work.wait(lk, [&] { return stop || !pending.empty() || !to_free.empty(); });
      }
      if (idle_wait) continue;
      for (auto& fr : frees) deferred.push_back(DeferredFree{fr.first, fr.second});
      if (!take.empty()) {
        std::vector<fides_op> ops(take.size());
        std::vector<uint32_t> ring_of(take.size());
        size_t bytes = 0;
        {
          std::lock_guard<std::mutex> lk(mu);
          for (size_t i = 0; i < take.size(); i++) {
            ops[i] = reqs[take[i]].op;
            ring_of[i] = reqs[take[i]].ring;
            bytes += reqs[take[i]].footprint;
          }
        }
        std::vector<int> rcs(ops.size(), FIDES_OK);
        InFlight f;
        for (size_t i = 0; i < ops.size(); i++) {
          f.reads.push_back({ring_of[i], ops[i].a});
          f.reads.push_back({ring_of[i], ops[i].b});
        }
        f.lane = 0;  // the first lane no batch in flight uses (one exists: fewer than max_inflight are in flight)
        for (bool used = true; used; f.lane += used ? 1 : 0) {
          used = false;
          for (const InFlight& o : inflight) used = used || o.lane == f.lane;
        }
        for (uint32_t g = 0; g < rings.size(); g++) {
          fides_ctx* ctx = rings[g].ctx;
          // this ring's bootstrap requests go through fides_eval_bootstrap_batch (all of them in flight
          // together; ring 0 holds the plan), the rest through fides_eval_batch
          std::vector<size_t> bi, oi;
          for (size_t i = 0; i < ops.size(); i++)
            if (ring_of[i] == g) (ops[i].op == FIDES_OP_BOOTSTRAP ? bi : oi).push_back(i);
          if (bi.empty() && oi.empty()) continue;
          cudaStream_t const lane = rings[g].lanes[f.lane];
          cudaStream_t const home = fgb::swap_ctx_stream(ctx, lane);  // every call below orders its work on the lane
          if (!oi.empty()) {
            std::vector<fides_op> sub(oi.size());
            for (size_t k = 0; k < oi.size(); k++) sub[k] = ops[oi[k]];
            const int rc = fides_eval_batch(ctx, sub.data(), (uint32_t)sub.size());
            for (size_t k = 0; k < oi.size(); k++) {
              if (rc != FIDES_OK && sub.size() > 1)  // one bad request must not fail its batch-mates
                rcs[oi[k]] = fides_eval_batch(ctx, &sub[k], 1);
              else
                rcs[oi[k]] = rc;
              ops[oi[k]].out = sub[k].out;
            }
          }
          if (!bi.empty()) {
            std::vector<uint32_t> in(bi.size()), outs(bi.size(), 0);
            for (size_t k = 0; k < bi.size(); k++) in[k] = ops[bi[k]].a;
            const bool plan_ok = has_plan && g == 0;
            const int rc = plan_ok ? fides_eval_bootstrap_batch(ctx, (uint32_t)in.size(), in.data(), &plan, outs.data())
                                   : fgb::set_last_error(FIDES_EINVAL, "no bootstrap plan set for this ring");
            for (size_t k = 0; k < bi.size(); k++) {
              if (rc != FIDES_OK && plan_ok && bi.size() > 1)
                rcs[bi[k]] = fides_eval_bootstrap(ctx, in[k], &plan, &outs[k]);
              else
                rcs[bi[k]] = rc;
              ops[bi[k]].out = outs[k];
            }
          }
          cudaEvent_t ev;
          cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
          cudaEventRecord(ev, lane);
          f.evs.push_back(ev);
          fgb::swap_ctx_stream(ctx, home);
        }
        f.tickets = take;
        f.footprint = bytes;
        {
          std::lock_guard<std::mutex> lk(mu);
          for (size_t i = 0; i < take.size(); i++) {
            Req& r = reqs[take[i]];
            r.rc = rcs[i];
            r.op.out = rcs[i] == FIDES_OK ? ops[i].out : 0;
          }
          batches++;
          batched_ops += take.size();
        }
        inflight_bytes += bytes;
        inflight.push_back(f);
        flush_frees();
        continue;
      }
      flush_frees();
      if (inflight.empty()) continue;
      // Retire a completed batch (the lanes run concurrently, so any of them may finish first).  While all run,
      // keep admitting new arrivals if a lane is free; with every lane busy, wait for the oldest batch.
      bool full;
      {
        std::lock_guard<std::mutex> lk(mu);
        full = inflight.size() >= cfg.max_inflight_batches || stop;
      }
      size_t done = inflight.size();
      for (size_t i = 0; i < inflight.size() && done == inflight.size(); i++) {
        bool busy = false;
        for (cudaEvent_t ev : inflight[i].evs) busy = busy || cudaEventQuery(ev) == cudaErrorNotReady;
        if (!busy) done = i;
      }
      if (done == inflight.size() && !full) {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait_for(lk, std::chrono::microseconds(20), [&] { return !pending.empty() || !to_free.empty(); });
        continue;
      }
      if (done == inflight.size()) done = 0;
      InFlight f = inflight[done];
      inflight.erase(inflight.begin() + (long)done);
      for (cudaEvent_t ev : f.evs) {
        cudaEventSynchronize(ev);
        cudaEventDestroy(ev);
      }
      const double t = now_ms();
      inflight_bytes -= f.footprint;
      flush_frees();  // results released while this batch ran may be free now
      std::lock_guard<std::mutex> lk(mu);
      for (uint64_t tk : f.tickets) {
        Req& r = reqs[tk];
        r.state = 2;
        r.t_done = t;
        latencies.push_back(t - r.t_submit);
      }
      last_done = t;
      cv_done.notify_all();
    }
    for (Ring& g : rings)
      for (cudaStream_t l : g.lanes)
        if (l) cudaStreamDestroy(l);
  }
};

extern "C" {

int fides_server_create_multi(fides_ctx* const* ctxs, uint32_t n, const fides_server_config* cfg,
                              fides_server** out) {
  if (!ctxs || n == 0 || !cfg || !out) return fgb::set_last_error(FIDES_EINVAL, "null argument");
  if (cfg->max_batch < 1 || cfg->max_inflight_batches < 1 || cfg->mem_budget_bytes == 0)
    return fgb::set_last_error(FIDES_EINVAL, "max_batch, max_inflight_batches and mem_budget_bytes must be > 0");
  fides_server* s = new fides_server();
  for (uint32_t g = 0; g < n; g++) {
    fides_ctx_shape shape{};
    if (!ctxs[g] || fides_ctx_get_shape(ctxs[g], &shape) != FIDES_OK) {
      delete s;
      return fgb::set_last_error(FIDES_EINVAL, "null or invalid context");
    }
    for (uint32_t h = 0; h < g; h++)
      if (ctxs[h] == ctxs[g]) {
        delete s;
        return fgb::set_last_error(FIDES_EINVAL, "a context may appear once");
      }
    s->rings.push_back(Ring{ctxs[g], shape.n, shape.np, shape.nq, shape.alpha ? shape.alpha : 1});
  }
  s->cfg = *cfg;
  cudaGetDevice(&s->device);
  s->worker = std::thread([s] { s->run(); });
  *out = s;
  return FIDES_OK;
}

int fides_server_create(fides_ctx* ctx, const fides_server_config* cfg, fides_server** out) {
  if (!ctx) return fgb::set_last_error(FIDES_EINVAL, "null argument");
  return fides_server_create_multi(&ctx, 1, cfg, out);
}

int fides_server_set_bootstrap_plan(fides_server* s, const fides_bootstrap_plan* plan) {
  if (!s || !plan || !plan->cheb_coeffs || plan->cheb_n == 0) return fgb::set_last_error(FIDES_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  if (!s->pending.empty()) return fgb::set_last_error(FIDES_EINVAL, "set the plan before submitting requests");
  s->coeffs.assign(plan->cheb_coeffs, plan->cheb_coeffs + plan->cheb_n);
  s->plan = *plan;
  s->plan.cheb_coeffs = s->coeffs.data();
  s->has_plan = true;
  return FIDES_OK;
}

int fides_server_submit_to(fides_server* s, uint32_t ring, const fides_op* op, uint64_t* ticket) {
  if (!s || !op || !ticket) return fgb::set_last_error(FIDES_EINVAL, "null argument");
  if (ring >= s->rings.size()) return fgb::set_last_error(FIDES_EINVAL, "ring index out of range");
  Req r;
  r.op = *op;
  r.op.out = 0;
  r.ring = ring;
  r.t_submit = now_ms();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    const uint64_t t = s->next_ticket++;
    s->reqs[t] = r;
    s->pending.push_back(t);
    if (s->first_submit < 0) s->first_submit = r.t_submit;
    *ticket = t;
  }
  s->cv_work.notify_one();
  return FIDES_OK;
}

int fides_server_submit(fides_server* s, const fides_op* op, uint64_t* ticket) {
  return fides_server_submit_to(s, 0, op, ticket);
}

int fides_server_wait(fides_server* s, uint64_t ticket, uint32_t* out, double* latency_ms) {
  if (!s) return fgb::set_last_error(FIDES_EINVAL, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return fgb::set_last_error(FIDES_EINVAL, "unknown ticket");
  s->cv_done.wait(lk, [&] { return s->reqs[ticket].state == 2; });
  Req& r = s->reqs[ticket];
  if (out) *out = r.op.out;
  if (latency_ms) *latency_ms = r.t_done - r.t_submit;
  return r.rc;
}

int fides_server_release(fides_server* s, uint64_t ticket) {
  if (!s) return fgb::set_last_error(FIDES_EINVAL, "null server");
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end() || it->second.state != 2) return fgb::set_last_error(FIDES_EINVAL, "ticket not done");
    if (it->second.op.out) s->to_free.push_back({it->second.ring, it->second.op.out});
    s->reqs.erase(it);
  }
  s->cv_work.notify_one();
  return FIDES_OK;
}

int fides_server_stats_get(fides_server* s, fides_server_stats* st) {
  if (!s || !st) return fgb::set_last_error(FIDES_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  std::vector<double> v = s->latencies;
  std::sort(v.begin(), v.end());
  *st = fides_server_stats{};
  st->completed = v.size();
  st->batches = s->batches;
  if (!v.empty()) {
    st->p50_ms = v[v.size() / 2];
    st->p99_ms = v[std::min(v.size() - 1, (size_t)(0.99 * (double)v.size()))];
    double sum = 0;
    for (double x : v) sum += x;
    st->mean_ms = sum / (double)v.size();
    st->max_ms = v.back();
    const double span = s->last_done - s->first_submit;
    st->ops_per_s = span > 0 ? (double)v.size() / (span / 1e3) : 0;
  }
  st->mean_batch = s->batches ? (double)s->batched_ops / (double)s->batches : 0;
  return FIDES_OK;
}

int fides_server_reset_stats(fides_server* s) {
  if (!s) return fgb::set_last_error(FIDES_EINVAL, "null server");
  std::lock_guard<std::mutex> lk(s->mu);
  s->latencies.clear();
  s->batches = s->batched_ops = 0;
  s->first_submit = -1;
  s->last_done = 0;
  return FIDES_OK;
}

int fides_server_destroy(fides_server* s) {
  if (!s) return FIDES_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  delete s;  // results that were not released stay in the context, owned by the caller
  return FIDES_OK;
}

}  // extern "C"
