// Serving engine: a request loop over resident disk stacks.
//
// The reference's callers solve one candidate geometry per call: the
// optimiser utilities (examples/transformer_optim_utilities.jl:11-144) move
// the disks and call transformer again, and frequency sweeps run @distributed
// over single-frequency calls.  Here a server accepts such solves as requests
// (bf_submit), keeps every stack's geometry and workspace resident on the
// device, and runs admitted requests concurrently on its workers' streams:
//   * workers: n_workers host threads, each owning one bf_handle (one stream);
//     a stack's bounce-loop workspace lives with the worker that grew it (its
//     "home") until the workspace is released, so a stack never pays a
//     reallocation for changing streams; transformer solves keep only the
//     overlap cache, which any worker's stream uses as it is, so their stacks
//     run on whichever worker is free;
//   * admission: the request's footprint + the bytes resident in served stacks
//     + the running requests' footprints must fit the budget; idle stacks'
//     workspaces are released least recently used first to make room; a queued
//     request that does not fit is passed over by smaller ones at most
//     kMaxPassOver times, after which nothing else starts until it fits;
//   * order and batching: one request per stack at a time, in submission order;
//     queued requests on the same stack with the same solver settings and no
//     geometry change join the first one's frequency batch (one solve);
//     transformer requests on different stacks that differ only in their air
//     gaps (the steps of several disk-position optimisers) join one group
//     solve (bf_transformer_group), up to kMaxGroup requests;
//   * latency lane (bf_server_set_latency_lane): requests marked lane = 1 run
//     only on the last workers, whose streams have the highest priority;
//   * completion: beta^2 (and the transformer boost) are copied to the caller's
//     buffers, then the status becomes final; bf_poll / bf_wait report it.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/boostfractor_gb300.h"
#include "bf_host.h"

namespace {

using Clock = std::chrono::steady_clock;
constexpr int kMaxPassOver = 8;
constexpr int kMaxBatchFreqs = 4096;
constexpr int kMaxGroup = 16;

struct Req {
  unsigned long long id = 0;
  bf_request r{};
  std::vector<double> freqs, distance;
  size_t est = 0;
  int nm = 0;
  int status = BF_PENDING;
  int passed_over = 0;
  int in_batch = 0;  // solved as part of an earlier request's batch
  double t_submit = 0, t_start = 0, t_done = 0;
};

struct StackInfo {
  int home = -1;      // worker holding the stack's bounce-loop workspace, -1 = none
  bool busy = false;
  double last_used = 0;
  size_t resident = 0;
};

struct Batch {
  std::vector<Req*> reqs;
  size_t need = 0;
  bool group = false;   // reqs on different stacks, one group solve
};

}  // namespace

struct bf_server {
  int device = 0, flags = 0;
  unsigned long long budget = 0;
  std::vector<bf_handle*> hs;
  std::vector<std::thread> th;
  int n_workers = 0, n_lane = 0;            // the last n_lane workers serve lane 1 only
  std::vector<cudaStream_t> lane_streams;   // their high-priority streams
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Req*> queue;
  std::unordered_map<unsigned long long, Req*> reqs;
  std::unordered_map<bf_stack*, StackInfo> stacks;
  size_t resident = 0, inflight = 0;
  unsigned long long next_id = 1;
  bool stop = false;
  std::string err;
  Clock::time_point t0;
  // statistics (per solver)
  std::vector<double> lat[4];
  double fpts[4] = {0, 0, 0, 0};
  unsigned long long failed[4] = {0, 0, 0, 0}, batched[4] = {0, 0, 0, 0};
  unsigned long long evictions = 0;
  double t_first = -1.0, t_last = 0.0;
  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
  bool dry() const { return flags & BF_SERVER_DRYRUN; }
};

namespace {

int server_fail(bf_server* s, int code, const std::string& msg) {
  s->err = msg;
  return code;
}

// Release the workspace of idle stacks, least recently used first, until
// `need` more bytes fit under `cap` (the budget, or the normal requests' part
// of it).  Caller holds the lock.
bool make_room(bf_server* S, size_t need, const bf_stack* keep, size_t cap) {
  while (S->resident + S->inflight + need > cap) {
    bf_stack* victim = nullptr;
    double oldest = 1e300;
    for (auto& kv : S->stacks)
      if (kv.first != keep && !kv.second.busy && kv.second.resident > 0 && kv.second.last_used < oldest) {
        oldest = kv.second.last_used;
        victim = kv.first;
      }
    if (!victim) return false;
    StackInfo& vi = S->stacks[victim];
    if (!S->dry()) bf_stack_trim(victim);
    S->resident -= vi.resident;
    vi.resident = 0;
    vi.home = -1;
    S->evictions++;
  }
  return true;
}

// Transformer requests whose stacks may share one group solve: same modes,
// frequencies and settings, and stacks that differ at most in distances (the
// library checks that only untilted air gaps differ and refuses otherwise).
bool groupable(const bf_server* S, const Req* a, const Req* b) {
  if (a->r.solver != BF_SOLVER_TRANSFORMER || b->r.solver != BF_SOLVER_TRANSFORMER) return false;
  if (a->r.modes != b->r.modes || a->r.prop_kind != b->r.prop_kind || a->r.precision != b->r.precision ||
      a->freqs != b->freqs)
    return false;
  if (S->dry()) return true;
  const bf_stack* x = a->r.stack;
  const bf_stack* y = b->r.stack;
  if (x->nd != y->nd || x->nx != y->nx || x->ny != y->ny || x->diskR != y->diskR || !x->surf.empty() ||
      !y->surf.empty() || x->X != y->X || x->Y != y->Y || x->tilt_x != y->tilt_x || x->tilt_y != y->tilt_y)
    return false;
  for (int j = 0; j < x->nd; ++j) {
    const cd e = x->eps[j], f = y->eps[j];
    if (!(e == f || (std::isnan(e.real()) && std::isnan(f.real()) && e.imag() == f.imag()))) return false;
  }
  return true;
}

bool mergeable(const Req* a, const Req* b) {
  return b->distance.empty() && a->r.solver == b->r.solver && a->r.modes == b->r.modes &&
         a->r.nmax == b->r.nmax && a->r.prop_kind == b->r.prop_kind && a->r.precision == b->r.precision &&
         a->r.beta2_scale == b->r.beta2_scale;
}

// Whether request R must wait for its stack's home worker (which holds the
// stack's workspace) rather than run on worker w.  A home worker of the other
// lane class cannot run R; the workspace then moves to w.
bool bound_elsewhere(const bf_server* S, const StackInfo& si, const Req* R, int w) {
  if (R->r.solver == BF_SOLVER_TRANSFORMER || si.home < 0 || si.home == w) return false;
  const bool home_in_lane = si.home >= S->n_workers - S->n_lane;
  const bool r_in_lane = S->n_lane && R->r.lane == 1;
  return home_in_lane == r_in_lane;
}

// The next batch worker w may start, or an empty batch.  Caller holds the lock.
Batch pick(bf_server* S, int w) {
  Batch b;
  const bool lane_worker = w >= S->n_workers - S->n_lane;
  // with a latency lane, normal requests use at most 7/8 of the budget, so
  // that the lane's (small) requests are never held back for memory
  const size_t normal_cap = S->n_lane ? S->budget - S->budget / 8 : S->budget;
  for (size_t qi = 0; qi < S->queue.size(); ++qi) {
    Req* R = S->queue[qi];
    // the lane's requests run only on its high-priority streams, the others
    // only on the normal workers
    if (lane_worker != (S->n_lane && R->r.lane == 1)) continue;
    StackInfo& si = S->stacks[R->r.stack];
    if (si.busy || bound_elsewhere(S, si, R, w)) continue;
    const size_t cap = R->r.lane ? S->budget : normal_cap;
    // the workspace the stack already holds is reused by the solve
    const size_t need = R->est > si.resident ? R->est - si.resident : 0;
    if (!make_room(S, need, R->r.stack, cap)) {
      if (++R->passed_over > kMaxPassOver) return b;  // hold the line for it
      continue;
    }
    // take R and the queued requests on the same stack that can join its batch
    b.reqs.push_back(R);
    b.need = need;
    int nf = R->r.nf;
    std::vector<size_t> taken = {qi};
    for (size_t qj = qi + 1; qj < S->queue.size(); ++qj) {
      Req* Q = S->queue[qj];
      if (Q->r.stack != R->r.stack) continue;
      if (!mergeable(R, Q) || nf + Q->r.nf > kMaxBatchFreqs) break;
      if (S->resident + S->inflight + b.need + Q->est > cap) break;
      b.reqs.push_back(Q);
      b.need += Q->est;
      nf += Q->r.nf;
      Q->in_batch = 1;
      taken.push_back(qj);
    }
    // a lone transformer request gathers the queued steps of other stacks
    // that can share its solve
    if (b.reqs.size() == 1 && R->r.solver == BF_SOLVER_TRANSFORMER) {
      // the queue position of each stack's first queued request (one pass,
      // so that a long queue costs linear time here, not quadratic)
      std::unordered_map<const bf_stack*, size_t> first;
      first.reserve(S->stacks.size());
      for (size_t qk = 0; qk < S->queue.size(); ++qk) first.emplace(S->queue[qk]->r.stack, qk);
      for (size_t qj = qi + 1; qj < S->queue.size() && (int)b.reqs.size() < kMaxGroup; ++qj) {
        Req* Q = S->queue[qj];
        if (!groupable(S, R, Q) || Q->r.lane != R->r.lane) continue;
        bool dup = false;
        for (Req* G : b.reqs) dup |= G->r.stack == Q->r.stack;
        if (dup) continue;
        StackInfo& qs = S->stacks[Q->r.stack];
        if (qs.busy) continue;
        // an earlier queued request on Q's stack keeps its turn
        if (first[Q->r.stack] != qj) continue;
        const size_t qneed = Q->est > qs.resident ? Q->est - qs.resident : 0;
        if (S->resident + S->inflight + b.need + qneed > cap) break;
        b.reqs.push_back(Q);
        b.need += qneed;
        Q->in_batch = 1;
        taken.push_back(qj);
      }
      if (b.reqs.size() > 1) {
        b.group = true;
        std::sort(taken.begin(), taken.end());
      }
    }
    for (auto it = taken.rbegin(); it != taken.rend(); ++it) S->queue.erase(S->queue.begin() + (long)*it);
    for (Req* G : b.reqs) {
      StackInfo& gi = S->stacks[G->r.stack];
      gi.busy = true;
      if (G->r.solver != BF_SOLVER_TRANSFORMER) gi.home = w;
    }
    S->inflight += b.need;
    return b;
  }
  return b;
}

double default_scale(const bf_stack* s) {
  const double dx = s->nx > 1 ? s->X[1] - s->X[0] : 1.0;
  const double dy = s->ny > 1 ? s->Y[1] - s->Y[0] : 1.0;
  return dx * dy / (M_PI * s->diskR * s->diskR);
}

// Run one batch on worker w's handle (no lock held).  Returns the status for
// every request of the batch and fills their outputs.
int run_batch(bf_server* S, int w, Batch& b, std::string& err) {
  Req* R0 = b.reqs[0];
  if (S->dry()) {
    std::this_thread::sleep_for(std::chrono::microseconds((long long)R0->r.nmax * (long long)b.reqs.size()));
    for (Req* R : b.reqs) std::fill(R->r.out_beta2, R->r.out_beta2 + R->r.nf, 0.0);
    return BF_OK;
  }
  bf_handle* h = S->hs[w];
  bf_stack* st = R0->r.stack;
  int rc = BF_OK;
  // an optimiser step moves the disks; a grid step only selects the interpolation point
  if (!R0->distance.empty() && R0->r.solver != BF_SOLVER_PGRID) rc = bf_stack_set_distance(h, st, R0->distance.data());
  if (rc != BF_OK) { err = h->err; return rc; }
  std::vector<double> freqs;
  for (Req* R : b.reqs) freqs.insert(freqs.end(), R->freqs.begin(), R->freqs.end());
  const int nf = (int)freqs.size();
  std::vector<double> b2(nf, 0.0);
  const bf_request& q = R0->r;
  if (q.solver == BF_SOLVER_PGRID) {
    std::vector<double> boost(q.out_boost ? (size_t)nf * R0->nm * 2 : 0);
    rc = bf_pgrid_transformer(h, q.pgrid, R0->distance.data(), nullptr, q.out_boost ? boost.data() : nullptr,
                              b2.data());
    if (rc == BF_OK && q.out_boost) std::memcpy(q.out_boost, boost.data(), sizeof(double) * boost.size());
  } else if (b.group) {
    // steps of several stacks in one group solve (each request's distances first)
    const int n = (int)b.reqs.size(), nfr = R0->r.nf, nm = R0->nm;
    std::vector<bf_stack*> sts(n);
    for (int r = 0; r < n && rc == BF_OK; ++r) {
      Req* R = b.reqs[r];
      sts[r] = R->r.stack;
      if (r > 0 && !R->distance.empty()) rc = bf_stack_set_distance(h, sts[r], R->distance.data());
    }
    if (rc != BF_OK) { err = h->err; return rc; }
    bool want = false;
    for (Req* R : b.reqs) want |= R->r.out_boost != nullptr;
    std::vector<double> gb2((size_t)n * nfr), gbo(want ? (size_t)n * nfr * nm * 2 : 0);
    rc = bf_transformer_group(h, n, sts.data(), q.modes, nfr, R0->freqs.data(), q.prop_kind, q.precision,
                              want ? gbo.data() : nullptr, gb2.data());
    if (rc == BF_ERR_INVALID) {
      // the stacks differ in more than their air gaps: solve them one by one
      rc = BF_OK;
      for (int r = 0; r < n && rc == BF_OK; ++r)
        rc = bf_transformer(h, sts[r], q.modes, nfr, R0->freqs.data(), q.prop_kind, q.precision, nullptr, nullptr,
                            nullptr, 0, want ? gbo.data() + (size_t)r * nfr * nm * 2 : nullptr, nullptr,
                            gb2.data() + (size_t)r * nfr);
    }
    if (rc != BF_OK) { err = h->err; return rc; }
    for (int r = 0; r < n; ++r) {
      Req* R = b.reqs[r];
      std::copy(gb2.begin() + (long)r * nfr, gb2.begin() + (long)(r + 1) * nfr, R->r.out_beta2);
      if (R->r.out_boost)
        std::memcpy(R->r.out_boost, gbo.data() + (size_t)r * nfr * nm * 2, sizeof(double) * nfr * nm * 2);
    }
    return BF_OK;
  } else if (q.solver == BF_SOLVER_TRANSFORMER) {
    bool want = false;
    for (Req* R : b.reqs) want |= R->r.out_boost != nullptr;
    std::vector<double> boost(want ? (size_t)nf * R0->nm * 2 : 0);
    rc = bf_transformer(h, st, q.modes, nf, freqs.data(), q.prop_kind, q.precision, nullptr, nullptr, nullptr, 0,
                        want ? boost.data() : nullptr, nullptr, b2.data());
    if (rc == BF_OK && want) {
      size_t off = 0;
      for (Req* R : b.reqs) {
        const size_t n = (size_t)R->r.nf * R0->nm * 2;
        if (R->r.out_boost) std::memcpy(R->r.out_boost, boost.data() + off, sizeof(double) * n);
        off += n;
      }
    }
  } else {
    const double scale = q.beta2_scale != 0.0 ? q.beta2_scale : default_scale(st);
    if (q.solver == BF_SOLVER_CHEERLEADER)
      rc = bf_stack_cheerleader(h, st, nf, freqs.data(), 0.0, q.nmax, q.prop_kind, q.precision, nullptr, nullptr, 0,
                                scale, 0, nullptr, nullptr, b2.data());
    else
      rc = bf_stack_dancer(h, st, nf, freqs.data(), 0.0, q.nmax, q.prop_kind, q.precision, nullptr, nullptr, 1, 1,
                           scale, 0, nullptr, b2.data());
  }
  if (rc != BF_OK) { err = h->err; return rc; }
  size_t off = 0;
  for (Req* R : b.reqs) {
    std::copy(b2.begin() + (long)off, b2.begin() + (long)off + R->r.nf, R->r.out_beta2);
    off += R->r.nf;
  }
  return BF_OK;
}

void worker(bf_server* S, int w) {
  if (!S->dry()) cudaSetDevice(S->device);
  std::unique_lock<std::mutex> lock(S->mu);
  for (;;) {
    Batch b;
    S->cv_work.wait(lock, [&] {
      if (S->stop) return true;
      b = pick(S, w);
      return !b.reqs.empty();
    });
    if (b.reqs.empty()) return;  // stopping
    const double t_start = S->now();
    for (Req* R : b.reqs) R->t_start = t_start;
    lock.unlock();
    std::string err;
    const int rc = run_batch(S, w, b, err);
    std::vector<bf_stack*> sts;
    std::vector<size_t> res;
    for (Req* R : b.reqs) {
      if (std::find(sts.begin(), sts.end(), R->r.stack) != sts.end()) continue;
      sts.push_back(R->r.stack);
      res.push_back(S->dry() ? (size_t)std::max<unsigned long long>(R->r.footprint_bytes, 1)
                             : bf_stack_device_bytes(R->r.stack));
    }
    if (!S->dry())
      for (Req* R : b.reqs) {
        R->r.stack->server_uses.n--;
        if (R->r.solver == BF_SOLVER_TRANSFORMER) bf_modes_server_use(R->r.modes, -1);
      }
    lock.lock();
    const double t_done = S->now();
    S->inflight -= b.need;
    for (size_t k = 0; k < sts.size(); ++k) {
      StackInfo& si = S->stacks[sts[k]];
      S->resident -= si.resident;
      si.resident = res[k];
      S->resident += res[k];
      si.busy = false;
      si.last_used = t_done;
    }
    if (rc != BF_OK) S->err = err;
    for (Req* R : b.reqs) {
      R->t_done = t_done;
      R->status = rc;
      const int k = R->r.solver;
      if (rc == BF_OK) {
        S->lat[k].push_back(1e3 * (t_done - R->t_submit));
        S->fpts[k] += R->r.nf;
      } else {
        S->failed[k]++;
      }
      if (R->in_batch) S->batched[k]++;
      R->freqs.clear();
      R->freqs.shrink_to_fit();
    }
    S->t_last = std::max(S->t_last, t_done);
    S->cv_done.notify_all();
    S->cv_work.notify_all();
  }
}

double percentile(std::vector<double> v, double p) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  size_t k = (size_t)std::ceil(p * (double)v.size());
  k = k == 0 ? 0 : k - 1;
  return v[std::min(k, v.size() - 1)];
}

int finish(bf_server* S, std::unordered_map<unsigned long long, Req*>::iterator it, int* status, double* times) {
  Req* R = it->second;
  if (status) *status = R->status;
  if (times) {
    times[0] = R->t_submit;
    times[1] = R->t_start;
    times[2] = R->t_done;
  }
  if (R->status != BF_PENDING) {
    delete R;
    S->reqs.erase(it);
  }
  return BF_OK;
}

}  // namespace

extern "C" int bf_server_create(int device, unsigned long long hbm_budget_bytes, int n_workers, int flags,
                                bf_server** out) {
  if (!out || n_workers < 1 || n_workers > 64) return BF_ERR_INVALID;
  *out = nullptr;
  bf_server* S = new bf_server();
  S->device = device;
  S->flags = flags;
  S->t0 = Clock::now();
  S->budget = hbm_budget_bytes;
  if (!S->dry()) {
    if (cudaSetDevice(device) != cudaSuccess) {
      cudaGetLastError();
      delete S;
      return BF_ERR_CUDA;
    }
    if (!S->budget) {
      size_t fr = 0, tot = 0;
      if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        cudaGetLastError();
        delete S;
        return BF_ERR_CUDA;
      }
      S->budget = fr;
    }
    for (int w = 0; w < n_workers; ++w) {
      bf_handle* h = nullptr;
      const int rc = bf_create(device, 0, &h);
      if (rc != BF_OK) {
        for (bf_handle* x : S->hs) bf_destroy(x);
        delete S;
        return rc;
      }
      S->hs.push_back(h);
    }
    if (flags & BF_SERVER_RESERVE_HBM) {
      // the pool is grown once here instead of by the first large solves, whose
      // mapping of new memory would stall the other workers' allocations
      size_t fr = 0, tot = 0;
      if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        cudaGetLastError();
        fr = 0;
      }
      const size_t margin = 2ull << 30;
      const size_t want = std::min<size_t>(S->budget, fr > margin ? fr - margin : 0);
      if (want && bf_pool_reserve(S->hs[0], want) != BF_OK) S->err = "HBM reservation failed; the pool grows on demand";
    }
  } else if (!S->budget) {
    S->budget = ~0ull;
  }
  S->n_workers = n_workers;
  for (int w = 0; w < n_workers; ++w) S->th.emplace_back(worker, S, w);
  *out = S;
  return BF_OK;
}

extern "C" int bf_server_destroy(bf_server* S) {
  if (!S) return BF_ERR_INVALID;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    S->stop = true;
    for (Req* R : S->queue) {
      R->status = BF_ERR_INVALID;
      R->t_done = S->now();
      if (!S->dry()) {
        R->r.stack->server_uses.n--;
        if (R->r.solver == BF_SOLVER_TRANSFORMER) bf_modes_server_use(R->r.modes, -1);
      }
    }
    S->queue.clear();
    S->cv_work.notify_all();
    S->cv_done.notify_all();
  }
  for (auto& t : S->th) t.join();
  if (!S->dry())
    for (auto& kv : S->stacks) bf_stack_trim(kv.first);
  for (bf_handle* h : S->hs) bf_destroy(h);
  for (cudaStream_t st : S->lane_streams) cudaStreamDestroy(st);
  for (auto& kv : S->reqs) delete kv.second;
  delete S;
  return BF_OK;
}

extern "C" int bf_submit(bf_server* S, const bf_request* q, unsigned long long* id) {
  if (!S || !q || !id) return BF_ERR_INVALID;
  *id = 0;
  if (q->solver < BF_SOLVER_CHEERLEADER || q->solver > BF_SOLVER_PGRID)
    return server_fail(S, BF_ERR_INVALID, "unknown solver");
  if (!q->stack || q->nf < 1 || !q->freqs || !q->out_beta2)
    return server_fail(S, BF_ERR_INVALID, "request needs a stack, frequencies and out_beta2");
  if (q->nf > kMaxBatchFreqs) return server_fail(S, BF_ERR_INVALID, "more than 4096 frequencies in one request");
  for (int i = 0; i < q->nf; ++i)
    if (!(q->freqs[i] > 0.0) || !std::isfinite(q->freqs[i]))
      return server_fail(S, BF_ERR_INVALID, "frequencies must be finite and positive");
  if (q->solver == BF_SOLVER_TRANSFORMER && !q->modes)
    return server_fail(S, BF_ERR_INVALID, "a transformer request needs a mode basis");
  if (q->solver < BF_SOLVER_TRANSFORMER && q->nmax < 0) return server_fail(S, BF_ERR_INVALID, "nmax < 0");
  if (q->solver == BF_SOLVER_PGRID && (!q->pgrid || !q->distance))
    return server_fail(S, BF_ERR_INVALID, "a grid request needs the grid and the per-disk shifts (distance)");
  const bool tf_only = q->precision == BF_PREC_TF32 || q->precision == BF_PREC_MIXED_SIMT;
  if (!(q->precision == BF_PREC_FP64 || q->precision == BF_PREC_MIXED ||
        (tf_only && q->solver == BF_SOLVER_TRANSFORMER)))
    return server_fail(S, BF_ERR_INVALID, "unknown precision for this solver");
  if (S->dry() && !q->footprint_bytes)
    return server_fail(S, BF_ERR_INVALID, "a dry-run request needs footprint_bytes");
  if (q->lane != 0 && q->lane != 1) return server_fail(S, BF_ERR_INVALID, "lane must be 0 or 1");
  Req* R = new Req();
  R->r = *q;
  R->freqs.assign(q->freqs, q->freqs + q->nf);
  if (!S->dry() && q->solver == BF_SOLVER_PGRID) {
    int gnf = 0, gnd = 0, gnm = 0;
    bf_stack* gs = nullptr;
    bf_pgrid_shape(q->pgrid, &gnf, &gnd, &gnm, &gs);
    if (gnf != q->nf) {
      delete R;
      return server_fail(S, BF_ERR_INVALID, "a grid request's frequencies must be the grid's");
    }
    R->r.stack = gs;   // requests on one grid run one at a time, like those on one stack
    R->nm = gnm;
    R->distance.assign(q->distance, q->distance + (gnd - 2) / 2);
    for (double d : R->distance)
      if (!std::isfinite(d)) {
        delete R;
        return server_fail(S, BF_ERR_INVALID, "non-finite shift");
      }
    R->est = q->footprint_bytes ? (size_t)q->footprint_bytes
                                : (size_t)gnf * gnd * gnm * gnm * 16 * 6 + (size_t)gnf * gnm * 64 + 4096;
  } else if (!S->dry()) {
    if (q->distance) {
      R->distance.assign(q->distance, q->distance + q->stack->nd);
      for (double d : R->distance)
        if (!std::isfinite(d)) {
          delete R;
          return server_fail(S, BF_ERR_INVALID, "non-finite distance");
        }
    }
    if (q->solver == BF_SOLVER_TRANSFORMER && bf_modes_get(S->hs[0], q->modes, &R->nm, nullptr, nullptr) != BF_OK) {
      delete R;
      return server_fail(S, BF_ERR_INVALID, "invalid mode basis");
    }
    R->est = q->footprint_bytes ? (size_t)q->footprint_bytes
                                : bf_solve_bytes_estimate(q->stack, q->solver, q->nf, R->nm, q->prop_kind, q->precision);
  } else {
    if (q->distance) R->distance.assign(1, 0.0);  // marks a geometry change (no stack to read)
    R->est = (size_t)q->footprint_bytes;
  }
  std::lock_guard<std::mutex> lock(S->mu);
  if (S->stop) {
    delete R;
    return server_fail(S, BF_ERR_INVALID, "server is shutting down");
  }
  const size_t cap = (S->n_lane && R->r.lane == 0) ? S->budget - S->budget / 8 : S->budget;
  if (R->est > cap) {
    const size_t est = R->est;
    delete R;
    return server_fail(S, BF_ERR_NOMEM, "request footprint of " + std::to_string(est) +
                                            " bytes exceeds the server's HBM budget" +
                                            (cap < S->budget ? " less the latency lane's eighth" : ""));
  }
  R->id = S->next_id++;
  R->t_submit = S->now();
  // the stack may not be destroyed while this request is queued or running
  if (!S->dry()) {
    R->r.stack->server_uses.n++;
    if (R->r.solver == BF_SOLVER_TRANSFORMER) bf_modes_server_use(R->r.modes, +1);
  }
  if (S->t_first < 0) S->t_first = R->t_submit;
  S->stacks.emplace(q->stack, StackInfo());
  S->reqs[R->id] = R;
  S->queue.push_back(R);
  *id = R->id;
  S->cv_work.notify_all();
  return BF_OK;
}

extern "C" int bf_poll(bf_server* S, unsigned long long id, int* status, double* times) {
  if (!S) return BF_ERR_INVALID;
  std::lock_guard<std::mutex> lock(S->mu);
  auto it = S->reqs.find(id);
  if (it == S->reqs.end()) return server_fail(S, BF_ERR_INVALID, "unknown request id");
  return finish(S, it, status, times);
}

extern "C" int bf_wait(bf_server* S, unsigned long long id, int timeout_ms, int* status, double* times) {
  if (!S) return BF_ERR_INVALID;
  std::unique_lock<std::mutex> lock(S->mu);
  auto it = S->reqs.find(id);
  if (it == S->reqs.end()) return server_fail(S, BF_ERR_INVALID, "unknown request id");
  Req* R = it->second;
  auto done = [&] { return R->status != BF_PENDING; };
  if (timeout_ms < 0) S->cv_done.wait(lock, done);
  else if (!S->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms), done)) {
    if (status) *status = BF_PENDING;
    return BF_ERR_TIMEOUT;
  }
  return finish(S, S->reqs.find(id), status, times);
}

extern "C" int bf_server_stats(bf_server* S, int solver, double* out) {
  if (!S || !out || solver < -1 || solver > 3) return BF_ERR_INVALID;
  std::lock_guard<std::mutex> lock(S->mu);
  std::vector<double> lat;
  double fp = 0, nf_ = 0, nb = 0;
  for (int k = 0; k < 4; ++k)
    if (solver < 0 || solver == k) {
      lat.insert(lat.end(), S->lat[k].begin(), S->lat[k].end());
      fp += S->fpts[k];
      nf_ += (double)S->failed[k];
      nb += (double)S->batched[k];
    }
  double mean = 0, mx = 0;
  for (double v : lat) {
    mean += v;
    mx = std::max(mx, v);
  }
  if (!lat.empty()) mean /= (double)lat.size();
  out[0] = (double)lat.size();
  out[1] = nf_;
  out[2] = fp;
  out[3] = percentile(lat, 0.50);
  out[4] = percentile(lat, 0.99);
  out[5] = mean;
  out[6] = mx;
  out[7] = S->t_first < 0 ? 0.0 : S->t_last - S->t_first;
  out[8] = nb;
  out[9] = (double)S->evictions;
  return BF_OK;
}

extern "C" int bf_server_set_latency_lane(bf_server* S, int n_lane) {
  if (!S) return BF_ERR_INVALID;
  std::lock_guard<std::mutex> lock(S->mu);
  if (n_lane < 1 || n_lane >= S->n_workers)
    return server_fail(S, BF_ERR_INVALID, "the latency lane needs 1 .. n_workers - 1 workers");
  if (S->n_lane != 0 || S->next_id != 1)
    return server_fail(S, BF_ERR_INVALID, "set the latency lane once, before the first request");
  if (!S->dry()) {
    if (cudaSetDevice(S->device) != cudaSuccess) {
      cudaGetLastError();
      return server_fail(S, BF_ERR_CUDA, "cudaSetDevice");
    }
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) {
      cudaGetLastError();
      return server_fail(S, BF_ERR_CUDA, "cudaDeviceGetStreamPriorityRange");
    }
    // the persistent tensor-core GEMM of the normal workers leaves the lane's
    // share of the SMs free, so a lane kernel never waits for a whole GEMM
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, S->device) != cudaSuccess || sms < 2) {
      cudaGetLastError();
      sms = 0;
    }
    const int reserve = sms ? std::max(1, sms * n_lane / S->n_workers) : 0;
    for (int w = 0; w < S->n_workers - n_lane && sms; ++w) S->hs[w]->sm_cap = sms - reserve;
    // the workers are idle (no request yet), so their handles may change streams
    for (int k = 0; k < n_lane; ++k) {
      cudaStream_t st = nullptr;
      if (cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, greatest) != cudaSuccess) {
        cudaGetLastError();
        return server_fail(S, BF_ERR_CUDA, "cudaStreamCreateWithPriority");
      }
      S->lane_streams.push_back(st);
      bf_set_stream(S->hs[S->n_workers - n_lane + k], st);
    }
  }
  S->n_lane = n_lane;
  return BF_OK;
}

extern "C" int bf_server_reset_stats(bf_server* S) {
  if (!S) return BF_ERR_INVALID;
  std::lock_guard<std::mutex> lock(S->mu);
  for (int k = 0; k < 4; ++k) {
    S->lat[k].clear();
    S->fpts[k] = 0.0;
    S->failed[k] = 0;
    S->batched[k] = 0;
  }
  S->evictions = 0;
  S->t_first = -1.0;
  S->t_last = 0.0;
  return BF_OK;
}

extern "C" const char* bf_server_last_error(const bf_server* S) { return S ? S->err.c_str() : ""; }
