// Solve server: resident gauge fields, HBM-budget admission, continuous MRHS
// batching and latency statistics.  No counterpart in the reference (which
// has no solver); built on the slot engine of solver.h.
//
// Each resident gauge field is a lane with its own session (stream, resident
// gauge, workspace), its own slot engine and a worker thread; lanes run
// concurrently, so work on different gauges overlaps on the device.  A
// request (gauge id, kappa, tolerance, nrhs sources) waits in its lane's
// queue until enough slots are free, is admitted between two iteration
// chunks of whatever is already running, and is retired when all of its RHS
// have finished; its solution is written to the caller's buffers then.
// Admission by HBM budget: a lane's slot capacity is fixed when its gauge is
// added, from the bytes the gauge and the engine fields need, against the
// server's budget.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "serve.h"

namespace qcu {

using Clock = std::chrono::steady_clock;

struct ServeRequest {
  int64_t id = 0;
  int gauge_id = 0;
  double kappa = 0, tol = 0;
  int nrhs = 0;
  std::vector<void*> b, x;
  Clock::time_point t_submit, t_admit, t_done;
  std::vector<int> slots;
  int finished = 0;
  bool done = false;
  int status = QCU_OK;
  int iterations = 0;
  double max_res = 0;
  int all_converged = 1;
  // recorded on the legacy default stream at submit: the lane's stream (a
  // non-blocking stream) waits for it, so work the caller queued there to
  // fill b comes first
  cudaEvent_t ready = nullptr;
  ~ServeRequest() {
    if (ready) cudaEventDestroy(ready);
  }
};

struct Lane {
  int gauge_id = 0;
  int device = 0;
  std::unique_ptr<Session> sess;
  std::unique_ptr<SlotEngine> eng;
  std::deque<std::shared_ptr<ServeRequest>> waiting;
  std::map<int, std::shared_ptr<ServeRequest>> owner;  // slot -> request
  std::thread worker;
  size_t bytes = 0;
};

struct Server::Impl {
  std::mutex m;
  std::condition_variable work_cv, done_cv;
  size_t budget = 0, used = 0;
  int max_slots = 24;
  SolveRequest proto;
  std::map<int, std::unique_ptr<Lane>> lanes;
  std::map<int64_t, std::shared_ptr<ServeRequest>> requests;
  std::vector<double> latencies;
  int64_t next_id = 1, submitted = 0, completed = 0, rhs_done = 0;
  Clock::time_point t_first, t_last;
  bool stop = false;

  void run_lane(Lane* L);
};

Server::Server(size_t hbm_budget, int max_slots, int inner_prec, int solver) : p_(new Impl) {
  QCU_REQUIRE(max_slots >= 1 && max_slots <= QCU_MAX_RHS, QCU_ERR_INVALID_ARGUMENT, "max slots must be in 1..256");
  QCU_REQUIRE(prec_valid(inner_prec), QCU_ERR_INVALID_ARGUMENT, "bad inner precision");
  p_->budget = hbm_budget;
  p_->max_slots = max_slots;
  p_->proto.inner_prec = inner_prec;
  p_->proto.solver = solver;
  p_->proto.src_mode = SRC_EO_FULL;
  p_->proto.max_iter = 20000;
}

Server::~Server() {
  {
    std::lock_guard<std::mutex> lk(p_->m);
    p_->stop = true;
  }
  p_->work_cv.notify_all();
  for (auto& kv : p_->lanes)
    if (kv.second->worker.joinable()) kv.second->worker.join();
  p_->lanes.clear();
}

size_t Server::used_bytes() const {
  std::lock_guard<std::mutex> lk(p_->m);
  return p_->used;
}

void Server::add_gauge(int gauge_id, const int L[4], int N, const void* gauge, int antiperiodic_t) {
  {
    std::lock_guard<std::mutex> lk(p_->m);
    QCU_REQUIRE(p_->lanes.find(gauge_id) == p_->lanes.end(), QCU_ERR_INVALID_ARGUMENT, "gauge id already resident");
  }
  int g[4] = {1, 1, 1, 1};
  std::unique_ptr<Lane> lane(new Lane);
  lane->gauge_id = gauge_id;
  QCU_CHECK_CUDA(cudaGetDevice(&lane->device));
  lane->sess.reset(new Session(L, g, N));
  Session& s = *lane->sess;
  s.nonblocking_stream = true;
  s.antiperiodic_t = antiperiodic_t != 0;
  // memory: FP64 master gauge + the inner-precision copy + engine fields
  size_t gauge_bytes = (size_t)8 * s.geo.vh * N * N * (16 + prec_complex_bytes(p_->proto.inner_prec));
  // BF16 inner solves also keep the site-major link copy of the tensor-core dslash
  if (prec_bf16(p_->proto.inner_prec)) gauge_bytes += tc_links_bytes(s.geo.vh);
  const size_t per_slot = SlotEngine::bytes_needed(s, 1, p_->proto.inner_prec);
  int cap = 0;
  {
    std::lock_guard<std::mutex> lk(p_->m);
    const size_t left = p_->budget > p_->used ? p_->budget - p_->used : 0;
    if (left > gauge_bytes) cap = (int)std::min<size_t>((size_t)p_->max_slots, (left - gauge_bytes) / per_slot);
    QCU_REQUIRE(cap >= 1, QCU_ERR_CAPACITY,
                "HBM budget too small for gauge " + std::to_string(gauge_id) + ": needs " +
                    std::to_string(gauge_bytes + per_slot) + " bytes for one slot, " + std::to_string(left) +
                    " left");
    lane->bytes = gauge_bytes + (size_t)cap * per_slot;
    p_->used += lane->bytes;
  }
  try {
    {  // order the copy after the caller's legacy-stream work on the gauge
      cudaEvent_t ev;
      QCU_CHECK_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
      const cudaError_t e1 = cudaEventRecord(ev, 0);
      const cudaError_t e2 = e1 == cudaSuccess ? cudaStreamWaitEvent(s.stream(), ev, 0) : e1;
      cudaEventDestroy(ev);
      QCU_CHECK_CUDA(e2);
    }
    s.load_gauge(gauge, 0);
    s.gauge(p_->proto.inner_prec);
    lane->eng.reset(new SlotEngine(s, cap, p_->proto, "srv"));
  } catch (...) {
    std::lock_guard<std::mutex> lk(p_->m);
    p_->used -= lane->bytes;
    throw;
  }
  Lane* raw = lane.get();
  {
    std::lock_guard<std::mutex> lk(p_->m);
    p_->lanes[gauge_id] = std::move(lane);
  }
  raw->worker = std::thread([this, raw] { p_->run_lane(raw); });
}

int64_t Server::submit(int gauge_id, double kappa, double tol, int nrhs, void* const* x, void* const* b) {
  QCU_REQUIRE(nrhs >= 1 && x && b, QCU_ERR_INVALID_ARGUMENT, "submit: bad arguments");
  QCU_REQUIRE(kappa > 0 && tol > 0, QCU_ERR_INVALID_ARGUMENT, "submit: kappa and tol must be positive");
  auto req = std::make_shared<ServeRequest>();
  req->gauge_id = gauge_id;
  req->kappa = kappa;
  req->tol = tol;
  req->nrhs = nrhs;
  req->b.assign(b, b + nrhs);
  req->x.assign(x, x + nrhs);
  req->t_submit = Clock::now();
  QCU_CHECK_CUDA(cudaEventCreateWithFlags(&req->ready, cudaEventDisableTiming));
  QCU_CHECK_CUDA(cudaEventRecord(req->ready, 0));
  {
    std::lock_guard<std::mutex> lk(p_->m);
    auto it = p_->lanes.find(gauge_id);
    QCU_REQUIRE(it != p_->lanes.end(), QCU_ERR_INVALID_ARGUMENT, "submit: gauge id not resident");
    QCU_REQUIRE(nrhs <= it->second->eng->capacity(), QCU_ERR_CAPACITY,
                "submit: nrhs exceeds the lane's slot capacity " + std::to_string(it->second->eng->capacity()));
    req->id = p_->next_id++;
    if (p_->submitted == 0) p_->t_first = req->t_submit;
    p_->submitted++;
    p_->requests[req->id] = req;
    it->second->waiting.push_back(req);
  }
  p_->work_cv.notify_all();
  return req->id;
}

bool Server::wait(int64_t id, double timeout_s, RequestInfo* info) {
  std::unique_lock<std::mutex> lk(p_->m);
  auto it = p_->requests.find(id);
  QCU_REQUIRE(it != p_->requests.end(), QCU_ERR_INVALID_ARGUMENT, "wait: unknown request id");
  std::shared_ptr<ServeRequest> r = it->second;
  const auto pred = [&] { return r->done; };
  if (timeout_s < 0)
    p_->done_cv.wait(lk, pred);
  else
    p_->done_cv.wait_for(lk, std::chrono::duration<double>(timeout_s), pred);
  if (info) {
    info->done = r->done;
    info->status = r->status;
    info->nrhs = r->nrhs;
    info->iterations = r->iterations;
    info->latency_s = r->done ? std::chrono::duration<double>(r->t_done - r->t_submit).count() : 0.0;
    info->queue_s = r->slots.empty() ? 0.0 : std::chrono::duration<double>(r->t_admit - r->t_submit).count();
    info->max_true_residual = r->max_res;
    info->all_converged = r->all_converged;
  }
  return r->done;
}

ServerStats Server::stats() const {
  std::lock_guard<std::mutex> lk(p_->m);
  ServerStats s;
  s.submitted = p_->submitted;
  s.completed = p_->completed;
  s.hbm_used = p_->used;
  std::vector<double> v = p_->latencies;
  std::sort(v.begin(), v.end());
  if (!v.empty()) {
    auto q = [&](double f) { return v[std::min(v.size() - 1, (size_t)std::floor(f * (v.size() - 1) + 0.5))]; };
    s.p50_s = q(0.50);
    s.p99_s = q(0.99);
    double m = 0;
    for (double x : v) m += x;
    s.mean_s = m / v.size();
    const double span = std::chrono::duration<double>(p_->t_last - p_->t_first).count();
    s.solves_per_s = span > 0 ? p_->completed / span : 0.0;
    s.rhs_per_s = span > 0 ? p_->rhs_done / span : 0.0;
  }
  return s;
}

void Server::Impl::run_lane(Lane* L) {
  cudaSetDevice(L->device);
  SlotEngine& eng = *L->eng;
  const int mode = proto.src_mode;
  for (;;) {
    // admit whatever fits, oldest first
    std::vector<std::shared_ptr<ServeRequest>> admit_now;
    {
      std::unique_lock<std::mutex> lk(m);
      if (eng.active_slots() == 0 && L->waiting.empty() && !stop)
        work_cv.wait(lk, [&] { return stop || !L->waiting.empty(); });
      if (stop) return;
      int free_n = (int)eng.free_slots().size();
      for (auto it = L->waiting.begin(); it != L->waiting.end();) {
        if ((*it)->nrhs <= free_n) {
          free_n -= (*it)->nrhs;
          admit_now.push_back(*it);
          it = L->waiting.erase(it);
        } else {
          ++it;
        }
      }
    }
    try {
      std::vector<int> fr = eng.free_slots();
      size_t k = 0;
      for (auto& r : admit_now) {
        std::vector<int> slots(fr.begin() + k, fr.begin() + k + r->nrhs);
        k += r->nrhs;
        std::vector<double> kap(r->nrhs, r->kappa), tol(r->nrhs, r->tol);
        r->slots = slots;
        r->t_admit = Clock::now();
        QCU_CHECK_CUDA(cudaStreamWaitEvent(L->sess->stream(), r->ready, 0));
        eng.admit(slots, r->b.data(), kap.data(), tol.data(), mode);
        for (int s : slots) L->owner[s] = r;
      }
      std::vector<int> fin = eng.step();
      for (int s : fin) {
        auto r = L->owner[s];
        r->finished++;
        if (r->finished == r->nrhs) {
          eng.retire(r->slots, r->x.data(), mode);
          bool bad_source = false;
          for (int t : r->slots) {
            const SlotState& h = eng.slot(t);
            r->iterations = std::max(r->iterations, h.iterations);
            r->max_res = std::max(r->max_res, std::sqrt(h.true_res2 / h.bb));
            r->all_converged &= h.converged;
            bad_source |= h.bad_source != 0;
            L->owner.erase(t);
          }
          std::lock_guard<std::mutex> lk(m);
          r->t_done = Clock::now();
          r->done = true;
          r->status = bad_source ? QCU_ERR_INVALID_ARGUMENT : r->all_converged ? QCU_OK : QCU_ERR_NOT_CONVERGED;
          latencies.push_back(std::chrono::duration<double>(r->t_done - r->t_submit).count());
          completed++;
          rhs_done += r->nrhs;
          t_last = r->t_done;
          done_cv.notify_all();
        }
      }
    } catch (const Error& e) {
      // fail every request of the lane; the lane stops
      std::lock_guard<std::mutex> lk(m);
      for (auto& kv : L->owner) {
        kv.second->done = true;
        kv.second->status = e.code;
      }
      for (auto& r : L->waiting) {
        r->done = true;
        r->status = e.code;
      }
      L->waiting.clear();
      L->owner.clear();
      done_cv.notify_all();
      return;
    }
  }
}

}  // namespace qcu
