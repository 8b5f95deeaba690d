// Solve server (serve.cu): resident gauges, HBM-budget admission, continuous
// MRHS batching, latency statistics.
#pragma once

#include <memory>

#include "solver.h"

namespace qcu {

struct RequestInfo {
  int done = 0;
  int status = 0;
  int nrhs = 0;
  int iterations = 0;
  double latency_s = 0.0;  // submit -> solution written
  double queue_s = 0.0;    // submit -> admitted into slots
  double max_true_residual = 0.0;
  int all_converged = 0;
};

struct ServerStats {
  int64_t submitted = 0, completed = 0;
  double p50_s = 0.0, p99_s = 0.0, mean_s = 0.0;
  double solves_per_s = 0.0, rhs_per_s = 0.0;
  size_t hbm_used = 0;
};

class Server {
 public:
  Server(size_t hbm_budget, int max_slots, int inner_prec, int solver);
  ~Server();
  void add_gauge(int gauge_id, const int L[4], int N, const void* gauge, int antiperiodic_t);
  int64_t submit(int gauge_id, double kappa, double tol, int nrhs, void* const* x, void* const* b);
  // waits up to timeout_s (< 0: forever); returns whether the request is done
  bool wait(int64_t id, double timeout_s, RequestInfo* info);
  ServerStats stats() const;
  size_t used_bytes() const;

 private:
  struct Impl;
  std::unique_ptr<Impl> p_;
};

}  // namespace qcu
