// Slot-based MRHS Krylov engine (solver.cu): the one-shot solves of
// qcuInvert / cg_inverter and the continuous-batching serving loop
// (serve.cu) both run on it.
#pragma once

#include <string>
#include <vector>

#include "session.h"

namespace qcu {

// per-slot device scalars (arrays of QCU_MAX_RHS entries)
struct SolverScalars {
  double *rr, *rr_new, *qq, *ss, *ss_true, *maxss, *stop2, *bb, *bo2, *kap_d, *nk2_d;
  double2 *alpha, *nalpha, *beta, *omega, *nomega, *rho, *tmp1, *tmp2, *nbo;
  double2 *cm, *ck, *cn, *zero, *one;  // masked-operation coefficients from sel
  float* nk2_f;                        // -kappa^2 for FP32 arithmetic
  int* active;                         // slot iterates
  int* upd;                            // slot asks for a reliable update
  int* sel;                            // slots selected for a masked operation
  int* status;                         // [0] active count of the last chunk
};

struct SlotState {
  enum Phase { FREE = 0, ACTIVE = 1, DONE = 2 };
  int phase = FREE;
  bool reported = false;
  int converged = 0;
  int bad_source = 0;  // the source held NaN or Inf: the slot is finished unsolved
  int iterations = 0;
  int updates = 0;
  double kappa = 0.0, tol = 0.0, bb = 1.0, stop2 = 0.0, true_res2 = 0.0;
};

class SlotEngine {
 public:
  SlotEngine(Session& s, int capacity, const SolveRequest& q, const std::string& tag);
  ~SlotEngine();
  SlotEngine(const SlotEngine&) = delete;
  SlotEngine& operator=(const SlotEngine&) = delete;

  // device memory the engine's fields take for this session and capacity
  static size_t bytes_needed(const Session& s, int capacity, int inner_prec);

  int capacity() const { return n_; }
  std::vector<int> free_slots() const;
  int active_slots() const;
  const SlotState& slot(int r) const { return host_[r]; }

  // Start solving M_r x_r = b_r in the given free slots (b_r: caller FP64
  // fields in src_mode layout, kappa_r, tolerance tol_r on |b - M x| / |b|).
  void admit(const std::vector<int>& slots, void* const* b, const double* kappa, const double* tol, int src_mode);
  // One chunk of iterations over the active slots and the per-slot reliable
  // updates it triggers.  Returns the slots that finished since the last call.
  std::vector<int> step();
  // Write the solutions of finished slots to x (caller FP64 fields) and free them.
  void retire(const std::vector<int>& slots, void* const* x, int src_mode);

 private:
  FieldRef ref(const FieldView& f) const;
  void upload_sel(const std::vector<int>& slots);
  void upload_kappa();
  void apply_mhat(const FieldView& out, const FieldView& in, const FieldView& tmp, const FieldView& tmp2, int dagger,
                  const int* mask);
  void op_apply(const FieldView& out_kp, const FieldView& in_kp, int dagger, const int* mask);
  void cg_iteration();
  void bicg_iteration();
  void run_chunk(int k);
  void restart(const std::vector<int>& slots, bool fresh);

  Session& s_;
  int n_;
  SolveRequest q_;
  int kp_, op_;
  double delta2_;
  cudaStream_t st_;
  FieldView be_, bo_, bh_, xh_, xo_, sh_, th_, tmp64_;
  FieldView xl_, sl_, rl_, pl_, ql_, wl_, r0l_;
  FieldView pop_, qop_, wop_, tmpop_;
  FieldView tmp64b_, tmpopb_;  // second temporaries of the clover operator
  bool cl_ = false;            // Wilson-clover: M = A - kappa D
  SolverScalars S_{};
  std::vector<SlotState> host_;
  cudaGraphExec_t graph_exec_ = nullptr;
  bool warm_ = false;
  bool verbose_ = getenv("QCU_SOLVER_VERBOSE") != nullptr;
  int chunk_ = getenv("QCU_SOLVER_CHUNK") ? std::max(1, atoi(getenv("QCU_SOLVER_CHUNK"))) : 8;
};

}  // namespace qcu
