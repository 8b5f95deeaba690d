// Even-odd preconditioned Krylov solves of M x = b, M = 1 - kappa D, for many
// right-hand sides at once.  The reference has no solver: cg_inverter is an
// empty stub (src/qcu.cu:173 of the reference); this is new work built on the
// MRHS hopping kernel.
//
// Schur system on the even sites:
//   Mhat = 1 - kappa^2 D_eo D_oe,   bhat = b_e + kappa D_eo b_o,
//   x_o  = b_o + kappa D_oe x_e,
// and Mhat^dag = 1 - kappa^2 D_eo^- D_oe^- (the dagger flag f = -1), because
// D^dag = gamma5 D gamma5 is the hop with f = -1.  With x_o reconstructed
// that way, |b - M x| over the full lattice equals |bhat - Mhat x_e|.
//
// CG  : CG on Mhat^dag Mhat that also tracks s = bhat - Mhat x (the residual
//       of the actual system), so convergence is tested on |s| / |b|.
// BiCGStab on Mhat directly.
//
// Mixed precision: the Krylov vectors live in FP32 (or FP64 for the plain
// FP64 solve) and the operator runs in the inner precision (FP64, FP32,
// FP16 or BF16 storage).  FP64 is used for exactly three things: the solution
// accumulator x, the true residual bhat - Mhat x recomputed at each reliable
// update, and every inner product / norm (FP64 accumulation in the BLAS
// reductions).  A reliable update happens when the iterated |s| of any RHS
// drops below delta times its value at the previous update, or when it
// reaches the tolerance.
//
// Per-RHS scalars (alpha, beta, omega, ...) and the activity mask stay on the
// device; a converged RHS is masked out of the hopping kernels and gets zero
// coefficients, so chunks of iterations run without host round trips and can
// be captured as CUDA graphs.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "session.h"

namespace qcu {
namespace {

constexpr int kChunk = 8;  // iterations between host checks

struct Scalars {
  double* rr;
  double* rr_new;
  double* qq;
  double* ss;
  double* ss_true;
  double* maxss;
  double* stop2;
  double* bb;
  double2* alpha;
  double2* nalpha;
  double2* beta;
  double2* omega;
  double2* nomega;
  double2* rho;
  double2* tmp1;
  double2* tmp2;
  double2* nbo;  // -beta * omega
  int* active;
  int* status;  // [0] active count, [1] update requested, [2] breakdown
};

__global__ void cg_alpha_kernel(Scalars S, int nrhs) {
  const int r = threadIdx.x;
  if (r >= nrhs) return;
  double a = 0.0;
  if (S.active[r]) {
    const double q = S.qq[r];
    if (q > 0.0 && isfinite(q)) {
      a = S.rr[r] / q;
    } else {
      S.active[r] = 0;
      S.status[2] = 1;
    }
  }
  S.alpha[r] = make_double2(a, 0.0);
  S.nalpha[r] = make_double2(-a, 0.0);
}

// beta, convergence and reliable-update test; one block of >= nrhs threads
__global__ void cg_beta_kernel(Scalars S, int nrhs, double delta2) {
  const int r = threadIdx.x;
  int act = 0, upd = 0;
  if (r < nrhs) {
    double b = 0.0;
    if (S.active[r]) {
      b = S.rr_new[r] / S.rr[r];
      S.rr[r] = S.rr_new[r];
      const double ss = S.ss[r];
      if (!(ss > S.stop2[r])) {  // reached the tolerance (or NaN): verify in FP64
        S.active[r] = 0;
        upd = 1;
      } else if (ss < delta2 * S.maxss[r]) {
        upd = 1;
      }
      act = S.active[r];
    }
    S.beta[r] = make_double2(b, 0.0);
  }
  const int n_act = __syncthreads_count(act);
  const int n_upd = __syncthreads_count(upd);
  if (threadIdx.x == 0) {
    S.status[0] = n_act;
    if (n_upd) S.status[1] = 1;
  }
}

// After a reliable update replaces r by the recomputed residual, restore the
// CG invariant <r, p> = |r|^2 by p <- p + c r, c = 1 - <r, p> / |r|^2 (tmp1 =
// <r, p>).  With a 16-bit operator the iterated residual drifts away from the
// true one between updates; keeping p unchanged then breaks conjugacy.
__global__ void cg_restore_kernel(Scalars S, int nrhs) {
  const int r = threadIdx.x;
  if (r >= nrhs) return;
  double2 c = make_double2(0.0, 0.0);
  const double rr = S.rr[r];
  if (S.active[r] && rr > 0.0 && isfinite(rr)) c = make_double2(1.0 - S.tmp1[r].x / rr, -S.tmp1[r].y / rr);
  S.tmp2[r] = c;
}

// BiCGStab: alpha = rho / <r0, v>
__global__ void bicg_alpha_kernel(Scalars S, int nrhs) {
  const int r = threadIdx.x;
  if (r >= nrhs) return;
  double2 a = make_double2(0.0, 0.0);
  if (S.active[r]) {
    const double2 d = S.tmp1[r], rho = S.rho[r];
    const double den = d.x * d.x + d.y * d.y;
    if (den > 0.0 && isfinite(den)) {
      a = make_double2((rho.x * d.x + rho.y * d.y) / den, (rho.y * d.x - rho.x * d.y) / den);
    } else {
      S.active[r] = 0;
      S.status[2] = 1;
    }
  }
  S.alpha[r] = a;
  S.nalpha[r] = make_double2(-a.x, -a.y);
}

// omega = <t, s> / <t, t>   (tmp1 = <t, s>, qq = |t|^2)
__global__ void bicg_omega_kernel(Scalars S, int nrhs) {
  const int r = threadIdx.x;
  if (r >= nrhs) return;
  double2 w = make_double2(0.0, 0.0);
  if (S.active[r]) {
    const double tt = S.qq[r];
    if (tt > 0.0 && isfinite(tt)) {
      w = make_double2(S.tmp1[r].x / tt, S.tmp1[r].y / tt);
    } else {
      S.active[r] = 0;
      S.status[2] = 1;
    }
  }
  S.omega[r] = w;
  S.nomega[r] = make_double2(-w.x, -w.y);
}

// beta = (rho_new / rho) (alpha / omega); tmp2 = rho_new; test |r|
__global__ void bicg_beta_kernel(Scalars S, int nrhs, double delta2) {
  const int r = threadIdx.x;
  int act = 0, upd = 0;
  if (r < nrhs) {
    double2 b = make_double2(0.0, 0.0), nbo = make_double2(0.0, 0.0);
    if (S.active[r]) {
      const double2 rn = S.tmp2[r], ro = S.rho[r], a = S.alpha[r], w = S.omega[r];
      // q1 = rn / ro, q2 = a / w
      const double d1 = ro.x * ro.x + ro.y * ro.y, d2 = w.x * w.x + w.y * w.y;
      if (d1 > 0.0 && d2 > 0.0 && isfinite(d1) && isfinite(d2)) {
        const double2 q1 = make_double2((rn.x * ro.x + rn.y * ro.y) / d1, (rn.y * ro.x - rn.x * ro.y) / d1);
        const double2 q2 = make_double2((a.x * w.x + a.y * w.y) / d2, (a.y * w.x - a.x * w.y) / d2);
        b = make_double2(q1.x * q2.x - q1.y * q2.y, q1.x * q2.y + q1.y * q2.x);
        nbo = make_double2(-(b.x * w.x - b.y * w.y), -(b.x * w.y + b.y * w.x));
        S.rho[r] = rn;
      } else {
        S.active[r] = 0;
        S.status[2] = 1;
      }
      const double ss = S.ss[r];
      if (S.active[r]) {
        if (!(ss > S.stop2[r])) {
          S.active[r] = 0;
          upd = 1;
        } else if (ss < delta2 * S.maxss[r]) {
          upd = 1;
        }
      }
      act = S.active[r];
    }
    S.beta[r] = b;
    S.nbo[r] = nbo;
  }
  const int n_act = __syncthreads_count(act);
  const int n_upd = __syncthreads_count(upd);
  if (threadIdx.x == 0) {
    S.status[0] = n_act;
    if (n_upd) S.status[1] = 1;
  }
}

FieldRef ref(const FieldView& f, const Session& s) {
  FieldRef r;
  r.data = f.data;
  r.prec = f.prec;
  r.nrhs = f.nrhs;
  r.n = (int64_t)s.geo.vh * 4 * s.N * f.nrhs;
  return r;
}

class Solver {
 public:
  Solver(Session& s, int nrhs, const SolveRequest& q) : s_(s), n_(nrhs), q_(q) {
    kp_ = q.inner_prec == PREC_DOUBLE ? PREC_DOUBLE : PREC_SINGLE;
    op_ = q.inner_prec;
    kappa2_ = q.kappa * q.kappa;
    delta2_ = (q.inner_prec == PREC_DOUBLE) ? 0.0 : q.delta * q.delta;
    st_ = s.stream();
    // FP64 fields
    be_ = s.alloc_field("sv.be", PREC_DOUBLE, n_);
    bo_ = s.alloc_field("sv.bo", PREC_DOUBLE, n_);
    bh_ = s.alloc_field("sv.bh", PREC_DOUBLE, n_);
    xh_ = s.alloc_field("sv.xh", PREC_DOUBLE, n_);
    xo_ = s.alloc_field("sv.xo", PREC_DOUBLE, n_);
    sh_ = s.alloc_field("sv.sh", PREC_DOUBLE, n_);
    th_ = s.alloc_field("sv.th", PREC_DOUBLE, n_);
    tmp64_ = s.alloc_field("sv.tmp64", PREC_DOUBLE, n_);
    // Krylov fields
    xl_ = s.alloc_field("sv.xl", kp_, n_);
    sl_ = s.alloc_field("sv.sl", kp_, n_);
    rl_ = s.alloc_field("sv.rl", kp_, n_);
    pl_ = s.alloc_field("sv.pl", kp_, n_);
    ql_ = s.alloc_field("sv.ql", kp_, n_);
    wl_ = s.alloc_field("sv.wl", kp_, n_);
    r0l_ = s.alloc_field("sv.r0l", kp_, n_);
    // operator-precision fields
    if (op_ != kp_) {
      pop_ = s.alloc_field("sv.pop", op_, n_);
      qop_ = s.alloc_field("sv.qop", op_, n_);
      wop_ = s.alloc_field("sv.wop", op_, n_);
    }
    tmpop_ = s.alloc_field("sv.tmpop", op_, n_);
    // scalars
    const int R = QCU_MAX_RHS;
    double* d = s.scalars((size_t)R * 40 + 16);
    S_.rr = d;
    S_.rr_new = d + R;
    S_.qq = d + 2 * R;
    S_.ss = d + 3 * R;
    S_.ss_true = d + 4 * R;
    S_.maxss = d + 5 * R;
    S_.stop2 = d + 6 * R;
    S_.bb = d + 7 * R;
    double2* c = reinterpret_cast<double2*>(d + 8 * R);
    S_.alpha = c;
    S_.nalpha = c + R;
    S_.beta = c + 2 * R;
    S_.omega = c + 3 * R;
    S_.nomega = c + 4 * R;
    S_.rho = c + 5 * R;
    S_.tmp1 = c + 6 * R;
    S_.tmp2 = c + 7 * R;
    S_.nbo = c + 8 * R;
    int* ip = reinterpret_cast<int*>(c + 9 * R);  // d + 26R ..
    S_.active = ip;
    S_.status = ip + R;
    ones_ = reinterpret_cast<double2*>(s.ws.get("sv.ones", sizeof(double2) * R));
    mones_ = reinterpret_cast<double2*>(s.ws.get("sv.mones", sizeof(double2) * R));
    kap_ = reinterpret_cast<double2*>(s.ws.get("sv.kap", sizeof(double2) * R));
    std::vector<double2> h(R);
    for (auto& v : h) v = make_double2(1.0, 0.0);
    QCU_CHECK_CUDA(cudaMemcpyAsync(ones_, h.data(), sizeof(double2) * R, cudaMemcpyHostToDevice, st_));
    for (auto& v : h) v = make_double2(-1.0, 0.0);
    QCU_CHECK_CUDA(cudaMemcpyAsync(mones_, h.data(), sizeof(double2) * R, cudaMemcpyHostToDevice, st_));
    QCU_CHECK_CUDA(cudaStreamSynchronize(st_));
  }

  ~Solver() {
    if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
  }

  SolveResult run(void* const* x, void* const* b) {
    auto t0 = std::chrono::steady_clock::now();
    SolveResult res;
    Blas& B = s_.blas();
    PtrArray pb{}, px{};
    for (int r = 0; r < n_; r++) {
      pb.p[r] = b[r];
      px.p[r] = x[r];
    }
    // zero every work field so masked RHS never meet uninitialised memory
    for (FieldView* f : {&xh_, &xo_, &sh_, &th_, &tmp64_, &xl_, &sl_, &rl_, &pl_, &ql_, &wl_, &r0l_, &pop_, &qop_,
                         &wop_, &tmpop_}) {
      if (!f->data) continue;
      QCU_CHECK_CUDA(cudaMemsetAsync(f->data, 0, s_.field_bytes(f->prec, n_), st_));
      if (f->norm) QCU_CHECK_CUDA(cudaMemsetAsync(f->norm, 0, s_.norm_bytes(f->prec, n_), st_));
    }
    pack_fermions(PREC_DOUBLE, s_.N, pb, q_.src_mode, 0, be_.data, nullptr, s_.geo, n_, st_);
    pack_fermions(PREC_DOUBLE, s_.N, pb, q_.src_mode, 1, bo_.data, nullptr, s_.geo, n_, st_);
    // |b|^2 over both parities; stop when |s|^2 <= tol^2 |b|^2
    B.norm2(ref(be_, s_), S_.bb, st_);
    B.norm2(ref(bo_, s_), S_.ss_true, st_);
    std::vector<double> bb(n_), bo2(n_);
    QCU_CHECK_CUDA(cudaMemcpyAsync(bb.data(), S_.bb, sizeof(double) * n_, cudaMemcpyDeviceToHost, st_));
    QCU_CHECK_CUDA(cudaMemcpyAsync(bo2.data(), S_.ss_true, sizeof(double) * n_, cudaMemcpyDeviceToHost, st_));
    QCU_CHECK_CUDA(cudaStreamSynchronize(st_));
    stop2_host_.resize(n_);
    bb_host_.resize(n_);
    for (int r = 0; r < n_; r++) {
      bb_host_[r] = bb[r] + bo2[r];
      stop2_host_[r] = q_.tol * q_.tol * bb_host_[r];
    }
    QCU_CHECK_CUDA(cudaMemcpyAsync(S_.stop2, stop2_host_.data(), sizeof(double) * n_, cudaMemcpyHostToDevice, st_));
    // bhat = b_e + kappa D_eo b_o
    s_.hop(bh_, bo_, be_, 0, 0, q_.kappa, 1.0);

    converged_.assign(n_, 0);
    std::vector<int> zero_act(n_, 0);
    int iters = 0;
    bool any_active = reliable_update(true);
    res.reliable_updates = 0;
    if (q_.solver == 0) {
      B.copy(ref(rl_, s_), ref(pl_, s_), st_);
    } else {
      B.copy(ref(sl_, s_), ref(r0l_, s_), st_);  // shadow residual
      B.copy(ref(sl_, s_), ref(pl_, s_), st_);
      B.cdot(ref(r0l_, s_), ref(sl_, s_), S_.rho, st_);
    }
    while (any_active && iters < q_.max_iter) {
      const int k = std::min(chunk_, q_.max_iter - iters);
      run_chunk(k);
      iters += k;
      int status[3];
      QCU_CHECK_CUDA(cudaMemcpyAsync(status, S_.status, sizeof(int) * 3, cudaMemcpyDeviceToHost, st_));
      QCU_CHECK_CUDA(cudaStreamSynchronize(st_));
      if (verbose_) trace(iters, status);
      if (status[1] || status[0] == 0 || status[2]) {
        any_active = reliable_update(false);
        res.reliable_updates++;
        if (any_active && q_.solver == 1) {
          // restart the BiCGStab recurrence from the corrected residual
          B.copy(ref(sl_, s_), ref(pl_, s_), st_);
          B.cdot(ref(r0l_, s_), ref(sl_, s_), S_.rho, st_);
        }
      }
    }
    if (any_active) reliable_update(false);
    // x_o = b_o + kappa D_oe x_e
    s_.hop(xo_, xh_, bo_, 1, 0, q_.kappa, 1.0);
    unpack_fermions(PREC_DOUBLE, s_.N, px, q_.src_mode, 0, xh_.data, nullptr, s_.geo, n_, st_);
    unpack_fermions(PREC_DOUBLE, s_.N, px, q_.src_mode, 1, xo_.data, nullptr, s_.geo, n_, st_);
    QCU_CHECK_CUDA(cudaStreamSynchronize(st_));
    res.iterations = iters;
    res.true_residual.resize(n_);
    res.converged = converged_;
    for (int r = 0; r < n_; r++) res.true_residual[r] = std::sqrt(ss_true_host_[r] / bb_host_[r]);
    res.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return res;
  }

 private:
  // out = Mhat in (dagger 0) or Mhat^dag in (dagger 1), fields in precision `prec`
  void apply_mhat(const FieldView& out, const FieldView& in, const FieldView& tmp, int dagger, const int* mask) {
    s_.hop(tmp, in, FieldView{}, 1, dagger, 1.0, 0.0, mask);
    s_.hop(out, tmp, in, 0, dagger, -kappa2_, 1.0, mask);
  }

  // Krylov-precision q = Mhat p (and w = Mhat^dag q when want_w)
  void op_apply(const FieldView& out_kp, const FieldView& in_kp, int dagger, const FieldView* chain_out = nullptr) {
    if (op_ == kp_) {
      apply_mhat(out_kp, in_kp, tmpop_, dagger, S_.active);
    } else {
      convert_field(kp_, in_kp.data, nullptr, op_, pop_.data, pop_.norm, s_.geo.vh, 4 * s_.N, n_, st_);
      apply_mhat(qop_, pop_, tmpop_, dagger, S_.active);
      convert_field(op_, qop_.data, qop_.norm, kp_, out_kp.data, nullptr, s_.geo.vh, 4 * s_.N, n_, st_);
    }
    (void)chain_out;
  }

  // CG step pieces: q = Mhat p, w = Mhat^dag q (reusing the operator-precision q)
  void cg_apply() {
    if (op_ == kp_) {
      apply_mhat(ql_, pl_, tmpop_, 0, S_.active);
      apply_mhat(wl_, ql_, tmpop_, 1, S_.active);
    } else {
      convert_field(kp_, pl_.data, nullptr, op_, pop_.data, pop_.norm, s_.geo.vh, 4 * s_.N, n_, st_);
      apply_mhat(qop_, pop_, tmpop_, 0, S_.active);
      apply_mhat(wop_, qop_, tmpop_, 1, S_.active);
      convert_field(op_, qop_.data, qop_.norm, kp_, ql_.data, nullptr, s_.geo.vh, 4 * s_.N, n_, st_);
      convert_field(op_, wop_.data, wop_.norm, kp_, wl_.data, nullptr, s_.geo.vh, 4 * s_.N, n_, st_);
    }
  }

  void cg_iteration() {
    Blas& B = s_.blas();
    cg_apply();
    B.norm2(ref(ql_, s_), S_.qq, st_);
    cg_alpha_kernel<<<1, QCU_MAX_RHS, 0, st_>>>(S_, n_);
    B.axpby(S_.alpha, ref(pl_, s_), nullptr, ref(xl_, s_), st_);               // x += a p
    B.axpby_norm(S_.nalpha, ref(ql_, s_), nullptr, ref(sl_, s_), S_.ss, st_);  // s -= a q
    B.axpby_norm(S_.nalpha, ref(wl_, s_), nullptr, ref(rl_, s_), S_.rr_new, st_);  // r -= a w
    cg_beta_kernel<<<1, QCU_MAX_RHS, 0, st_>>>(S_, n_, delta2_);
    B.axpby(nullptr, ref(rl_, s_), S_.beta, ref(pl_, s_), st_);  // p = r + b p
  }

  void bicg_iteration() {
    Blas& B = s_.blas();
    // v = Mhat p (into ql)
    op_apply(ql_, pl_, 0);
    B.cdot(ref(r0l_, s_), ref(ql_, s_), S_.tmp1, st_);
    bicg_alpha_kernel<<<1, QCU_MAX_RHS, 0, st_>>>(S_, n_);
    // s = r - alpha v   (in place on sl, which holds r)
    B.axpby(S_.nalpha, ref(ql_, s_), nullptr, ref(sl_, s_), st_);
    // t = Mhat s (into wl)
    op_apply(wl_, sl_, 0);
    B.cdot(ref(wl_, s_), ref(sl_, s_), S_.tmp1, st_);
    B.norm2(ref(wl_, s_), S_.qq, st_);
    bicg_omega_kernel<<<1, QCU_MAX_RHS, 0, st_>>>(S_, n_);
    // x += alpha p + omega s
    B.axpbypcz(S_.alpha, ref(pl_, s_), S_.omega, ref(sl_, s_), nullptr, ref(xl_, s_), st_);
    // r = s - omega t  (sl becomes r)
    B.axpby_norm(S_.nomega, ref(wl_, s_), nullptr, ref(sl_, s_), S_.ss, st_);
    B.cdot(ref(r0l_, s_), ref(sl_, s_), S_.tmp2, st_);
    bicg_beta_kernel<<<1, QCU_MAX_RHS, 0, st_>>>(S_, n_, delta2_);
    // p = r + beta p - beta omega v
    B.axpbypcz(ones_, ref(sl_, s_), S_.nbo, ref(ql_, s_), S_.beta, ref(pl_, s_), st_);
  }

  void run_chunk(int k) {
    QCU_CHECK_CUDA(cudaMemsetAsync(S_.status, 0, sizeof(int) * 3, st_));
    if (q_.use_graph && k == chunk_) {
      if (!graph_exec_) {
        // the kernel shapes must be tuned before capture; one eager chunk does it
        if (!warm_) {
          for (int i = 0; i < k; i++) q_.solver == 0 ? cg_iteration() : bicg_iteration();
          warm_ = true;
          return;
        }
        cudaGraph_t g;
        QCU_CHECK_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
        try {
          for (int i = 0; i < k; i++) q_.solver == 0 ? cg_iteration() : bicg_iteration();
        } catch (...) {
          cudaGraph_t dummy;
          cudaStreamEndCapture(st_, &dummy);
          if (dummy) cudaGraphDestroy(dummy);
          throw;
        }
        QCU_CHECK_CUDA(cudaStreamEndCapture(st_, &g));
        QCU_CHECK_CUDA(cudaGraphInstantiate(&graph_exec_, g, 0));
        QCU_CHECK_CUDA(cudaGraphDestroy(g));
      }
      QCU_CHECK_CUDA(cudaGraphLaunch(graph_exec_, st_));
    } else {
      for (int i = 0; i < k; i++) q_.solver == 0 ? cg_iteration() : bicg_iteration();
    }
  }

  // x += x_lo; s = bhat - Mhat x in FP64; reset the Krylov residuals.
  // Returns whether any RHS is still unconverged.
  bool reliable_update(bool first) {
    Blas& B = s_.blas();
    if (!first) {
      B.add_to(ref(xl_, s_), ref(xh_, s_), st_);
      B.zero(ref(xl_, s_), st_);
    }
    // s = bhat - Mhat x
    apply_mhat(th_, xh_, tmp64_, 0, nullptr);
    B.copy(ref(bh_, s_), ref(sh_, s_), st_);
    B.axpby_norm(mones_, ref(th_, s_), nullptr, ref(sh_, s_), S_.ss_true, st_);
    ss_true_host_.resize(n_);
    QCU_CHECK_CUDA(cudaMemcpyAsync(ss_true_host_.data(), S_.ss_true, sizeof(double) * n_, cudaMemcpyDeviceToHost, st_));
    QCU_CHECK_CUDA(cudaStreamSynchronize(st_));
    std::vector<int> act(n_);
    bool any = false;
    for (int r = 0; r < n_; r++) {
      converged_[r] = ss_true_host_[r] <= stop2_host_[r] ? 1 : 0;
      act[r] = converged_[r] ? 0 : 1;
      any |= act[r] != 0;
    }
    if (verbose_) {
      fprintf(stderr, "qcu solver: reliable update %d, true |s|/|b| per RHS:", updates_);
      for (int r = 0; r < n_; r++) fprintf(stderr, " %.3e", std::sqrt(ss_true_host_[r] / bb_host_[r]));
      fprintf(stderr, "\n");
    }
    updates_++;
    QCU_CHECK_CUDA(cudaMemcpyAsync(S_.active, act.data(), sizeof(int) * n_, cudaMemcpyHostToDevice, st_));
    QCU_CHECK_CUDA(cudaMemcpyAsync(S_.maxss, S_.ss_true, sizeof(double) * n_, cudaMemcpyDeviceToDevice, st_));
    QCU_CHECK_CUDA(cudaMemcpyAsync(S_.ss, S_.ss_true, sizeof(double) * n_, cudaMemcpyDeviceToDevice, st_));
    // Krylov residuals in the low precision
    B.copy(ref(sh_, s_), ref(sl_, s_), st_);
    if (q_.solver == 0) {
      op_apply(rl_, sl_, 1);  // r = Mhat^dag s
      B.norm2(ref(rl_, s_), S_.rr, st_);
      if (!first) {
        B.cdot(ref(rl_, s_), ref(pl_, s_), S_.tmp1, st_);
        cg_restore_kernel<<<1, QCU_MAX_RHS, 0, st_>>>(S_, n_);
        B.axpby(S_.tmp2, ref(rl_, s_), nullptr, ref(pl_, s_), st_);  // p += c r
      }
    }
    QCU_CHECK_CUDA(cudaStreamSynchronize(st_));
    return any;
  }

  Session& s_;
  int n_;
  SolveRequest q_;
  int kp_, op_;
  double kappa2_, delta2_;
  cudaStream_t st_;
  FieldView be_, bo_, bh_, xh_, xo_, sh_, th_, tmp64_;
  FieldView xl_, sl_, rl_, pl_, ql_, wl_, r0l_;
  FieldView pop_, qop_, wop_, tmpop_;
  Scalars S_;
  double2 *ones_, *mones_, *kap_;
  std::vector<double> stop2_host_, bb_host_, ss_true_host_;
  std::vector<int> converged_;
  cudaGraphExec_t graph_exec_ = nullptr;
  bool warm_ = false;
  bool verbose_ = getenv("QCU_SOLVER_VERBOSE") != nullptr;
  int updates_ = 0;
  int chunk_ = getenv("QCU_SOLVER_CHUNK") ? std::max(1, atoi(getenv("QCU_SOLVER_CHUNK"))) : kChunk;

  // per-chunk scalars of RHS 0 (QCU_SOLVER_VERBOSE)
  void trace(int iters, const int* status) {
    double v[5];
    double2 c[2];
    QCU_CHECK_CUDA(cudaMemcpyAsync(&v[0], S_.rr, sizeof(double), cudaMemcpyDeviceToHost, st_));
    QCU_CHECK_CUDA(cudaMemcpyAsync(&v[1], S_.qq, sizeof(double), cudaMemcpyDeviceToHost, st_));
    QCU_CHECK_CUDA(cudaMemcpyAsync(&v[2], S_.ss, sizeof(double), cudaMemcpyDeviceToHost, st_));
    QCU_CHECK_CUDA(cudaMemcpyAsync(&c[0], S_.alpha, sizeof(double2), cudaMemcpyDeviceToHost, st_));
    QCU_CHECK_CUDA(cudaMemcpyAsync(&c[1], S_.beta, sizeof(double2), cudaMemcpyDeviceToHost, st_));
    QCU_CHECK_CUDA(cudaStreamSynchronize(st_));
    fprintf(stderr, "qcu solver: iter %d active %d update %d | rhs0 rr %.3e qq %.3e ss/bb %.3e alpha %.3e beta %.3e\n",
            iters, status[0], status[1], v[0], v[1], v[2] / bb_host_[0], c[0].x, c[1].x);
  }
};

}  // namespace

SolveResult solve(Session& s, void* const* x, void* const* b, int nrhs, const SolveRequest& req) {
  QCU_REQUIRE(nrhs >= 1 && nrhs <= QCU_MAX_RHS, QCU_ERR_INVALID_ARGUMENT, "nrhs must be in 1..256");
  QCU_REQUIRE(req.solver == 0 || req.solver == 1, QCU_ERR_INVALID_ARGUMENT, "unknown solver");
  QCU_REQUIRE(prec_valid(req.inner_prec), QCU_ERR_INVALID_ARGUMENT, "bad inner precision");
  QCU_REQUIRE(req.tol > 0 && req.max_iter > 0, QCU_ERR_INVALID_ARGUMENT, "tol and max_iter must be positive");
  QCU_REQUIRE(req.src_mode == SRC_EO_FULL || req.src_mode == SRC_LEX, QCU_ERR_INVALID_ARGUMENT,
              "solver fields must be full eo or lexicographic");
  Solver sv(s, nrhs, req);
  return sv.run(x, b);
}

}  // namespace qcu
