// Even-odd preconditioned Krylov solves of M x = b, M = 1 - kappa D, for many
// right-hand sides at once.  The reference has no solver: cg_inverter is an
// empty stub (src/qcu.cu:173 of the reference); this is new work built on the
// MRHS hopping kernel.
//
// Schur system on the even sites, per RHS r with its own kappa_r:
//   Mhat_r = 1 - kappa_r^2 D_eo D_oe,   bhat_r = b_e + kappa_r D_eo b_o,
//   x_o    = b_o + kappa_r D_oe x_e,
// and Mhat^dag = 1 - kappa^2 D_eo^- D_oe^- (the dagger flag f = -1), because
// D^dag = gamma5 D gamma5 is the hop with f = -1.  With x_o reconstructed
// that way, |b - M x| over the full lattice equals |bhat - Mhat x_e|.
// With a clover field (M = A - kappa D, A Hermitian and block diagonal in
// chirality, so A commutes with gamma5):
//   Mhat_r = A_ee - kappa_r^2 D_eo A_oo^-1 D_oe,  bhat_r = b_e + kappa_r D_eo A_oo^-1 b_o,
//   x_o    = A_oo^-1 (b_o + kappa_r D_oe x_e),   Mhat^dag = Mhat with f = -1.
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
// reductions).
//
// Slots.  The engine owns `capacity` RHS slots.  A slot is admitted (its
// source packed, its state initialised), iterates, and is retired (its
// solution unpacked) independently of the others: every per-RHS scalar
// (alpha, beta, kappa, tolerance, ...) and the activity mask live in device
// arrays, and every per-slot initialisation / update is a masked operation.
// Reliable updates are per slot too: slot r is updated when its own iterated
// residual has dropped by delta since its last update or reached its
// tolerance.  A slot's arithmetic therefore depends only on its own data and
// iteration count, not on which other slots are occupied.  Iterations run in
// chunks of 8 with no host round trip; a chunk is captured once as a CUDA
// graph and replayed.  Between chunks the host retires finished slots and
// admits new ones (continuous batching, used by the serving loop).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "solver.h"

namespace qcu {
namespace {

__global__ void cg_alpha_kernel(SolverScalars S, int nrhs) {
  const int r = threadIdx.x;
  if (r >= nrhs) return;
  double a = 0.0;
  if (S.active[r]) {
    const double q = S.qq[r];
    if (q > 0.0 && isfinite(q)) {
      a = S.rr[r] / q;
    } else {
      S.active[r] = 0;
      S.upd[r] = 1;
    }
  }
  S.alpha[r] = make_double2(a, 0.0);
  S.nalpha[r] = make_double2(-a, 0.0);
}

// beta, convergence and reliable-update test per slot; one block of >= nrhs threads
__global__ void cg_beta_kernel(SolverScalars S, int nrhs, double delta2) {
  const int r = threadIdx.x;
  int act = 0;
  if (r < nrhs) {
    double b = 0.0;
    if (S.active[r]) {
      b = S.rr_new[r] / S.rr[r];
      S.rr[r] = S.rr_new[r];
      const double ss = S.ss[r];
      if (!(ss > S.stop2[r])) {  // reached the tolerance (or NaN): verify in FP64
        S.active[r] = 0;
        S.upd[r] = 1;
      } else if (ss < delta2 * S.maxss[r]) {
        S.upd[r] = 1;
      }
      act = S.active[r];
    }
    S.beta[r] = make_double2(b, 0.0);
  }
  const int n_act = __syncthreads_count(act);
  if (threadIdx.x == 0) S.status[0] = n_act;
}

// BiCGStab: alpha = rho / <r0, v>
__global__ void bicg_alpha_kernel(SolverScalars S, int nrhs) {
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
      S.upd[r] = 1;
    }
  }
  S.alpha[r] = a;
  S.nalpha[r] = make_double2(-a.x, -a.y);
}

// omega = <t, s> / <t, t>   (tmp1 = <t, s>, qq = |t|^2)
__global__ void bicg_omega_kernel(SolverScalars S, int nrhs) {
  const int r = threadIdx.x;
  if (r >= nrhs) return;
  double2 w = make_double2(0.0, 0.0);
  if (S.active[r]) {
    const double tt = S.qq[r];
    if (tt > 0.0 && isfinite(tt)) {
      w = make_double2(S.tmp1[r].x / tt, S.tmp1[r].y / tt);
    } else {
      S.active[r] = 0;
      S.upd[r] = 1;
    }
  }
  S.omega[r] = w;
  S.nomega[r] = make_double2(-w.x, -w.y);
}

// beta = (rho_new / rho) (alpha / omega); tmp2 = rho_new; test |r|
__global__ void bicg_beta_kernel(SolverScalars S, int nrhs, double delta2) {
  const int r = threadIdx.x;
  int act = 0;
  if (r < nrhs) {
    double2 b = make_double2(0.0, 0.0), nbo = make_double2(0.0, 0.0);
    if (S.active[r]) {
      const double2 rn = S.tmp2[r], ro = S.rho[r], a = S.alpha[r], w = S.omega[r];
      const double d1 = ro.x * ro.x + ro.y * ro.y, d2 = w.x * w.x + w.y * w.y;
      if (d1 > 0.0 && d2 > 0.0 && isfinite(d1) && isfinite(d2)) {
        const double2 q1 = make_double2((rn.x * ro.x + rn.y * ro.y) / d1, (rn.y * ro.x - rn.x * ro.y) / d1);
        const double2 q2 = make_double2((a.x * w.x + a.y * w.y) / d2, (a.y * w.x - a.x * w.y) / d2);
        b = make_double2(q1.x * q2.x - q1.y * q2.y, q1.x * q2.y + q1.y * q2.x);
        nbo = make_double2(-(b.x * w.x - b.y * w.y), -(b.x * w.y + b.y * w.x));
        S.rho[r] = rn;
      } else {
        S.active[r] = 0;
        S.upd[r] = 1;
      }
      const double ss = S.ss[r];
      if (S.active[r]) {
        if (!(ss > S.stop2[r])) {
          S.active[r] = 0;
          S.upd[r] = 1;
        } else if (ss < delta2 * S.maxss[r]) {
          S.upd[r] = 1;
        }
      }
      act = S.active[r];
    }
    S.beta[r] = b;
    S.nbo[r] = nbo;
  }
  const int n_act = __syncthreads_count(act);
  if (threadIdx.x == 0) S.status[0] = n_act;
}

// masked-operation coefficients from sel: cm = sel, ck = 1 - sel, cn = -sel
__global__ void select_coeffs_kernel(SolverScalars S, int nrhs) {
  const int r = threadIdx.x;
  if (r >= nrhs) return;
  const double m = S.sel[r] ? 1.0 : 0.0;
  S.cm[r] = make_double2(m, 0.0);
  S.ck[r] = make_double2(1.0 - m, 0.0);
  S.cn[r] = make_double2(-m, 0.0);
  S.zero[r] = make_double2(0.0, 0.0);
  S.one[r] = make_double2(1.0, 0.0);
}

// after a (re)start of the selected slots: rr, maxss and ss from the fresh
// residuals; the CG invariant <r, p> = |r|^2 restored by p += c r with
// c = 1 - <r, p> / |r|^2 (fresh slots have p = 0, so p becomes r).  The
// update p += c r runs over every slot, so c = 0 for the slots not restarted.
__global__ void restart_kernel(SolverScalars S, int nrhs) {
  const int r = threadIdx.x;
  if (r >= nrhs) return;
  if (!S.sel[r]) {
    S.tmp2[r] = make_double2(0.0, 0.0);
    return;
  }
  S.rr[r] = S.rr_new[r];
  S.maxss[r] = S.ss_true[r];
  S.ss[r] = S.ss_true[r];
  S.upd[r] = 0;
  const double rr = S.rr_new[r];
  double2 c = make_double2(0.0, 0.0);
  if (rr > 0.0 && isfinite(rr)) c = make_double2(1.0 - S.tmp1[r].x / rr, -S.tmp1[r].y / rr);
  S.tmp2[r] = c;
}

// BiCGStab restart of the selected slots: rho = <r0, r> (tmp1)
__global__ void bicg_restart_kernel(SolverScalars S, int nrhs) {
  const int r = threadIdx.x;
  if (r >= nrhs || !S.sel[r]) return;
  S.maxss[r] = S.ss_true[r];
  S.ss[r] = S.ss_true[r];
  S.upd[r] = 0;
  S.rho[r] = S.tmp1[r];
}

}  // namespace

FieldRef SlotEngine::ref(const FieldView& f) const {
  FieldRef r;
  r.data = f.data;
  r.prec = f.prec;
  r.nrhs = f.nrhs;
  r.n = (int64_t)s_.geo.vh * 4 * s_.N * f.nrhs;
  return r;
}

size_t SlotEngine::bytes_needed(const Session& s, int capacity, int inner_prec) {
  const int kp = inner_prec == PREC_DOUBLE ? PREC_DOUBLE : PREC_SINGLE;
  size_t b = 8 * s.field_bytes(PREC_DOUBLE, capacity) + 7 * s.field_bytes(kp, capacity);
  if (s.has_clover()) b += s.field_bytes(PREC_DOUBLE, capacity) + s.field_bytes(inner_prec, capacity) +
                           s.norm_bytes(inner_prec, capacity);
  if (inner_prec != kp) b += 3 * (s.field_bytes(inner_prec, capacity) + s.norm_bytes(inner_prec, capacity));
  b += s.field_bytes(inner_prec, capacity) + s.norm_bytes(inner_prec, capacity);
  return b;
}

SlotEngine::SlotEngine(Session& s, int capacity, const SolveRequest& q, const std::string& tag)
    : s_(s), n_(capacity), q_(q) {
  inject_failure("solver");
  QCU_REQUIRE(capacity >= 1 && capacity <= QCU_MAX_RHS, QCU_ERR_INVALID_ARGUMENT, "slot capacity must be in 1..256");
  QCU_REQUIRE(q.solver == 0 || q.solver == 1, QCU_ERR_INVALID_ARGUMENT, "unknown solver");
  QCU_REQUIRE(prec_valid(q.inner_prec), QCU_ERR_INVALID_ARGUMENT, "bad inner precision");
  QCU_REQUIRE(!(q.clover && prec_site_major(q.inner_prec)), QCU_ERR_UNSUPPORTED,
              "clover: site-major BF16 fields are not supported");
  QCU_REQUIRE(!prec_site_major(q.inner_prec) || capacity % 4 == 0, QCU_ERR_UNSUPPORTED,
              "site-major BF16 inner fields take the tensor-core dslash: the RHS count must be a multiple of 4");
  kp_ = q.inner_prec == PREC_DOUBLE ? PREC_DOUBLE : PREC_SINGLE;
  op_ = q.inner_prec;
  delta2_ = (q.inner_prec == PREC_DOUBLE) ? 0.0 : q.delta * q.delta;
  st_ = s.stream();
  const std::string t = tag + ".";
  be_ = s.alloc_field(t + "be", PREC_DOUBLE, n_);
  bo_ = s.alloc_field(t + "bo", PREC_DOUBLE, n_);
  bh_ = s.alloc_field(t + "bh", PREC_DOUBLE, n_);
  xh_ = s.alloc_field(t + "xh", PREC_DOUBLE, n_);
  xo_ = s.alloc_field(t + "xo", PREC_DOUBLE, n_);
  sh_ = s.alloc_field(t + "sh", PREC_DOUBLE, n_);
  th_ = s.alloc_field(t + "th", PREC_DOUBLE, n_);
  tmp64_ = s.alloc_field(t + "tmp64", PREC_DOUBLE, n_);
  xl_ = s.alloc_field(t + "xl", kp_, n_);
  sl_ = s.alloc_field(t + "sl", kp_, n_);
  rl_ = s.alloc_field(t + "rl", kp_, n_);
  pl_ = s.alloc_field(t + "pl", kp_, n_);
  ql_ = s.alloc_field(t + "ql", kp_, n_);
  wl_ = s.alloc_field(t + "wl", kp_, n_);
  r0l_ = s.alloc_field(t + "r0l", kp_, n_);
  if (op_ != kp_) {
    pop_ = s.alloc_field(t + "pop", op_, n_);
    qop_ = s.alloc_field(t + "qop", op_, n_);
    wop_ = s.alloc_field(t + "wop", op_, n_);
  }
  tmpop_ = s.alloc_field(t + "tmpop", op_, n_);
  // BF16 operator fields are internal: they take the site-major layout where
  // the tensor-core dslash on it is measured faster (same bytes either way)
  if (op_ == PREC_BF16 && !q.clover && s.prefer_site_major(pop_, qop_)) {
    op_ = PREC_BF16S;
    for (FieldView* f : {&pop_, &qop_, &wop_, &tmpop_}) f->prec = PREC_BF16S;
  }
  cl_ = q.clover;
  QCU_REQUIRE(!cl_ || s.has_clover(), QCU_ERR_NO_OPERATOR, "clover solve requested but no clover field loaded");
  if (cl_) {
    tmp64b_ = s.alloc_field(t + "tmp64b", PREC_DOUBLE, n_);
    tmpopb_ = s.alloc_field(t + "tmpopb", op_, n_);
  }
  // per-slot device scalars
  const int R = QCU_MAX_RHS;
  char* d = static_cast<char*>(s.ws.get(t + "scalars", (size_t)R * 64 * sizeof(double) + 4096));
  double* dd = reinterpret_cast<double*>(d);
  S_.rr = dd;
  S_.rr_new = dd + R;
  S_.qq = dd + 2 * R;
  S_.ss = dd + 3 * R;
  S_.ss_true = dd + 4 * R;
  S_.maxss = dd + 5 * R;
  S_.stop2 = dd + 6 * R;
  S_.bb = dd + 7 * R;
  S_.bo2 = dd + 8 * R;
  S_.kap_d = dd + 9 * R;
  S_.nk2_d = dd + 10 * R;
  double2* c = reinterpret_cast<double2*>(dd + 11 * R);
  S_.alpha = c;
  S_.nalpha = c + R;
  S_.beta = c + 2 * R;
  S_.omega = c + 3 * R;
  S_.nomega = c + 4 * R;
  S_.rho = c + 5 * R;
  S_.tmp1 = c + 6 * R;
  S_.tmp2 = c + 7 * R;
  S_.nbo = c + 8 * R;
  S_.cm = c + 9 * R;
  S_.ck = c + 10 * R;
  S_.cn = c + 11 * R;
  S_.zero = c + 12 * R;
  S_.one = c + 13 * R;
  float* ff = reinterpret_cast<float*>(c + 14 * R);  // at dd + 39R
  S_.nk2_f = ff;
  int* ip = reinterpret_cast<int*>(ff + R);
  S_.active = ip;
  S_.upd = ip + R;
  S_.sel = ip + 2 * R;
  S_.status = ip + 3 * R;
  host_.assign(n_, SlotState{});
  QCU_CHECK_CUDA(cudaMemsetAsync(d, 0, (size_t)R * 64 * sizeof(double) + 4096, st_));
  // every field starts at zero: masked slots never meet uninitialised memory
  for (FieldView* f : {&be_, &bo_, &bh_, &xh_, &xo_, &sh_, &th_, &tmp64_, &xl_, &sl_, &rl_, &pl_, &ql_, &wl_, &r0l_,
                       &pop_, &qop_, &wop_, &tmpop_, &tmp64b_, &tmpopb_}) {
    if (!f->data) continue;
    QCU_CHECK_CUDA(cudaMemsetAsync(f->data, 0, s.field_bytes(f->prec, n_), st_));
    if (f->norm) QCU_CHECK_CUDA(cudaMemsetAsync(f->norm, 0, s.norm_bytes(f->prec, n_), st_));
  }
  s.blas();  // BLAS scratch, before any graph capture
  QCU_CHECK_CUDA(cudaStreamSynchronize(st_));
}

SlotEngine::~SlotEngine() {
  if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
}

std::vector<int> SlotEngine::free_slots() const {
  std::vector<int> f;
  for (int r = 0; r < n_; r++)
    if (host_[r].phase == SlotState::FREE) f.push_back(r);
  return f;
}

int SlotEngine::active_slots() const {
  int k = 0;
  for (int r = 0; r < n_; r++) k += host_[r].phase == SlotState::ACTIVE;
  return k;
}

void SlotEngine::upload_sel(const std::vector<int>& slots) {
  std::vector<int> m(n_, 0);
  for (int r : slots) m[r] = 1;
  QCU_CHECK_CUDA(cudaMemcpyAsync(S_.sel, m.data(), sizeof(int) * n_, cudaMemcpyHostToDevice, st_));
  select_coeffs_kernel<<<1, QCU_MAX_RHS, 0, st_>>>(S_, n_);
  QCU_CHECK_CUDA(cudaGetLastError());
  // the upload reads host memory asynchronously: keep it alive until done
  QCU_CHECK_CUDA(cudaStreamSynchronize(st_));
}

void SlotEngine::upload_kappa() {
  std::vector<double> k(n_), nk2(n_);
  std::vector<float> nk2f(n_);
  for (int r = 0; r < n_; r++) {
    k[r] = host_[r].kappa;
    nk2[r] = -host_[r].kappa * host_[r].kappa;
    nk2f[r] = (float)nk2[r];
  }
  QCU_CHECK_CUDA(cudaMemcpyAsync(S_.kap_d, k.data(), sizeof(double) * n_, cudaMemcpyHostToDevice, st_));
  QCU_CHECK_CUDA(cudaMemcpyAsync(S_.nk2_d, nk2.data(), sizeof(double) * n_, cudaMemcpyHostToDevice, st_));
  QCU_CHECK_CUDA(cudaMemcpyAsync(S_.nk2_f, nk2f.data(), sizeof(float) * n_, cudaMemcpyHostToDevice, st_));
  QCU_CHECK_CUDA(cudaStreamSynchronize(st_));
}

// out = Mhat in (dagger 0) or Mhat^dag in (dagger 1) for the slots in mask,
// fields in precision `prec` with per-slot kappa
void SlotEngine::apply_mhat(const FieldView& out, const FieldView& in, const FieldView& tmp, const FieldView& tmp2,
                            int dagger, const int* mask) {
  s_.hop(tmp, in, FieldView{}, 1, dagger, 1.0, 0.0, mask);
  FieldView hop_in = tmp, x = in;
  if (cl_) {  // A_oo^-1 D_oe in, and A_ee in for the xpay term
    s_.clover_apply(tmp2, tmp, FieldView{}, 1, true, 1.0, 0.0, mask);
    s_.clover_apply(tmp, in, FieldView{}, 0, false, 1.0, 0.0, mask);
    hop_in = tmp2;
    x = tmp;
  }
  if (in.prec == PREC_DOUBLE)
    s_.hop(out, hop_in, x, 0, dagger, 0.0, 1.0, mask, nullptr, S_.nk2_d);
  else
    s_.hop(out, hop_in, x, 0, dagger, 0.0, 1.0, mask, S_.nk2_f, nullptr);
}

// Krylov-precision out = Mhat in (or Mhat^dag) for the slots in mask
void SlotEngine::op_apply(const FieldView& out_kp, const FieldView& in_kp, int dagger, const int* mask) {
  if (op_ == kp_) {
    apply_mhat(out_kp, in_kp, tmpop_, tmpopb_, dagger, mask);
  } else {
    convert_field(kp_, in_kp.data, nullptr, op_, pop_.data, pop_.norm, s_.geo.vh, 4 * s_.N, n_, st_, mask);
    apply_mhat(qop_, pop_, tmpop_, tmpopb_, dagger, mask);
    convert_field(op_, qop_.data, qop_.norm, kp_, out_kp.data, nullptr, s_.geo.vh, 4 * s_.N, n_, st_, mask);
  }
}

void SlotEngine::cg_iteration() {
  Blas& B = s_.blas();
  if (op_ == kp_) {
    apply_mhat(ql_, pl_, tmpop_, tmpopb_, 0, S_.active);
    apply_mhat(wl_, ql_, tmpop_, tmpopb_, 1, S_.active);
  } else {
    convert_field(kp_, pl_.data, nullptr, op_, pop_.data, pop_.norm, s_.geo.vh, 4 * s_.N, n_, st_, S_.active);
    apply_mhat(qop_, pop_, tmpop_, tmpopb_, 0, S_.active);
    apply_mhat(wop_, qop_, tmpop_, tmpopb_, 1, S_.active);
    convert_field(op_, qop_.data, qop_.norm, kp_, ql_.data, nullptr, s_.geo.vh, 4 * s_.N, n_, st_, S_.active);
    convert_field(op_, wop_.data, wop_.norm, kp_, wl_.data, nullptr, s_.geo.vh, 4 * s_.N, n_, st_, S_.active);
  }
  B.norm2(ref(ql_), S_.qq, st_, false);
  cg_alpha_kernel<<<1, QCU_MAX_RHS, 0, st_>>>(S_, n_);
  B.axpby(S_.alpha, ref(pl_), nullptr, ref(xl_), st_);                  // x += a p
  B.axpby_norm(S_.nalpha, ref(ql_), nullptr, ref(sl_), S_.ss, st_);      // s -= a q
  B.axpby_norm(S_.nalpha, ref(wl_), nullptr, ref(rl_), S_.rr_new, st_);  // r -= a w
  cg_beta_kernel<<<1, QCU_MAX_RHS, 0, st_>>>(S_, n_, delta2_);
  B.axpby(nullptr, ref(rl_), S_.beta, ref(pl_), st_);  // p = r + b p
}

void SlotEngine::bicg_iteration() {
  Blas& B = s_.blas();
  op_apply(ql_, pl_, 0, S_.active);  // v = Mhat p
  B.cdot(ref(r0l_), ref(ql_), S_.tmp1, st_);
  bicg_alpha_kernel<<<1, QCU_MAX_RHS, 0, st_>>>(S_, n_);
  B.axpby(S_.nalpha, ref(ql_), nullptr, ref(sl_), st_);  // s = r - alpha v (sl holds r)
  op_apply(wl_, sl_, 0, S_.active);                       // t = Mhat s
  B.cdot(ref(wl_), ref(sl_), S_.tmp1, st_);
  B.norm2(ref(wl_), S_.qq, st_, false);
  bicg_omega_kernel<<<1, QCU_MAX_RHS, 0, st_>>>(S_, n_);
  B.axpbypcz(S_.alpha, ref(pl_), S_.omega, ref(sl_), nullptr, ref(xl_), st_);  // x += alpha p + omega s
  B.axpby_norm(S_.nomega, ref(wl_), nullptr, ref(sl_), S_.ss, st_);            // r = s - omega t
  B.cdot(ref(r0l_), ref(sl_), S_.tmp2, st_);
  bicg_beta_kernel<<<1, QCU_MAX_RHS, 0, st_>>>(S_, n_, delta2_);
  B.axpbypcz(S_.one, ref(sl_), S_.nbo, ref(ql_), S_.beta, ref(pl_), st_);  // p = r + beta p - beta omega v
}

void SlotEngine::run_chunk(int k) {
  QCU_CHECK_CUDA(cudaMemsetAsync(S_.status, 0, sizeof(int) * 4, st_));
  if (q_.use_graph && k == chunk_) {
    if (!graph_exec_) {
      // kernel shapes are tuned in the first (eager) chunk; later chunks replay a graph
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
        cudaGraph_t dummy = nullptr;
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

// (Re)start the slots in `slots`: fold x_lo into x, recompute the true
// residual s = bhat - Mhat x in FP64, decide convergence, and restart the
// Krylov recurrence of the slots that go on.  `fresh` slots start from x = 0
// with p = r.
void SlotEngine::restart(const std::vector<int>& slots, bool fresh) {
  if (slots.empty()) return;
  Blas& B = s_.blas();
  upload_sel(slots);
  if (!fresh) B.axpby(S_.cm, ref(xl_), nullptr, ref(xh_), st_);  // x += x_lo
  B.axpby(S_.zero, ref(xl_), S_.ck, ref(xl_), st_);              // x_lo = 0
  if (fresh) {
    B.axpby(S_.zero, ref(xh_), S_.ck, ref(xh_), st_);  // x = 0
    B.axpby(S_.zero, ref(pl_), S_.ck, ref(pl_), st_);  // p = 0
  }
  // s = bhat - Mhat x  (only the selected slots are computed); fresh slots
  // start from x = 0, so their true residual is bhat itself
  B.axpby(S_.cm, ref(bh_), S_.ck, ref(sh_), st_);
  if (fresh) {
    B.norm2(ref(sh_), S_.ss_true, st_);
  } else {
    apply_mhat(th_, xh_, tmp64_, tmp64b_, 0, S_.sel);
    B.axpby_norm(S_.cn, ref(th_), nullptr, ref(sh_), S_.ss_true, st_);
  }
  std::vector<double> ss(n_);
  QCU_CHECK_CUDA(cudaMemcpyAsync(ss.data(), S_.ss_true, sizeof(double) * n_, cudaMemcpyDeviceToHost, st_));
  std::vector<int> act(n_);
  QCU_CHECK_CUDA(cudaMemcpyAsync(act.data(), S_.active, sizeof(int) * n_, cudaMemcpyDeviceToHost, st_));
  QCU_CHECK_CUDA(cudaStreamSynchronize(st_));
  std::vector<int> go_on;
  for (int r : slots) {
    SlotState& h = host_[r];
    h.true_res2 = ss[r];
    h.updates += fresh ? 0 : 1;
    if (verbose_)
      fprintf(stderr, "qcu solver: slot %d %s after %d iterations, true |s|/|b| %.3e\n", r,
              fresh ? "admitted" : "reliable update", h.iterations, std::sqrt(ss[r] / h.bb));
    if (ss[r] <= h.stop2) {
      h.phase = SlotState::DONE;
      h.converged = 1;
      act[r] = 0;
    } else if (h.iterations >= q_.max_iter || !std::isfinite(ss[r])) {
      h.phase = SlotState::DONE;
      h.converged = 0;
      act[r] = 0;
    } else {
      h.phase = SlotState::ACTIVE;
      act[r] = 1;
      go_on.push_back(r);
    }
  }
  QCU_CHECK_CUDA(cudaMemcpyAsync(S_.active, act.data(), sizeof(int) * n_, cudaMemcpyHostToDevice, st_));
  if (go_on.empty()) {
    QCU_CHECK_CUDA(cudaStreamSynchronize(st_));
    return;
  }
  upload_sel(go_on);
  B.axpby(S_.cm, ref(sh_), S_.ck, ref(sl_), st_);  // s_lo = s
  if (q_.solver == 0) {
    op_apply(rl_, sl_, 1, S_.sel);  // r = Mhat^dag s
    B.norm2(ref(rl_), S_.rr_new, st_, false);
    B.cdot(ref(rl_), ref(pl_), S_.tmp1, st_);
    restart_kernel<<<1, QCU_MAX_RHS, 0, st_>>>(S_, n_);
    B.axpby(S_.tmp2, ref(rl_), nullptr, ref(pl_), st_);  // p += c r
  } else {
    B.axpby(S_.cm, ref(sl_), S_.ck, ref(r0l_), st_);  // shadow residual r0 = r
    B.axpby(S_.cm, ref(sl_), S_.ck, ref(pl_), st_);   // p = r
    B.cdot(ref(r0l_), ref(sl_), S_.tmp1, st_);
    bicg_restart_kernel<<<1, QCU_MAX_RHS, 0, st_>>>(S_, n_);
  }
  QCU_CHECK_CUDA(cudaGetLastError());
  QCU_CHECK_CUDA(cudaStreamSynchronize(st_));
}

void SlotEngine::admit(const std::vector<int>& slots, void* const* b, const double* kappa, const double* tol,
                       int src_mode) {
  if (slots.empty()) return;
  Blas& B = s_.blas();
  PtrArray pb{};
  for (size_t i = 0; i < slots.size(); i++) {
    const int r = slots[i];
    QCU_REQUIRE(r >= 0 && r < n_ && host_[r].phase == SlotState::FREE, QCU_ERR_INVALID_ARGUMENT,
                "admit: slot is not free");
    QCU_REQUIRE(tol[i] > 0 && kappa[i] > 0, QCU_ERR_INVALID_ARGUMENT, "kappa and tol must be positive");
    pb.p[r] = b[i];
    SlotState& h = host_[r];
    h = SlotState{};
    h.kappa = kappa[i];
    h.tol = tol[i];
    h.phase = SlotState::ACTIVE;
  }
  upload_kappa();
  pack_fermions(PREC_DOUBLE, s_.N, pb, src_mode, 0, be_.data, nullptr, s_.geo, n_, st_);
  pack_fermions(PREC_DOUBLE, s_.N, pb, src_mode, 1, bo_.data, nullptr, s_.geo, n_, st_);
  // |b|^2 over both parities; the slot stops when |s|^2 <= tol^2 |b|^2
  B.norm2(ref(be_), S_.bb, st_);
  B.norm2(ref(bo_), S_.bo2, st_);
  std::vector<double> bb(n_), bo2(n_), stop2(n_);
  QCU_CHECK_CUDA(cudaMemcpyAsync(bb.data(), S_.bb, sizeof(double) * n_, cudaMemcpyDeviceToHost, st_));
  QCU_CHECK_CUDA(cudaMemcpyAsync(bo2.data(), S_.bo2, sizeof(double) * n_, cudaMemcpyDeviceToHost, st_));
  QCU_CHECK_CUDA(cudaMemcpyAsync(stop2.data(), S_.stop2, sizeof(double) * n_, cudaMemcpyDeviceToHost, st_));
  QCU_CHECK_CUDA(cudaStreamSynchronize(st_));
  for (int r : slots) {
    SlotState& h = host_[r];
    const double b2 = bb[r] + bo2[r];
    // a non-finite source is not solved: its true residual is non-finite, so
    // restart() finishes the slot unconverged, and the caller is told why
    h.bad_source = std::isfinite(b2) ? 0 : 1;
    h.bb = (b2 > 0 && std::isfinite(b2)) ? b2 : 1.0;  // a zero source: x = 0 is exact
    h.stop2 = h.tol * h.tol * h.bb;
    stop2[r] = h.stop2;
  }
  QCU_CHECK_CUDA(cudaMemcpyAsync(S_.stop2, stop2.data(), sizeof(double) * n_, cudaMemcpyHostToDevice, st_));
  // bhat = b_e + kappa_r D_eo b_o (clover: b_e + kappa_r D_eo A_oo^-1 b_o) for the new slots
  upload_sel(slots);
  if (cl_) {
    s_.clover_apply(tmp64b_, bo_, FieldView{}, 1, true, 1.0, 0.0, S_.sel);
    s_.hop(bh_, tmp64b_, be_, 0, 0, 0.0, 1.0, S_.sel, nullptr, S_.kap_d);
  } else {
    s_.hop(bh_, bo_, be_, 0, 0, 0.0, 1.0, S_.sel, nullptr, S_.kap_d);
  }
  restart(slots, true);
}

std::vector<int> SlotEngine::step() {
  std::vector<int> finished;
  for (int r = 0; r < n_; r++)
    if (host_[r].phase == SlotState::DONE && !host_[r].reported) {
      host_[r].reported = true;
      finished.push_back(r);
    }
  if (active_slots() == 0) return finished;
  const int k = chunk_;
  run_chunk(k);
  std::vector<int> act(n_), upd(n_);
  QCU_CHECK_CUDA(cudaMemcpyAsync(act.data(), S_.active, sizeof(int) * n_, cudaMemcpyDeviceToHost, st_));
  QCU_CHECK_CUDA(cudaMemcpyAsync(upd.data(), S_.upd, sizeof(int) * n_, cudaMemcpyDeviceToHost, st_));
  s_.sync();
  std::vector<int> sel;
  for (int r = 0; r < n_; r++) {
    if (host_[r].phase != SlotState::ACTIVE) continue;
    host_[r].iterations += k;
    if (upd[r] || !act[r] || host_[r].iterations >= q_.max_iter) sel.push_back(r);
  }
  restart(sel, false);
  for (int r : sel)
    if (host_[r].phase == SlotState::DONE && !host_[r].reported) {
      host_[r].reported = true;
      finished.push_back(r);
    }
  return finished;
}

void SlotEngine::retire(const std::vector<int>& slots, void* const* x, int src_mode) {
  if (slots.empty()) return;
  PtrArray px{};
  for (size_t i = 0; i < slots.size(); i++) {
    const int r = slots[i];
    QCU_REQUIRE(r >= 0 && r < n_ && host_[r].phase == SlotState::DONE, QCU_ERR_INVALID_ARGUMENT,
                "retire: slot has not finished");
    px.p[r] = x[i];
  }
  upload_sel(slots);
  // x_o = b_o + kappa_r D_oe x_e (clover: A_oo^-1 of it)
  if (cl_) {
    s_.hop(tmp64b_, xh_, bo_, 1, 0, 0.0, 1.0, S_.sel, nullptr, S_.kap_d);
    s_.clover_apply(xo_, tmp64b_, FieldView{}, 1, true, 1.0, 0.0, S_.sel);
  } else {
    s_.hop(xo_, xh_, bo_, 1, 0, 0.0, 1.0, S_.sel, nullptr, S_.kap_d);
  }
  unpack_fermions(PREC_DOUBLE, s_.N, px, src_mode, 0, xh_.data, nullptr, s_.geo, n_, st_);
  unpack_fermions(PREC_DOUBLE, s_.N, px, src_mode, 1, xo_.data, nullptr, s_.geo, n_, st_);
  QCU_CHECK_CUDA(cudaStreamSynchronize(st_));
  for (int r : slots) host_[r].phase = SlotState::FREE;
}

SolveResult solve(Session& s, void* const* x, void* const* b, int nrhs, const SolveRequest& req) {
  QCU_REQUIRE(nrhs >= 1 && nrhs <= QCU_MAX_RHS, QCU_ERR_INVALID_ARGUMENT, "nrhs must be in 1..256");
  QCU_REQUIRE(req.tol > 0 && req.max_iter > 0, QCU_ERR_INVALID_ARGUMENT, "tol and max_iter must be positive");
  QCU_REQUIRE(req.src_mode == SRC_EO_FULL || req.src_mode == SRC_LEX, QCU_ERR_INVALID_ARGUMENT,
              "solver fields must be full eo or lexicographic");
  auto t0 = std::chrono::steady_clock::now();
  SlotEngine eng(s, nrhs, req, "sv");
  std::vector<int> slots(nrhs);
  std::vector<double> kap(nrhs, req.kappa), tol(nrhs, req.tol);
  for (int r = 0; r < nrhs; r++) slots[r] = r;
  eng.admit(slots, b, kap.data(), tol.data(), req.src_mode);
  int chunks = 0;
  while (eng.active_slots() > 0) {
    eng.step();
    chunks++;
  }
  eng.retire(slots, x, req.src_mode);
  SolveResult res;
  res.true_residual.resize(nrhs);
  res.converged.resize(nrhs);
  res.bad_source.resize(nrhs);
  for (int r = 0; r < nrhs; r++) {
    const SlotState& h = eng.slot(r);
    res.true_residual[r] = std::sqrt(h.true_res2 / h.bb);
    res.converged[r] = h.converged;
    res.bad_source[r] = h.bad_source;
    res.iterations = std::max(res.iterations, h.iterations);
    res.reliable_updates = std::max(res.reliable_updates, h.updates);
  }
  res.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  (void)chunks;
  return res;
}

}  // namespace qcu
