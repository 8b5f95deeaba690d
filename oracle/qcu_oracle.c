/*
 * FP64 CPU oracle for the multi-right-hand-side even-odd Wilson dslash,
 * its layout conversions, the clover term and the (Wilson-clover) solve
 * built on them.
 *
 * TEST INFRASTRUCTURE ONLY.  The parity tests, the smoke check and the
 * CPU-baseline leg of the benchmark load it to check results.  The product
 * library never links or calls it and has no CPU fallback.
 *
 * Parity pinning: the dslash here is checked against the reference's own GPU
 * kernel (include/kernels/wilson_dslash_4d.cuh, rebuilt for sm_103a by
 * oracle/build_ref.sh and run by tests/golden/make_golden.py); the committed
 * fixtures under tests/golden/ hold the reference kernel's outputs.
 *
 * Conventions restated from the reference (paths relative to the reference
 * project):
 *  - half-lattice index  i = ((t*Lz + z)*Ly + y)*(Lx/2) + xh, parity
 *    p = (X+y+z+t) mod 2, X = 2*xh + (p ^ ((y+z+t)&1))
 *    (include/basic_data/qcu_point.cuh:41-49, wilson_dslash_4d.cuh:35-43);
 *  - periodic neighbours in all four directions (qcu_point.cuh:33-78);
 *  - caller ("non-coalesced") layouts: gauge [mu=4][parity=2][Vh][N][N]
 *    row-major U_ab, fermion [Vh][Ns=4][N] spin-major per RHS
 *    (include/kernels/storage/storage_kernels.cuh:14-101);
 *  - hop term, DeGrand-Rossi gammas, flag f = +1 (no dagger) / -1 (dagger):
 *      out(x) = sum_mu (1 - f g_mu) U_mu(x) psi(x+mu)
 *                    + (1 + f g_mu) U_mu(x-mu)^dag psi(x-mu)
 *    (include/kernels/wilson_dslash_4d.cuh:59-293, flag at
 *    src/qcd/qcu_wilson.cu:41); the output is overwritten
 *    (wilson_dslash_4d.cuh:55-57,296-300).
 * Antiperiodic time boundaries (absent from the reference) multiply every hop
 * that crosses the t = Lt-1 <-> 0 boundary by -1, which equals negating
 * U_t on the t = Lt-1 slice before calling the reference.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NS 4

/* gamma_mu row r has a single non-zero entry g[mu][r] in column perm[mu][r]
 * (wilson_dslash_4d.cuh:74-81 for x, :134-141 y, :193-200 z, :253-260 t).
 * Entries are stored as (re, im). */
static const int g_perm[4][4] = {{3, 2, 1, 0}, {3, 2, 1, 0}, {2, 3, 0, 1}, {2, 3, 0, 1}};
static const double g_val[4][4][2] = {
    {{0, 1}, {0, 1}, {0, -1}, {0, -1}},  /* gamma_x: i, i, -i, -i */
    {{-1, 0}, {1, 0}, {1, 0}, {-1, 0}},  /* gamma_y: -1, 1, 1, -1 */
    {{0, 1}, {0, -1}, {0, -1}, {0, 1}},  /* gamma_z: i, -i, -i, i */
    {{1, 0}, {1, 0}, {1, 0}, {1, 0}},    /* gamma_t: 1, 1, 1, 1 */
};

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* Full coordinate of half-lattice site i at parity p (qcu_point.cuh:41-49). */
static void eo_coords(int64_t i, int p, const int L[4], int c[4]) {
  int hx = L[0] / 2;
  int64_t r = i;
  int xh = (int)(r % hx);
  r /= hx;
  int y = (int)(r % L[1]);
  r /= L[1];
  int z = (int)(r % L[2]);
  int t = (int)(r / L[2]);
  int eo = (y + z + t) & 1;
  c[0] = 2 * xh + (p ^ eo);
  c[1] = y;
  c[2] = z;
  c[3] = t;
}

static int64_t eo_index(const int c[4], const int L[4]) {
  return (((int64_t)c[3] * L[2] + c[2]) * L[1] + c[1]) * (L[0] / 2) + c[0] / 2;
}

/* out[nrhs][Vh][4][N], in[nrhs][Vh][4][N], gauge[4][2][Vh][N][N]; all complex
 * double, interleaved (re, im).  Output parity = `parity`, input parity is the
 * opposite one.  dagger: 0 -> f=+1, 1 -> f=-1. */
void oracle_dslash(double *out, const double *in, const double *gauge, const int L[4], int N, int nrhs, int parity,
                   int dagger, int antiperiodic_t) {
  const int64_t Vh = (int64_t)L[0] * L[1] * L[2] * L[3] / 2;
  const int64_t sp = (int64_t)NS * N * 2;      /* doubles per site spinor */
  const int64_t lk = (int64_t)N * N * 2;       /* doubles per link */
  const double f = dagger ? -1.0 : 1.0;

#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < Vh; i++) {
    int c[4];
    eo_coords(i, parity, L, c);
    double acc[NS * 16 * 2]; /* N <= 16 */
    double h[2][16][2], t[2][16][2];
    for (int r = 0; r < nrhs; r++) {
      memset(acc, 0, sizeof(double) * NS * N * 2);
      for (int mu = 0; mu < 4; mu++) {
        for (int dir = 0; dir < 2; dir++) { /* dir 0 = forward, 1 = backward */
          int nc[4] = {c[0], c[1], c[2], c[3]};
          double bc = 1.0;
          if (dir == 0) {
            nc[mu] = c[mu] + 1;
            if (nc[mu] == L[mu]) {
              nc[mu] = 0;
              if (mu == 3 && antiperiodic_t) bc = -1.0;
            }
          } else {
            nc[mu] = c[mu] - 1;
            if (nc[mu] < 0) {
              nc[mu] = L[mu] - 1;
              if (mu == 3 && antiperiodic_t) bc = -1.0;
            }
          }
          int64_t j = eo_index(nc, L);
          /* s = -f for forward (1 - f g), +f for backward (1 + f g). */
          double s = dir == 0 ? -f : f;
          const double *psi = in + ((int64_t)r * Vh + j) * sp;
          /* forward: U_mu(x) at parity p, site i; backward: U_mu(x-mu) at
           * parity 1-p, site j, used as its conjugate transpose
           * (wilson_dslash_4d.cuh:61, :88-89). */
          const double *U = dir == 0 ? gauge + (((int64_t)mu * 2 + parity) * Vh + i) * lk
                                     : gauge + (((int64_t)mu * 2 + (1 - parity)) * Vh + j) * lk;
          /* spin projection onto the two upper rows: h_u = psi_u + s g(u) psi_perm(u) */
          for (int u = 0; u < 2; u++) {
            int pu = g_perm[mu][u];
            double gr = s * g_val[mu][u][0], gi = s * g_val[mu][u][1];
            for (int a = 0; a < N; a++) {
              double xr = psi[(pu * N + a) * 2], xi = psi[(pu * N + a) * 2 + 1];
              h[u][a][0] = psi[(u * N + a) * 2] + (gr * xr - gi * xi);
              h[u][a][1] = psi[(u * N + a) * 2 + 1] + (gr * xi + gi * xr);
            }
          }
          /* colour multiply: t = U h (forward) or U^dag h (backward) */
          for (int u = 0; u < 2; u++) {
            for (int a = 0; a < N; a++) {
              double sr = 0, si = 0;
              for (int b = 0; b < N; b++) {
                double ur, ui;
                if (dir == 0) {
                  ur = U[(a * N + b) * 2];
                  ui = U[(a * N + b) * 2 + 1];
                } else {
                  ur = U[(b * N + a) * 2];
                  ui = -U[(b * N + a) * 2 + 1];
                }
                sr += ur * h[u][b][0] - ui * h[u][b][1];
                si += ur * h[u][b][1] + ui * h[u][b][0];
              }
              t[u][a][0] = bc * sr;
              t[u][a][1] = bc * si;
            }
          }
          /* reconstruction: row u += t_u; row perm(u) += s g(perm(u)) t_u */
          for (int u = 0; u < 2; u++) {
            int lo = g_perm[mu][u];
            double gr = s * g_val[mu][lo][0], gi = s * g_val[mu][lo][1];
            for (int a = 0; a < N; a++) {
              double tr = t[u][a][0], ti = t[u][a][1];
              acc[(u * N + a) * 2] += tr;
              acc[(u * N + a) * 2 + 1] += ti;
              acc[(lo * N + a) * 2] += gr * tr - gi * ti;
              acc[(lo * N + a) * 2 + 1] += gr * ti + gi * tr;
            }
          }
        }
      }
      memcpy(out + ((int64_t)r * Vh + i) * sp, acc, sizeof(double) * sp);
    }
  }
}

/* Lexicographic full-lattice field [V][ncomp] (site index ((t*Lz+z)*Ly+y)*Lx+X)
 * to the even-odd split [2][Vh][ncomp] (even half first).  The reference
 * callers hand over parity-split data directly (src/qcu.cu:88-101); this
 * conversion is the lexicographic entry the solve path accepts. */
void oracle_lex_to_eo(double *eo, const double *lex, const int L[4], int ncomp) {
  const int64_t V = (int64_t)L[0] * L[1] * L[2] * L[3];
  const int64_t Vh = V / 2;
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < V; s++) {
    int64_t r = s;
    int c[4];
    c[0] = (int)(r % L[0]);
    r /= L[0];
    c[1] = (int)(r % L[1]);
    r /= L[1];
    c[2] = (int)(r % L[2]);
    c[3] = (int)(r / L[2]);
    int p = (c[0] + c[1] + c[2] + c[3]) & 1;
    int64_t i = eo_index(c, L);
    memcpy(eo + ((int64_t)p * Vh + i) * ncomp * 2, lex + s * ncomp * 2, sizeof(double) * ncomp * 2);
  }
}

void oracle_eo_to_lex(double *lex, const double *eo, const int L[4], int ncomp) {
  const int64_t V = (int64_t)L[0] * L[1] * L[2] * L[3];
  const int64_t Vh = V / 2;
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < V; s++) {
    int64_t r = s;
    int c[4];
    c[0] = (int)(r % L[0]);
    r /= L[0];
    c[1] = (int)(r % L[1]);
    r /= L[1];
    c[2] = (int)(r % L[2]);
    c[3] = (int)(r / L[2]);
    int p = (c[0] + c[1] + c[2] + c[3]) & 1;
    int64_t i = eo_index(c, L);
    memcpy(lex + s * ncomp * 2, eo + ((int64_t)p * Vh + i) * ncomp * 2, sizeof(double) * ncomp * 2);
  }
}

/* Full Wilson operator on an even-odd split field, one RHS:
 *   out = in - kappa * D in,   in/out [2][Vh][4][N]
 * (kappa = 1/(2(4+m)) as at include/qcu_dirac.h:26; the reference never
 * applies it -- the solve path is new work, src/qcu.cu:173). */
/* Clover term of one parity (the reference only fixes its storage,
 * include/basic_data/qcu_point.cuh:98-101: (Nc*Ns)^2/2 complex per site): per
 * site two (2N x 2N) complex blocks, block 0 acting on spins 0, 1 and block 1
 * on spins 2, 3 (the chirality blocks of the DeGrand-Rossi basis), row and
 * column index = local spin * N + colour.  clover: [2][Vh][2][2N][2N] complex
 * for both parities.  out = A_p in (dagger: A_p^dag in) for nrhs fields
 * [nrhs][Vh][4][N]. */
void oracle_clover_apply(double *out, const double *in, const double *clover, const int L[4], int N, int nrhs,
                         int parity, int dagger) {
  const int64_t Vh = (int64_t)L[0] * L[1] * L[2] * L[3] / 2;
  const int n2 = 2 * N, blk = n2 * n2;
#pragma omp parallel for collapse(2) schedule(static)
  for (int r = 0; r < nrhs; r++)
    for (int64_t i = 0; i < Vh; i++) {
      const double *a = clover + (((int64_t)parity * Vh + i) * 2 * blk) * 2;
      const double *v = in + (((int64_t)r * Vh + i) * NS * N) * 2;
      double *o = out + (((int64_t)r * Vh + i) * NS * N) * 2;
      for (int b = 0; b < 2; b++)
        for (int row = 0; row < n2; row++) {
          double re = 0, im = 0;
          for (int col = 0; col < n2; col++) {
            const int64_t e = dagger ? (int64_t)b * blk + col * n2 + row : (int64_t)b * blk + row * n2 + col;
            const double mr = a[2 * e], mi = dagger ? -a[2 * e + 1] : a[2 * e + 1];
            const double *x = v + ((int64_t)(2 * b) * N + col) * 2;
            re += mr * x[0] - mi * x[1];
            im += mr * x[1] + mi * x[0];
          }
          o[((int64_t)(2 * b) * N + row) * 2] = re;
          o[((int64_t)(2 * b) * N + row) * 2 + 1] = im;
        }
    }
}

/* Full-lattice operator M = A - kappa D (A = 1 without a clover field, the
 * Wilson operator), fields [2][Vh][4][N]; dagger: M^dag = A^dag - kappa D^dag.
 * scratch: [2][Vh][4][N] complex. */
void oracle_wilson_full(double *out, const double *in, const double *gauge, const double *clover, const int L[4],
                        int N, double kappa, int dagger, int antiperiodic_t, double *scratch) {
  const int64_t Vh = (int64_t)L[0] * L[1] * L[2] * L[3] / 2;
  const int64_t n = Vh * NS * N * 2;
  for (int p = 0; p < 2; p++) {
    oracle_dslash(scratch, in + (int64_t)(1 - p) * n, gauge, L, N, 1, p, dagger, antiperiodic_t);
    double *o = out + (int64_t)p * n;
    const double *x = in + (int64_t)p * n;
    if (clover) {
      oracle_clover_apply(scratch + n, x, clover, L, N, 1, p, dagger);
      x = scratch + n;
    }
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; k++) o[k] = x[k] - kappa * scratch[k];
  }
}

static double dot_re(const double *a, const double *b, int64_t n) {
  double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int64_t k = 0; k < n; k++) s += a[k] * b[k];
  return s;
}

/* CGNR on the full (unpreconditioned) Wilson system M x = b, one RHS, FP64:
 * an independent check of the even-odd preconditioned GPU solve.  Returns the
 * iteration count; *relres receives the true residual |b - M x| / |b|. */
int oracle_cgnr_full(double *x, const double *b, const double *gauge, const double *clover, const int L[4], int N,
                     double kappa, int antiperiodic_t, double tol, int maxiter, double *relres) {
  const int64_t Vh = (int64_t)L[0] * L[1] * L[2] * L[3] / 2;
  const int64_t n = 2 * Vh * NS * N * 2;
  double *r = malloc(sizeof(double) * n), *p = malloc(sizeof(double) * n), *Ap = malloc(sizeof(double) * n);
  double *t = malloc(sizeof(double) * n), *sc = malloc(sizeof(double) * n);
  /* x = 0; r = M^dag b; p = r */
  memset(x, 0, sizeof(double) * n);
  oracle_wilson_full(r, b, gauge, clover, L, N, kappa, 1, antiperiodic_t, sc);
  memcpy(p, r, sizeof(double) * n);
  double bb = dot_re(b, b, n);
  double rr = dot_re(r, r, n);
  int it = 0;
  for (; it < maxiter; it++) {
    oracle_wilson_full(t, p, gauge, clover, L, N, kappa, 0, antiperiodic_t, sc);
    double pAp = dot_re(t, t, n);
    oracle_wilson_full(Ap, t, gauge, clover, L, N, kappa, 1, antiperiodic_t, sc);
    double alpha = rr / pAp;
    for (int64_t k = 0; k < n; k++) {
      x[k] += alpha * p[k];
      r[k] -= alpha * Ap[k];
    }
    double rr_new = dot_re(r, r, n);
    /* stop on the true residual of M x = b */
    oracle_wilson_full(t, x, gauge, clover, L, N, kappa, 0, antiperiodic_t, sc);
    double res = 0;
    for (int64_t k = 0; k < n; k++) res += (b[k] - t[k]) * (b[k] - t[k]);
    if (sqrt(res / bb) < tol) {
      it++;
      break;
    }
    double beta = rr_new / rr;
    rr = rr_new;
    for (int64_t k = 0; k < n; k++) p[k] = r[k] + beta * p[k];
  }
  oracle_wilson_full(t, x, gauge, clover, L, N, kappa, 0, antiperiodic_t, sc);
  double res = 0;
  for (int64_t k = 0; k < n; k++) res += (b[k] - t[k]) * (b[k] - t[k]);
  *relres = sqrt(res / bb);
  free(r);
  free(p);
  free(Ap);
  free(t);
  free(sc);
  return it;
}

/* True residual |b - M x| / |b| of a full-lattice eo-split solution, one RHS. */
double oracle_true_residual(const double *x, const double *b, const double *gauge, const double *clover,
                            const int L[4], int N, double kappa, int antiperiodic_t) {
  const int64_t Vh = (int64_t)L[0] * L[1] * L[2] * L[3] / 2;
  const int64_t n = 2 * Vh * NS * N * 2;
  double *t = malloc(sizeof(double) * n), *sc = malloc(sizeof(double) * n);
  oracle_wilson_full(t, x, gauge, clover, L, N, kappa, 0, antiperiodic_t, sc);
  double res = 0, bb = 0;
  for (int64_t k = 0; k < n; k++) {
    res += (b[k] - t[k]) * (b[k] - t[k]);
    bb += b[k] * b[k];
  }
  free(t);
  free(sc);
  return sqrt(res / bb);
}
