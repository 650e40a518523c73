/*
 * pn_oracle.c -- CPU restatement of the reference PN march, forward and adjoint, in FP64.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library: the tests, the smoke
 * check and the bench's CPU-baseline leg load it; the product never does.
 *
 * It restates, loop for loop and in the reference's memory layout (per class an array of
 * per-point moment vectors, moment index fastest, then x, y, z), the Julia code of:
 *   starmap/src/solver.jl:107-196        apply_boundary!, calc_du!, update!, step_pde!
 *   starmap/src/solver_core.jl:7-137     eo_range, expm1div, matmuldiff! (CSC), right_hand_side!, kernel!
 *   starmap/src/boundary_conditions.jl:67-102   apply_boundary_source!, apply_boundary_zero!
 *   pn_solver/pn_problem.jl:205-271      update_boundary_condition!, weighted_sum!, update_problem!
 *   pn_solver/pn_intensities.jl:129-164,189-212,325-413  integrate_adjoint_densities!,
 *                                        calc_x_ray_generation_field, calc_intensities (+ adjoint)
 *   pn_solver/x_ray_intensities.jl:155-234  compute_adjoint_source!, integrate_step_and_add(!,_pullback!)
 * with every class (active or not), every ghost point (corners included) and the reference's
 * evaluation order of each floating-point expression.  Compile with -ffp-contract=off: Julia
 * does not fuse multiply-adds.
 *
 * Parity status: the reference is Julia and no Julia toolchain exists here, so this restatement
 * could not be run against the reference itself ("parity unpinned").  Its building blocks are
 * pinned by known-answer tests instead (advection blocks against quadrature, boundary blocks
 * against the half-range integral they equal, class sizes, reflection symmetry, k = 1 for a
 * sample equal to its standard, finite-difference gradients), and by a second, independent numpy
 * restatement for small grids.
 */
#include "pn_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Host threads per solve.  The loops over the points of a class are split across threads when
   the file is built with OpenMP; each point's arithmetic, and every sum over points (intensities),
   keeps the serial evaluation order, so the results do not depend on the thread count.  The
   workers of ora_solve_many run one solve each and force one thread. */
static int g_threads = 1;
static __thread int tl_serial = 0;

int ora_openmp(void) {
#ifdef _OPENMP
  return 1;
#else
  return 0;
#endif
}

int ora_set_threads(int n) {
#ifdef _OPENMP
  if (n < 1) n = 1;
  g_threads = n;
#else
  (void)n;
  g_threads = 1;
#endif
  return g_threads;
}

/* ------------------------------------------------------------------------------------------ */
/* problem geometry and moments                                                               */
/* ------------------------------------------------------------------------------------------ */

static int floordiv2(int a) { return a >= 0 ? a / 2 : -((-a + 1) / 2); }

/* N_eee (pn_variable.jl:2) */
static int n_eee(int N) {
  int v = floordiv2(N + 2) * floordiv2(N + 4) / 2;
  return v > 0 ? v : 0;
}

static int bit(int c, int d) { return (c >> (2 - d)) & 1; }
static int sw(int c, int d) { return c ^ (4 >> d); }

/* moment parity per axis, 1 = odd (moment_specification.jl:26-36) */
static int moment_class(int l, int k) {
  int even_x = (k >= 0 && k % 2 == 0) || (k < 0 && k % 2 != 0);
  int even_y = k >= 0;
  int even_z = ((l + k) % 2 + 2) % 2 == 0;
  return 4 * (!even_x) + 2 * (!even_y) + (!even_z);
}

typedef struct {
  int ncol, nnz;
  int* colptr;    /* ncol + 1 */
  int* row;
  double* val;
} csc_t;

typedef struct {
  const pn_desc* d;
  int threads;            /* host threads for the loops over points */
  int N, ne, nr, ns;
  int nm[8];              /* moments per class */
  int deg[8][ORA_MAXM];   /* degree of each moment */
  int shape[8][3];
  int64_t npts[8];        /* points per class */
  int64_t off_state[8];   /* offset of class in state (doubles) */
  int64_t off_rho[8];     /* offset of class in rho (doubles) */
  int64_t n_state, n_rho;
  int singleton[3];
  double h[3];
  csc_t A[3][8];          /* advection, forward sign */
  const double* Bf[3][8]; /* boundary blocks (row-major n_c x n_sw) */
  const double* Ba[3][8];
  const double* gx[8];    /* beam face per odd-in-x class: [z][y][m] */
} ora_t;

static void csc_free(csc_t* a) { free(a->colptr); free(a->row); free(a->val); }

static int csc_from_dense(csc_t* a, const double* D, int nrow, int ncol, double sign) {
  a->ncol = ncol;
  a->colptr = (int*)calloc((size_t)ncol + 1, sizeof(int));
  int nnz = 0;
  for (int j = 0; j < ncol; ++j)
    for (int i = 0; i < nrow; ++i)
      if (D[(int64_t)i * ncol + j] != 0.0) ++nnz;
  a->nnz = nnz;
  a->row = (int*)malloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
  a->val = (double*)malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
  int k = 0;
  for (int j = 0; j < ncol; ++j) {
    a->colptr[j] = k;
    for (int i = 0; i < nrow; ++i) {
      double v = D[(int64_t)i * ncol + j];
      if (v != 0.0) { a->row[k] = i; a->val[k] = sign * v; ++k; }
    }
  }
  a->colptr[ncol] = k;
  return 0;
}

static int ora_init(ora_t* o, const pn_desc* d) {
  memset(o, 0, sizeof(*o));
  o->d = d;
  o->threads = tl_serial ? 1 : g_threads;
  o->N = d->order;
  o->ne = d->n_elements;
  o->nr = d->n_xrays;
  o->ns = d->n_steps;
  if (o->N < 0 || o->N > ORA_MAXN) return -1;
  int sizes[8] = {n_eee(o->N), n_eee(o->N - 1), n_eee(o->N - 1), n_eee(o->N - 2),
                  n_eee(o->N - 1), n_eee(o->N - 2), n_eee(o->N - 2), n_eee(o->N - 3)};
  int cnt[8] = {0};
  for (int l = 0; l <= o->N; ++l)
    for (int k = -l; k <= l; ++k) {
      int c = moment_class(l, k);
      o->deg[c][cnt[c]++] = l;
    }
  for (int c = 0; c < 8; ++c) {
    if (cnt[c] != sizes[c]) return -2;
    o->nm[c] = cnt[c];
  }
  for (int dd = 0; dd < 3; ++dd) {
    o->singleton[dd] = d->n_points[dd] == 1;
    o->h[dd] = d->h[dd];
  }
  int64_t so = 0, ro = 0;
  for (int c = 0; c < 8; ++c) {
    int64_t np = 1;
    for (int dd = 0; dd < 3; ++dd) {
      int M = d->n_points[dd];
      o->shape[c][dd] = o->singleton[dd] ? 1 : (bit(c, dd) ? M + 1 : M);
      np *= o->shape[c][dd];
    }
    o->npts[c] = np;
    o->off_state[c] = so;
    o->off_rho[c] = ro;
    so += np * o->nm[c];
    ro += np * o->ne;
  }
  o->n_state = so;
  o->n_rho = ro;
  const double* pa = d->advection;
  const double* pbf = d->boundary_fwd;
  const double* pba = d->boundary_adj;
  for (int dd = 0; dd < 3; ++dd)
    for (int c = 0; c < 8; ++c) {
      int nr_ = o->nm[c], nc_ = o->nm[sw(c, dd)];
      csc_from_dense(&o->A[dd][c], pa, nr_, nc_, 1.0);
      pa += (int64_t)nr_ * nc_;
      if (bit(c, dd)) {
        o->Bf[dd][c] = pbf;
        o->Ba[dd][c] = pba;
        pbf += (int64_t)nr_ * nc_;
        pba += (int64_t)nr_ * nc_;
      }
    }
  const double* pg = d->beam_face;
  for (int c = 4; c < 8; ++c) {
    o->gx[c] = pg;
    pg += (int64_t)o->shape[c][1] * o->shape[c][2] * o->nm[c];
  }
  return 0;
}

static void ora_free(ora_t* o) {
  for (int dd = 0; dd < 3; ++dd)
    for (int c = 0; c < 8; ++c) csc_free(&o->A[dd][c]);
}

int64_t ora_state_size(const pn_desc* d) {
  ora_t o;
  if (ora_init(&o, d)) return -1;
  int64_t n = o.n_state;
  ora_free(&o);
  return n;
}

int64_t ora_rho_size(const pn_desc* d) {
  ora_t o;
  if (ora_init(&o, d)) return -1;
  int64_t n = o.n_rho;
  ora_free(&o);
  return n;
}

/* index of point (i,j,k) (0-based) in class c */
static inline int64_t pidx(const ora_t* o, int c, int i, int j, int k) {
  return ((int64_t)k * o->shape[c][1] + j) * o->shape[c][0] + i;
}

/* ------------------------------------------------------------------------------------------ */
/* problem state: coefficients, S, C, Q, boundary source                                      */
/* ------------------------------------------------------------------------------------------ */
typedef struct {
  int adjoint;                 /* 0 forward problem, 1 adjoint problem */
  double s[ORA_MAXE];          /* s_e (same for all moments) */
  double c[ORA_MAXE][ORA_MAXN + 1];
  double bc;                   /* beam energy weight (forward) */
  double* S;                   /* per class per point per moment (state layout) */
  double* C;
  double* Q;                   /* adjoint source (state layout), NULL = zeros */
  int has_Q;
} prob_t;

static void update_problem(const ora_t* o, prob_t* p, const double* rho, const double* s,
                           const double* c, double bc) {
  for (int e = 0; e < o->ne; ++e) {
    p->s[e] = s[e];
    for (int l = 0; l <= o->N; ++l) p->c[e][l] = c[e * (o->N + 1) + l];
  }
  p->bc = bc;
  /* weighted_sum!: S[i] .= 0; for e: S[i] .+= rho[i][e] .* s[e] */
  for (int cl = 0; cl < 8; ++cl) {
    int nm = o->nm[cl];
#pragma omp parallel for schedule(static) num_threads(o->threads) if (o->threads > 1)
    for (int64_t q = 0; q < o->npts[cl]; ++q) {
      const double* r = rho + o->off_rho[cl] + q * o->ne;
      double* S = p->S + o->off_state[cl] + q * nm;
      double* C = p->C + o->off_state[cl] + q * nm;
      for (int m = 0; m < nm; ++m) { S[m] = 0.0; C[m] = 0.0; }
      for (int e = 0; e < o->ne; ++e)
        for (int m = 0; m < nm; ++m) S[m] = S[m] + r[e] * p->s[e];
      for (int e = 0; e < o->ne; ++e)
        for (int m = 0; m < nm; ++m) C[m] = C[m] + r[e] * p->c[e][o->deg[cl][m]];
    }
  }
}

/* ------------------------------------------------------------------------------------------ */
/* boundary conditions (boundary_conditions.jl:67-102, solver.jl:88-120)                      */
/* ------------------------------------------------------------------------------------------ */
static void matvec(const double* M, int nr_, int nc_, const double* v, double* out) {
  for (int r = 0; r < nr_; ++r) {
    double acc = 0.0;
    for (int q = 0; q < nc_; ++q) acc = acc + M[(int64_t)r * nc_ + q] * v[q];
    out[r] = acc;
  }
}

/* u odd in dim, v = switch(u, dim) even in dim */
static void apply_bc_class(const ora_t* o, const prob_t* p, double* st, int cl, int dim) {
  const int vc = sw(cl, dim);
  const int nu = o->nm[cl], nv = o->nm[vc];
  const double* B = p->adjoint ? o->Ba[dim][cl] : o->Bf[dim][cl];
  const int source = (!p->adjoint && dim == 0);
  double* U = st + o->off_state[cl];
  const double* V = st + o->off_state[vc];
  const int nx = o->shape[cl][0], ny = o->shape[cl][1], nz = o->shape[cl][2];
  const int sh[3] = {nx, ny, nz};
  /* the two axes across the face, in x, y, z order; a face point f is (f % sh[a], f / sh[a]) */
  const int a = dim == 0 ? 1 : 0, b = dim == 2 ? 1 : 2;
  const int64_t nf = (int64_t)sh[a] * sh[b];
  /* left face: index 0 along dim, every point across */
#pragma omp parallel for schedule(static) num_threads(o->threads) if (o->threads > 1)
  for (int64_t f = 0; f < nf; ++f) {
    double tmp[ORA_MAXM];
    int ii[3];
    ii[dim] = 0;
    ii[a] = (int)(f % sh[a]);
    ii[b] = (int)(f / sh[a]);
    int64_t q = pidx(o, cl, ii[0], ii[1], ii[2]);
    int64_t qv = pidx(o, vc, ii[0], ii[1], ii[2]);
    int rr[3] = {ii[0], ii[1], ii[2]};
    rr[dim] += 1;
    int64_t qr = pidx(o, cl, rr[0], rr[1], rr[2]);
    matvec(B, nu, nv, V + qv * nv, tmp);
    for (int m = 0; m < nu; ++m) {
      double g = 0.0; /* left source g[1,:,:] is zero (only gx_temp[2,...] is set) */
      if (source) U[q * nu + m] = 2.0 * (-tmp[m] + g) - U[qr * nu + m];
      else U[q * nu + m] = -2.0 * tmp[m] - U[qr * nu + m];
    }
  }
  /* right face: last index along dim */
#pragma omp parallel for schedule(static) num_threads(o->threads) if (o->threads > 1)
  for (int64_t f = 0; f < nf; ++f) {
    double tmp[ORA_MAXM];
    int ii[3];
    ii[dim] = sh[dim] - 1;
    ii[a] = (int)(f % sh[a]);
    ii[b] = (int)(f / sh[a]);
    const int i = ii[0], j = ii[1], k = ii[2];
    int64_t q = pidx(o, cl, i, j, k);
    int ll[3] = {i, j, k};
    ll[dim] -= 1;
    int64_t qv = pidx(o, vc, ll[0], ll[1], ll[2]);
    int64_t ql = pidx(o, cl, ll[0], ll[1], ll[2]);
    matvec(B, nu, nv, V + qv * nv, tmp);
    for (int m = 0; m < nu; ++m) {
      if (source) {
        /* g[2, j, k] = gx_temp[2, j, k] * bc ; dim == 0 so (j, k) index the face */
        double g = o->gx[cl][((int64_t)k * ny + j) * nu + m] * p->bc;
        U[q * nu + m] = 2.0 * (tmp[m] + g) - U[ql * nu + m];
      } else {
        U[q * nu + m] = 2.0 * tmp[m] - U[ql * nu + m];
      }
    }
  }
}

static void apply_boundary(const ora_t* o, const prob_t* p, double* st, int parity) {
  for (int dim = 0; dim < 3; ++dim) {
    if (o->singleton[dim]) continue;
    /* the two classes odd in dim with this parity, in class order */
    for (int cl = 0; cl < 8; ++cl) {
      if (!bit(cl, dim)) continue;
      int par = (bit(cl, 0) + bit(cl, 1) + bit(cl, 2)) & 1;
      if (par != parity) continue;
      apply_bc_class(o, p, st, cl, dim);
    }
  }
}

/* ------------------------------------------------------------------------------------------ */
/* stencil (solver_core.jl:38-137)                                                             */
/* ------------------------------------------------------------------------------------------ */
static double expm1div(double c) {
  if (fabs(c) <= 0.0002) return 1.0 + 0.5 * c + 1.0 / 6.0 * (c * c);
  return (exp(c) - 1.0) / c;
}

static void kernel_class(const ora_t* o, const prob_t* p, double* du, const double* st, int cl,
                         double dt, int use_expm1div) {
  const int nm = o->nm[cl];
  const int n[3] = {o->shape[cl][0], o->shape[cl][1], o->shape[cl][2]};
  int lo[3], hi[3];
  for (int dd = 0; dd < 3; ++dd) {
    if (bit(cl, dd)) { lo[dd] = 1; hi[dd] = n[dd] - 1; }  /* 2:n-1 */
    else { lo[dd] = 0; hi[dd] = n[dd]; }                   /* 1:n   */
  }
  const double adv_sign = p->adjoint ? -1.0 : 1.0;
#pragma omp parallel for collapse(2) schedule(static) num_threads(o->threads) if (o->threads > 1)
  for (int k = lo[2]; k < hi[2]; ++k)
    for (int j = lo[1]; j < hi[1]; ++j)
      for (int i = lo[0]; i < hi[0]; ++i) {
        int64_t q = pidx(o, cl, i, j, k);
        double* D = du + o->off_state[cl] + q * nm;
        for (int m = 0; m < nm; ++m) D[m] = 0.0;
        int ii[3] = {i, j, k};
        for (int dd = 0; dd < 3; ++dd) {
          if (n[dd] == 1) continue;
          int fc = sw(cl, dd);
          int nf = o->nm[fc];
          /* eo_index_right/left (solver_core.jl:21-35) in 0-based indices: an odd target io
             reads the even grid at io (right) and io - 1 (left); an even target ie reads the
             odd grid at ie + 1 (right) and ie (left) */
          int r[3] = {ii[0], ii[1], ii[2]}, l[3] = {ii[0], ii[1], ii[2]};
          if (bit(cl, dd)) { r[dd] = ii[dd]; l[dd] = ii[dd] - 1; }
          else { r[dd] = ii[dd] + 1; l[dd] = ii[dd]; }
          const double* UR = st + o->off_state[fc] + pidx(o, fc, r[0], r[1], r[2]) * nf;
          const double* UL = st + o->off_state[fc] + pidx(o, fc, l[0], l[1], l[2]) * nf;
          const csc_t* A = &o->A[dd][cl];
          const double hh = o->h[dd];
          for (int mc = 0; mc < A->ncol; ++mc) {
            double dv = (UR[mc] - UL[mc]) / hh;
            for (int t = A->colptr[mc]; t < A->colptr[mc + 1]; ++t)
              D[A->row[t]] = D[A->row[t]] + (adv_sign * A->val[t]) * dv;
          }
        }
        const double* U = st + o->off_state[cl] + q * nm;
        const double* S = p->S + o->off_state[cl] + q * nm;
        const double* C = p->C + o->off_state[cl] + q * nm;
        const double* Qv = p->has_Q ? p->Q + o->off_state[cl] + q * nm : NULL;
        for (int m = 0; m < nm; ++m) {
          double num = (Qv ? (Qv[m] - D[m]) : (-D[m])) - C[m] * U[m];
          if (use_expm1div) D[m] = num / S[m] * expm1div(-C[m] / S[m] * dt);
          else D[m] = num / S[m];
        }
      }
}

static void calc_du(const ora_t* o, const prob_t* p, double* du, const double* st, int parity,
                    double dt, int use_expm1div) {
  for (int cl = 0; cl < 8; ++cl) {
    int par = (bit(cl, 0) + bit(cl, 1) + bit(cl, 2)) & 1;
    if (par == parity) kernel_class(o, p, du, st, cl, dt, use_expm1div);
  }
}

static void update(const ora_t* o, double* st, const double* du, int parity, double dt) {
  for (int cl = 0; cl < 8; ++cl) {
    int par = (bit(cl, 0) + bit(cl, 1) + bit(cl, 2)) & 1;
    if (par != parity) continue;
    int64_t n = o->npts[cl] * o->nm[cl];
    double* U = st + o->off_state[cl];
    const double* D = du + o->off_state[cl];
#pragma omp parallel for schedule(static) num_threads(o->threads) if (o->threads > 1)
    for (int64_t q = 0; q < n; ++q) U[q] = U[q] + dt * D[q];
  }
}

static void step_pde(const ora_t* o, const prob_t* p, double* st, double* du, double dt) {
  double dt2 = dt / 2;
  apply_boundary(o, p, st, 0);
  calc_du(o, p, du, st, 1, dt2, 1);
  update(o, st, du, 1, dt2);
  apply_boundary(o, p, st, 1);
  calc_du(o, p, du, st, 0, dt, 1);
  update(o, st, du, 0, dt);
  apply_boundary(o, p, st, 0);
  calc_du(o, p, du, st, 1, dt2, 1);
  update(o, st, du, 1, dt2);
}

/* ------------------------------------------------------------------------------------------ */
/* intensities                                                                                 */
/* ------------------------------------------------------------------------------------------ */
static void integrate_step_and_add(const ora_t* o, double* I, const double* st, const double* noa,
                                   const double* acs, const double* sigma, double weight) {
  const int64_t ncell = o->npts[0];
  const int nm = o->nm[0];
  double integral[ORA_MAXR];
  for (int r = 0; r < o->nr; ++r) integral[r] = 0.0;
  for (int64_t i = 0; i < ncell; ++i)
    for (int r = 0; r < o->nr; ++r) {
      int el = o->d->xray_element[r];
      integral[r] = integral[r] + acs[i * o->nr + r] * noa[i * o->ne + el] * st[o->off_state[0] + i * nm];
    }
  const double dE = o->d->delta_e, dvol = o->d->dvol;
  for (int r = 0; r < o->nr; ++r) I[r] = I[r] + dE * dvol * sigma[r] * integral[r] * weight;
}

/* dst = src over n doubles, split across the solve's threads */
static void copy_state(const ora_t* o, double* dst, const double* src, int64_t n) {
  const int64_t chunk = 1 << 16;
  const int64_t nchunk = (n + chunk - 1) / chunk;
#pragma omp parallel for schedule(static) num_threads(o->threads) if (o->threads > 1)
  for (int64_t c = 0; c < nchunk; ++c) {
    int64_t a = c * chunk, len = n - a < chunk ? n - a : chunk;
    memcpy(dst + a, src + a, sizeof(double) * (size_t)len);
  }
}

static int alloc_prob(const ora_t* o, prob_t* p, int adjoint, int with_Q) {
  memset(p, 0, sizeof(*p));
  p->adjoint = adjoint;
  p->S = (double*)calloc((size_t)o->n_state, sizeof(double));
  p->C = (double*)calloc((size_t)o->n_state, sizeof(double));
  if (with_Q) { p->Q = (double*)calloc((size_t)o->n_state, sizeof(double)); p->has_Q = 1; }
  return (p->S && p->C && (!with_Q || p->Q)) ? 0 : -1;
}

static void free_prob(prob_t* p) { free(p->S); free(p->C); free(p->Q); }

int ora_forward(const pn_desc* d, const double* rho, const double* noa, const double* acs,
                double* intensities, double* tape) {
  ora_t o;
  if (ora_init(&o, d)) return -1;
  prob_t p;
  double* st = (double*)calloc((size_t)o.n_state, sizeof(double));
  double* du = (double*)calloc((size_t)o.n_state, sizeof(double));
  if (alloc_prob(&o, &p, 0, 0) || !st || !du) { free(st); free(du); free_prob(&p); ora_free(&o); return -3; }
  const int N1 = o.N + 1;
  for (int r = 0; r < o.nr; ++r) intensities[r] = 0.0;
  if (tape) copy_state(&o, tape, st, o.n_state);
  integrate_step_and_add(&o, intensities, st, noa, acs, d->fwd_sigma, d->fwd_weight[0]);
  for (int i = 0; i < o.ns; ++i) {
    update_problem(&o, &p, rho, d->fwd_s + (int64_t)i * o.ne, d->fwd_c + (int64_t)i * o.ne * N1, d->fwd_bc[i]);
    step_pde(&o, &p, st, du, d->delta_e);
    if (tape) copy_state(&o, tape + (int64_t)(i + 1) * o.n_state, st, o.n_state);
    integrate_step_and_add(&o, intensities, st, noa, acs, d->fwd_sigma + (int64_t)(i + 1) * o.nr,
                           d->fwd_weight[i + 1]);
  }
  free(st); free(du); free_prob(&p); ora_free(&o);
  return 0;
}

int ora_generation_field(const pn_desc* d, const double* rho, double* field) {
  ora_t o;
  if (ora_init(&o, d)) return -1;
  prob_t p;
  double* st = (double*)calloc((size_t)o.n_state, sizeof(double));
  double* du = (double*)calloc((size_t)o.n_state, sizeof(double));
  if (alloc_prob(&o, &p, 0, 0) || !st || !du) { free(st); free(du); free_prob(&p); ora_free(&o); return -3; }
  const int N1 = o.N + 1;
  const int64_t ncell = o.npts[0];
  const int nm = o.nm[0];
  for (int64_t q = 0; q < ncell * o.nr; ++q) field[q] = 0.0;
  for (int i = 0; i <= o.ns; ++i) {
    if (i > 0) {
      update_problem(&o, &p, rho, d->fwd_s + (int64_t)(i - 1) * o.ne, d->fwd_c + (int64_t)(i - 1) * o.ne * N1,
                     d->fwd_bc[i - 1]);
      step_pde(&o, &p, st, du, d->delta_e);
    }
    const double* sg = d->fwd_sigma + (int64_t)i * o.nr;
#pragma omp parallel for schedule(static) num_threads(o.threads) if (o.threads > 1)
    for (int64_t c = 0; c < ncell; ++c)
      for (int r = 0; r < o.nr; ++r)
        field[c * o.nr + r] = field[c * o.nr + r] + st[o.off_state[0] + c * nm] * d->delta_e * sg[r] * d->fwd_weight[i];
  }
  free(st); free(du); free_prob(&p); ora_free(&o);
  return 0;
}

int ora_step(const pn_desc* d, const double* rho, double* state, int step) {
  ora_t o;
  if (ora_init(&o, d)) return -1;
  if (step < 0 || step >= o.ns) { ora_free(&o); return -2; }
  prob_t p;
  double* du = (double*)calloc((size_t)o.n_state, sizeof(double));
  if (alloc_prob(&o, &p, 0, 0) || !du) { free(du); free_prob(&p); ora_free(&o); return -3; }
  const int N1 = o.N + 1;
  update_problem(&o, &p, rho, d->fwd_s + (int64_t)step * o.ne, d->fwd_c + (int64_t)step * o.ne * N1, d->fwd_bc[step]);
  step_pde(&o, &p, state, du, d->delta_e);
  free(du); free_prob(&p); ora_free(&o);
  return 0;
}

/* integrate_adjoint_densities! (pn_intensities.jl:129-164) */
static void integrate_adjoint_densities(const ora_t* o, prob_t* pf, const double* rho, double* u,
                                        double* du, const double* lam, const double* s,
                                        const double* c, double bc, double* rho_bar, double weight) {
  update_problem(o, pf, rho, s, c, bc);
  apply_boundary(o, pf, u, 0);
  apply_boundary(o, pf, u, 1);
  calc_du(o, pf, du, u, 0, o->d->delta_e, 0);
  calc_du(o, pf, du, u, 1, o->d->delta_e, 0);
  const double dvol = o->d->dvol, dE = o->d->delta_e;
  for (int cl = 0; cl < 8; ++cl) {
    const int nm = o->nm[cl];
    const int n[3] = {o->shape[cl][0], o->shape[cl][1], o->shape[cl][2]};
    int lo[3], hi[3];
    for (int dd = 0; dd < 3; ++dd) {
      if (bit(cl, dd)) { lo[dd] = 1; hi[dd] = n[dd] - 1; }
      else { lo[dd] = 0; hi[dd] = n[dd]; }
    }
#pragma omp parallel for collapse(3) schedule(static) num_threads(o->threads) if (o->threads > 1)
    for (int i = lo[0]; i < hi[0]; ++i)
      for (int j = lo[1]; j < hi[1]; ++j)
        for (int k = lo[2]; k < hi[2]; ++k) {
          int64_t q = pidx(o, cl, i, j, k);
          const double* L = lam + o->off_state[cl] + q * nm;
          const double* D = du + o->off_state[cl] + q * nm;
          const double* U = u + o->off_state[cl] + q * nm;
          double* RB = rho_bar + o->off_rho[cl] + q * o->ne;
          for (int e = 0; e < o->ne; ++e)
            for (int m = 0; m < nm; ++m)
              RB[e] = RB[e] + L[m] * (pf->s[e] * D[m] + pf->c[e][o->deg[cl][m]] * U[m]) * dvol * dE * weight;
        }
  }
}

static void integrate_step_and_add_pullback(const ora_t* o, const double* u, const double* noa,
                                            const double* acs, const double* sigma, double weight,
                                            const double* Ibar, double* noa_bar, double* acs_bar) {
  const double dE = o->d->delta_e, dvol = o->d->dvol;
  double integral_[ORA_MAXR];
  for (int r = 0; r < o->nr; ++r) integral_[r] = 0.0 + dE * dvol * sigma[r] * weight * Ibar[r];
  const int64_t ncell = o->npts[0];
  const int nm = o->nm[0];
#pragma omp parallel for schedule(static) num_threads(o->threads) if (o->threads > 1)
  for (int64_t i = 0; i < ncell; ++i)
    for (int r = 0; r < o->nr; ++r) {
      int el = o->d->xray_element[r];
      double u0 = u[o->off_state[0] + i * nm];
      acs_bar[i * o->nr + r] = acs_bar[i * o->nr + r] + noa[i * o->ne + el] * u0 * integral_[r];
      noa_bar[i * o->ne + el] = noa_bar[i * o->ne + el] + acs[i * o->nr + r] * u0 * integral_[r];
    }
}

static void compute_adjoint_source(const ora_t* o, double* Q, const double* Ibar, const double* noa,
                                   const double* acs, const double* sigma) {
  const int64_t ncell = o->npts[0];
  const int nm = o->nm[0];
#pragma omp parallel for schedule(static) num_threads(o->threads) if (o->threads > 1)
  for (int64_t i = 0; i < ncell; ++i) {
    double* Qi = Q + o->off_state[0] + i * nm;
    Qi[0] = 0.0;
    for (int r = 0; r < o->nr; ++r) {
      int el = o->d->xray_element[r];
      Qi[0] = Qi[0] - sigma[r] * acs[i * o->nr + r] * noa[i * o->ne + el] * Ibar[r];
    }
  }
}

int ora_adjoint(const pn_desc* d, const double* rho, const double* noa, const double* acs,
                const double* Ibar, double* intensities, double* rho_bar, double* noa_bar,
                double* acs_bar) {
  ora_t o;
  if (ora_init(&o, d)) return -1;
  const int64_t ns1 = (int64_t)o.ns + 1;
  double* tape = (double*)malloc(sizeof(double) * (size_t)(ns1 * o.n_state));
  if (!tape) { ora_free(&o); return -3; }
  double Itmp[ORA_MAXR];
  int rc = ora_forward(d, rho, noa, acs, intensities ? intensities : Itmp, tape);
  if (rc) { free(tape); ora_free(&o); return rc; }
  prob_t pf, pa;
  double* lam = (double*)calloc((size_t)o.n_state, sizeof(double));
  double* dlam = (double*)calloc((size_t)o.n_state, sizeof(double));
  double* du = (double*)calloc((size_t)o.n_state, sizeof(double));
  if (alloc_prob(&o, &pf, 0, 0) || alloc_prob(&o, &pa, 1, 1) || !lam || !dlam || !du) {
    free(tape); free(lam); free(dlam); free(du); free_prob(&pf); free_prob(&pa); ora_free(&o);
    return -3;
  }
  memset(rho_bar, 0, sizeof(double) * (size_t)o.n_rho);
  memset(noa_bar, 0, sizeof(double) * (size_t)(o.npts[0] * o.ne));
  memset(acs_bar, 0, sizeof(double) * (size_t)(o.npts[0] * o.nr));
  const int N1 = o.N + 1;
  for (int j = 0; j < o.ns; ++j) {
    int i = o.ns - j; /* tape state after forward step i */
    double* u = tape + (int64_t)i * o.n_state;
    integrate_adjoint_densities(&o, &pf, rho, u, du, lam, d->adj_int_s + (int64_t)j * o.ne,
                                d->adj_int_c + (int64_t)j * o.ne * N1, d->adj_int_bc[j], rho_bar,
                                d->adj_weight[j]);
    integrate_step_and_add_pullback(&o, u, noa, acs, d->adj_sigma + (int64_t)j * o.nr, d->adj_weight[j],
                                    Ibar, noa_bar, acs_bar);
    compute_adjoint_source(&o, pa.Q, Ibar, noa, acs, d->adj_src_sigma + (int64_t)j * o.nr);
    update_problem(&o, &pa, rho, d->adj_s + (int64_t)j * o.ne, d->adj_c + (int64_t)j * o.ne * N1, 0.0);
    step_pde(&o, &pa, lam, dlam, d->delta_e);
  }
  {
    int j = o.ns;
    double* u = tape;
    integrate_adjoint_densities(&o, &pf, rho, u, du, lam, d->adj_int_s + (int64_t)j * o.ne,
                                d->adj_int_c + (int64_t)j * o.ne * N1, d->adj_int_bc[j], rho_bar,
                                d->adj_weight[j]);
    integrate_step_and_add_pullback(&o, u, noa, acs, d->adj_sigma + (int64_t)j * o.nr, d->adj_weight[j],
                                    Ibar, noa_bar, acs_bar);
  }
  free(tape); free(lam); free(dlam); free(du); free_prob(&pf); free_prob(&pa); ora_free(&o);
  return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* many independent solves on host threads (the CPU baseline of the benchmark)                */
/* ------------------------------------------------------------------------------------------ */
#include <pthread.h>

typedef struct {
  const pn_desc* const* d;
  const double* const* rho;
  const double* const* noa;
  const double* const* acs;
  const double* const* Ibar;
  double* const* I;
  double* const* rho_bar;
  double* const* noa_bar;
  double* const* acs_bar;
  int n;
  int next;
  int rc;
  pthread_mutex_t mu;
} many_t;

static void* many_worker(void* arg) {
  many_t* w = (many_t*)arg;
  tl_serial = 1;
  for (;;) {
    pthread_mutex_lock(&w->mu);
    int i = w->next++;
    pthread_mutex_unlock(&w->mu);
    if (i >= w->n) break;
    int rc = ora_adjoint(w->d[i], w->rho[i], w->noa[i], w->acs[i], w->Ibar[i], w->I[i],
                         w->rho_bar[i], w->noa_bar[i], w->acs_bar[i]);
    if (rc) {
      pthread_mutex_lock(&w->mu);
      w->rc = rc;
      pthread_mutex_unlock(&w->mu);
    }
  }
  return NULL;
}

int ora_solve_many(const pn_desc* const* d, const double* const* rho, const double* const* noa,
                   const double* const* acs, const double* const* Ibar, double* const* intensities,
                   double* const* rho_bar, double* const* noa_bar, double* const* acs_bar, int n,
                   int threads) {
  many_t w = {d, rho, noa, acs, Ibar, intensities, rho_bar, noa_bar, acs_bar, n, 0, 0};
  pthread_mutex_init(&w.mu, NULL);
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  pthread_t th[256];
  int started = 0;
  for (int t = 0; t < threads; ++t)
    if (pthread_create(&th[t], NULL, many_worker, &w) == 0) ++started;
  if (started == 0) many_worker(&w);
  for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
  pthread_mutex_destroy(&w.mu);
  return w.rc;
}
