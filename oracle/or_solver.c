/*
 * or_solver.c -- oracle Poisson/Helmholtz solve.  TEST INFRASTRUCTURE ONLY.
 *
 * The linear systems are assembled exactly as the reference assembles them
 * for HYPRE: solver.f90:158-372 (init_matrix_3d) and solver.f90:687-842 +
 * 981-1020 (init_matrix_2d / init_n_2d_matrices: 5-point operator per
 * wavenumber, diagonal shifted by lambda(k)*dl1_2*dl2_2).  The blocks are
 * laid out in the global index space of initmpi.f90:50-103 (HYPRE's Struct
 * grid): one bounding box with inactive cells where no block lies, periodic
 * wrap where solver.f90:224 sets the grid periodic.
 *
 * HYPRE's PFMG iterates are not reproduced: the system is solved by
 * conjugate gradients preconditioned with a geometric multigrid V(1,1)
 * cycle (nu=2 red-black Gauss-Seidel sweeps before and after, summed restriction, injected prolongation,
 * rediscretised coarse operators, dense coarsest solve), to a relative
 * residual ||r||/||b|| <= tol (HYPRE's stopping quantity).  Singular
 * (all-Neumann/periodic, zero shift) systems get their right-hand side
 * projected onto the range (mean removed) before the solve.
 */
#include "or_internal.h"
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define LOCAL(b, ax, q) ((q) - (b)->lo[ax] + 1) /* index into (n+2) metric arrays */

static int wrapi(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

/* neighbour of cell (i,j,k) along axis a, direction s (0:-1, 1:+1); -1 if outside a non-periodic box */
static long nbr(const or_poisson *P, const or_level *L, int i, int j, int k, int a, int s) {
  int c[3] = {i, j, k};
  c[a] += s ? 1 : -1;
  if (c[a] < 0 || c[a] >= L->n[a]) {
    if (!P->periodic[a]) return -1;
    c[a] = wrapi(c[a], L->n[a]);
  }
  return c[0] + (long)L->n[0] * (c[1] + (long)L->n[1] * c[2]);
}

static int naxes(const or_poisson *P) { return P->mode3d ? 3 : 2; }

/* fold type code for a physical boundary: 1 N (sgn +1), 2 centred D (sgn -1), 3 staggered D (sgn 0) */
static int fold_type(char cbc, int centered) {
  if (cbc == 'N') return 1;
  if (cbc == 'D') return centered ? 2 : 3;
  return 0;
}
static double fold_sgn(int t) { return t == 1 ? 1.0 : (t == 2 ? -1.0 : 0.0); }

static void free_level(or_level *L) {
  for (int a = 0; a < 3; a++) { free(L->W[a]); free(L->cp[a]); }
  free(L->code); free(L->cc); free(L->x); free(L->b); free(L->r); free(L->dinv);
  memset(L, 0, sizeof(*L));
}

void or_poisson_destroy(or_poisson *P) {
  if (!P) return;
  for (int l = 0; l < P->nlev; l++) free_level(&P->L[l]);
  free(P->shift); free(P->singular); free(P->p); free(P->q); free(P->z); free(P->lam);
  free(P);
}

static void alloc_level(or_poisson *P, or_level *L) {
  L->ncell = (long)L->n[0] * L->n[1] * L->n[2];
  for (int a = 0; a < 3; a++) {
    L->W[a] = calloc(L->n[a], sizeof(double));
    L->cp[a] = calloc(L->ncell, sizeof(double));
  }
  L->code = calloc(L->ncell, sizeof(unsigned short));
  L->cc = calloc(L->ncell, sizeof(double));
  L->x = calloc(L->ncell * P->nsys, sizeof(double));
  L->b = calloc(L->ncell * P->nsys, sizeof(double));
  L->r = calloc(L->ncell * P->nsys, sizeof(double));
}

/* rediscretised operator on a coarse level from its widths and codes */
static void build_coarse_operator(or_poisson *P, or_level *L, double alpha) {
  int na = naxes(P);
  for (int k = 0; k < L->n[2]; k++)
    for (int j = 0; j < L->n[1]; j++)
      for (int i = 0; i < L->n[0]; i++) {
        long c = i + (long)L->n[0] * (j + (long)L->n[1] * k);
        int idx[3] = {i, j, k};
        for (int a = 0; a < 3; a++) L->cp[a][c] = 0.0;
        L->cc[c] = 0.0;
        if (L->code[c] & 0x8000) continue;
        double weight = 1.0;
        for (int a = 0; a < na; a++) weight *= L->W[a][idx[a]];
        double cm[3] = {0, 0, 0}, cpv[3] = {0, 0, 0}, sum = 0.0;
        for (int a = 0; a < na; a++) {
          if (P->periodic[a] && L->n[a] == 1) continue; /* self-coupled periodic ring: no contribution */
          double wt = 1.0;
          for (int b2 = 0; b2 < na; b2++) if (b2 != a) wt *= L->W[b2][idx[b2]];
          int n = L->n[a], q = idx[a];
          double Wq = L->W[a][q];
          double Wm = (q > 0) ? L->W[a][q - 1] : (P->periodic[a] ? L->W[a][n - 1] : Wq);
          double Wp = (q < n - 1) ? L->W[a][q + 1] : (P->periodic[a] ? L->W[a][0] : Wq);
          int tm = (L->code[c] >> (2 * (2 * a + 0))) & 3, tp = (L->code[c] >> (2 * (2 * a + 1))) & 3;
          double dm = tm ? Wq : 0.5 * (Wm + Wq);
          double dp = tp ? Wq : 0.5 * (Wq + Wp);
          cm[a] = 1.0 / dm * wt;
          cpv[a] = 1.0 / dp * wt;
          sum += cm[a] + cpv[a];
        }
        double cc = -sum + alpha * weight;
        for (int a = 0; a < na; a++) {
          int tm = (L->code[c] >> (2 * (2 * a + 0))) & 3, tp = (L->code[c] >> (2 * (2 * a + 1))) & 3;
          if (tm) { cc += fold_sgn(tm) * cm[a]; cm[a] = 0; }
          if (tp) { cc += fold_sgn(tp) * cpv[a]; cpv[a] = 0; }
          L->cp[a][c] = cpv[a];
        }
        L->cc[c] = cc;
      }
}

/* field descriptors: main.f90:771-805 (velocity: cbcvel(:,:,c), is_centered false along c, hi - 1
 * at a wall along c), main.f90:830-838 (scalars: s%cbc, centred) and the pressure */
char or_field_cbc(const or_block *B, int field, int p, int side) {
  if (field == OR_HF_P) return B->desc.cbcpre[p][side];
  if (field < OR_HF_S0) return B->desc.cbcvel[field][p][side];
  return B->desc.cbcscal[field - OR_HF_S0][p][side];
}
double or_field_bc(const or_block *B, int field, int p, int side) {
  if (field == OR_HF_P) return B->desc.bcpre[p][side];
  if (field < OR_HF_S0) return B->desc.bcvel[field][p][side];
  return B->desc.bcscal[field - OR_HF_S0][p][side];
}
int or_field_centered(int field, int p) { return !(field >= OR_HF_U && field < OR_HF_S0 && field == p); }
int or_field_hi(const or_block *B, int field, int p) {
  return B->hi[p] - ((!or_field_centered(field, p) && B->is_bound[p][1]) ? 1 : 0);
}

/* diagonal entry for system s: plane mode adds (lambda*W0)*W1 (solver.f90:1010-1017); a 3-D Helmholtz
 * problem adds alphai*W0*W1*W2 (add_weighted_constant_to_diagonal, solve_helmholtz.f90:134) */
static inline double diag_of(const or_poisson *P, const or_level *L, long c, int i, int j, int s) {
  if (P->mode3d) {
    if (P->shift[s] == 0.0) return L->cc[c];
    int k = (int)(c / ((long)L->n[0] * L->n[1]));
    return L->cc[c] + P->shift[s] * (L->W[0][i] * L->W[1][j] * L->W[2][k]);
  }
  return L->cc[c] + P->shift[s] * L->W[0][i] * L->W[1][j];
}

/* y = A x for system s on level L (inactive cells give 0) */
static void apply_A(const or_poisson *P, const or_level *L, int s, const double *x, double *y) {
  long off = L->ncell * s;
  int na = naxes(P);
#pragma omp parallel for if (P->nsys == 1 && L->ncell >= 32768)
  for (int k = 0; k < L->n[2]; k++)
    for (int j = 0; j < L->n[1]; j++)
      for (int i = 0; i < L->n[0]; i++) {
        long c = i + (long)L->n[0] * (j + (long)L->n[1] * k);
        if (L->code[c] & 0x8000) { y[off + c] = 0.0; continue; }
        double acc = diag_of(P, L, c, i, j, s) * x[off + c];
        for (int a = 0; a < na; a++) {
          if (P->periodic[a] && L->n[a] == 1) continue;
          long cpn = nbr(P, L, i, j, k, a, 1), cmn = nbr(P, L, i, j, k, a, 0);
          if (cpn >= 0) acc += L->cp[a][c] * x[off + cpn];
          if (cmn >= 0) acc += L->cp[a][cmn] * x[off + cmn];
        }
        y[off + c] = acc;
      }
}

/* one red-black Gauss-Seidel colour sweep */
static void rbgs(const or_poisson *P, or_level *L, int s, int color) {
  long off = L->ncell * s;
  int na = naxes(P);
  double *x = L->x, *b = L->b;
#pragma omp parallel for if (P->nsys == 1 && L->ncell >= 32768)
  for (int k = 0; k < L->n[2]; k++)
    for (int j = 0; j < L->n[1]; j++)
      for (int i = 0; i < L->n[0]; i++) {
        if (((i + j + k) & 1) != color) continue;
        long c = i + (long)L->n[0] * (j + (long)L->n[1] * k);
        if (L->code[c] & 0x8000) continue;
        double acc = b[off + c];
        for (int a = 0; a < na; a++) {
          if (P->periodic[a] && L->n[a] == 1) continue;
          long cpn = nbr(P, L, i, j, k, a, 1), cmn = nbr(P, L, i, j, k, a, 0);
          if (cpn >= 0) acc -= L->cp[a][c] * x[off + cpn];
          if (cmn >= 0) acc -= L->cp[a][cmn] * x[off + cmn];
        }
        x[off + c] = acc / diag_of(P, L, c, i, j, s);
      }
}

static void coarse_solve(const or_poisson *P, or_level *L, int s) {
  long n = L->ncell, off = n * s;
  if (L->dinv) {
    const double *M = L->dinv + (size_t)n * n * s;
    for (long r = 0; r < n; r++) {
      double acc = 0.0;
      for (long c = 0; c < n; c++) acc += M[r * n + c] * L->b[off + c];
      L->x[off + r] = acc;
    }
  } else {
    for (long c = 0; c < n; c++) L->x[off + c] = 0.0;
    for (int it = 0; it < 40; it++) { rbgs(P, L, s, 0); rbgs(P, L, s, 1); rbgs(P, L, s, 1); rbgs(P, L, s, 0); }
  }
}

/* V(1,1) cycle on level l for system s: L[l].x <- M L[l].b (zero initial guess) */
static void vcycle(or_poisson *P, int l, int s) {
  or_level *L = &P->L[l];
  long off = L->ncell * s;
  if (l == P->nlev - 1) { coarse_solve(P, L, s); return; }
  for (long c = 0; c < L->ncell; c++) L->x[off + c] = 0.0;
  for (int it = 0; it < P->nu; it++) { rbgs(P, L, s, 0); rbgs(P, L, s, 1); }
  apply_A(P, L, s, L->x, L->r);
  for (long c = 0; c < L->ncell; c++) L->r[off + c] = L->b[off + c] - L->r[off + c];
  or_level *C = &P->L[l + 1];
  long coff = C->ncell * s;
  for (long c = 0; c < C->ncell; c++) C->b[coff + c] = 0.0;
  for (int k = 0; k < L->n[2]; k++)
    for (int j = 0; j < L->n[1]; j++)
      for (int i = 0; i < L->n[0]; i++) {
        int I = C->coarsened[0] ? i / 2 : i, J = C->coarsened[1] ? j / 2 : j, K = C->coarsened[2] ? k / 2 : k;
        long c = i + (long)L->n[0] * (j + (long)L->n[1] * k);
        long cc = I + (long)C->n[0] * (J + (long)C->n[1] * K);
        if (!(L->code[c] & 0x8000)) C->b[coff + cc] += L->r[off + c];
      }
  vcycle(P, l + 1, s);
  for (int k = 0; k < L->n[2]; k++)
    for (int j = 0; j < L->n[1]; j++)
      for (int i = 0; i < L->n[0]; i++) {
        int I = C->coarsened[0] ? i / 2 : i, J = C->coarsened[1] ? j / 2 : j, K = C->coarsened[2] ? k / 2 : k;
        long c = i + (long)L->n[0] * (j + (long)L->n[1] * k);
        long cc = I + (long)C->n[0] * (J + (long)C->n[1] * K);
        if (!(L->code[c] & 0x8000)) L->x[off + c] += C->x[coff + cc];
      }
  for (int it = 0; it < P->nu; it++) { rbgs(P, L, s, 1); rbgs(P, L, s, 0); }
}

static double dot(const or_level *L, int s, const double *a, const double *b) {
  long off = L->ncell * s;
  double acc = 0.0;
  for (long c = 0; c < L->ncell; c++) acc += a[off + c] * b[off + c];
  return acc;
}

/* dense inverse of the coarsest operator of system s (Cholesky of -A, plus 11^T when singular) */
static int build_dense(or_poisson *P, or_level *L, int s, double *M) {
  long n = L->ncell;
  double *A = calloc((size_t)n * n, sizeof(double));
  double *e = calloc(n, sizeof(double)), *col = calloc(n, sizeof(double));
  long nact = 0;
  for (long c = 0; c < n; c++) if (!(L->code[c] & 0x8000)) nact++;
  /* A = -operator, column by column */
  double *save_x = L->x; /* use a private vector through apply_A's interface */
  for (long c = 0; c < n; c++) {
    memset(e, 0, sizeof(double) * n);
    e[c] = 1.0;
    /* apply_A reads x[off+...]; emulate with s=0 offsets on private arrays */
    or_level tmp = *L;
    tmp.ncell = n;
    or_poisson Pt = *P;
    Pt.nsys = 1;
    double shift_s = P->shift[s];
    Pt.shift = &shift_s;
    apply_A(&Pt, &tmp, 0, e, col);
    for (long r = 0; r < n; r++) A[r * n + c] = -col[r];
  }
  (void)save_x;
  double dsum = 0.0;
  for (long c = 0; c < n; c++) {
    if (L->code[c] & 0x8000) { for (long r = 0; r < n; r++) { A[r * n + c] = 0; A[c * n + r] = 0; } A[c * n + c] = 1.0; }
    else dsum += A[c * n + c];
  }
  if (P->singular[s] && nact > 0) {
    double sh = dsum / nact;
    for (long r = 0; r < n; r++)
      for (long c = 0; c < n; c++)
        if (!(L->code[r] & 0x8000) && !(L->code[c] & 0x8000)) A[r * n + c] += sh;
  }
  /* Cholesky A = G G^T in place (lower) */
  for (long j = 0; j < n; j++) {
    double d = A[j * n + j];
    for (long k = 0; k < j; k++) d -= A[j * n + k] * A[j * n + k];
    if (d <= 0.0) { free(A); free(e); free(col); return -1; }
    d = sqrt(d);
    A[j * n + j] = d;
    for (long i = j + 1; i < n; i++) {
      double v = A[i * n + j];
      for (long k = 0; k < j; k++) v -= A[i * n + k] * A[j * n + k];
      A[i * n + j] = v / d;
    }
  }
  /* inverse column by column; M = -(A^{-1}) so that x = M b solves the original operator */
  for (long c = 0; c < n; c++) {
    memset(e, 0, sizeof(double) * n);
    e[c] = 1.0;
    for (long i = 0; i < n; i++) { double v = e[i]; for (long k = 0; k < i; k++) v -= A[i * n + k] * e[k]; e[i] = v / A[i * n + i]; }
    for (long i = n - 1; i >= 0; i--) { double v = e[i]; for (long k = i + 1; k < n; k++) v -= A[k * n + i] * e[k]; e[i] = v / A[i * n + i]; }
    for (long r = 0; r < n; r++) M[r * n + c] = (L->code[r] & 0x8000) || (L->code[c] & 0x8000) ? 0.0 : -e[r];
  }
  free(A); free(e); free(col);
  return 0;
}

or_poisson *or_poisson_create(or_domain *d, int field, double alpha, const double *lambda, char *err, int errlen) {
  or_poisson *P = calloc(1, sizeof(or_poisson));
  int centered[3];
  for (int p = 0; p < 3; p++) centered[p] = or_field_centered(field, p);
  P->field = field;
  P->helm = field != OR_HF_P;
  P->mode3d = d->fft_axis == 0;
  if (P->mode3d) { P->ax[0] = 0; P->ax[1] = 1; P->ax[2] = 2; }
  else { P->ax[0] = d->il; P->ax[1] = d->iu; P->ax[2] = d->fft_axis - 1; }
  P->tol = d->c.tol;
  P->maxiter = d->c.maxiter;
  P->nu = 2;
  int lo_min[3], hi_max[3];
  for (int p = 0; p < 3; p++) {
    lo_min[p] = d->b[0].lo[p]; hi_max[p] = or_field_hi(&d->b[0], field, p);
    for (int ib = 1; ib < d->nblocks; ib++) {
      if (d->b[ib].lo[p] < lo_min[p]) lo_min[p] = d->b[ib].lo[p];
      if (or_field_hi(&d->b[ib], field, p) > hi_max[p]) hi_max[p] = or_field_hi(&d->b[ib], field, p);
    }
    P->lo_min[p] = lo_min[p];
  }
  or_level *L = &P->L[0];
  int na = naxes(P);
  for (int a = 0; a < 3; a++) {
    int p = P->ax[a];
    L->n[a] = (a < na) ? hi_max[p] - lo_min[p] + 1 : 1;
    P->periodic[a] = (a < na) ? (d->periods[p] != 0) : 0;
  }
  if (!P->mode3d) {
    int pf = P->ax[2];
    P->nsys = hi_max[pf] - lo_min[pf] + 1;
    for (int ib = 0; ib < d->nblocks; ib++)
      if (d->b[ib].lo[pf] != lo_min[pf] || or_field_hi(&d->b[ib], field, pf) != hi_max[pf]) {
        snprintf(err, errlen, "blocks must span the whole transform direction");
        or_poisson_destroy(P); return NULL;
      }
  } else P->nsys = 1;
  P->shift = calloc(P->nsys, sizeof(double));
  P->singular = calloc(P->nsys, sizeof(int));
  for (int s = 0; s < P->nsys; s++) P->shift[s] = P->mode3d ? 0.0 : lambda[s];
  alloc_level(P, L);
  for (long c = 0; c < L->ncell; c++) L->code[c] = 0x8000;
  int have_w[3][4096];
  memset(have_w, 0, sizeof(have_w));
  /* assemble level 0 block by block with each block's own metric arrays */
  double *cm[3];
  for (int a = 0; a < 3; a++) cm[a] = calloc(L->ncell, sizeof(double));
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    const double *d1[3], *d2[3];
    int q3[3];
    for (int p = 0; p < 3; p++) {
      d1[p] = centered[p] ? B->g[p][0] : B->g[p][1];
      d2[p] = centered[p] ? B->g[p][1] : B->g[p][0];
      q3[p] = centered[p] ? 0 : 1;
    }
    int loc[3], hic[3], bhi[3];
    for (int p = 0; p < 3; p++) bhi[p] = or_field_hi(B, field, p);
    for (int a = 0; a < 3; a++) {
      int p = P->ax[a];
      loc[a] = (a < na) ? B->lo[p] : 0;
      hic[a] = (a < na) ? bhi[p] : 0;
    }
    for (int g2 = loc[2]; g2 <= hic[2]; g2++)
      for (int g1 = loc[1]; g1 <= hic[1]; g1++)
        for (int g0 = loc[0]; g0 <= hic[0]; g0++) {
          int gg[3] = {g0, g1, g2};
          int idx[3];
          for (int a = 0; a < 3; a++) idx[a] = (a < na) ? gg[a] - lo_min[P->ax[a]] : 0;
          long c = idx[0] + (long)L->n[0] * (idx[1] + (long)L->n[1] * idx[2]);
          if (!(L->code[c] & 0x8000)) { snprintf(err, errlen, "overlapping blocks in the solver box"); goto fail; }
          L->code[c] = 0;
          /* widths (consistency across blocks checked) */
          for (int a = 0; a < na; a++) {
            int p = P->ax[a];
            double wv = d2[p][LOCAL(B, p, gg[a])];
            if (idx[a] < 4096 && have_w[a][idx[a]] && L->W[a][idx[a]] != wv) {
              snprintf(err, errlen, "inconsistent grid spacing along axis %d at global index %d", p + 1, gg[a]);
              goto fail;
            }
            L->W[a][idx[a]] = wv;
            if (idx[a] < 4096) have_w[a][idx[a]] = 1;
          }
          double weight, cmv[3] = {0, 0, 0}, cpv[3] = {0, 0, 0}, cc;
          if (P->mode3d) {
            /* solver.f90:289-297 */
            double dx2 = d2[0][LOCAL(B, 0, g0)], dy2 = d2[1][LOCAL(B, 1, g1)], dz2 = d2[2][LOCAL(B, 2, g2)];
            weight = dx2 * dy2 * dz2;
            cmv[0] = 1.0 / (d1[0][LOCAL(B, 0, g0 - 1 + q3[0])]) * dy2 * dz2;
            cpv[0] = 1.0 / (d1[0][LOCAL(B, 0, g0 + q3[0])]) * dy2 * dz2;
            cmv[1] = 1.0 / (d1[1][LOCAL(B, 1, g1 - 1 + q3[1])]) * dx2 * dz2;
            cpv[1] = 1.0 / (d1[1][LOCAL(B, 1, g1 + q3[1])]) * dx2 * dz2;
            cmv[2] = 1.0 / (d1[2][LOCAL(B, 2, g2 - 1 + q3[2])]) * dx2 * dy2;
            cpv[2] = 1.0 / (d1[2][LOCAL(B, 2, g2 + q3[2])]) * dx2 * dy2;
            /* a periodic axis of one cell couples each cell to itself (HYPRE's periodic wrap): the +/- terms cancel */
            for (int a = 0; a < 3; a++)
              if (P->periodic[a] && L->n[a] == 1) cmv[a] = cpv[a] = 0.0;
            cc = 0.0;
            cc = cc - (cmv[0] + cpv[0] + cmv[1] + cpv[1] + cmv[2] + cpv[2]) + alpha * weight;
          } else {
            /* solver.f90:779-785 */
            int p1 = P->ax[0], p2 = P->ax[1];
            double w1 = d2[p1][LOCAL(B, p1, g0)], w2 = d2[p2][LOCAL(B, p2, g1)];
            weight = w1 * w2;
            cmv[0] = 1.0 / (d1[p1][LOCAL(B, p1, g0 - 1 + q3[p1])]) * w2;
            cpv[0] = 1.0 / (d1[p1][LOCAL(B, p1, g0 + q3[p1])]) * w2;
            cmv[1] = 1.0 / (d1[p2][LOCAL(B, p2, g1 - 1 + q3[p2])]) * w1;
            cpv[1] = 1.0 / (d1[p2][LOCAL(B, p2, g1 + q3[p2])]) * w1;
            for (int a = 0; a < 2; a++)
              if (P->periodic[a] && L->n[a] == 1) cmv[a] = cpv[a] = 0.0;
            cc = -(cmv[0] + cpv[0] + cmv[1] + cpv[1]) + alpha * weight;
          }
          /* boundary folding, solver.f90:298-351 / 786-822 */
          unsigned short code = 0;
          for (int a = 0; a < na; a++) {
            int p = P->ax[a];
            if (d->periods[p] != 0) continue;
            if (B->is_bound[p][0] && gg[a] == B->lo[p]) {
              int t = fold_type(or_field_cbc(B, field, p, 0), centered[p]);
              cc = cc + fold_sgn(t) * cmv[a];
              cmv[a] = 0.0;
              code |= (unsigned short)(t << (2 * (2 * a)));
            }
            if (B->is_bound[p][1] && gg[a] == bhi[p]) {
              int t = fold_type(or_field_cbc(B, field, p, 1), centered[p]);
              cc = cc + fold_sgn(t) * cpv[a];
              cpv[a] = 0.0;
              code |= (unsigned short)(t << (2 * (2 * a + 1)));
            }
          }
          L->code[c] = code;
          L->cc[c] = cc;
          for (int a = 0; a < na; a++) { L->cp[a][c] = cpv[a]; cm[a][c] = cmv[a]; }
        }
  }
  /* symmetry / connectivity check: cm(c) must equal cp(c - e_a) */
  for (int k = 0; k < L->n[2]; k++)
    for (int j = 0; j < L->n[1]; j++)
      for (int i = 0; i < L->n[0]; i++) {
        long c = i + (long)L->n[0] * (j + (long)L->n[1] * k);
        if (L->code[c] & 0x8000) continue;
        for (int a = 0; a < na; a++) {
          long m = nbr(P, L, i, j, k, a, 0);
          int tm = (L->code[c] >> (2 * (2 * a))) & 3;
          if (m < 0 || (L->code[m] & 0x8000)) {
            if (!tm) { snprintf(err, errlen, "unfolded block face on the solver box boundary"); goto fail; }
            continue;
          }
          int tpn = (L->code[m] >> (2 * (2 * a + 1))) & 3;
          if (tm && tpn) continue; /* two physical faces back to back: uncoupled */
          if (tm || tpn || cm[a][c] != L->cp[a][m]) {
            snprintf(err, errlen, "inconsistent coupling between adjacent cells along axis %d", P->ax[a] + 1);
            goto fail;
          }
        }
      }
  for (int a = 0; a < 3; a++) { free(cm[a]); cm[a] = NULL; }
  /* singular systems: no Dirichlet fold anywhere, zero diagonal constant */
  int has_dir = 0;
  for (long c = 0; c < L->ncell; c++) {
    if (L->code[c] & 0x8000) continue;
    for (int f = 0; f < 6; f++) { int t = (L->code[c] >> (2 * f)) & 3; if (t == 2 || t == 3) has_dir = 1; }
  }
  for (int s = 0; s < P->nsys; s++) P->singular[s] = !P->helm && (!has_dir && alpha == 0.0 && P->shift[s] == 0.0);
  /* hierarchy: coarsen an axis while every block keeps an even offset and extent */
  int boff[64][3], bext[64][3];
  if (d->nblocks > 64) { snprintf(err, errlen, "too many blocks for the oracle solver"); goto fail; }
  for (int ib = 0; ib < d->nblocks; ib++)
    for (int a = 0; a < 3; a++) {
      int p = P->ax[a];
      boff[ib][a] = (a < na) ? d->b[ib].lo[p] - lo_min[p] : 0;
      bext[ib][a] = (a < na) ? or_field_hi(&d->b[ib], field, p) - d->b[ib].lo[p] + 1 : 1;
    }
  P->nlev = 1;
  while (P->nlev < OR_MAXLEV) {
    or_level *F = &P->L[P->nlev - 1];
    if (F->ncell <= OR_DENSE_MAX) break;
    /* eligible axes keep even block offsets/extents (and even periodic rings); among them
       only the strongly coupled ones (smallest spacing within a factor 2) are halved,
       semicoarsening as PFMG does */
    double hmin[3] = {1e300, 1e300, 1e300}, hall = 1e300;
    int elig[3] = {0, 0, 0};
    for (int a = 0; a < na; a++) {
      if (F->n[a] < 2 || F->n[a] % 2) continue;
      int ok = 1;
      for (int ib = 0; ib < d->nblocks; ib++) if (boff[ib][a] % 2 || bext[ib][a] % 2) ok = 0;
      if (P->periodic[a] && (F->n[a] / 2) % 2 && F->n[a] / 2 != 1) ok = 0;
      if (!ok) continue;
      elig[a] = 1;
      for (int q = 0; q < F->n[a]; q++) if (F->W[a][q] < hmin[a]) hmin[a] = F->W[a][q];
      if (hmin[a] < hall) hall = hmin[a];
    }
    int co[3] = {0, 0, 0}, any = 0;
    for (int a = 0; a < na; a++)
      if (elig[a] && hmin[a] <= 2.0 * hall) { co[a] = 1; any = 1; }
    if (!any) break;
    or_level *C = &P->L[P->nlev];
    for (int a = 0; a < 3; a++) { C->n[a] = co[a] ? F->n[a] / 2 : F->n[a]; C->coarsened[a] = co[a]; }
    alloc_level(P, C);
    for (int a = 0; a < 3; a++)
      for (int q = 0; q < C->n[a]; q++) C->W[a][q] = co[a] ? F->W[a][2 * q] + F->W[a][2 * q + 1] : F->W[a][q];
    for (int k = 0; k < C->n[2]; k++)
      for (int j = 0; j < C->n[1]; j++)
        for (int i = 0; i < C->n[0]; i++) {
          long c = i + (long)C->n[0] * (j + (long)C->n[1] * k);
          int f0[3] = {co[0] ? 2 * i : i, co[1] ? 2 * j : j, co[2] ? 2 * k : k};
          long fc = f0[0] + (long)F->n[0] * (f0[1] + (long)F->n[1] * f0[2]);
          unsigned short code = F->code[fc];
          if (!(code & 0x8000)) {
            code &= 0x7fff;
            for (int a = 0; a < 3; a++) {
              if (!co[a]) continue;
              int f1[3] = {f0[0], f0[1], f0[2]};
              f1[a] += 1;
              long fc1 = f1[0] + (long)F->n[0] * (f1[1] + (long)F->n[1] * f1[2]);
              int tp = (F->code[fc1] >> (2 * (2 * a + 1))) & 3;
              code = (unsigned short)((code & ~(3u << (2 * (2 * a + 1)))) | (tp << (2 * (2 * a + 1))));
            }
          }
          C->code[c] = code;
        }
    build_coarse_operator(P, C, alpha);
    for (int ib = 0; ib < d->nblocks; ib++)
      for (int a = 0; a < 3; a++) if (co[a]) { boff[ib][a] /= 2; bext[ib][a] /= 2; }
    P->nlev++;
  }
  {
    or_level *C = &P->L[P->nlev - 1];
    /* Helmholtz problems: the dense inverse would depend on the shift; their coarsest level is
       diagonally dominant and is smoothed instead */
    if (C->ncell <= OR_DENSE_MAX && !P->helm) {
      C->dinv = calloc((size_t)C->ncell * C->ncell * P->nsys, sizeof(double));
      for (int s = 0; s < P->nsys; s++)
        if (build_dense(P, C, s, C->dinv + (size_t)C->ncell * C->ncell * s)) {
          snprintf(err, errlen, "coarsest operator of system %d is not definite", s);
          goto fail;
        }
    }
  }
  P->p = calloc(L->ncell * P->nsys, sizeof(double));
  P->q = calloc(L->ncell * P->nsys, sizeof(double));
  P->z = calloc(L->ncell * P->nsys, sizeof(double));
  return P;
fail:
  for (int a = 0; a < 3; a++) free(cm[a]);
  or_poisson_destroy(P);
  return NULL;
}

/* singular systems: the preconditioned residual is taken orthogonal to the null space (the constant
 * over the active cells), so that the search directions carry no constant and x - x0 stays mean-free;
 * without it the smoother's constant drift accumulates in x and swamps the residual in cancellation */
static void remove_mean(const or_level *L, int s, double *v) {
  long n = L->ncell, off = n * s, na = 0;
  double sum = 0.0;
  for (long c = 0; c < n; c++) if (!(L->code[c] & 0x8000)) { sum += v[off + c]; na++; }
  double mean = na ? sum / na : 0.0;
  for (long c = 0; c < n; c++) if (!(L->code[c] & 0x8000)) v[off + c] -= mean;
}

/* Solve A x = b for every system; x holds the initial guess on entry. */
int or_poisson_solve(or_poisson *P, double *b, double *x) {
  or_level *L = &P->L[0];
  long n = L->ncell;
  int maxit_seen = 0;
  double worst = 0.0;
  int fail = 0;
#pragma omp parallel for if (P->nsys > 1) schedule(dynamic) reduction(max : maxit_seen, worst) reduction(| : fail)
  for (int s = 0; s < P->nsys; s++) {
    long off = n * s;
    double *r = L->r, *z, *p = P->p, *q = P->q;
    if (P->singular[s]) {
      double sum = 0.0; long na = 0;
      for (long c = 0; c < n; c++) if (!(L->code[c] & 0x8000)) { sum += b[off + c]; na++; }
      double mean = na ? sum / na : 0.0;
      for (long c = 0; c < n; c++) if (!(L->code[c] & 0x8000)) b[off + c] -= mean;
    }
    double bb = dot(L, s, b, b);
    if (bb == 0.0) { for (long c = 0; c < n; c++) x[off + c] = 0.0; continue; }
    /* residual r = b - A x (kept in P->z to leave L->r to the V-cycle) */
    z = P->z;
    apply_A(P, L, s, x, q);
    for (long c = 0; c < n; c++) z[off + c] = b[off + c] - q[off + c];
    double rr = dot(L, s, z, z);
    if (rr > bb) { /* a warm start worse than zero is dropped: x = 0, r = b */
      for (long c = 0; c < n; c++) { x[off + c] = 0.0; z[off + c] = b[off + c]; }
      rr = bb;
    }
    if (P->singular[s]) { remove_mean(L, s, z); rr = dot(L, s, z, z); } /* consistent correction equation */
    int it = 0;
    double rel = sqrt(rr / bb);
    if (rel > P->tol) {
      /* V-cycle on the residual: L->b <- r, M r in L->x */
      memcpy(L->b + off, z + off, sizeof(double) * n);
      vcycle(P, 0, s);
      if (P->singular[s]) remove_mean(L, s, L->x);
      for (long c = 0; c < n; c++) p[off + c] = L->x[off + c];
      double rz = dot(L, s, z, L->x);
      for (it = 1; it <= P->maxiter; it++) {
        apply_A(P, L, s, p, q);
        double pq = dot(L, s, p, q);
        double alpha = rz / pq;
        for (long c = 0; c < n; c++) { x[off + c] += alpha * p[off + c]; z[off + c] -= alpha * q[off + c]; }
        rr = dot(L, s, z, z);
        rel = sqrt(rr / bb);
        if (rel <= P->tol) break;
        memcpy(L->b + off, z + off, sizeof(double) * n);
        vcycle(P, 0, s);
        if (P->singular[s]) remove_mean(L, s, L->x);
        double rzn = dot(L, s, z, L->x);
        double beta = rzn / rz;
        rz = rzn;
        for (long c = 0; c < n; c++) p[off + c] = L->x[off + c] + beta * p[off + c];
      }
      if (it > P->maxiter) { it = P->maxiter; fail = 1; }
    }
    (void)r;
    if (it > maxit_seen) maxit_seen = it;
    if (rel > worst) worst = rel;
  }
  P->last_iter = maxit_seen;
  P->last_res = worst;
  return fail ? 1 : 0;
}

/* gather the interior of field `kind` of every block into box layout (plane mode: [i1,i2,k]) */
void or_box_gather(or_domain *d, or_poisson *P, int kind, double *box) {
  or_level *L = &P->L[0];
  memset(box, 0, sizeof(double) * L->ncell * P->nsys);
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    int nx = B->hi[0] - B->lo[0] + 1, ny = B->hi[1] - B->lo[1] + 1;
    double *f = B->fld[kind];
    int h0 = or_field_hi(B, P->field, 0), h1 = or_field_hi(B, P->field, 1), h2 = or_field_hi(B, P->field, 2);
    for (int k = B->lo[2]; k <= h2; k++)
      for (int j = B->lo[1]; j <= h1; j++)
        for (int i = B->lo[0]; i <= h0; i++) {
          int g[3] = {i, j, k};
          long c, s;
          int a0 = g[P->ax[0]] - P->lo_min[P->ax[0]], a1 = g[P->ax[1]] - P->lo_min[P->ax[1]];
          int a2 = g[P->ax[2]] - P->lo_min[P->ax[2]];
          if (P->mode3d) { c = a0 + (long)L->n[0] * (a1 + (long)L->n[1] * a2); s = 0; }
          else { c = a0 + (long)L->n[0] * a1; s = a2; }
          box[s * L->ncell + c] = f[(i - B->lo[0] + 1) + (size_t)(nx + 2) * ((j - B->lo[1] + 1) + (size_t)(ny + 2) * (k - B->lo[2] + 1))];
        }
  }
}

void or_box_scatter(or_domain *d, or_poisson *P, double *box, int kind) {
  or_level *L = &P->L[0];
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    int nx = B->hi[0] - B->lo[0] + 1, ny = B->hi[1] - B->lo[1] + 1;
    double *f = B->fld[kind];
    int h0 = or_field_hi(B, P->field, 0), h1 = or_field_hi(B, P->field, 1), h2 = or_field_hi(B, P->field, 2);
    for (int k = B->lo[2]; k <= h2; k++)
      for (int j = B->lo[1]; j <= h1; j++)
        for (int i = B->lo[0]; i <= h0; i++) {
          int g[3] = {i, j, k};
          long c, s;
          int a0 = g[P->ax[0]] - P->lo_min[P->ax[0]], a1 = g[P->ax[1]] - P->lo_min[P->ax[1]];
          int a2 = g[P->ax[2]] - P->lo_min[P->ax[2]];
          if (P->mode3d) { c = a0 + (long)L->n[0] * (a1 + (long)L->n[1] * a2); s = 0; }
          else { c = a0 + (long)L->n[0] * a1; s = a2; }
          f[(i - B->lo[0] + 1) + (size_t)(nx + 2) * ((j - B->lo[1] + 1) + (size_t)(ny + 2) * (k - B->lo[2] + 1))] = box[s * L->ncell + c];
        }
  }
}
