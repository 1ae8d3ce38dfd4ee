/*
 * or_domain.c -- oracle restatement of the set-up and of one RK3 step with
 * all blocks held by one process.  TEST INFRASTRUCTURE ONLY.
 *
 * The reference runs one MPI rank per block; MPI_SENDRECV halo exchanges
 * (bound.f90:587-650) are restated as plane copies between the blocks'
 * arrays, done direction by direction (x for every block, then y, then z)
 * and before any physical boundary condition, which is the order the
 * paired SENDRECVs impose.  Allreduce results are plain sums/maxima over
 * blocks in block order.
 */
#include "or_internal.h"
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static const double PI = 3.14159265358979323846264338327950288;
/* rkcoeff, param.f90:11-14 */
static const double RKC[3][2] = {{32.0 / 60.0, 0.0}, {25.0 / 60.0, -17.0 / 60.0}, {45.0 / 60.0, -25.0 / 60.0}};

void or_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ---- initgrid.f90:171-287 (grid stretching functions) ---- */
static double gp_one_end(double alpha, double r0) {
  if (alpha != 0.0) return 1.0 * (1.0 + tanh((r0 - 1.0) * alpha) / tanh(alpha / 1.0));
  return r0;
}
static double gp_geo_one_end(double alpha, double r0) {
  const double power = 1.0 / 3.0;
  if (r0 == 1.0) return r0;
  return r0 * pow((1.0 - pow(r0, alpha)) / (1.0 - r0) / alpha, power);
}
static double gridpoint(int gt, double alpha, double r0) {
  switch (gt) {
    case 1: return gp_one_end(alpha, r0);
    case 2:
      if (alpha != 0.0) {
        if (r0 <= 0.5) return 0.5 * (1.0 - 1.0 + tanh(2.0 * alpha * (r0 - 0.0)) / tanh(alpha));
        return 0.5 * (1.0 + 1.0 + tanh(2.0 * alpha * (r0 - 1.0)) / tanh(alpha));
      }
      return r0;
    case 3:
      if (alpha != 0.0) return 1.0 - 1.0 * (1.0 + tanh((1.0 - r0 - 1.0) * alpha) / tanh(alpha / 1.0));
      return r0;
    case 4: return gp_geo_one_end(alpha, r0);
    case 5: return 1.0 - gp_geo_one_end(alpha, 1.0 - r0);
    case 6:
      if (r0 <= 0.5) return gp_geo_one_end(alpha / 2.0, 2.0 * r0) / 2.0;
      return 1.0 - gp_geo_one_end(alpha / 2.0, 2.0 * (1.0 - r0)) / 2.0;
    case 7:
      if (r0 <= 0.5) return (1.0 - gp_geo_one_end(alpha / 2.0, (0.5 - r0) * 2.0)) / 2.0;
      return (1.0 + gp_geo_one_end(alpha / 2.0, (r0 - 0.5) * 2.0)) / 2.0;
    default: /* 0: cluster_two_end, initgrid.f90:171-184 */
      if (alpha != 0.0) return 0.5 * (1.0 + tanh((r0 - 0.5) * alpha) / tanh(alpha / 2.0));
      return r0;
  }
}

/* initgrid.f90:9-83; arrays hold lo-1..hi+1 */
void or_initgrid(int lo, int hi, int gt, double gr, double lmin, double lmax,
                 double *drc, double *drf, double *rc, double *rf) {
#define AT(a, q) (a)[(q) - lo + 1]
  int n = hi - lo + 1;
  for (int q = lo; q <= hi; q++) {
    double r0 = ((double)(q - lo + 1) - 0.0) / (1.0 * n);
    AT(rf, q) = gridpoint(gt, gr, r0);
    AT(rf, q) = lmin + AT(rf, q) * (lmax - lmin);
  }
  AT(rf, lo - 1) = lmin;
  for (int q = lo; q <= hi; q++) AT(drf, q) = AT(rf, q) - AT(rf, q - 1);
  AT(drf, lo - 1) = AT(drf, lo);
  AT(drf, hi + 1) = AT(drf, hi);
  for (int q = lo - 1; q <= hi; q++) AT(drc, q) = 0.5 * (AT(drf, q) + AT(drf, q + 1));
  AT(drc, hi + 1) = AT(drc, hi);
  AT(rc, lo - 1) = lmin - AT(drc, lo - 1) / 2.0;
  AT(rf, lo - 1) = lmin;
  for (int q = lo; q <= hi + 1; q++) {
    AT(rc, q) = AT(rc, q - 1) + AT(drc, q - 1);
    AT(rf, q) = AT(rf, q - 1) + AT(drf, q);
  }
#undef AT
}

/* initgrid.f90:144-165 (load_grid): file = rf,rc,drf,drc over lo..hi */
static void load_grid(int lo, int hi, const double *file, double *rf, double *rc, double *drf, double *drc) {
#define AT(a, q) (a)[(q) - lo + 1]
  int n = hi - lo + 1;
  for (int q = lo; q <= hi; q++) {
    AT(rf, q) = file[q - lo];
    AT(rc, q) = file[n + q - lo];
    AT(drf, q) = file[2 * n + q - lo];
    AT(drc, q) = file[3 * n + q - lo];
  }
  AT(drf, lo - 1) = AT(drf, lo);
  AT(drf, hi + 1) = AT(drf, hi);
  AT(drc, lo - 1) = AT(drf, lo);
  AT(drc, hi + 1) = AT(drc, hi);
  AT(rf, lo - 1) = AT(rf, lo) - AT(drf, lo);
  AT(rf, hi + 1) = AT(rf, hi) + AT(drf, hi);
  AT(rc, lo - 1) = AT(rc, lo) - AT(drc, lo - 1);
  AT(rc, hi + 1) = AT(rc, hi) + AT(drc, hi);
#undef AT
}

/* initmpi.f90:50-98: breadth-first placement of the blocks in a global index space */
int or_place_blocks(int nblocks, const or_block_desc *bl, int (*lo)[3]) {
  int *done = calloc(nblocks, sizeof(int)), *unl = calloc(nblocks, sizeof(int));
  int iblock = 0, rc = 0;
  for (int a = 0; a < 3; a++) lo[0][a] = 1;
  unl[0] = 1;
  for (;;) {
    int all = 1;
    for (int q = 0; q < nblocks; q++) if (!done[q]) all = 0;
    if (all) break;
    if (iblock < 0 || iblock >= nblocks) { rc = -1; break; }
    for (int idir = 0; idir < 3; idir++) {
      for (int inb = 0; inb < 2; inb++) {
        if (bl[iblock].cbcpre[idir][inb] != 'F') continue;
        int ifr = (int)lround(bl[iblock].bcpre[idir][inb]) - 1;
        if (ifr < 0 || ifr >= nblocks) { rc = -2; goto out; }
        if (unl[ifr]) continue;
        if (inb == 0 && bl[ifr].lmin[idir] > bl[iblock].lmin[idir]) continue;
        if (inb == 1 && bl[ifr].lmin[idir] < bl[iblock].lmin[idir]) continue;
        int ioff = -(1 - inb) * bl[ifr].ng[idir] + inb * bl[iblock].ng[idir];
        lo[ifr][idir] = lo[iblock][idir] + ioff;
        for (int t = 0; t < 3; t++) if (t != idir) lo[ifr][t] = lo[iblock][t];
        unl[ifr] = 1;
      }
    }
    done[iblock] = 1;
    iblock = -1;
    for (int q = 0; q < nblocks; q++) if (!done[q] && unl[q]) { iblock = q; break; }
  }
out:
  free(done); free(unl);
  return rc;
}

static double *fld_alloc(const or_block *B, int halo) {
  size_t n = halo ? (size_t)(B->ng[0] + 2) * (B->ng[1] + 2) * (B->ng[2] + 2) : (size_t)B->ng[0] * B->ng[1] * B->ng[2];
  return calloc(n, sizeof(double));
}

or_domain *or_create(const or_case *c, const or_block_desc *blocks, char *err, int errlen) {
  or_domain *d = calloc(1, sizeof(or_domain));
  d->c = *c;
  d->nblocks = c->nblocks;
  d->b = calloc(d->nblocks, sizeof(or_block));
  int (*lo)[3] = calloc(d->nblocks, sizeof(int[3]));
  if (or_place_blocks(d->nblocks, blocks, lo)) { snprintf(err, errlen, "invalid block connectivity"); goto fail; }
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    B->desc = blocks[ib];
    for (int a = 0; a < 3; a++) {
      B->ng[a] = blocks[ib].ng[a];
      B->lo[a] = lo[ib][a];
      B->hi[a] = lo[ib][a] + B->ng[a] - 1;
    }
  }
  /* param.f90:460-487 (is_periodic) and initmpi.f90:107-113 (periods) */
  for (int q = 0; q < 3; q++) {
    d->is_periodic[q] = 1;
    int lmn = d->b[0].lo[q], hmx = d->b[0].hi[q];
    for (int ib = 0; ib < d->nblocks; ib++) {
      if (!(blocks[ib].cbcpre[q][0] == 'F' && blocks[ib].cbcpre[q][1] == 'F')) d->is_periodic[q] = 0;
      if (d->b[ib].lo[q] < lmn) lmn = d->b[ib].lo[q];
      if (d->b[ib].hi[q] > hmx) hmx = d->b[ib].hi[q];
    }
    d->periods[q] = d->is_periodic[q] ? hmx - lmn + 1 : 0;
  }
  /* neighbours (initmpi.f90:150-237, one rank per block) */
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    for (int q = 0; q < 3; q++)
      for (int s = 0; s < 2; s++) {
        B->nb[q][s] = -1;
        if (blocks[ib].cbcpre[q][s] == 'F') {
          int f = (int)lround(blocks[ib].bcpre[q][s]) - 1;
          if (f < 0 || f >= d->nblocks) { snprintf(err, errlen, "block %d: friend %d does not exist", ib + 1, f + 1); goto fail; }
          or_block *Fb = &d->b[f];
          int ok = blocks[f].cbcpre[q][1 - s] == 'F' && (int)lround(blocks[f].bcpre[q][1 - s]) - 1 == ib;
          for (int t = 0; t < 3; t++)
            if (t != q) ok = ok && Fb->lo[t] == B->lo[t] && Fb->hi[t] == B->hi[t] &&
                              blocks[f].lmin[t] == blocks[ib].lmin[t] && blocks[f].lmax[t] == blocks[ib].lmax[t] &&
                              blocks[f].gr[t] == blocks[ib].gr[t] && blocks[f].gt[t] == blocks[ib].gt[t];
          /* adjacency in the global index space, directly or through the periodic wrap */
          if (s == 0) ok = ok && (Fb->hi[q] + 1 == B->lo[q] || (d->periods[q] && Fb->hi[q] - B->lo[q] + 1 == d->periods[q]));
          else ok = ok && (B->hi[q] + 1 == Fb->lo[q] || (d->periods[q] && B->hi[q] - Fb->lo[q] + 1 == d->periods[q]));
          if (!ok) { snprintf(err, errlen, "block %d: inconsistent connectivity with block %d", ib + 1, f + 1); goto fail; }
          B->nb[q][s] = f;
        }
        B->is_bound[q][s] = B->nb[q][s] < 0;
      }
  }
  /* grids: initgrid.f90:9-83, optional load_grid, distribute_grid, bound_grid (initgrid.f90:91-127) */
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    for (int a = 0; a < 3; a++) {
      int n2 = B->ng[a] + 2;
      for (int w = 0; w < 4; w++) B->g[a][w] = calloc(n2, sizeof(double));
      or_initgrid(B->lo[a], B->hi[a], blocks[ib].gt[a], blocks[ib].gr[a], blocks[ib].lmin[a], blocks[ib].lmax[a],
                  B->g[a][OR_G_DXC], B->g[a][OR_G_DXF], B->g[a][OR_G_XC], B->g[a][OR_G_XF]);
      if (blocks[ib].grid_file[a])
        load_grid(B->lo[a], B->hi[a], blocks[ib].grid_file[a], B->g[a][OR_G_XF], B->g[a][OR_G_XC], B->g[a][OR_G_DXF], B->g[a][OR_G_DXC]);
    }
  }
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    for (int a = 0; a < 3; a++) {
      int n = B->ng[a];
      double *df = B->g[a][OR_G_DXF], *dc = B->g[a][OR_G_DXC];
      if (B->nb[a][0] >= 0) { or_block *N = &d->b[B->nb[a][0]]; df[0] = N->g[a][OR_G_DXF][N->ng[a]]; }
      if (B->nb[a][1] >= 0) { or_block *N = &d->b[B->nb[a][1]]; df[n + 1] = N->g[a][OR_G_DXF][1]; }
    }
  }
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    for (int a = 0; a < 3; a++) {
      int n = B->ng[a];
      double *df = B->g[a][OR_G_DXF], *dc = B->g[a][OR_G_DXC];
      dc[0] = (df[1] + df[0]) / 2.0;
      dc[n] = (df[n + 1] + df[n]) / 2.0;
      dc[n + 1] = dc[n];
    }
  }
  /* vol_all, param.f90:493-494 */
  d->vol_all = 0.0;
  for (int ib = 0; ib < d->nblocks; ib++)
    d->vol_all += (blocks[ib].lmax[0] - blocks[ib].lmin[0]) * (blocks[ib].lmax[1] - blocks[ib].lmin[1]) *
                  (blocks[ib].lmax[2] - blocks[ib].lmin[2]);
  /* fields */
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    for (int f = OR_U; f <= OR_PO; f++) B->fld[f] = fld_alloc(B, 1);
    for (int f = OR_DUDTRKO; f <= OR_DWDTRKO; f++) B->fld[f] = fld_alloc(B, 0);
    for (int s = 0; s < c->nscal; s++) { B->fld[OR_S0 + s] = fld_alloc(B, 1); B->fld[OR_DSDTRKO0 + s] = fld_alloc(B, 0); }
    B->rhsp[0] = calloc((size_t)B->ng[1] * B->ng[2] * 2, sizeof(double));
    B->rhsp[1] = calloc((size_t)B->ng[0] * B->ng[2] * 2, sizeof(double));
    B->rhsp[2] = calloc((size_t)B->ng[0] * B->ng[1] * 2, sizeof(double));
  }
  /* pressure BC rhs, main.f90:725-731 (dl from the global grid, is_centered = T) */
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    double dl[3][2];
    int cen[3] = {1, 1, 1};
    for (int a = 0; a < 3; a++) {
      double *drc = calloc(B->ng[a] + 2, sizeof(double)), *drf = calloc(B->ng[a] + 2, sizeof(double)),
             *rc = calloc(B->ng[a] + 2, sizeof(double)), *rf = calloc(B->ng[a] + 2, sizeof(double));
      or_initgrid(B->lo[a], B->hi[a], blocks[ib].gt[a], blocks[ib].gr[a], blocks[ib].lmin[a], blocks[ib].lmax[a], drc, drf, rc, rf);
      if (blocks[ib].grid_file[a]) load_grid(B->lo[a], B->hi[a], blocks[ib].grid_file[a], rf, rc, drf, drc);
      dl[a][0] = drc[0];
      dl[a][1] = drc[B->ng[a]];
      free(drc); free(drf); free(rc); free(rf);
    }
    or_init_bc_rhs(blocks[ib].cbcpre, blocks[ib].bcpre, (const double(*)[2])dl, (const int(*)[2])B->is_bound, cen,
                   B->lo, B->hi, d->periods, B->g[0][0], B->g[0][1], B->g[1][0], B->g[1][1], B->g[2][0], B->g[2][1],
                   B->rhsp[0], B->rhsp[1], B->rhsp[2], NULL, NULL, NULL, c->fft_axis);
    if (ib == 0) {
      d->fft_axis = c->fft_axis;
      if (c->fft_axis) {
        int idir = c->fft_axis - 1;
        d->il = idir == 0 ? 1 : 0;
        d->iu = idir == 2 ? 1 : 2;
        int n = B->ng[idir];
        double norm[2];
        or_find_fft(blocks[0].cbcpre[idir], 1, &d->kind_fwd, &d->kind_bwd, norm);
        if (d->kind_fwd < 0) { snprintf(err, errlen, "unsupported boundary pair along the transform direction"); goto fail; }
        d->normfft = 1.0 / (norm[0] * (n + norm[1] - 0));
        d->lambda = calloc(n, sizeof(double));
        if (or_eigenvalues(n, blocks[0].cbcpre[idir], 1, d->lambda)) { snprintf(err, errlen, "no eigenvalues for this boundary pair"); goto fail; }
        for (int l = 0; l < n; l++) d->lambda[l] = d->lambda[l] / (dl[idir][0] * dl[idir][0]);
      }
    }
  }
  {
    d->ps = or_poisson_create(d, OR_HF_P, 0.0, d->lambda, err, errlen);
    if (!d->ps) goto fail;
    long nbox = d->ps->L[0].ncell * d->ps->nsys;
    d->box_b = calloc(nbox, sizeof(double));
    d->box_x = calloc(nbox, sizeof(double));
  }
  /* inflow BCs (main.f90:592-632 with init_inflow, initflow.f90:369-429); chk_inflow (sanity.f90:173-189) */
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    for (int a = 0; a < 3; a++)
      for (int s = 0; s < 2; s++) {
        const int type = blocks[ib].inflow_type[a][s];
        if (type < 0 || type > 2) { snprintf(err, errlen, "block %d: inflow_type must be 0, 1 or 2", ib + 1); goto fail; }
        if (type > 0 && d->periods[a] != 0) {
          snprintf(err, errlen, "block %d: periodicity and inflow BCs cannot be combined", ib + 1);
          goto fail;
        }
        B->inflow[a][s] = B->is_bound[a][s] && type > 0 && blocks[ib].cbcvel[a][a][s] == 'D';
        if (!B->inflow[a][s]) continue;
        const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
        const int n1 = B->ng[t1] + 2, n2 = B->ng[t2] + 2;
        for (int comp = 0; comp < 3; comp++) B->vin[a][s][comp] = calloc((size_t)n1 * n2, sizeof(double));
        double *veln = B->vin[a][s][a], *velt2 = B->vin[a][s][t2];
        const double uref = blocks[ib].bcvel[a][a][s], lref = 1.0, visc = 1.0 / c->visci;
        const double *x1c = B->g[t1][OR_G_XC], *x2c = B->g[t2][OR_G_XC], *x2f = B->g[t2][OR_G_XF];
        const double pi = acos(-1.0);
        if (type == 1) {
          const int q1 = d->periods[t1] == 0, q2 = d->periods[t2] == 0;
          const double l10 = blocks[ib].lmin[t1], l11 = blocks[ib].lmax[t1];
          const double l20 = blocks[ib].lmin[t2], l21 = blocks[ib].lmax[t2];
          for (int i2 = 0; i2 < n2; i2++)
            for (int i1 = 0; i1 < n1; i1++) {
              /* poiseuille_square (initflow.f90:353-367) raised to q = 0 (periodic) or 1 */
              const double r1 = (x1c[i1] - l10) / (l11 - l10), r2 = (x2c[i2] - l20) / (l21 - l20);
              const double p1 = q1 ? 6.0 * (r1 * (1.0 - r1)) : 1.0, p2 = q2 ? 6.0 * (r2 * (1.0 - r2)) : 1.0;
              veln[i1 + (size_t)n1 * i2] = uref * p1 * p2;
            }
        } else {
          const double reb = uref * lref / visc;
          const double lambda = reb / 2.0 - sqrt(reb * reb / 4.0 + 4.0 * (pi * pi));
          const double x0 = -0.5;
          for (int i2 = 0; i2 < n2; i2++)
            for (int i1 = 0; i1 < n1; i1++) {
              veln[i1 + (size_t)n1 * i2] = 1.0 - exp(lambda * x0) * cos(2.0 * pi * x2c[i2]);
              velt2[i1 + (size_t)n1 * i2] = lambda / (2.0 * pi) * exp(lambda * x0) * sin(2.0 * pi * x2f[i2]);
            }
        }
      }
  }
  /* IMPDIFF (main.f90:771-839): BC planes and a Helmholtz problem for u, v, w and every scalar */
  if (c->impdiff) {
    for (int hf = OR_HF_U; hf < OR_HF_S0 + c->nscal; hf++) {
      double dl_fft = 0.0; /* dl(0, idir) of the field (main.f90:771-773, 781) */
      for (int ib = 0; ib < d->nblocks; ib++) {
        or_block *B = &d->b[ib];
        double dl[3][2];
        int cen[3], hif[3];
        char cb[3][2];
        double bv[3][2];
        for (int a = 0; a < 3; a++) {
          cen[a] = or_field_centered(hf, a);
          hif[a] = or_field_hi(B, hf, a);
          for (int sd = 0; sd < 2; sd++) { cb[a][sd] = or_field_cbc(B, hf, a, sd); bv[a][sd] = or_field_bc(B, hf, a, sd); }
          /* dl of main.f90:771-773 (dxf at lo and hi along a staggered axis, dxc at lo-1 and hi otherwise),
             from the block's own grid */
          double *drc = calloc(B->ng[a] + 2, sizeof(double)), *drf = calloc(B->ng[a] + 2, sizeof(double)),
                 *rc = calloc(B->ng[a] + 2, sizeof(double)), *rf = calloc(B->ng[a] + 2, sizeof(double));
          or_initgrid(B->lo[a], B->hi[a], blocks[ib].gt[a], blocks[ib].gr[a], blocks[ib].lmin[a], blocks[ib].lmax[a], drc, drf, rc, rf);
          if (blocks[ib].grid_file[a]) load_grid(B->lo[a], B->hi[a], blocks[ib].grid_file[a], rf, rc, drf, drc);
          dl[a][0] = cen[a] ? drc[0] : drf[1];
          dl[a][1] = cen[a] ? drc[B->ng[a]] : drf[B->ng[a]];
          if (c->fft_axis && a == c->fft_axis - 1 && ib == 0) dl_fft = dl[a][0];
          free(drc); free(drf); free(rc); free(rf);
        }
        const int nf[3] = {hif[0] - B->lo[0] + 1, hif[1] - B->lo[1] + 1, hif[2] - B->lo[2] + 1};
        B->rhsh[hf][0] = calloc((size_t)nf[1] * nf[2] * 2, sizeof(double));
        B->rhsh[hf][1] = calloc((size_t)nf[0] * nf[2] * 2, sizeof(double));
        B->rhsh[hf][2] = calloc((size_t)nf[0] * nf[1] * 2, sizeof(double));
        const double *d1[3], *d2[3];
        for (int a = 0; a < 3; a++) { d1[a] = cen[a] ? B->g[a][0] : B->g[a][1]; d2[a] = cen[a] ? B->g[a][1] : B->g[a][0]; }
        /* the velocity components pass bcu%x.. (main.f90:580-582, 605-625): bcvel over each plane, or
           the interior of the inflow plane on an inflow face */
        double *bcp[3] = {NULL, NULL, NULL};
        if (hf < OR_HF_S0) {
          for (int a = 0; a < 3; a++) {
            const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
            const int m1 = nf[t1], m2 = nf[t2];
            const size_t np = (size_t)m1 * m2;
            bcp[a] = malloc(np * 2 * sizeof(double));
            for (int sd = 0; sd < 2; sd++)
              for (int i2 = 0; i2 < m2; i2++)
                for (int i1 = 0; i1 < m1; i1++)
                  bcp[a][i1 + (size_t)m1 * i2 + np * sd] =
                      B->inflow[a][sd] ? B->vin[a][sd][hf - OR_HF_U][(i1 + 1) + (size_t)(B->ng[t1] + 2) * (i2 + 1)]
                                       : bv[a][sd];
          }
        }
        or_init_bc_rhs((const char(*)[2])cb, (const double(*)[2])bv, (const double(*)[2])dl, (const int(*)[2])B->is_bound,
                       cen, B->lo, hif, d->periods, d1[0], d2[0], d1[1], d2[1], d1[2], d2[2], B->rhsh[hf][0],
                       B->rhsh[hf][1], B->rhsh[hf][2], bcp[0], bcp[1], bcp[2], c->fft_axis);
        for (int a = 0; a < 3; a++) free(bcp[a]);
      }
      double *lam = NULL;
      int kf = -1, kb = -1, nfft = 0;
      double normfft = 1.0;
      if (c->fft_axis) {
        /* init_fft_reduction (solver.f90:1124-1138) with the field's boundary pair and centring along
           the transform axis; fftini drops the last point (q = 1) of a staggered non-periodic axis */
        const int pf = c->fft_axis - 1, cen_f = or_field_centered(hf, pf);
        const or_block *B0 = &d->b[0];
        const char bc2[2] = {or_field_cbc(B0, hf, pf, 0), or_field_cbc(B0, hf, pf, 1)};
        const int n_full = B0->ng[pf], q = (bc2[0] == 'F' && bc2[1] == 'F') || cen_f ? 0 : 1;
        double norm[2];
        or_find_fft(bc2, cen_f, &kf, &kb, norm);
        if (kf < 0) { snprintf(err, errlen, "unsupported boundary pair along the transform direction"); goto fail; }
        nfft = n_full - q;
        normfft = 1.0 / (norm[0] * (n_full + norm[1] - q));
        lam = calloc(n_full, sizeof(double));
        if (or_eigenvalues(n_full, bc2, cen_f, lam)) {
          free(lam);
          snprintf(err, errlen, "no eigenvalues for this boundary pair (the reference defines none)");
          goto fail;
        }
        for (int l = 0; l < n_full; l++) lam[l] = lam[l] / (dl_fft * dl_fft);
      }
      d->ph[hf] = or_poisson_create(d, hf, 0.0, lam, err, errlen);
      if (!d->ph[hf]) { free(lam); goto fail; }
      d->ph[hf]->lam = lam;
      d->ph[hf]->kind_fwd = kf;
      d->ph[hf]->kind_bwd = kb;
      d->ph[hf]->nfft = nfft;
      d->ph[hf]->normfft = normfft;
      long nbox = d->ph[hf]->L[0].ncell * d->ph[hf]->nsys;
      d->hbox_b[hf] = calloc(nbox, sizeof(double));
      d->hbox_x[hf] = calloc(nbox, sizeof(double));
    }
  }
  d->dt = 0.0;
  free(lo);
  return d;
fail:
  free(lo);
  or_destroy(d);
  return NULL;
}

void or_destroy(or_domain *d) {
  if (!d) return;
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    for (int a = 0; a < 3; a++) for (int w = 0; w < 4; w++) free(B->g[a][w]);
    for (int f = 0; f < OR_NFIELDS; f++) free(B->fld[f]);
    for (int a = 0; a < 3; a++) free(B->rhsp[a]);
    for (int hf = 0; hf < 3 + OR_MAX_SCAL; hf++) for (int a = 0; a < 3; a++) free(B->rhsh[hf][a]);
    for (int a = 0; a < 3; a++) for (int s = 0; s < 2; s++) for (int q = 0; q < 3; q++) free(B->vin[a][s][q]);
  }
  free(d->b);
  free(d->lambda);
  or_poisson_destroy(d->ps);
  free(d->box_b); free(d->box_x);
  for (int hf = 0; hf < 3 + OR_MAX_SCAL; hf++) { or_poisson_destroy(d->ph[hf]); free(d->hbox_b[hf]); free(d->hbox_x[hf]); }
  free(d);
}

int or_block_geometry(const or_domain *d, int ib, int lo[3], int hi[3], int nb[3][2], int is_bound[3][2]) {
  if (ib < 0 || ib >= d->nblocks) return -1;
  const or_block *B = &d->b[ib];
  for (int a = 0; a < 3; a++) {
    lo[a] = B->lo[a]; hi[a] = B->hi[a];
    for (int s = 0; s < 2; s++) { nb[a][s] = B->nb[a][s]; is_bound[a][s] = B->is_bound[a][s]; }
  }
  return 0;
}
double *or_field(or_domain *d, int ib, int kind) { return (ib >= 0 && ib < d->nblocks && kind >= 0 && kind < OR_NFIELDS) ? d->b[ib].fld[kind] : NULL; }
double *or_grid(or_domain *d, int ib, int axis, int which) { return d->b[ib].g[axis][which]; }
double or_vol_all(const or_domain *d) { return d->vol_all; }
double or_dt(const or_domain *d) { return d->dt; }
void or_set_dt(or_domain *d, double dt) { d->dt = dt; }
int or_istep(const or_domain *d) { return d->istep; }
double or_time(const or_domain *d) { return d->time; }
int or_last_iterations(const or_domain *d) { return d->ps ? d->ps->last_iter : 0; }
double or_last_residual(const or_domain *d) { return d->ps ? d->ps->last_res : 0.0; }

/* ---- halo exchange: the MPI_SENDRECV pairs of bound.f90:587-650 as copies ---- */
static void exchange_dir(or_domain *d, int kind, int a) {
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    long st[3] = {1, B->ng[0] + 2, (long)(B->ng[0] + 2) * (B->ng[1] + 2)};
    int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
    for (int s = 0; s < 2; s++) {
      int f = B->nb[a][s];
      if (f < 0) continue;
      or_block *N = &d->b[f];
      long sn[3] = {1, N->ng[0] + 2, (long)(N->ng[0] + 2) * (N->ng[1] + 2)};
      int dst = s ? B->ng[a] + 1 : 0;  /* ghost plane hi+1 (s=1) or lo-1 (s=0) */
      int src = s ? 1 : N->ng[a];      /* friend's plane lo (s=1) or hi (s=0) */
      for (int y = 0; y < B->ng[t2] + 2; y++)
        for (int x = 0; x < B->ng[t1] + 2; x++)
          B->fld[kind][dst * st[a] + x * st[t1] + y * st[t2]] = N->fld[kind][src * sn[a] + x * sn[t1] + y * sn[t2]];
    }
  }
}

/* bound.f90:8-66 */
void or_bounduvw(or_domain *d, int is_correc) {
  for (int comp = 0; comp < 3; comp++)
    for (int a = 0; a < 3; a++) exchange_dir(d, OR_U + comp, a);
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    for (int a = 0; a < 3; a++)
      for (int s = 0; s < 2; s++) {
        if (!B->is_bound[a][s]) continue;
        for (int comp = 0; comp < 3; comp++) {
          int centered = comp != a;
          if (!centered && is_correc) continue;
          const double *dr = centered ? B->g[a][OR_G_DXC] : B->g[a][OR_G_DXF];
          double drv = s ? dr[B->ng[a]] : dr[0];
          or_set_bc(B->desc.cbcvel[comp][a][s], s, B->lo, B->hi, a + 1, centered, B->desc.bcvel[comp][a][s], drv,
                    B->fld[OR_U + comp]);
        }
      }
  }
}

/* bound.f90:438-477 on every block, faces x0, x1, y0, y1, z0, z1; local indices 1..n, halo 0 and n+1 */
void or_inflow(or_domain *d, int is_correc) {
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    const int nx = B->ng[0], ny = B->ng[1];
    for (int a = 0; a < 3; a++)
      for (int s = 0; s < 2; s++) {
        if (!B->inflow[a][s]) continue;
        const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
        const int n1 = B->ng[t1] + 2, n2 = B->ng[t2] + 2;
        const int qn = s ? B->ng[a] : 0, qt = s ? B->ng[a] + 1 : 0, dq = s ? -1 : 1;
        for (int comp = 0; comp < 3; comp++) {
          if (comp == a && is_correc) continue;
          double *f = B->fld[OR_U + comp];
          const double *in = B->vin[a][s][comp];
          for (int i2 = 0; i2 < n2; i2++)
            for (int i1 = 0; i1 < n1; i1++) {
              int c[3];
              c[t1] = i1; c[t2] = i2;
              const double vin = in[i1 + (size_t)n1 * i2];
#define FI(p) f[(p)[0] + (size_t)(nx + 2) * ((p)[1] + (size_t)(ny + 2) * (p)[2])]
              if (comp == a) { c[a] = qn; FI(c) = vin; }
              else {
                c[a] = qt + dq;
                const double inner = FI(c);
                c[a] = qt;
                FI(c) = -inner + 2.0 * vin;
              }
#undef FI
            }
        }
      }
  }
}

/* load_one (load.f90:92-160): the interior of one field in Fortran order, then [time, istep] */
static void ckpt_name(char *buf, size_t len, const char *prefix, int ib, int kind) {
  if (kind >= OR_S0 && kind <= OR_S3) snprintf(buf, len, "%s_b_%03d_s_%03d.bin", prefix, ib + 1, kind - OR_S0 + 1);
  else snprintf(buf, len, "%s_b_%03d_%c.bin", prefix, ib + 1, "uvwp"[kind - OR_U]);
}

int or_checkpoint_save(or_domain *d, const char *prefix) {
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    const int nx = B->ng[0], ny = B->ng[1], nz = B->ng[2];
    double *out = malloc(sizeof(double) * ((size_t)nx * ny * nz + 2));
    for (int f = 0; f < 4 + d->c.nscal; f++) {
      const int kind = f < 4 ? OR_U + f : OR_S0 + (f - 4);
      const double *fl = B->fld[kind];
      size_t q = 0;
      for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
          for (int i = 1; i <= nx; i++) out[q++] = fl[i + (size_t)(nx + 2) * (j + (size_t)(ny + 2) * k)];
      out[q++] = d->time;
      out[q++] = 1.0 * d->istep;
      char name[4096];
      ckpt_name(name, sizeof(name), prefix, ib, kind);
      FILE *fp = fopen(name, "wb");
      if (!fp) { free(out); return -1; }
      const size_t nw = fwrite(out, sizeof(double), q, fp);
      if (fclose(fp) != 0 || nw != q) { free(out); return -1; }
    }
    free(out);
  }
  return 0;
}

int or_checkpoint_load(or_domain *d, const char *prefix) {
  double info[2] = {0.0, 0.0};
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    const int nx = B->ng[0], ny = B->ng[1], nz = B->ng[2];
    const size_t n = (size_t)nx * ny * nz + 2;
    double *in = malloc(sizeof(double) * n);
    for (int f = 0; f < 4 + d->c.nscal; f++) {
      const int kind = f < 4 ? OR_U + f : OR_S0 + (f - 4);
      char name[4096];
      ckpt_name(name, sizeof(name), prefix, ib, kind);
      FILE *fp = fopen(name, "rb");
      if (!fp) { free(in); return -1; }
      fseek(fp, 0, SEEK_END);
      const long size = ftell(fp);
      fseek(fp, 0, SEEK_SET);
      if (size < 0 || (size_t)size != n * sizeof(double)) { fclose(fp); free(in); return -2; }
      const size_t nr = fread(in, sizeof(double), n, fp);
      fclose(fp);
      if (nr != n) { free(in); return -1; }
      double *fl = B->fld[kind];
      size_t q = 0;
      for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
          for (int i = 1; i <= nx; i++) fl[i + (size_t)(nx + 2) * (j + (size_t)(ny + 2) * k)] = in[q++];
      info[0] = in[q];
      info[1] = in[q + 1];
    }
    free(in);
  }
  d->time = info[0];
  d->istep = (int)lround(info[1]);
  return 0;
}

/* Fortran's E15.7 edit descriptor: 0.ddddddd with 7 significant digits (correctly rounded, as printf's
   %.6e), then E+ee, or +eee beyond two exponent digits, right-justified in 15 columns */
void or_fortran_e15_7(double v, char *out) {
  char mant[40], expo[24], body[96];
  int e10 = 0;
  const int neg = signbit(v) && v != 0.0;
  if (v == 0.0) snprintf(mant, sizeof(mant), "0.0000000");
  else {
    char buf[40];
    snprintf(buf, sizeof(buf), "%.6e", fabs(v));
    e10 = atoi(buf + 9) + 1;
    snprintf(mant, sizeof(mant), "0.%c%.6s", buf[0], buf + 2);
  }
  if (e10 >= -99 && e10 <= 99) snprintf(expo, sizeof(expo), "E%c%02d", e10 < 0 ? '-' : '+', abs(e10));
  else snprintf(expo, sizeof(expo), "%c%03d", e10 < 0 ? '-' : '+', abs(e10));
  snprintf(body, sizeof(body), "%s%s%s", neg ? "-" : "", mant, expo);
  snprintf(out, 128, "%15s", body);
}

int or_out1d(or_domain *d, int ib, int kind, int idir, double *coord, double *prof, const char *fname) {
  if (ib < 0 || ib >= d->nblocks || idir < 1 || idir > 3) return -1;
  or_block *B = &d->b[ib];
  const int nx = B->ng[0], ny = B->ng[1], nz = B->ng[2];
  const double *f = B->fld[kind];
  /* out1d.h90: u uses dxc,dyf,dzf at xf,yc,zc; v dxf,dyc,dzf at xc,yf,zc; w dxf,dyf,dzc at xc,yc,zf; p dxf.. */
  const double *dl[3], *xg[3];
  double l[3];
  for (int a = 0; a < 3; a++) {
    const int stag = kind >= OR_U && kind <= OR_W && kind - OR_U == a;
    dl[a] = stag ? B->g[a][OR_G_DXC] : B->g[a][OR_G_DXF];
    xg[a] = stag ? B->g[a][OR_G_XF] : B->g[a][OR_G_XC];
    l[a] = B->desc.lmax[a] - B->desc.lmin[a];
  }
#define F(i, j, k) f[(i) + (size_t)(nx + 2) * ((j) + (size_t)(ny + 2) * (k))]
  const int a = idir - 1, n = B->ng[a];
  for (int q = 0; q < n; q++) prof[q] = 0.0;
  if (idir == 3)
    for (int k = 1; k <= nz; k++)
      for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) prof[k - 1] = prof[k - 1] + F(i, j, k) * dl[0][i] * dl[1][j] / (l[0] * l[1]);
  else if (idir == 2)
    for (int j = 1; j <= ny; j++)
      for (int k = 1; k <= nz; k++)
        for (int i = 1; i <= nx; i++) prof[j - 1] = prof[j - 1] + F(i, j, k) * dl[0][i] * dl[2][k] / (l[0] * l[2]);
  else
    for (int i = 1; i <= nx; i++)
      for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++) prof[i - 1] = prof[i - 1] + F(i, j, k) * dl[1][j] * dl[2][k] / (l[1] * l[2]);
#undef F
  for (int q = 0; q < n; q++) coord[q] = xg[a][q + 1];
  if (fname) {
    FILE *fp = fopen(fname, "w");
    if (!fp) return -1;
    char s1[128], s2[128];
    for (int q = 0; q < n; q++) {
      or_fortran_e15_7(coord[q], s1);
      or_fortran_e15_7(prof[q], s2);
      fprintf(fp, "%s%s\n", s1, s2);
    }
    if (fclose(fp) != 0) return -1;
  }
  return 0;
}

void or_time_istep(const or_domain *d, double *time, int *istep) {
  *time = d->time;
  *istep = d->istep;
}

/* bound.f90:68-106; scalars use their own cbc/bc (main.f90:936) */
void or_boundp(or_domain *d, int kind) {
  for (int a = 0; a < 3; a++) exchange_dir(d, kind, a);
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    for (int a = 0; a < 3; a++)
      for (int s = 0; s < 2; s++) {
        if (!B->is_bound[a][s]) continue;
        char cb; double bv;
        if (kind >= OR_S0 && kind <= OR_S3) { cb = B->desc.cbcscal[kind - OR_S0][a][s]; bv = B->desc.bcscal[kind - OR_S0][a][s]; }
        else { cb = B->desc.cbcpre[a][s]; bv = B->desc.bcpre[a][s]; }
        double drv = s ? B->g[a][OR_G_DXC][B->ng[a]] : B->g[a][OR_G_DXC][0];
        or_set_bc(cb, s, B->lo, B->hi, a + 1, 1, bv, drv, B->fld[kind]);
      }
  }
}

static int helm_solve(or_domain *d, int hf, int kind, double alphai);

/* solve_impdiff_field (solve_helmholtz.f90:32-138) of one field of every block: field 0..2 = u, v, w,
 * 3 + s = scalar s; returns non-zero when the solve did not reach the tolerance */
int or_impdiff_solve(or_domain *d, int field, double alphai) {
  if (!d->c.impdiff) return -1;
  if (field < 3) return helm_solve(d, OR_HF_U + field, OR_U + field, alphai);
  return helm_solve(d, OR_HF_S0 + field - 3, OR_S0 + field - 3, alphai);
}

void or_fillps_all(or_domain *d, double dtrk) {
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    or_fillps(B->lo, B->hi, B->g[0][1], B->g[1][1], B->g[2][1], dtrk, B->fld[OR_U], B->fld[OR_V], B->fld[OR_W],
              B->fld[OR_PP], d->fft_axis);
  }
}

void or_updt_rhs_all(or_domain *d) {
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    or_updt_rhs(B->lo, B->hi, (const int(*)[2])B->is_bound, B->rhsp[0], B->rhsp[1], B->rhsp[2], B->fld[OR_PP]);
  }
}

/* transform the interior of pp of every block along the FFT axis (fft.f90:85-94) */
/* fft(plan, arr(lo:hi,...)) on every block: every line of the interior along the transform axis, its first
   nl points (nl = 0: all) */
static void transform_field(or_domain *d, int fkind, int kind, int nl_in) {
  int idir = d->fft_axis - 1;
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    int n[3] = {B->ng[0], B->ng[1], B->ng[2]};
    long st[3] = {1, n[0] + 2, (long)(n[0] + 2) * (n[1] + 2)};
    double *f = B->fld[fkind];
    int t1 = idir == 0 ? 1 : 0, t2 = idir == 2 ? 1 : 2;
    int nl = nl_in > 0 ? nl_in : n[idir];
#pragma omp parallel
    {
      double *in = malloc(sizeof(double) * nl), *out = malloc(sizeof(double) * nl);
#pragma omp for collapse(2)
      for (int y = 1; y <= n[t2]; y++)
        for (int x = 1; x <= n[t1]; x++) {
          long base = x * st[t1] + y * st[t2];
          for (int q = 0; q < nl; q++) in[q] = f[base + (q + 1) * st[idir]];
          or_r2r(kind, nl, in, out);
          for (int q = 0; q < nl; q++) f[base + (q + 1) * st[idir]] = out[q];
        }
      free(in); free(out);
    }
  }
}

/* main.f90:1004-1022: transform, per-wavenumber (or 3-D) solves warm-started from po, back-transform + normfft */
int or_solve_pressure(or_domain *d) {
  if (d->fft_axis) transform_field(d, OR_PP, d->kind_fwd, 0);
  or_box_gather(d, d->ps, OR_PP, d->box_b);
  int rc = or_poisson_solve(d->ps, d->box_b, d->box_x);
  or_box_scatter(d, d->ps, d->box_x, OR_PP);
  if (d->fft_axis) {
    transform_field(d, OR_PP, d->kind_bwd, 0);
    for (int ib = 0; ib < d->nblocks; ib++) {
      or_block *B = &d->b[ib];
      int nx = B->ng[0], ny = B->ng[1];
      for (int k = 1; k <= B->ng[2]; k++)
        for (int j = 1; j <= ny; j++)
          for (int i = 1; i <= nx; i++) B->fld[OR_PP][i + (long)(nx + 2) * (j + (long)(ny + 2) * k)] *= d->normfft;
    }
  }
  return rc;
}

void or_correc_all(or_domain *d, double dtrk) {
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    or_correc(B->lo, B->hi, B->g[0][0], B->g[1][0], B->g[2][0], dtrk, B->fld[OR_PP], B->fld[OR_U], B->fld[OR_V], B->fld[OR_W]);
  }
}

void or_updt_pressure_all(or_domain *d, double alpha) {
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    or_updt_pressure(B->lo, B->hi, B->g[0][0], B->g[0][1], B->g[1][0], B->g[1][1], B->g[2][0], B->g[2][1], alpha,
                     B->fld[OR_PP], B->fld[OR_P], d->c.impdiff);
  }
}

/* chkdt.f90:8-56 with the MPI reductions over blocks; max(visc, alpha_max) as main.f90:660 */
double or_chkdt(or_domain *d) {
  double dti = 0.0, dlmin = 1e300;
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    double t, m;
    or_chkdt_local(B->lo, B->hi, B->g[0][0], B->g[0][1], B->g[1][0], B->g[1][1], B->g[2][0], B->g[2][1],
                   B->fld[OR_U], B->fld[OR_V], B->fld[OR_W], &t, &m);
    if (t > dti) dti = t;
    if (m < dlmin) dlmin = m;
  }
  if (dti == 0.0) dti = 1.0;
  double dtmax = sqrt(3.0) / dti;
  if (!d->c.impdiff) {
    double visc = 1.0 / d->c.visci, amax = 0.0;
    for (int s = 0; s < d->c.nscal; s++) { double a = 1.0 / d->c.alphai[s]; if (a > amax) amax = a; }
    double ve = visc > amax ? visc : amax;
    double lim = 1.65 / 12.0 / ve * (dlmin * dlmin);
    if (lim < dtmax) dtmax = lim;
  }
  return dtmax;
}

void or_chkdiv(or_domain *d, double *divtot, double *divmax) {
  double tot = 0.0, mx = 0.0;
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    double t, m;
    or_chkdiv_local(B->lo, B->hi, B->g[0][1], B->g[1][1], B->g[2][1], B->fld[OR_U], B->fld[OR_V], B->fld[OR_W],
                    d->vol_all, &t, &m);
    tot += t;
    if (m > mx) mx = m;
  }
  *divtot = tot;
  *divmax = mx;
}

/* kinetic energy 0.5*sum(u^2 dxc dyf dzf + v^2 dxf dyc dzf + w^2 dxf dyf dzc)/vol over interior faces */
double or_kinetic_energy(or_domain *d) {
  double ke = 0.0;
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    int nx = B->ng[0], ny = B->ng[1];
    double *dxc = B->g[0][0], *dxf = B->g[0][1], *dyc = B->g[1][0], *dyf = B->g[1][1], *dzc = B->g[2][0], *dzf = B->g[2][1];
    for (int k = 1; k <= B->ng[2]; k++)
      for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
          long c = i + (long)(nx + 2) * (j + (long)(ny + 2) * k);
          double u = B->fld[OR_U][c], v = B->fld[OR_V][c], w = B->fld[OR_W][c];
          ke += u * u * dxc[i] * dyf[j] * dzf[k] + v * v * dxf[i] * dyc[j] * dzf[k] + w * w * dxf[i] * dyf[j] * dzc[k];
        }
  }
  return 0.5 * ke / d->vol_all;
}

static void set_dt_from_cfl(or_domain *d) {
  double dt_cfl = or_chkdt(d);
  d->dt = d->c.dt_f > 0.0 ? d->c.dt_f : (d->c.cfl * dt_cfl < d->c.dtmax ? d->c.cfl * dt_cfl : d->c.dtmax);
}

/* solve_impdiff_field_3d (solve_helmholtz.f90:109-138): phi <- alphai * phi * dx2 dy2 dz2 (the field's
 * control volume), the BC planes added at the boundary cells (updt_rhs over lo..hif), then
 * (A + alphai V) phi = rhs warm-started from the previous solution (phio) */
static int helm_solve(or_domain *d, int hf, int kind, double alphai) {
  or_poisson *P = d->ph[hf];
  const int pf = d->fft_axis - 1; /* solve_impdiff_field_fft: no weight along the transform axis */
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    int hif[3], cen[3];
    const double *d2[3];
    for (int a = 0; a < 3; a++) {
      hif[a] = or_field_hi(B, hf, a);
      cen[a] = or_field_centered(hf, a);
      d2[a] = cen[a] ? B->g[a][1] : B->g[a][0];
    }
    const int nx = B->ng[0], ny = B->ng[1];
    const int nf[3] = {hif[0] - B->lo[0] + 1, hif[1] - B->lo[1] + 1, hif[2] - B->lo[2] + 1};
    double *f = B->fld[kind];
#define FI(i, j, k) f[(i) + (size_t)(nx + 2) * ((j) + (size_t)(ny + 2) * (k))]
    /* solve_helmholtz.f90:123-129 scales over lo..hi, including a wall face that the solve leaves alone */
    for (int k = 1; k <= B->ng[2]; k++)
      for (int j = 1; j <= B->ng[1]; j++)
        for (int i = 1; i <= B->ng[0]; i++) {
          double v = FI(i, j, k) * alphai;
          if (pf != 0) v = v * d2[0][i];
          if (pf != 1) v = v * d2[1][j];
          if (pf != 2) v = v * d2[2][k];
          FI(i, j, k) = v;
        }
    const double *rx = B->rhsh[hf][0], *ry = B->rhsh[hf][1], *rz = B->rhsh[hf][2];
    /* bound.f90:543-585 with hi = hif, in its order x0, x1, y0, y1, z0, z1 (an edge cell takes two planes) */
    for (int sd = 0; sd < 2; sd++)
      if (B->is_bound[0][sd])
        for (int k = 1; k <= nf[2]; k++)
          for (int j = 1; j <= nf[1]; j++) FI(sd ? nf[0] : 1, j, k) += rx[(j - 1) + (size_t)nf[1] * ((k - 1) + (size_t)nf[2] * sd)];
    for (int sd = 0; sd < 2; sd++)
      if (B->is_bound[1][sd])
        for (int k = 1; k <= nf[2]; k++)
          for (int i = 1; i <= nf[0]; i++) FI(i, sd ? nf[1] : 1, k) += ry[(i - 1) + (size_t)nf[0] * ((k - 1) + (size_t)nf[2] * sd)];
    for (int sd = 0; sd < 2; sd++)
      if (B->is_bound[2][sd])
        for (int j = 1; j <= nf[1]; j++)
          for (int i = 1; i <= nf[0]; i++) FI(i, j, sd ? nf[2] : 1) += rz[(i - 1) + (size_t)nf[0] * ((j - 1) + (size_t)nf[1] * sd)];
#undef FI
  }
  if (pf < 0) {
    P->shift[0] = alphai;
    or_box_gather(d, P, kind, d->hbox_b[hf]);
    int rc = or_poisson_solve(P, d->hbox_b[hf], d->hbox_x[hf]);
    or_box_scatter(d, P, d->hbox_x[hf], kind);
    return rc;
  }
  /* transform, per-wavenumber solves of (A + (lambda_k + alphai) w) x = rhs, back-transform, normfft over
     the whole interior (solve_helmholtz.f90:86-101) */
  for (int s = 0; s < P->nsys; s++) P->shift[s] = P->lam[s] + alphai;
  transform_field(d, kind, P->kind_fwd, P->nfft);
  or_box_gather(d, P, kind, d->hbox_b[hf]);
  int rc = or_poisson_solve(P, d->hbox_b[hf], d->hbox_x[hf]);
  or_box_scatter(d, P, d->hbox_x[hf], kind);
  transform_field(d, kind, P->kind_bwd, P->nfft);
  for (int ib = 0; ib < d->nblocks; ib++) {
    or_block *B = &d->b[ib];
    const int nx = B->ng[0], ny = B->ng[1];
    for (int k = 1; k <= B->ng[2]; k++)
      for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) B->fld[kind][i + (long)(nx + 2) * (j + (long)(ny + 2) * k)] *= P->normfft;
  }
  return rc;
}

/* main.f90:907-936 for the explicit-diffusion path: rk_scal on every block, the bulk mean summed over
 * blocks as the MPI_ALLREDUCE of scal.f90:175 sums it over ranks, bulk_forcing_s, boundp of the scalar */
static int scalar_stage(or_domain *d, int irk) {
  int rc = 0;
  for (int s = 0; s < d->c.nscal; s++) {
    const int forced = d->c.is_sforced[s];
    double msum = 0.0;
    for (int ib = 0; ib < d->nblocks; ib++) {
      or_block *B = &d->b[ib];
      double fb = 0.0;
      or_rk_scal(RKC[irk], B->lo, B->hi, B->g[0][0], B->g[0][1], B->g[1][0], B->g[1][1], B->g[2][0], B->g[2][1],
                 d->dt, 1.0 / d->c.alphai[s], d->vol_all, B->fld[OR_U], B->fld[OR_V], B->fld[OR_W], forced,
                 d->c.scalf[s], d->c.ssource[s], B->fld[OR_DSDTRKO0 + s], B->fld[OR_S0 + s], &fb, d->c.impdiff);
      if (forced) msum += d->c.scalf[s] - fb; /* this block's share of the bulk mean */
    }
    const double f = forced ? d->c.scalf[s] - msum : 0.0;
    for (int ib = 0; ib < d->nblocks; ib++) {
      or_block *B = &d->b[ib];
      or_bulk_forcing_s(B->lo, B->hi, forced, f, B->fld[OR_S0 + s]);
    }
    if (d->c.impdiff) { /* main.f90:914-934: alpha = -s%alpha*dtrk/2 */
      const double dtrk = (RKC[irk][0] + RKC[irk][1]) * d->dt;
      const double alpha = -(1.0 / d->c.alphai[s]) * dtrk / 2.0;
      rc |= helm_solve(d, OR_HF_S0 + s, OR_S0 + s, 1.0 / alpha);
    }
    or_boundp(d, OR_S0 + s);
  }
  return rc;
}

/* main.f90:893-1069 with scalars, Boussinesq buoyancy and IMPDIFF (3-D solves) */
int or_step(or_domain *d, int nsteps) {

  if (d->dt == 0.0) set_dt_from_cfl(d);          /* main.f90:660-661 */
  double visc = 1.0 / d->c.visci;
  int rc = 0;
  for (int st = 0; st < nsteps; st++) {
    d->istep++;
    d->time += d->dt;
    for (int irk = 0; irk < 3; irk++) {
      double dtrk = (RKC[irk][0] + RKC[irk][1]) * d->dt;
      double alpha = -visc * dtrk / 2.0;
      rc |= scalar_stage(d, irk);
      const int bq = d->c.boussinesq && d->c.nscal > 0;
      for (int ib = 0; ib < d->nblocks; ib++) {
        or_block *B = &d->b[ib];
        or_rk_mom(RKC[irk], B->lo, B->hi, B->g[0][0], B->g[0][1], B->g[1][0], B->g[1][1], B->g[2][0], B->g[2][1],
                  d->dt, d->c.bforce, d->c.gacc, d->c.beta, bq ? B->fld[OR_S0] : NULL, visc, B->fld[OR_U],
                  B->fld[OR_V], B->fld[OR_W], B->fld[OR_P], B->fld[OR_DUDTRKO], B->fld[OR_DVDTRKO],
                  B->fld[OR_DWDTRKO], d->c.impdiff, bq);
      }
      if (d->c.impdiff) /* main.f90:947-995: the three Helmholtz solves of u, v, w with alphai = 1/alpha */
        for (int comp = 0; comp < 3; comp++) rc |= helm_solve(d, OR_HF_U + comp, OR_U + comp, 1.0 / alpha);
      or_bounduvw(d, 0);
      or_inflow(d, 0);
      or_fillps_all(d, dtrk);
      or_updt_rhs_all(d);
      rc |= or_solve_pressure(d);
      or_boundp(d, OR_PP);
      or_correc_all(d, dtrk);
      or_bounduvw(d, 1);
      or_inflow(d, 1);
      or_updt_pressure_all(d, alpha);
      or_boundp(d, OR_P);
    }
    if (d->c.icheck > 0 && d->istep % d->c.icheck == 0) set_dt_from_cfl(d); /* main.f90:1048-1053 */
  }
  return rc;
}
