/*
 * or_stencil.c -- oracle restatement of the per-cell hot-path routines.
 * TEST INFRASTRUCTURE ONLY (see snac_oracle.h).
 *
 * Each function keeps the reference's loop structure and the Fortran
 * left-to-right evaluation order of every expression, so that with
 * -ffp-contract=off the results are rounding-identical to a gfortran build
 * without FMA contraction.
 */
#include "snac_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NX (hi[0] - lo[0] + 1)
#define NY (hi[1] - lo[1] + 1)
#define NZ (hi[2] - lo[2] + 1)
/* halo'd field f(lo-1:hi+1,...) */
#define F(a, i, j, k) (a)[((i) - lo[0] + 1) + (size_t)(NX + 2) * (((j) - lo[1] + 1) + (size_t)(NY + 2) * ((k) - lo[2] + 1))]
/* interior array d(lo:hi,...) */
#define D(a, i, j, k) (a)[((i) - lo[0]) + (size_t)NX * (((j) - lo[1]) + (size_t)NY * ((k) - lo[2]))]
/* 1-D metrics dxc(lo-1:hi+1) */
#define MX(a, i) (a)[(i) - lo[0] + 1]
#define MY(a, j) (a)[(j) - lo[1] + 1]
#define MZ(a, k) (a)[(k) - lo[2] + 1]

/* mom.f90:221-327 (momx_d/momy_d/momz_d), accumulating into dudt */
static void mom_d(const int lo[3], const int hi[3], const double *dxc, const double *dxf,
                  const double *dyc, const double *dyf, const double *dzc, const double *dzf,
                  double visc, const double *u, const double *v, const double *w,
                  double *dudt, double *dvdt, double *dwdt) {
#pragma omp parallel for
  for (int k = lo[2]; k <= hi[2]; k++)
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) {
        /* momx_d mom.f90:444-456 */
        double dudxp = (F(u, i + 1, j, k) - F(u, i, j, k)) / MX(dxf, i + 1);
        double dudxm = (F(u, i, j, k) - F(u, i - 1, j, k)) / MX(dxf, i);
        double dudyp = (F(u, i, j + 1, k) - F(u, i, j, k)) / MY(dyc, j);
        double dudym = (F(u, i, j, k) - F(u, i, j - 1, k)) / MY(dyc, j - 1);
        double dudzp = (F(u, i, j, k + 1) - F(u, i, j, k)) / MZ(dzc, k);
        double dudzm = (F(u, i, j, k) - F(u, i, j, k - 1)) / MZ(dzc, k - 1);
        D(dudt, i, j, k) = D(dudt, i, j, k) + visc * (dudxp - dudxm) / MX(dxc, i) +
                           visc * (dudyp - dudym) / MY(dyf, j) + visc * (dudzp - dudzm) / MZ(dzf, k);
        /* momy_d mom.f90:480-492 */
        double dvdxp = (F(v, i + 1, j, k) - F(v, i, j, k)) / MX(dxc, i);
        double dvdxm = (F(v, i, j, k) - F(v, i - 1, j, k)) / MX(dxc, i - 1);
        double dvdyp = (F(v, i, j + 1, k) - F(v, i, j, k)) / MY(dyf, j + 1);
        double dvdym = (F(v, i, j, k) - F(v, i, j - 1, k)) / MY(dyf, j);
        double dvdzp = (F(v, i, j, k + 1) - F(v, i, j, k)) / MZ(dzc, k);
        double dvdzm = (F(v, i, j, k) - F(v, i, j, k - 1)) / MZ(dzc, k - 1);
        D(dvdt, i, j, k) = D(dvdt, i, j, k) + visc * (dvdxp - dvdxm) / MX(dxf, i) +
                           visc * (dvdyp - dvdym) / MY(dyc, j) + visc * (dvdzp - dvdzm) / MZ(dzf, k);
        /* momz_d mom.f90:516-528 */
        double dwdxp = (F(w, i + 1, j, k) - F(w, i, j, k)) / MX(dxc, i);
        double dwdxm = (F(w, i, j, k) - F(w, i - 1, j, k)) / MX(dxc, i - 1);
        double dwdyp = (F(w, i, j + 1, k) - F(w, i, j, k)) / MY(dyc, j);
        double dwdym = (F(w, i, j, k) - F(w, i, j - 1, k)) / MY(dyc, j - 1);
        double dwdzp = (F(w, i, j, k + 1) - F(w, i, j, k)) / MZ(dzf, k + 1);
        double dwdzm = (F(w, i, j, k) - F(w, i, j, k - 1)) / MZ(dzf, k);
        D(dwdt, i, j, k) = D(dwdt, i, j, k) + visc * (dwdxp - dwdxm) / MX(dxf, i) +
                           visc * (dwdyp - dwdym) / MY(dyf, j) + visc * (dwdzp - dwdzm) / MZ(dzc, k);
      }
}

/* mom.f90:112-219 (momx_a_vv/momy_a_vv/momz_a_vv, the variant rk.f90:9-11 aliases) */
static void mom_a_vv(const int lo[3], const int hi[3], const double *dxc, const double *dxf,
                     const double *dyc, const double *dyf, const double *dzc, const double *dzf,
                     const double *u, const double *v, const double *w,
                     double *dudt, double *dvdt, double *dwdt) {
#pragma omp parallel for
  for (int k = lo[2]; k <= hi[2]; k++)
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) {
        /* momx_a_vv mom.f90:129-142 */
        double uuip = 0.25 * (F(u, i, j, k) * MY(dyf, j) * MZ(dzf, k) + F(u, i + 1, j, k) * MY(dyf, j) * MZ(dzf, k)) * F(u, i + 1, j, k);
        double uuim = 0.25 * (F(u, i, j, k) * MY(dyf, j) * MZ(dzf, k) + F(u, i - 1, j, k) * MY(dyf, j) * MZ(dzf, k)) * F(u, i - 1, j, k);
        double uvjp = 0.25 * (F(v, i, j, k) * MX(dxf, i) * MZ(dzf, k) + F(v, i + 1, j, k) * MX(dxf, i + 1) * MZ(dzf, k)) * F(u, i, j + 1, k);
        double uvjm = 0.25 * (F(v, i, j - 1, k) * MX(dxf, i) * MZ(dzf, k) + F(v, i + 1, j - 1, k) * MX(dxf, i + 1) * MZ(dzf, k)) * F(u, i, j - 1, k);
        double uwkp = 0.25 * (F(w, i, j, k) * MX(dxf, i) * MY(dyf, j) + F(w, i + 1, j, k) * MX(dxf, i + 1) * MY(dyf, j)) * F(u, i, j, k + 1);
        double uwkm = 0.25 * (F(w, i, j, k - 1) * MX(dxf, i) * MY(dyf, j) + F(w, i + 1, j, k - 1) * MX(dxf, i + 1) * MY(dyf, j)) * F(u, i, j, k - 1);
        D(dudt, i, j, k) = D(dudt, i, j, k) + ((-uuip + uuim) + (-uvjp + uvjm) + (-uwkp + uwkm)) /
                                                  (MX(dxc, i) * MY(dyf, j) * MZ(dzf, k));
        /* momy_a_vv mom.f90:165-178 */
        double uvip = 0.25 * (F(u, i, j, k) * MY(dyf, j) * MZ(dzf, k) + F(u, i, j + 1, k) * MY(dyf, j + 1) * MZ(dzf, k)) * F(v, i + 1, j, k);
        double uvim = 0.25 * (F(u, i - 1, j, k) * MY(dyf, j) * MZ(dzf, k) + F(u, i - 1, j + 1, k) * MY(dyf, j + 1) * MZ(dzf, k)) * F(v, i - 1, j, k);
        double vvjp = 0.25 * (F(v, i, j, k) * MX(dxf, i) * MZ(dzf, k) + F(v, i, j + 1, k) * MX(dxf, i) * MZ(dzf, k)) * F(v, i, j + 1, k);
        double vvjm = 0.25 * (F(v, i, j, k) * MX(dxf, i) * MZ(dzf, k) + F(v, i, j - 1, k) * MX(dxf, i) * MZ(dzf, k)) * F(v, i, j - 1, k);
        double wvkp = 0.25 * (F(w, i, j, k) * MY(dyf, j) * MX(dxf, i) + F(w, i, j + 1, k) * MY(dyf, j + 1) * MX(dxf, i)) * F(v, i, j, k + 1);
        double wvkm = 0.25 * (F(w, i, j, k - 1) * MY(dyf, j) * MX(dxf, i) + F(w, i, j + 1, k - 1) * MY(dyf, j + 1) * MX(dxf, i)) * F(v, i, j, k - 1);
        D(dvdt, i, j, k) = D(dvdt, i, j, k) + ((-uvip + uvim) + (-vvjp + vvjm) + (-wvkp + wvkm)) /
                                                  (MX(dxf, i) * MY(dyc, j) * MZ(dzf, k));
        /* momz_a_vv mom.f90:202-215 */
        double uwip = 0.25 * (F(u, i, j, k) * MZ(dzf, k) * MY(dyf, j) + F(u, i, j, k + 1) * MZ(dzf, k + 1) * MY(dyf, j)) * F(w, i + 1, j, k);
        double uwim = 0.25 * (F(u, i - 1, j, k) * MZ(dzf, k) * MY(dyf, j) + F(u, i - 1, j, k + 1) * MZ(dzf, k + 1) * MY(dyf, j)) * F(w, i - 1, j, k);
        double vwjp = 0.25 * (F(v, i, j, k) * MZ(dzf, k) * MX(dxf, i) + F(v, i, j, k + 1) * MZ(dzf, k + 1) * MX(dxf, i)) * F(w, i, j + 1, k);
        double vwjm = 0.25 * (F(v, i, j - 1, k) * MZ(dzf, k) * MX(dxf, i) + F(v, i, j - 1, k + 1) * MZ(dzf, k + 1) * MX(dxf, i)) * F(w, i, j - 1, k);
        double wwkp = 0.25 * (F(w, i, j, k) * MX(dxf, i) * MY(dyf, j) + F(w, i, j, k + 1) * MX(dxf, i) * MY(dyf, j)) * F(w, i, j, k + 1);
        double wwkm = 0.25 * (F(w, i, j, k) * MX(dxf, i) * MY(dyf, j) + F(w, i, j, k - 1) * MX(dxf, i) * MY(dyf, j)) * F(w, i, j, k - 1);
        D(dwdt, i, j, k) = D(dwdt, i, j, k) + ((-uwip + uwim) + (-vwjp + vwjm) + (-wwkp + wwkm)) /
                                                  (MX(dxf, i) * MY(dyf, j) * MZ(dzc, k));
      }
}

/* rk.f90:7-128 (rk_mom) with mom.f90:328-386 (momx_p/momy_p/momz_p) */
void or_rk_mom(const double rkpar[2], const int lo[3], const int hi[3],
               const double *dxc, const double *dxf, const double *dyc, const double *dyf,
               const double *dzc, const double *dzf, double dt, const double bforce[3],
               const double gacc[3], double beta, const double *s1, double visc,
               double *u, double *v, double *w, const double *p,
               double *dudtrko, double *dvdtrko, double *dwdtrko,
               int impdiff, int boussinesq) {
  size_t n = (size_t)NX * NY * NZ;
  double factor1 = rkpar[0] * dt, factor2 = rkpar[1] * dt;
  double factor12 = factor1 + factor2;
  double *dudtrk = calloc(n, sizeof(double)), *dvdtrk = calloc(n, sizeof(double)),
         *dwdtrk = calloc(n, sizeof(double));
  double *dudtrkd = NULL, *dvdtrkd = NULL, *dwdtrkd = NULL;
  if (!impdiff) {
    mom_d(lo, hi, dxc, dxf, dyc, dyf, dzc, dzf, visc, u, v, w, dudtrk, dvdtrk, dwdtrk); /* rk.f90:47-49 */
  } else {
    dudtrkd = calloc(n, sizeof(double));
    dvdtrkd = calloc(n, sizeof(double));
    dwdtrkd = calloc(n, sizeof(double));
    mom_d(lo, hi, dxc, dxf, dyc, dyf, dzc, dzf, visc, u, v, w, dudtrkd, dvdtrkd, dwdtrkd); /* rk.f90:56-58 */
  }
  mom_a_vv(lo, hi, dxc, dxf, dyc, dyf, dzc, dzf, u, v, w, dudtrk, dvdtrk, dwdtrk); /* rk.f90:60-62 */
#pragma omp parallel for
  for (int k = lo[2]; k <= hi[2]; k++) /* rk.f90:68-85 */
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) {
        F(u, i, j, k) = F(u, i, j, k) + factor1 * D(dudtrk, i, j, k) + factor2 * D(dudtrko, i, j, k);
        F(v, i, j, k) = F(v, i, j, k) + factor1 * D(dvdtrk, i, j, k) + factor2 * D(dvdtrko, i, j, k);
        F(w, i, j, k) = F(w, i, j, k) + factor1 * D(dwdtrk, i, j, k) + factor2 * D(dwdtrko, i, j, k);
        if (impdiff) {
          F(u, i, j, k) = F(u, i, j, k) + factor12 * D(dudtrkd, i, j, k);
          F(v, i, j, k) = F(v, i, j, k) + factor12 * D(dvdtrkd, i, j, k);
          F(w, i, j, k) = F(w, i, j, k) + factor12 * D(dwdtrkd, i, j, k);
        }
        D(dudtrko, i, j, k) = D(dudtrk, i, j, k);
        D(dvdtrko, i, j, k) = D(dvdtrk, i, j, k);
        D(dwdtrko, i, j, k) = D(dwdtrk, i, j, k);
      }
#pragma omp parallel for
  for (int k = lo[2]; k <= hi[2]; k++) /* rk.f90:91-93 -> mom.f90:544-590 */
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) {
        D(dudtrk, i, j, k) = -(F(p, i + 1, j, k) - F(p, i, j, k)) / MX(dxc, i) + bforce[0];
        D(dvdtrk, i, j, k) = -(F(p, i, j + 1, k) - F(p, i, j, k)) / MY(dyc, j) + bforce[1];
        D(dwdtrk, i, j, k) = -(F(p, i, j, k + 1) - F(p, i, j, k)) / MZ(dzc, k) + bforce[2];
      }
#pragma omp parallel for
  for (int k = lo[2]; k <= hi[2]; k++) /* rk.f90:98-111 */
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) {
        F(u, i, j, k) = F(u, i, j, k) + factor12 * D(dudtrk, i, j, k);
        F(v, i, j, k) = F(v, i, j, k) + factor12 * D(dvdtrk, i, j, k);
        F(w, i, j, k) = F(w, i, j, k) + factor12 * D(dwdtrk, i, j, k);
        if (boussinesq) {
          F(u, i, j, k) = F(u, i, j, k) - factor12 * gacc[0] * beta * 0.5 * (F(s1, i + 1, j, k) + F(s1, i, j, k));
          F(v, i, j, k) = F(v, i, j, k) - factor12 * gacc[1] * beta * 0.5 * (F(s1, i, j + 1, k) + F(s1, i, j, k));
          F(w, i, j, k) = F(w, i, j, k) - factor12 * gacc[2] * beta * 0.5 * (F(s1, i, j, k + 1) + F(s1, i, j, k));
        }
      }
  if (impdiff) {
#pragma omp parallel for
    for (int k = lo[2]; k <= hi[2]; k++) /* rk.f90:118-126 */
      for (int j = lo[1]; j <= hi[1]; j++)
        for (int i = lo[0]; i <= hi[0]; i++) {
          F(u, i, j, k) = F(u, i, j, k) - 0.5 * factor12 * D(dudtrkd, i, j, k);
          F(v, i, j, k) = F(v, i, j, k) - 0.5 * factor12 * D(dvdtrkd, i, j, k);
          F(w, i, j, k) = F(w, i, j, k) - 0.5 * factor12 * D(dwdtrkd, i, j, k);
        }
    free(dudtrkd); free(dvdtrkd); free(dwdtrkd);
  }
  free(dudtrk); free(dvdtrk); free(dwdtrk);
}

/* rk.f90:130-204 (rk_scal) with scal.f90:89-179 (scal_d, scal_a, bulk_mean_s) */
void or_rk_scal(const double rkpar[2], const int lo[3], const int hi[3],
                const double *dxc, const double *dxf, const double *dyc, const double *dyf,
                const double *dzc, const double *dzf, double dt, double alpha, double vol_all,
                const double *u, const double *v, const double *w,
                int is_forced, double scalf, double ssource, double *dsdtrko, double *s,
                double *f, int impdiff) {
  size_t n = (size_t)NX * NY * NZ;
  double factor1 = rkpar[0] * dt, factor2 = rkpar[1] * dt;
  double factor12 = factor1 + factor2;
  double *dsdtrk = calloc(n, sizeof(double));
  double *dsdtrkd = impdiff ? calloc(n, sizeof(double)) : NULL;
  double *dd = impdiff ? dsdtrkd : dsdtrk;
#pragma omp parallel for
  for (int k = lo[2]; k <= hi[2]; k++) /* scal.f90:101-117 (scal_d) */
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) {
        double dsdxp = (F(s, i + 1, j, k) - F(s, i, j, k)) / MX(dxc, i);
        double dsdxm = (F(s, i, j, k) - F(s, i - 1, j, k)) / MX(dxc, i - 1);
        double dsdyp = (F(s, i, j + 1, k) - F(s, i, j, k)) / MY(dyc, j);
        double dsdym = (F(s, i, j, k) - F(s, i, j - 1, k)) / MY(dyc, j - 1);
        double dsdzp = (F(s, i, j, k + 1) - F(s, i, j, k)) / MZ(dzc, k);
        double dsdzm = (F(s, i, j, k) - F(s, i, j, k - 1)) / MZ(dzc, k - 1);
        D(dd, i, j, k) = D(dd, i, j, k) + alpha * (dsdxp - dsdxm) / MX(dxf, i) +
                         alpha * (dsdyp - dsdym) / MY(dyf, j) + alpha * (dsdzp - dsdzm) / MZ(dzf, k);
      }
#pragma omp parallel for
  for (int k = lo[2]; k <= hi[2]; k++) /* scal.f90:135-151 (scal_a) */
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) {
        double usim = 0.5 * (F(s, i - 1, j, k) + F(s, i, j, k)) * F(u, i - 1, j, k);
        double usip = 0.5 * (F(s, i + 1, j, k) + F(s, i, j, k)) * F(u, i, j, k);
        double vsjm = 0.5 * (F(s, i, j - 1, k) + F(s, i, j, k)) * F(v, i, j - 1, k);
        double vsjp = 0.5 * (F(s, i, j + 1, k) + F(s, i, j, k)) * F(v, i, j, k);
        double wskm = 0.5 * (F(s, i, j, k - 1) + F(s, i, j, k)) * F(w, i, j, k - 1);
        double wskp = 0.5 * (F(s, i, j, k + 1) + F(s, i, j, k)) * F(w, i, j, k);
        D(dsdtrk, i, j, k) = D(dsdtrk, i, j, k) + (-usip + usim) / MX(dxf, i) +
                             (-vsjp + vsjm) / MY(dyf, j) + (-wskp + wskm) / MZ(dzf, k);
      }
#pragma omp parallel for
  for (int k = lo[2]; k <= hi[2]; k++) /* rk.f90:173-184 */
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) {
        F(s, i, j, k) = F(s, i, j, k) + factor1 * D(dsdtrk, i, j, k) + factor2 * D(dsdtrko, i, j, k) +
                        factor12 * ssource;
        if (impdiff) F(s, i, j, k) = F(s, i, j, k) + factor12 * D(dsdtrkd, i, j, k);
        D(dsdtrko, i, j, k) = D(dsdtrk, i, j, k);
      }
  *f = 0.0; /* rk.f90:185-189; bulk_mean_s scal.f90:156-179 (single-process sum) */
  if (is_forced) {
    double mean = 0.0;
    for (int k = lo[2]; k <= hi[2]; k++)
      for (int j = lo[1]; j <= hi[1]; j++)
        for (int i = lo[0]; i <= hi[0]; i++)
          mean = mean + F(s, i, j, k) * MX(dxf, i) * MY(dyf, j) * MZ(dzf, k);
    mean = mean / vol_all;
    *f = scalf - mean;
  }
  if (impdiff) {
#pragma omp parallel for
    for (int k = lo[2]; k <= hi[2]; k++) /* rk.f90:196-202 */
      for (int j = lo[1]; j <= hi[1]; j++)
        for (int i = lo[0]; i <= hi[0]; i++)
          F(s, i, j, k) = F(s, i, j, k) - 0.5 * factor12 * D(dsdtrkd, i, j, k);
    free(dsdtrkd);
  }
  free(dsdtrk);
}

/* scal.f90:181-199 (bulk_forcing_s) */
void or_bulk_forcing_s(const int lo[3], const int hi[3], int is_forced, double ff, double *s) {
  if (!is_forced) return;
  for (int k = lo[2]; k <= hi[2]; k++)
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) F(s, i, j, k) = F(s, i, j, k) + ff;
}

/* fillps.f90:7-54; fft_axis selects the _FFT_X/_FFT_Y/_FFT_Z weighting (fillps.f90:33-49) */
void or_fillps(const int lo[3], const int hi[3], const double *dxf, const double *dyf,
               const double *dzf, double dt, const double *u, const double *v, const double *w,
               double *p, int fft_axis) {
#pragma omp parallel for
  for (int k = lo[2]; k <= hi[2]; k++)
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) {
        double dw = F(w, i, j, k) - F(w, i, j, k - 1);
        double dv = F(v, i, j, k) - F(v, i, j - 1, k);
        double du = F(u, i, j, k) - F(u, i - 1, j, k);
        double r;
        switch (fft_axis) {
          case 3: r = dw / MZ(dzf, k) * MX(dxf, i) * MY(dyf, j) + dv * MX(dxf, i) + du * MY(dyf, j); break;
          case 2: r = dw * MX(dxf, i) + dv / MY(dyf, j) * MX(dxf, i) * MZ(dzf, k) + du * MZ(dzf, k); break;
          case 1: r = dw * MY(dyf, j) + dv * MZ(dzf, k) + du / MX(dxf, i) * MY(dyf, j) * MZ(dzf, k); break;
          default: r = dw * MX(dxf, i) * MY(dyf, j) + dv * MX(dxf, i) * MZ(dzf, k) + du * MY(dyf, j) * MZ(dzf, k);
        }
        F(p, i, j, k) = r / dt;
      }
}

/* correc.f90:7-48 (over the extended ranges, ghosts included) */
void or_correc(const int lo[3], const int hi[3], const double *dxc, const double *dyc,
               const double *dzc, double dt, const double *p, double *u, double *v, double *w) {
#pragma omp parallel for
  for (int k = lo[2] - 1; k <= hi[2] + 1; k++)
    for (int j = lo[1] - 1; j <= hi[1] + 1; j++)
      for (int i = lo[0] - 1; i <= hi[0]; i++)
        F(u, i, j, k) = F(u, i, j, k) - dt * (F(p, i + 1, j, k) - F(p, i, j, k)) / MX(dxc, i);
#pragma omp parallel for
  for (int k = lo[2] - 1; k <= hi[2] + 1; k++)
    for (int j = lo[1] - 1; j <= hi[1]; j++)
      for (int i = lo[0] - 1; i <= hi[0] + 1; i++)
        F(v, i, j, k) = F(v, i, j, k) - dt * (F(p, i, j + 1, k) - F(p, i, j, k)) / MY(dyc, j);
#pragma omp parallel for
  for (int k = lo[2] - 1; k <= hi[2]; k++)
    for (int j = lo[1] - 1; j <= hi[1] + 1; j++)
      for (int i = lo[0] - 1; i <= hi[0] + 1; i++)
        F(w, i, j, k) = F(w, i, j, k) - dt * (F(p, i, j, k + 1) - F(p, i, j, k)) / MZ(dzc, k);
}

/* updt_pressure.f90:7-47 */
void or_updt_pressure(const int lo[3], const int hi[3], const double *dxc, const double *dxf,
                      const double *dyc, const double *dyf, const double *dzc, const double *dzf,
                      double alpha, const double *pp, double *p, int impdiff) {
#pragma omp parallel for
  for (int k = lo[2]; k <= hi[2]; k++)
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) F(p, i, j, k) = F(p, i, j, k) + F(pp, i, j, k);
  if (!impdiff) return;
#pragma omp parallel for
  for (int k = lo[2]; k <= hi[2]; k++)
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++)
        F(p, i, j, k) = F(p, i, j, k) +
            alpha * (((F(pp, i + 1, j, k) - F(pp, i, j, k)) / MX(dxc, i) -
                      (F(pp, i, j, k) - F(pp, i - 1, j, k)) / MX(dxc, i - 1)) / MX(dxf, i) +
                     ((F(pp, i, j + 1, k) - F(pp, i, j, k)) / MY(dyc, j) -
                      (F(pp, i, j, k) - F(pp, i, j - 1, k)) / MY(dyc, j - 1)) / MY(dyf, j) +
                     ((F(pp, i, j, k + 1) - F(pp, i, j, k)) / MZ(dzc, k) -
                      (F(pp, i, j, k) - F(pp, i, j, k - 1)) / MZ(dzc, k - 1)) / MZ(dzf, k));
}

/* chkdt.f90:24-55, the per-rank part before the MPI reductions */
void or_chkdt_local(const int lo[3], const int hi[3], const double *dxc, const double *dxf,
                    const double *dyc, const double *dyf, const double *dzc, const double *dzf,
                    const double *u, const double *v, const double *w, double *dti_out, double *dlmin) {
  double dti = 0.0;
#pragma omp parallel for reduction(max : dti)
  for (int k = lo[2]; k <= hi[2]; k++)
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) {
        double ux = fabs(F(u, i, j, k));
        double vx = 0.25 * fabs(F(v, i, j, k) + F(v, i, j - 1, k) + F(v, i + 1, j, k) + F(v, i + 1, j - 1, k));
        double wx = 0.25 * fabs(F(w, i, j, k) + F(w, i, j, k - 1) + F(w, i + 1, j, k) + F(w, i + 1, j, k - 1));
        double dtix = ux / MX(dxc, i) + vx / MY(dyf, j) + wx / MZ(dzf, k);
        double uy = 0.25 * fabs(F(u, i, j, k) + F(u, i, j + 1, k) + F(u, i - 1, j + 1, k) + F(u, i - 1, j, k));
        double vy = fabs(F(v, i, j, k));
        double wy = 0.25 * fabs(F(w, i, j, k) + F(w, i, j + 1, k) + F(w, i, j + 1, k - 1) + F(w, i, j, k - 1));
        double dtiy = uy / MX(dxf, i) + vy / MY(dyc, j) + wy / MZ(dzf, k);
        double uz = 0.25 * fabs(F(u, i, j, k) + F(u, i - 1, j, k) + F(u, i - 1, j, k + 1) + F(u, i, j, k + 1));
        double vz = 0.25 * fabs(F(v, i, j, k) + F(v, i, j - 1, k) + F(v, i, j - 1, k + 1) + F(v, i, j, k + 1));
        double wz = fabs(F(w, i, j, k));
        double dtiz = uz / MX(dxf, i) + vz / MY(dyf, j) + wz / MZ(dzc, k);
        double m = dtix;
        if (dtiy > m) m = dtiy;
        if (dtiz > m) m = dtiz;
        if (m > dti) dti = m;
      }
  *dti_out = dti;
  /* dlmin = min(minval(dxf),minval(dyf),minval(dzf)) over the whole (lo-1:hi+1) arrays, chkdt.f90:47 */
  double dm = dxf[0];
  for (int q = 0; q < NX + 2; q++) if (dxf[q] < dm) dm = dxf[q];
  for (int q = 0; q < NY + 2; q++) if (dyf[q] < dm) dm = dyf[q];
  for (int q = 0; q < NZ + 2; q++) if (dzf[q] < dm) dm = dzf[q];
  *dlmin = dm;
}

/* chkdiv.f90:24-43, per-rank part */
void or_chkdiv_local(const int lo[3], const int hi[3], const double *dxf, const double *dyf,
                     const double *dzf, const double *u, const double *v, const double *w,
                     double vol, double *divtot_out, double *divmax_out) {
  double divtot = 0.0, divmax = 0.0;
  for (int k = lo[2]; k <= hi[2]; k++)
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) {
        double div = (F(w, i, j, k) - F(w, i, j, k - 1)) / MZ(dzf, k) +
                     (F(v, i, j, k) - F(v, i, j - 1, k)) / MY(dyf, j) +
                     (F(u, i, j, k) - F(u, i - 1, j, k)) / MX(dxf, i);
        if (fabs(div) > divmax) divmax = fabs(div);
        divtot = divtot + div * MX(dxf, i) * MY(dyf, j) * MZ(dzf, k) / vol;
      }
  *divtot_out = divtot;
  *divmax_out = divmax;
}

/* bound.f90:543-585 (updt_rhs) */
void or_updt_rhs(const int lo[3], const int hi[3], const int is_bound[3][2],
                 const double *rhsx, const double *rhsy, const double *rhsz, double *p) {
  int nx = NX, ny = NY, nz = NZ;
  for (int s = 0; s < 2; s++) {
    if (is_bound[0][s]) {
      int i = s ? hi[0] : lo[0];
      for (int k = lo[2]; k <= hi[2]; k++)
        for (int j = lo[1]; j <= hi[1]; j++)
          F(p, i, j, k) = F(p, i, j, k) + rhsx[(j - lo[1]) + (size_t)ny * ((k - lo[2]) + (size_t)nz * s)];
    }
  }
  for (int s = 0; s < 2; s++) {
    if (is_bound[1][s]) {
      int j = s ? hi[1] : lo[1];
      for (int k = lo[2]; k <= hi[2]; k++)
        for (int i = lo[0]; i <= hi[0]; i++)
          F(p, i, j, k) = F(p, i, j, k) + rhsy[(i - lo[0]) + (size_t)nx * ((k - lo[2]) + (size_t)nz * s)];
    }
  }
  for (int s = 0; s < 2; s++) {
    if (is_bound[2][s]) {
      int k = s ? hi[2] : lo[2];
      for (int j = lo[1]; j <= hi[1]; j++)
        for (int i = lo[0]; i <= hi[0]; i++)
          F(p, i, j, k) = F(p, i, j, k) + rhsz[(i - lo[0]) + (size_t)nx * ((j - lo[1]) + (size_t)ny * s)];
    }
  }
}

/* bound.f90:108-248 (set_bc) on one face plane (including ghost rows) */
void or_set_bc(char ctype, int ibound, const int lo[3], const int hi[3], int idir,
               int centered, double rvalue, double dr, double *p) {
  double factor = rvalue, sgn = 0.0;
  if (ctype == 'D' && centered) { factor = 2.0 * factor; sgn = -1.0; }
  if (ctype == 'N') {
    if (ibound == 0) factor = -dr * factor;
    else factor = dr * factor;
    sgn = 1.0;
  }
  if (ctype != 'D' && ctype != 'N') return;
  int nx = NX, ny = NY, nz = NZ;
  int n[3] = {nx, ny, nz};
  int d = idir - 1;
  int t1 = (d == 0) ? 1 : 0, t2 = (d == 2) ? 1 : 2;
  /* offsets in local 0..n+1 coordinates */
  long st[3] = {1, (long)(nx + 2), (long)(nx + 2) * (ny + 2)};
  int ng = n[d];
  for (int b = 0; b < n[t2] + 2; b++)
    for (int a = 0; a < n[t1] + 2; a++) {
      long base = a * st[t1] + b * st[t2];
#define AT(q) p[base + (long)(q) * st[d]]
      if (centered) {
        if (ibound == 0) AT(0) = factor + sgn * AT(1);
        else AT(ng + 1) = factor + sgn * AT(ng);
      } else if (ctype == 'D') {
        if (ibound == 0) AT(0) = factor;
        else { AT(ng) = factor; AT(ng + 1) = AT(ng - 1); }
      } else { /* staggered N */
        if (ibound == 0) AT(0) = factor + AT(1);
        else { AT(ng) = factor + AT(ng - 1); AT(ng + 1) = AT(ng); }
      }
#undef AT
    }
  (void)nz;
}

/* updthalo (bound.f90:587-650) of one block whose neighbour on side s of direction idir is the block itself
 * (a periodic direction it spans alone, MPI_SENDRECV to its own rank): ghost plane lo-1 receives interior
 * plane hi and ghost plane hi+1 interior plane lo, each plane including the ghost rows of the other two
 * directions.  Sides whose neighbour is another rank are left alone (that exchange is not this rank's). */
static void or_self_halo(const int lo[3], const int hi[3], int idir, const int nb[2], int myrank, double *p) {
  int nx = NX, ny = NY;
  int n[3] = {nx, ny, NZ};
  int d = idir - 1;
  int t1 = (d == 0) ? 1 : 0, t2 = (d == 2) ? 1 : 2;
  long st[3] = {1, (long)(nx + 2), (long)(nx + 2) * (ny + 2)};
  for (int b = 0; b < n[t2] + 2; b++)
    for (int a = 0; a < n[t1] + 2; a++) {
      long base = a * st[t1] + b * st[t2];
      if (nb[0] == myrank) p[base] = p[base + (long)n[d] * st[d]];
      if (nb[1] == myrank) p[base + (long)(n[d] + 1) * st[d]] = p[base + st[d]];
    }
}

/* bound.f90:8-66 (bounduvw) for one block: the halo exchange x, y, z of u, v and w (self-neighbour sides
 * only, see or_self_halo), then set_bc face by face in the reference's order, the wall-normal component
 * skipped when is_correc.  cbc[c][d][s], bc[c][d][s] hold cbc(s,d,c), bc(s,d,c); metrics from lo-1. */
void or_bounduvw_block(const char cbc[3][3][2], const int lo[3], const int hi[3], const double bc[3][3][2],
                       int is_correc, const int is_bound[3][2], const int nb[3][2], int myrank,
                       const double *dxc, const double *dxf, const double *dyc, const double *dyf,
                       const double *dzc, const double *dzf, double *u, double *v, double *w) {
  double *f[3] = {u, v, w};
  const double *dc[3] = {dxc, dyc, dzc}, *df[3] = {dxf, dyf, dzf};
  for (int c = 0; c < 3; c++)
    for (int d = 1; d <= 3; d++) or_self_halo(lo, hi, d, nb[d - 1], myrank, f[c]);
  for (int d = 0; d < 3; d++)
    for (int s = 0; s < 2; s++) {
      if (!is_bound[d][s]) continue;
      const int q = s ? hi[d] - lo[d] + 1 : 0;  /* dl(lo-1) or dl(hi) */
      for (int c = 0; c < 3; c++) {
        const int centered = c != d;
        if (!centered && is_correc) continue;
        or_set_bc(cbc[c][d][s], s, lo, hi, d + 1, centered, bc[c][d][s], centered ? dc[d][q] : df[d][q], f[c]);
      }
    }
}

/* bound.f90:68-106 (boundp) for one block, as or_bounduvw_block for one centred field */
void or_boundp_block(const char cbc[3][2], const int lo[3], const int hi[3], const double bc[3][2],
                     const int is_bound[3][2], const int nb[3][2], int myrank, const double *dxc,
                     const double *dyc, const double *dzc, double *p) {
  const double *dc[3] = {dxc, dyc, dzc};
  for (int d = 1; d <= 3; d++) or_self_halo(lo, hi, d, nb[d - 1], myrank, p);
  for (int d = 0; d < 3; d++)
    for (int s = 0; s < 2; s++) {
      if (!is_bound[d][s]) continue;
      const int q = s ? hi[d] - lo[d] + 1 : 0;
      or_set_bc(cbc[d][s], s, lo, hi, d + 1, 1, bc[d][s], dc[d][q], p);
    }
}

/* post.f90:8-156: vorticity, strain rate S_ij S_ij, rotation rate W_ij W_ij and the Q criterion at cell
 * centres of one block.  n = interior extents; ux, uy, uz halo'd (0:n+1); metrics indexed 0..n+1; outputs
 * interior (1:n, Fortran order). */
#define PH(a, i, j, k) a[(i) + (size_t)(n[0] + 2) * ((j) + (size_t)(n[1] + 2) * (k))]
#define PI_(a, i, j, k) a[((i) - 1) + (size_t)n[0] * (((j) - 1) + (size_t)n[1] * ((k) - 1))]
void or_cmpt_vorticity(const int n[3], const double *dxc, const double *dyc, const double *dzc, const double *ux,
                       const double *uy, const double *uz, double *vox, double *voy, double *voz) {
  for (int k = 1; k <= n[2]; k++)
    for (int j = 1; j <= n[1]; j++)
      for (int i = 1; i <= n[0]; i++) {
        PI_(vox, i, j, k) = 0.25 * ((PH(uz, i, j + 1, k) - PH(uz, i, j, k)) / dyc[j] - (PH(uy, i, j, k + 1) - PH(uy, i, j, k)) / dzc[k] +
                                    (PH(uz, i, j + 1, k - 1) - PH(uz, i, j, k - 1)) / dyc[j] - (PH(uy, i, j, k) - PH(uy, i, j, k - 1)) / dzc[k - 1] +
                                    (PH(uz, i, j, k) - PH(uz, i, j - 1, k)) / dyc[j - 1] - (PH(uy, i, j - 1, k + 1) - PH(uy, i, j - 1, k)) / dzc[k] +
                                    (PH(uz, i, j, k - 1) - PH(uz, i, j - 1, k - 1)) / dyc[j - 1] - (PH(uy, i, j - 1, k) - PH(uy, i, j - 1, k - 1)) / dzc[k - 1]);
        PI_(voy, i, j, k) = 0.25 * ((PH(ux, i, j, k + 1) - PH(ux, i, j, k)) / dzc[k] - (PH(uz, i + 1, j, k) - PH(uz, i, j, k)) / dxc[i] +
                                    (PH(ux, i, j, k) - PH(ux, i, j, k - 1)) / dzc[k - 1] - (PH(uz, i + 1, j, k - 1) - PH(uz, i, j, k - 1)) / dxc[i] +
                                    (PH(ux, i - 1, j, k + 1) - PH(ux, i - 1, j, k)) / dzc[k] - (PH(uz, i, j, k) - PH(uz, i - 1, j, k)) / dxc[i - 1] +
                                    (PH(ux, i - 1, j, k) - PH(ux, i - 1, j, k - 1)) / dzc[k - 1] - (PH(uz, i, j, k - 1) - PH(uz, i - 1, j, k - 1)) / dxc[i - 1]);
        PI_(voz, i, j, k) = 0.25 * ((PH(uy, i + 1, j, k) - PH(uy, i, j, k)) / dxc[i] - (PH(ux, i, j + 1, k) - PH(ux, i, j, k)) / dyc[j] +
                                    (PH(uy, i + 1, j - 1, k) - PH(uy, i, j - 1, k)) / dxc[i] - (PH(ux, i, j, k) - PH(ux, i, j - 1, k)) / dyc[j - 1] +
                                    (PH(uy, i, j, k) - PH(uy, i - 1, j, k)) / dxc[i - 1] - (PH(ux, i - 1, j + 1, k) - PH(ux, i - 1, j, k)) / dyc[j] +
                                    (PH(uy, i, j - 1, k) - PH(uy, i - 1, j - 1, k)) / dxc[i - 1] - (PH(ux, i - 1, j, k) - PH(ux, i - 1, j - 1, k)) / dyc[j - 1]);
      }
}

static double sq(double a) { return a * a; }

/* sgn = +1: strain rate sum of squares of (du_i/dx_j + du_j/dx_i)/2 terms (post.f90:55-98);
 * sgn = -1: rotation rate (post.f90:100-139) */
static void or_rate(const int n[3], const double *dxc, const double *dyc, const double *dzc, const double *dxf,
                    const double *dyf, const double *dzf, const double *ux, const double *uy, const double *uz,
                    double sgn, double *out) {
  for (int k = 1; k <= n[2]; k++)
    for (int j = 1; j <= n[1]; j++)
      for (int i = 1; i <= n[0]; i++) {
        const double a12 = .25 * (sq((PH(ux, i, j + 1, k) - PH(ux, i, j, k)) / dyc[j] + sgn * ((PH(uy, i + 1, j, k) - PH(uy, i, j, k)) / dxc[i])) +
                                  sq((PH(ux, i, j, k) - PH(ux, i, j - 1, k)) / dyc[j - 1] + sgn * ((PH(uy, i + 1, j - 1, k) - PH(uy, i, j - 1, k)) / dxc[i])) +
                                  sq((PH(ux, i - 1, j + 1, k) - PH(ux, i - 1, j, k)) / dyc[j] + sgn * ((PH(uy, i, j, k) - PH(uy, i - 1, j, k)) / dxc[i - 1])) +
                                  sq((PH(ux, i - 1, j, k) - PH(ux, i - 1, j - 1, k)) / dyc[j - 1] + sgn * ((PH(uy, i, j - 1, k) - PH(uy, i - 1, j - 1, k)) / dxc[i - 1]))) * .25;
        const double a13 = .25 * (sq((PH(ux, i, j, k + 1) - PH(ux, i, j, k)) / dzc[k] + sgn * ((PH(uz, i + 1, j, k) - PH(uz, i, j, k)) / dxc[i])) +
                                  sq((PH(ux, i, j, k) - PH(ux, i, j, k - 1)) / dzc[k - 1] + sgn * ((PH(uz, i + 1, j, k - 1) - PH(uz, i, j, k - 1)) / dxc[i])) +
                                  sq((PH(ux, i - 1, j, k + 1) - PH(ux, i - 1, j, k)) / dzc[k] + sgn * ((PH(uz, i, j, k) - PH(uz, i - 1, j, k)) / dxc[i - 1])) +
                                  sq((PH(ux, i - 1, j, k) - PH(ux, i - 1, j, k - 1)) / dzc[k - 1] + sgn * ((PH(uz, i, j, k - 1) - PH(uz, i - 1, j, k - 1)) / dxc[i - 1]))) * .25;
        const double a23 = .25 * (sq((PH(uy, i, j, k + 1) - PH(uy, i, j, k)) / dzc[k] + sgn * ((PH(uz, i, j + 1, k) - PH(uz, i, j, k)) / dyc[j])) +
                                  sq((PH(uy, i, j, k) - PH(uy, i, j, k - 1)) / dzc[k - 1] + sgn * ((PH(uz, i, j + 1, k - 1) - PH(uz, i, j, k - 1)) / dyc[j])) +
                                  sq((PH(uy, i, j - 1, k + 1) - PH(uy, i, j - 1, k)) / dzc[k] + sgn * ((PH(uz, i, j, k) - PH(uz, i, j - 1, k)) / dyc[j - 1])) +
                                  sq((PH(uy, i, j - 1, k) - PH(uy, i, j - 1, k - 1)) / dzc[k - 1] + sgn * ((PH(uz, i, j, k - 1) - PH(uz, i, j - 1, k - 1)) / dyc[j - 1]))) * .25;
        if (sgn > 0) {
          const double s11 = sq((PH(ux, i, j, k) - PH(ux, i - 1, j, k)) / dxf[i]);
          const double s22 = sq((PH(uy, i, j, k) - PH(uy, i, j - 1, k)) / dyf[j]);
          const double s33 = sq((PH(uz, i, j, k) - PH(uz, i, j, k - 1)) / dzf[k]);
          PI_(out, i, j, k) = s11 + s22 + s33 + 2 * (a12 + a13 + a23);
        } else {
          PI_(out, i, j, k) = 2.0 * (a12 + a13 + a23);
        }
      }
}
void or_cmpt_strain_rate(const int n[3], const double *dxc, const double *dyc, const double *dzc, const double *dxf,
                         const double *dyf, const double *dzf, const double *ux, const double *uy, const double *uz,
                         double *str) {
  or_rate(n, dxc, dyc, dzc, dxf, dyf, dzf, ux, uy, uz, 1.0, str);
}
void or_cmpt_rotation_rate(const int n[3], const double *dxc, const double *dyc, const double *dzc, const double *ux,
                           const double *uy, const double *uz, double *ens) {
  or_rate(n, dxc, dyc, dzc, dxc, dyc, dzc, ux, uy, uz, -1.0, ens);
}
void or_cmpt_q_criterion(const int n[3], const double *ens, const double *str, double *qcr) {
  const size_t m = (size_t)n[0] * n[1] * n[2];
  for (size_t q = 0; q < m; q++) qcr[q] = .5 * (ens[q] - str[q]);
}
#undef PH
#undef PI_

/* solver.f90:44-157 (init_bc_rhs).  fft_axis selects the weight of solver.f90:98-106. */
void or_init_bc_rhs(const char cbc[3][2], const double bc[3][2], const double dl[3][2],
                    const int is_bound[3][2], const int is_centered[3], const int lo[3],
                    const int hi[3], const int periods[3],
                    const double *dx1, const double *dx2, const double *dy1, const double *dy2,
                    const double *dz1, const double *dz2,
                    double *rhsx, double *rhsy, double *rhsz,
                    const double *bcx, const double *bcy, const double *bcz, int fft_axis) {
  int nx = NX, ny = NY, nz = NZ;
  int qqq[3];
  double factor[3][2], sgn[3][2];
  for (int q = 0; q < 3; q++) {
    qqq[q] = is_centered[q] ? 0 : 1;
    for (int s = 0; s < 2; s++) {
      factor[q][s] = 0.0; sgn[q][s] = 0.0;
      if (is_bound[q][s]) {
        if (cbc[q][s] == 'N') {
          factor[q][s] = 1.0 * dl[q][s] * bc[q][s];
          if (s == 1) factor[q][s] = -factor[q][s];
          sgn[q][s] = 1.0;
        } else if (cbc[q][s] == 'D') {
          if (is_centered[q]) { factor[q][s] = -2.0 * bc[q][s]; sgn[q][s] = -1.0; }
          else { factor[q][s] = -1.0 * bc[q][s]; sgn[q][s] = 0.0; }
        }
      }
    }
  }
  memset(rhsx, 0, sizeof(double) * ny * nz * 2);
  memset(rhsy, 0, sizeof(double) * nx * nz * 2);
  memset(rhsz, 0, sizeof(double) * nx * ny * 2);
#define W(i, j, k) (fft_axis == 1 ? MY(dy2, j) * MZ(dz2, k) : fft_axis == 2 ? MX(dx2, i) * MZ(dz2, k) : \
                    fft_axis == 3 ? MX(dx2, i) * MY(dy2, j) : MX(dx2, i) * MY(dy2, j) * MZ(dz2, k))
  for (int idir = 0; idir < 3; idir++) {
    if (periods[idir] != 0) continue;
    int stp[3] = {1, 1, 1};
    if (idir == 0) stp[0] = (hi[0] - lo[0]) > 1 ? hi[0] - lo[0] : 1;
    if (idir == 1) stp[1] = (hi[1] - lo[1]) > 1 ? hi[1] - lo[1] : 1;
    if (idir == 2) stp[2] = (hi[2] - lo[2]) > 1 ? hi[2] - lo[2] : 1;
    for (int k = lo[2]; k <= hi[2]; k += stp[2])
      for (int j = lo[1]; j <= hi[1]; j += stp[1])
        for (int i = lo[0]; i <= hi[0]; i += stp[0]) {
          double weight = W(i, j, k);
          int c = idir == 0 ? i : idir == 1 ? j : k;
          int ib;
          if (c == lo[idir]) ib = 0;
          else if (c == hi[idir]) ib = 1;
          else continue;
          /* the reference visits lo and hi; when lo==hi both branches hit the same cell (ib=0) */
          if (!is_bound[idir][ib]) continue;
          double rhs;
          if (idir == 0) {
            rhs = factor[0][ib] * weight / (MX(dx1, i - (1 - ib) + qqq[0]) * MX(dx2, i));
            if (bcx && bc[0][ib] != 0.0) rhs = rhs * bcx[(j - lo[1]) + (size_t)ny * ((k - lo[2]) + (size_t)nz * ib)] / bc[0][ib];
            rhsx[(j - lo[1]) + (size_t)ny * ((k - lo[2]) + (size_t)nz * ib)] = rhs;
          } else if (idir == 1) {
            rhs = factor[1][ib] * weight / (MY(dy1, j - (1 - ib) + qqq[1]) * MY(dy2, j));
            if (bcy && bc[1][ib] != 0.0) rhs = rhs * bcy[(i - lo[0]) + (size_t)nx * ((k - lo[2]) + (size_t)nz * ib)] / bc[1][ib];
            rhsy[(i - lo[0]) + (size_t)nx * ((k - lo[2]) + (size_t)nz * ib)] = rhs;
          } else {
            rhs = factor[2][ib] * weight / (MZ(dz1, k - (1 - ib) + qqq[2]) * MZ(dz2, k));
            if (bcz && bc[2][ib] != 0.0) rhs = rhs * bcz[(i - lo[0]) + (size_t)nx * ((j - lo[1]) + (size_t)ny * ib)] / bc[2][ib];
            rhsz[(i - lo[0]) + (size_t)nx * ((j - lo[1]) + (size_t)ny * ib)] = rhs;
          }
        }
  }
#undef W
}

/* ---------------------------------------------------------------- open / outflow boundaries
 * bound.f90:250-328 (set_open_bc_uvw), 330-375 (set_open_bc_p), 377-436 (cmpt_estimated_traction),
 * 479-515 (outflow), 517-541 (outflow_p).  idir is 1..3 as in the reference; the traction planes tr are
 * (lo_t1-1:hi_t1+1, lo_t2-1:hi_t2+1, 0:1), t1 < t2 the two other axes.  The plane loops run over every cell of
 * the halo'd plane, as the reference's whole-array assignments do. */
static double *cell_at(double *a, const int lo[3], const int hi[3], int ax, int q, int c1, int c2) {
  int c[3];
  const int t1 = ax == 0 ? 1 : 0, t2 = ax == 2 ? 1 : 2;
  c[ax] = q; c[t1] = c1; c[t2] = c2;
  return &F(a, c[0], c[1], c[2]);
}
static double *tr_at(double *tr, const int lo[3], const int hi[3], int ax, int ib, int c1, int c2) {
  const int t1 = ax == 0 ? 1 : 0, t2 = ax == 2 ? 1 : 2;
  const int m1 = hi[t1] - lo[t1] + 3, m2 = hi[t2] - lo[t2] + 3;
  return &tr[(c1 - lo[t1] + 1) + (size_t)m1 * ((c2 - lo[t2] + 1) + (size_t)m2 * ib)];
}
#define PLANE_LOOP(ax)                                                               \
  const int t1_ = (ax) == 0 ? 1 : 0, t2_ = (ax) == 2 ? 1 : 2;                        \
  for (int c2 = lo[t2_] - 1; c2 <= hi[t2_] + 1; c2++)                                \
    for (int c1 = lo[t1_] - 1; c1 <= hi[t1_] + 1; c1++)

void or_set_open_bc_uvw(int ibound, const int lo[3], const int hi[3], int idir, double visc, double dr, double *u,
                        double *v, double *w, const double *p, double *tr) {
  const int ax = idir - 1;
  double *f = ax == 0 ? u : (ax == 1 ? v : w);
  const double norm = ibound == 0 ? 1.0 : -1.0;
  const int q = ibound == 0 ? lo[ax] - 1 : hi[ax];
  const double factor = -norm * dr / (2 * visc);
  PLANE_LOOP(ax) {
    double *t = tr_at(tr, lo, hi, ax, ibound, c1, c2);
    if (ibound == 0) {
      const double fn = *cell_at(f, lo, hi, ax, q + 1, c1, c2);
      const double m = fmin(0.0, norm * fn);
      *t = *t + .5 * (m * m);
      *cell_at(f, lo, hi, ax, q, c1, c2) = fn + factor * (*t + *cell_at((double *)p, lo, hi, ax, q + 1, c1, c2));
    } else {
      const double fn = *cell_at(f, lo, hi, ax, q - 1, c1, c2);
      const double m = fmin(0.0, norm * fn);
      *t = *t + .5 * (m * m);
      *cell_at(f, lo, hi, ax, q, c1, c2) = fn + factor * (*t + *cell_at((double *)p, lo, hi, ax, q, c1, c2));
    }
  }
  if (ibound == 1) {
    PLANE_LOOP(ax) *cell_at(f, lo, hi, ax, hi[ax] + 1, c1, c2) = *cell_at(f, lo, hi, ax, hi[ax], c1, c2);
  }
}

void or_set_open_bc_p(int ibound, const int lo[3], const int hi[3], int idir, const double drc[2], double drf,
                      double alpha, double *p) {
  const int ax = idir - 1;
  const int q = ibound == 0 ? lo[ax] : hi[ax];
  PLANE_LOOP(ax) {
    const double p0 = *cell_at(p, lo, hi, ax, q, c1, c2);
    if (ibound == 0) {
      const double pp = *cell_at(p, lo, hi, ax, q + 1, c1, c2);
      *cell_at(p, lo, hi, ax, q - 1, c1, c2) = p0 + alpha * drc[0] * drf * p0 - (pp - p0) * drc[0] / drc[1];
    } else {
      const double pm = *cell_at(p, lo, hi, ax, q - 1, c1, c2);
      *cell_at(p, lo, hi, ax, q + 1, c1, c2) = p0 + alpha * drc[1] * drf * p0 + (p0 - pm) * drc[1] / drc[0];
    }
  }
}

void or_cmpt_estimated_traction(int ibound, const int lo[3], const int hi[3], int idir, double visc, double dr,
                                const double *u, const double *v, const double *w, const double *p, double *tr) {
  const int ax = idir - 1;
  double *f = (double *)(ax == 0 ? u : (ax == 1 ? v : w));
  const int q = ibound == 0 ? lo[ax] - 1 : hi[ax];
  const double factor = 2. * visc / dr;
  PLANE_LOOP(ax) {
    double *t = tr_at(tr, lo, hi, ax, ibound, c1, c2);
    if (ibound == 0)
      *t = -*cell_at((double *)p, lo, hi, ax, q + 1, c1, c2) +
           factor * (*cell_at(f, lo, hi, ax, q + 2, c1, c2) - *cell_at(f, lo, hi, ax, q + 1, c1, c2));
    else
      *t = -*cell_at((double *)p, lo, hi, ax, q - 1, c1, c2) +
           factor * (*cell_at(f, lo, hi, ax, q - 1, c1, c2) - *cell_at(f, lo, hi, ax, q - 2, c1, c2));
  }
}

void or_outflow(const int is_outflow_bound[3][2], const int is_estimated_traction[3][2], const int lo[3],
                const int hi[3], const double dl[3][2], const double dl_h[3][2], double visc, double *u, double *v,
                double *w, double *p, double *tr_x, double *tr_y, double *tr_z) {
  double *tr[3] = {tr_x, tr_y, tr_z};
  for (int ax = 0; ax < 3; ax++)
    for (int ib = 0; ib < 2; ib++) {
      if (!is_outflow_bound[ax][ib]) continue;
      PLANE_LOOP(ax) *tr_at(tr[ax], lo, hi, ax, ib, c1, c2) = 0.0;
      if (is_estimated_traction[ax][ib]) or_cmpt_estimated_traction(ib, lo, hi, ax + 1, visc, dl_h[ax][ib], u, v, w, p, tr[ax]);
      or_set_open_bc_uvw(ib, lo, hi, ax + 1, visc, dl[ax][ib], u, v, w, p, tr[ax]);
    }
}

void or_outflow_p(const int is_outflow_bound[3][2], const int lo[3], const int hi[3], const double dlc[3][2][2],
                  const double dlf[3][2], double alpha, double *p) {
  for (int ax = 0; ax < 3; ax++)
    for (int ib = 0; ib < 2; ib++)
      if (is_outflow_bound[ax][ib]) or_set_open_bc_p(ib, lo, hi, ax + 1, dlc[ax][ib], dlf[ax][ib], alpha, p);
}
