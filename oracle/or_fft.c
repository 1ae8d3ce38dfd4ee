/*
 * or_fft.c -- oracle restatement of fft.f90 (find_fft, eigenvalues, fftini
 * normalisation) with FFTW's unnormalised real-to-real kinds evaluated
 * directly, O(n^2), from their published definitions (FFTW 3 manual,
 * "What FFTW Really Computes").  TEST INFRASTRUCTURE ONLY.
 */
#include "snac_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

static const double PI = 3.14159265358979323846264338327950288;

/* fft.f90:96-149 (find_fft).  bc = bc(0:1) pair, is_centered as in the reference. */
void or_find_fft(const char bc[2], int is_centered, int *kind_fwd, int *kind_bwd, double norm[2]) {
  char a = bc[0], b = bc[1];
  *kind_fwd = *kind_bwd = -1;
  norm[0] = norm[1] = 0.0;
  if (is_centered) {
    if (a == 'F' && b == 'F') { *kind_fwd = OR_R2HC; *kind_bwd = OR_HC2R; norm[0] = 1; norm[1] = 0; }
    else if (a == 'N' && b == 'N') { *kind_fwd = OR_REDFT10; *kind_bwd = OR_REDFT01; norm[0] = 2; norm[1] = 0; }
    else if (a == 'D' && b == 'D') { *kind_fwd = OR_RODFT10; *kind_bwd = OR_RODFT01; norm[0] = 2; norm[1] = 0; }
    else if (a == 'N' && b == 'D') { *kind_fwd = OR_REDFT11; *kind_bwd = OR_REDFT11; norm[0] = 2; norm[1] = 0; }
    else if (a == 'D' && b == 'N') { *kind_fwd = OR_RODFT11; *kind_bwd = OR_RODFT11; norm[0] = 2; norm[1] = 0; }
  } else {
    if (a == 'F' && b == 'F') { *kind_fwd = OR_R2HC; *kind_bwd = OR_HC2R; norm[0] = 1; norm[1] = 0; }
    else if (a == 'N' && b == 'N') { *kind_fwd = OR_REDFT00; *kind_bwd = OR_REDFT00; norm[0] = 2; norm[1] = -1; }
    else if (a == 'D' && b == 'D') { *kind_fwd = OR_RODFT00; *kind_bwd = OR_RODFT00; norm[0] = 2; norm[1] = 1; }
    else if (a == 'N' && b == 'D') { *kind_fwd = OR_REDFT10; *kind_bwd = OR_REDFT01; norm[0] = 2; norm[1] = 0; }
    else if (a == 'D' && b == 'N') { *kind_fwd = OR_RODFT01; *kind_bwd = OR_RODFT10; norm[0] = 2; norm[1] = 0; }
  }
}

/* fft.f90:151-189 (eigenvalues).  Returns -1 for the pair the reference leaves
 * undefined ('DN'); for non-centred 'DD' only n-1 entries are defined by the
 * reference, the n-th is set to 0 here. */
int or_eigenvalues(int n, const char bc[2], int is_centered, double *lambda) {
  char a = bc[0], b = bc[1];
  if (a == 'F' && b == 'F') {
    for (int l = 1; l <= n; l++) { double s = sin((1.0 * (l - 1)) * PI / (1.0 * n)); lambda[l - 1] = -4.0 * s * s; }
  } else if (a == 'N' && b == 'N') {
    if (is_centered)
      for (int l = 1; l <= n; l++) { double s = sin((1.0 * (l - 1)) * PI / (2.0 * n)); lambda[l - 1] = -4.0 * s * s; }
    else
      for (int l = 1; l <= n; l++) { double s = sin((1.0 * (l - 1)) * PI / (2.0 * (n - 1 + 1))); lambda[l - 1] = -4.0 * s * s; }
  } else if (a == 'D' && b == 'D') {
    if (is_centered)
      for (int l = 1; l <= n; l++) { double s = sin((1.0 * (l - 0)) * PI / (2.0 * n)); lambda[l - 1] = -4.0 * s * s; }
    else {
      for (int l = 1; l <= n - 1; l++) { double s = sin((1.0 * (l - 0)) * PI / (2.0 * (n + 1 - 1))); lambda[l - 1] = -4.0 * s * s; }
      lambda[n - 1] = 0.0;
    }
  } else if (a == 'N' && b == 'D') {
    for (int l = 1; l <= n; l++) { double s = sin((1.0 * (2 * l - 1)) * PI / (4.0 * n)); lambda[l - 1] = -4.0 * s * s; }
  } else {
    return -1;
  }
  return 0;
}

/* one unnormalised FFTW r2r transform of length n */
void or_r2r(int kind, int n, const double *x, double *y) {
  for (int k = 0; k < n; k++) {
    double s = 0.0;
    switch (kind) {
      case OR_R2HC:
        if (k <= n / 2) { for (int j = 0; j < n; j++) s += x[j] * cos(2.0 * PI * (double)((long)j * k % n) / n); }
        else { int kk = n - k; for (int j = 0; j < n; j++) s -= x[j] * sin(2.0 * PI * (double)((long)j * kk % n) / n); }
        break;
      case OR_HC2R: {
        s = x[0];
        for (int m = 1; m < (n + 1) / 2; m++) {
          double ang = 2.0 * PI * (double)((long)k * m % n) / n;
          s += 2.0 * (x[m] * cos(ang) - x[n - m] * sin(ang));
        }
        if (n % 2 == 0) s += x[n / 2] * ((k % 2) ? -1.0 : 1.0);
      } break;
      case OR_REDFT00:
        s = x[0] + ((k % 2) ? -1.0 : 1.0) * x[n - 1];
        for (int j = 1; j <= n - 2; j++) s += 2.0 * x[j] * cos(PI * j * k / (double)(n - 1));
        break;
      case OR_REDFT10:
        for (int j = 0; j < n; j++) s += 2.0 * x[j] * cos(PI * (j + 0.5) * k / n);
        break;
      case OR_REDFT01:
        s = x[0];
        for (int j = 1; j < n; j++) s += 2.0 * x[j] * cos(PI * j * (k + 0.5) / n);
        break;
      case OR_REDFT11:
        for (int j = 0; j < n; j++) s += 2.0 * x[j] * cos(PI * (j + 0.5) * (k + 0.5) / n);
        break;
      case OR_RODFT00:
        for (int j = 0; j < n; j++) s += 2.0 * x[j] * sin(PI * (j + 1) * (k + 1) / (double)(n + 1));
        break;
      case OR_RODFT10:
        for (int j = 0; j < n; j++) s += 2.0 * x[j] * sin(PI * (j + 0.5) * (k + 1) / n);
        break;
      case OR_RODFT01:
        s = ((k % 2) ? -1.0 : 1.0) * x[n - 1];
        for (int j = 0; j <= n - 2; j++) s += 2.0 * x[j] * sin(PI * (j + 1) * (k + 0.5) / n);
        break;
      case OR_RODFT11:
        for (int j = 0; j < n; j++) s += 2.0 * x[j] * sin(PI * (j + 0.5) * (k + 0.5) / n);
        break;
    }
    y[k] = s;
  }
}

/* in-place batched transform of `howmany` lines (guru plan of fft.f90:33-67) */
void or_r2r_lines(int kind, int n, int howmany, long stride, long dist, double *arr) {
  if (n <= 0) return;
#pragma omp parallel
  {
    double *in = malloc(sizeof(double) * n), *out = malloc(sizeof(double) * n);
#pragma omp for
    for (int h = 0; h < howmany; h++) {
      double *a = arr + (long)h * dist;
      for (int j = 0; j < n; j++) in[j] = a[(long)j * stride];
      or_r2r(kind, n, in, out);
      for (int j = 0; j < n; j++) a[(long)j * stride] = out[j];
    }
    free(in); free(out);
  }
}
