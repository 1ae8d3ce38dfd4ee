/* or_internal.h -- private structures of the oracle.  TEST INFRASTRUCTURE ONLY. */
#ifndef OR_INTERNAL_H
#define OR_INTERNAL_H
#include "snac_oracle.h"

#define OR_MAXLEV 16
#define OR_DENSE_MAX 256

typedef struct or_block {
  int ng[3], lo[3], hi[3];
  int nb[3][2], is_bound[3][2];
  or_block_desc desc;
  double *g[3][4];            /* per axis: [dc, df, c, f], (n+2) entries for lo-1..hi+1 */
  double *fld[OR_NFIELDS];
  double *rhsp[3];            /* init_bc_rhs planes for the pressure (rhsp%x/y/z) */
} or_block;

/* one multigrid level of a box problem */
typedef struct or_level {
  int n[3];                   /* coupled extents (n[2]=1 for plane problems) */
  long ncell;
  double *W[3];               /* cell widths per axis (dl_2 analogue) */
  unsigned short *code;       /* per cell: bit15 inactive; 2 bits per face (a*2+s) */
  double *cc;                 /* assembled diagonal without the per-system shift */
  double *cp[3];              /* coupling to the +1 neighbour along axis a (0 if folded) */
  double *x, *b, *r;          /* ncell * nsys */
  double *dinv;               /* coarsest: dense inverse per system (ncell^2 * nsys) */
  int coarsened[3];
} or_level;

typedef struct or_poisson {
  int mode3d;                 /* 1: one 3-D system; 0: 2-D planes batched along the transform axis */
  int ax[3];                  /* box axis -> physical axis (ax[2] = transform axis in plane mode) */
  int periodic[3];            /* per box axis */
  int nsys;                   /* systems (wavenumbers) */
  int lo_min[3];              /* global index of box origin, per physical axis */
  double *shift;              /* per system: lambda_k (plane mode), 0 in 3-D */
  int *singular;              /* per system */
  int nlev;
  or_level L[OR_MAXLEV];
  double *p, *q, *z;          /* CG work, level-0 size * nsys */
  int last_iter; double last_res;
  double tol; int maxiter;
  int nu;                     /* smoothing sweeps (red+black pairs) before and after */
} or_poisson;

struct or_domain {
  or_case c;
  int nblocks;
  or_block *b;
  int periods[3], is_periodic[3];
  double vol_all;
  double dt, time; int istep;
  /* pressure solver */
  int fft_axis, il, iu;       /* 0-based physical axes */
  int kind_fwd, kind_bwd; double normfft;
  double *lambda;             /* eigenvalues/dl^2 along the transform axis */
  or_poisson *ps;
  double *box_b, *box_x;      /* gathered rhs and warm start (po in transformed space) */
};

/* solver module */
or_poisson *or_poisson_create(or_domain *d, const int centered[3], double alpha,
                              const double *lambda, char *err, int errlen);
void or_poisson_destroy(or_poisson *P);
int  or_poisson_solve(or_poisson *P, double *b, double *x);
void or_box_gather(or_domain *d, or_poisson *P, int kind, double *box);
void or_box_scatter(or_domain *d, or_poisson *P, double *box, int kind);
#endif
