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
  double *rhsh[3 + OR_MAX_SCAL][3]; /* IMPDIFF: init_bc_rhs planes of u, v, w and the scalars (rhsu%x, ...) */
  int inflow[3][2];           /* is_bound_inflow (main.f90:596) */
  double *vin[3][2][3];       /* u_in%x.. per axis, side, component over (lo-1:hi+1)^2 of the in-plane axes */
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

/* the field a box problem solves for: the pressure, or (IMPDIFF Helmholtz problems) velocity
 * component c (OR_HF_U + c) or scalar s (OR_HF_S0 + s) */
enum { OR_HF_P = -1, OR_HF_U = 0, OR_HF_S0 = 3 };

typedef struct or_poisson {
  int field;                  /* OR_HF_P, OR_HF_U + c or OR_HF_S0 + s */
  int helm;                   /* Helmholtz problem: never singular, iterative coarsest level */
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
  /* IMPDIFF Helmholtz problems with a transform axis (solve_impdiff_field_fft): the field's own
     transform (fftini with its centring), nfft = n - q points, and lambda_k / dl^2 of its wavenumbers */
  int kind_fwd, kind_bwd, nfft;
  double normfft;
  double *lam;
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
  /* IMPDIFF Helmholtz problems of u, v, w and the scalars (3-D mode), with their warm starts */
  or_poisson *ph[3 + OR_MAX_SCAL];
  double *hbox_b[3 + OR_MAX_SCAL], *hbox_x[3 + OR_MAX_SCAL];
};

/* solver module */
or_poisson *or_poisson_create(or_domain *d, int field, double alpha, const double *lambda, char *err, int errlen);
/* the field's boundary letter, centring and last solved index of block B along physical axis p */
char or_field_cbc(const or_block *B, int field, int p, int side);
double or_field_bc(const or_block *B, int field, int p, int side);
int  or_field_centered(int field, int p);
int  or_field_hi(const or_block *B, int field, int p);
void or_poisson_destroy(or_poisson *P);
int  or_poisson_solve(or_poisson *P, double *b, double *x);
void or_box_gather(or_domain *d, or_poisson *P, int kind, double *box);
void or_box_scatter(or_domain *d, or_poisson *P, double *box, int kind);
#endif
