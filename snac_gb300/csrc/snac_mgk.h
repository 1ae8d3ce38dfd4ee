// snac_mgk.h -- work areas of the batched Krylov/multigrid driver.
#pragma once
#include "snac_solver.h"

namespace snac {

struct MgGeom {
  int mode3d;
  int periodic[3];
};

// per-system scalars of one Krylov iteration
struct SysScal {
  double rz, rr, bb, rel, scale, alpha, beta;
  int first, zero_rhs;
  int restart;  // the warm start was worse than zero (rel > 1): the solve restarts from x = 0
  double tol;   // this system's own relative tolerance in the running loop (0: the loop's)
  double zmean; // singular system: mean of the preconditioned residual z over its active cells (taken out of p)
};

// Partial sums: one row of `stride` doubles per system; a producer kernel writes one entry per CTA
// and reports how many it wrote, the finalising kernel sums that many in a fixed order.
struct CgWork {
  void *r, *z, *p, *p2, *q;  // level-0 vectors (type of the running Krylov loop); p/p2 alternate
  double *part0, *part1, *part2;
  double *part3, *part4;     // singular systems: partial sums of z and of r over the active cells
  int stride;                // partial entries per system (capacity)
  SysScal *sc;               // nsys
  int *active;               // nsys flags of the running loop
  int *d_count;              // [0] still-active systems, [1] systems with a zero right-hand side (device)
  int *h_count;              // pinned host copy
};

// residual r = b - A x on level 0 with norms: sets rr (and bb, first, zero_rhs when set_bb), rel, active, count;
// with want_scale also scale = RMS(r) over the nact active cells
template <typename T>
int mg_residual(const MgProblem &P, CgWork &W, const T *x, const T *b, T *r, double tol, int set_bb, int want_scale,
                long nact, cudaStream_t st);
// preconditioned CG iterations on level 0, starting from the residual in W.r and the scalars set by
// mg_residual / mg_ir_down; zero_x: x is taken as zero (overwritten on the first update)
template <typename T>
int mg_pcg(const MgProblem &P, CgWork &W, T *x, int maxiter, double tol, bool zero_x, bool check_host, int *iters,
           cudaStream_t st);
int mg_project_singular(const MgProblem &P, CgWork &W, double *b, cudaStream_t st);
// mixed path: r32 = r64 / scale, e32 = 0, inner norms (active copied from the outer loop)
int mg_ir_down(const MgProblem &P, const CgWork &Wout, CgWork &W32, const double *r64, float *r32, float *e32,
               double inner_tol, double outer_tol, cudaStream_t st);
int mg_ir_up(const MgProblem &P, const CgWork &Wout, const float *e32, double *x, cudaStream_t st);
int mg_zero_rhs_systems(const MgProblem &P, const CgWork &W, double *x, cudaStream_t st);
// the next mg_pcg starts a new Krylov sequence (first iteration: beta = 0) for every system of W
int mg_restart_krylov(const MgProblem &P, CgWork &W, cudaStream_t st);
// systems whose warm start is worse than zero (set by mg_residual with set_bb): x = 0, r = b
int mg_restart_bad_guess(const MgProblem &P, CgWork &W, double *x, const double *b, double *r, cudaStream_t st);

// plane-mode level-0 Krylov kernels batched over systems (k_mg_plane.cu); partials per 32 x 32 patch
template <typename T>
int plane_resid(const MgProblem &P, const T *shift, const int *active, const T *x, const T *b, T *r, double *part_rr,
                double *part_bb, int stride, cudaStream_t st);
template <typename T, bool FUSEP>
int plane_apply(const MgProblem &P, const T *shift, const int *active, const SysScal *sc, const T *z, const T *po,
                T *pn, T *q, double *part, int stride, cudaStream_t st);

}  // namespace snac
