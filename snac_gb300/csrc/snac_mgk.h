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
};

struct CgWork {
  void *r, *z, *p, *q;      // level-0 vectors (type of the running Krylov loop)
  double *part0, *part1;    // nsys * nchunk partial sums
  SysScal *sc;              // nsys
  int *active;              // nsys flags of the running loop
  int *d_count;             // still-active systems (device)
  int *h_count;             // pinned host copy
};

template <typename T>
int mg_pcg(const MgProblem &P, CgWork &W, T *x, T *b, int maxiter, double tol, bool check_host, int *iters,
           cudaStream_t st);
int mg_project_singular(const MgProblem &P, CgWork &W, double *b, cudaStream_t st);
int mg_ir_down(const MgProblem &P, CgWork &W, const double *r64, float *r32, float *e32, long nact, cudaStream_t st);
int mg_ir_up(const MgProblem &P, CgWork &W, const float *e32, double *x, cudaStream_t st);
int mg_set_active(int nsys, int *active, const int *src, cudaStream_t st);

}  // namespace snac
