// k_open.cu -- open and outflow boundaries of one block, with the reference's argument lists: the
// estimated-traction and zero-traction open BC on the wall-normal velocity and the traction BC on the
// correction pressure (Bozonnet et al., JCP 2021), bound.f90:250-541.  Each face is one launch over its whole
// halo'd plane, in the reference's order (x0, x1, y0, y1, z0, z1); the arithmetic is the reference's, term by
// term without FMA contraction, so the planes match the oracle bit for bit.  The traction planes tr are
// (lo_t1-1:hi_t1+1, lo_t2-1:hi_t2+1, 0:1), t1 < t2 the two axes other than the face's.
#include "snac_host.h"

namespace snac {

namespace {

enum OpenOp { OP_TRACTION = 0, OP_UVW = 1, OP_P = 2 };

struct OpenArgs {
  int op, ib, ax;     // operation, side 0/1, axis 0..2
  int n[3];           // interior extents
  double visc, dr, drc0, drc1, drf, alpha;
  double *f;          // the wall-normal velocity component (OP_TRACTION, OP_UVW)
  double *p;          // pressure (OP_TRACTION, OP_UVW read it; OP_P writes its ghost plane)
  double *tr;         // traction planes of this axis
  unsigned long long *bchk;
};

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

__global__ void k_open_face(OpenArgs a) {
  const int t1 = a.ax == 0 ? 1 : 0, t2 = a.ax == 2 ? 1 : 2;
  const int m1 = a.n[t1] + 2, m2 = a.n[t2] + 2;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m1 * m2) return;
  int c[3];
  c[t1] = e % m1 - 1;
  c[t2] = e / m1 - 1;
  c[a.ax] = 0;
  DBlock B;
  B.n[0] = a.n[0]; B.n[1] = a.n[1]; B.n[2] = a.n[2];
  B.bchk = a.bchk;
  if (!bchk(B, BK_SETBC, c[0], c[1], c[2], -1, 1)) return;
  const long st = a.ax == 0 ? 1 : (a.ax == 1 ? (long)(a.n[0] + 2) : (long)(a.n[0] + 2) * (a.n[1] + 2));
  const long base = hidx(c[0], c[1], c[2], a.n[0], a.n[1]);  // index 0 along the axis
  const int n = a.n[a.ax];
  double *tr = a.tr ? a.tr + e + (long)m1 * m2 * a.ib : nullptr;
#define AT(arr, qq) (arr)[base + (long)(qq) * st]
  switch (a.op) {
    case OP_TRACTION: {  // bound.f90:377-436
      const double factor = (2. * a.visc) / a.dr;
      if (a.ib == 0) *tr = dadd(-AT(a.p, 0), dmul(factor, dsub(AT(a.f, 1), AT(a.f, 0))));
      else *tr = dadd(-AT(a.p, n - 2), dmul(factor, dsub(AT(a.f, n - 2), AT(a.f, n - 3))));
      break;
    }
    case OP_UVW: {  // bound.f90:250-328
      const double norm = a.ib == 0 ? 1. : -1.;
      const double factor = (-norm * a.dr) / (2 * a.visc);
      if (a.ib == 0) {  // q = lo - 1
        const double fn = AT(a.f, 0), m = fmin(0., dmul(norm, fn));
        *tr = dadd(*tr, dmul(.5, dmul(m, m)));
        AT(a.f, -1) = dadd(fn, dmul(factor, dadd(*tr, AT(a.p, 0))));
      } else {  // q = hi
        const double fn = AT(a.f, n - 2), m = fmin(0., dmul(norm, fn));
        *tr = dadd(*tr, dmul(.5, dmul(m, m)));
        const double v = dadd(fn, dmul(factor, dadd(*tr, AT(a.p, n - 1))));
        AT(a.f, n - 1) = v;
        AT(a.f, n) = v;
      }
      break;
    }
    default: {  // OP_P, bound.f90:330-375
      if (a.ib == 0) {  // q = lo
        const double p0 = AT(a.p, 0), pp = AT(a.p, 1);
        AT(a.p, -1) = dsub(dadd(p0, dmul(dmul(dmul(a.alpha, a.drc0), a.drf), p0)), dmul(dsub(pp, p0), a.drc0) / a.drc1);
      } else {  // q = hi
        const double p0 = AT(a.p, n - 1), pm = AT(a.p, n - 2);
        AT(a.p, n) = dadd(dadd(p0, dmul(dmul(dmul(a.alpha, a.drc1), a.drf), p0)), dmul(dsub(p0, pm), a.drc1) / a.drc0);
      }
    }
  }
#undef AT
}

int launch_open(const OpenArgs &a) {
  const int t1 = a.ax == 0 ? 1 : 0, t2 = a.ax == 2 ? 1 : 2;
  const int m = (a.n[t1] + 2) * (a.n[t2] + 2);
  k_open_face<<<(m + 255) / 256, 256>>>(a), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

// extents from lo/hi; false (with the error set) when an axis is empty
bool extents(const int lo[3], const int hi[3], int n[3], const char *who) {
  for (int q = 0; q < 3; q++) {
    n[q] = hi[q] - lo[q] + 1;
    if (n[q] < 1) { set_error("%s: hi < lo along axis %d", who, q + 1); return false; }
  }
  return true;
}

size_t halo_bytes(const int n[3]) { return (size_t)(n[0] + 2) * (n[1] + 2) * (n[2] + 2) * sizeof(double); }
size_t plane_bytes(const int n[3], int ax) {
  const int t1 = ax == 0 ? 1 : 0, t2 = ax == 2 ? 1 : 2;
  return (size_t)(n[t1] + 2) * (n[t2] + 2) * 2 * sizeof(double);
}

}  // namespace

}  // namespace snac

using namespace snac;

// set_open_bc_uvw (bound.f90:250-328): the wall-normal velocity's ghost (side 0) or boundary face (side 1) from
// the adjacent interior value, the pressure and the traction plane, which first gains 0.5 min(0, norm u)^2
int snac_set_open_bc_uvw(int ibound, const int lo[3], const int hi[3], int idir, double visc, double dr, double *u,
                         double *v, double *w, const double *p, double *tr) {
  int n[3];
  if (!lo || !hi || !u || !v || !w || !p || !tr || (ibound != 0 && ibound != 1) || idir < 1 || idir > 3) {
    set_error("snac_set_open_bc_uvw: bad argument");
    return SNAC_ERR_ARG;
  }
  if (!extents(lo, hi, n, "snac_set_open_bc_uvw")) return SNAC_ERR_ARG;
  const int ax = idir - 1;
  double *f = ax == 0 ? u : (ax == 1 ? v : w);
  ArgArray F, P, T;
  SNAC_TRY(F.bind(f, halo_bytes(n), true, true));
  SNAC_TRY(P.bind(p, halo_bytes(n), true, false));
  SNAC_TRY(T.bind(tr, plane_bytes(n, ax), true, true));
  OpenArgs a = {};
  a.op = OP_UVW; a.ib = ibound; a.ax = ax;
  for (int q = 0; q < 3; q++) a.n[q] = n[q];
  a.visc = visc; a.dr = dr;
  a.f = (double *)F.dev; a.p = (double *)P.dev; a.tr = (double *)T.dev;
  a.bchk = bounds_flag();
  SNAC_TRY(launch_open(a));
  SNAC_CUDA(cudaDeviceSynchronize());
  SNAC_TRY(bounds_check(0));
  SNAC_TRY(F.finish());
  SNAC_TRY(T.finish());
  return SNAC_OK;
}

// set_open_bc_p (bound.f90:330-375): the correction pressure's ghost plane from the traction condition
int snac_set_open_bc_p(int ibound, const int lo[3], const int hi[3], int idir, const double drc[2], double drf,
                       double alpha, double *p) {
  int n[3];
  if (!lo || !hi || !drc || !p || (ibound != 0 && ibound != 1) || idir < 1 || idir > 3) {
    set_error("snac_set_open_bc_p: bad argument");
    return SNAC_ERR_ARG;
  }
  if (!extents(lo, hi, n, "snac_set_open_bc_p")) return SNAC_ERR_ARG;
  if (n[idir - 1] < 2) { set_error("snac_set_open_bc_p: the face's axis needs two cells"); return SNAC_ERR_ARG; }
  ArgArray P;
  SNAC_TRY(P.bind(p, halo_bytes(n), true, true));
  OpenArgs a = {};
  a.op = OP_P; a.ib = ibound; a.ax = idir - 1;
  for (int q = 0; q < 3; q++) a.n[q] = n[q];
  a.drc0 = drc[0]; a.drc1 = drc[1]; a.drf = drf; a.alpha = alpha;
  a.p = (double *)P.dev;
  a.bchk = bounds_flag();
  SNAC_TRY(launch_open(a));
  SNAC_CUDA(cudaDeviceSynchronize());
  SNAC_TRY(bounds_check(0));
  SNAC_TRY(P.finish());
  return SNAC_OK;
}

// cmpt_estimated_traction (bound.f90:377-436): the traction plane from the cell next to the boundary cell
int snac_cmpt_estimated_traction(int ibound, const int lo[3], const int hi[3], int idir, double visc, double dr,
                                 const double *u, const double *v, const double *w, const double *p, double *tr) {
  int n[3];
  if (!lo || !hi || !u || !v || !w || !p || !tr || (ibound != 0 && ibound != 1) || idir < 1 || idir > 3) {
    set_error("snac_cmpt_estimated_traction: bad argument");
    return SNAC_ERR_ARG;
  }
  if (!extents(lo, hi, n, "snac_cmpt_estimated_traction")) return SNAC_ERR_ARG;
  const int ax = idir - 1;
  if (n[ax] < 2) { set_error("snac_cmpt_estimated_traction: the face's axis needs two cells"); return SNAC_ERR_ARG; }
  const double *f = ax == 0 ? u : (ax == 1 ? v : w);
  ArgArray F, P, T;
  SNAC_TRY(F.bind(f, halo_bytes(n), true, false));
  SNAC_TRY(P.bind(p, halo_bytes(n), true, false));
  SNAC_TRY(T.bind(tr, plane_bytes(n, ax), true, true));
  OpenArgs a = {};
  a.op = OP_TRACTION; a.ib = ibound; a.ax = ax;
  for (int q = 0; q < 3; q++) a.n[q] = n[q];
  a.visc = visc; a.dr = dr;
  a.f = (double *)F.dev; a.p = (double *)P.dev; a.tr = (double *)T.dev;
  a.bchk = bounds_flag();
  SNAC_TRY(launch_open(a));
  SNAC_CUDA(cudaDeviceSynchronize());
  SNAC_TRY(bounds_check(0));
  SNAC_TRY(T.finish());
  return SNAC_OK;
}

// outflow (bound.f90:479-515): on every outflow face, in the reference's order, the traction plane zeroed,
// estimated when asked, then the open BC on the wall-normal velocity
int snac_outflow(const int is_outflow_bound[3][2], const int is_estimated_traction[3][2], const int lo[3],
                 const int hi[3], const double dl[3][2], const double dl_h[3][2], double visc, double *u, double *v,
                 double *w, double *p, double *tr_x, double *tr_y, double *tr_z) {
  int n[3];
  if (!is_outflow_bound || !is_estimated_traction || !lo || !hi || !dl || !dl_h || !u || !v || !w || !p || !tr_x ||
      !tr_y || !tr_z) {
    set_error("snac_outflow: null argument");
    return SNAC_ERR_ARG;
  }
  if (!extents(lo, hi, n, "snac_outflow")) return SNAC_ERR_ARG;
  for (int ax = 0; ax < 3; ax++)
    if (n[ax] < 2 && (is_outflow_bound[ax][0] || is_outflow_bound[ax][1])) {
      set_error("snac_outflow: an outflow face's axis needs two cells");
      return SNAC_ERR_ARG;
    }
  double *fh[3] = {u, v, w}, *trh[3] = {tr_x, tr_y, tr_z};
  ArgArray F[3], P, T[3];
  for (int ax = 0; ax < 3; ax++) {
    SNAC_TRY(F[ax].bind(fh[ax], halo_bytes(n), true, true));
    SNAC_TRY(T[ax].bind(trh[ax], plane_bytes(n, ax), true, true));
  }
  SNAC_TRY(P.bind(p, halo_bytes(n), true, false));
  for (int ax = 0; ax < 3; ax++)
    for (int ib = 0; ib < 2; ib++) {
      if (!is_outflow_bound[ax][ib]) continue;
      const int t1 = ax == 0 ? 1 : 0, t2 = ax == 2 ? 1 : 2;
      const size_t plane = (size_t)(n[t1] + 2) * (n[t2] + 2);
      SNAC_CUDA(cudaMemset((double *)T[ax].dev + plane * ib, 0, plane * sizeof(double)));
      OpenArgs a = {};
      a.ib = ib; a.ax = ax;
      for (int q = 0; q < 3; q++) a.n[q] = n[q];
      a.visc = visc;
      a.f = (double *)F[ax].dev; a.p = (double *)P.dev; a.tr = (double *)T[ax].dev;
      a.bchk = bounds_flag();
      if (is_estimated_traction[ax][ib]) {
        a.op = OP_TRACTION;
        a.dr = dl_h[ax][ib];
        SNAC_TRY(launch_open(a));
      }
      a.op = OP_UVW;
      a.dr = dl[ax][ib];
      SNAC_TRY(launch_open(a));
    }
  SNAC_CUDA(cudaDeviceSynchronize());
  SNAC_TRY(bounds_check(0));
  for (int ax = 0; ax < 3; ax++) {
    SNAC_TRY(F[ax].finish());
    SNAC_TRY(T[ax].finish());
  }
  return SNAC_OK;
}

// outflow_p (bound.f90:517-541): the traction BC on the correction pressure at every outflow face
int snac_outflow_p(const int is_outflow_bound[3][2], const int lo[3], const int hi[3], const double dlc[3][2][2],
                   const double dlf[3][2], double alpha, double *p) {
  int n[3];
  if (!is_outflow_bound || !lo || !hi || !dlc || !dlf || !p) { set_error("snac_outflow_p: null argument"); return SNAC_ERR_ARG; }
  if (!extents(lo, hi, n, "snac_outflow_p")) return SNAC_ERR_ARG;
  for (int ax = 0; ax < 3; ax++)
    if (n[ax] < 2 && (is_outflow_bound[ax][0] || is_outflow_bound[ax][1])) {
      set_error("snac_outflow_p: an outflow face's axis needs two cells");
      return SNAC_ERR_ARG;
    }
  ArgArray P;
  SNAC_TRY(P.bind(p, halo_bytes(n), true, true));
  for (int ax = 0; ax < 3; ax++)
    for (int ib = 0; ib < 2; ib++) {
      if (!is_outflow_bound[ax][ib]) continue;
      OpenArgs a = {};
      a.op = OP_P; a.ib = ib; a.ax = ax;
      for (int q = 0; q < 3; q++) a.n[q] = n[q];
      a.drc0 = dlc[ax][ib][0]; a.drc1 = dlc[ax][ib][1]; a.drf = dlf[ax][ib]; a.alpha = alpha;
      a.p = (double *)P.dev;
      a.bchk = bounds_flag();
      SNAC_TRY(launch_open(a));
    }
  SNAC_CUDA(cudaDeviceSynchronize());
  SNAC_TRY(bounds_check(0));
  SNAC_TRY(P.finish());
  return SNAC_OK;
}
