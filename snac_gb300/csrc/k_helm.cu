// k_helm.cu -- the IMPDIFF Helmholtz solves of u, v, w and the scalars (3-D solve).
//
// solve_impdiff_field_3d (solve_helmholtz.f90:109-138) per field:
//   phi <- phi * alphai * dx2 dy2 dz2           (the field's control volume, over lo..hi)
//   phi <- phi + BC planes at the boundary cells  (updt_rhs, bound.f90:543-585, over lo..hif)
//   (A + alphai V) phi = rhs, warm-started from the previous solution
// where hif is hi minus one along a velocity component's own direction at a wall there.  The
// scaling and the planes are one kernel over the domain's tiles; gather/scatter move the field
// between the blocks and the solver box over lo..hif.
#include "snac_host.h"
#include "snac_solver.h"

namespace snac {

// per-block tables of a Helmholtz solver
struct HelmBlk {
  const double *rx, *ry, *rz;  // BC planes rhs?(.., .., 0:1) over the field's extents nf
  int nf[3];                   // solved cells per axis (hif - lo + 1)
  int isb[6];                  // is_bound, side fastest
  int boff[3];                 // offset of the block in the solver box
  int cen[3];                  // centred along each axis (else staggered)
  int wskip;                   // transform axis, left out of the weight (-1: 3-D solve)
};

__device__ inline double *helm_field(const DBlock &B, int field) {
  if (field == HF_U) return B.u;
  if (field == HF_U + 1) return B.v;
  if (field == HF_U + 2) return B.w;
  return B.s[field - HF_S0];
}

__global__ void __launch_bounds__(TX * TY * TZ)
k_helm_rhs(const DBlock *__restrict__ Bs, const Tile *__restrict__ T, const HelmBlk *__restrict__ HB, int field,
           double alphai) {
  const Tile t = T[blockIdx.x];
  const DBlock &B = Bs[t.x];
  const HelmBlk &H = HB[t.x];
  const int i = t.y + (int)threadIdx.x, j = t.z + (int)threadIdx.y, k = t.w + (int)threadIdx.z;
  if (i >= B.n[0] || j >= B.n[1] || k >= B.n[2]) return;  // the scaling runs over lo..hi
  double *__restrict__ f = helm_field(B, field);
  const long c = hidx(i, j, k, B.n[0], B.n[1]);
  double v = f[c] * alphai;
  if (H.wskip != 0) v = v * AX(B, 0, H.cen[0] ? AX_DF : AX_DC, i);
  if (H.wskip != 1) v = v * AX(B, 1, H.cen[1] ? AX_DF : AX_DC, j);
  if (H.wskip != 2) v = v * AX(B, 2, H.cen[2] ? AX_DF : AX_DC, k);
  const int n0 = H.nf[0], n1 = H.nf[1], n2 = H.nf[2];
  if (i >= n0 || j >= n1 || k >= n2) { f[c] = v; return; }  // the planes only over lo..hif
  if (H.isb[0] && i == 0) v += H.rx[j + (long)n1 * (k + (long)n2 * 0)];
  if (H.isb[1] && i == n0 - 1) v += H.rx[j + (long)n1 * (k + (long)n2 * 1)];
  if (H.isb[2] && j == 0) v += H.ry[i + (long)n0 * (k + (long)n2 * 0)];
  if (H.isb[3] && j == n1 - 1) v += H.ry[i + (long)n0 * (k + (long)n2 * 1)];
  if (H.isb[4] && k == 0) v += H.rz[i + (long)n0 * (j + (long)n1 * 0)];
  if (H.isb[5] && k == n2 - 1) v += H.rz[i + (long)n0 * (j + (long)n1 * 1)];
  f[c] = v;
}

// field <-> solver box (3-D mode, one system) over the solved cells
__global__ void __launch_bounds__(TX * TY * TZ)
k_helm_io(const DBlock *__restrict__ Bs, const Tile *__restrict__ T, const HelmBlk *__restrict__ HB, int field, int bn0,
          int bn1, double *box, int to_box) {
  const Tile t = T[blockIdx.x];
  const DBlock &B = Bs[t.x];
  const HelmBlk &H = HB[t.x];
  const int i = t.y + (int)threadIdx.x, j = t.z + (int)threadIdx.y, k = t.w + (int)threadIdx.z;
  if (i >= H.nf[0] || j >= H.nf[1] || k >= H.nf[2]) return;
  double *__restrict__ f = helm_field(B, field);
  const long c = hidx(i, j, k, B.n[0], B.n[1]);
  const long cell = (long)(i + H.boff[0]) + (long)bn0 * ((long)(j + H.boff[1]) + (long)bn1 * (k + H.boff[2]));
  if (to_box) box[cell] = f[c];
  else f[c] = box[cell];
}

// shift of every system: alphai (3-D) or lambda_k + alphai (per wavenumber)
__global__ void k_set_shift(double *shift, float *shiftf, const double *lambda, int nsys, double alphai) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nsys) return;
  const double v = lambda ? lambda[k] + alphai : alphai;
  shift[k] = v;
  shiftf[k] = (float)v;
}

int helm_upload_tables(Domain &d, PoissonSolver &S, const std::vector<std::vector<double>> (&planes)[3]) {
  std::vector<HelmBlk> hb(d.nblocks);
  for (int b = 0; b < d.nblocks; b++) {
    const HostBlock &H = d.hb[b];
    HelmBlk &e = hb[b];
    for (int a = 0; a < 3; a++) {
      e.nf[a] = field_hi(H, S.field, a) - H.lo[a] + 1;
      e.boff[a] = H.lo[a] - S.lo_min[a];
      e.cen[a] = field_centered(S.field, a);
      e.wskip = S.fft_axis ? S.fft_axis - 1 : -1;
      for (int s = 0; s < 2; s++) e.isb[2 * a + s] = H.is_bound[a][s];
    }
    const double **dst[3] = {&e.rx, &e.ry, &e.rz};
    for (int a = 0; a < 3; a++) {
      const auto &v = planes[a][b];
      double *p = (double *)S.alloc(std::max<size_t>(1, v.size()) * sizeof(double));
      if (!p) { set_error("device allocation failed (Helmholtz BC planes)"); return SNAC_ERR_NOMEM; }
      if (!v.empty()) SNAC_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice));
      *dst[a] = p;
    }
  }
  S.d_hb = (HelmBlk *)S.alloc(hb.size() * sizeof(HelmBlk));
  if (!S.d_hb) { set_error("device allocation failed (Helmholtz tables)"); return SNAC_ERR_NOMEM; }
  SNAC_CUDA(cudaMemcpy(S.d_hb, hb.data(), hb.size() * sizeof(HelmBlk), cudaMemcpyHostToDevice));
  return SNAC_OK;
}

int helm_rhs(Domain &d, PoissonSolver &S, double alphai, cudaStream_t st) {
  k_helm_rhs<<<d.ntiles, dim3(TX, TY, TZ), 0, st>>>(d.d_db, d.d_tiles, S.d_hb, S.field, alphai), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

// the diagonal shift of this solve (add_weighted_constant_to_diagonal / _n_diagonals): the 1/diagonal
// tables of the plane smoothers follow it
int helm_shift(PoissonSolver &S, double alphai, cudaStream_t st) {
  const int ns = S.nsys;
  k_set_shift<<<(ns + 127) / 128, 128, 0, st>>>(const_cast<double *>(S.P.shift), const_cast<float *>(S.P.shiftf),
                                                S.fft_axis ? S.d_lambda : nullptr, ns, alphai), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  if (!S.mode3d) SNAC_TRY(plane_make_invd(S.P, S.invd_tab, S.invd_tabf, st));
  return SNAC_OK;
}

int helm_io(Domain &d, PoissonSolver &S, double *box, int to_box, cudaStream_t st) {
  k_helm_io<<<d.ntiles, dim3(TX, TY, TZ), 0, st>>>(d.d_db, d.d_tiles, S.d_hb, S.field, S.P.L[0].n[0], S.P.L[0].n[1],
                                                   box, to_box), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

}  // namespace snac
