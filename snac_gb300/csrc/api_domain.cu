// api_domain.cu -- domain layer of the C ABI: all blocks resident in HBM.
//
// snac_init restates the set-up of main.f90:188-886 that the hot path needs:
// block placement in the global index space (initmpi.f90:50-98), neighbours
// (initmpi.f90:150-237), grids (initgrid.f90:9-165 with bound_grid), the
// pressure BC planes (solver.f90:44-157) and the solver set-up.  snac_step
// runs the RK3 loop of main.f90:893-1069.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "snac_host.h"

namespace snac {

static const double RKC[3][2] = {{32.0 / 60.0, 0.0}, {25.0 / 60.0, -17.0 / 60.0}, {45.0 / 60.0, -25.0 / 60.0}};

static Domain *g_dom = nullptr;
Domain *domain() { return g_dom; }

void *Domain::alloc(size_t bytes) {
  void *p = nullptr;
  if (cudaMalloc(&p, bytes ? bytes : 8) != cudaSuccess) return nullptr;
  cudaMemset(p, 0, bytes ? bytes : 8);
  allocs.push_back(p);
  return p;
}
Domain::~Domain() {
  if (guess) guess_destroy(guess);
  tma_destroy(*this);
  ps.reset();
  for (auto &h : hs) h.reset();
  for (void *p : allocs) cudaFree(p);
  if (h_red) cudaFreeHost(h_red);
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  if (st) cudaStreamDestroy(st);
  if (st_copy) cudaStreamDestroy(st_copy);
}

// ---- initgrid.f90:171-287 ----
static double gp_geo_one_end(double alpha, double r0) {
  if (r0 == 1.0) return r0;
  return r0 * std::pow((1.0 - std::pow(r0, alpha)) / (1.0 - r0) / alpha, 1.0 / 3.0);
}
static double gridpoint(int gt, double alpha, double r0) {
  switch (gt) {
    case 1: return alpha != 0.0 ? 1.0 * (1.0 + std::tanh((r0 - 1.0) * alpha) / std::tanh(alpha / 1.0)) : r0;
    case 2:
      if (alpha == 0.0) return r0;
      if (r0 <= 0.5) return 0.5 * (1.0 - 1.0 + std::tanh(2.0 * alpha * (r0 - 0.0)) / std::tanh(alpha));
      return 0.5 * (1.0 + 1.0 + std::tanh(2.0 * alpha * (r0 - 1.0)) / std::tanh(alpha));
    case 3: return alpha != 0.0 ? 1.0 - 1.0 * (1.0 + std::tanh((1.0 - r0 - 1.0) * alpha) / std::tanh(alpha / 1.0)) : r0;
    case 4: return gp_geo_one_end(alpha, r0);
    case 5: return 1.0 - gp_geo_one_end(alpha, 1.0 - r0);
    case 6:
      if (r0 <= 0.5) return gp_geo_one_end(alpha / 2.0, 2.0 * r0) / 2.0;
      return 1.0 - gp_geo_one_end(alpha / 2.0, 2.0 * (1.0 - r0)) / 2.0;
    case 7:
      if (r0 <= 0.5) return (1.0 - gp_geo_one_end(alpha / 2.0, (0.5 - r0) * 2.0)) / 2.0;
      return (1.0 + gp_geo_one_end(alpha / 2.0, (r0 - 0.5) * 2.0)) / 2.0;
    default: return alpha != 0.0 ? 0.5 * (1.0 + std::tanh((r0 - 0.5) * alpha) / std::tanh(alpha / 2.0)) : r0;
  }
}

// initgrid.f90:9-83
void initgrid(int lo, int hi, int gt, double gr, double lmin, double lmax, double *drc, double *drf, double *rc,
              double *rf) {
  auto at = [&](double *a, int q) -> double & { return a[q - lo + 1]; };
  const int n = hi - lo + 1;
  for (int q = lo; q <= hi; q++) {
    const double r0 = ((double)(q - lo + 1) - 0.0) / (1.0 * n);
    at(rf, q) = gridpoint(gt, gr, r0);
    at(rf, q) = lmin + at(rf, q) * (lmax - lmin);
  }
  at(rf, lo - 1) = lmin;
  for (int q = lo; q <= hi; q++) at(drf, q) = at(rf, q) - at(rf, q - 1);
  at(drf, lo - 1) = at(drf, lo);
  at(drf, hi + 1) = at(drf, hi);
  for (int q = lo - 1; q <= hi; q++) at(drc, q) = 0.5 * (at(drf, q) + at(drf, q + 1));
  at(drc, hi + 1) = at(drc, hi);
  at(rc, lo - 1) = lmin - at(drc, lo - 1) / 2.0;
  at(rf, lo - 1) = lmin;
  for (int q = lo; q <= hi + 1; q++) {
    at(rc, q) = at(rc, q - 1) + at(drc, q - 1);
    at(rf, q) = at(rf, q - 1) + at(drf, q);
  }
}

// initgrid.f90:144-165 (load_grid)
static void load_grid(int lo, int hi, const double *file, double *rf, double *rc, double *drf, double *drc) {
  auto at = [&](double *a, int q) -> double & { return a[q - lo + 1]; };
  const int n = hi - lo + 1;
  for (int q = lo; q <= hi; q++) {
    at(rf, q) = file[q - lo];
    at(rc, q) = file[n + q - lo];
    at(drf, q) = file[2 * n + q - lo];
    at(drc, q) = file[3 * n + q - lo];
  }
  at(drf, lo - 1) = at(drf, lo);
  at(drf, hi + 1) = at(drf, hi);
  at(drc, lo - 1) = at(drf, lo);
  at(drc, hi + 1) = at(drc, hi);
  at(rf, lo - 1) = at(rf, lo) - at(drf, lo);
  at(rf, hi + 1) = at(rf, hi) + at(drf, hi);
  at(rc, lo - 1) = at(rc, lo) - at(drc, lo - 1);
  at(rc, hi + 1) = at(rc, hi) + at(drc, hi);
}

// fft.f90:96-149
void find_fft(char a, char b, int is_centered, int *kf, int *kb, double norm[2]) {
  *kf = *kb = -1;
  norm[0] = norm[1] = 0.0;
  auto set = [&](int f, int bw, double n0, double n1) { *kf = f; *kb = bw; norm[0] = n0; norm[1] = n1; };
  if (is_centered) {
    if (a == 'F' && b == 'F') set(SNAC_R2HC, SNAC_HC2R, 1, 0);
    else if (a == 'N' && b == 'N') set(SNAC_REDFT10, SNAC_REDFT01, 2, 0);
    else if (a == 'D' && b == 'D') set(SNAC_RODFT10, SNAC_RODFT01, 2, 0);
    else if (a == 'N' && b == 'D') set(SNAC_REDFT11, SNAC_REDFT11, 2, 0);
    else if (a == 'D' && b == 'N') set(SNAC_RODFT11, SNAC_RODFT11, 2, 0);
  } else {
    if (a == 'F' && b == 'F') set(SNAC_R2HC, SNAC_HC2R, 1, 0);
    else if (a == 'N' && b == 'N') set(SNAC_REDFT00, SNAC_REDFT00, 2, -1);
    else if (a == 'D' && b == 'D') set(SNAC_RODFT00, SNAC_RODFT00, 2, 1);
    else if (a == 'N' && b == 'D') set(SNAC_REDFT10, SNAC_REDFT01, 2, 0);
    else if (a == 'D' && b == 'N') set(SNAC_RODFT01, SNAC_RODFT10, 2, 0);
  }
}

// fft.f90:151-189; the reference defines no 'DN' case (returns -1 here)
int eigenvalues(int n, char a, char b, int is_centered, double *lambda) {
  const double PI = 3.14159265358979323846264338327950288;
  auto s2 = [](double x) { const double s = std::sin(x); return -4.0 * s * s; };
  if (a == 'F' && b == 'F') for (int l = 1; l <= n; l++) lambda[l - 1] = s2((1.0 * (l - 1)) * PI / (1.0 * n));
  else if (a == 'N' && b == 'N') {
    if (is_centered) for (int l = 1; l <= n; l++) lambda[l - 1] = s2((1.0 * (l - 1)) * PI / (2.0 * n));
    else for (int l = 1; l <= n; l++) lambda[l - 1] = s2((1.0 * (l - 1)) * PI / (2.0 * (n - 1 + 1)));
  } else if (a == 'D' && b == 'D') {
    if (is_centered) for (int l = 1; l <= n; l++) lambda[l - 1] = s2((1.0 * (l - 0)) * PI / (2.0 * n));
    else { for (int l = 1; l <= n - 1; l++) lambda[l - 1] = s2((1.0 * (l - 0)) * PI / (2.0 * (n + 1 - 1))); lambda[n - 1] = 0.0; }
  } else if (a == 'N' && b == 'D') for (int l = 1; l <= n; l++) lambda[l - 1] = s2((1.0 * (2 * l - 1)) * PI / (4.0 * n));
  else return -1;
  return 0;
}

// solver.f90:44-157 (init_bc_rhs) for the pressure, centred in every direction
static void init_bc_rhs_p(const HostBlock &H, const int periods[3], int fft_axis, std::vector<double> rhs[3]) {
  const int nx = H.ng[0], ny = H.ng[1], nz = H.ng[2];
  rhs[0].assign((size_t)ny * nz * 2, 0.0);
  rhs[1].assign((size_t)nx * nz * 2, 0.0);
  rhs[2].assign((size_t)nx * ny * 2, 0.0);
  double factor[3][2];
  for (int q = 0; q < 3; q++)
    for (int s = 0; s < 2; s++) {
      factor[q][s] = 0.0;
      if (!H.is_bound[q][s]) continue;
      const char cb = H.desc.cbcpre[q][s];
      const double bc = H.desc.bcpre[q][s];
      if (cb == 'N') { factor[q][s] = 1.0 * H.dl[q][s] * bc; if (s == 1) factor[q][s] = -factor[q][s]; }
      else if (cb == 'D') factor[q][s] = -2.0 * bc;
    }
  const double *dx1 = H.g[0][0].data(), *dx2 = H.g[0][1].data(), *dy1 = H.g[1][0].data(), *dy2 = H.g[1][1].data(),
               *dz1 = H.g[2][0].data(), *dz2 = H.g[2][1].data();
  auto W = [&](int i, int j, int k) {  // local 1-based indices into (n+2) arrays
    switch (fft_axis) {
      case 1: return dy2[j] * dz2[k];
      case 2: return dx2[i] * dz2[k];
      case 3: return dx2[i] * dy2[j];
      default: return dx2[i] * dy2[j] * dz2[k];
    }
  };
  for (int idir = 0; idir < 3; idir++) {
    if (periods[idir] != 0) continue;
    const int n = H.ng[idir];
    const int sides = n > 1 ? 2 : 1;
    for (int sd = 0; sd < sides; sd++) {
      const int ib = sd;
      if (!H.is_bound[idir][ib]) continue;
      const int cface = ib ? n : 1;  // local 1-based index of the boundary cell
      if (idir == 0)
        for (int k = 1; k <= nz; k++)
          for (int j = 1; j <= ny; j++)
            rhs[0][(j - 1) + (size_t)ny * ((k - 1) + (size_t)nz * ib)] = factor[0][ib] * W(cface, j, k) / (dx1[cface - (1 - ib)] * dx2[cface]);
      else if (idir == 1)
        for (int k = 1; k <= nz; k++)
          for (int i = 1; i <= nx; i++)
            rhs[1][(i - 1) + (size_t)nx * ((k - 1) + (size_t)nz * ib)] = factor[1][ib] * W(i, cface, k) / (dy1[cface - (1 - ib)] * dy2[cface]);
      else
        for (int j = 1; j <= ny; j++)
          for (int i = 1; i <= nx; i++)
            rhs[2][(i - 1) + (size_t)nx * ((j - 1) + (size_t)ny * ib)] = factor[2][ib] * W(i, j, cface) / (dz1[cface - (1 - ib)] * dz2[cface]);
    }
  }
}

// init_inflow (initflow.f90:369-429) on one face: the normal component veln and the tangential ones of the
// two in-plane axes (velt1, velt2) over (lo-1:hi+1)^2, from the block's own centre/face coordinates
static void init_inflow_face(int type, const int per[2], const int n[2], const double lmin[2], const double lmax[2],
                             const double *x1c, const double *x2c, const double *x2f, double uref, double lref,
                             double visc, std::vector<double> &veln, std::vector<double> &velt1,
                             std::vector<double> &velt2) {
  const int n1 = n[0] + 2, n2 = n[1] + 2;
  veln.assign((size_t)n1 * n2, 0.0);
  velt1.assign((size_t)n1 * n2, 0.0);
  velt2.assign((size_t)n1 * n2, 0.0);
  // poiseuille_square (initflow.f90:353-367): 6 rr (1 - rr) on [lmin, lmax]
  auto pois = [](double r, double l0, double l1) {
    const double rr = (r - l0) / (l1 - l0);
    return 6.0 * (rr * (1.0 - rr));
  };
  const double pi = std::acos(-1.0);
  if (type == 1) {  // the profile does not vary along a periodic axis (an integer power 0)
    for (int i2 = 0; i2 < n2; i2++)
      for (int i1 = 0; i1 < n1; i1++) {
        const double f1 = per[0] == 0 ? pois(x1c[i1], lmin[0], lmax[0]) : 1.0;
        const double f2 = per[1] == 0 ? pois(x2c[i2], lmin[1], lmax[1]) : 1.0;
        veln[i1 + (size_t)n1 * i2] = uref * f1 * f2;
      }
  } else if (type == 2) {  // Kovasznay flow at x0 = -0.5
    const double reb = uref * lref / visc;
    const double lambda = reb / 2.0 - std::sqrt(reb * reb / 4.0 + 4.0 * (pi * pi));
    const double x0 = -0.5;
    for (int i2 = 0; i2 < n2; i2++)
      for (int i1 = 0; i1 < n1; i1++) {
        veln[i1 + (size_t)n1 * i2] = 1.0 - std::exp(lambda * x0) * std::cos(2.0 * pi * x2c[i2]);
        velt2[i1 + (size_t)n1 * i2] = lambda / (2.0 * pi) * std::exp(lambda * x0) * std::sin(2.0 * pi * x2f[i2]);
      }
  }
}

// inflow set-up of main.f90:592-632: a face is an inflow face when it is a physical boundary, its
// inflow_type is positive and the normal velocity component is 'D'; periodic axes reject an inflow
// (chk_inflow, sanity.f90:173-189)
static int init_inflow_planes(Domain &d, const snac_block_desc *blocks) {
  for (int b = 0; b < d.nblocks; b++) {
    HostBlock &H = d.hb[b];
    for (int a = 0; a < 3; a++)
      for (int s = 0; s < 2; s++) {
        const int type = blocks[b].inflow_type[a][s];
        if (type < 0 || type > 2) { set_error("block %d: inflow_type must be 0, 1 or 2", b + 1); return SNAC_ERR_ARG; }
        if (type > 0 && d.periods[a] != 0) {
          set_error("block %d: periodicity and inflow BCs cannot be combined", b + 1);
          return SNAC_ERR_ARG;
        }
        H.inflow[a][s] = H.is_bound[a][s] && type > 0 && blocks[b].cbcvel[a][a][s] == 'D';
        if (!H.inflow[a][s]) continue;
        const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
        const int per[2] = {d.periods[t1], d.periods[t2]}, n[2] = {H.ng[t1], H.ng[t2]};
        const double lmin[2] = {blocks[b].lmin[t1], blocks[b].lmin[t2]};
        const double lmax[2] = {blocks[b].lmax[t1], blocks[b].lmax[t2]};
        init_inflow_face(type, per, n, lmin, lmax, H.g[t1][2].data(), H.g[t2][2].data(), H.g[t2][3].data(),
                         blocks[b].bcvel[a][a][s], 1.0, 1.0 / d.c.visci, H.vin[a][s][a], H.vin[a][s][t1],
                         H.vin[a][s][t2]);
      }
  }
  return SNAC_OK;
}

static int build_domain(Domain &d, const snac_case *c, const snac_block_desc *blocks) {
  d.c = *c;
  d.nblocks = c->nblocks;
  if (d.nblocks < 1) { set_error("nblocks must be >= 1"); return SNAC_ERR_ARG; }
  if (c->nscal < 0 || c->nscal > SNAC_MAX_SCAL) { set_error("nscal out of range"); return SNAC_ERR_ARG; }
  for (int q = 0; q < c->nscal; q++)
    if (!(c->alphai[q] > 0.0)) { set_error("alphai of scalar %d must be positive", q + 1); return SNAC_ERR_ARG; }
  d.hb.resize(d.nblocks);
  // placement (initmpi.f90:50-98)
  std::vector<int> done(d.nblocks, 0), unl(d.nblocks, 0);
  for (int a = 0; a < 3; a++) d.hb[0].lo[a] = 1;
  unl[0] = 1;
  int ib = 0;
  while (true) {
    bool all = true;
    for (int q = 0; q < d.nblocks; q++) if (!done[q]) all = false;
    if (all) break;
    if (ib < 0) { set_error("invalid block connectivity (unreachable block)"); return SNAC_ERR_ARG; }
    for (int idir = 0; idir < 3; idir++)
      for (int inb = 0; inb < 2; inb++) {
        if (blocks[ib].cbcpre[idir][inb] != 'F') continue;
        const int f = (int)std::lround(blocks[ib].bcpre[idir][inb]) - 1;
        if (f < 0 || f >= d.nblocks) { set_error("block %d: friend block %d does not exist", ib + 1, f + 1); return SNAC_ERR_ARG; }
        if (unl[f]) continue;
        if (inb == 0 && blocks[f].lmin[idir] > blocks[ib].lmin[idir]) continue;
        if (inb == 1 && blocks[f].lmin[idir] < blocks[ib].lmin[idir]) continue;
        const int ioff = -(1 - inb) * blocks[f].ng[idir] + inb * blocks[ib].ng[idir];
        d.hb[f].lo[idir] = d.hb[ib].lo[idir] + ioff;
        for (int t = 0; t < 3; t++) if (t != idir) d.hb[f].lo[t] = d.hb[ib].lo[t];
        unl[f] = 1;
      }
    done[ib] = 1;
    ib = -1;
    for (int q = 0; q < d.nblocks; q++) if (!done[q] && unl[q]) { ib = q; break; }
  }
  for (int b = 0; b < d.nblocks; b++) {
    HostBlock &H = d.hb[b];
    H.desc = blocks[b];
    for (int a = 0; a < 3; a++) {
      H.ng[a] = blocks[b].ng[a];
      if (H.ng[a] < 1) { set_error("block %d: ng must be >= 1", b + 1); return SNAC_ERR_ARG; }
      H.hi[a] = H.lo[a] + H.ng[a] - 1;
    }
  }
  for (int q = 0; q < 3; q++) {
    d.is_periodic[q] = 1;
    int lmn = d.hb[0].lo[q], hmx = d.hb[0].hi[q];
    for (int b = 0; b < d.nblocks; b++) {
      if (!(blocks[b].cbcpre[q][0] == 'F' && blocks[b].cbcpre[q][1] == 'F')) d.is_periodic[q] = 0;
      lmn = std::min(lmn, d.hb[b].lo[q]);
      hmx = std::max(hmx, d.hb[b].hi[q]);
    }
    d.periods[q] = d.is_periodic[q] ? hmx - lmn + 1 : 0;
  }
  for (int b = 0; b < d.nblocks; b++) {
    HostBlock &H = d.hb[b];
    for (int q = 0; q < 3; q++)
      for (int s = 0; s < 2; s++) {
        H.nb[q][s] = -1;
        if (blocks[b].cbcpre[q][s] == 'F') {
          const int f = (int)std::lround(blocks[b].bcpre[q][s]) - 1;
          const HostBlock &F = d.hb[f];
          bool ok = blocks[f].cbcpre[q][1 - s] == 'F' && (int)std::lround(blocks[f].bcpre[q][1 - s]) - 1 == b;
          for (int t = 0; t < 3; t++)
            if (t != q)
              ok = ok && F.lo[t] == H.lo[t] && F.hi[t] == H.hi[t] && blocks[f].lmin[t] == blocks[b].lmin[t] &&
                   blocks[f].lmax[t] == blocks[b].lmax[t] && blocks[f].gr[t] == blocks[b].gr[t] &&
                   blocks[f].gt[t] == blocks[b].gt[t];
          if (s == 0) ok = ok && (F.hi[q] + 1 == H.lo[q] || (d.periods[q] && F.hi[q] - H.lo[q] + 1 == d.periods[q]));
          else ok = ok && (H.hi[q] + 1 == F.lo[q] || (d.periods[q] && H.hi[q] - F.lo[q] + 1 == d.periods[q]));
          if (!ok) { set_error("block %d: inconsistent connectivity with block %d", b + 1, f + 1); return SNAC_ERR_ARG; }
          H.nb[q][s] = f;
        }
        H.is_bound[q][s] = H.nb[q][s] < 0;
      }
  }
  // grids
  for (int b = 0; b < d.nblocks; b++) {
    HostBlock &H = d.hb[b];
    for (int a = 0; a < 3; a++) {
      for (int w = 0; w < 4; w++) H.g[a][w].assign(H.ng[a] + 2, 0.0);
      initgrid(H.lo[a], H.hi[a], blocks[b].gt[a], blocks[b].gr[a], blocks[b].lmin[a], blocks[b].lmax[a],
               H.g[a][0].data(), H.g[a][1].data(), H.g[a][2].data(), H.g[a][3].data());
      if (blocks[b].grid_file[a])
        load_grid(H.lo[a], H.hi[a], blocks[b].grid_file[a], H.g[a][3].data(), H.g[a][2].data(), H.g[a][1].data(),
                  H.g[a][0].data());
      // dl(0:1,a) = drc_g(lo_g-1), drc_g(hi_g) of the block's own (unexchanged) grid, main.f90:725-727
      H.dl[a] = {H.g[a][0][0], H.g[a][0][H.ng[a]]};
    }
  }
  // bound_grid (initgrid.f90:91-127)
  std::vector<HostBlock> orig = d.hb;
  for (int b = 0; b < d.nblocks; b++) {
    HostBlock &H = d.hb[b];
    for (int a = 0; a < 3; a++) {
      const int n = H.ng[a];
      if (H.nb[a][0] >= 0) H.g[a][1][0] = orig[H.nb[a][0]].g[a][1][orig[H.nb[a][0]].ng[a]];
      if (H.nb[a][1] >= 0) H.g[a][1][n + 1] = orig[H.nb[a][1]].g[a][1][1];
      auto &df = H.g[a][1];
      auto &dc = H.g[a][0];
      dc[0] = (df[1] + df[0]) / 2.0;
      dc[n] = (df[n + 1] + df[n]) / 2.0;
      dc[n + 1] = dc[n];
    }
  }
  d.vol_all = 0.0;
  for (int b = 0; b < d.nblocks; b++)
    d.vol_all += (blocks[b].lmax[0] - blocks[b].lmin[0]) * (blocks[b].lmax[1] - blocks[b].lmin[1]) *
                 (blocks[b].lmax[2] - blocks[b].lmin[2]);
  for (int b = 0; b < d.nblocks; b++) init_bc_rhs_p(d.hb[b], d.periods, c->fft_axis, d.hb[b].rhsp);
  SNAC_TRY(init_inflow_planes(d, blocks));
  return SNAC_OK;
}

static int upload_domain(Domain &d) {
  SNAC_CUDA(cudaStreamCreateWithFlags(&d.st, cudaStreamNonBlocking));
  d.db.resize(d.nblocks);
  std::vector<std::array<int, 3>> sz, szh;
  size_t rh = 0;
  for (int b = 0; b < d.nblocks; b++) {
    HostBlock &H = d.hb[b];
    DBlock &B = d.db[b];
    memset(&B, 0, sizeof(B));
    for (int a = 0; a < 3; a++) { B.n[a] = H.ng[a]; B.lo[a] = H.lo[a]; }
    B.bchk = bounds_flag();
    const size_t nh = (size_t)(H.ng[0] + 2) * (H.ng[1] + 2) * (H.ng[2] + 2) * sizeof(double);
    const size_t ni = (size_t)H.ng[0] * H.ng[1] * H.ng[2] * sizeof(double);
    B.u = (double *)d.alloc(nh); B.v = (double *)d.alloc(nh); B.w = (double *)d.alloc(nh);
    B.p = (double *)d.alloc(nh); B.pp = (double *)d.alloc(nh);
    B.ru = (double *)d.alloc(ni); B.rv = (double *)d.alloc(ni); B.rw = (double *)d.alloc(ni);
    B.nu = (double *)d.alloc(nh); B.nv = (double *)d.alloc(nh); B.nw = (double *)d.alloc(nh);
    if (!B.u || !B.v || !B.w || !B.p || !B.pp || !B.ru || !B.nu || !B.nw) { set_error("device allocation failed (fields)"); return SNAC_ERR_NOMEM; }
    for (int q = 0; q < d.c.nscal; q++) {
      B.s[q] = (double *)d.alloc(nh);
      B.rs[q] = (double *)d.alloc(ni);
      if (!B.s[q] || !B.rs[q]) { set_error("device allocation failed (scalars)"); return SNAC_ERR_NOMEM; }
    }
    if (d.c.nscal > 0 && !(B.ns = (double *)d.alloc(ni))) { set_error("device allocation failed (scalars)"); return SNAC_ERR_NOMEM; }
    for (int a = 0; a < 3; a++) {
      auto t = axis_tables(H.g[a][0].data(), H.g[a][1].data(), H.ng[a]);
      double *p = (double *)d.alloc(t.size() * sizeof(double));
      if (!p) return SNAC_ERR_NOMEM;
      SNAC_CUDA(cudaMemcpy(p, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice));
      B.ax[a] = p;
    }
    sz.push_back({H.ng[0], H.ng[1], H.ng[2]});
    szh.push_back({H.ng[0] + 2, H.ng[1] + 2, H.ng[2] + 2});
    d.rhsp_off.push_back(rh);
    rh += H.rhsp[0].size() + H.rhsp[1].size() + H.rhsp[2].size();
  }
  for (int par = 0; par < 2; par++) {  // the block table as set up, and with u, v, w and nu, nv, nw swapped
    std::vector<DBlock> t = d.db;
    if (par)
      for (auto &B : t) { std::swap(B.u, B.nu); std::swap(B.v, B.nv); std::swap(B.w, B.nw); }
    d.d_db_set[par] = (DBlock *)d.alloc(d.nblocks * sizeof(DBlock));
    if (!d.d_db_set[par]) { set_error("device allocation failed (block table)"); return SNAC_ERR_NOMEM; }
    SNAC_CUDA(cudaMemcpy(d.d_db_set[par], t.data(), d.nblocks * sizeof(DBlock), cudaMemcpyHostToDevice));
  }
  d.uvw_par = 0;
  d.d_db = d.d_db_set[0];
  auto tl = make_tiles(sz, TX, TY, TZ), th = make_tiles(szh, TX, TY, TZ);
  d.ntiles = (int)tl.size();
  d.ntiles_halo = (int)th.size();
  d.d_tiles = (Tile *)d.alloc(tl.size() * sizeof(Tile));
  d.d_tiles_halo = (Tile *)d.alloc(th.size() * sizeof(Tile));
  SNAC_CUDA(cudaMemcpy(d.d_tiles, tl.data(), tl.size() * sizeof(Tile), cudaMemcpyHostToDevice));
  SNAC_CUDA(cudaMemcpy(d.d_tiles_halo, th.data(), th.size() * sizeof(Tile), cudaMemcpyHostToDevice));
  // pressure BC planes
  std::vector<double> allr;
  for (int b = 0; b < d.nblocks; b++)
    for (int a = 0; a < 3; a++) allr.insert(allr.end(), d.hb[b].rhsp[a].begin(), d.hb[b].rhsp[a].end());
  d.d_rhsp = (double *)d.alloc(allr.size() * sizeof(double));
  SNAC_CUDA(cudaMemcpy(d.d_rhsp, allr.data(), allr.size() * sizeof(double), cudaMemcpyHostToDevice));
  // halo links
  for (int a = 0; a < 3; a++) {
    std::vector<FaceLink> fl;
    const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
    int mp = 0;
    for (int b = 0; b < d.nblocks; b++) {
      for (int s = 0; s < 2; s++)
        if (d.hb[b].nb[a][s] >= 0) fl.push_back({b, d.hb[b].nb[a][s], s, 0});
      mp = std::max(mp, (d.hb[b].ng[t1] + 2) * (d.hb[b].ng[t2] + 2));
    }
    d.nlinks[a] = (int)fl.size();
    d.maxplane[a] = mp;
    d.d_links[a] = (FaceLink *)d.alloc(std::max<size_t>(1, fl.size()) * sizeof(FaceLink));
    if (!fl.empty()) SNAC_CUDA(cudaMemcpy(d.d_links[a], fl.data(), fl.size() * sizeof(FaceLink), cudaMemcpyHostToDevice));
  }
  // inflow faces per axis and side
  for (int a = 0; a < 3; a++)
    for (int s = 0; s < 2; s++) {
      std::vector<InflowFace> fc;
      const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
      for (int b = 0; b < d.nblocks; b++) {
        HostBlock &H = d.hb[b];
        if (!H.inflow[a][s]) continue;
        InflowFace F{b, 0, {nullptr, nullptr, nullptr}};
        for (int comp = 0; comp < 3; comp++) {
          const auto &v = H.vin[a][s][comp];
          double *p = (double *)d.alloc(v.size() * sizeof(double));
          if (!p) { set_error("device allocation failed (inflow planes)"); return SNAC_ERR_NOMEM; }
          SNAC_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice));
          F.pl[comp] = p;
        }
        fc.push_back(F);
        d.inflow_plane[a][s] = std::max(d.inflow_plane[a][s], (H.ng[t1] + 2) * (H.ng[t2] + 2));
      }
      d.ninflow[a][s] = (int)fc.size();
      if (fc.empty()) continue;
      d.d_inflow[a][s] = (InflowFace *)d.alloc(fc.size() * sizeof(InflowFace));
      if (!d.d_inflow[a][s]) { set_error("device allocation failed (inflow faces)"); return SNAC_ERR_NOMEM; }
      SNAC_CUDA(cudaMemcpy(d.d_inflow[a][s], fc.data(), fc.size() * sizeof(InflowFace), cudaMemcpyHostToDevice));
    }
  int flds[5 + SNAC_MAX_SCAL];
  for (int q = 0; q < 5 + SNAC_MAX_SCAL; q++) flds[q] = q;
  d.d_flds = (int *)d.alloc(sizeof(flds));
  SNAC_CUDA(cudaMemcpy(d.d_flds, flds, sizeof(flds), cudaMemcpyHostToDevice));
  // boundary-condition tables (bound.f90:36-105)
  for (int kind = 0; kind < 4 + d.c.nscal; kind++)
    for (int a = 0; a < 3; a++) {
      std::vector<BcEntry> E;
      for (int b = 0; b < d.nblocks; b++) {
        const HostBlock &H = d.hb[b];
        const int nf = kind < 2 ? 3 : 1;
        for (int fi = 0; fi < nf; fi++) {
          BcEntry e;
          memset(&e, 0, sizeof(e));
          e.b = b;
          e.f = kind < 2 ? fi : (kind == 2 ? 3 : (kind == 3 ? 4 : 5 + (kind - 4)));
          bool any = false;
          for (int s = 0; s < 2; s++) {
            e.mode[s] = BC_NONE;
            if (!H.is_bound[a][s]) continue;
            char ct;
            double val, dr;
            int centered;
            if (kind < 2) {
              centered = fi != a;
              if (!centered && kind == 1) continue;  // is_correc skips the wall-normal component
              ct = H.desc.cbcvel[fi][a][s];
              val = H.desc.bcvel[fi][a][s];
              dr = centered ? H.g[a][0][s ? H.ng[a] : 0] : H.g[a][1][s ? H.ng[a] : 0];
            } else if (kind < 4) {
              centered = 1;
              ct = H.desc.cbcpre[a][s];
              val = H.desc.bcpre[a][s];
              dr = H.g[a][0][s ? H.ng[a] : 0];
            } else {  // scalar kind-4: its own cbc/bc (main.f90:936, boundp(s%cbc, ..., s%bc, ...))
              centered = 1;
              ct = H.desc.cbcscal[kind - 4][a][s];
              val = H.desc.bcscal[kind - 4][a][s];
              dr = H.g[a][0][s ? H.ng[a] : 0];
            }
            bc_mode(ct, s, centered, val, dr, &e.mode[s], &e.factor[s], &e.sgn[s]);
            any = any || e.mode[s] != BC_NONE;
          }
          if (any) E.push_back(e);
        }
      }
      d.nbc[kind][a] = (int)E.size();
      d.d_bc[kind][a] = (BcEntry *)d.alloc(std::max<size_t>(1, E.size()) * sizeof(BcEntry));
      if (!E.empty()) SNAC_CUDA(cudaMemcpy(d.d_bc[kind][a], E.data(), E.size() * sizeof(BcEntry), cudaMemcpyHostToDevice));
    }
  d.d_part = (double *)d.alloc((size_t)std::max(d.ntiles, 1) * 2 * sizeof(double));
  d.d_red = (double *)d.alloc(4 * sizeof(double));
  SNAC_CUDA(cudaMallocHost(&d.h_red, 4 * sizeof(double)));
  return SNAC_OK;
}

static int bound_uvw(Domain &d, int is_correc) {
  for (int a = 0; a < 3; a++)
    SNAC_TRY(launch_exchange(d.d_db, d.d_links[a], d.nlinks[a], d.d_flds, 3, a, d.maxplane[a], d.st));
  for (int a = 0; a < 3; a++) SNAC_TRY(launch_setbc(d.d_db, d.d_bc[is_correc ? 1 : 0][a], d.nbc[is_correc ? 1 : 0][a], a, d.maxplane[a], d.st));
  return SNAC_OK;
}

// inflow (bound.f90:438-477) on every inflow face, x0, x1, y0, y1, z0, z1
static int inflow_all(Domain &d, int is_correc) {
  for (int a = 0; a < 3; a++)
    for (int s = 0; s < 2; s++)
      SNAC_TRY(launch_inflow(d.d_db, d.d_inflow[a][s], d.ninflow[a][s], a, s, d.inflow_plane[a][s], is_correc, d.st));
  return SNAC_OK;
}

static int bound_p(Domain &d, int field) {
  const bool scal = field >= SNAC_S0 && field < SNAC_S0 + d.c.nscal;
  const int fsel = field == SNAC_P ? 3 : (scal ? 5 + (field - SNAC_S0) : 4);
  const int kind = field == SNAC_P ? 2 : (scal ? 4 + (field - SNAC_S0) : 3);
  for (int a = 0; a < 3; a++) SNAC_TRY(launch_exchange(d.d_db, d.d_links[a], d.nlinks[a], d.d_flds + fsel, 1, a, d.maxplane[a], d.st));
  for (int a = 0; a < 3; a++) SNAC_TRY(launch_setbc(d.d_db, d.d_bc[kind][a], d.nbc[kind][a], a, d.maxplane[a], d.st));
  return SNAC_OK;
}

static int updt_rhs_all(Domain &d) {
  for (int b = 0; b < d.nblocks; b++) {
    const HostBlock &H = d.hb[b];
    int isb[6];
    for (int a = 0; a < 3; a++) for (int s = 0; s < 2; s++) isb[2 * a + s] = H.is_bound[a][s];
    const double *rx = d.d_rhsp + d.rhsp_off[b];
    const double *ry = rx + H.rhsp[0].size();
    const double *rz = ry + H.rhsp[1].size();
    SNAC_TRY(launch_updt_rhs(H.ng[0], H.ng[1], H.ng[2], isb, rx, ry, rz, d.db[b].pp, d.st));
  }
  return SNAC_OK;
}

// one Helmholtz solve; the largest iteration count and residual of the step are kept with the pressure's
static int helm_step(Domain &d, PoissonSolver &S, double alphai) {
  const int rc = solver_solve_helmholtz(d, S, alphai);
  if (rc != SNAC_OK && rc != SNAC_ERR_NOT_CONVERGED) return rc;
  d.last_helm_iters = std::max(d.last_helm_iters, S.last_iters);
  d.last_helm_res = std::max(d.last_helm_res, S.last_res);
  if (rc == SNAC_ERR_NOT_CONVERGED) d.helm_not_converged = true;  // reported by snac_step like the pressure's
  return SNAC_OK;
}

// u, v, w and nu, nv, nw trade places on the host mirror, in the block table the kernels read and in the
// TMA-staged kernel's tensor maps
static int swap_uvw(Domain &d) {
  for (auto &B : d.db) { std::swap(B.u, B.nu); std::swap(B.v, B.nv); std::swap(B.w, B.nw); }
  d.uvw_par ^= 1;
  d.d_db = d.d_db_set[d.uvw_par];
  std::swap(d.tma, d.tma_alt);
  return SNAC_OK;
}

static int rk_mom_all(Domain &d, int irk) {
  RkMomParams prm;
  prm.f1 = RKC[irk][0] * d.dt;
  prm.f2 = RKC[irk][1] * d.dt;
  prm.f12 = prm.f1 + prm.f2;
  for (int a = 0; a < 3; a++) { prm.bforce[a] = d.c.bforce[a]; prm.gb[a] = 0.0; }
  prm.visc = 1.0 / d.c.visci;
  prm.impdiff = d.c.impdiff;
  prm.boussinesq = d.c.boussinesq && d.c.nscal > 0;  // rk.f90:104-108 with scalars(1)
  if (prm.boussinesq)
    for (int a = 0; a < 3; a++) prm.gb[a] = prm.f12 * d.c.gacc[a] * d.c.beta * 0.5;
  prm.halo_out = 1;
  SNAC_TRY(launch_rk_mom(d.d_db, d.d_tiles, d.ntiles, prm, d.st));
  // the new interior is in nu, nv, nw: give them the halo of before and let the buffers trade places (the
  // reference updates u in place, rk.f90:82-101, which leaves the same values)
  SNAC_TRY(launch_uvw_halo_copy(d.d_db, d.nblocks, std::max(d.maxplane[0], std::max(d.maxplane[1], d.maxplane[2])), d.st));
  SNAC_TRY(swap_uvw(d));
  if (d.c.impdiff) {  // main.f90:947-995: u, v, w Helmholtz solves with alphai = 1/(-visc*dtrk/2)
    const double alpha = -prm.visc * ((RKC[irk][0] + RKC[irk][1]) * d.dt) / 2.0;
    for (int comp = 0; comp < 3; comp++) SNAC_TRY(helm_step(d, *d.hs[HF_U + comp], 1.0 / alpha));
  }
  return SNAC_OK;
}

// main.f90:907-936 (explicit diffusion): rk_scal on every block with the bulk mean of all blocks
// (the MPI_ALLREDUCE of scal.f90:175), bulk_forcing_s with f = scalf - mean, then boundp of the scalar.
// The mean stays on the device: the forcing kernel reads it there.
static int rk_scal_all(Domain &d, int irk) {
  for (int q = 0; q < d.c.nscal; q++) {
    RkScalParams prm;
    prm.f1 = RKC[irk][0] * d.dt;
    prm.f2 = RKC[irk][1] * d.dt;
    prm.f12 = prm.f1 + prm.f2;
    prm.alpha = 1.0 / d.c.alphai[q];
    prm.ssource = d.c.ssource[q];
    prm.impdiff = d.c.impdiff;
    prm.sidx = q;
    const bool forced = d.c.is_sforced[q] != 0;
    SNAC_TRY(launch_rk_scal(d.d_db, d.d_tiles, d.ntiles, prm, forced ? d.d_part : nullptr, d.st));
    SNAC_TRY(launch_rk_scal_writeback(d.d_db, d.d_tiles, d.ntiles, q, d.st));
    if (forced) {
      SNAC_TRY(launch_reduce_final(d.d_part, d.ntiles, d.d_red, d.st));
      SNAC_TRY(launch_bulk_forcing_s(d.d_db, d.d_tiles, d.ntiles, q, d.c.scalf[q], 1.0 / d.vol_all, d.d_red, d.st));
    }
    if (d.c.impdiff) {  // main.f90:914-934: alpha = -s%alpha*dtrk/2, the scalar's Helmholtz solve
      const double alpha = -prm.alpha * ((RKC[irk][0] + RKC[irk][1]) * d.dt) / 2.0;
      SNAC_TRY(helm_step(d, *d.hs[HF_S0 + q], 1.0 / alpha));
    }
    SNAC_TRY(bound_p(d, SNAC_S0 + q));
  }
  return SNAC_OK;
}

static int reduce(Domain &d, int which, double out[2]) {
  if (which == 0) SNAC_TRY(launch_chkdt_partial(d.d_db, d.d_tiles, d.ntiles, d.d_part, d.st));
  else if (which == 1) SNAC_TRY(launch_chkdiv_partial(d.d_db, d.d_tiles, d.ntiles, d.vol_all, d.d_part, d.st));
  else SNAC_TRY(launch_ke_partial(d.d_db, d.d_tiles, d.ntiles, d.d_part, d.st));
  SNAC_TRY(launch_reduce_final(d.d_part, d.ntiles, d.d_red, d.st));
  SNAC_CUDA(cudaMemcpyAsync(d.h_red, d.d_red, 2 * sizeof(double), cudaMemcpyDeviceToHost, d.st));
  SNAC_CUDA(cudaStreamSynchronize(d.st));
  out[0] = d.h_red[0];
  out[1] = d.h_red[1];
  return SNAC_OK;
}

// chkdt.f90 incl. reductions; the caller's visc is max(visc, alpha_max) (main.f90:660)
static int chkdt_all(Domain &d, double *dt_cfl) {
  double r[2];
  SNAC_TRY(reduce(d, 0, r));
  double dti = r[1];
  if (std::isinf(dti)) { set_error("chkdt: non-finite velocity"); return SNAC_ERR_NAN; }
  if (dti == 0.0) dti = 1.0;
  double dtmax = std::sqrt(3.0) / dti;
  if (!d.c.impdiff) {
    double dlmin = 1e300;
    for (auto &H : d.hb)
      for (int a = 0; a < 3; a++)
        for (double v : H.g[a][1]) dlmin = std::min(dlmin, v);
    double visc = 1.0 / d.c.visci, amax = 0.0;
    for (int s = 0; s < d.c.nscal; s++) amax = std::max(amax, 1.0 / d.c.alphai[s]);
    dtmax = std::min(dtmax, 1.65 / 12.0 / std::max(visc, amax) * (dlmin * dlmin));
  }
  *dt_cfl = dtmax;
  return SNAC_OK;
}

static int set_dt_from_cfl(Domain &d) {
  double dt_cfl;
  SNAC_TRY(chkdt_all(d, &dt_cfl));
  d.dt = d.c.dt_f > 0.0 ? d.c.dt_f : std::min(d.c.cfl * dt_cfl, d.c.dtmax);
  return SNAC_OK;
}

// fillps on every block: the TMA-staged kernel where its tiled copies apply, else the plain one
static int fillps_all(Domain &d, double dtrk) {
  int done = 0;
  SNAC_TRY(launch_fillps_tma(d, dtrk, &done));
  if (!done) SNAC_TRY(launch_fillps(d.d_db, d.d_tiles, d.ntiles, dtrk, d.c.fft_axis, d.st));
  return SNAC_OK;
}

static int one_stage(Domain &d, int irk) {
  const double dtrk = (RKC[irk][0] + RKC[irk][1]) * d.dt;
  const double alpha = -(1.0 / d.c.visci) * dtrk / 2.0;
  SNAC_TRY(rk_scal_all(d, irk));
  SNAC_TRY(rk_mom_all(d, irk));
  SNAC_TRY(bound_uvw(d, 0));
  SNAC_TRY(inflow_all(d, 0));
  SNAC_TRY(fillps_all(d, dtrk));
  SNAC_TRY(updt_rhs_all(d));
  int rc = solver_solve_pressure(d, *d.ps);
  if (rc != SNAC_OK && rc != SNAC_ERR_NOT_CONVERGED) return rc;
  d.last_solve_iters = std::max(d.last_solve_iters, d.ps->last_iters);
  d.last_solve_res = std::max(d.last_solve_res, d.ps->last_res);
  d.solves++;
  SNAC_TRY(bound_p(d, SNAC_PP));
  SNAC_TRY(launch_correc(d.d_db, d.d_tiles_halo, d.ntiles_halo, dtrk, d.st));
  SNAC_TRY(bound_uvw(d, 1));
  SNAC_TRY(inflow_all(d, 1));
  SNAC_TRY(launch_updt_pressure(d.d_db, d.d_tiles, d.ntiles, alpha, d.c.impdiff, d.st));
  SNAC_TRY(bound_p(d, SNAC_P));
  return rc;
}

static int field_ptr(Domain &d, int ib, int field, double **p, size_t *bytes) {
  if (ib < 0 || ib >= d.nblocks) { set_error("block index out of range"); return SNAC_ERR_ARG; }
  DBlock &B = d.db[ib];
  const size_t nh = (size_t)(B.n[0] + 2) * (B.n[1] + 2) * (B.n[2] + 2) * sizeof(double);
  const size_t ni = (size_t)B.n[0] * B.n[1] * B.n[2] * sizeof(double);
  switch (field) {
    case SNAC_U: *p = B.u; *bytes = nh; break;
    case SNAC_V: *p = B.v; *bytes = nh; break;
    case SNAC_W: *p = B.w; *bytes = nh; break;
    case SNAC_P: *p = B.p; *bytes = nh; break;
    case SNAC_PP: *p = B.pp; *bytes = nh; break;
    case SNAC_DUDTRKO: *p = B.ru; *bytes = ni; break;
    case SNAC_DVDTRKO: *p = B.rv; *bytes = ni; break;
    case SNAC_DWDTRKO: *p = B.rw; *bytes = ni; break;
    default:
      if (field >= SNAC_S0 && field < SNAC_S0 + d.c.nscal) { *p = B.s[field - SNAC_S0]; *bytes = nh; break; }
      if (field >= SNAC_DSDTRKO0 && field < SNAC_DSDTRKO0 + d.c.nscal) {
        *p = B.rs[field - SNAC_DSDTRKO0];
        *bytes = ni;
        break;
      }
      set_error("unknown field %d", field);
      return SNAC_ERR_ARG;
  }
  return SNAC_OK;
}

}  // namespace snac

using namespace snac;

#define NEED_DOMAIN                                                         \
  Domain *d = domain();                                                     \
  if (!d) { set_error("snac_init has not been called"); return SNAC_ERR_STATE; }

extern "C" {

int snac_initgrid(int lo, int hi, int gt, double gr, double lmin, double lmax, double *drc, double *drf, double *rc,
                  double *rf) {
  if (hi < lo) { set_error("hi < lo"); return SNAC_ERR_ARG; }
  initgrid(lo, hi, gt, gr, lmin, lmax, drc, drf, rc, rf);
  return SNAC_OK;
}

int snac_find_fft(const char bc[2], int is_centered, int *kind_fwd, int *kind_bwd, double norm[2]) {
  find_fft(bc[0], bc[1], is_centered, kind_fwd, kind_bwd, norm);
  if (*kind_fwd < 0) { set_error("no transform for this boundary pair"); return SNAC_ERR_ARG; }
  return SNAC_OK;
}

int snac_eigenvalues(int n, const char bc[2], int is_centered, double *lambda) {
  if (eigenvalues(n, bc[0], bc[1], is_centered, lambda)) { set_error("the reference defines no eigenvalues for this pair"); return SNAC_ERR_UNSUPPORTED; }
  return SNAC_OK;
}

int snac_fft(int kind, int idir, const int n[3], int q, double *arr) {
  if (idir < 1 || idir > 3 || q < 0 || q > 1) { set_error("snac_fft: bad idir or q"); return SNAC_ERR_ARG; }
  ArgArray A;
  SNAC_TRY(A.bind(arr, (size_t)n[0] * n[1] * n[2] * sizeof(double), true, true));
  SNAC_TRY(r2r_array(kind, idir, n, q, (double *)A.dev, 0));
  SNAC_TRY(A.finish());
  return SNAC_OK;
}

int snac_init(const snac_case *c, const snac_block_desc *blocks, const snac_options *opt) {
  if (!c || !blocks) { set_error("snac_init: null argument"); return SNAC_ERR_ARG; }
  snac_finalize();
  auto *d = new Domain();
  if (opt) d->opt = *opt;
  g_pdl = d->opt.pdl == -1 ? 0 : 1;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { delete d; set_error("no CUDA device"); return SNAC_ERR_CUDA; }
  if (cudaSetDevice(d->opt.device) != cudaSuccess) { delete d; set_error("cannot select device %d", d->opt.device); return SNAC_ERR_CUDA; }
  int rc = build_domain(*d, c, blocks);
  if (rc == SNAC_OK) rc = upload_domain(*d);
  if (rc == SNAC_OK) {
    d->ps.reset(new PoissonSolver());
    rc = solver_create(*d, *d->ps);
  }
  // IMPDIFF (main.f90:771-869): one Helmholtz solver per velocity component and scalar
  for (int f = HF_U; rc == SNAC_OK && c->impdiff && f < HF_S0 + c->nscal; f++) {
    d->hs[f].reset(new PoissonSolver());
    rc = solver_create(*d, *d->hs[f], true, f);
  }
  if (rc == SNAC_OK) rc = tma_setup(*d);  // the TMA-staged fillps where its tiled copies apply
  if (rc != SNAC_OK) { delete d; return rc; }
  g_dom = d;
  return SNAC_OK;
}

int snac_check_case(const snac_case *c, const snac_block_desc *blocks, int *levels, long *coarse_cells) {
  if (!c || !blocks) { set_error("snac_check_case: null argument"); return SNAC_ERR_ARG; }
  Domain d;
  SNAC_TRY(build_domain(d, c, blocks));
  PoissonSolver S;
  SNAC_TRY(solver_create(d, S, false));
  if (levels) *levels = S.host_levels;
  if (coarse_cells) *coarse_cells = S.host_coarse_cells;
  return SNAC_OK;
}

int snac_finalize(void) {
  if (g_dom) {
    cudaDeviceSynchronize();
    delete g_dom;
    g_dom = nullptr;
  }
  return SNAC_OK;
}

int snac_block_geometry(int ib, int lo[3], int hi[3], int nb[3][2], int is_bound[3][2]) {
  NEED_DOMAIN
  if (ib < 0 || ib >= d->nblocks) { set_error("block index out of range"); return SNAC_ERR_ARG; }
  const HostBlock &H = d->hb[ib];
  for (int a = 0; a < 3; a++) {
    lo[a] = H.lo[a]; hi[a] = H.hi[a];
    for (int s = 0; s < 2; s++) { nb[a][s] = H.nb[a][s]; is_bound[a][s] = H.is_bound[a][s]; }
  }
  return SNAC_OK;
}

int snac_get_grid(int ib, int axis, int which, double *out) {
  NEED_DOMAIN
  if (ib < 0 || ib >= d->nblocks || axis < 0 || axis > 2 || which < 0 || which > 3) { set_error("bad grid request"); return SNAC_ERR_ARG; }
  const auto &g = d->hb[ib].g[axis][which];
  std::copy(g.begin(), g.end(), out);
  return SNAC_OK;
}

double snac_vol_all(void) { return domain() ? domain()->vol_all : 0.0; }

// ---------------------------------------------------------------- checkpoints (load.f90:92-160)
static std::string ckpt_name(const char *prefix, int ib, int field) {
  char buf[64];
  if (field >= SNAC_S0) snprintf(buf, sizeof(buf), "_b_%03d_s_%03d.bin", ib + 1, field - SNAC_S0 + 1);
  else snprintf(buf, sizeof(buf), "_b_%03d_%c.bin", ib + 1, "uvwp"[field - SNAC_U]);
  return std::string(prefix) + buf;
}

static int ckpt_fields(const Domain &d, std::vector<int> &f) {
  f = {SNAC_U, SNAC_V, SNAC_W, SNAC_P};
  for (int q = 0; q < d.c.nscal; q++) f.push_back(SNAC_S0 + q);
  return SNAC_OK;
}

int snac_checkpoint_save(const char *prefix) {
  NEED_DOMAIN
  if (!prefix) { set_error("snac_checkpoint_save: null prefix"); return SNAC_ERR_ARG; }
  std::vector<int> fl;
  ckpt_fields(*d, fl);
  SNAC_CUDA(cudaStreamSynchronize(d->st));
  for (int b = 0; b < d->nblocks; b++) {
    const int nx = d->hb[b].ng[0], ny = d->hb[b].ng[1], nz = d->hb[b].ng[2];
    std::vector<double> halo((size_t)(nx + 2) * (ny + 2) * (nz + 2)), out((size_t)nx * ny * nz + 2);
    for (int f : fl) {
      double *p; size_t bytes;
      SNAC_TRY(field_ptr(*d, b, f, &p, &bytes));
      SNAC_CUDA(cudaMemcpy(halo.data(), p, bytes, cudaMemcpyDeviceToHost));
      size_t q = 0;
      for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
          for (int i = 0; i < nx; i++) out[q++] = halo[hidx(i, j, k, nx, ny)];
      out[q++] = d->time;
      out[q++] = 1.0 * d->istep;
      const std::string name = ckpt_name(prefix, b, f);
      FILE *fp = fopen(name.c_str(), "wb");
      if (!fp) { set_error("cannot create checkpoint file %s", name.c_str()); return SNAC_ERR_IO; }
      const size_t nw = fwrite(out.data(), sizeof(double), out.size(), fp);
      const int cl = fclose(fp);
      if (nw != out.size() || cl != 0) { set_error("cannot write checkpoint file %s", name.c_str()); return SNAC_ERR_IO; }
    }
  }
  return SNAC_OK;
}

int snac_checkpoint_load(const char *prefix) {
  NEED_DOMAIN
  if (!prefix) { set_error("snac_checkpoint_load: null prefix"); return SNAC_ERR_ARG; }
  std::vector<int> fl;
  ckpt_fields(*d, fl);
  SNAC_CUDA(cudaStreamSynchronize(d->st));
  double info[2] = {0.0, 0.0};
  for (int b = 0; b < d->nblocks; b++) {
    const int nx = d->hb[b].ng[0], ny = d->hb[b].ng[1], nz = d->hb[b].ng[2];
    const size_t good = ((size_t)nx * ny * nz + 2) * sizeof(double);
    std::vector<double> halo((size_t)(nx + 2) * (ny + 2) * (nz + 2)), in((size_t)nx * ny * nz + 2);
    for (int f : fl) {
      const std::string name = ckpt_name(prefix, b, f);
      FILE *fp = fopen(name.c_str(), "rb");
      if (!fp) { set_error("cannot open checkpoint file %s", name.c_str()); return SNAC_ERR_IO; }
      fseek(fp, 0, SEEK_END);
      const long size = ftell(fp);
      fseek(fp, 0, SEEK_SET);
      if (size < 0 || (size_t)size != good) {
        fclose(fp);
        set_error("checkpoint file with incorrect size: %s | expected size: %zu | actual size: %ld", name.c_str(), good, size);
        return SNAC_ERR_IO;
      }
      const size_t nr = fread(in.data(), sizeof(double), in.size(), fp);
      fclose(fp);
      if (nr != in.size()) { set_error("cannot read checkpoint file %s", name.c_str()); return SNAC_ERR_IO; }
      double *p; size_t bytes;
      SNAC_TRY(field_ptr(*d, b, f, &p, &bytes));
      SNAC_CUDA(cudaMemcpy(halo.data(), p, bytes, cudaMemcpyDeviceToHost));
      size_t q = 0;
      for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
          for (int i = 0; i < nx; i++) halo[hidx(i, j, k, nx, ny)] = in[q++];
      SNAC_CUDA(cudaMemcpy(p, halo.data(), bytes, cudaMemcpyHostToDevice));
      info[0] = in[q];
      info[1] = in[q + 1];
    }
  }
  d->time = info[0];
  d->istep = (int)std::lround(info[1]);
  return SNAC_OK;
}

// ---------------------------------------------------------------- output (output.f90)
// spacing and coordinate tables of a field along axis a: staggered along a (u along x, ...) -> d?c and the
// face coordinates, else d?f and the centres (out1d.h90)
static bool out_staggered(int field, int a) { return field >= SNAC_U && field <= SNAC_W && field - SNAC_U == a; }

// Fortran's Ew.d edit descriptor for w = 15, d = 7 with the default scale factor: [-]0.ddddddd followed by
// E+ee (or +eee when |exponent| > 99), right-justified; the digits are the value rounded to 7 significant
// figures, as printf's %.6e rounds them
static void fortran_e15_7(double v, char out[128]) {
  char mant[32];
  int e10 = 0;
  const bool neg = std::signbit(v) && v != 0.0;
  if (v == 0.0) {
    std::snprintf(mant, sizeof(mant), "0.0000000");
  } else {
    char buf[32];
    std::snprintf(buf, sizeof(buf), "%.6e", std::fabs(v));  // d.dddddde[+-]xx
    e10 = std::atoi(buf + 9) + 1;
    std::snprintf(mant, sizeof(mant), "0.%c%.6s", buf[0], buf + 2);
  }
  char expo[24];
  if (e10 >= -99 && e10 <= 99) std::snprintf(expo, sizeof(expo), "E%c%02d", e10 < 0 ? '-' : '+', std::abs(e10));
  else std::snprintf(expo, sizeof(expo), "%c%03d", e10 < 0 ? '-' : '+', std::abs(e10));
  char body[96];
  std::snprintf(body, sizeof(body), "%s%s%s", neg ? "-" : "", mant, expo);
  std::snprintf(out, 128, "%15s", body);
}

int snac_out1d(int ib, int field, int idir, double *coord, double *prof) {
  NEED_DOMAIN
  if (ib < 0 || ib >= d->nblocks) { set_error("block index out of range"); return SNAC_ERR_ARG; }
  if (idir < 1 || idir > 3) { set_error("idir must be 1, 2 or 3"); return SNAC_ERR_ARG; }
  if (!coord || !prof) { set_error("snac_out1d: null output"); return SNAC_ERR_ARG; }
  double *f; size_t bytes;
  SNAC_TRY(field_ptr(*d, ib, field, &f, &bytes));
  if (field == SNAC_DUDTRKO || field == SNAC_DVDTRKO || field == SNAC_DWDTRKO ||
      (field >= SNAC_DSDTRKO0 && field < SNAC_DSDTRKO0 + SNAC_MAX_SCAL)) {
    set_error("snac_out1d: halo'd fields only");
    return SNAC_ERR_ARG;
  }
  const HostBlock &H = d->hb[ib];
  const DBlock &B = d->db[ib];
  const int a = idir - 1, ta = a == 0 ? 1 : 0, tb = a == 2 ? 1 : 2;
  // device weight tables: the interior entries of B.ax[axis][which]
  auto wtab = [&](int ax) {
    const int which = out_staggered(field, ax) ? AX_DC : AX_DF;
    return B.ax[ax] + (size_t)which * (B.n[ax] + 2) + 1;
  };
  const double lprod = (H.desc.lmax[ta] - H.desc.lmin[ta]) * (H.desc.lmax[tb] - H.desc.lmin[tb]);
  double *dprof = (double *)d->alloc((size_t)H.ng[a] * sizeof(double));
  if (!dprof) { set_error("device allocation failed (profile)"); return SNAC_ERR_NOMEM; }
  SNAC_TRY(launch_out1d(f, H.ng, a, wtab(ta), wtab(tb), lprod, dprof, d->st));
  SNAC_CUDA(cudaMemcpyAsync(prof, dprof, (size_t)H.ng[a] * sizeof(double), cudaMemcpyDeviceToHost, d->st));
  SNAC_CUDA(cudaStreamSynchronize(d->st));
  d->allocs.pop_back();
  SNAC_CUDA(cudaFree(dprof));
  const std::vector<double> &x = H.g[a][out_staggered(field, a) ? 3 : 2];
  for (int q = 0; q < H.ng[a]; q++) coord[q] = x[q + 1];
  return SNAC_OK;
}

int snac_out1d_write(const char *fname, int ib, int field, int idir) {
  NEED_DOMAIN
  if (!fname) { set_error("snac_out1d_write: null file name"); return SNAC_ERR_ARG; }
  if (ib < 0 || ib >= d->nblocks || idir < 1 || idir > 3) { set_error("block or direction out of range"); return SNAC_ERR_ARG; }
  const int n = d->hb[ib].ng[idir - 1];
  std::vector<double> x(n), p(n);
  SNAC_TRY(snac_out1d(ib, field, idir, x.data(), p.data()));
  FILE *fp = fopen(fname, "w");
  if (!fp) { set_error("cannot create %s", fname); return SNAC_ERR_IO; }
  char a[128], b[128];
  for (int q = 0; q < n; q++) {
    fortran_e15_7(x[q], a);
    fortran_e15_7(p[q], b);
    fprintf(fp, "%s%s\n", a, b);
  }
  if (fclose(fp) != 0) { set_error("cannot write %s", fname); return SNAC_ERR_IO; }
  return SNAC_OK;
}

int snac_out3d_write(const char *fname, int ib, int field) {
  NEED_DOMAIN
  if (!fname) { set_error("snac_out3d_write: null file name"); return SNAC_ERR_ARG; }
  if (ib < 0 || ib >= d->nblocks) { set_error("block index out of range"); return SNAC_ERR_ARG; }
  double *p; size_t bytes;
  SNAC_TRY(field_ptr(*d, ib, field, &p, &bytes));
  const int nx = d->hb[ib].ng[0], ny = d->hb[ib].ng[1], nz = d->hb[ib].ng[2];
  if (bytes != (size_t)(nx + 2) * (ny + 2) * (nz + 2) * sizeof(double)) { set_error("snac_out3d_write: halo'd fields only"); return SNAC_ERR_ARG; }
  std::vector<double> halo((size_t)(nx + 2) * (ny + 2) * (nz + 2)), out((size_t)nx * ny * nz);
  SNAC_CUDA(cudaStreamSynchronize(d->st));
  SNAC_CUDA(cudaMemcpy(halo.data(), p, bytes, cudaMemcpyDeviceToHost));
  size_t q = 0;
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) out[q++] = halo[hidx(i, j, k, nx, ny)];
  FILE *fp = fopen(fname, "wb");
  if (!fp) { set_error("cannot create %s", fname); return SNAC_ERR_IO; }
  const size_t nw = fwrite(out.data(), sizeof(double), out.size(), fp);
  if (fclose(fp) != 0 || nw != out.size()) { set_error("cannot write %s", fname); return SNAC_ERR_IO; }
  return SNAC_OK;
}

int snac_set_field(int ib, int field, const double *host) {
  NEED_DOMAIN
  double *p; size_t bytes;
  SNAC_TRY(field_ptr(*d, ib, field, &p, &bytes));
  SNAC_CUDA(cudaMemcpyAsync(p, host, bytes, cudaMemcpyHostToDevice, d->st));
  SNAC_CUDA(cudaStreamSynchronize(d->st));
  return SNAC_OK;
}

int snac_get_field(int ib, int field, double *host) {
  NEED_DOMAIN
  double *p; size_t bytes;
  SNAC_TRY(field_ptr(*d, ib, field, &p, &bytes));
  SNAC_CUDA(cudaMemcpyAsync(host, p, bytes, cudaMemcpyDeviceToHost, d->st));
  SNAC_CUDA(cudaStreamSynchronize(d->st));
  return SNAC_OK;
}

// batched host <-> device copies: alternate between the library stream and a second stream so that two
// copy engines share the transfers; one synchronisation at the end
static int copy_fields(Domain &d, int n, const int *ib, const int *field, void *const *host, bool to_device) {
  if (n < 0 || (n > 0 && (!ib || !field || !host))) { set_error("batched field copy: bad argument"); return SNAC_ERR_ARG; }
  if (!d.st_copy) SNAC_CUDA(cudaStreamCreateWithFlags(&d.st_copy, cudaStreamNonBlocking));
  std::vector<std::pair<double *, size_t>> dev(n);
  for (int q = 0; q < n; q++) {
    SNAC_TRY(field_ptr(d, ib[q], field[q], &dev[q].first, &dev[q].second));
    if (!host[q]) { set_error("batched field copy: null host array %d", q); return SNAC_ERR_ARG; }
  }
  SNAC_CUDA(cudaStreamSynchronize(d.st));  // the fields are not in use by queued work
  // on a failed copy the copies already issued may still be reading or writing the caller's host arrays:
  // both streams are drained before the first error is returned
  cudaError_t first = cudaSuccess;
  for (int q = 0; q < n && first == cudaSuccess; q++) {
    cudaStream_t s = (q & 1) ? d.st_copy : d.st;
    first = to_device ? cudaMemcpyAsync(dev[q].first, host[q], dev[q].second, cudaMemcpyHostToDevice, s)
                      : cudaMemcpyAsync(host[q], dev[q].first, dev[q].second, cudaMemcpyDeviceToHost, s);
  }
  const cudaError_t e1 = cudaStreamSynchronize(d.st_copy);
  const cudaError_t e2 = cudaStreamSynchronize(d.st);
  if (first != cudaSuccess)
    return cuda_fail(first, to_device ? "cudaMemcpyAsync (host to device)" : "cudaMemcpyAsync (device to host)",
                     __FILE__, __LINE__);
  SNAC_CUDA(e1);
  SNAC_CUDA(e2);
  return SNAC_OK;
}

int snac_set_fields(int n, const int *ib, const int *field, const double *const *host) {
  NEED_DOMAIN
  return copy_fields(*d, n, ib, field, (void *const *)host, true);
}

int snac_get_fields(int n, const int *ib, const int *field, double *const *host) {
  NEED_DOMAIN
  return copy_fields(*d, n, ib, field, (void *const *)host, false);
}

int snac_rk_mom_all(int irk) {
  NEED_DOMAIN
  if (irk < 0 || irk > 2) { set_error("irk must be 0..2"); return SNAC_ERR_ARG; }
  SNAC_TRY(rk_mom_all(*d, irk));
  SNAC_CUDA(cudaStreamSynchronize(d->st));
  return SNAC_OK;
}
int snac_bounduvw_all(int is_correc) {
  NEED_DOMAIN
  SNAC_TRY(bound_uvw(*d, is_correc));
  SNAC_CUDA(cudaStreamSynchronize(d->st));
  return SNAC_OK;
}
int snac_inflow_all(int is_correc) {
  NEED_DOMAIN
  SNAC_TRY(inflow_all(*d, is_correc));
  SNAC_CUDA(cudaStreamSynchronize(d->st));
  return SNAC_OK;
}
int snac_boundp_all(int field) {
  NEED_DOMAIN
  if (field != SNAC_P && field != SNAC_PP && !(field >= SNAC_S0 && field < SNAC_S0 + d->c.nscal)) {
    set_error("snac_boundp_all: field must be SNAC_P, SNAC_PP or a scalar");
    return SNAC_ERR_ARG;
  }
  SNAC_TRY(bound_p(*d, field));
  SNAC_CUDA(cudaStreamSynchronize(d->st));
  return SNAC_OK;
}
int snac_impdiff_solve(int field, double alphai_new, double alphai_old) {
  NEED_DOMAIN
  (void)alphai_old;  // the shift of this solve is set whole from alphai_new (the reference adds the difference)
  if (!d->c.impdiff) { set_error("snac_impdiff_solve: the domain was set up without IMPDIFF"); return SNAC_ERR_STATE; }
  int hf;
  if (field >= SNAC_U && field <= SNAC_W) hf = HF_U + (field - SNAC_U);
  else if (field >= SNAC_S0 && field < SNAC_S0 + d->c.nscal) hf = HF_S0 + (field - SNAC_S0);
  else { set_error("snac_impdiff_solve: field must be SNAC_U, SNAC_V, SNAC_W or a scalar"); return SNAC_ERR_ARG; }
  if (!d->hs[hf]) { set_error("snac_impdiff_solve: no Helmholtz solver for field %d", field); return SNAC_ERR_STATE; }
  const int rc = solver_solve_helmholtz(*d, *d->hs[hf], alphai_new);
  SNAC_CUDA(cudaStreamSynchronize(d->st));
  return rc;
}

int snac_fillps_all(double dtrk) {
  NEED_DOMAIN
  SNAC_TRY(fillps_all(*d, dtrk));
  SNAC_CUDA(cudaStreamSynchronize(d->st));
  SNAC_TRY(tma_check(*d));
  return bounds_check(d->st);
}
int snac_updt_rhs_all(void) {
  NEED_DOMAIN
  SNAC_TRY(updt_rhs_all(*d));
  SNAC_CUDA(cudaStreamSynchronize(d->st));
  return SNAC_OK;
}
int snac_bench_smoother(int level, int reps, double *ms_per_launch, double *bytes_per_launch) {
  NEED_DOMAIN
  if (!ms_per_launch || !bytes_per_launch || reps < 1) { set_error("snac_bench_smoother: bad arguments"); return SNAC_ERR_ARG; }
  const MgProblem &P = d->ps->P;
  if (level < 0 || level >= P.nlev - 1 || !tile2d_ok(P, level, 0)) {
    set_error("snac_bench_smoother: level %d has no tiled smoother (plane systems only)", level);
    return SNAC_ERR_UNSUPPORTED;
  }
  const MgLevelD &L = P.L[level];
  cudaEvent_t e0, e1;
  SNAC_CUDA(cudaEventCreate(&e0));
  SNAC_CUDA(cudaEventCreate(&e1));
  int rc = SNAC_OK;
  const MgLevelD &C = P.L[level + 1];
  const bool restrict_ = P.tile_restrict != 0;
  for (int q = 0; q < 2 + reps && rc == SNAC_OK; q++) {
    if (q == 2) cudaEventRecord(e0, d->st);
    if (restrict_)
      rc = launch_rbgs_tile2d_restrict<float>(P, level, nullptr, L.xpf, L.bf, C.bf, nullptr, d->st);
    else
      rc = launch_rbgs_tile2d<float>(P, level, nullptr, 0, 0, L.xpf, L.bf, nullptr, nullptr, nullptr, nullptr, nullptr,
                                     0, nullptr, d->st);
  }
  cudaEventRecord(e1, d->st);
  float ms = 0.f;
  if (rc == SNAC_OK) {
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) rc = SNAC_ERR_CUDA;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  SNAC_TRY(rc);
  *ms_per_launch = ms / reps;
  *bytes_per_launch = (12.0 * (double)L.ncell + (restrict_ ? 4.0 * (double)C.ncell : 0.0)) * (double)P.nsys;
  return SNAC_OK;
}

int snac_solve_pressure(void) {
  NEED_DOMAIN
  const int rc = solver_solve_pressure(*d, *d->ps);
  SNAC_CUDA(cudaStreamSynchronize(d->st));
  d->last_solve_iters = d->ps->last_iters;  // the statistics then describe this solve
  d->last_solve_res = d->ps->last_res;
  return rc;
}
int snac_correc_all(double dtrk) {
  NEED_DOMAIN
  SNAC_TRY(launch_correc(d->d_db, d->d_tiles_halo, d->ntiles_halo, dtrk, d->st));
  SNAC_CUDA(cudaStreamSynchronize(d->st));
  return SNAC_OK;
}
int snac_updt_pressure_all(double alpha) {
  NEED_DOMAIN
  SNAC_TRY(launch_updt_pressure(d->d_db, d->d_tiles, d->ntiles, alpha, d->c.impdiff, d->st));
  SNAC_CUDA(cudaStreamSynchronize(d->st));
  return SNAC_OK;
}
int snac_chkdt_all(double *dt_cfl) {
  NEED_DOMAIN
  return chkdt_all(*d, dt_cfl);
}
int snac_chkdiv_all(double *divtot, double *divmax) {
  NEED_DOMAIN
  double r[2];
  SNAC_TRY(reduce(*d, 1, r));
  *divtot = r[0];
  *divmax = r[1];
  if (std::isinf(r[1]) || r[0] != r[0]) { set_error("chkdiv: non-finite divergence"); return SNAC_ERR_NAN; }
  return SNAC_OK;
}
int snac_kinetic_energy(double *ke) {
  NEED_DOMAIN
  double r[2];
  SNAC_TRY(reduce(*d, 2, r));
  *ke = 0.5 * r[0] / d->vol_all;
  return SNAC_OK;
}

int snac_step(int nsteps) {
  NEED_DOMAIN
  if (d->dt == 0.0) SNAC_TRY(set_dt_from_cfl(*d));
  int rc_all = SNAC_OK;
  if (!d->ev0) {
    SNAC_CUDA(cudaEventCreate(&d->ev0));
    SNAC_CUDA(cudaEventCreate(&d->ev1));
  }
  SNAC_CUDA(cudaEventRecord(d->ev0, d->st));
  for (int s = 0; s < nsteps; s++) {
    d->istep++;
    d->time += d->dt;
    d->last_solve_iters = 0;
    d->last_solve_res = 0.0;
    d->last_helm_iters = 0;
    d->last_helm_res = 0.0;
    d->solves = 0;
    for (int irk = 0; irk < 3; irk++) {
      d->helm_not_converged = false;
      const int rc = one_stage(*d, irk);
      if (rc == SNAC_ERR_NOT_CONVERGED || (rc == SNAC_OK && d->helm_not_converged)) rc_all = SNAC_ERR_NOT_CONVERGED;
      else if (rc != SNAC_OK) return rc;
    }
    if (d->c.icheck > 0 && d->istep % d->c.icheck == 0) SNAC_TRY(set_dt_from_cfl(*d));
  }
  SNAC_CUDA(cudaEventRecord(d->ev1, d->st));
  SNAC_CUDA(cudaStreamSynchronize(d->st));
  float ms = 0.f;
  SNAC_CUDA(cudaEventElapsedTime(&ms, d->ev0, d->ev1));
  d->device_ms = ms;
  SNAC_TRY(tma_check(*d));  // a bounded wait of the TMA-staged kernel that ran out
  SNAC_TRY(bounds_check(d->st));
  return rc_all;
}

int snac_get_stats(snac_step_stats *st) {
  NEED_DOMAIN
  st->istep = d->istep;
  st->time = d->time;
  st->dt = d->dt;
  st->solve_iters_max = d->last_solve_iters;
  st->solve_residual_max = d->last_solve_res;
  st->solves = d->solves;
  st->device_ms = d->device_ms;
  st->helm_iters_max = d->last_helm_iters;
  st->helm_residual_max = d->last_helm_res;
  return SNAC_OK;
}
int snac_set_dt(double dt) {
  NEED_DOMAIN
  d->dt = dt;
  return SNAC_OK;
}
int snac_get_dt(double *dt) {
  NEED_DOMAIN
  *dt = d->dt;
  return SNAC_OK;
}

}  // extern "C"
