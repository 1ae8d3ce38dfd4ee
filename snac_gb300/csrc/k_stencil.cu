// k_stencil.cu -- FP64 cell kernels of the per-stage hot path on sm_103a.
//
// GB300 executes FP64 at a small fraction of its FP32/tensor rates, so these
// kernels are arranged to minimise FP64 instructions per cell rather than
// bytes: every division of the reference loops (mom.f90, scal.f90, fillps.f90,
// correc.f90, chkdt.f90, chkdiv.f90) is replaced by a multiply with a 1-D
// table built once per block (DBlock::ax), common factors are folded into
// those tables, and the three velocity components of a cell are produced by
// one thread so that neighbour loads are shared through registers and L1.
// One CTA covers one TX x TY x TZ tile of one block (tile lists make uneven
// multi-block layouts a single launch).
#include "snac_internal.h"
#include "snac_mgdev.h"
#include "snac_prof.h"

namespace snac {

#define TILE_SETUP                                                  \
  const Tile t = T[blockIdx.x];                                     \
  const DBlock &B = Bs[t.x];                                        \
  const int nx = B.n[0], ny = B.n[1], nz = B.n[2];                  \
  const int i = t.y + (int)threadIdx.x, j = t.z + (int)threadIdx.y, \
            k = t.w + (int)threadIdx.z;                             \
  if (i >= nx || j >= ny || k >= nz) return;                        \
  if (!bchk(B, BK_TILE, i, j, k, 0, 0)) return;

// ---------------------------------------------------------------- rk_mom
// rk.f90:7-128 with momx/y/z_d (mom.f90:221-327), momx/y/z_a_vv (mom.f90:112-219),
// momx/y/z_p (mom.f90:328-386).  Writes the new interior velocity to B.nu/nv/nw
// (the reference updates u in place; the neighbour reads here still need the old
// values, so the write-back is a second, memory-only pass) and dudtrko in place.
__global__ void __launch_bounds__(TX * TY * TZ)
k_rk_mom(const DBlock *__restrict__ Bs, const Tile *__restrict__ T, RkMomParams prm) {
  pdl_enter();
  TILE_SETUP
  const long sy = nx + 2, sz = (long)(nx + 2) * (ny + 2);
  const long c = hidx(i, j, k, nx, ny);
  const double *__restrict__ u = B.u;
  const double *__restrict__ v = B.v;
  const double *__restrict__ w = B.w;
  // neighbourhood
  const double u0 = u[c], uxm = u[c - 1], uxp = u[c + 1], uym = u[c - sy], uyp = u[c + sy], uzm = u[c - sz], uzp = u[c + sz];
  const double uxmyp = u[c - 1 + sy], uxmzp = u[c - 1 + sz];
  const double v0 = v[c], vxm = v[c - 1], vxp = v[c + 1], vym = v[c - sy], vyp = v[c + sy], vzm = v[c - sz], vzp = v[c + sz];
  const double vxpym = v[c + 1 - sy], vymzp = v[c - sy + sz];
  const double w0 = w[c], wxm = w[c - 1], wxp = w[c + 1], wym = w[c - sy], wyp = w[c + sy], wzm = w[c - sz], wzp = w[c + sz];
  const double wxpzm = w[c + 1 - sz], wypzm = w[c + sy - sz];
  // 1-D tables
  const double xa = AX(B, 0, AX_A, i), xe0 = AX(B, 0, AX_E0, i), xe1 = AX(B, 0, AX_E1, i), xrf = AX(B, 0, AX_RF, i),
               xrc = AX(B, 0, AX_RC, i);
  const double ya = AX(B, 1, AX_A, j), ye0 = AX(B, 1, AX_E0, j), ye1 = AX(B, 1, AX_E1, j), yrf = AX(B, 1, AX_RF, j),
               yrc = AX(B, 1, AX_RC, j);
  const double za = AX(B, 2, AX_A, k), ze0 = AX(B, 2, AX_E0, k), ze1 = AX(B, 2, AX_E1, k), zrf = AX(B, 2, AX_RF, k),
               zrc = AX(B, 2, AX_RC, k);
  const double visc = prm.visc;
  // ---- diffusion (mom.f90:444-528): visc * sum_dir [ (f+ - f0)*P - (f0 - f-)*M ]
  double du, dv, dw;
  {
    const double sxp = AX(B, 0, AX_SP, i), sxm = AX(B, 0, AX_SM, i), cxp = AX(B, 0, AX_CP, i), cxm = AX(B, 0, AX_CM, i);
    const double syp = AX(B, 1, AX_SP, j), sym = AX(B, 1, AX_SM, j), cyp = AX(B, 1, AX_CP, j), cym = AX(B, 1, AX_CM, j);
    const double szp = AX(B, 2, AX_SP, k), szm = AX(B, 2, AX_SM, k), czp = AX(B, 2, AX_CP, k), czm = AX(B, 2, AX_CM, k);
    double a;
    a = (uxp - u0) * sxp - (u0 - uxm) * sxm;
    a = fma(uyp - u0, cyp, a) - (u0 - uym) * cym;
    a = fma(uzp - u0, czp, a) - (u0 - uzm) * czm;
    du = visc * a;
    a = (vxp - v0) * cxp - (v0 - vxm) * cxm;
    a = fma(vyp - v0, syp, a) - (v0 - vym) * sym;
    a = fma(vzp - v0, czp, a) - (v0 - vzm) * czm;
    dv = visc * a;
    a = (wxp - w0) * cxp - (w0 - wxm) * cxm;
    a = fma(wyp - w0, cyp, a) - (w0 - wym) * cym;
    a = fma(wzp - w0, szp, a) - (w0 - wzm) * szm;
    dw = visc * a;
  }
  // ---- advection, volume-weighted form (mom.f90:129-215) with the cell volume cancelled
  double au, av, aw;
  {
    // u: x-fluxes 0.25/dxc * [(u0+u-)u- - (u0+u+)u+]
    double tx = (u0 + uxm) * uxm - (u0 + uxp) * uxp;
    // y-fluxes: (e0 v(i,j) + e1 v(i+1,j)) interpolations, 1/dyf
    const double vm = fma(xe0, vym, xe1 * vxpym), vp = fma(xe0, v0, xe1 * vxp);
    double ty = vm * uym - vp * uyp;
    const double wm = fma(xe0, wzm, xe1 * wxpzm), wp = fma(xe0, w0, xe1 * wxp);
    double tz = wm * uzm - wp * uzp;
    au = fma(tx, xa, fma(ty, yrf, tz * zrf));
    // v: y-fluxes 0.25/dyc * [(v0+v-)v- - (v0+v+)v+]
    tx = fma(ye0, uxm, ye1 * uxmyp) * vxm - fma(ye0, u0, ye1 * uyp) * vxp;
    ty = (v0 + vym) * vym - (v0 + vyp) * vyp;
    tz = fma(ye0, wzm, ye1 * wypzm) * vzm - fma(ye0, w0, ye1 * wyp) * vzp;
    av = fma(tx, xrf, fma(ty, ya, tz * zrf));
    // w
    tx = fma(ze0, uxm, ze1 * uxmzp) * wxm - fma(ze0, u0, ze1 * uzp) * wxp;
    ty = fma(ze0, vym, ze1 * vymzp) * wym - fma(ze0, v0, ze1 * vzp) * wyp;
    tz = (w0 + wzm) * wzm - (w0 + wzp) * wzp;
    aw = fma(tx, xrf, fma(ty, yrf, tz * za));
  }
  const long ci = iidx(i, j, k, nx, ny);
  double ru, rv, rw, rdu, rdv, rdw;
  if (!prm.impdiff) { ru = du + au; rv = dv + av; rw = dw + aw; rdu = rdv = rdw = 0.0; }
  else { ru = au; rv = av; rw = aw; rdu = du; rdv = dv; rdw = dw; }
  // rk.f90:72-82
  double un = fma(prm.f2, B.ru[ci], fma(prm.f1, ru, u0));
  double vn = fma(prm.f2, B.rv[ci], fma(prm.f1, rv, v0));
  double wn = fma(prm.f2, B.rw[ci], fma(prm.f1, rw, w0));
  if (prm.impdiff) { un = fma(prm.f12, rdu, un); vn = fma(prm.f12, rdv, vn); wn = fma(prm.f12, rdw, wn); }
  B.ru[ci] = ru; B.rv[ci] = rv; B.rw[ci] = rw;
  // rk.f90:91-103: pressure gradient of the previous p and body force
  const double *__restrict__ p = B.p;
  const double p0 = p[c];
  un = fma(prm.f12, fma(-(p[c + 1] - p0), xrc, prm.bforce[0]), un);
  vn = fma(prm.f12, fma(-(p[c + sy] - p0), yrc, prm.bforce[1]), vn);
  wn = fma(prm.f12, fma(-(p[c + sz] - p0), zrc, prm.bforce[2]), wn);
  if (prm.boussinesq) {  // rk.f90:104-108
    const double *__restrict__ s = B.s[0];
    const double s0 = s[c];
    un = fma(-prm.gb[0], s[c + 1] + s0, un);
    vn = fma(-prm.gb[1], s[c + sy] + s0, vn);
    wn = fma(-prm.gb[2], s[c + sz] + s0, wn);
  }
  if (prm.impdiff) {  // rk.f90:118-126
    const double h = 0.5 * prm.f12;
    un = fma(-h, rdu, un); vn = fma(-h, rdv, vn); wn = fma(-h, rdw, wn);
  }
  if (prm.halo_out) { B.nu[c] = un; B.nv[c] = vn; B.nw[c] = wn; }
  else { B.nu[ci] = un; B.nv[ci] = vn; B.nw[ci] = wn; }
}

__global__ void __launch_bounds__(TX * TY * TZ)
k_rk_mom_writeback(const DBlock *__restrict__ Bs, const Tile *__restrict__ T) {
  pdl_enter();
  TILE_SETUP
  const long c = hidx(i, j, k, nx, ny), ci = iidx(i, j, k, nx, ny);
  B.u[c] = B.nu[ci];
  B.v[c] = B.nv[ci];
  B.w[c] = B.nw[ci];
}

int launch_rk_mom(const DBlock *dB, const Tile *dT, int ntiles, const RkMomParams &prm, cudaStream_t st) {
  if (ntiles <= 0) return SNAC_OK;
  prof_begin(KID_RK_MOM, st);
  SNAC_CUDA(launch_k(k_rk_mom, dim3(ntiles), dim3(TX, TY, TZ), 0, st, dB, dT, prm));
  prof_end(KID_RK_MOM, st);
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}
int launch_rk_mom_writeback(const DBlock *dB, const Tile *dT, int ntiles, cudaStream_t st) {
  if (ntiles <= 0) return SNAC_OK;
  SNAC_CUDA(launch_k(k_rk_mom_writeback, dim3(ntiles), dim3(TX, TY, TZ), 0, st, dB, dT));
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

// The six halo planes of u, v, w into nu, nv, nw, one CTA row per (face, block): the new interior the
// momentum stage wrote plus the halo of before is exactly the field the reference's in-place update leaves.
__global__ void k_uvw_halo_copy(const DBlock *__restrict__ Bs) {
  pdl_enter();
  const DBlock &B = Bs[blockIdx.y];
  const int a = blockIdx.z >> 1, side = blockIdx.z & 1;
  const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
  const int m1 = B.n[t1] + 2, m2 = B.n[t2] + 2;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= m1 * m2) return;
  int c[3];
  c[t1] = q % m1 - 1;
  c[t2] = q / m1 - 1;
  c[a] = side ? B.n[a] : -1;
  if (!bchk(B, BK_TILE, c[0], c[1], c[2], -1, 1)) return;
  const long h = hidx(c[0], c[1], c[2], B.n[0], B.n[1]);
  B.nu[h] = B.u[h];
  B.nv[h] = B.v[h];
  B.nw[h] = B.w[h];
}

int launch_uvw_halo_copy(const DBlock *dB, int nblocks, int maxplane, cudaStream_t st) {
  if (nblocks <= 0) return SNAC_OK;
  SNAC_CUDA(launch_k(k_uvw_halo_copy, dim3((maxplane + 255) / 256, nblocks, 6), dim3(256), 0, st, dB));
  return SNAC_OK;
}

// ---------------------------------------------------------------- rk_scal
// rk.f90:130-204 with scal_d (scal.f90:89-121) and scal_a (scal.f90:123-154)
template <int OP>
__device__ inline void tile_reduce(double s, double m, double *part);

// `part` (optional): per-tile sums of s*dxf*dyf*dzf of the updated scalar before the
// IMPDIFF correction -- the bulk mean of rk.f90:185-189, which precedes rk.f90:196-202.
__global__ void __launch_bounds__(TX * TY * TZ)
k_rk_scal(const DBlock *__restrict__ Bs, const Tile *__restrict__ T, RkScalParams prm, double *part) {
  const Tile t = T[blockIdx.x];
  const DBlock &B = Bs[t.x];
  const int nx = B.n[0], ny = B.n[1], nz = B.n[2];
  const int i = t.y + (int)threadIdx.x, j = t.z + (int)threadIdx.y, k = t.w + (int)threadIdx.z;
  const bool valid = i < nx && j < ny && k < nz;
  double msum = 0.0;
  if (valid) {
  const long sy = nx + 2, sz = (long)(nx + 2) * (ny + 2);
  const long c = hidx(i, j, k, nx, ny), ci = iidx(i, j, k, nx, ny);
  const double *__restrict__ s = B.s[prm.sidx];
  const double s0 = s[c], sxm = s[c - 1], sxp = s[c + 1], sym = s[c - sy], syp = s[c + sy], szm = s[c - sz], szp = s[c + sz];
  // scal_d: centred diffusion, alpha * [(s+ - s0)/dc(q) - (s0 - s-)/dc(q-1)]/df(q)
  double a = (sxp - s0) * AX(B, 0, AX_CP, i) - (s0 - sxm) * AX(B, 0, AX_CM, i);
  a = fma(syp - s0, AX(B, 1, AX_CP, j), a) - (s0 - sym) * AX(B, 1, AX_CM, j);
  a = fma(szp - s0, AX(B, 2, AX_CP, k), a) - (s0 - szm) * AX(B, 2, AX_CM, k);
  const double dd = prm.alpha * a;
  // scal_a: 0.5*(s-+s0)*u- - 0.5*(s++s0)*u0, per 1/df
  const double tx = (sxm + s0) * B.u[c - 1] - (sxp + s0) * B.u[c];
  const double ty = (sym + s0) * B.v[c - sy] - (syp + s0) * B.v[c];
  const double tz = (szm + s0) * B.w[c - sz] - (szp + s0) * B.w[c];
  const double ad = 0.5 * fma(tx, AX(B, 0, AX_RF, i), fma(ty, AX(B, 1, AX_RF, j), tz * AX(B, 2, AX_RF, k)));
  double r, rd;
  if (!prm.impdiff) { r = dd + ad; rd = 0.0; } else { r = ad; rd = dd; }
  double *__restrict__ ro = B.rs[prm.sidx];
  double sn = fma(prm.f12, prm.ssource, fma(prm.f2, ro[ci], fma(prm.f1, r, s0)));
  if (prm.impdiff) sn = fma(prm.f12, rd, sn);
  ro[ci] = r;
  msum = sn * AX(B, 0, AX_DF, i) * AX(B, 1, AX_DF, j) * AX(B, 2, AX_DF, k);
  if (prm.impdiff) sn = fma(-0.5 * prm.f12, rd, sn);
  B.ns[ci] = sn;
  }
  if (part) tile_reduce<4>(msum, 0.0, part);
}

__global__ void __launch_bounds__(TX * TY * TZ)
k_rk_scal_writeback(const DBlock *__restrict__ Bs, const Tile *__restrict__ T, int sidx) {
  TILE_SETUP
  B.s[sidx][hidx(i, j, k, nx, ny)] = B.ns[iidx(i, j, k, nx, ny)];
}

int launch_rk_scal(const DBlock *dB, const Tile *dT, int ntiles, const RkScalParams &prm, double *part,
                   cudaStream_t st) {
  if (ntiles <= 0) return SNAC_OK;
  k_rk_scal<<<ntiles, dim3(TX, TY, TZ), 0, st>>>(dB, dT, prm, part), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}
int launch_rk_scal_writeback(const DBlock *dB, const Tile *dT, int ntiles, int sidx, cudaStream_t st) {
  if (ntiles <= 0) return SNAC_OK;
  k_rk_scal_writeback<<<ntiles, dim3(TX, TY, TZ), 0, st>>>(dB, dT, sidx), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

// bulk_forcing_s (scal.f90:181-199) with f = scalf - mean, mean = red[0] * inv_vol read on the device
__global__ void __launch_bounds__(TX * TY * TZ)
k_bulk_forcing_s(const DBlock *__restrict__ Bs, const Tile *__restrict__ T, int sidx, double scalf, double inv_vol,
                 const double *__restrict__ red) {
  TILE_SETUP
  const double f = scalf - red[0] * inv_vol;
  B.s[sidx][hidx(i, j, k, nx, ny)] += f;
}
int launch_bulk_forcing_s(const DBlock *dB, const Tile *dT, int ntiles, int sidx, double scalf, double inv_vol,
                          const double *red, cudaStream_t st) {
  if (ntiles <= 0) return SNAC_OK;
  k_bulk_forcing_s<<<ntiles, dim3(TX, TY, TZ), 0, st>>>(dB, dT, sidx, scalf, inv_vol, red), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

// ---------------------------------------------------------------- fillps (fillps.f90:27-53)
__global__ void __launch_bounds__(TX * TY * TZ)
k_fillps(const DBlock *__restrict__ Bs, const Tile *__restrict__ T, double rdt, int fft_axis) {
  pdl_enter();
  TILE_SETUP
  const long sy = nx + 2, sz = (long)(nx + 2) * (ny + 2);
  const long c = hidx(i, j, k, nx, ny);
  const double dwv = B.w[c] - B.w[c - sz], dvv = B.v[c] - B.v[c - sy], duv = B.u[c] - B.u[c - 1];
  const double dxf = AX(B, 0, AX_DF, i), dyf = AX(B, 1, AX_DF, j), dzf = AX(B, 2, AX_DF, k);
  double r;
  switch (fft_axis) {
    case 3: r = fma(dwv * AX(B, 2, AX_RF, k), dxf * dyf, fma(dvv, dxf, duv * dyf)); break;
    case 2: r = fma(dwv, dxf, fma(dvv * AX(B, 1, AX_RF, j), dxf * dzf, duv * dzf)); break;
    case 1: r = fma(dwv, dyf, fma(dvv, dzf, duv * AX(B, 0, AX_RF, i) * (dyf * dzf))); break;
    default: r = fma(dwv, dxf * dyf, fma(dvv, dxf * dzf, duv * (dyf * dzf)));
  }
  B.pp[c] = r * rdt;
}

int launch_fillps(const DBlock *dB, const Tile *dT, int ntiles, double dt, int fft_axis, cudaStream_t st) {
  if (ntiles <= 0) return SNAC_OK;
  prof_begin(KID_FILLPS, st);
  SNAC_CUDA(launch_k(k_fillps, dim3(ntiles), dim3(TX, TY, TZ), 0, st, dB, dT, 1.0 / dt, fft_axis));
  prof_end(KID_FILLPS, st);
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

// ---------------------------------------------------------------- correc (correc.f90:21-47)
// Tiles cover the halo'd extent: i,j,k here run over -1..n (tile origins shifted by -1).
__global__ void __launch_bounds__(TX * TY * TZ)
k_correc(const DBlock *__restrict__ Bs, const Tile *__restrict__ T, double dt) {
  pdl_enter();
  const Tile t = T[blockIdx.x];
  const DBlock &B = Bs[t.x];
  const int nx = B.n[0], ny = B.n[1], nz = B.n[2];
  const int i = t.y - 1 + (int)threadIdx.x, j = t.z - 1 + (int)threadIdx.y, k = t.w - 1 + (int)threadIdx.z;
  if (i > nx || j > ny || k > nz) return;
  const long sy = nx + 2, sz = (long)(nx + 2) * (ny + 2);
  const long c = hidx(i, j, k, nx, ny);
  const double p0 = B.pp[c];
  if (i <= nx - 1) B.u[c] = fma(-dt * (B.pp[c + 1] - p0), AX(B, 0, AX_RC, i), B.u[c]);
  if (j <= ny - 1) B.v[c] = fma(-dt * (B.pp[c + sy] - p0), AX(B, 1, AX_RC, j), B.v[c]);
  if (k <= nz - 1) B.w[c] = fma(-dt * (B.pp[c + sz] - p0), AX(B, 2, AX_RC, k), B.w[c]);
}

int launch_correc(const DBlock *dB, const Tile *dT, int ntiles, double dt, cudaStream_t st) {
  if (ntiles <= 0) return SNAC_OK;
  prof_begin(KID_CORREC, st);
  SNAC_CUDA(launch_k(k_correc, dim3(ntiles), dim3(TX, TY, TZ), 0, st, dB, dT, dt));
  prof_end(KID_CORREC, st);
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

// ---------------------------------------------------------------- updt_pressure (updt_pressure.f90:21-46)
__global__ void __launch_bounds__(TX * TY * TZ)
k_updt_pressure(const DBlock *__restrict__ Bs, const Tile *__restrict__ T, double alpha, int impdiff) {
  pdl_enter();
  TILE_SETUP
  const long c = hidx(i, j, k, nx, ny);
  const double *__restrict__ pp = B.pp;
  const double q0 = pp[c];
  double pn = B.p[c] + q0;
  if (impdiff) {
    const long sy = nx + 2, sz = (long)(nx + 2) * (ny + 2);
    double a = (pp[c + 1] - q0) * AX(B, 0, AX_CP, i) - (q0 - pp[c - 1]) * AX(B, 0, AX_CM, i);
    a = fma(pp[c + sy] - q0, AX(B, 1, AX_CP, j), a) - (q0 - pp[c - sy]) * AX(B, 1, AX_CM, j);
    a = fma(pp[c + sz] - q0, AX(B, 2, AX_CP, k), a) - (q0 - pp[c - sz]) * AX(B, 2, AX_CM, k);
    pn = fma(alpha, a, pn);
  }
  B.p[c] = pn;
}

int launch_updt_pressure(const DBlock *dB, const Tile *dT, int ntiles, double alpha, int impdiff, cudaStream_t st) {
  if (ntiles <= 0) return SNAC_OK;
  SNAC_CUDA(launch_k(k_updt_pressure, dim3(ntiles), dim3(TX, TY, TZ), 0, st, dB, dT, alpha, impdiff));
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

// ---------------------------------------------------------------- reductions
// Each tile writes (sum, max) of its cells to part[2*tile]; the final pass adds
// the tiles in tile order, so the result does not depend on scheduling.
template <int OP>
__device__ inline void tile_reduce(double s, double m, double *part) {
  __shared__ double ss[TX * TY * TZ / 32], sm[TX * TY * TZ / 32];
  const int tid = threadIdx.x + TX * (threadIdx.y + TY * threadIdx.z);
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_down_sync(0xffffffffu, s, o);
    m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  }
  if ((tid & 31) == 0) { ss[tid >> 5] = s; sm[tid >> 5] = m; }
  __syncthreads();
  if (tid == 0) {
    double S = 0.0, M = 0.0;
    for (int q = 0; q < TX * TY * TZ / 32; q++) { S += ss[q]; M = fmax(M, sm[q]); }
    part[2 * blockIdx.x] = S;
    part[2 * blockIdx.x + 1] = M;
  }
}

// chkdt.f90:24-55: m = max(dtix, dtiy, dtiz) per cell
__global__ void __launch_bounds__(TX * TY * TZ)
k_chkdt(const DBlock *__restrict__ Bs, const Tile *__restrict__ T, double *part) {
  const Tile t = T[blockIdx.x];
  const DBlock &B = Bs[t.x];
  const int nx = B.n[0], ny = B.n[1], nz = B.n[2];
  const int i = t.y + (int)threadIdx.x, j = t.z + (int)threadIdx.y, k = t.w + (int)threadIdx.z;
  double m = 0.0;
  if (i < nx && j < ny && k < nz) {
    const long sy = nx + 2, sz = (long)(nx + 2) * (ny + 2);
    const long c = hidx(i, j, k, nx, ny);
    const double *u = B.u, *v = B.v, *w = B.w;
    const double ux = fabs(u[c]);
    const double vx = 0.25 * fabs(v[c] + v[c - sy] + v[c + 1] + v[c + 1 - sy]);
    const double wx = 0.25 * fabs(w[c] + w[c - sz] + w[c + 1] + w[c + 1 - sz]);
    const double dtix = fma(ux, AX(B, 0, AX_RC, i), fma(vx, AX(B, 1, AX_RF, j), wx * AX(B, 2, AX_RF, k)));
    const double uy = 0.25 * fabs(u[c] + u[c + sy] + u[c - 1 + sy] + u[c - 1]);
    const double vy = fabs(v[c]);
    const double wy = 0.25 * fabs(w[c] + w[c + sy] + w[c + sy - sz] + w[c - sz]);
    const double dtiy = fma(uy, AX(B, 0, AX_RF, i), fma(vy, AX(B, 1, AX_RC, j), wy * AX(B, 2, AX_RF, k)));
    const double uz = 0.25 * fabs(u[c] + u[c - 1] + u[c - 1 + sz] + u[c + sz]);
    const double vz = 0.25 * fabs(v[c] + v[c - sy] + v[c - sy + sz] + v[c + sz]);
    const double wz = fabs(w[c]);
    const double dtiz = fma(uz, AX(B, 0, AX_RF, i), fma(vz, AX(B, 1, AX_RF, j), wz * AX(B, 2, AX_RC, k)));
    m = fmax(dtix, fmax(dtiy, dtiz));
    if (!(m == m)) m = __longlong_as_double(0x7ff0000000000000ll);  // NaN -> +Inf so it survives fmax
  }
  tile_reduce<0>(0.0, m, part);
}

// chkdiv.f90:24-43: sum of div*vol_cell/vol and max |div|
__global__ void __launch_bounds__(TX * TY * TZ)
k_chkdiv(const DBlock *__restrict__ Bs, const Tile *__restrict__ T, double rvol, double *part) {
  const Tile t = T[blockIdx.x];
  const DBlock &B = Bs[t.x];
  const int nx = B.n[0], ny = B.n[1], nz = B.n[2];
  const int i = t.y + (int)threadIdx.x, j = t.z + (int)threadIdx.y, k = t.w + (int)threadIdx.z;
  double s = 0.0, m = 0.0;
  if (i < nx && j < ny && k < nz) {
    const long sy = nx + 2, sz = (long)(nx + 2) * (ny + 2);
    const long c = hidx(i, j, k, nx, ny);
    const double div = fma(B.w[c] - B.w[c - sz], AX(B, 2, AX_RF, k),
                           fma(B.v[c] - B.v[c - sy], AX(B, 1, AX_RF, j), (B.u[c] - B.u[c - 1]) * AX(B, 0, AX_RF, i)));
    m = fabs(div);
    if (!(m == m)) m = __longlong_as_double(0x7ff0000000000000ll);
    s = div * (AX(B, 0, AX_DF, i) * AX(B, 1, AX_DF, j) * AX(B, 2, AX_DF, k)) * rvol;
  }
  tile_reduce<1>(s, m, part);
}

// kinetic energy: 0.5*(u^2 dxc dyf dzf + v^2 dxf dyc dzf + w^2 dxf dyf dzc) per cell
__global__ void __launch_bounds__(TX * TY * TZ)
k_ke(const DBlock *__restrict__ Bs, const Tile *__restrict__ T, double *part) {
  const Tile t = T[blockIdx.x];
  const DBlock &B = Bs[t.x];
  const int nx = B.n[0], ny = B.n[1], nz = B.n[2];
  const int i = t.y + (int)threadIdx.x, j = t.z + (int)threadIdx.y, k = t.w + (int)threadIdx.z;
  double s = 0.0;
  if (i < nx && j < ny && k < nz) {
    const long c = hidx(i, j, k, nx, ny);
    const double u = B.u[c], v = B.v[c], w = B.w[c];
    const double xc = AX(B, 0, AX_DC, i), xf = AX(B, 0, AX_DF, i), yc = AX(B, 1, AX_DC, j), yf = AX(B, 1, AX_DF, j),
                 zc = AX(B, 2, AX_DC, k), zf = AX(B, 2, AX_DF, k);
    s = u * u * xc * yf * zf + v * v * xf * yc * zf + w * w * xf * yf * zc;
  }
  tile_reduce<2>(s, 0.0, part);
}

// bulk_mean_s (scal.f90:168-176): sum of s*dxf*dyf*dzf
__global__ void __launch_bounds__(TX * TY * TZ)
k_bulk(const DBlock *__restrict__ Bs, const Tile *__restrict__ T, int sidx, double *part) {
  const Tile t = T[blockIdx.x];
  const DBlock &B = Bs[t.x];
  const int nx = B.n[0], ny = B.n[1], nz = B.n[2];
  const int i = t.y + (int)threadIdx.x, j = t.z + (int)threadIdx.y, k = t.w + (int)threadIdx.z;
  double s = 0.0;
  if (i < nx && j < ny && k < nz)
    s = B.s[sidx][hidx(i, j, k, nx, ny)] * AX(B, 0, AX_DF, i) * AX(B, 1, AX_DF, j) * AX(B, 2, AX_DF, k);
  tile_reduce<3>(s, 0.0, part);
}

// updt_rhs (bound.f90:543-585): add the BC planes on the boundary cells
__global__ void k_updt_rhs(int nx, int ny, int nz, int4 isb0, int2 isb1, const double *rx, const double *ry,
                           const double *rz, double *p) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int isb[6] = {isb0.x, isb0.y, isb0.z, isb0.w, isb1.x, isb1.y};
  // x faces: ny*nz cells each
  for (int s = 0; s < 2; s++) {
    if (isb[s] && q < ny * nz) {
      const int j = q % ny, k = q / ny;
      p[hidx(s ? nx - 1 : 0, j, k, nx, ny)] += rx[q + (long)ny * nz * s];
    }
  }
}
__global__ void k_updt_rhs_y(int nx, int ny, int nz, int sb0, int sb1, const double *ry, double *p) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nx * nz) return;
  const int i = q % nx, k = q / nx;
  if (sb0) p[hidx(i, 0, k, nx, ny)] += ry[q];
  if (sb1) p[hidx(i, ny - 1, k, nx, ny)] += ry[q + (long)nx * nz];
}
__global__ void k_updt_rhs_z(int nx, int ny, int nz, int sb0, int sb1, const double *rz, double *p) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nx * ny) return;
  const int i = q % nx, j = q / nx;
  if (sb0) p[hidx(i, j, 0, nx, ny)] += rz[q];
  if (sb1) p[hidx(i, j, nz - 1, nx, ny)] += rz[q + (long)nx * ny];
}

// the reference adds x, then y, then z planes (edges receive several contributions in that order)
int launch_updt_rhs(int nx, int ny, int nz, const int isb[6], const double *rx, const double *ry, const double *rz,
                    double *p, cudaStream_t st) {
  if (isb[0] || isb[1]) {
    k_updt_rhs<<<(ny * nz + 255) / 256, 256, 0, st>>>(nx, ny, nz, make_int4(isb[0], isb[1], 0, 0), make_int2(0, 0),
                                                      rx, ry, rz, p), ::snac::count_launch();
    SNAC_CUDA(cudaGetLastError());
  }
  if (isb[2] || isb[3]) {
    k_updt_rhs_y<<<(nx * nz + 255) / 256, 256, 0, st>>>(nx, ny, nz, isb[2], isb[3], ry, p), ::snac::count_launch();
    SNAC_CUDA(cudaGetLastError());
  }
  if (isb[4] || isb[5]) {
    k_updt_rhs_z<<<(nx * ny + 255) / 256, 256, 0, st>>>(nx, ny, nz, isb[4], isb[5], rz, p), ::snac::count_launch();
    SNAC_CUDA(cudaGetLastError());
  }
  return SNAC_OK;
}

int launch_bulk_partial(const DBlock *dB, const Tile *dT, int ntiles, int sidx, double *part, cudaStream_t st) {
  if (ntiles <= 0) return SNAC_OK;
  k_bulk<<<ntiles, dim3(TX, TY, TZ), 0, st>>>(dB, dT, sidx, part), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

constexpr int RED_THREADS = 1024;
// one CTA, fixed order: thread t sums tiles t, t + 1024, ... in turn, each warp combines its lanes by a fixed
// shuffle tree, then warp 0 combines the 32 warp results the same way (deterministic, two levels)
__global__ void __launch_bounds__(RED_THREADS) k_reduce_final(const double *part, int n, double *out) {
  __shared__ double ws[RED_THREADS / 32], wm[RED_THREADS / 32];
  const int t = threadIdx.x, l = t & 31, w = t >> 5;
  double s = 0.0, m = 0.0;
  for (int q = t; q < n; q += RED_THREADS) { s += part[2 * q]; m = fmax(m, part[2 * q + 1]); }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_down_sync(0xffffffffu, s, o);
    m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  }
  if (l == 0) { ws[w] = s; wm[w] = m; }
  __syncthreads();
  if (w == 0) {
    s = ws[l];
    m = wm[l];
    for (int o = 16; o > 0; o >>= 1) {
      s += __shfl_down_sync(0xffffffffu, s, o);
      m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    }
    if (l == 0) { out[0] = s; out[1] = m; }
  }
}

int launch_chkdt_partial(const DBlock *dB, const Tile *dT, int ntiles, double *part, cudaStream_t st) {
  if (ntiles <= 0) return SNAC_OK;
  k_chkdt<<<ntiles, dim3(TX, TY, TZ), 0, st>>>(dB, dT, part), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}
int launch_chkdiv_partial(const DBlock *dB, const Tile *dT, int ntiles, double vol, double *part, cudaStream_t st) {
  if (ntiles <= 0) return SNAC_OK;
  k_chkdiv<<<ntiles, dim3(TX, TY, TZ), 0, st>>>(dB, dT, 1.0 / vol, part), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}
int launch_ke_partial(const DBlock *dB, const Tile *dT, int ntiles, double *part, cudaStream_t st) {
  if (ntiles <= 0) return SNAC_OK;
  k_ke<<<ntiles, dim3(TX, TY, TZ), 0, st>>>(dB, dT, part), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}
int launch_reduce_final(const double *part, int ntiles, double *out, cudaStream_t st) {
  k_reduce_final<<<1, RED_THREADS, 0, st>>>(part, ntiles, out), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

std::vector<Tile> make_tiles(const std::vector<std::array<int, 3>> &sizes, int tx, int ty, int tz) {
  std::vector<Tile> t;
  for (size_t b = 0; b < sizes.size(); b++)
    for (int k = 0; k < sizes[b][2]; k += tz)
      for (int j = 0; j < sizes[b][1]; j += ty)
        for (int i = 0; i < sizes[b][0]; i += tx) t.push_back(make_int4((int)b, i, j, k));
  return t;
}

}  // namespace snac

namespace snac {

// out1d (output.f90:34-125): one CTA per index along idir sums p * w_a * w_b / (l_a l_b) over its plane,
// with the field's weight tables wa (along axis ta) and wb (along tb) on the device
__global__ void __launch_bounds__(256) k_out1d(const double *__restrict__ f, int nx, int ny, int nz, int idir,
                                               const double *__restrict__ wa, const double *__restrict__ wb,
                                               double lprod, double *__restrict__ prof) {
  const int q = blockIdx.x;
  const int n[3] = {nx, ny, nz};
  const int ta = idir == 0 ? 1 : 0, tb = idir == 2 ? 1 : 2;
  const long npl = (long)n[ta] * n[tb];
  double acc = 0.0;
  for (long e = threadIdx.x; e < npl; e += blockDim.x) {
    int c[3];
    c[idir] = q;
    c[ta] = (int)(e % n[ta]);
    c[tb] = (int)(e / n[ta]);
    acc += f[hidx(c[0], c[1], c[2], nx, ny)] * wa[c[ta]] * wb[c[tb]] / lprod;
  }
  const double t = block_sum1<double>(acc);
  if (threadIdx.x == 0) prof[q] = t;
}

int launch_out1d(const double *f, const int n[3], int idir, const double *wa, const double *wb, double lprod,
                 double *prof, cudaStream_t st) {
  k_out1d<<<n[idir], 256, 0, st>>>(f, n[0], n[1], n[2], idir, wa, wb, lprod, prof), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

}  // namespace snac
