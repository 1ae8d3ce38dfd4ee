// k_bound.cu -- block-to-block halo exchange and physical boundary conditions.
//
// bound.f90:8-106 exchanges ghost planes with MPI_SENDRECV (updthalo,
// bound.f90:587-650) direction by direction, x then y then z, each plane
// including the ghost rows of the other two directions, and applies the
// physical conditions (set_bc, bound.f90:108-248) only after all exchanges.
// Here every block lives in the same HBM: one launch per direction copies the
// friend planes of all blocks and all requested fields, then one launch per
// direction applies the boundary conditions.  The phase order is the
// reference's, so corner and edge ghosts end up with identical values.
#include "snac_bound.h"

namespace snac {

__device__ inline double *field_ptr(const DBlock &B, int f) {
  switch (f) {
    case 0: return B.u;
    case 1: return B.v;
    case 2: return B.w;
    case 3: return B.p;
    case 4: return B.pp;
    default: return B.s[f - 5];
  }
}

// copy the friend's interior plane into the ghost plane, for one axis
__global__ void k_exchange(const DBlock *__restrict__ Bs, const FaceLink *__restrict__ F, const int *__restrict__ flds,
                           int a) {
  pdl_enter();
  const FaceLink fl = F[blockIdx.y];
  const DBlock &D = Bs[fl.dst];
  const DBlock &S = Bs[fl.src];
  const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
  const int m1 = D.n[t1] + 2, m2 = D.n[t2] + 2;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= m1 * m2) return;
  const int x = q % m1 - 1, y = q / m1 - 1;  // -1..n
  int cd[3], cs[3];
  cd[t1] = x; cd[t2] = y; cs[t1] = x; cs[t2] = y;
  cd[a] = fl.side ? D.n[a] : -1;
  cs[a] = fl.side ? 0 : S.n[a] - 1;
  if (!bchk(D, BK_EXCHANGE_DST, cd[0], cd[1], cd[2], -1, 1) || !bchk(S, BK_EXCHANGE_SRC, cs[0], cs[1], cs[2], -1, 1)) return;
  const long id = hidx(cd[0], cd[1], cd[2], D.n[0], D.n[1]);
  const long is = hidx(cs[0], cs[1], cs[2], S.n[0], S.n[1]);
  const int f = flds[blockIdx.z];
  field_ptr(D, f)[id] = field_ptr(S, f)[is];
}

// set_bc on both faces of one axis; side 0 then side 1 by the same thread
__global__ void k_setbc(const DBlock *__restrict__ Bs, const BcEntry *__restrict__ E, int a) {
  pdl_enter();
  const BcEntry e = E[blockIdx.y];
  const DBlock &B = Bs[e.b];
  const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
  const int m1 = B.n[t1] + 2, m2 = B.n[t2] + 2;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= m1 * m2) return;
  int c[3];
  c[t1] = q % m1 - 1;
  c[t2] = q / m1 - 1;
  const int n = B.n[a];
  const long st = a == 0 ? 1 : (a == 1 ? (long)(B.n[0] + 2) : (long)(B.n[0] + 2) * (B.n[1] + 2));
  c[a] = 0;
  if (!bchk(B, BK_SETBC, c[0], c[1], c[2], -1, 1)) return;  // the plane's cells along a span -1..n
  double *p = field_ptr(B, e.f) + hidx(c[0], c[1], c[2], B.n[0], B.n[1]);  // points at index 0 along a
#define AT(qq) p[(long)(qq) * st]
  for (int s = 0; s < 2; s++) {
    const double fa = e.factor[s], sg = e.sgn[s];
    switch (e.mode[s]) {
      case BC_CENTRED:
        if (s == 0) AT(-1) = fa + sg * AT(0);
        else AT(n) = fa + sg * AT(n - 1);
        break;
      case BC_STAG_D:
        if (s == 0) AT(-1) = fa;
        else { AT(n - 1) = fa; AT(n) = AT(n - 2); }
        break;
      case BC_STAG_N:
        if (s == 0) AT(-1) = fa + AT(0);
        else { AT(n - 1) = fa + AT(n - 2); AT(n) = AT(n - 1); }
        break;
      default: break;
    }
  }
#undef AT
}

int launch_exchange(const DBlock *dB, const FaceLink *dF, int nlinks, const int *dflds, int nflds, int a,
                    int maxplane, cudaStream_t st) {
  if (nlinks <= 0 || nflds <= 0) return SNAC_OK;
  dim3 g((maxplane + 255) / 256, nlinks, nflds);
  SNAC_CUDA(launch_k(k_exchange, g, dim3(256), 0, st, dB, dF, dflds, a));
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

int launch_setbc(const DBlock *dB, const BcEntry *dE, int nent, int a, int maxplane, cudaStream_t st) {
  if (nent <= 0) return SNAC_OK;
  dim3 g((maxplane + 255) / 256, nent);
  SNAC_CUDA(launch_k(k_setbc, g, dim3(256), 0, st, dB, dE, a));
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

// inflow (bound.f90:438-477), one face of every listed block: the normal component on the boundary face
// (qn = lo-1 | hi) unless is_correc, the tangential ones at qt = lo-1 | hi+1 mirrored about the inflow value
// (-f(qt+dq) + 2 f_in), over the whole halo'd plane.  The faces of one block run in the reference's order
// (x0, x1, y0, y1, z0, z1), one launch each, so edge ghosts end up as in the reference.
__global__ void k_inflow(const DBlock *__restrict__ dB, const InflowFace *__restrict__ dI, int a, int side,
                         int is_correc) {
  const InflowFace F = dI[blockIdx.y];
  const DBlock &B = dB[F.b];
  const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
  const int n1 = B.n[t1] + 2, n2 = B.n[t2] + 2;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n1 * n2) return;
  int c[3];
  c[t1] = q % n1 - 1;
  c[t2] = q / n1 - 1;
  const int na = B.n[a];
  const int qn = side ? na - 1 : -1, qt = side ? na : -1, dq = side ? -1 : 1;
  c[a] = qt;
  if (!bchk(B, BK_INFLOW, c[0], c[1], c[2], -1, 1)) return;  // qn and qt + dq lie between qt and the interior
  double *f[3] = {B.u, B.v, B.w};
  for (int comp = 0; comp < 3; comp++) {
    const double vin = F.pl[comp][q];
    if (comp == a) {
      if (is_correc) continue;
      c[a] = qn;
      f[comp][hidx(c[0], c[1], c[2], B.n[0], B.n[1])] = vin;
    } else {
      c[a] = qt + dq;
      const double inner = f[comp][hidx(c[0], c[1], c[2], B.n[0], B.n[1])];
      c[a] = qt;
      f[comp][hidx(c[0], c[1], c[2], B.n[0], B.n[1])] = -inner + 2.0 * vin;
    }
  }
}

int launch_inflow(const DBlock *dB, const InflowFace *dI, int nface, int a, int side, int maxplane, int is_correc,
                  cudaStream_t st) {
  if (nface <= 0) return SNAC_OK;
  dim3 g((maxplane + 255) / 256, nface);
  k_inflow<<<g, 256, 0, st>>>(dB, dI, a, side, is_correc), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

// set_bc parameters of one face, bound.f90:121-133
void bc_mode(char ctype, int ibound, int centered, double rvalue, double dr, int *mode, double *factor, double *sgn) {
  *mode = BC_NONE;
  *factor = rvalue;
  *sgn = 0.0;
  if (ctype == 'D' && centered) { *factor = 2.0 * rvalue; *sgn = -1.0; }
  if (ctype == 'N') { *factor = (ibound == 0 ? -dr : dr) * rvalue; *sgn = 1.0; }
  if (ctype != 'D' && ctype != 'N') return;
  if (centered) *mode = BC_CENTRED;
  else *mode = ctype == 'D' ? BC_STAG_D : BC_STAG_N;
}

}  // namespace snac
