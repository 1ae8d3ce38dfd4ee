// k_mg_plane.cu -- multigrid and Krylov kernels of the plane systems, batched over systems.
//
// In plane mode every system of a solve (one per wavenumber of the transformed
// direction) has the same 2-D operator apart from the diagonal shift
// lambda_s * W0(i) W1(j).  These kernels give each thread the neighbour indices
// and couplings of its cells once and then apply them to a batch of systems
// (blockIdx.z selects the batch), so the operator is read and the boundary
// cases are resolved once per batch instead of once per system.  Term order and
// rounding are those of the generic kernels (snac_mgdev.h), so both give the
// same iterates.  The FP64 smoother reads 1/d from a table made once per solver
// (FP64 arithmetic is the scarce resource on this GPU), and so does FP32 (one load
// instead of a reciprocal per cell and system).
#include <algorithm>
#include <cstdlib>

#include "snac_solver.h"
#include "snac_mgk.h"
#include "snac_mgdev.h"
#include "snac_prof.h"

namespace snac {

namespace {
constexpr int RROWS = 2;  // rows per thread in the kernels that reduce (32 x 16 cells per CTA)
const dim3 BLK(32, 8);
}  // namespace

// partials per system written by plane_resid / plane_apply (one per 32 x 8*RROWS patch)
int plane_nchunk(const MgLevelD &L) { return ((L.n[0] + 31) / 32) * ((L.n[1] + 8 * RROWS - 1) / (8 * RROWS)); }
// partials per system written by plane_resid in FP64 (prec 1, 4 rows per thread) or FP32
int plane_resid_nchunk(const MgLevelD &L, int prec) {
  const int rr = prec ? 4 : RROWS;
  return ((L.n[0] + 31) / 32) * ((L.n[1] + 8 * rr - 1) / (8 * rr));
}

// systems per CTA: enough CTAs for about P.waves waves of `per_sm` resident CTAs on every multiprocessor (a
// large value gives one system per CTA)
int plane_batch(const MgProblem &P, long ctas_per_system, int per_sm) {
  const long waves = P.waves > 0 ? P.waves : 2;
  const long target = waves * std::max(1, P.nsm) * per_sm;
  long sb = (ctas_per_system * P.nsys) / std::max(1L, target);
  sb = std::max(1L, std::min(sb, (long)P.nsys));
  const long nb = (P.nsys + sb - 1) / sb;
  return (int)((P.nsys + nb - 1) / nb);
}

// ---------------------------------------------------------------- V-cycle kernels
template <typename T>
__global__ void __launch_bounds__(256) k_p_rbgs(MgLevelD L, int per0, int per1, const T *__restrict__ shift,
                                                const int *__restrict__ active, int nsys, int sb, int color, T *x,
                                                const T *__restrict__ b) {
  const int j = blockIdx.y * 8 + threadIdx.y;
  const int i = 2 * (int)(blockIdx.x * 32 + threadIdx.x) + ((color + j) & 1);
  if (i >= L.n[0] || j >= L.n[1]) return;
  const int c = i + L.n[0] * j;
  if (L.code[c] & 0x8000) return;
  const PlaneCell<T> pc = plane_cell<T>(L, per0, per1, i, j);
  const T cc = LA<T>::cc(L)[c], wt = LA<T>::w01(L)[c];
  const T *__restrict__ invd = LA<T>::invd(L);
  for (int s = (int)blockIdx.z; s < nsys; s += (int)gridDim.z) {  // systems strided over the CTA groups
    if (active && !active[s]) continue;
    const long off = L.ncell * (long)s;
    const T *xs = x + off;
    const T acc = plane_acc(pc, [&](int e) { return xs[e]; });
    const T iv = invd ? invd[off + c] : rcpt(fmat(shift[s], wt, cc));
    x[off + c] = (b[off + c] - acc) * iv;
  }
}

// coarse b <- sum over children of (b - A x); coarse x <- 0.  E0 x E1 children (the halved axes).
template <typename T, int E0, int E1>
__global__ void __launch_bounds__(256) k_p_restrict(MgLevelD F, MgLevelD C, int per0, int per1,
                                                    const T *__restrict__ shift, const int *__restrict__ active,
                                                    int nsys, int sb, const T *__restrict__ xf,
                                                    const T *__restrict__ bf, T *__restrict__ bc, T *__restrict__ xc) {
  constexpr int NCH = E0 * E1;
  const int I = blockIdx.x * 32 + threadIdx.x, J = blockIdx.y * 8 + threadIdx.y;
  if (I >= C.n[0] || J >= C.n[1]) return;
  PlaneCell<T> ch[NCH];
  T ccv[NCH], wtv[NCH];
  unsigned live = 0;
#pragma unroll
  for (int q = 0; q < NCH; q++) {  // children in the order (dj outer, di inner)
    const int di = q % E0, dj = q / E0;
    const int i = E0 == 2 ? 2 * I + di : I, j = E1 == 2 ? 2 * J + dj : J;
    ch[q] = plane_cell<T>(F, per0, per1, i, j);
    ccv[q] = wtv[q] = T(0);
    if (!(F.code[ch[q].c] & 0x8000)) {
      live |= 1u << q;
      ccv[q] = LA<T>::cc(F)[ch[q].c];
      wtv[q] = LA<T>::w01(F)[ch[q].c];
    }
  }
  const int cq = I + C.n[0] * J;
  pdl_enter();  // the children's couplings above are constant tables
  for (int s = (int)blockIdx.z; s < nsys; s += (int)gridDim.z) {  // systems strided over the CTA groups
    if (active && !active[s]) continue;
    const long offf = F.ncell * (long)s, offc = C.ncell * (long)s;
    const T *__restrict__ xs = xf + offf;
    const T sh = shift[s];
    T sum = 0;
#pragma unroll
    for (int q = 0; q < NCH; q++) {
      if (!(live >> q & 1)) continue;
      const T acc = plane_acc(ch[q], [&](int e) { return xs[e]; });
      sum += bf[offf + ch[q].c] - fmat(fmat(sh, wtv[q], ccv[q]), xs[ch[q].c], acc);
    }
    bc[offc + cq] = sum;
    xc[offc + cq] = 0;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_p_prolong(MgLevelD F, MgLevelD C, const int *__restrict__ active, int nsys,
                                                   int sb, T *__restrict__ xf, const T *__restrict__ xc) {
  const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
  if (i >= F.n[0] || j >= F.n[1]) return;
  const int c = i + F.n[0] * j;
  if (F.code[c] & 0x8000) return;
  const int pc = (C.coarsened[0] ? i / 2 : i) + C.n[0] * (C.coarsened[1] ? j / 2 : j);
  for (int s = (int)blockIdx.z; s < nsys; s += (int)gridDim.z) {  // systems strided over the CTA groups
    if (active && !active[s]) continue;
    xf[F.ncell * (long)s + c] += xc[C.ncell * (long)s + pc];
  }
}

// table of 1 / diagonal per system and cell (0 for inactive cells), in the smoother's precision
template <typename T>
__global__ void k_p_invd(MgLevelD L, const T *__restrict__ shift, T *__restrict__ out) {
  const int s = blockIdx.y;
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= L.ncell) return;
  out[L.ncell * s + c] = (L.code[c] & 0x8000) ? T(0) : rcpt(fmat(shift[s], LA<T>::w01(L)[c], LA<T>::cc(L)[c]));
}

// ---------------------------------------------------------------- Krylov kernels
// r = b - A x; partials of r.r (and b.b when part_bb); RR rows per thread.  FP64 arithmetic is the scarce
// resource here: every FP64 add of the block reduction costs as much as a stencil FMA, so the FP64 residual
// gives each thread 4 rows (one reduction tree per 4 cells) and reduces b.b only when it is asked for.
template <typename T, int RR>
__global__ void __launch_bounds__(256, (RR >= 4 ? 3 : 1)) k_p_resid(MgLevelD L, int per0, int per1, const T *__restrict__ shift,
                                                 const int *__restrict__ active, int nsys, int sb,
                                                 const T *__restrict__ x, const T *__restrict__ b,
                                                 T *__restrict__ r, double *__restrict__ part_rr,
                                                 double *__restrict__ part_bb, int stride) {
  const int i = blockIdx.x * 32 + threadIdx.x;
  PlaneCell<T> pc[RR];
  T ccv[RR], wtv[RR];
  unsigned inb = 0, live = 0;
#pragma unroll
  for (int q = 0; q < RR; q++) {
    const int j = blockIdx.y * (8 * RR) + threadIdx.y + 8 * q;
    ccv[q] = wtv[q] = T(0);
    pc[q] = PlaneCell<T>{0, 0, 0, 0, 0, T(0), T(0), T(0), T(0)};
    if (i < L.n[0] && j < L.n[1]) {
      inb |= 1u << q;
      pc[q] = plane_cell<T>(L, per0, per1, i, j);
      if (!(L.code[pc[q].c] & 0x8000)) {
        live |= 1u << q;
        ccv[q] = LA<T>::cc(L)[pc[q].c];
        wtv[q] = LA<T>::w01(L)[pc[q].c];
      }
    }
  }
  const long chunk = blockIdx.x + (long)gridDim.x * blockIdx.y;
  pdl_enter();
  for (int s = (int)blockIdx.z; s < nsys; s += (int)gridDim.z) {  // systems strided over the CTA groups
    if (active && !active[s]) continue;
    const long off = L.ncell * (long)s;
    const T *__restrict__ xs = x + off;
    const T sh = shift[s];
    T rr = 0, bb = 0;
#pragma unroll
    for (int q = 0; q < RR; q++) {
      if (!(inb >> q & 1)) continue;
      const int c = pc[q].c;
      T rv = 0;
      if (live >> q & 1) {
        const T acc = plane_acc(pc[q], [&](int e) { return xs[e]; });
        const T bv = b[off + c];
        rv = bv - fmat(fmat(sh, wtv[q], ccv[q]), xs[c], acc);
        rr = fmat(rv, rv, rr);
        if (part_bb) bb = fmat(bv, bv, bb);
      }
      r[off + c] = rv;
    }
    double trr, tbb = 0.0;
    if (part_bb) block_sum2<T>(rr, bb, trr, tbb);
    else trr = block_sum1<T>(rr);
    if (threadIdx.x == 0 && threadIdx.y == 0) {
      part_rr[(long)s * stride + chunk] = trr;
      if (part_bb) part_bb[(long)s * stride + chunk] = tbb;
    }
  }
}

// q = A p; partials of p.q.  FUSEP: p = (z - zmean) + beta p_old is formed on the fly and written to pn.
template <typename T, bool FUSEP>
__global__ void __launch_bounds__(256) k_p_apply(MgLevelD L, int per0, int per1, const T *__restrict__ shift,
                                                 const int *__restrict__ active, int nsys, int sb,
                                                 const SysScal *__restrict__ sc, const T *__restrict__ z,
                                                 const T *__restrict__ po, T *__restrict__ pn, T *__restrict__ q,
                                                 double *__restrict__ part, int stride) {
  const int i = blockIdx.x * 32 + threadIdx.x;
  PlaneCell<T> pc[RROWS];
  T ccv[RROWS], wtv[RROWS];
  unsigned inb = 0, live = 0;
#pragma unroll
  for (int qq = 0; qq < RROWS; qq++) {
    const int j = blockIdx.y * (8 * RROWS) + threadIdx.y + 8 * qq;
    ccv[qq] = wtv[qq] = T(0);
    pc[qq] = PlaneCell<T>{0, 0, 0, 0, 0, T(0), T(0), T(0), T(0)};
    if (i < L.n[0] && j < L.n[1]) {
      inb |= 1u << qq;
      pc[qq] = plane_cell<T>(L, per0, per1, i, j);
      if (!(L.code[pc[qq].c] & 0x8000)) {
        live |= 1u << qq;
        ccv[qq] = LA<T>::cc(L)[pc[qq].c];
        wtv[qq] = LA<T>::w01(L)[pc[qq].c];
      }
    }
  }
  const long chunk = blockIdx.x + (long)gridDim.x * blockIdx.y;
  pdl_enter();
  for (int s = (int)blockIdx.z; s < nsys; s += (int)gridDim.z) {  // systems strided over the CTA groups
    if (active && !active[s]) continue;
    const long off = L.ncell * (long)s;
    const T *__restrict__ zs = z + off;
    const T *__restrict__ ps = po + off;
    const T beta = FUSEP ? (T)sc[s].beta : T(0), zm = FUSEP ? (T)sc[s].zmean : T(0);
    const T sh = shift[s];
    auto pv = [&](int e) -> T { return FUSEP ? fmat(beta, ps[e], zs[e] - zm) : ps[e]; };
    T pq = 0;
#pragma unroll
    for (int qq = 0; qq < RROWS; qq++) {
      if (!(inb >> qq & 1)) continue;
      const int c = pc[qq].c;
      const T pcv = pv(c);
      if (FUSEP) pn[off + c] = pcv;
      T y = 0;
      if (live >> qq & 1) y = fmat(fmat(sh, wtv[qq], ccv[qq]), pcv, plane_acc(pc[qq], pv));
      q[off + c] = y;
      pq = fmat(pcv, y, pq);
    }
    const double t = block_sum1<T>(pq);
    if (threadIdx.x == 0 && threadIdx.y == 0) part[(long)s * stride + chunk] = t;
  }
}

// ---------------------------------------------------------------- launchers
template <typename T>
int plane_sweep(const MgProblem &P, int l, const T *shift, const int *active, int color, T *x, const T *b,
                cudaStream_t st) {
  const MgLevelD &L = P.L[l];
  const dim3 g((unsigned)(((L.n[0] + 1) / 2 + 31) / 32), (unsigned)((L.n[1] + 7) / 8), 1);
  const int sb = plane_batch(P, (long)g.x * g.y, 8);
  const dim3 gz(g.x, g.y, (unsigned)((P.nsys + sb - 1) / sb));
  prof_begin(KID_RBGS, st);
  k_p_rbgs<T><<<gz, BLK, 0, st>>>(L, P.periodic[0], P.periodic[1], shift, active, P.nsys, sb, color, x, b), ::snac::count_launch();
  prof_end(KID_RBGS, st);
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

template <typename T>
int plane_restrict(const MgProblem &P, int l, const T *shift, const int *active, const T *xf, const T *bf, T *bc,
                   T *xc, cudaStream_t st) {
  const MgLevelD &F = P.L[l], &C = P.L[l + 1];
  const dim3 g((unsigned)((C.n[0] + 31) / 32), (unsigned)((C.n[1] + 7) / 8), 1);
  const int sb = plane_batch(P, (long)g.x * g.y, 8);
  const dim3 gz(g.x, g.y, (unsigned)((P.nsys + sb - 1) / sb));
  prof_begin(KID_RESTRICT, st);
  const int e0 = C.coarsened[0] ? 2 : 1, e1 = C.coarsened[1] ? 2 : 1;
  if (e0 == 1 && e1 == 2)
    SNAC_CUDA(launch_k(k_p_restrict<T, 1, 2>, gz, BLK, 0, st, F, C, P.periodic[0], P.periodic[1], shift, active, P.nsys, sb, xf, bf, bc, xc));
  else if (e0 == 2 && e1 == 1)
    SNAC_CUDA(launch_k(k_p_restrict<T, 2, 1>, gz, BLK, 0, st, F, C, P.periodic[0], P.periodic[1], shift, active, P.nsys, sb, xf, bf, bc, xc));
  else if (e0 == 2 && e1 == 2)
    SNAC_CUDA(launch_k(k_p_restrict<T, 2, 2>, gz, BLK, 0, st, F, C, P.periodic[0], P.periodic[1], shift, active, P.nsys, sb, xf, bf, bc, xc));
  else
    SNAC_CUDA(launch_k(k_p_restrict<T, 1, 1>, gz, BLK, 0, st, F, C, P.periodic[0], P.periodic[1], shift, active, P.nsys, sb, xf, bf, bc, xc));
  prof_end(KID_RESTRICT, st);
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

template <typename T>
int plane_prolong(const MgProblem &P, int l, const int *active, T *xf, const T *xc, cudaStream_t st) {
  const MgLevelD &F = P.L[l], &C = P.L[l + 1];
  const dim3 g((unsigned)((F.n[0] + 31) / 32), (unsigned)((F.n[1] + 7) / 8), 1);
  const int sb = plane_batch(P, (long)g.x * g.y, 8);
  const dim3 gz(g.x, g.y, (unsigned)((P.nsys + sb - 1) / sb));
  k_p_prolong<T><<<gz, BLK, 0, st>>>(F, C, active, P.nsys, sb, xf, xc), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

int plane_make_invd(MgProblem &P, double *const *out, float *const *outf, cudaStream_t st) {
  for (int l = 0; l < P.nlev; l++) {
    const MgLevelD &L = P.L[l];
    const dim3 g((unsigned)((L.ncell + 255) / 256), (unsigned)P.nsys);
    k_p_invd<double><<<g, 256, 0, st>>>(L, P.shift, out[l]), ::snac::count_launch();
    k_p_invd<float><<<g, 256, 0, st>>>(L, P.shiftf, outf[l]), ::snac::count_launch();
    SNAC_CUDA(cudaGetLastError());
    P.L[l].invd = out[l];
    P.L[l].invdf = outf[l];
  }
  return SNAC_OK;
}

// the reducing kernels batch systems like the others (P.red_batch = 0: one system per CTA)
static int red_batch(const MgProblem &P, long ctas_per_system) {
  return P.red_batch ? plane_batch(P, ctas_per_system, 8) : 1;
}

template <typename T>
int plane_resid(const MgProblem &P, const T *shift, const int *active, const T *x, const T *b, T *r, double *part_rr,
                double *part_bb, int stride, cudaStream_t st) {
  constexpr int RR = sizeof(T) == 8 ? 4 : RROWS;
  const MgLevelD &L = P.L[0];
  const dim3 g((unsigned)((L.n[0] + 31) / 32), (unsigned)((L.n[1] + 8 * RR - 1) / (8 * RR)), 1);
  const int sb = red_batch(P, (long)g.x * g.y);
  const dim3 gz(g.x, g.y, (unsigned)((P.nsys + sb - 1) / sb));
  SNAC_CUDA(launch_k(k_p_resid<T, RR>, gz, BLK, 0, st, L, P.periodic[0], P.periodic[1], shift, active, P.nsys, sb, x, b,
                     r, part_rr, part_bb, stride));
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

template <typename T, bool FUSEP>
int plane_apply(const MgProblem &P, const T *shift, const int *active, const SysScal *sc, const T *z, const T *po,
                T *pn, T *q, double *part, int stride, cudaStream_t st) {
  const MgLevelD &L = P.L[0];
  const dim3 g((unsigned)((L.n[0] + 31) / 32), (unsigned)((L.n[1] + 8 * RROWS - 1) / (8 * RROWS)), 1);
  const int sb = red_batch(P, (long)g.x * g.y);
  const dim3 gz(g.x, g.y, (unsigned)((P.nsys + sb - 1) / sb));
  SNAC_CUDA(launch_k(k_p_apply<T, FUSEP>, gz, BLK, 0, st, L, P.periodic[0], P.periodic[1], shift, active, P.nsys, sb,
                     sc, z, po, pn, q, part, stride));
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

#define SNAC_PLANE_INST(T)                                                                                           \
  template int plane_sweep<T>(const MgProblem &, int, const T *, const int *, int, T *, const T *, cudaStream_t);    \
  template int plane_restrict<T>(const MgProblem &, int, const T *, const int *, const T *, const T *, T *, T *,     \
                                 cudaStream_t);                                                                      \
  template int plane_prolong<T>(const MgProblem &, int, const int *, T *, const T *, cudaStream_t);                  \
  template int plane_resid<T>(const MgProblem &, const T *, const int *, const T *, const T *, T *, double *,         \
                              double *, int, cudaStream_t);                                                          \
  template int plane_apply<T, true>(const MgProblem &, const T *, const int *, const SysScal *, const T *,           \
                                    const T *, T *, T *, double *, int, cudaStream_t);                               \
  template int plane_apply<T, false>(const MgProblem &, const T *, const int *, const SysScal *, const T *,          \
                                     const T *, T *, T *, double *, int, cudaStream_t);
SNAC_PLANE_INST(double)
SNAC_PLANE_INST(float)
#undef SNAC_PLANE_INST

}  // namespace snac
