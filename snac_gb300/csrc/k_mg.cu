// k_mg.cu -- batched geometric multigrid and conjugate-gradient kernels.
//
// Replaces the HYPRE PFMG/CG solves of solver.f90:524-573 and 843-922.  All
// systems of a solve (every wavenumber of every block in plane mode) advance
// together; one launch covers all of them and systems that have converged are
// skipped through the per-system `active` flags.
//
// Level kernels run on (32, 8) blocks over (i, j) with grid.z = system (plane
// mode) or k plane (3-D mode), so cell coordinates come from the launch shape and
// no thread divides.  Red-black sweeps launch only the cells of one colour.
// Reductions are two-pass: per-CTA partials (accumulated in the vector's own
// type, combined across warps in double) in a fixed layout, then a fixed-order
// sum per system, so results do not depend on scheduling.
//
// T = double runs the plain FP64 path; T = float runs the V-cycles and the
// inner Krylov iterations of the mixed path (FP32 inside FP64 refinement).
#include <algorithm>
#include <utility>

#include "snac_solver.h"
#include "snac_mgk.h"
#include "snac_prof.h"
#include "snac_mgdev.h"

namespace snac {

namespace {
constexpr int FLAT = 2048;  // elements of one system per CTA in the flat vector kernels (256 threads x 8)
constexpr int RROWS = 4;    // rows per thread in the stencil kernels that reduce (32 x 32 cells per CTA)

inline unsigned zdim(const MgProblem &P, const MgLevelD &L) { return P.mode3d ? (unsigned)L.n[2] : (unsigned)P.nsys; }
inline dim3 grid_rb(const MgProblem &P, const MgLevelD &L) {
  return dim3((unsigned)(((L.n[0] + 1) / 2 + 31) / 32), (unsigned)((L.n[1] + 7) / 8), zdim(P, L));
}
inline dim3 grid_cell(const MgProblem &P, const MgLevelD &L) {
  return dim3((unsigned)((L.n[0] + 31) / 32), (unsigned)((L.n[1] + 7) / 8), zdim(P, L));
}
inline dim3 grid_red(const MgProblem &P, const MgLevelD &L) {
  return dim3((unsigned)((L.n[0] + 31) / 32), (unsigned)((L.n[1] + 31) / 32), zdim(P, L));
}
// partials per system of the reducing stencil kernels (generic 3-D ones, or the plane ones)
inline int nchunk_red(const MgProblem &P, const MgLevelD &L) {
  if (!P.mode3d) return plane_nchunk(L);
  const dim3 g = grid_red(P, L);
  return (int)(g.x * g.y * g.z);
}
inline dim3 grid_flat(long n, int nsys) { return dim3((unsigned)((n + FLAT - 1) / FLAT), (unsigned)nsys); }
const dim3 BLK(32, 8);
}  // namespace

int mg_partial_stride(const MgProblem &P) {
  const MgLevelD &L = P.L[0];
  int m = std::max(nchunk_red(P, L), (int)((L.ncell + FLAT - 1) / FLAT));
  if (!P.mode3d) m = std::max(m, tile2d_max_parts(L));
  return m;
}

// ---------------------------------------------------------------- smoothing / transfer
// one red-black half-sweep: the cells with (i + j + k) % 2 == color
// SEP (3-D mode, FP32): couplings and diagonal from the 1-D factors (offdiag_sep / diag_sep), which leaves the
// V-cycle reading x, b, cc and the cell codes instead of five per-cell coefficient arrays
template <typename T, bool SEP>
__global__ void __launch_bounds__(256) k_rbgs(MgLevelD L, MgGeom G, const T *shift, const int *active, int color,
                                              T *x, const T *b) {
  int k, s;
  zpos(G, k, s);
  if (active && !active[s]) return;
  const int j = blockIdx.y * 8 + threadIdx.y;
  const int i = 2 * (int)(blockIdx.x * 32 + threadIdx.x) + ((color + j + k) & 1);
  if (i >= L.n[0] || j >= L.n[1]) return;
  const int c = i + L.n[0] * (j + L.n[1] * k);
  const unsigned cd = L.code[c];
  const long off = L.ncell * s;
  T *__restrict__ xs = x + off;
  // the operands are read before the cell's code is tested (an inactive cell's neighbours are in range too), so
  // the loads do not wait for it; only the store depends on it
  T d, acc;
  if constexpr (SEP) {
    d = diag_sep(L, shift[s], c, i, j, k);
    acc = offdiag_sep(L, G, [&](int e) { return xs[e]; }, c, i, j, k, cd);
  } else {
    d = diag_of<T>(L, G, shift[s], c);
    acc = offdiag<T>(L, G, [&](int e) { return xs[e]; }, c, i, j, k);
  }
  const T bv = b[off + c];
  if (cd & 0x8000) return;
  xs[c] = (bv - acc) * rcpt(d);
}

// coarse b <- sum over children of (b - A x) on the fine level; coarse x <- 0
template <typename T, bool SEP>
__global__ void __launch_bounds__(256) k_resid_restrict(MgLevelD F, MgLevelD C, MgGeom G, const T *shift,
                                                        const int *active, const T *xf, const T *bf, T *bc, T *xc) {
  int K, s;
  zpos(G, K, s);
  if (active && !active[s]) return;
  const int I = blockIdx.x * 32 + threadIdx.x, J = blockIdx.y * 8 + threadIdx.y;
  if (I >= C.n[0] || J >= C.n[1]) return;
  const int cc = I + C.n[0] * (J + C.n[1] * K);
  const long offf = F.ncell * s, offc = C.ncell * s;
  const T *__restrict__ xs = xf + offf;
  const T sh = shift[s];
  T sum = 0;
  const int e0 = C.coarsened[0] ? 2 : 1, e1 = C.coarsened[1] ? 2 : 1, e2 = C.coarsened[2] ? 2 : 1;
  for (int dk = 0; dk < e2; dk++)
    for (int dj = 0; dj < e1; dj++)
      for (int di = 0; di < e0; di++) {
        const int i = C.coarsened[0] ? 2 * I + di : I, j = C.coarsened[1] ? 2 * J + dj : J,
                  k = C.coarsened[2] ? 2 * K + dk : K;
        const int c = i + F.n[0] * (j + F.n[1] * k);
        const unsigned cd = F.code[c];
        if (cd & 0x8000) continue;
        if constexpr (SEP) {
          const T acc = offdiag_sep(F, G, [&](int e) { return xs[e]; }, c, i, j, k, cd);
          sum += bf[offf + c] - fmat(diag_sep(F, sh, c, i, j, k), xs[c], acc);
        } else {
          const T acc = offdiag<T>(F, G, [&](int e) { return xs[e]; }, c, i, j, k);
          sum += bf[offf + c] - fmat(diag_of<T>(F, G, sh, c), xs[c], acc);
        }
      }
  bc[offc + cc] = sum;
  xc[offc + cc] = 0;
}

template <typename T>
__global__ void __launch_bounds__(256) k_prolong(MgLevelD F, MgLevelD C, MgGeom G, const int *active, T *xf,
                                                 const T *xc) {
  int k, s;
  zpos(G, k, s);
  if (active && !active[s]) return;
  const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
  if (i >= F.n[0] || j >= F.n[1]) return;
  const int c = i + F.n[0] * (j + F.n[1] * k);
  if (F.code[c] & 0x8000) return;
  const int I = C.coarsened[0] ? i / 2 : i, J = C.coarsened[1] ? j / 2 : j, K = C.coarsened[2] ? k / 2 : k;
  xf[F.ncell * s + c] += xc[C.ncell * s + I + (long)C.n[0] * (J + (long)C.n[1] * K)];
}

// coarsest level: x = Dinv b, one CTA per system
template <typename T>
__global__ void k_dense(MgLevelD L, const int *active, T *x, const T *b) {
  const int s = blockIdx.x;
  if (active && !active[s]) return;
  __shared__ T sb[MG_DENSE_MAX];
  const int n = (int)L.ncell;
  const long off = (long)n * s;
  for (int q = threadIdx.x; q < n; q += blockDim.x) sb[q] = b[off + q];
  __syncthreads();
  // the inverse is stored by columns (M[c n + r]): a warp's loads of one step are contiguous
  const T *M = LA<T>::dinv(L) + (size_t)n * n * s;
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    T acc = 0;
#pragma unroll 8
    for (int c = 0; c < n; c++) acc = fmat(M[(size_t)c * n + r], sb[c], acc);
    x[off + r] = acc;
  }
}

template <typename T>
__global__ void k_zero(long n, T *x, int nsys, const int *active) {
  const int s = blockIdx.y;
  if (active && !active[s]) return;
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) x[n * s + c] = 0;
}

// the factored-coupling kernels serve the FP32 V-cycles and Krylov iterations of the 3-D mode
template <typename T>
inline bool sep_ok(const MgProblem &P) { return sizeof(T) == 4 && P.mode3d && P.sep; }

template <typename T>
int launch_rbgs3(const MgProblem &P, const MgLevelD &L, const MgGeom &G, const T *shift, const int *active, int color,
                 T *x, const T *b, cudaStream_t st) {
  prof_begin(KID_RBGS, st);
  if (sep_ok<T>(P)) k_rbgs<T, true><<<grid_rb(P, L), BLK, 0, st>>>(L, G, shift, active, color, x, b), ::snac::count_launch();
  else k_rbgs<T, false><<<grid_rb(P, L), BLK, 0, st>>>(L, G, shift, active, color, x, b), ::snac::count_launch();
  prof_end(KID_RBGS, st);
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

// V-cycle on level l: x_l <- M b_l (zero initial guess); x and b of each level are the level's own arrays.
// At level 0 the last smoothing pass may also produce the partials of b.x (= r.z) into part_bx, and for the
// singular systems those of x and of b into part_x and part_b.
template <typename T>
int mg_vcycle_impl(const MgProblem &P, const MgGeom &G, int l, const T *shift, const int *active, double *part_bx,
                   double *part_x, double *part_b, int part_stride, int *nchunk_bx, cudaStream_t st) {
  const MgLevelD &L = P.L[l];
  T *x = LA<T>::x(L);
  T *b = LA<T>::b(L);
  const int prec = sizeof(T) == 8 ? 1 : 0;
  const int fuse = prec ? P.fused >> 2 : P.fused & 3;
  if (nchunk_bx) *nchunk_bx = 0;
  trace("vcycle: enter level", st);
  if ((fuse & 2) && !P.mode3d && l >= P.cta_level[prec]) return launch_vcycle_coarse<T>(P, l, shift, active, x, b, st);
  if ((fuse & 2) && P.mode3d && l >= P.cta_level[prec]) return launch_vcycle_coarse3d<T>(P, G, l, shift, active, x, b, st);
  if (l == P.nlev - 1) {
    if (LA<T>::dinv(L)) {
      k_dense<T><<<P.nsys, 256, 0, st>>>(L, active, x, b), ::snac::count_launch();
    } else {
      const dim3 g((unsigned)((L.ncell + 255) / 256), P.nsys);
      k_zero<T><<<g, 256, 0, st>>>(L.ncell, x, P.nsys, active), ::snac::count_launch();
      for (int it = 0; it < 40; it++)
        for (int col : {0, 1, 1, 0}) {
          if (P.mode3d) SNAC_TRY(launch_rbgs3<T>(P, L, G, shift, active, col, x, b, st));
          else SNAC_TRY(plane_sweep<T>(P, l, shift, active, col, x, b, st));
        }
    }
    SNAC_CUDA(cudaGetLastError());
    return SNAC_OK;
  }
  const MgLevelD &C = P.L[l + 1];
  if ((fuse & 1) && tile2d_ok(P, l, prec)) {
    T *xp = LA<T>::xp(P.L[l]);  // pre-smoothed x (the post-smoother reads it while writing x)
    if (!prec && P.tile_restrict) {
      // the pre-smoother restricts its own residual; the coarse x needs zeroing only where the next level is
      // swept from x (neither the one-CTA coarse V-cycle nor a tiled pre-smoother, which start from zero)
      const bool next_from_zero = ((fuse & 2) && l + 1 >= P.cta_level[prec]) || ((fuse & 1) && tile2d_ok(P, l + 1, prec));
      SNAC_TRY(launch_rbgs_tile2d_restrict<T>(P, l, active, xp, b, LA<T>::b(C), next_from_zero ? nullptr : LA<T>::x(C),
                                              st));
    } else {
      SNAC_TRY(launch_rbgs_tile2d<T>(P, l, active, 0, 0, xp, b, (const T *)nullptr, (const T *)nullptr, nullptr,
                                     nullptr, nullptr, 0, nullptr, st));
      SNAC_TRY(plane_restrict<T>(P, l, shift, active, xp, b, LA<T>::b(C), LA<T>::x(C), st));
    }
    SNAC_TRY(mg_vcycle_impl<T>(P, G, l + 1, shift, active, nullptr, nullptr, nullptr, 0, nullptr, st));
    return launch_rbgs_tile2d<T>(P, l, active, 1, 1, x, b, (const T *)xp, (const T *)LA<T>::x(C), part_bx, part_x,
                                 part_b, part_stride, nchunk_bx, st);
  }
  if (l == 0) {  // coarse x is zeroed by the restriction
    const dim3 g((unsigned)((L.ncell + 255) / 256), P.nsys);
    k_zero<T><<<g, 256, 0, st>>>(L.ncell, x, P.nsys, active), ::snac::count_launch();
  }
  if (!P.mode3d) {  // plane systems: kernels batched over systems
    for (int it = 0; it < 2 * mg_nu(P, l); it++) SNAC_TRY(plane_sweep<T>(P, l, shift, active, it & 1, x, b, st));
    SNAC_TRY(plane_restrict<T>(P, l, shift, active, x, b, LA<T>::b(C), LA<T>::x(C), st));
    SNAC_TRY(mg_vcycle_impl<T>(P, G, l + 1, shift, active, nullptr, nullptr, nullptr, 0, nullptr, st));
    SNAC_TRY(plane_prolong<T>(P, l, active, x, LA<T>::x(C), st));
    for (int it = 0; it < 2 * mg_nu(P, l); it++) SNAC_TRY(plane_sweep<T>(P, l, shift, active, 1 - (it & 1), x, b, st));
    return SNAC_OK;
  }
  for (int it = 0; it < 2 * mg_nu(P, l); it++) {
    SNAC_TRY(launch_rbgs3<T>(P, L, G, shift, active, it & 1, x, b, st));
  }
  prof_begin(KID_RESTRICT, st);
  if (sep_ok<T>(P))
    k_resid_restrict<T, true><<<grid_cell(P, C), BLK, 0, st>>>(L, C, G, shift, active, x, b, LA<T>::b(C), LA<T>::x(C)), ::snac::count_launch();
  else
    k_resid_restrict<T, false><<<grid_cell(P, C), BLK, 0, st>>>(L, C, G, shift, active, x, b, LA<T>::b(C), LA<T>::x(C)), ::snac::count_launch();
  prof_end(KID_RESTRICT, st);
  SNAC_CUDA(cudaGetLastError());
  SNAC_TRY(mg_vcycle_impl<T>(P, G, l + 1, shift, active, nullptr, nullptr, nullptr, 0, nullptr, st));
  k_prolong<T><<<grid_cell(P, L), BLK, 0, st>>>(L, C, G, active, x, LA<T>::x(C)), ::snac::count_launch();
  for (int it = 0; it < 2 * mg_nu(P, l); it++) {
    SNAC_TRY(launch_rbgs3<T>(P, L, G, shift, active, 1 - (it & 1), x, b, st));
  }
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

// ---------------------------------------------------------------- Krylov kernels (level 0)
// r = b - A x; partials of r.r and b.b.  Each thread covers RROWS rows of a 32 x 32 patch.
template <typename T>
__global__ void __launch_bounds__(256) k_cg_resid(MgLevelD L, MgGeom G, const T *shift, const int *active, const T *x,
                                                  const T *b, T *r, double *part_rr, double *part_bb, int stride) {
  int k, s;
  zpos(G, k, s);
  if (active && !active[s]) return;
  const long off = L.ncell * s;
  const T *__restrict__ xs = x + off;
  const T sh = shift[s];
  const int i = blockIdx.x * 32 + threadIdx.x;
  T rr = 0, bb = 0;
  for (int q = 0; q < RROWS; q++) {
    const int j = blockIdx.y * 32 + threadIdx.y + 8 * q;
    if (i >= L.n[0] || j >= L.n[1]) continue;
    const int c = i + L.n[0] * (j + L.n[1] * k);
    T rv = 0;
    if (!(L.code[c] & 0x8000)) {
      const T acc = offdiag<T>(L, G, [&](int e) { return xs[e]; }, c, i, j, k);
      const T bv = b[off + c];
      rv = bv - fmat(diag_of<T>(L, G, sh, c), xs[c], acc);
      rr = fmat(rv, rv, rr);
      bb = fmat(bv, bv, bb);
    }
    r[off + c] = rv;
  }
  double trr, tbb;
  block_sum2<T>(rr, bb, trr, tbb);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    const long e = (long)s * stride + blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * (long)k);
    part_rr[e] = trr;
    if (part_bb) part_bb[e] = tbb;
  }
}

// partial dot a.b (flat); for the singular systems (singular given) also the partial sums of b and of a over
// the active cells, into part_b and part_a
template <typename T>
__global__ void __launch_bounds__(256) k_cg_dot(long n, const int *active, const T *a, const T *b, double *part,
                                                int stride, const unsigned short *code, const int *singular,
                                                double *part_a, double *part_b) {
  const int s = blockIdx.y;
  if (active && !active[s]) return;
  const long base = (long)blockIdx.x * FLAT + threadIdx.x, o = n * s;
  T v = 0;
#pragma unroll
  for (int e = 0; e < FLAT / 256; e++) {
    const long c = base + 256 * e;
    if (c < n) v = fmat(a[o + c], b[o + c], v);
  }
  const double t = block_sum1<T>(v);
  if (threadIdx.x == 0) part[(long)s * stride + blockIdx.x] = t;
  if (singular && singular[s]) {
    T sa = 0, sb = 0;
    for (int e = 0; e < FLAT / 256; e++) {
      const long c = base + 256 * e;
      if (c < n && !(code[c] & 0x8000)) { sa += a[o + c]; sb += b[o + c]; }
    }
    double ta, tb;
    block_sum2<T>(sa, sb, ta, tb);
    if (threadIdx.x == 0) { part_a[(long)s * stride + blockIdx.x] = ta; part_b[(long)s * stride + blockIdx.x] = tb; }
  }
}

// fixed-order sum of the n partials of system s by one CTA (result valid in every thread)
__device__ __forceinline__ double cta_sum_parts(const double *part, int s, int stride, int n) {
  double acc = 0.0;
  for (int q = threadIdx.x; q < n; q += blockDim.x) acc += part[(long)s * stride + q];
  __shared__ double tot;
  const double t = block_sum1<double>(acc);
  if (threadIdx.x == 0) tot = t;
  __syncthreads();
  return tot;
}

// convergence of system s from its r.r (k_cg_norms without set_bb; thread 0 only): the system leaves the
// running loop when its relative residual reaches its tolerance or its right-hand side is zero
__device__ __forceinline__ bool cg_converged(SysScal &q, double rr, double tol) {
  q.rr = rr;
  const double bb = q.bb;
  const double rel = bb > 0.0 ? sqrt(rr / bb) : 0.0;
  q.rel = rel;
  const double ts = q.tol > 0.0 ? q.tol : tol;
  if (bb == 0.0) { q.zero_rhs = 1; return true; }
  return rel <= ts;
}

// The start of a Krylov iteration after the V-cycle z = M r, one CTA per system:
//  * r.z from the partials of the V-cycle's last pass or of k_cg_dot; for a singular system z is taken
//    orthogonal to the constant (its null space): zmean = sum(z)/nact over the active cells, which the new
//    search direction leaves out (p = z - zmean + beta p), and r.z becomes r.(z - zmean) = r.z - zmean sum(r),
//    from the partial sums of z and r made by the same pass;
//  * beta = r.z / r.z_old (0 on the first iteration).
__global__ void k_cg_beta2(const int *active, const int *singular, SysScal *sc, const double *part_rz,
                           const double *part_z, const double *part_r, int nrz, long nact, int stride) {
  pdl_enter();
  const int s = blockIdx.x;
  if (!active[s]) return;
  double rz = cta_sum_parts(part_rz, s, stride, nrz);
  double zmean = 0.0;
  if (singular[s]) {
    const double sz = cta_sum_parts(part_z, s, stride, nrz);
    const double sr = cta_sum_parts(part_r, s, stride, nrz);
    zmean = nact > 0 ? sz / (double)nact : 0.0;
    rz -= zmean * sr;
  }
  if (threadIdx.x == 0) {
    sc[s].zmean = zmean;
    sc[s].beta = sc[s].first ? 0.0 : rz / sc[s].rz;
    sc[s].rz = rz;
    sc[s].first = 0;
  }
}

// convergence test after an update without a host check (k_cg_norms without the count), one CTA per system
__global__ void k_cg_conv(int *active, SysScal *sc, const double *part_rr, int nrr, double tol, int stride) {
  pdl_enter();
  const int s = blockIdx.x;
  if (!active[s]) return;
  const double rr = cta_sum_parts(part_rr, s, stride, nrr);
  if (threadIdx.x == 0 && cg_converged(sc[s], rr, tol)) active[s] = 0;
}

// alpha = rz / p.q; one CTA per system
__global__ void k_cg_alpha(const int *active, SysScal *sc, const double *part, int stride, int n) {
  pdl_enter();
  const int s = blockIdx.x;
  if (active && !active[s]) return;
  const double pq = cta_sum_parts(part, s, stride, n);
  if (threadIdx.x == 0) sc[s].alpha = sc[s].rz / pq;
}

// p = (z - zmean) + beta p (flat; FP64 path)
template <typename T>
__global__ void __launch_bounds__(256) k_cg_p(long n, const int *active, const SysScal *sc, const T *z, T *p) {
  const int s = blockIdx.y;
  if (active && !active[s]) return;
  const T beta = (T)sc[s].beta, zm = (T)sc[s].zmean;
  const long base = (long)blockIdx.x * FLAT + threadIdx.x, o = n * s;
#pragma unroll
  for (int e = 0; e < FLAT / 256; e++) {
    const long c = base + 256 * e;
    if (c < n) p[o + c] = fmat(beta, p[o + c], z[o + c] - zm);
  }
}

// q = A p; partials of p.q.  FUSEP: the new direction p = (z - zmean) + beta p_old is formed on the fly (at
// the centre and at the neighbours) and written to pn, so p_old and pn must be different arrays.
template <typename T, bool FUSEP, bool SEP = false>
__global__ void __launch_bounds__(256) k_cg_apply(MgLevelD L, MgGeom G, const T *shift, const int *active,
                                                  const SysScal *sc, const T *z, const T *po, T *pn, T *q,
                                                  double *part, int stride) {
  int k, s;
  zpos(G, k, s);
  if (active && !active[s]) return;
  const long off = L.ncell * s;
  const T *__restrict__ zs = z + off;
  const T *__restrict__ ps = po + off;
  const T beta = FUSEP ? (T)sc[s].beta : T(0), zm = FUSEP ? (T)sc[s].zmean : T(0);
  const T sh = shift[s];
  auto pv = [&](int e) -> T { return FUSEP ? fmat(beta, ps[e], zs[e] - zm) : ps[e]; };
  const int i = blockIdx.x * 32 + threadIdx.x;
  T pq = 0;
  for (int qq = 0; qq < RROWS; qq++) {
    const int j = blockIdx.y * 32 + threadIdx.y + 8 * qq;
    if (i >= L.n[0] || j >= L.n[1]) continue;
    const int c = i + L.n[0] * (j + L.n[1] * k);
    const T pc = pv(c);
    if (FUSEP) pn[off + c] = pc;
    T y = 0;
    const unsigned cd = L.code[c];
    if (!(cd & 0x8000)) {
      if constexpr (SEP) {
        const T acc = offdiag_sep(L, G, pv, c, i, j, k, cd);
        y = fmat(diag_sep(L, sh, c, i, j, k), pc, acc);
      } else {
        const T acc = offdiag<T>(L, G, pv, c, i, j, k);
        y = fmat(diag_of<T>(L, G, sh, c), pc, acc);
      }
    }
    q[off + c] = y;
    pq = fmat(pc, y, pq);
  }
  const double t = block_sum1<T>(pq);
  if (threadIdx.x == 0 && threadIdx.y == 0)
    part[(long)s * stride + blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * (long)k)] = t;
}

// x += alpha p (x = alpha p when zero_x); r -= alpha q; partials of r.r (flat)
template <typename T>
__global__ void __launch_bounds__(256) k_cg_xr(long n, const int *active, const SysScal *sc, const T *p, const T *q,
                                               T *x, T *r, double *part_rr, int stride, int zero_x) {
  pdl_enter();
  const int s = blockIdx.y;
  if (active && !active[s]) return;
  const T alpha = (T)sc[s].alpha;
  const long base = (long)blockIdx.x * FLAT + threadIdx.x, o = n * s;
  T rr = 0;
#pragma unroll
  for (int e = 0; e < FLAT / 256; e++) {
    const long c = base + 256 * e;
    if (c < n) {
      x[o + c] = zero_x ? alpha * p[o + c] : fmat(alpha, p[o + c], x[o + c]);
      const T rv = fmat(-alpha, q[o + c], r[o + c]);
      r[o + c] = rv;
      rr = fmat(rv, rv, rr);
    }
  }
  const double t = block_sum1<T>(rr);
  if (threadIdx.x == 0) part_rr[(long)s * stride + blockIdx.x] = t;
}

// Residual norms: rel = sqrt(rr/bb); active flags; count[0] += still active, count[1] += zero right-hand
// sides.  One CTA per system.  set_bb: bb (and the start-of-solve flags) from part_bb.  want_scale:
// scale = RMS of the residual over nact cells.  src_active: flags are first copied from there.
__global__ void k_cg_norms(int *active, const int *src_active, SysScal *sc, const double *part_rr,
                           const double *part_bb, int stride, int n, double tol, int set_bb, int want_scale,
                           long nact, int *count, const SysScal *outer, double outer_tol) {
  pdl_enter();
  const int s = blockIdx.x;
  if (src_active) {
    if (threadIdx.x == 0) active[s] = src_active[s];
    __syncthreads();
  }
  if (!active[s]) return;
  double rr = cta_sum_parts(part_rr, s, stride, n);
  const double bbn = set_bb ? cta_sum_parts(part_bb, s, stride, n) : 0.0;
  if (threadIdx.x != 0) return;
  if (set_bb) {
    sc[s].bb = bbn;
    sc[s].first = 1;
    sc[s].zero_rhs = 0;
    // a warm start worse than zero (||b - A x0|| > ||b||) is dropped: the solve then starts from x = 0,
    // r = b, which also avoids the cancellation of a large A x0 against a small b
    sc[s].restart = (bbn > 0.0 && rr > bbn) ? 1 : 0;
    if (sc[s].restart) rr = bbn;
    // the start of an inner solve of iterative refinement: reduce this system's residual only as far as its
    // outer residual needs (a tenth of outer_tol / its relative outer residual), never below tol
    sc[s].tol = 0.0;
    if (outer) sc[s].tol = fmin(0.5, fmax(tol, 0.1 * outer_tol / outer[s].rel));
  }
  sc[s].rr = rr;
  if (want_scale) {
    const double v = sqrt(rr / (double)(nact > 0 ? nact : 1));
    sc[s].scale = v > 0.0 ? v : 1.0;
  }
  const double bb = sc[s].bb;
  const double rel = bb > 0.0 ? sqrt(rr / bb) : 0.0;
  sc[s].rel = rel;
  const double ts = sc[s].tol > 0.0 ? sc[s].tol : tol;
  if (bb == 0.0) { sc[s].zero_rhs = 1; active[s] = 0; atomicAdd(count + 1, 1); }
  else if (rel <= ts) active[s] = 0;
  else atomicAdd(count, 1);
}

// systems flagged by k_cg_norms: x = 0, r = b
template <typename T>
__global__ void k_restart_systems(long n, const SysScal *sc, T *x, const T *b, T *r) {
  const int s = blockIdx.y;
  if (!sc[s].restart) return;
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) { x[n * s + c] = 0; r[n * s + c] = b[n * s + c]; }
}

// systems with an all-zero right-hand side get x = 0 (as HYPRE does)
template <typename T>
__global__ void k_zero_rhs_systems(long n, const SysScal *sc, T *x) {
  const int s = blockIdx.y;
  if (!sc[s].zero_rhs) return;
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) x[n * s + c] = 0;
}

// singular systems: b -= mean(b) over active cells (two passes, flat chunks)
template <typename T>
__global__ void __launch_bounds__(256) k_sum_active(MgLevelD L, const int *sing_list, const T *b, double *part,
                                                    double *partn, int stride) {
  const int s = sing_list[blockIdx.y];  // the singular systems only
  const long base = (long)blockIdx.x * FLAT + threadIdx.x, n = L.ncell;
  double v = 0.0, m = 0.0;
  for (int e = 0; e < FLAT / 256; e++) {
    const long c = base + 256 * e;
    if (c < n && !(L.code[c] & 0x8000)) { v += (double)b[n * s + c]; m += 1.0; }
  }
  double tv, tm;
  block_sum2<double>(v, m, tv, tm);
  if (threadIdx.x == 0) { part[(long)s * stride + blockIdx.x] = tv; partn[(long)s * stride + blockIdx.x] = tm; }
}
template <typename T>
__global__ void __launch_bounds__(256) k_sub_mean(MgLevelD L, const int *sing_list, T *b, const double *part,
                                                  const double *partn, int stride, int nchunk) {
  const int s = sing_list[blockIdx.y];
  const double na = cta_sum_parts(partn, s, stride, nchunk);
  const double sm = cta_sum_parts(part, s, stride, nchunk);
  const double mean = na > 0.0 ? sm / na : 0.0;
  const long base = (long)blockIdx.x * FLAT + threadIdx.x, n = L.ncell;
  for (int e = 0; e < FLAT / 256; e++) {
    const long c = base + 256 * e;
    if (c < n && !(L.code[c] & 0x8000)) b[n * s + c] -= (T)mean;
  }
}

// mixed path: r32 = r64 / scale_s; e32 = 0; partials of r32.r32
__global__ void __launch_bounds__(256) k_ir_down(long n, const int *active, const SysScal *sc, const double *r,
                                                 float *r32, float *e32, double *part, int stride) {
  pdl_enter();
  const int s = blockIdx.y;
  if (active && !active[s]) return;
  const double inv = 1.0 / sc[s].scale;
  const long base = (long)blockIdx.x * FLAT + threadIdx.x, o = n * s;
  float rr = 0.f;
#pragma unroll
  for (int e = 0; e < FLAT / 256; e++) {
    const long c = base + 256 * e;
    if (c < n) {
      const float v = (float)(r[o + c] * inv);
      r32[o + c] = v;
      e32[o + c] = 0.0f;
      rr = fmat(v, v, rr);
    }
  }
  const double t = block_sum1<float>(rr);
  if (threadIdx.x == 0) part[(long)s * stride + blockIdx.x] = t;
}
__global__ void __launch_bounds__(256) k_ir_up(long n, const int *active, const SysScal *sc, const float *e32,
                                               double *x) {
  pdl_enter();
  const int s = blockIdx.y;
  if (active && !active[s]) return;
  const double scale = sc[s].scale;
  const long base = (long)blockIdx.x * FLAT + threadIdx.x, o = n * s;
#pragma unroll
  for (int e = 0; e < FLAT / 256; e++) {
    const long c = base + 256 * e;
    if (c < n) x[o + c] = fmat(scale, (double)e32[o + c], x[o + c]);
  }
}

__global__ void k_sc_first(int nsys, SysScal *sc) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys) sc[s].first = 1;
}

// active[s] = src ? src[s] : 1
__global__ void k_set_active(int nsys, int *active, const int *src) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys) active[s] = src ? src[s] : 1;
}

// Explicit instantiation of every kernel template for both precisions, so that the
// device code of each kernel exists whatever host template reaches its launch.
#define SNAC_MG_KERNELS(T)                                                                                           \
  template __global__ void k_rbgs<T, false>(MgLevelD, MgGeom, const T *, const int *, int, T *, const T *);          \
  template __global__ void k_resid_restrict<T, false>(MgLevelD, MgLevelD, MgGeom, const T *, const int *, const T *, \
                                               const T *, T *, T *);                                                 \
  template __global__ void k_prolong<T>(MgLevelD, MgLevelD, MgGeom, const int *, T *, const T *);                    \
  template __global__ void k_dense<T>(MgLevelD, const int *, T *, const T *);                                        \
  template __global__ void k_zero<T>(long, T *, int, const int *);                                                   \
  template __global__ void k_cg_resid<T>(MgLevelD, MgGeom, const T *, const int *, const T *, const T *, T *,        \
                                         double *, double *, int);                                                   \
  template __global__ void k_cg_dot<T>(long, const int *, const T *, const T *, double *, int,                      \
                                       const unsigned short *, const int *, double *, double *);                     \
  template __global__ void k_cg_p<T>(long, const int *, const SysScal *, const T *, T *);                            \
  template __global__ void k_cg_apply<T, true>(MgLevelD, MgGeom, const T *, const int *, const SysScal *, const T *, \
                                               const T *, T *, T *, double *, int);                                  \
  template __global__ void k_cg_apply<T, false>(MgLevelD, MgGeom, const T *, const int *, const SysScal *,          \
                                                const T *, const T *, T *, T *, double *, int);                      \
  template __global__ void k_cg_xr<T>(long, const int *, const SysScal *, const T *, const T *, T *, T *, double *,  \
                                      int, int);                                                                     \
  template __global__ void k_zero_rhs_systems<T>(long, const SysScal *, T *);                                       \
  template __global__ void k_sum_active<T>(MgLevelD, const int *, const T *, double *, double *, int);               \
  template __global__ void k_sub_mean<T>(MgLevelD, const int *, T *, const double *, const double *, int, int);
SNAC_MG_KERNELS(double)
SNAC_MG_KERNELS(float)
#undef SNAC_MG_KERNELS
template __global__ void k_rbgs<float, true>(MgLevelD, MgGeom, const float *, const int *, int, float *, const float *);
template __global__ void k_resid_restrict<float, true>(MgLevelD, MgLevelD, MgGeom, const float *, const int *,
                                                       const float *, const float *, float *, float *);
template __global__ void k_cg_apply<float, true, true>(MgLevelD, MgGeom, const float *, const int *, const SysScal *,
                                                       const float *, const float *, float *, float *, double *, int);

// ---------------------------------------------------------------- host drivers
namespace {
MgGeom geom_of(const MgProblem &P) {
  MgGeom G;
  G.mode3d = P.mode3d;
  for (int a = 0; a < 3; a++) G.periodic[a] = P.periodic[a];
  return G;
}
template <typename T> const T *shift_of(const MgProblem &P);
template <> const double *shift_of<double>(const MgProblem &P) { return P.shift; }
template <> const float *shift_of<float>(const MgProblem &P) { return P.shiftf; }
}  // namespace

template <typename T>
int mg_vcycle(const MgProblem &P, int l, const int *active, cudaStream_t st) {
  return mg_vcycle_impl<T>(P, geom_of(P), l, shift_of<T>(P), active, nullptr, nullptr, nullptr, 0, nullptr, st);
}
template int mg_vcycle<double>(const MgProblem &, int, const int *, cudaStream_t);
template int mg_vcycle<float>(const MgProblem &, int, const int *, cudaStream_t);

int mg_set_active(int nsys, int *active, const int *src, cudaStream_t st) {
  k_set_active<<<(nsys + 127) / 128, 128, 0, st>>>(nsys, active, src), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

template <typename T>
int mg_residual(const MgProblem &P, CgWork &W, const T *x, const T *b, T *r, double tol, int set_bb, int want_scale,
                long nact, cudaStream_t st) {
  const MgGeom G = geom_of(P);
  const MgLevelD &L0 = P.L[0];
  if (P.mode3d)
    k_cg_resid<T><<<grid_red(P, L0), BLK, 0, st>>>(L0, G, shift_of<T>(P), W.active, x, b, r, W.part0,
                                                   set_bb ? W.part1 : nullptr, W.stride), ::snac::count_launch();
  else
    SNAC_TRY(plane_resid<T>(P, shift_of<T>(P), W.active, x, b, r, W.part0, set_bb ? W.part1 : nullptr, W.stride, st));
  SNAC_CUDA(cudaMemsetAsync(W.d_count, 0, 2 * sizeof(int), st));
  const int nres = P.mode3d ? nchunk_red(P, L0) : plane_resid_nchunk(L0, sizeof(T) == 8 ? 1 : 0);
  k_cg_norms<<<P.nsys, 256, 0, st>>>(W.active, nullptr, W.sc, W.part0, W.part1, W.stride, nres, tol,
                                     set_bb, want_scale, nact, W.d_count, nullptr, 0.0), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}
template int mg_residual<double>(const MgProblem &, CgWork &, const double *, const double *, double *, double, int,
                                 int, long, cudaStream_t);
template int mg_residual<float>(const MgProblem &, CgWork &, const float *, const float *, float *, double, int, int,
                                long, cudaStream_t);

int mg_restart_bad_guess(const MgProblem &P, CgWork &W, double *x, const double *b, double *r, cudaStream_t st) {
  const long n = P.L[0].ncell;
  k_restart_systems<double><<<dim3((unsigned)((n + 255) / 256), P.nsys), 256, 0, st>>>(n, W.sc, x, b, r), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

int mg_restart_krylov(const MgProblem &P, CgWork &W, cudaStream_t st) {
  k_sc_first<<<(P.nsys + 127) / 128, 128, 0, st>>>(P.nsys, W.sc), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

int mg_zero_rhs_systems(const MgProblem &P, const CgWork &W, double *x, cudaStream_t st) {
  const long n = P.L[0].ncell;
  k_zero_rhs_systems<double><<<dim3((unsigned)((n + 255) / 256), P.nsys), 256, 0, st>>>(n, W.sc, x), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

// preconditioned CG on level 0 of P for all active systems (T-typed vectors); returns iterations done
template <typename T>
int mg_pcg(const MgProblem &P, CgWork &W, T *x, int maxiter, double tol, bool zero_x, bool check_host, int *iters,
           cudaStream_t st) {
  const MgGeom G = geom_of(P);
  const T *shift = shift_of<T>(P);
  const MgLevelD &L0 = P.L[0];
  const long n = L0.ncell;
  const dim3 gf = grid_flat(n, P.nsys);
  const int nflat = (int)gf.x, nred = nchunk_red(P, L0);
  constexpr bool fusep = sizeof(T) == 4;  // FP32: the p update is folded into the operator application
  T *r = (T *)W.r, *z = (T *)W.z, *q = (T *)W.q;
  T *p = (T *)W.p, *pn = (T *)W.p2;
  int it = 0;
  for (it = 1; it <= maxiter; it++) {
    if (check_host) {
      SNAC_CUDA(cudaMemcpyAsync(W.h_count, W.d_count, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
      SNAC_CUDA(cudaStreamSynchronize(st));
      if (W.h_count[0] == 0) { it--; break; }
    }
    // z = M r : V-cycle with level-0 b = r, x = z; its last pass may already give the r.z partials
    MgProblem Pz = P;
    if constexpr (sizeof(T) == 8) { Pz.L[0].b = (double *)r; Pz.L[0].x = (double *)z; }
    else { Pz.L[0].bf = (float *)r; Pz.L[0].xf = (float *)z; }
    int nrz = 0;
    SNAC_TRY(mg_vcycle_impl<T>(Pz, G, 0, shift, W.active, W.part2, W.part3, W.part4, W.stride, &nrz, st));
    trace("pcg: V-cycle", st);
    if (nrz == 0) {
      k_cg_dot<T><<<gf, 256, 0, st>>>(n, W.active, r, z, W.part2, W.stride, L0.code,
                                      P.any_singular ? P.singular : nullptr, W.part4, W.part3), ::snac::count_launch();
      nrz = nflat;
    }
    // singular systems: the search directions carry no constant (z's mean is left out of p), so x - x0 stays
    // mean-free, and r.z is taken with the projected z (r's mean is zero only up to rounding, and the V-cycle's
    // constant drift can be large)
    SNAC_CUDA(launch_k(k_cg_beta2, dim3(P.nsys), dim3(256), 0, st, W.active, P.singular, W.sc, W.part2, W.part3,
                       W.part4, nrz, P.nact0, W.stride));
    prof_begin(KID_CG_APPLY, st);
    if constexpr (fusep) {
      if (P.mode3d && sep_ok<T>(P))
        k_cg_apply<T, true, true><<<grid_red(P, L0), BLK, 0, st>>>(L0, G, shift, W.active, W.sc, z, p, pn, q,
                                                                   W.part1, W.stride), ::snac::count_launch();
      else if (P.mode3d)
        k_cg_apply<T, true><<<grid_red(P, L0), BLK, 0, st>>>(L0, G, shift, W.active, W.sc, z, p, pn, q, W.part1,
                                                             W.stride), ::snac::count_launch();
      else
        SNAC_TRY((plane_apply<T, true>(P, shift, W.active, W.sc, z, p, pn, q, W.part1, W.stride, st)));
      std::swap(p, pn);
    } else {
      k_cg_p<T><<<gf, 256, 0, st>>>(n, W.active, W.sc, z, p), ::snac::count_launch();
      if (P.mode3d)
        k_cg_apply<T, false><<<grid_red(P, L0), BLK, 0, st>>>(L0, G, shift, W.active, W.sc, z, p, nullptr, q,
                                                              W.part1, W.stride), ::snac::count_launch();
      else
        SNAC_TRY((plane_apply<T, false>(P, shift, W.active, W.sc, z, p, nullptr, q, W.part1, W.stride, st)));
    }
    prof_end(KID_CG_APPLY, st);
    SNAC_CUDA(launch_k(k_cg_alpha, dim3(P.nsys), dim3(256), 0, st, W.active, W.sc, W.part1, W.stride, nred));
    SNAC_CUDA(launch_k(k_cg_xr<T>, gf, dim3(256), 0, st, n, W.active, W.sc, p, q, x, r, W.part0, W.stride,
                       (zero_x && it == 1) ? 1 : 0));
    if (check_host) {  // the host reads the count before the next iteration
      SNAC_CUDA(cudaMemsetAsync(W.d_count, 0, 2 * sizeof(int), st));
      k_cg_norms<<<P.nsys, 256, 0, st>>>(W.active, nullptr, W.sc, W.part0, nullptr, W.stride, nflat, tol, 0, 0, 0,
                                         W.d_count, nullptr, 0.0), ::snac::count_launch();
    } else if (it < maxiter) {  // converged systems leave the loop before the next V-cycle (no count needed)
      SNAC_CUDA(launch_k(k_cg_conv, dim3(P.nsys), dim3(256), 0, st, W.active, W.sc, W.part0, nflat, tol, W.stride));
    }
    SNAC_CUDA(cudaGetLastError());
    trace("pcg: iteration", st);
  }
  if (it > maxiter) it = maxiter;
  *iters = it;
  return SNAC_OK;
}
template int mg_pcg<double>(const MgProblem &, CgWork &, double *, int, double, bool, bool, int *, cudaStream_t);
template int mg_pcg<float>(const MgProblem &, CgWork &, float *, int, double, bool, bool, int *, cudaStream_t);

int mg_project_singular(const MgProblem &P, CgWork &W, double *b, cudaStream_t st) {
  if (!P.any_singular) return SNAC_OK;
  const long n = P.L[0].ncell;
  const dim3 g(grid_flat(n, P.nsys).x, (unsigned)P.nsing);
  k_sum_active<double><<<g, 256, 0, st>>>(P.L[0], P.sing_list, b, W.part0, W.part1, W.stride), ::snac::count_launch();
  k_sub_mean<double><<<g, 256, 0, st>>>(P.L[0], P.sing_list, b, W.part0, W.part1, W.stride, (int)g.x), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

int mg_ir_down(const MgProblem &P, const CgWork &Wout, CgWork &W32, const double *r64, float *r32, float *e32,
               double inner_tol, double outer_tol, cudaStream_t st) {
  const long n = P.L[0].ncell;
  const dim3 gf = grid_flat(n, P.nsys);
  SNAC_CUDA(launch_k(k_ir_down, gf, dim3(256), 0, st, n, Wout.active, Wout.sc, r64, r32, e32, W32.part0, W32.stride));
  SNAC_CUDA(cudaMemsetAsync(W32.d_count, 0, 2 * sizeof(int), st));
  k_cg_norms<<<P.nsys, 256, 0, st>>>(W32.active, Wout.active, W32.sc, W32.part0, W32.part0, W32.stride, (int)gf.x,
                                     inner_tol, 1, 0, 0, W32.d_count, outer_tol > 0.0 ? Wout.sc : nullptr, outer_tol),
      ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}
int mg_ir_up(const MgProblem &P, const CgWork &Wout, const float *e32, double *x, cudaStream_t st) {
  const long n = P.L[0].ncell;
  SNAC_CUDA(launch_k(k_ir_up, grid_flat(n, P.nsys), dim3(256), 0, st, n, Wout.active, Wout.sc, e32, x));
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

}  // namespace snac
