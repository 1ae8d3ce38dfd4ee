// k_mg.cu -- batched geometric multigrid and conjugate-gradient kernels.
//
// Replaces the HYPRE PFMG/CG solves of solver.f90:524-573 and 843-922.  All
// systems of a solve (every wavenumber of every block in plane mode) advance
// together; one launch covers all of them (blockIdx.y = system) and systems
// that have converged are skipped through the per-system `active` flags.
// Reductions are two-pass: per-CTA partials in a fixed layout, then a fixed
// summation order, so results do not depend on scheduling.
//
// T = double runs the plain FP64 path; T = float runs the V-cycles and the
// inner Krylov iterations of the mixed path (FP32 inside FP64 refinement).
#include "snac_solver.h"
#include "snac_mgk.h"
#include "snac_prof.h"
#include "snac_mgdev.h"

namespace snac {


// ---------------------------------------------------------------- smoothing / transfer
template <typename T>
__global__ void k_rbgs(MgLevelD L, MgGeom G, const T *shift, const int *active, int color, T *x, const T *b) {
  const int s = blockIdx.y;
  if (active && !active[s]) return;
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= L.ncell) return;
  int i, j, k;
  decompose(L, c, i, j, k);
  if (((i + j + k) & 1) != color) return;
  if (L.code[c] & 0x8000) return;
  const long off = L.ncell * s;
  const T acc = b[off + c] - offdiag<T>(L, G, x, off, c, i, j, k);
  x[off + c] = acc / diag_of<T>(L, G, shift, c, i, j, s);
}

// coarse b <- sum over children of (b - A x) on the fine level; coarse x <- 0
template <typename T>
__global__ void k_resid_restrict(MgLevelD F, MgLevelD C, MgGeom G, const T *shift, const int *active, const T *xf,
                                 const T *bf, T *bc, T *xc) {
  const int s = blockIdx.y;
  if (active && !active[s]) return;
  const long cc = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (cc >= C.ncell) return;
  int I, J, K;
  decompose(C, cc, I, J, K);
  const long offf = F.ncell * s, offc = C.ncell * s;
  T sum = 0;
  const int e0 = C.coarsened[0] ? 2 : 1, e1 = C.coarsened[1] ? 2 : 1, e2 = C.coarsened[2] ? 2 : 1;
  for (int dk = 0; dk < e2; dk++)
    for (int dj = 0; dj < e1; dj++)
      for (int di = 0; di < e0; di++) {
        const int i = C.coarsened[0] ? 2 * I + di : I, j = C.coarsened[1] ? 2 * J + dj : J,
                  k = C.coarsened[2] ? 2 * K + dk : K;
        const long c = i + (long)F.n[0] * (j + (long)F.n[1] * k);
        if (F.code[c] & 0x8000) continue;
        const T ax = diag_of<T>(F, G, shift, c, i, j, s) * xf[offf + c] + offdiag<T>(F, G, xf, offf, c, i, j, k);
        sum += bf[offf + c] - ax;
      }
  bc[offc + cc] = sum;
  xc[offc + cc] = 0;
}

template <typename T>
__global__ void k_prolong(MgLevelD F, MgLevelD C, const int *active, T *xf, const T *xc) {
  const int s = blockIdx.y;
  if (active && !active[s]) return;
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= F.ncell) return;
  if (F.code[c] & 0x8000) return;
  int i, j, k;
  decompose(F, c, i, j, k);
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
  const T *M = LA<T>::dinv(L) + (size_t)n * n * s;
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    T acc = 0;
    for (int c = 0; c < n; c++) acc += M[(size_t)r * n + c] * sb[c];
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

static inline dim3 grid_for(long ncell, int nsys) { return dim3((unsigned)((ncell + 255) / 256), (unsigned)nsys); }

// V-cycle on level l: x_l <- M b_l (zero initial guess); x and b of each level are the level's own arrays
template <typename T>
int mg_vcycle_impl(const MgProblem &P, const MgGeom &G, int l, const T *shift, const int *active, cudaStream_t st) {
  const MgLevelD &L = P.L[l];
  T *x = LA<T>::x(L);
  T *b = LA<T>::b(L);
  const dim3 g = grid_for(L.ncell, P.nsys);
  trace("vcycle: enter level", st);
  if (P.fused && l >= P.cta_level[sizeof(T) == 8 ? 1 : 0]) return launch_vcycle_coarse<T>(P, G, l, shift, active, x, b, st);
  const bool tile = P.fused && !P.mode3d && L.n[0] >= 32 && L.n[1] >= 16 && 2 * P.nu <= 4;
  if (tile && l < P.nlev - 1) {
    const MgLevelD &C = P.L[l + 1];
    SNAC_TRY(launch_rbgs_tile2d<T>(P, l, shift, active, 0, 0, x, b, (const T *)nullptr, st));
    prof_begin(KID_RESTRICT, st);
    k_resid_restrict<T><<<grid_for(C.ncell, P.nsys), 256, 0, st>>>(L, C, G, shift, active, x, b, LA<T>::b(C),
                                                                   LA<T>::x(C));
    prof_end(KID_RESTRICT, st);
    SNAC_CUDA(cudaGetLastError());
    SNAC_TRY(mg_vcycle_impl<T>(P, G, l + 1, shift, active, st));
    return launch_rbgs_tile2d<T>(P, l, shift, active, 1, 1, x, b, (const T *)LA<T>::x(C), st);
  }
  if (l == P.nlev - 1) {
    if (LA<T>::dinv(L)) {
      k_dense<T><<<P.nsys, 256, 0, st>>>(L, active, x, b);
    } else {
      k_zero<T><<<g, 256, 0, st>>>(L.ncell, x, P.nsys, active);
      for (int it = 0; it < 40; it++)
        for (int col : {0, 1, 1, 0}) k_rbgs<T><<<g, 256, 0, st>>>(L, G, shift, active, col, x, b);
    }
    SNAC_CUDA(cudaGetLastError());
    return SNAC_OK;
  }
  if (l == 0) k_zero<T><<<g, 256, 0, st>>>(L.ncell, x, P.nsys, active);  // coarse x is zeroed by the restriction
  for (int it = 0; it < 2 * P.nu; it++) {
    prof_begin(KID_RBGS, st);
    k_rbgs<T><<<g, 256, 0, st>>>(L, G, shift, active, it & 1, x, b);
    prof_end(KID_RBGS, st);
  }
  const MgLevelD &C = P.L[l + 1];
  prof_begin(KID_RESTRICT, st);
  k_resid_restrict<T><<<grid_for(C.ncell, P.nsys), 256, 0, st>>>(L, C, G, shift, active, x, b, LA<T>::b(C), LA<T>::x(C));
  prof_end(KID_RESTRICT, st);
  SNAC_CUDA(cudaGetLastError());
  SNAC_TRY(mg_vcycle_impl<T>(P, G, l + 1, shift, active, st));
  k_prolong<T><<<g, 256, 0, st>>>(L, C, active, x, LA<T>::x(C));
  for (int it = 0; it < 2 * P.nu; it++) {
    prof_begin(KID_RBGS, st);
    k_rbgs<T><<<g, 256, 0, st>>>(L, G, shift, active, 1 - (it & 1), x, b);
    prof_end(KID_RBGS, st);
  }
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

// ---------------------------------------------------------------- Krylov vector kernels (level 0)
// per-CTA partial sums in double: part[s*nchunk + blockIdx.x]
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double sh[8];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int q = 0; q < (int)(blockDim.x >> 5); q++) s += sh[q];
  __syncthreads();
  return s;
}

// r = b - A x ; partials rr and bb
template <typename T>
__global__ void k_cg_resid(MgLevelD L, MgGeom G, const T *shift, const int *active, const T *x, const T *b, T *r,
                           double *part_rr, double *part_bb, int nchunk) {
  const int s = blockIdx.y;
  if (active && !active[s]) return;
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  double rr = 0.0, bb = 0.0;
  if (c < L.ncell && !(L.code[c] & 0x8000)) {
    int i, j, k;
    decompose(L, c, i, j, k);
    const long off = L.ncell * s;
    const T ax = diag_of<T>(L, G, shift, c, i, j, s) * x[off + c] + offdiag<T>(L, G, x, off, c, i, j, k);
    const T rv = b[off + c] - ax;
    r[off + c] = rv;
    rr = (double)rv * (double)rv;
    bb = (double)b[off + c] * (double)b[off + c];
  } else if (c < L.ncell) {
    r[L.ncell * s + c] = 0;
  }
  rr = block_sum(rr);
  bb = block_sum(bb);
  if (threadIdx.x == 0) { part_rr[(long)s * nchunk + blockIdx.x] = rr; part_bb[(long)s * nchunk + blockIdx.x] = bb; }
}

// partial dot a.b
template <typename T>
__global__ void k_cg_dot(long n, const int *active, const T *a, const T *b, double *part, int nchunk) {
  const int s = blockIdx.y;
  if (active && !active[s]) return;
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (c < n) v = (double)a[n * s + c] * (double)b[n * s + c];
  v = block_sum(v);
  if (threadIdx.x == 0) part[(long)s * nchunk + blockIdx.x] = v;
}

// Per-system sum of the chunk partials by one warp: lane-strided, then a shuffle tree (fixed order).
__device__ __forceinline__ double warp_sum_parts(const double *part, int s, int nchunk) {
  const int l = threadIdx.x & 31;
  double acc = 0.0;
  for (int q = l; q < nchunk; q += 32) acc += part[(long)s * nchunk + q];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  return __shfl_sync(0xffffffffu, acc, 0);
}

// rz_new = r.z; beta = rz_new/rz_old (0 on the first iteration); one warp per system
__global__ void k_cg_beta(int nsys, const int *active, SysScal *sc, const double *part_rz, int nchunk) {
  const int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (s >= nsys || (active && !active[s])) return;
  const double rz = warp_sum_parts(part_rz, s, nchunk);
  if ((threadIdx.x & 31) == 0) {
    sc[s].beta = sc[s].first ? 0.0 : rz / sc[s].rz;
    sc[s].rz = rz;
    sc[s].first = 0;
  }
}

// alpha = rz/pq; one warp per system
__global__ void k_cg_alpha(int nsys, const int *active, SysScal *sc, const double *part_pq, int nchunk) {
  const int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (s >= nsys || (active && !active[s])) return;
  const double pq = warp_sum_parts(part_pq, s, nchunk);
  if ((threadIdx.x & 31) == 0) sc[s].alpha = sc[s].rz / pq;
}

// p = z + beta p
template <typename T>
__global__ void k_cg_p(long n, const int *active, const SysScal *sc, const T *z, T *p) {
  const int s = blockIdx.y;
  if (active && !active[s]) return;
  const T beta = (T)sc[s].beta;
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) p[n * s + c] = z[n * s + c] + beta * p[n * s + c];
}

// q = A p ; partial p.q
template <typename T>
__global__ void k_cg_apply(MgLevelD L, MgGeom G, const T *shift, const int *active, const T *p, T *q, double *part,
                           int nchunk) {
  const int s = blockIdx.y;
  if (active && !active[s]) return;
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (c < L.ncell) {
    const long off = L.ncell * s;
    T y = 0;
    if (!(L.code[c] & 0x8000)) {
      int i, j, k;
      decompose(L, c, i, j, k);
      y = diag_of<T>(L, G, shift, c, i, j, s) * p[off + c] + offdiag<T>(L, G, p, off, c, i, j, k);
    }
    q[off + c] = y;
    v = (double)p[off + c] * (double)y;
  }
  v = block_sum(v);
  if (threadIdx.x == 0) part[(long)s * nchunk + blockIdx.x] = v;
}

// alpha = rz/pq; x += alpha p; r -= alpha q; partial r.r
template <typename T>
__global__ void k_cg_xr(long n, const int *active, const SysScal *sc, const T *p, const T *q, T *x, T *r,
                        double *part_rr) {
  const int s = blockIdx.y;
  if (active && !active[s]) return;
  const double alpha_s = sc[s].alpha;
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (c < n) {
    const long o = n * s + c;
    x[o] = x[o] + (T)alpha_s * p[o];
    const T rv = r[o] - (T)alpha_s * q[o];
    r[o] = rv;
    v = (double)rv * (double)rv;
  }
  v = block_sum(v);
  if (threadIdx.x == 0) part_rr[(long)s * gridDim.x + blockIdx.x] = v;
}

// finalize residual norms: rel = sqrt(rr/bb); update active flags; count still-active systems.
// One warp per system; `count` must be zero on entry (cleared by the caller).
__global__ void k_cg_norms(int nsys, int *active, SysScal *sc, const double *part_rr, const double *part_bb,
                           int nchunk, double tol, int set_bb, int *count) {
  const int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (s >= nsys || !active[s]) return;
  const double rr = warp_sum_parts(part_rr, s, nchunk);
  const double bbn = set_bb ? warp_sum_parts(part_bb, s, nchunk) : 0.0;
  if ((threadIdx.x & 31) != 0) return;
  if (set_bb) { sc[s].bb = bbn; sc[s].first = 1; sc[s].zero_rhs = 0; }
  sc[s].rr = rr;
  const double bb = sc[s].bb;
  const double rel = bb > 0.0 ? sqrt(rr / bb) : 0.0;
  sc[s].rel = rel;
  if (bb == 0.0) { sc[s].zero_rhs = 1; active[s] = 0; }
  else if (rel <= tol) active[s] = 0;
  else atomicAdd(count, 1);
}

// systems with an all-zero right-hand side get x = 0 (as HYPRE does)
template <typename T>
__global__ void k_zero_rhs_systems(long n, const SysScal *sc, T *x) {
  const int s = blockIdx.y;
  if (!sc[s].zero_rhs) return;
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) x[n * s + c] = 0;
}

// singular systems: b -= mean(b) over active cells (two passes)
template <typename T>
__global__ void k_sum_active(MgLevelD L, const int *singular, const T *b, double *part, double *partn, int nchunk) {
  const int s = blockIdx.y;
  if (!singular[s]) return;
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0, m = 0.0;
  if (c < L.ncell && !(L.code[c] & 0x8000)) { v = (double)b[L.ncell * s + c]; m = 1.0; }
  v = block_sum(v);
  m = block_sum(m);
  if (threadIdx.x == 0) { part[(long)s * nchunk + blockIdx.x] = v; partn[(long)s * nchunk + blockIdx.x] = m; }
}
template <typename T>
__global__ void k_sub_mean(MgLevelD L, const int *singular, T *b, const double *part, const double *partn, int nchunk) {
  const int s = blockIdx.y;
  if (!singular[s]) return;
  __shared__ double mean;
  if (threadIdx.x < 32) {
    const double na = warp_sum_parts(partn, s, nchunk);
    const double sm = warp_sum_parts(part, s, nchunk);
    if (threadIdx.x == 0) mean = na > 0.0 ? sm / na : 0.0;
  }
  __syncthreads();
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < L.ncell && !(L.code[c] & 0x8000)) b[L.ncell * s + c] -= (T)mean;
}

// mixed path: r32 = r64 / scale_s (scale = RMS of r over the system); e32 = 0
__global__ void k_ir_down(long n, const int *active, SysScal *sc, const double *r, float *r32, float *e32) {
  const int s = blockIdx.y;
  if (active && !active[s]) return;
  const double inv = 1.0 / sc[s].scale;
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) { r32[n * s + c] = (float)(r[n * s + c] * inv); e32[n * s + c] = 0.0f; }
}
__global__ void k_ir_scale(int nsys, const int *active, SysScal *sc, long ncell_active) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys || (active && !active[s])) return;
  double sc2 = sqrt(sc[s].rr / (double)(ncell_active > 0 ? ncell_active : 1));
  sc[s].scale = sc2 > 0.0 ? sc2 : 1.0;
}
__global__ void k_ir_up(long n, const int *active, const SysScal *sc, const float *e32, double *x) {
  const int s = blockIdx.y;
  if (active && !active[s]) return;
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) x[n * s + c] += sc[s].scale * (double)e32[n * s + c];
}

// Explicit instantiation of every kernel template for both precisions, so that the
// device code of each kernel exists whatever host template reaches its launch.
#define SNAC_MG_KERNELS(T)                                                                                          \
  template __global__ void k_rbgs<T>(MgLevelD, MgGeom, const T *, const int *, int, T *, const T *);                \
  template __global__ void k_resid_restrict<T>(MgLevelD, MgLevelD, MgGeom, const T *, const int *, const T *,       \
                                               const T *, T *, T *);                                                \
  template __global__ void k_prolong<T>(MgLevelD, MgLevelD, const int *, T *, const T *);                           \
  template __global__ void k_dense<T>(MgLevelD, const int *, T *, const T *);                                       \
  template __global__ void k_zero<T>(long, T *, int, const int *);                                                  \
  template __global__ void k_cg_resid<T>(MgLevelD, MgGeom, const T *, const int *, const T *, const T *, T *,       \
                                         double *, double *, int);                                                  \
  template __global__ void k_cg_dot<T>(long, const int *, const T *, const T *, double *, int);                     \
  template __global__ void k_cg_p<T>(long, const int *, const SysScal *, const T *, T *);                           \
  template __global__ void k_cg_apply<T>(MgLevelD, MgGeom, const T *, const int *, const T *, T *, double *, int);  \
  template __global__ void k_cg_xr<T>(long, const int *, const SysScal *, const T *, const T *, T *, T *, double *); \
  template __global__ void k_zero_rhs_systems<T>(long, const SysScal *, T *);                                      \
  template __global__ void k_sum_active<T>(MgLevelD, const int *, const T *, double *, double *, int);              \
  template __global__ void k_sub_mean<T>(MgLevelD, const int *, T *, const double *, const double *, int);
SNAC_MG_KERNELS(double)
SNAC_MG_KERNELS(float)
#undef SNAC_MG_KERNELS

// ---------------------------------------------------------------- host drivers
template <typename T>
int mg_vcycle(const MgProblem &P, int l, const int *active, cudaStream_t st) {
  MgGeom G;
  G.mode3d = P.mode3d;
  for (int a = 0; a < 3; a++) G.periodic[a] = P.periodic[a];
  const T *shift = nullptr;
  if constexpr (sizeof(T) == 8) shift = (const T *)P.shift; else shift = (const T *)P.shiftf;
  return mg_vcycle_impl<T>(P, G, l, shift, active, st);
}
template int mg_vcycle<double>(const MgProblem &, int, const int *, cudaStream_t);
template int mg_vcycle<float>(const MgProblem &, int, const int *, cudaStream_t);

// preconditioned CG on level 0 of P for all active systems (T-typed vectors); returns iterations done
template <typename T>
int mg_pcg(const MgProblem &P, CgWork &W, T *x, T *b, int maxiter, double tol, bool check_host, int *iters,
           cudaStream_t st) {
  MgGeom G;
  G.mode3d = P.mode3d;
  for (int a = 0; a < 3; a++) G.periodic[a] = P.periodic[a];
  const T *shift;
  if constexpr (sizeof(T) == 8) shift = (const T *)P.shift; else shift = (const T *)P.shiftf;
  MgLevelD L0 = P.L[0];
  const long n = L0.ncell;
  const int nchunk = (int)((n + 255) / 256);
  const dim3 g(nchunk, P.nsys);
  T *r = (T *)W.r, *z = (T *)W.z, *p = (T *)W.p, *q = (T *)W.q;
  const unsigned gsys = (unsigned)((P.nsys + 7) / 8);  // one warp per system, 8 per CTA
  k_cg_resid<T><<<g, 256, 0, st>>>(L0, G, shift, W.active, x, b, r, W.part0, W.part1, nchunk);
  SNAC_CUDA(cudaMemsetAsync(W.d_count, 0, sizeof(int), st));
  k_cg_norms<<<gsys, 256, 0, st>>>(P.nsys, W.active, W.sc, W.part0, W.part1, nchunk, tol, 1, W.d_count);
  SNAC_CUDA(cudaGetLastError());
  k_zero_rhs_systems<T><<<g, 256, 0, st>>>(n, W.sc, x);
  trace(sizeof(T) == 8 ? "pcg64: initial residual" : "pcg32: initial residual", st);
  int it = 0;
  for (it = 1; it <= maxiter; it++) {
    if (check_host) {
      SNAC_CUDA(cudaMemcpyAsync(W.h_count, W.d_count, sizeof(int), cudaMemcpyDeviceToHost, st));
      SNAC_CUDA(cudaStreamSynchronize(st));
      if (*W.h_count == 0) { it--; break; }
    }
    // z = M r : V-cycle with level-0 b = r, x = z
    MgProblem Pz = P;
    if constexpr (sizeof(T) == 8) { Pz.L[0].b = (double *)r; Pz.L[0].x = (double *)z; }
    else { Pz.L[0].bf = (float *)r; Pz.L[0].xf = (float *)z; }
    SNAC_TRY(mg_vcycle_impl<T>(Pz, G, 0, shift, W.active, st));
    trace("pcg: V-cycle", st);
    k_cg_dot<T><<<g, 256, 0, st>>>(n, W.active, r, z, W.part0, nchunk);
    k_cg_beta<<<gsys, 256, 0, st>>>(P.nsys, W.active, W.sc, W.part0, nchunk);
    k_cg_p<T><<<g, 256, 0, st>>>(n, W.active, W.sc, z, p);
    prof_begin(KID_CG_APPLY, st);
    k_cg_apply<T><<<g, 256, 0, st>>>(L0, G, shift, W.active, p, q, W.part1, nchunk);
    prof_end(KID_CG_APPLY, st);
    k_cg_alpha<<<gsys, 256, 0, st>>>(P.nsys, W.active, W.sc, W.part1, nchunk);
    k_cg_xr<T><<<g, 256, 0, st>>>(n, W.active, W.sc, p, q, x, r, W.part0);
    SNAC_CUDA(cudaMemsetAsync(W.d_count, 0, sizeof(int), st));
    k_cg_norms<<<gsys, 256, 0, st>>>(P.nsys, W.active, W.sc, W.part0, nullptr, nchunk, tol, 0, W.d_count);
    SNAC_CUDA(cudaGetLastError());
    trace("pcg: iteration", st);
  }
  if (it > maxiter) it = maxiter;
  *iters = it;
  return SNAC_OK;
}
template int mg_pcg<double>(const MgProblem &, CgWork &, double *, double *, int, double, bool, int *, cudaStream_t);
template int mg_pcg<float>(const MgProblem &, CgWork &, float *, float *, int, double, bool, int *, cudaStream_t);

// active[s] = src ? src[s] : 1
__global__ void k_set_active(int nsys, int *active, const int *src) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nsys) active[s] = src ? src[s] : 1;
}
int mg_set_active(int nsys, int *active, const int *src, cudaStream_t st) {
  k_set_active<<<(nsys + 127) / 128, 128, 0, st>>>(nsys, active, src);
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

int mg_project_singular(const MgProblem &P, CgWork &W, double *b, cudaStream_t st) {
  const long n = P.L[0].ncell;
  const int nchunk = (int)((n + 255) / 256);
  const dim3 g(nchunk, P.nsys);
  k_sum_active<double><<<g, 256, 0, st>>>(P.L[0], P.singular, b, W.part0, W.part1, nchunk);
  k_sub_mean<double><<<g, 256, 0, st>>>(P.L[0], P.singular, b, W.part0, W.part1, nchunk);
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

int mg_ir_down(const MgProblem &P, CgWork &W, const double *r64, float *r32, float *e32, long nact, cudaStream_t st) {
  const long n = P.L[0].ncell;
  const dim3 g((unsigned)((n + 255) / 256), P.nsys);
  k_ir_scale<<<(P.nsys + 127) / 128, 128, 0, st>>>(P.nsys, W.active, W.sc, nact);
  k_ir_down<<<g, 256, 0, st>>>(n, W.active, W.sc, r64, r32, e32);
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}
int mg_ir_up(const MgProblem &P, CgWork &W, const float *e32, double *x, cudaStream_t st) {
  const long n = P.L[0].ncell;
  const dim3 g((unsigned)((n + 255) / 256), P.nsys);
  k_ir_up<<<g, 256, 0, st>>>(n, W.active, W.sc, e32, x);
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

}  // namespace snac
