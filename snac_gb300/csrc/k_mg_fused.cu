// k_mg_fused.cu -- fused multigrid kernels for the plane (2-D) systems.
//
// k_rbgs_tile2d: all 2*nu red-black half-sweeps of one plane level in one launch.
//   A CTA of 8 warps owns a 64 x 8R tile (a halo of TH = 4 cells on every side
//   around its 56 x (8R - 8) output cells).  Lane l of warp w owns the column
//   pair (2l, 2l+1) of rows w, w+8, ..., so in every half-sweep each thread
//   updates exactly one cell per row and no lane idles.  The tile lives in
//   shared memory split into even and odd columns (conflict-free neighbour
//   reads); b, 1/d and the four couplings of the owned cells stay in registers
//   for all sweeps.  After t half-sweeps only cells within t of the tile edge
//   can differ from a global sweep, so the output cells are exact after TH.
//   The pre-smoother starts from x = 0 without reading x; the post-smoother adds
//   the coarse-grid correction while loading (prolongation fused) and can emit
//   the partials of b.x (r.z of the Krylov iteration).
// k_vcycle_coarse: one CTA of 1024 threads per system runs the V-cycle from
//   level l0 down to the coarsest solve and back, with x, b, the diagonal and
//   the couplings of every level in shared memory.
// Both follow the arithmetic of k_rbgs / k_resid_restrict / k_prolong / k_dense
// term by term, so fused and unfused V-cycles give identical results.
#include <algorithm>
#include <mutex>

#include "snac_solver.h"
#include "snac_mgk.h"
#include "snac_mgdev.h"
#include "snac_prof.h"

namespace snac {

namespace {
constexpr int TH = 4;              // tile halo = most half-sweeps per launch (2 nu with nu <= 2)
constexpr int TSW = 64;            // tile width
constexpr int TBX = TSW - 2 * TH;  // output columns per tile
inline int tile_by(int R) { return 8 * R - 2 * TH; }
inline int tiles_for(const MgLevelD &L, int R) {
  return ((L.n[0] + TBX - 1) / TBX) * ((L.n[1] + tile_by(R) - 1) / tile_by(R));
}
// rows per warp: the choice that processes the fewest tile rows (ties: the smaller tile)
int choose_rows(const MgLevelD &L, int prec) {
  static const int rf[] = {2, 3, 4, 6}, rd[] = {2, 3};
  const int *opts = prec ? rd : rf;
  const int nopt = prec ? 2 : 4;
  int best = opts[0];
  long bestc = -1;
  for (int q = 0; q < nopt; q++) {
    const int R = opts[q];
    const long cost = (long)((L.n[1] + tile_by(R) - 1) / tile_by(R)) * 8 * R;
    if (bestc < 0 || cost < bestc) { bestc = cost; best = R; }
  }
  return best;
}
__device__ __forceinline__ int wrap(int g, int n) {
  if (g >= 0 && g < n) return g;
  g %= n;
  return g < 0 ? g + n : g;
}
}  // namespace

int tile2d_max_tiles(const MgLevelD &L) { return tiles_for(L, 2); }

bool tile2d_ok(const MgProblem &P, int l, int prec) {
  (void)prec;
  if (P.mode3d || l >= P.nlev - 1 || 2 * P.nu > TH) return false;
  const MgLevelD &L = P.L[l];
  for (int a = 0; a < 2; a++)
    if (P.periodic[a] && L.n[a] > 1 && (L.n[a] & 1)) return false;  // red-black colouring must wrap consistently
  return true;
}

template <typename T, int R>
__global__ void __launch_bounds__(256) k_rbgs_tile2d(MgLevelD L, MgLevelD C, int per0, int per1,
                                                     const T *__restrict__ shift, const int *__restrict__ active,
                                                     int first_color, int nhalf, int mode, T *__restrict__ x,
                                                     const T *__restrict__ b, const T *__restrict__ xc,
                                                     double *__restrict__ part_bx, int part_stride) {
  constexpr int SH = 8 * R, BY = SH - 2 * TH;
  __shared__ T xe[SH][32], xo[SH][32];
  const int s = blockIdx.y;
  if (active && !active[s]) return;
  const int n0 = L.n[0], n1 = L.n[1];
  const int ntx = (n0 + TBX - 1) / TBX;
  const int i0 = (int)(blockIdx.x % ntx) * TBX - TH, j0 = (int)(blockIdx.x / ntx) * BY - TH;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long off = L.ncell * s;
  const T sh = shift[s];
  const bool skip0 = per0 && n0 == 1, skip1 = per1 && n1 == 1;
  const T *__restrict__ cc = LA<T>::cc(L);
  const T *__restrict__ w01 = LA<T>::w01(L);
  const T *__restrict__ cp0 = LA<T>::cp(L, 0);
  const T *__restrict__ cp1 = LA<T>::cp(L, 1);
  T bv[R][2], iv[R][2], ce[R][2], cw[R][2], cn[R][2], cs[R][2];
#pragma unroll
  for (int q = 0; q < R; q++) {
    const int r = w + 8 * q;
#pragma unroll
    for (int p = 0; p < 2; p++) {
      int gi = i0 + 2 * lane + p, gj = j0 + r;
      bool in = true;
      if (gi < 0 || gi >= n0) { if (per0) gi = wrap(gi, n0); else in = false; }
      if (gj < 0 || gj >= n1) { if (per1) gj = wrap(gj, n1); else in = false; }
      T b_ = 0, i_ = 0, e_ = 0, w_ = 0, n_ = 0, s_ = 0, x_ = 0;
      if (in) {
        const int c = gi + n0 * gj;
        if (!(L.code[c] & 0x8000)) {
          i_ = T(1) / fmat(sh, w01[c], cc[c]);
          b_ = b[off + c];
          if (!skip0) {
            e_ = cp0[c];
            w_ = gi > 0 ? cp0[c - 1] : (per0 ? cp0[c + n0 - 1] : T(0));
          }
          if (!skip1) {
            n_ = cp1[c];
            s_ = gj > 0 ? cp1[c - n0] : (per1 ? cp1[c + n0 * (n1 - 1)] : T(0));
          }
          if (mode == 1) {
            const int I = C.coarsened[0] ? gi / 2 : gi, J = C.coarsened[1] ? gj / 2 : gj;
            x_ = x[off + c] + xc[C.ncell * s + I + C.n[0] * J];
          }
        }
      }
      bv[q][p] = b_;
      iv[q][p] = i_;
      ce[q][p] = e_;
      cw[q][p] = w_;
      cn[q][p] = n_;
      cs[q][p] = s_;
      if (p) xo[r][lane] = x_;
      else xe[r][lane] = x_;
    }
  }
  for (int t = 0; t < nhalf; t++) {
    __syncthreads();
    const int color = (first_color + t) & 1;
#pragma unroll
    for (int q = 0; q < R; q++) {
      const int r = w + 8 * q;
      if (r == 0 || r == SH - 1) continue;
      if (((color + i0 + j0 + r) & 1) == 0) {  // even column 2*lane: E = odd(lane), W = odd(lane-1)
        const T xE = xo[r][lane];
        const T xW = lane > 0 ? xo[r][lane - 1] : T(0);
        T acc = fmat(ce[q][0], xE, T(0));
        acc = fmat(cw[q][0], xW, acc);
        acc = fmat(cn[q][0], xe[r + 1][lane], acc);
        acc = fmat(cs[q][0], xe[r - 1][lane], acc);
        if (lane > 0) xe[r][lane] = (bv[q][0] - acc) * iv[q][0];
      } else {                                  // odd column 2*lane+1: E = even(lane+1), W = even(lane)
        const T xE = lane < 31 ? xe[r][lane + 1] : T(0);
        const T xW = xe[r][lane];
        T acc = fmat(ce[q][1], xE, T(0));
        acc = fmat(cw[q][1], xW, acc);
        acc = fmat(cn[q][1], xo[r + 1][lane], acc);
        acc = fmat(cs[q][1], xo[r - 1][lane], acc);
        if (lane < 31) xo[r][lane] = (bv[q][1] - acc) * iv[q][1];
      }
    }
  }
  // every thread stores only cells it updated itself: no barrier needed
  T bx = 0;
#pragma unroll
  for (int q = 0; q < R; q++) {
    const int r = w + 8 * q;
#pragma unroll
    for (int p = 0; p < 2; p++) {
      const int col = 2 * lane + p;
      if (r < TH || r >= TH + BY || col < TH || col >= TH + TBX) continue;
      const int gi = i0 + col, gj = j0 + r;
      if (gi >= n0 || gj >= n1 || iv[q][p] == T(0)) continue;
      const T v = p ? xo[r][lane] : xe[r][lane];
      x[off + gi + n0 * gj] = v;
      bx = fmat(bv[q][p], v, bx);
    }
  }
  if (part_bx) {
    const double t = block_sum1<T>(bx);
    if (threadIdx.x == 0) part_bx[(long)s * part_stride + blockIdx.x] = t;
  }
}

// ---------------------------------------------------------------- whole coarse V-cycle in one CTA
// one half-sweep of a level held in shared memory (inactive cells have d = 0)
template <typename T>
__device__ __forceinline__ void cta_sweep_xy(int n0, int n1, int per0, int per1, T *x, const T *b, const T *d,
                                             const T *c0, const T *c1, int color) {
  const int h0 = (n0 + 1) >> 1, half = h0 * n1;
  for (int q = threadIdx.x; q < half; q += blockDim.x) {
    const int j = q / h0, i = 2 * (q - j * h0) + ((color + j) & 1);
    if (i >= n0) continue;
    const int c = i + n0 * j;
    const T dv = d[c];
    if (dv == T(0)) continue;
    const T acc = offdiag_xy<T>(n0, n1, per0, per1, c0, c1, [&](int e) { return x[e]; }, c, i, j);
    x[c] = (b[c] - acc) * (T(1) / dv);
  }
  __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(1024, 1) k_vcycle_coarse(MgProblem P, int l0, const T *__restrict__ shift,
                                                           const int *__restrict__ active, T *__restrict__ xout,
                                                           const T *__restrict__ bin) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int s = blockIdx.x;
  if (active && !active[s]) return;
  const int last = P.nlev - 1;
  const bool dense = LA<T>::dinv(P.L[last]) != nullptr;
  const int per0 = P.periodic[0], per1 = P.periodic[1];
  // level l occupies [x | b | d | c0 | c1] (the dense coarsest level only [x | b]) from offset lo[l]
  __shared__ int lo[MG_MAXLEV];
  if (threadIdx.x == 0) {
    int o = 0;
    for (int l = l0; l < P.nlev; l++) {
      lo[l] = o;
      o += ((l == last && dense) ? 2 : 5) * (int)P.L[l].ncell;
    }
  }
  __syncthreads();
  T *const base = (T *)smem_raw;
  auto X = [&](int l) { return base + lo[l]; };
  auto B = [&](int l) { return base + lo[l] + (int)P.L[l].ncell; };
  auto D = [&](int l) { return base + lo[l] + 2 * (int)P.L[l].ncell; };
  auto C0 = [&](int l) { return base + lo[l] + 3 * (int)P.L[l].ncell; };
  auto C1 = [&](int l) { return base + lo[l] + 4 * (int)P.L[l].ncell; };
  const T sh = shift[s];
  for (int l = l0; l < P.nlev; l++) {
    if (l == last && dense) break;
    const MgLevelD &L = P.L[l];
    const int n = (int)L.ncell;
    const T *__restrict__ cc = LA<T>::cc(L);
    const T *__restrict__ w01 = LA<T>::w01(L);
    const T *__restrict__ cp0 = LA<T>::cp(L, 0);
    const T *__restrict__ cp1 = LA<T>::cp(L, 1);
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
      D(l)[c] = (L.code[c] & 0x8000) ? T(0) : fmat(sh, w01[c], cc[c]);
      C0(l)[c] = cp0[c];
      C1(l)[c] = cp1[c];
    }
  }
  {
    const int n = (int)P.L[l0].ncell;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
      B(l0)[c] = bin[(long)n * s + c];
      X(l0)[c] = 0;
    }
  }
  __syncthreads();
  // down: pre-smoothing and restriction of the residual
  for (int l = l0; l < last; l++) {
    const MgLevelD &L = P.L[l];
    const MgLevelD &C = P.L[l + 1];
    const int n0 = L.n[0], n1 = L.n[1];
    T *x = X(l);
    const T *b = B(l), *d = D(l), *c0 = C0(l), *c1 = C1(l);
    for (int it = 0; it < 2 * P.nu; it++) cta_sweep_xy<T>(n0, n1, per0, per1, x, b, d, c0, c1, it & 1);
    const int cn0 = C.n[0], nc = (int)C.ncell;
    const int e0 = C.coarsened[0] ? 2 : 1, e1 = C.coarsened[1] ? 2 : 1;
    for (int q = threadIdx.x; q < nc; q += blockDim.x) {
      const int J = q / cn0, I = q - J * cn0;
      T sum = 0;
      for (int dj = 0; dj < e1; dj++)
        for (int di = 0; di < e0; di++) {
          const int i = C.coarsened[0] ? 2 * I + di : I, j = C.coarsened[1] ? 2 * J + dj : J;
          const int c = i + n0 * j;
          const T dv = d[c];
          if (dv == T(0)) continue;
          const T acc = offdiag_xy<T>(n0, n1, per0, per1, c0, c1, [&](int e) { return x[e]; }, c, i, j);
          sum += b[c] - fmat(dv, x[c], acc);
        }
      B(l + 1)[q] = sum;
      X(l + 1)[q] = 0;
    }
    __syncthreads();
  }
  // coarsest level
  {
    const MgLevelD &L = P.L[last];
    const int n = (int)L.ncell;
    if (dense) {
      const T *__restrict__ M = LA<T>::dinv(L) + (size_t)n * n * s;
      for (int r = threadIdx.x; r < n; r += blockDim.x) {
        T acc = 0;
        for (int c = 0; c < n; c++) acc = fmat(M[(size_t)r * n + c], B(last)[c], acc);
        X(last)[r] = acc;
      }
      __syncthreads();
    } else {
      for (int it = 0; it < 40; it++)
        for (int col = 0; col < 4; col++)
          cta_sweep_xy<T>(L.n[0], L.n[1], per0, per1, X(last), B(last), D(last), C0(last), C1(last),
                          (col == 1 || col == 2) ? 1 : 0);
    }
  }
  // up: prolongation and post-smoothing
  for (int l = last - 1; l >= l0; l--) {
    const MgLevelD &L = P.L[l];
    const MgLevelD &C = P.L[l + 1];
    const int n0 = L.n[0], n1 = L.n[1], n = (int)L.ncell, cn0 = C.n[0];
    T *x = X(l);
    const T *xc = X(l + 1), *d = D(l);
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
      if (d[c] == T(0)) continue;
      const int j = c / n0, i = c - j * n0;
      const int I = C.coarsened[0] ? i / 2 : i, J = C.coarsened[1] ? j / 2 : j;
      x[c] += xc[I + cn0 * J];
    }
    __syncthreads();
    for (int it = 0; it < 2 * P.nu; it++)
      cta_sweep_xy<T>(n0, n1, per0, per1, x, B(l), d, C0(l), C1(l), 1 - (it & 1));
  }
  const int n = (int)P.L[l0].ncell;
  for (int c = threadIdx.x; c < n; c += blockDim.x) xout[(long)n * s + c] = X(l0)[c];
}

// ---------------------------------------------------------------- launchers
template <typename T>
int launch_rbgs_tile2d(const MgProblem &P, int l, const T *shift, const int *active, int first_color, int mode,
                       T *x, const T *b, const T *xc, double *part_bx, int part_stride, int *nchunk, cudaStream_t st) {
  const MgLevelD &L = P.L[l];
  const MgLevelD &C = l + 1 < P.nlev ? P.L[l + 1] : P.L[l];
  const int R = choose_rows(L, sizeof(T) == 8 ? 1 : 0);
  const int nt = tiles_for(L, R);
  if (part_bx && nt > part_stride) { set_error("partial-sum area too small for the tiled smoother"); return SNAC_ERR_ARG; }
  const dim3 g((unsigned)nt, (unsigned)P.nsys);
  const int nh = 2 * P.nu;
  prof_begin(KID_RBGS, st);
#define SNAC_TILE_LAUNCH(RR)                                                                                        \
  k_rbgs_tile2d<T, RR><<<g, 256, 0, st>>>(L, C, P.periodic[0], P.periodic[1], shift, active, first_color, nh, mode, \
                                          x, b, xc, part_bx, part_stride)
  if constexpr (sizeof(T) == 8) {
    if (R == 2) SNAC_TILE_LAUNCH(2);
    else SNAC_TILE_LAUNCH(3);
  } else {
    if (R == 2) SNAC_TILE_LAUNCH(2);
    else if (R == 3) SNAC_TILE_LAUNCH(3);
    else if (R == 4) SNAC_TILE_LAUNCH(4);
    else SNAC_TILE_LAUNCH(6);
  }
#undef SNAC_TILE_LAUNCH
  prof_end(KID_RBGS, st);
  SNAC_CUDA(cudaGetLastError());
  if (nchunk) *nchunk = part_bx ? nt : 0;
  return SNAC_OK;
}

template <typename T>
size_t coarse_smem_bytes(const MgProblem &P, int l0) {
  const int last = P.nlev - 1;
  const bool dense = LA<T>::dinv(P.L[last]) != nullptr;
  size_t n = 0;
  for (int l = l0; l < P.nlev; l++) n += (size_t)((l == last && dense) ? 2 : 5) * (size_t)P.L[l].ncell;
  return n * sizeof(T);
}

template <typename T>
int launch_vcycle_coarse(const MgProblem &P, int l0, const T *shift, const int *active, T *x, const T *b,
                         cudaStream_t st) {
  const size_t smem = coarse_smem_bytes<T>(P, l0);
  if (smem > MG_COARSE_SMEM_MAX) { set_error("coarse levels exceed the shared-memory budget"); return SNAC_ERR_ARG; }
  if (smem > 48 * 1024) {
    // the opt-in limit is a per-device function attribute: set it once for every device used
    static std::mutex mu;
    static unsigned long long done = 0;
    int dev = 0;
    SNAC_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    if (dev >= 64 || !(done >> dev & 1ull)) {
      SNAC_CUDA(cudaFuncSetAttribute((const void *)k_vcycle_coarse<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)MG_COARSE_SMEM_MAX));
      if (dev < 64) done |= 1ull << dev;
    }
  }
  prof_begin(KID_COARSE, st);
  k_vcycle_coarse<T><<<P.nsys, 1024, smem, st>>>(P, l0, shift, active, x, b);
  prof_end(KID_COARSE, st);
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

template int launch_rbgs_tile2d<double>(const MgProblem &, int, const double *, const int *, int, int, double *,
                                        const double *, const double *, double *, int, int *, cudaStream_t);
template int launch_rbgs_tile2d<float>(const MgProblem &, int, const float *, const int *, int, int, float *,
                                       const float *, const float *, double *, int, int *, cudaStream_t);
template size_t coarse_smem_bytes<double>(const MgProblem &, int);
template size_t coarse_smem_bytes<float>(const MgProblem &, int);
template int launch_vcycle_coarse<double>(const MgProblem &, int, const double *, const int *, double *,
                                          const double *, cudaStream_t);
template int launch_vcycle_coarse<float>(const MgProblem &, int, const float *, const int *, float *, const float *,
                                         cudaStream_t);

}  // namespace snac
