// k_mg_fused.cu -- fused multigrid kernels (fewer launches, fewer passes over HBM).
//
// k_rbgs_tile2d: all 2*nu red-black half-sweeps of one plane level in one launch.
//   Each CTA stages a (BX+2H) x (BY+2H) tile of x, b and the operator in shared
//   memory (H = number of half-sweeps); after t half-sweeps only cells within t
//   of the tile edge are stale, so the BX x BY interior is exact after H.  The
//   arithmetic per cell is that of k_rbgs, so results equal the unfused sweeps.
//   The pre-smoother starts from x = 0 without reading x; the post-smoother adds
//   the coarse-grid correction while loading (prolongation fused).
// k_vcycle_coarse: one CTA per system runs the V-cycle from level l0 down to the
//   dense coarsest solve and back, with every level's x and b in shared memory.
#include "snac_solver.h"
#include "snac_mgk.h"
#include "snac_mgdev.h"
#include "snac_prof.h"

namespace snac {

template <typename T, int BX, int BY, int H>
__global__ void __launch_bounds__(256)
k_rbgs_tile2d(MgLevelD L, MgLevelD C, int per0, int per1, const T *__restrict__ shift, const int *__restrict__ active,
              int first_color, int nhalf, int mode, T *__restrict__ x, const T *__restrict__ b,
              const T *__restrict__ xc) {
  constexpr int SW = BX + 2 * H, SH = BY + 2 * H, SN = SW * SH;
  __shared__ T xs[SN], bs[SN], cxs[SN], cys[SN], ds[SN];
  const int s = blockIdx.y;
  if (active && !active[s]) return;
  const int n0 = L.n[0], n1 = L.n[1];
  const int ntx = (n0 + BX - 1) / BX;
  const int ti = blockIdx.x % ntx, tj = blockIdx.x / ntx;
  const int i0 = ti * BX - H, j0 = tj * BY - H;
  const long off = L.ncell * s;
  const T sh = shift[s];
  const bool skip0 = per0 && n0 == 1, skip1 = per1 && n1 == 1;
  const T *__restrict__ cc = LA<T>::cc(L);
  const T *__restrict__ cp0 = LA<T>::cp(L, 0);
  const T *__restrict__ cp1 = LA<T>::cp(L, 1);
  const T *__restrict__ W0 = LA<T>::W(L, 0);
  const T *__restrict__ W1 = LA<T>::W(L, 1);
  for (int q = threadIdx.x; q < SN; q += blockDim.x) {
    const int li = q % SW, lj = q / SW;
    int gi = i0 + li, gj = j0 + lj;
    bool in = true;
    if (gi < 0 || gi >= n0) {
      if (per0) gi = ((gi % n0) + n0) % n0;
      else in = false;
    }
    if (gj < 0 || gj >= n1) {
      if (per1) gj = ((gj % n1) + n1) % n1;
      else in = false;
    }
    T xv = 0, bv = 0, cx = 0, cy = 0, dv = 0;
    if (in) {
      const long c = gi + (long)n0 * gj;
      if (!(L.code[c] & 0x8000)) {
        bv = b[off + c];
        cx = skip0 ? (T)0 : cp0[c];
        cy = skip1 ? (T)0 : cp1[c];
        dv = cc[c] + sh * W0[gi] * W1[gj];
        if (mode == 1) {
          const int I = C.coarsened[0] ? gi / 2 : gi, J = C.coarsened[1] ? gj / 2 : gj;
          xv = x[off + c] + xc[C.ncell * s + I + (long)C.n[0] * J];
        }
      }
    }
    xs[q] = xv;
    bs[q] = bv;
    cxs[q] = cx;
    cys[q] = cy;
    ds[q] = dv;
  }
  for (int t = 0; t < nhalf; t++) {
    __syncthreads();
    const int color = (first_color + t) & 1;
    for (int q = threadIdx.x; q < SN; q += blockDim.x) {
      const int li = q % SW, lj = q / SW;
      if (li == 0 || li == SW - 1 || lj == 0 || lj == SH - 1) continue;
      if ((((i0 + li) + (j0 + lj)) & 1) != color) continue;
      const T d = ds[q];
      if (d == (T)0) continue;
      T acc = 0;
      if (!skip0) {
        acc += cxs[q] * xs[q + 1];
        acc += cxs[q - 1] * xs[q - 1];
      }
      if (!skip1) {
        acc += cys[q] * xs[q + SW];
        acc += cys[q - SW] * xs[q - SW];
      }
      xs[q] = (bs[q] - acc) / d;
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < BX * BY; q += blockDim.x) {
    const int li = H + q % BX, lj = H + q / BX;
    const int gi = i0 + li, gj = j0 + lj;
    if (gi >= n0 || gj >= n1) continue;
    const int sq = li + SW * lj;
    if (ds[sq] == (T)0) continue;
    x[off + gi + (long)n0 * gj] = xs[sq];
  }
}

// ---------------------------------------------------------------- whole coarse V-cycle in one CTA
template <typename T>
__device__ void cta_sweep(const MgLevelD &L, const MgGeom &G, T sh, int s, T *xs, const T *bs, int color) {
  for (long c = threadIdx.x; c < L.ncell; c += blockDim.x) {
    int i, j, k;
    decompose(L, c, i, j, k);
    if (((i + j + k) & 1) != color) continue;
    if (L.code[c] & 0x8000) continue;
    const T acc = bs[c] - offdiag<T>(L, G, xs, 0, c, i, j, k);
    const T d = G.mode3d ? LA<T>::cc(L)[c] : LA<T>::cc(L)[c] + sh * LA<T>::W(L, 0)[i] * LA<T>::W(L, 1)[j];
    xs[c] = acc / d;
  }
  __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(256)
k_vcycle_coarse(MgProblem P, MgGeom G, int l0, const T *__restrict__ shift, const int *__restrict__ active,
                T *__restrict__ xout, const T *__restrict__ bin) {
  extern __shared__ unsigned char smem_raw[];
  const int s = blockIdx.x;
  if (active && !active[s]) return;
  T *xs[MG_MAXLEV], *bs[MG_MAXLEV];
  {
    T *p = (T *)smem_raw;
    for (int l = l0; l < P.nlev; l++) {
      xs[l] = p;
      p += P.L[l].ncell;
      bs[l] = p;
      p += P.L[l].ncell;
    }
  }
  const T sh = shift[s];
  const MgLevelD &L0 = P.L[l0];
  for (long c = threadIdx.x; c < L0.ncell; c += blockDim.x) {
    bs[l0][c] = bin[L0.ncell * s + c];
    xs[l0][c] = 0;
  }
  __syncthreads();
  // down
  for (int l = l0; l < P.nlev - 1; l++) {
    const MgLevelD &L = P.L[l];
    for (int it = 0; it < 2 * P.nu; it++) cta_sweep<T>(L, G, sh, s, xs[l], bs[l], it & 1);
    const MgLevelD &C = P.L[l + 1];
    for (long cc = threadIdx.x; cc < C.ncell; cc += blockDim.x) {
      int I, J, K;
      decompose(C, cc, I, J, K);
      T sum = 0;
      const int e0 = C.coarsened[0] ? 2 : 1, e1 = C.coarsened[1] ? 2 : 1, e2 = C.coarsened[2] ? 2 : 1;
      for (int dk = 0; dk < e2; dk++)
        for (int dj = 0; dj < e1; dj++)
          for (int di = 0; di < e0; di++) {
            const int i = C.coarsened[0] ? 2 * I + di : I, j = C.coarsened[1] ? 2 * J + dj : J,
                      k = C.coarsened[2] ? 2 * K + dk : K;
            const long c = i + (long)L.n[0] * (j + (long)L.n[1] * k);
            if (L.code[c] & 0x8000) continue;
            const T d = G.mode3d ? LA<T>::cc(L)[c] : LA<T>::cc(L)[c] + sh * LA<T>::W(L, 0)[i] * LA<T>::W(L, 1)[j];
            const T ax = d * xs[l][c] + offdiag<T>(L, G, xs[l], 0, c, i, j, k);
            sum += bs[l][c] - ax;
          }
      bs[l + 1][cc] = sum;
      xs[l + 1][cc] = 0;
    }
    __syncthreads();
  }
  // coarsest
  {
    const int l = P.nlev - 1;
    const MgLevelD &L = P.L[l];
    const int n = (int)L.ncell;
    if (LA<T>::dinv(L)) {
      const T *M = LA<T>::dinv(L) + (size_t)n * n * s;
      for (int r = threadIdx.x; r < n; r += blockDim.x) {
        T acc = 0;
        for (int c = 0; c < n; c++) acc += M[(size_t)r * n + c] * bs[l][c];
        xs[l][r] = acc;
      }
      __syncthreads();
    } else {
      for (int it = 0; it < 40; it++) {
        cta_sweep<T>(L, G, sh, s, xs[l], bs[l], 0);
        cta_sweep<T>(L, G, sh, s, xs[l], bs[l], 1);
        cta_sweep<T>(L, G, sh, s, xs[l], bs[l], 1);
        cta_sweep<T>(L, G, sh, s, xs[l], bs[l], 0);
      }
    }
  }
  // up
  for (int l = P.nlev - 2; l >= l0; l--) {
    const MgLevelD &L = P.L[l];
    const MgLevelD &C = P.L[l + 1];
    for (long c = threadIdx.x; c < L.ncell; c += blockDim.x) {
      if (L.code[c] & 0x8000) continue;
      int i, j, k;
      decompose(L, c, i, j, k);
      const int I = C.coarsened[0] ? i / 2 : i, J = C.coarsened[1] ? j / 2 : j, K = C.coarsened[2] ? k / 2 : k;
      xs[l][c] += xs[l + 1][I + (long)C.n[0] * (J + (long)C.n[1] * K)];
    }
    __syncthreads();
    for (int it = 0; it < 2 * P.nu; it++) cta_sweep<T>(L, G, sh, s, xs[l], bs[l], 1 - (it & 1));
  }
  for (long c = threadIdx.x; c < L0.ncell; c += blockDim.x) xout[L0.ncell * s + c] = xs[l0][c];
}

// ---------------------------------------------------------------- launchers
template <typename T>
int launch_rbgs_tile2d(const MgProblem &P, int l, const T *shift, const int *active, int first_color, int mode,
                       T *x, const T *b, const T *xc, cudaStream_t st) {
  const MgLevelD &L = P.L[l];
  const MgLevelD &C = l + 1 < P.nlev ? P.L[l + 1] : P.L[l];
  constexpr int BX = 32, BY = 16, H = 4;
  const int nt = ((L.n[0] + BX - 1) / BX) * ((L.n[1] + BY - 1) / BY);
  prof_begin(KID_RBGS, st);
  k_rbgs_tile2d<T, BX, BY, H><<<dim3(nt, P.nsys), 256, 0, st>>>(L, C, P.periodic[0], P.periodic[1], shift, active,
                                                                 first_color, 2 * P.nu, mode, x, b, xc);
  prof_end(KID_RBGS, st);
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

template <typename T>
size_t coarse_smem_bytes(const MgProblem &P, int l0) {
  size_t n = 0;
  for (int l = l0; l < P.nlev; l++) n += 2 * (size_t)P.L[l].ncell;
  return n * sizeof(T);
}

template <typename T>
int launch_vcycle_coarse(const MgProblem &P, const MgGeom &G, int l0, const T *shift, const int *active, T *x,
                         const T *b, cudaStream_t st) {
  const size_t smem = coarse_smem_bytes<T>(P, l0);
  static size_t configured = 0;
  if (smem > 48 * 1024 && smem > configured) {
    SNAC_CUDA(cudaFuncSetAttribute((const void *)k_vcycle_coarse<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
    configured = smem;
  }
  k_vcycle_coarse<T><<<P.nsys, 256, smem, st>>>(P, G, l0, shift, active, x, b);
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

template int launch_rbgs_tile2d<double>(const MgProblem &, int, const double *, const int *, int, int, double *,
                                        const double *, const double *, cudaStream_t);
template int launch_rbgs_tile2d<float>(const MgProblem &, int, const float *, const int *, int, int, float *,
                                       const float *, const float *, cudaStream_t);
template size_t coarse_smem_bytes<double>(const MgProblem &, int);
template size_t coarse_smem_bytes<float>(const MgProblem &, int);
template int launch_vcycle_coarse<double>(const MgProblem &, const MgGeom &, int, const double *, const int *,
                                          double *, const double *, cudaStream_t);
template int launch_vcycle_coarse<float>(const MgProblem &, const MgGeom &, int, const float *, const int *, float *,
                                         const float *, cudaStream_t);
template __global__ void k_rbgs_tile2d<double, 32, 16, 4>(MgLevelD, MgLevelD, int, int, const double *, const int *,
                                                          int, int, int, double *, const double *, const double *);
template __global__ void k_rbgs_tile2d<float, 32, 16, 4>(MgLevelD, MgLevelD, int, int, const float *, const int *, int,
                                                         int, int, float *, const float *, const float *);
template __global__ void k_vcycle_coarse<double>(MgProblem, MgGeom, int, const double *, const int *, double *,
                                                 const double *);
template __global__ void k_vcycle_coarse<float>(MgProblem, MgGeom, int, const float *, const int *, float *,
                                                const float *);

}  // namespace snac
