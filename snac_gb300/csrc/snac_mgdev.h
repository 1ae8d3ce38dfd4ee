// snac_mgdev.h -- device helpers shared by the multigrid kernels (level accessors, stencil).
//
// Every kernel that applies the operator (smoothers, residuals, the tiled and the
// one-CTA kernels) forms the same sums in the same order with explicit FMAs:
//   diagonal  d   = fma(lambda_s, w01, cc)          (plane mode; cc alone in 3-D)
//   couplings acc = +x, -x, +y, -y (, +z, -z) terms, each acc = fma(c, v, acc)
//   smoother  x   = (b - acc) * (1 / d)
//   residual  r   = b - fma(d, x, acc)
// so fused and unfused V-cycles produce identical iterates.
#pragma once
#include "snac_mgk.h"

namespace snac {

template <typename T> struct LA;
template <> struct LA<double> {
  static __host__ __device__ __forceinline__ const double *cc(const MgLevelD &L) { return L.cc; }
  static __host__ __device__ __forceinline__ const double *cp(const MgLevelD &L, int a) { return L.cp[a]; }
  static __host__ __device__ __forceinline__ const double *W(const MgLevelD &L, int a) { return L.W[a]; }
  static __host__ __device__ __forceinline__ const double *w01(const MgLevelD &L) { return L.w01; }
  static __host__ __device__ __forceinline__ double *x(const MgLevelD &L) { return L.x; }
  static __host__ __device__ __forceinline__ double *b(const MgLevelD &L) { return L.b; }
  static __host__ __device__ __forceinline__ const double *dinv(const MgLevelD &L) { return L.dinv; }
};
template <> struct LA<float> {
  static __host__ __device__ __forceinline__ const float *cc(const MgLevelD &L) { return L.ccf; }
  static __host__ __device__ __forceinline__ const float *cp(const MgLevelD &L, int a) { return L.cpf[a]; }
  static __host__ __device__ __forceinline__ const float *W(const MgLevelD &L, int a) { return L.Wf[a]; }
  static __host__ __device__ __forceinline__ const float *w01(const MgLevelD &L) { return L.w01f; }
  static __host__ __device__ __forceinline__ float *x(const MgLevelD &L) { return L.xf; }
  static __host__ __device__ __forceinline__ float *b(const MgLevelD &L) { return L.bf; }
  static __host__ __device__ __forceinline__ const float *dinv(const MgLevelD &L) { return L.dinvf; }
};

__device__ __forceinline__ float fmat(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fmat(double a, double b, double c) { return __fma_rn(a, b, c); }

template <typename T>
__device__ __forceinline__ T diag_of(const MgLevelD &L, const MgGeom &G, T sh, int c) {
  if (G.mode3d) return LA<T>::cc(L)[c];
  return fmat(sh, LA<T>::w01(L)[c], LA<T>::cc(L)[c]);
}

// in-plane couplings of cell c = (i, j); v(e) returns the value at cell e of the same system
template <typename T, typename V>
__device__ __forceinline__ T offdiag_xy(int n0, int n1, int per0, int per1, const T *__restrict__ c0,
                                        const T *__restrict__ c1, V v, int c, int i, int j) {
  T acc = 0;
  if (!(per0 && n0 == 1)) {
    if (i + 1 < n0) acc = fmat(c0[c], v(c + 1), acc);
    else if (per0) acc = fmat(c0[c], v(c + 1 - n0), acc);
    if (i > 0) acc = fmat(c0[c - 1], v(c - 1), acc);
    else if (per0) acc = fmat(c0[c + n0 - 1], v(c + n0 - 1), acc);
  }
  if (!(per1 && n1 == 1)) {
    if (j + 1 < n1) acc = fmat(c1[c], v(c + n0), acc);
    else if (per1) acc = fmat(c1[c], v(c + n0 - n0 * n1), acc);
    if (j > 0) acc = fmat(c1[c - n0], v(c - n0), acc);
    else if (per1) acc = fmat(c1[c + n0 * (n1 - 1)], v(c + n0 * (n1 - 1)), acc);
  }
  return acc;
}

// all couplings of cell c = (i, j, k) of level L (cell indices of one system fit in 32 bits)
template <typename T, typename V>
__device__ __forceinline__ T offdiag(const MgLevelD &L, const MgGeom &G, V v, int c, int i, int j, int k) {
  const int n0 = L.n[0], n1 = L.n[1];
  T acc = offdiag_xy<T>(n0, n1, G.periodic[0], G.periodic[1], LA<T>::cp(L, 0), LA<T>::cp(L, 1), v, c, i, j);
  if (G.mode3d) {
    const int n2 = L.n[2], st = n0 * n1;
    if (!(G.periodic[2] && n2 == 1)) {
      const T *__restrict__ c2 = LA<T>::cp(L, 2);
      if (k + 1 < n2) acc = fmat(c2[c], v(c + st), acc);
      else if (G.periodic[2]) acc = fmat(c2[c], v(c + st - st * n2), acc);
      if (k > 0) acc = fmat(c2[c - st], v(c - st), acc);
      else if (G.periodic[2]) acc = fmat(c2[c + st * (n2 - 1)], v(c + st * (n2 - 1)), acc);
    }
  }
  return acc;
}

// Level kernels run on (32, 8) blocks: grid.z is the system (plane mode) or the k plane (3-D mode).
__device__ __forceinline__ void zpos(const MgGeom &G, int &k, int &s) {
  if (G.mode3d) { k = blockIdx.z; s = 0; }
  else { k = 0; s = blockIdx.z; }
}

// Block-wide sums of per-thread accumulators (any block shape); thread 0 receives the totals.
template <typename A>
__device__ __forceinline__ void block_sum2(A a, A b, double &ta, double &tb) {
  __shared__ double sa[32], sb[32];
  const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  if ((t & 31) == 0) { sa[t >> 5] = (double)a; sb[t >> 5] = (double)b; }
  __syncthreads();
  ta = tb = 0.0;
  if (t == 0)
    for (int q = 0; q < nw; q++) { ta += sa[q]; tb += sb[q]; }
}
template <typename A>
__device__ __forceinline__ double block_sum1(A a) {
  __shared__ double sa[32];
  const int t = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
  for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
  if ((t & 31) == 0) sa[t >> 5] = (double)a;
  __syncthreads();
  double ta = 0.0;
  if (t == 0)
    for (int q = 0; q < nw; q++) ta += sa[q];
  return ta;
}

}  // namespace snac
