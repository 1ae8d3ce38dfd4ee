// snac_mgdev.h -- device helpers shared by the multigrid kernels (level accessors, stencil).
#pragma once
#include "snac_mgk.h"

namespace snac {

template <typename T> struct LA;
template <> struct LA<double> {
  static __host__ __device__ __forceinline__ const double *cc(const MgLevelD &L) { return L.cc; }
  static __host__ __device__ __forceinline__ const double *cp(const MgLevelD &L, int a) { return L.cp[a]; }
  static __host__ __device__ __forceinline__ const double *W(const MgLevelD &L, int a) { return L.W[a]; }
  static __host__ __device__ __forceinline__ double *x(const MgLevelD &L) { return L.x; }
  static __host__ __device__ __forceinline__ double *b(const MgLevelD &L) { return L.b; }
  static __host__ __device__ __forceinline__ const double *dinv(const MgLevelD &L) { return L.dinv; }
};
template <> struct LA<float> {
  static __host__ __device__ __forceinline__ const float *cc(const MgLevelD &L) { return L.ccf; }
  static __host__ __device__ __forceinline__ const float *cp(const MgLevelD &L, int a) { return L.cpf[a]; }
  static __host__ __device__ __forceinline__ const float *W(const MgLevelD &L, int a) { return L.Wf[a]; }
  static __host__ __device__ __forceinline__ float *x(const MgLevelD &L) { return L.xf; }
  static __host__ __device__ __forceinline__ float *b(const MgLevelD &L) { return L.bf; }
  static __host__ __device__ __forceinline__ const float *dinv(const MgLevelD &L) { return L.dinvf; }
};

__device__ __forceinline__ long nbr_idx(const MgLevelD &L, const MgGeom &G, int i, int j, int k, int a, int s) {
  int c[3] = {i, j, k};
  c[a] += s ? 1 : -1;
  if (c[a] < 0 || c[a] >= L.n[a]) {
    if (!G.periodic[a]) return -1;
    c[a] = c[a] < 0 ? c[a] + L.n[a] : c[a] - L.n[a];
  }
  return c[0] + (long)L.n[0] * (c[1] + (long)L.n[1] * c[2]);
}

template <typename T>
__device__ __forceinline__ T diag_of(const MgLevelD &L, const MgGeom &G, const T *shift, long c, int i, int j, int s) {
  const T d = LA<T>::cc(L)[c];
  if (G.mode3d) return d;
  return d + shift[s] * LA<T>::W(L, 0)[i] * LA<T>::W(L, 1)[j];
}

// sum over coupled neighbours of coefficient * v(neighbour)
template <typename T>
__device__ __forceinline__ T offdiag(const MgLevelD &L, const MgGeom &G, const T *v, long off, long c, int i, int j,
                                     int k) {
  T acc = 0;
  const int na = G.mode3d ? 3 : 2;
  for (int a = 0; a < na; a++) {
    if (G.periodic[a] && L.n[a] == 1) continue;
    const long cpn = nbr_idx(L, G, i, j, k, a, 1), cmn = nbr_idx(L, G, i, j, k, a, 0);
    if (cpn >= 0) acc += LA<T>::cp(L, a)[c] * v[off + cpn];
    if (cmn >= 0) acc += LA<T>::cp(L, a)[cmn] * v[off + cmn];
  }
  return acc;
}

__device__ __forceinline__ void decompose(const MgLevelD &L, long c, int &i, int &j, int &k) {
  i = (int)(c % L.n[0]);
  const long r = c / L.n[0];
  j = (int)(r % L.n[1]);
  k = (int)(r / L.n[1]);
}

}  // namespace snac
