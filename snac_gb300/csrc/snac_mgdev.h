// snac_mgdev.h -- device helpers shared by the multigrid kernels (level accessors, stencil).
//
// Every kernel that applies the operator (smoothers, residuals, the tiled and the
// one-CTA kernels) forms the same sums in the same order with explicit FMAs:
//   diagonal  d   = fma(shift_s, w01, cc)           (w01: area in plane mode, volume in 3-D)
//   couplings acc = +x, -x, +y, -y (, +z, -z) terms, each acc = fma(c, v, acc)
//   smoother  x   = (b - acc) * rcpt(d)
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
  static __host__ __device__ __forceinline__ double *xp(const MgLevelD &L) { return L.xp; }
  static __host__ __device__ __forceinline__ const double *dinv(const MgLevelD &L) { return L.dinv; }
  static __host__ __device__ __forceinline__ const double *invd(const MgLevelD &L) { return L.invd; }
};
template <> struct LA<float> {
  static __host__ __device__ __forceinline__ const float *cc(const MgLevelD &L) { return L.ccf; }
  static __host__ __device__ __forceinline__ const float *cp(const MgLevelD &L, int a) { return L.cpf[a]; }
  static __host__ __device__ __forceinline__ const float *W(const MgLevelD &L, int a) { return L.Wf[a]; }
  static __host__ __device__ __forceinline__ const float *w01(const MgLevelD &L) { return L.w01f; }
  static __host__ __device__ __forceinline__ float *x(const MgLevelD &L) { return L.xf; }
  static __host__ __device__ __forceinline__ float *b(const MgLevelD &L) { return L.bf; }
  static __host__ __device__ __forceinline__ float *xp(const MgLevelD &L) { return L.xpf; }
  static __host__ __device__ __forceinline__ const float *dinv(const MgLevelD &L) { return L.dinvf; }
  static __host__ __device__ __forceinline__ const float *invd(const MgLevelD &L) { return L.invdf; }
};

__device__ __forceinline__ float fmat(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fmat(double a, double b, double c) { return __fma_rn(a, b, c); }
// correctly rounded reciprocal (the value of 1/d); every smoother uses it for 1/diagonal
__device__ __forceinline__ float rcpt(float d) { return __frcp_rn(d); }
__device__ __forceinline__ double rcpt(double d) { return __drcp_rn(d); }

// diagonal of cell c for a system with shift sh: cc + sh * w01 (w01 = area in plane mode, where sh is the
// wavenumber's eigenvalue; volume in 3-D mode, where sh is 0 for the pressure and alphai for IMPDIFF)
template <typename T>
__device__ __forceinline__ T diag_of(const MgLevelD &L, const MgGeom &G, T sh, int c) {
  (void)G;
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

// 3-D mode with factored couplings (MgProblem::sep): the couplings of cell c = (i, j, k) formed from the 1-D
// face factors caf[a] and the widths Wf, in the order of offdiag (+x, -x, +y, -y, +z, -z); a folded face (its
// code bits non-zero) contributes nothing, an unfolded face always has its neighbour (periodic wrap included).
// FP32 only: the products round differently from the stored FP32 couplings, which is immaterial for the
// preconditioner they serve (a coupling is the same value seen from either cell, so it stays symmetric).
template <typename V>
__device__ __forceinline__ float offdiag_sep(const MgLevelD &L, const MgGeom &G, V v, int c, int i, int j, int k,
                                             unsigned cd) {
  const int n0 = L.n[0], n1 = L.n[1], n2 = L.n[2], st = n0 * n1;
  const float w0 = L.Wf[0][i], w1 = L.Wf[1][j], w2 = L.Wf[2][k];
  // every neighbour value and 1-D factor is read before the fold bits are tested (the wrapped indices are in
  // range for every cell), so these loads do not wait for the cell's code; the FMAs run in the same order
  const float xe = v(i + 1 < n0 ? c + 1 : c + 1 - n0), xw = v(i > 0 ? c - 1 : c + n0 - 1);
  const float xn = v(j + 1 < n1 ? c + n0 : c + n0 - st), xs = v(j > 0 ? c - n0 : c + st - n0);
  const float xt = v(k + 1 < n2 ? c + st : c + st - st * n2), xb = v(k > 0 ? c - st : c + st * (n2 - 1));
  const float ae = L.caf[0][i], aw = L.caf[0][i > 0 ? i - 1 : n0 - 1];
  const float an = L.caf[1][j], as = L.caf[1][j > 0 ? j - 1 : n1 - 1];
  const float at = L.caf[2][k], ab = L.caf[2][k > 0 ? k - 1 : n2 - 1];
  float acc = 0.f;
  if (!(G.periodic[0] && n0 == 1)) {
    const float wt = w1 * w2;
    if (!((cd >> 2) & 3)) acc = fmat(ae * wt, xe, acc);
    if (!(cd & 3)) acc = fmat(aw * wt, xw, acc);
  }
  if (!(G.periodic[1] && n1 == 1)) {
    const float wt = w0 * w2;
    if (!((cd >> 6) & 3)) acc = fmat(an * wt, xn, acc);
    if (!((cd >> 4) & 3)) acc = fmat(as * wt, xs, acc);
  }
  if (!(G.periodic[2] && n2 == 1)) {
    const float wt = w0 * w1;
    if (!((cd >> 10) & 3)) acc = fmat(at * wt, xt, acc);
    if (!((cd >> 8) & 3)) acc = fmat(ab * wt, xb, acc);
  }
  return acc;
}
// the diagonal with factored couplings: cc, plus the shift times the cell volume W0 W1 W2 when there is one
__device__ __forceinline__ float diag_sep(const MgLevelD &L, float sh, int c, int i, int j, int k) {
  const float cc = L.ccf[c];
  return sh == 0.f ? cc : fmat(sh, L.Wf[0][i] * L.Wf[1][j] * L.Wf[2][k], cc);
}

// One cell of the plane operator: neighbour indices and couplings in the order +x, -x, +y, -y.  A
// neighbour that does not exist gets index c and coupling 0, which leaves the FMA chain unchanged.
template <typename T>
struct PlaneCell {
  int c, ie, iw, in, is;
  T ce, cw, cn, cs;
};
template <typename T>
__device__ __forceinline__ PlaneCell<T> plane_cell(const MgLevelD &L, int per0, int per1, int i, int j) {
  const int n0 = L.n[0], n1 = L.n[1];
  const T *__restrict__ cp0 = LA<T>::cp(L, 0);
  const T *__restrict__ cp1 = LA<T>::cp(L, 1);
  PlaneCell<T> P;
  const int c = i + n0 * j;
  P.c = P.ie = P.iw = P.in = P.is = c;
  P.ce = P.cw = P.cn = P.cs = T(0);
  if (!(per0 && n0 == 1)) {
    if (i + 1 < n0) { P.ie = c + 1; P.ce = cp0[c]; }
    else if (per0) { P.ie = c + 1 - n0; P.ce = cp0[c]; }
    if (i > 0) { P.iw = c - 1; P.cw = cp0[c - 1]; }
    else if (per0) { P.iw = c + n0 - 1; P.cw = cp0[c + n0 - 1]; }
  }
  if (!(per1 && n1 == 1)) {
    if (j + 1 < n1) { P.in = c + n0; P.cn = cp1[c]; }
    else if (per1) { P.in = c + n0 - n0 * n1; P.cn = cp1[c]; }
    if (j > 0) { P.is = c - n0; P.cs = cp1[c - n0]; }
    else if (per1) { P.is = c + n0 * (n1 - 1); P.cs = cp1[c + n0 * (n1 - 1)]; }
  }
  return P;
}
template <typename T, typename V>
__device__ __forceinline__ T plane_acc(const PlaneCell<T> &P, V v) {
  T acc = fmat(P.ce, v(P.ie), T(0));
  acc = fmat(P.cw, v(P.iw), acc);
  acc = fmat(P.cn, v(P.in), acc);
  return fmat(P.cs, v(P.is), acc);
}

// Level kernels run on (32, 8) blocks: grid.z is the system (plane mode) or the k plane (3-D mode).
__device__ __forceinline__ void zpos(const MgGeom &G, int &k, int &s) {
  if (G.mode3d) { k = blockIdx.z; s = 0; }
  else { k = 0; s = blockIdx.z; }
}

// Asynchronous global -> shared copies of N bytes (4, 8 or 16), zero-filled when !valid (then nothing is
// read); a thread may read what it copied itself after cp_async_wait.
template <int N>
__device__ __forceinline__ void cp_async_zfill(void *dst, const void *src, bool valid) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  const int sz = valid ? N : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(d), "l"(src), "n"(N), "r"(sz) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Block-wide sums of per-thread accumulators (any block shape); thread 0 receives the totals.
// Every thread of the block must call them (they contain barriers).
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
  __syncthreads();  // sa/sb may be reused by the next call
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
  __syncthreads();  // sa may be reused by the next call
  return ta;
}

}  // namespace snac
