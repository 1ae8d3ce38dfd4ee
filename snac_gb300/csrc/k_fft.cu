// k_fft.cu -- real-to-real transforms along the FFT axis (fft.f90:10-94).
//
// The reference calls FFTW guru r2r plans on each block's interior and then
// copies every wavenumber slice into HYPRE (solver.f90:869-875).  Here one
// launch transforms the lines of all blocks and writes the result directly in
// the solver box layout [wavenumber][i1][i0], and the inverse reads the box,
// transforms back, applies normfft (main.f90:1017-1019) and writes pp.
//
// R2HC/HC2R with a power-of-two length use a shared-memory radix-2 FFT on
// pairs of real lines packed as one complex line; every other kind (and any
// length) uses a dense n x n matrix of FFTW's documented definition.
#include <cmath>

#include "snac_host.h"
#include "snac_prof.h"

namespace snac {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ int bitrev(int q, int logn) { return (int)(__brev((unsigned)q) >> (32 - logn)); }

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }

// in-place radix-2 DIT FFT (exp(-i...)) of npair complex lines of length n = 2^logn held in bit-reversed
// order (index arithmetic by shifts and masks).  Two consecutive stages (spans h and 2h) run as one pass:
// a thread loads the 4 points of a group of 4h and applies the same butterflies and twiddles as the two
// radix-2 stages would, so the results are those of the stage-by-stage form with half the passes over
// shared memory and half the barriers.
__device__ void fft_pairs(double2 *zb, int npair, int n, int logn, const double2 *__restrict__ tw) {
  const int half = n >> 1, lhalf = logn - 1;
  int lh = 0;
  for (; lh + 1 < logn; lh += 2) {
    __syncthreads();
    const int h = 1 << lh, lq = logn - 2, quarter = n >> 2;
    const int s1 = lhalf - lh, s2 = lhalf - lh - 1;  // twiddle strides n / (2h) and n / (4h)
    for (int t = threadIdx.x; t < (npair << lq); t += blockDim.x) {
      const int p = t >> lq, b = t & (quarter - 1);
      const int grp = b >> lh, k = b & (h - 1);
      double2 *z = zb + p * n + (grp << (lh + 2)) + k;
      const double2 a0 = z[0], a1 = z[h], a2 = z[2 * h], a3 = z[3 * h];
      const double2 w1 = tw[k << s1];
      const double2 t1 = cmul(w1, a1), t3 = cmul(w1, a3);
      const double2 b0 = cadd(a0, t1), b1 = csub(a0, t1), b2 = cadd(a2, t3), b3 = csub(a2, t3);
      const double2 u2 = cmul(tw[k << s2], b2), u3 = cmul(tw[(k + h) << s2], b3);
      z[0] = cadd(b0, u2);
      z[2 * h] = csub(b0, u2);
      z[h] = cadd(b1, u3);
      z[3 * h] = csub(b1, u3);
    }
  }
  if (lh < logn) {  // a last single stage (odd logn)
    __syncthreads();
    const int h = 1 << lh, lstep = lhalf - lh;
    for (int t = threadIdx.x; t < (npair << lhalf); t += blockDim.x) {
      const int p = t >> lhalf, b = t & (half - 1);
      const int grp = b >> lh, k = b & (h - 1);
      const int i0 = (grp << (lh + 1)) + k, i1 = i0 + h;
      const double2 w = tw[k << lstep];
      double2 *z = zb + p * n;
      const double2 x0 = z[i0], t1 = cmul(w, z[i1]);
      z[i0] = cadd(x0, t1);
      z[i1] = csub(x0, t1);
    }
  }
  __syncthreads();
}

// transform nl lines (nl even for the FFT path) of length n held in s (line-major) in place
__device__ void transform_smem(int kind, int n, int use_fft, int logn, const double2 *__restrict__ tw,
                               const double *__restrict__ mat, double *s, double2 *zb, int nl) {
  if (!use_fft) {
    // dense: out[l][k] = sum_j M[k][j] s[l][j]; results staged in zb (as doubles)
    double *o = (double *)zb;
    __syncthreads();
    for (int t = threadIdx.x; t < nl * n; t += blockDim.x) {
      const int l = t / n, k = t - l * n;
      const double *x = s + l * n;
      const double *M = mat + (size_t)k * n;
      double acc = 0.0;
      for (int j = 0; j < n; j++) acc = fma(M[j], x[j], acc);
      o[t] = acc;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nl * n; t += blockDim.x) s[t] = o[t];
    __syncthreads();
    return;
  }
  const int npair = nl >> 1;
  __syncthreads();
  if (kind == SNAC_R2HC) {
    for (int t = threadIdx.x; t < npair * n; t += blockDim.x) {
      const int p = t >> logn, q = t & (n - 1);
      zb[p * n + (logn ? bitrev(q, logn) : 0)] = make_double2(s[(2 * p) * n + q], s[(2 * p + 1) * n + q]);
    }
    fft_pairs(zb, npair, n, logn, tw);
    for (int t = threadIdx.x; t < npair * n; t += blockDim.x) {
      const int p = t >> logn, m = t & (n - 1);
      const double2 Zm = zb[p * n + m], Zc = zb[p * n + ((n - m) & (n - 1))];
      double a, b;
      if (2 * m <= n) { a = 0.5 * (Zm.x + Zc.x); b = 0.5 * (Zm.y + Zc.y); }
      else { a = 0.5 * (Zc.y - Zm.y); b = 0.5 * (Zm.x - Zc.x); }
      s[(2 * p) * n + m] = a;
      s[(2 * p + 1) * n + m] = b;
    }
  } else {  // HC2R
    for (int t = threadIdx.x; t < npair * n; t += blockDim.x) {
      const int p = t >> logn, k = t & (n - 1);
      const double *A = s + (2 * p) * n, *B = s + (2 * p + 1) * n;
      const int kk = (2 * k <= n) ? k : n - k;
      const double ra = A[kk], rb = B[kk];
      double ia, ib;
      if (k == 0 || 2 * k == n) { ia = 0.0; ib = 0.0; }
      else if (2 * k < n) { ia = A[n - k]; ib = B[n - k]; }
      else { ia = -A[k]; ib = -B[k]; }
      // conj(Z) with Z = A + iB
      zb[p * n + (logn ? bitrev(k, logn) : 0)] = make_double2(ra - ib, -(ia + rb));
    }
    fft_pairs(zb, npair, n, logn, tw);
    for (int t = threadIdx.x; t < npair * n; t += blockDim.x) {
      const int p = t >> logn, q = t & (n - 1);
      const double2 z = zb[p * n + q];
      s[(2 * p) * n + q] = z.x;
      s[(2 * p + 1) * n + q] = -z.y;
    }
  }
  __syncthreads();
}

struct LineGeom {
  int a, t1, t2;       // transform axis and the two other axes (t1 < t2)
  int n, logn, use_fft, kind, lp, llp;  // lp = 2^llp lines per CTA
  long ncell;          // box cells per system (plane mode)
  int n0;              // box extent along t1
  int field;           // HF_P: pp; HF_U + c: u, v, w; HF_S0 + s: scalar s
};

__device__ __forceinline__ double *line_field(const DBlock &B, int field) {
  if (field == HF_P) return B.pp;
  if (field == HF_U) return B.u;
  if (field == HF_U + 1) return B.v;
  if (field == HF_U + 2) return B.w;
  return B.s[field - HF_S0];
}

// forward: the field's interior lines of all blocks (their first n points along the transform axis) ->
// box[q][i1][i0]; a line outside the solved extents (a wall face of a staggered component) is transformed
// in place, as fft() transforms the whole interior (solve_helmholtz.f90:86)
__global__ void k_fft_fwd_box(const DBlock *__restrict__ Bs, const int2 *__restrict__ LT, const int2 *__restrict__ boff,
                              const int2 *__restrict__ lext, LineGeom g, const double2 *__restrict__ tw,
                              const double *__restrict__ mat, double *__restrict__ box) {
  extern __shared__ double smem[];
  const int2 lt = LT[blockIdx.x];
  const DBlock &B = Bs[lt.x];
  const int n1 = B.n[g.t1], nlines = B.n[g.t1] * B.n[g.t2];
  const int2 ex = lext[lt.x];
  double *__restrict__ f = line_field(B, g.field);
  double *s = smem;
  double2 *zb = (double2 *)(smem + g.lp * g.n);
  const int n = g.n;
  // the line of this thread is the same in every pass (blockDim.x is a multiple of lp = 2^llp)
  const int l = threadIdx.x & (g.lp - 1), q0 = threadIdx.x >> g.llp, qs = blockDim.x >> g.llp;
  const int line = lt.y + l;
  const bool valid = line < nlines;
  const int x1 = valid ? line % n1 : 0, x2 = valid ? line / n1 : 0;
  int c[3];
  c[g.a] = 0; c[g.t1] = x1; c[g.t2] = x2;
  const long fb = hidx(c[0], c[1], c[2], B.n[0], B.n[1]);
  const long fs = g.a == 0 ? 1 : g.a == 1 ? (long)(B.n[0] + 2) : (long)(B.n[0] + 2) * (B.n[1] + 2);
  for (int q = q0; q < n; q += qs) s[l * n + q] = valid ? f[fb + fs * q] : 0.0;
  transform_smem(g.kind, n, g.use_fft, g.logn, tw, mat, s, zb, g.lp);
  if (!valid) return;
  const int2 o = boff[lt.x];
  if (x1 < ex.x && x2 < ex.y) {
    double *__restrict__ bx = box + (long)(x1 + o.x) + (long)g.n0 * (x2 + o.y);
    for (int q = q0; q < n; q += qs) bx[g.ncell * q] = s[l * n + q];
  } else {
    for (int q = q0; q < n; q += qs) f[fb + fs * q] = s[l * n + q];
  }
}

// backward: box (or, outside the solved extents, the field) -> field interior lines, times normfft; points
// of a line beyond the transform length (a wall face along the transform axis) are scaled by normfft too
__global__ void k_fft_bwd_box(const DBlock *__restrict__ Bs, const int2 *__restrict__ LT, const int2 *__restrict__ boff,
                              const int2 *__restrict__ lext, LineGeom g, const double2 *__restrict__ tw,
                              const double *__restrict__ mat, const double *__restrict__ box, double normfft) {
  extern __shared__ double smem[];
  const int2 lt = LT[blockIdx.x];
  const DBlock &B = Bs[lt.x];
  const int n1 = B.n[g.t1], nlines = B.n[g.t1] * B.n[g.t2];
  const int2 ex = lext[lt.x];
  double *__restrict__ f = line_field(B, g.field);
  double *s = smem;
  double2 *zb = (double2 *)(smem + g.lp * g.n);
  const int n = g.n;
  const int2 o = boff[lt.x];
  const int l = threadIdx.x & (g.lp - 1), q0 = threadIdx.x >> g.llp, qs = blockDim.x >> g.llp;
  const int line = lt.y + l;
  const bool valid = line < nlines;
  const int x1 = valid ? line % n1 : 0, x2 = valid ? line / n1 : 0;
  int c[3];
  c[g.a] = 0; c[g.t1] = x1; c[g.t2] = x2;
  const long fb = hidx(c[0], c[1], c[2], B.n[0], B.n[1]);
  const long fs = g.a == 0 ? 1 : g.a == 1 ? (long)(B.n[0] + 2) : (long)(B.n[0] + 2) * (B.n[1] + 2);
  const bool inbox = valid && x1 < ex.x && x2 < ex.y;
  const double *__restrict__ bx = box + (long)(x1 + o.x) + (long)g.n0 * (x2 + o.y);
  for (int q = q0; q < n; q += qs) s[l * n + q] = !valid ? 0.0 : inbox ? bx[g.ncell * q] : f[fb + fs * q];
  transform_smem(g.kind, n, g.use_fft, g.logn, tw, mat, s, zb, g.lp);
  if (!valid) return;
  const int na = B.n[g.a];
  for (int q = q0; q < na; q += qs) {
    double *p = &f[fb + fs * q];
    *p = (q < n ? s[l * n + q] : *p) * normfft;
  }
}

// 3-D mode: block interiors <-> box
__global__ void k_box_io(const DBlock *__restrict__ Bs, const Tile *__restrict__ T, const int4 *__restrict__ boff3,
                         int n0, int n1, double *box, int to_box) {
  const Tile t = T[blockIdx.x];
  const DBlock &B = Bs[t.x];
  const int nx = B.n[0], ny = B.n[1], nz = B.n[2];
  const int i = t.y + (int)threadIdx.x, j = t.z + (int)threadIdx.y, k = t.w + (int)threadIdx.z;
  if (i >= nx || j >= ny || k >= nz) return;
  const int4 o = boff3[t.x];
  const long cell = (long)(i + o.x) + (long)n0 * ((long)(j + o.y) + (long)n1 * (k + o.z));
  const long c = hidx(i, j, k, nx, ny);
  if (to_box) box[cell] = B.pp[c];
  else B.pp[c] = box[cell];
}

// generic strided lines (snac_fft): line l starts at base(l) = (l % m1)*s1 + (l / m1)*s2, element q at q*sa
__global__ void k_r2r_strided(double *arr, int m1, long s1, long s2, long sa, int nlines, LineGeom g,
                              const double2 *__restrict__ tw, const double *__restrict__ mat) {
  extern __shared__ double smem[];
  double *s = smem;
  double2 *zb = (double2 *)(smem + g.lp * g.n);
  const int n = g.n;
  const int l0 = blockIdx.x * g.lp;
  for (int t = threadIdx.x; t < g.lp * n; t += blockDim.x) {
    const int l = t % g.lp, q = t / g.lp, line = l0 + l;
    s[l * n + q] = line < nlines ? arr[(line % m1) * s1 + (line / m1) * s2 + q * sa] : 0.0;
  }
  transform_smem(g.kind, n, g.use_fft, g.logn, tw, mat, s, zb, g.lp);
  for (int t = threadIdx.x; t < g.lp * n; t += blockDim.x) {
    const int l = t % g.lp, q = t / g.lp, line = l0 + l;
    if (line < nlines) arr[(line % m1) * s1 + (line / m1) * s2 + q * sa] = s[l * n + q];
  }
}

// a power of two from 2 to 16 (the kernels take a thread's line as threadIdx.x mod lp)
static int lines_per_cta(int n) {
  const int cap = 6144 / (n > 0 ? n : 1);
  int lp = 2;
  while (lp * 2 <= 16 && lp * 2 <= cap) lp *= 2;
  return lp;
}
static size_t smem_bytes(int n, int lp) { return (size_t)lp * n * sizeof(double) * 2; }

static int ilog2(int n) {
  int l = 0;
  while ((1 << l) < n) l++;
  return l;
}

// host: FFTW's unnormalised r2r kinds as dense matrices, M[k*n + j]
std::vector<double> r2r_matrix(int kind, int n) {
  const double PI = 3.14159265358979323846264338327950288;
  std::vector<double> M((size_t)n * n, 0.0);
  for (int k = 0; k < n; k++)
    for (int j = 0; j < n; j++) {
      double v = 0.0;
      switch (kind) {
        case SNAC_R2HC:
          if (2 * k <= n) v = cos(2.0 * PI * (double)((long)j * k % n) / n);
          else v = -sin(2.0 * PI * (double)((long)j * (n - k) % n) / n);
          break;
        case SNAC_HC2R:
          if (j == 0) v = 1.0;
          else if (2 * j < n) v = 2.0 * cos(2.0 * PI * (double)((long)k * j % n) / n);
          else if (2 * j == n) v = (k % 2) ? -1.0 : 1.0;
          else v = -2.0 * sin(2.0 * PI * (double)((long)k * (n - j) % n) / n);
          break;
        case SNAC_REDFT00:
          if (j == 0) v = 1.0;
          else if (j == n - 1) v = (k % 2) ? -1.0 : 1.0;
          else v = 2.0 * cos(PI * j * k / (double)(n - 1));
          break;
        case SNAC_REDFT10: v = 2.0 * cos(PI * (j + 0.5) * k / n); break;
        case SNAC_REDFT01: v = j == 0 ? 1.0 : 2.0 * cos(PI * j * (k + 0.5) / n); break;
        case SNAC_REDFT11: v = 2.0 * cos(PI * (j + 0.5) * (k + 0.5) / n); break;
        case SNAC_RODFT00: v = 2.0 * sin(PI * (j + 1) * (k + 1) / (double)(n + 1)); break;
        case SNAC_RODFT10: v = 2.0 * sin(PI * (j + 0.5) * (k + 1) / n); break;
        case SNAC_RODFT01: v = j == n - 1 ? ((k % 2) ? -1.0 : 1.0) : 2.0 * sin(PI * (j + 1) * (k + 0.5) / n); break;
        case SNAC_RODFT11: v = 2.0 * sin(PI * (j + 0.5) * (k + 0.5) / n); break;
      }
      M[(size_t)k * n + j] = v;
    }
  return M;
}

static std::vector<double> twiddles(int n) {
  const double PI = 3.14159265358979323846264338327950288;
  std::vector<double> tw(2 * (size_t)std::max(1, n / 2));
  for (int k = 0; k < n / 2; k++) {
    tw[2 * k] = cos(2.0 * PI * k / n);
    tw[2 * k + 1] = -sin(2.0 * PI * k / n);
  }
  return tw;
}

static bool pow2(int n) { return n >= 2 && (n & (n - 1)) == 0; }

struct FftLaunch {
  int lp;
  size_t smem;
};
static int prep_launch(int n, FftLaunch &L, const void *fn) {
  L.lp = lines_per_cta(n);
  L.smem = smem_bytes(n, L.lp);
  if (L.smem > 48 * 1024) SNAC_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem));
  return SNAC_OK;
}

// tables of line tiles, box offsets and solved line extents, built once per solver
static int ensure_tables(Domain &d, PoissonSolver &S) {
  if (S.tabs_ready) return SNAC_OK;
  const int a = S.fft_axis ? S.fft_axis - 1 : 0;
  const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
  S.lt_lp = lines_per_cta(S.fft_axis ? S.nfft : 1);
  std::vector<int2> lt, bo, ex;
  std::vector<int4> bo3;
  for (int b = 0; b < d.nblocks; b++) {
    const HostBlock &H = d.hb[b];
    if (S.fft_axis) {
      const int nl = H.ng[t1] * H.ng[t2];
      for (int l = 0; l < nl; l += S.lt_lp) lt.push_back(make_int2(b, l));
      bo.push_back(make_int2(H.lo[t1] - S.lo_min[t1], H.lo[t2] - S.lo_min[t2]));
      ex.push_back(make_int2(field_hi(H, S.field, t1) - H.lo[t1] + 1, field_hi(H, S.field, t2) - H.lo[t2] + 1));
    }
    bo3.push_back(make_int4(H.lo[0] - S.lo_min[0], H.lo[1] - S.lo_min[1], H.lo[2] - S.lo_min[2], 0));
  }
  S.nlt = (int)lt.size();
  if (!lt.empty()) {
    S.d_lt = (int2 *)S.alloc(lt.size() * sizeof(int2));
    S.d_boff = (int2 *)S.alloc(bo.size() * sizeof(int2));
    S.d_lext = (int2 *)S.alloc(ex.size() * sizeof(int2));
    if (!S.d_lt || !S.d_boff || !S.d_lext) { set_error("device allocation failed (transform tables)"); return SNAC_ERR_NOMEM; }
    SNAC_CUDA(cudaMemcpy(S.d_lt, lt.data(), lt.size() * sizeof(int2), cudaMemcpyHostToDevice));
    SNAC_CUDA(cudaMemcpy(S.d_boff, bo.data(), bo.size() * sizeof(int2), cudaMemcpyHostToDevice));
    SNAC_CUDA(cudaMemcpy(S.d_lext, ex.data(), ex.size() * sizeof(int2), cudaMemcpyHostToDevice));
  }
  S.d_boff3 = (int4 *)S.alloc(bo3.size() * sizeof(int4));
  if (!S.d_boff3) { set_error("device allocation failed (box offsets)"); return SNAC_ERR_NOMEM; }
  SNAC_CUDA(cudaMemcpy(S.d_boff3, bo3.data(), bo3.size() * sizeof(int4), cudaMemcpyHostToDevice));
  S.tabs_ready = 1;
  return SNAC_OK;
}

static LineGeom line_geom(const PoissonSolver &S, int kind) {
  LineGeom g;
  g.a = S.fft_axis - 1;
  g.t1 = g.a == 0 ? 1 : 0;
  g.t2 = g.a == 2 ? 1 : 2;
  g.n = S.nfft;
  g.logn = ilog2(S.nfft);
  g.use_fft = S.use_fft;
  g.kind = kind;
  g.lp = S.lt_lp;
  g.llp = ilog2(S.lt_lp);
  g.ncell = S.ncell0;
  g.n0 = S.P.L[0].n[0];
  g.field = S.field;
  return g;
}

int fft_forward_to_box(Domain &d, PoissonSolver &S, cudaStream_t st) {
  SNAC_TRY(ensure_tables(d, S));
  LineGeom g = line_geom(S, S.kind_fwd);
  FftLaunch L;
  SNAC_TRY(prep_launch(g.n, L, (const void *)k_fft_fwd_box));
  prof_begin(KID_FFT_FWD, st);
  k_fft_fwd_box<<<S.nlt, 256, L.smem, st>>>(d.d_db, S.d_lt, S.d_boff, S.d_lext, g, (const double2 *)S.d_tw,
                                            S.d_mat_fwd, S.box_b), ::snac::count_launch();
  prof_end(KID_FFT_FWD, st);
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

int fft_backward_from_box(Domain &d, PoissonSolver &S, cudaStream_t st) {
  SNAC_TRY(ensure_tables(d, S));
  LineGeom g = line_geom(S, S.kind_bwd);
  FftLaunch L;
  SNAC_TRY(prep_launch(g.n, L, (const void *)k_fft_bwd_box));
  prof_begin(KID_FFT_BWD, st);
  k_fft_bwd_box<<<S.nlt, 256, L.smem, st>>>(d.d_db, S.d_lt, S.d_boff, S.d_lext, g, (const double2 *)S.d_tw,
                                            S.d_mat_bwd, S.box_x, S.normfft), ::snac::count_launch();
  prof_end(KID_FFT_BWD, st);
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

int box_gather(Domain &d, PoissonSolver &S, cudaStream_t st) {
  SNAC_TRY(ensure_tables(d, S));
  k_box_io<<<d.ntiles, dim3(TX, TY, TZ), 0, st>>>(d.d_db, d.d_tiles, S.d_boff3, S.P.L[0].n[0], S.P.L[0].n[1],
                                                  S.box_b, 1), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

int box_scatter(Domain &d, PoissonSolver &S, cudaStream_t st) {
  SNAC_TRY(ensure_tables(d, S));
  k_box_io<<<d.ntiles, dim3(TX, TY, TZ), 0, st>>>(d.d_db, d.d_tiles, S.d_boff3, S.P.L[0].n[0], S.P.L[0].n[1],
                                                  S.box_x, 0), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

// upload twiddles / matrices of a transform pair
int fft_setup(PoissonSolver &S) {
  const int n = S.nfft;
  S.use_fft = (S.kind_fwd == SNAC_R2HC && pow2(n)) ? 1 : 0;
  if (S.use_fft) {
    auto tw = twiddles(n);
    S.d_tw = (double *)S.alloc(tw.size() * sizeof(double));
    SNAC_CUDA(cudaMemcpy(S.d_tw, tw.data(), tw.size() * sizeof(double), cudaMemcpyHostToDevice));
  } else {
    auto mf = r2r_matrix(S.kind_fwd, n), mb = r2r_matrix(S.kind_bwd, n);
    S.d_mat_fwd = (double *)S.alloc(mf.size() * sizeof(double));
    S.d_mat_bwd = (double *)S.alloc(mb.size() * sizeof(double));
    SNAC_CUDA(cudaMemcpy(S.d_mat_fwd, mf.data(), mf.size() * sizeof(double), cudaMemcpyHostToDevice));
    SNAC_CUDA(cudaMemcpy(S.d_mat_bwd, mb.data(), mb.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  return SNAC_OK;
}

// reference-signature transform of a compact interior array arr(n1,n2,n3) along idir (device pointer)
int r2r_array(int kind, int idir, const int nn[3], int q, double *darr, cudaStream_t st) {
  const int a = idir - 1;
  const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
  const long str[3] = {1, (long)nn[0], (long)nn[0] * nn[1]};
  const int n = nn[a] - q;
  if (n <= 0) return SNAC_OK;
  LineGeom g;
  g.a = a; g.t1 = t1; g.t2 = t2; g.n = n; g.logn = ilog2(n); g.kind = kind;
  g.use_fft = ((kind == SNAC_R2HC || kind == SNAC_HC2R) && pow2(n)) ? 1 : 0;
  g.lp = lines_per_cta(n);
  g.llp = ilog2(g.lp);
  g.ncell = 0; g.n0 = 0;
  double *dtw = nullptr, *dmat = nullptr;
  if (g.use_fft) {
    auto tw = twiddles(n);
    SNAC_CUDA(cudaMalloc(&dtw, tw.size() * sizeof(double)));
    SNAC_CUDA(cudaMemcpy(dtw, tw.data(), tw.size() * sizeof(double), cudaMemcpyHostToDevice));
  } else {
    auto m = r2r_matrix(kind, n);
    SNAC_CUDA(cudaMalloc(&dmat, m.size() * sizeof(double)));
    SNAC_CUDA(cudaMemcpy(dmat, m.data(), m.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  FftLaunch L;
  int rc = prep_launch(n, L, (const void *)k_r2r_strided);
  const int nlines = nn[t1] * nn[t2];
  if (rc == SNAC_OK) {
    k_r2r_strided<<<(nlines + L.lp - 1) / L.lp, 256, L.smem, st>>>(darr, nn[t1], str[t1], str[t2], str[a], nlines, g,
                                                                    (const double2 *)dtw, dmat), ::snac::count_launch();
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_fail(e, "k_r2r_strided", __FILE__, __LINE__);
  }
  if (dtw) cudaFree(dtw);
  if (dmat) cudaFree(dmat);
  return rc;
}

}  // namespace snac
