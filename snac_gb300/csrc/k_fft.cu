// k_fft.cu -- real-to-real transforms along the FFT axis (fft.f90:10-94).
//
// The reference calls FFTW guru r2r plans on each block's interior and then
// copies every wavenumber slice into HYPRE (solver.f90:869-875).  Here one
// launch transforms the lines of all blocks and writes the result directly in
// the solver box layout [wavenumber][i1][i0], and the inverse reads the box,
// transforms back, applies normfft (main.f90:1017-1019) and writes pp.
//
// R2HC/HC2R with a power-of-two length use a shared-memory radix-2 FFT on
// pairs of real lines packed as one complex line.  Every kind of any length
// whose complex transform length factors into 2, 3 and 5 runs as a
// mixed-radix Stockham FFT (radices 4, 2, 3, 5) in shared memory, with the
// kinds of FFTW's definitions reduced to complex DFTs of symmetric extensions:
//   R2HC / HC2R: length n, two real lines packed as one complex line;
//   REDFT10 (DCT-II): the even extension of length 2n, times exp(-i pi k/2n);
//   REDFT01 (DCT-III): the length-2n DFT of w_j x_j exp(-i pi j/2n), w = 1, 2, 2, ...;
//   REDFT11 (DCT-IV): the length-2n DFT of x_j exp(-i pi j/2n), times 2 exp(-i pi (2k+1)/4n);
//   RODFT10 / RODFT01 / RODFT11 from the DCT of the same type (Wang's relations
//   DST-II_k = DCT-II((-1)^j x)_{n-1-k}, DST-III_k = (-1)^k DCT-III(x reversed)_k,
//   DST-IV_k = (-1)^k DCT-IV(x reversed)_k);
//   REDFT00 (DCT-I): the even extension of length 2(n-1);
//   RODFT00 (DST-I): the odd extension of length 2(n+1), Y_k = -Im of its DFT at k+1.
// Other lengths keep the dense n x n matrix of FFTW's documented definition.
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
  int N, nst;          // use_fft 2: complex length and number of passes
  int rad[16];         // use_fft 2: radix of each pass
};

// ---------------------------------------------------------------- mixed-radix path (use_fft 2)
// small in-register DFT of size R (2, 3, 4, 5): W_R^m = tw[m * NR] with tw[q] = exp(-2 pi i q / N), NR = N / R
__device__ __forceinline__ void dft_small(double2 *v, int R, const double2 *__restrict__ tw, int NR) {
  if (R == 2) {
    const double2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else if (R == 4) {
    const double2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]), t2 = cadd(v[1], v[3]);
    const double2 dd = csub(v[1], v[3]);
    const double2 t3 = make_double2(dd.y, -dd.x);  // -i (v1 - v3)
    v[0] = cadd(t0, t2);
    v[2] = csub(t0, t2);
    v[1] = cadd(t1, t3);
    v[3] = csub(t1, t3);
  } else {
    double2 o[5];
    for (int k = 0; k < R; k++) {
      double2 acc = v[0];
      for (int q = 1; q < R; q++) {
        const double2 w = tw[((q * k) % R) * NR];
        acc = cadd(acc, cmul(v[q], w));
      }
      o[k] = acc;
    }
    for (int k = 0; k < R; k++) v[k] = o[k];
  }
}

// Stockham autosort FFT (exp(-i...)) of nl complex lines of length N in a, ping-ponging with b; the result
// ends in a (the pointers are swapped as needed).  Pass with radix R after sub-transforms of size Ns: item j
// of a line reads x[j + r N/R], applies exp(-2 pi i r (j mod Ns) / (Ns R)), a size-R DFT, and writes
// y[(j - j mod Ns) R + j mod Ns + r Ns].
__device__ void fft_stockham(double2 *&a, double2 *&b, int nl, int N, int nst, const int *rad,
                             const double2 *__restrict__ tw) {
  int Ns = 1;
  for (int st = 0; st < nst; st++) {
    const int R = rad[st], NR = N / R, tscale = N / (Ns * R);
    __syncthreads();
    for (int t = threadIdx.x; t < nl * NR; t += blockDim.x) {
      const int l = t / NR, j = t - l * NR;
      const double2 *x = a + (size_t)l * N;
      double2 *y = b + (size_t)l * N;
      const int jm = j % Ns, tb = jm * tscale;
      double2 v[5];
      v[0] = x[j];
      for (int r = 1; r < R; r++) v[r] = cmul(x[j + r * NR], tw[r * tb]);
      dft_small(v, R, tw, NR);
      const int idx = (j - jm) * R + jm;
      for (int r = 0; r < R; r++) y[idx + r * Ns] = v[r];
    }
    double2 *tmp = a;
    a = b;
    b = tmp;
    Ns *= R;
  }
  __syncthreads();
}

// one kind on nl real lines of length n in s (line-major), through the complex buffers A and B (nl lines of
// g.N each); gt = [tw (N) | pre (n) | post (n)] of this kind.  R2HC/HC2R pack two lines per complex line.
__device__ void transform_general(const LineGeom &g, int kind, const double2 *__restrict__ gt, double *s, double2 *A,
                                  double2 *B, int nl) {
  const int n = g.n, N = g.N;
  const double2 *__restrict__ tw = gt;
  const double2 *__restrict__ pre = gt + N;
  const double2 *__restrict__ post = gt + N + n;
  const bool pairs = kind == SNAC_R2HC || kind == SNAC_HC2R;
  const int nc = pairs ? nl >> 1 : nl;  // complex lines
  __syncthreads();
  for (int t = threadIdx.x; t < nc * N; t += blockDim.x) {
    const int l = t / N, m = t - l * N;
    double2 v = make_double2(0.0, 0.0);
    if (kind == SNAC_R2HC) {
      v = make_double2(s[(2 * l) * n + m], s[(2 * l + 1) * n + m]);
    } else if (kind == SNAC_HC2R) {  // conj(Z), Z = A + i B from the two half-complex lines
      const double *Ah = s + (2 * l) * n, *Bh = s + (2 * l + 1) * n;
      const int k = m, kk = (2 * k <= n) ? k : n - k;
      const double ra = Ah[kk], rb = Bh[kk];
      double ia, ib;
      if (k == 0 || 2 * k == n) { ia = 0.0; ib = 0.0; }
      else if (2 * k < n) { ia = Ah[n - k]; ib = Bh[n - k]; }
      else { ia = -Ah[k]; ib = -Bh[k]; }
      v = make_double2(ra - ib, -(ia + rb));
    } else {
      const double *x = s + l * n;
      switch (kind) {
        case SNAC_REDFT10: v.x = m < n ? x[m] : x[2 * n - 1 - m]; break;
        case SNAC_RODFT10: { const int q = m < n ? m : 2 * n - 1 - m; v.x = (q & 1) ? -x[q] : x[q]; } break;
        case SNAC_REDFT01: case SNAC_REDFT11:
          if (m < n) v = make_double2(x[m] * pre[m].x, x[m] * pre[m].y);
          break;
        case SNAC_RODFT01: case SNAC_RODFT11:
          if (m < n) v = make_double2(x[n - 1 - m] * pre[m].x, x[n - 1 - m] * pre[m].y);
          break;
        case SNAC_REDFT00: v.x = m < n ? x[m] : x[2 * n - 2 - m]; break;
        case SNAC_RODFT00:
          if (m >= 1 && m <= n) v.x = x[m - 1];
          else if (m >= n + 2) v.x = -x[N - m - 1];
          break;
      }
    }
    A[t] = v;
  }
  fft_stockham(A, B, nc, N, g.nst, g.rad, tw);
  for (int t = threadIdx.x; t < nl * n; t += blockDim.x) {
    const int l = t / n, k = t - l * n;
    double y;
    if (kind == SNAC_R2HC) {
      const double2 *Z = A + (l >> 1) * N;
      const double2 Zm = Z[k], Zc = Z[k ? n - k : 0];
      if (!(l & 1)) y = (2 * k <= n) ? 0.5 * (Zm.x + Zc.x) : 0.5 * (Zc.y - Zm.y);
      else y = (2 * k <= n) ? 0.5 * (Zm.y + Zc.y) : 0.5 * (Zm.x - Zc.x);
    } else if (kind == SNAC_HC2R) {
      const double2 z = A[(l >> 1) * N + k];
      y = (l & 1) ? -z.y : z.x;
    } else {
      const double2 *Z = A + l * N;
      switch (kind) {
        case SNAC_REDFT10: { const double2 c = Z[k]; y = c.x * post[k].x - c.y * post[k].y; } break;
        case SNAC_RODFT10: {
          const int q = n - 1 - k;
          const double2 c = Z[q];
          y = c.x * post[q].x - c.y * post[q].y;
        } break;
        case SNAC_REDFT01: y = Z[k].x; break;
        case SNAC_RODFT01: y = (k & 1) ? -Z[k].x : Z[k].x; break;
        case SNAC_REDFT11: { const double2 c = Z[k]; y = c.x * post[k].x - c.y * post[k].y; } break;
        case SNAC_RODFT11: {
          const double2 c = Z[k];
          const double v = c.x * post[k].x - c.y * post[k].y;
          y = (k & 1) ? -v : v;
        } break;
        case SNAC_REDFT00: y = Z[k].x; break;
        default: y = -Z[k + 1].y; break;  // RODFT00
      }
    }
    s[t] = y;
  }
  __syncthreads();
}

// the lines of one CTA in s: the path chosen for this transform (zb: complex buffers behind s)
__device__ __forceinline__ void transform_lines(const LineGeom &g, const double2 *__restrict__ tw,
                                                const double *__restrict__ mat, double *s, double2 *zb) {
  if (g.use_fft == 2) transform_general(g, g.kind, tw, s, zb, zb + (size_t)g.lp * g.N, g.lp);
  else transform_smem(g.kind, g.n, g.use_fft, g.logn, tw, mat, s, zb, g.lp);
}

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
  pdl_enter();
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
  transform_lines(g, tw, mat, s, zb);
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
  pdl_enter();
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
  transform_lines(g, tw, mat, s, zb);
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
  transform_lines(g, tw, mat, s, zb);
  for (int t = threadIdx.x; t < g.lp * n; t += blockDim.x) {
    const int l = t % g.lp, q = t / g.lp, line = l0 + l;
    if (line < nlines) arr[(line % m1) * s1 + (line / m1) * s2 + q * sa] = s[l * n + q];
  }
}

// a power of two from 2 to 16 (the kernels take a thread's line as threadIdx.x mod lp); Nc > 0: the complex
// length of the mixed-radix path, whose two complex buffers per line bound the lines to about 96 KB a CTA
static int lines_per_cta(int n, int Nc = 0) {
  const long per_line = Nc > 0 ? 8L * n + 32L * Nc : 16L * n;
  const long cap = (Nc > 0 ? 96L * 1024 : 96L * 1024) / (per_line > 0 ? per_line : 1);
  int lp = 2;
  while (lp * 2 <= 16 && lp * 2 <= cap) lp *= 2;
  return lp;
}
static size_t smem_bytes(int n, int lp, int Nc = 0) {
  return Nc > 0 ? (size_t)lp * (8 * (size_t)n + 32 * (size_t)Nc) : (size_t)lp * n * sizeof(double) * 2;
}

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

// complex transform length of a kind of real length n on the mixed-radix path
static int complex_length(int kind, int n) {
  switch (kind) {
    case SNAC_R2HC: case SNAC_HC2R: return n;
    case SNAC_REDFT00: return n >= 2 ? 2 * (n - 1) : 0;
    case SNAC_RODFT00: return 2 * (n + 1);
    default: return 2 * n;
  }
}
// radices 4, 2, 3, 5 of N (4 first: fewer passes); false when another prime divides N
static bool radices(int N, int *rad, int *nst) {
  int m = N, k = 0;
  for (int r : {4, 2, 3, 5})
    while (m % r == 0 && k < 16) { rad[k++] = r; m /= r; }
  *nst = k;
  return m == 1 && N >= 2;
}
// [tw (N) | pre (n) | post (n)] of a kind, complex: tw = exp(-2 pi i q/N); the DCT/DST pre- and post-factors
static std::vector<double> general_tables(int kind, int n, int N) {
  const double PI = 3.14159265358979323846264338327950288;
  std::vector<double> t(2 * ((size_t)N + 2 * (size_t)n), 0.0);
  for (int q = 0; q < N; q++) { t[2 * q] = cos(2.0 * PI * q / N); t[2 * q + 1] = -sin(2.0 * PI * q / N); }
  double *pre = t.data() + 2 * (size_t)N, *post = pre + 2 * (size_t)n;
  for (int j = 0; j < n; j++) {
    const double c = cos(PI * j / (2.0 * n)), sn = -sin(PI * j / (2.0 * n));
    const double w = (kind == SNAC_REDFT01 || kind == SNAC_RODFT01) ? (j == 0 ? 1.0 : 2.0) : 1.0;
    pre[2 * j] = w * c;
    pre[2 * j + 1] = w * sn;
    if (kind == SNAC_REDFT10 || kind == SNAC_RODFT10) { post[2 * j] = c; post[2 * j + 1] = sn; }
    if (kind == SNAC_REDFT11 || kind == SNAC_RODFT11) {
      post[2 * j] = 2.0 * cos(PI * (2 * j + 1) / (4.0 * n));
      post[2 * j + 1] = -2.0 * sin(PI * (2 * j + 1) / (4.0 * n));
    }
  }
  return t;
}
// the mixed-radix path applies to this kind and length
static bool general_ok(int kind, int n, int *N, int *rad, int *nst) {
  *N = complex_length(kind, n);
  if (*N < 2 || !radices(*N, rad, nst)) return false;
  if ((kind == SNAC_R2HC || kind == SNAC_HC2R) && n < 2) return false;
  return true;
}

struct FftLaunch {
  int lp;
  size_t smem;
};
static int prep_launch(int n, FftLaunch &L, const void *fn, int Nc = 0) {
  L.lp = lines_per_cta(n, Nc);
  L.smem = smem_bytes(n, L.lp, Nc);
  if (L.smem > 48 * 1024) SNAC_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem));
  return SNAC_OK;
}

// tables of line tiles, box offsets and solved line extents, built once per solver
static int ensure_tables(Domain &d, PoissonSolver &S) {
  if (S.tabs_ready) return SNAC_OK;
  const int a = S.fft_axis ? S.fft_axis - 1 : 0;
  const int t1 = a == 0 ? 1 : 0, t2 = a == 2 ? 1 : 2;
  S.lt_lp = lines_per_cta(S.fft_axis ? S.nfft : 1, S.use_fft == 2 ? S.nfft_c : 0);
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
  g.N = S.nfft_c;
  g.nst = S.fft_nst;
  for (int q = 0; q < 16; q++) g.rad[q] = S.fft_rad[q];
  return g;
}

int fft_forward_to_box(Domain &d, PoissonSolver &S, cudaStream_t st) {
  SNAC_TRY(ensure_tables(d, S));
  LineGeom g = line_geom(S, S.kind_fwd);
  FftLaunch L;
  SNAC_TRY(prep_launch(g.n, L, (const void *)k_fft_fwd_box, S.use_fft == 2 ? S.nfft_c : 0));
  prof_begin(KID_FFT_FWD, st);
  SNAC_CUDA(launch_k(k_fft_fwd_box, dim3(S.nlt), dim3(256), L.smem, st, d.d_db, S.d_lt, S.d_boff, S.d_lext, g,
                     (const double2 *)(S.use_fft == 2 ? S.d_gt_fwd : S.d_tw), S.d_mat_fwd, S.box_b));
  prof_end(KID_FFT_FWD, st);
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

int fft_backward_from_box(Domain &d, PoissonSolver &S, cudaStream_t st) {
  SNAC_TRY(ensure_tables(d, S));
  LineGeom g = line_geom(S, S.kind_bwd);
  FftLaunch L;
  SNAC_TRY(prep_launch(g.n, L, (const void *)k_fft_bwd_box, S.use_fft == 2 ? S.nfft_c : 0));
  prof_begin(KID_FFT_BWD, st);
  SNAC_CUDA(launch_k(k_fft_bwd_box, dim3(S.nlt), dim3(256), L.smem, st, d.d_db, S.d_lt, S.d_boff, S.d_lext, g,
                     (const double2 *)(S.use_fft == 2 ? S.d_gt_bwd : S.d_tw), S.d_mat_bwd, S.box_x, S.normfft));
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
  int Nf = 0, nstf = 0, radf[16], Nb = 0, nstb = 0, radb[16];
  S.use_fft = (S.kind_fwd == SNAC_R2HC && pow2(n)) ? 1 : 0;
  if (!S.use_fft && general_ok(S.kind_fwd, n, &Nf, radf, &nstf) && general_ok(S.kind_bwd, n, &Nb, radb, &nstb) &&
      Nf == Nb) {
    S.use_fft = 2;
    S.nfft_c = Nf;
    S.fft_nst = nstf;
    for (int q = 0; q < 16; q++) S.fft_rad[q] = radf[q];
    auto tf = general_tables(S.kind_fwd, n, Nf), tb = general_tables(S.kind_bwd, n, Nb);
    S.d_gt_fwd = (double *)S.alloc(tf.size() * sizeof(double));
    S.d_gt_bwd = (double *)S.alloc(tb.size() * sizeof(double));
    if (!S.d_gt_fwd || !S.d_gt_bwd) { set_error("device allocation failed (transform tables)"); return SNAC_ERR_NOMEM; }
    SNAC_CUDA(cudaMemcpy(S.d_gt_fwd, tf.data(), tf.size() * sizeof(double), cudaMemcpyHostToDevice));
    SNAC_CUDA(cudaMemcpy(S.d_gt_bwd, tb.data(), tb.size() * sizeof(double), cudaMemcpyHostToDevice));
    return SNAC_OK;
  }
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
  g.N = 0;
  g.nst = 0;
  if (!g.use_fft && general_ok(kind, n, &g.N, g.rad, &g.nst)) g.use_fft = 2;
  else g.N = 0;
  g.lp = lines_per_cta(n, g.N);
  g.llp = ilog2(g.lp);
  g.ncell = 0; g.n0 = 0;
  double *dtw = nullptr, *dmat = nullptr;
  if (g.use_fft == 2) {
    auto t = general_tables(kind, n, g.N);
    SNAC_CUDA(cudaMalloc(&dtw, t.size() * sizeof(double)));
    SNAC_CUDA(cudaMemcpy(dtw, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice));
  } else if (g.use_fft) {
    auto tw = twiddles(n);
    SNAC_CUDA(cudaMalloc(&dtw, tw.size() * sizeof(double)));
    SNAC_CUDA(cudaMemcpy(dtw, tw.data(), tw.size() * sizeof(double), cudaMemcpyHostToDevice));
  } else {
    auto m = r2r_matrix(kind, n);
    SNAC_CUDA(cudaMalloc(&dmat, m.size() * sizeof(double)));
    SNAC_CUDA(cudaMemcpy(dmat, m.data(), m.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  FftLaunch L;
  int rc = prep_launch(n, L, (const void *)k_r2r_strided, g.N);
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
