// k_guess.cu -- the learned initial guess of the plane-mode pressure solve (the 3-D solve's U-Net is in
// k_unet.cu; this file's entry points hand the 3-D case to it).
//
// A three-layer convolutional network (3x3, 16 channels, ReLU between layers) maps the residual of the
// previous solution, r0 = b - A x_prev, of one wavenumber system (normalised by its RMS) and the system's
// scaled eigenvalue (a constant channel) to the diagonally scaled correction D (x - x_prev) / RMS(r0), D the
// diagonal of the system's operator: for a strongly shifted system that map is close to the identity, for
// the weakly shifted ones it spreads.  The correction c = RMS(r0) D^-1 net(...) is then applied with the step
// that minimises the residual of the system, x0 = x_prev + alpha c, alpha = <r0, A c> / <A c, A c>, so the
// guess never leaves a larger residual than x_prev.  The multigrid still iterates to the same tolerance: the
// network only changes where the iterations start.  Inference uses the tcgen05 convolution (BF16 operands,
// FP32 accumulation); training runs on the GPU with this file's FP32 backward kernels and Adam, on pairs
// recorded from the solver's own solves.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

#include "snac_host.h"
#include "snac_mgdev.h"

namespace snac {

int launch_conv3x3_tc(const __nv_bfloat16 *x, int nplanes, int H, int W, const float *wts, const float *bias, int relu,
                      float *y, int ny, __nv_bfloat16 *yb, int *err, cudaStream_t st);

namespace {
constexpr int GC = 16;               // channels
constexpr int GL = 3;                // layers
constexpr int GWN = GC * GC * 9;     // weights per layer
constexpr int GB = 16;               // planes per training batch (snac_guess_train)
}  // namespace

// ---------------------------------------------------------------- kernels
// one CTA per plane: RMS of the plane's residual, then the BF16 network input (channel 0 = r / RMS,
// channel 1 = the scaled eigenvalue, others 0).  Inactive cells and singular systems give zero planes.
__global__ void __launch_bounds__(256) k_gn_input(const double *__restrict__ r, const unsigned short *__restrict__ code,
                                                  const double *__restrict__ shift, double lam_scale,
                                                  const int *__restrict__ singular, const int *__restrict__ sys,
                                                  long ncell, int H, int W, __nv_bfloat16 *__restrict__ x0,
                                                  float *__restrict__ rms, float *__restrict__ xf) {
  const int p = blockIdx.x, s = sys[p];
  const double *rs = r + ncell * s;
  double acc = 0.0, cnt = 0.0;
  for (long c = threadIdx.x; c < ncell; c += blockDim.x)
    if (!(code[c] & 0x8000)) { acc += rs[c] * rs[c]; cnt += 1.0; }
  double ta, tc;
  block_sum2<double>(acc, cnt, ta, tc);
  __shared__ double srms;
  if (threadIdx.x == 0) srms = (tc > 0.0 && ta > 0.0 && !singular[s]) ? sqrt(ta / tc) : 0.0;
  __syncthreads();
  const double m = srms;
  if (threadIdx.x == 0) rms[p] = (float)m;
  const float lam = (float)(shift[s] / lam_scale);
  for (long c = threadIdx.x; c < ncell; c += blockDim.x) {
    const bool live = m > 0.0 && !(code[c] & 0x8000);
    const float v = live ? (float)(rs[c] / m) : 0.f;
    if (x0) {
      const int h = (int)(c / W), w = (int)(c - (long)h * W);
      __nv_bfloat16 *o = x0 + act_idx(p, 0, h, w, H, W);
      o[0] = __float2bfloat16(v);
      o[1] = __float2bfloat16(live ? lam : 0.f);
      for (int ch = 2; ch < 8; ch++) o[ch] = __float2bfloat16(0.f);
      __nv_bfloat16 *o2 = x0 + act_idx(p, 8, h, w, H, W);
      for (int ch = 0; ch < 8; ch++) o2[ch] = __float2bfloat16(0.f);
    }
    if (xf) xf[(long)p * ncell + c] = v;
  }
}

// diagonal of system s's operator at cell c (the plane operator: shift * w01 + cc)
__device__ __forceinline__ double gn_diag(const double *shift, const double *w01, const double *cc, int s, long c) {
  return fma(shift[s], w01[c], cc[c]);
}

// trial correction of the listed systems: c = RMS(r0) D^-1 y (channel 0 of the network output) and
// x = x_prev + c (its residual gives A c)
__global__ void k_gn_corr(const float *__restrict__ y3, const float *__restrict__ rms, const int *__restrict__ sys,
                          const unsigned short *__restrict__ code, const double *__restrict__ shift,
                          const double *__restrict__ w01, const double *__restrict__ cc, long ncell,
                          const double *__restrict__ xprev, double *__restrict__ corr, double *__restrict__ x) {
  const int p = blockIdx.y, s = sys[p];
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  const long o = ncell * s + c;
  double v = 0.0;
  if (!(code[c] & 0x8000) && rms[p] != 0.f)
    v = (double)rms[p] * (double)y3[(long)p * GC * ncell + c] / gn_diag(shift, w01, cc, s, c);
  corr[o] = v;
  x[o] = xprev[o] + v;
}

// one CTA per system: with w = r0 - r1 = A c, the step alpha = <r0, w> / <w, w> minimises |r0 - alpha w|;
// x = x_prev + alpha c, and ratio = |r0 - alpha w| / |r0| (1 for a system the network does not touch)
__global__ void __launch_bounds__(256) k_gn_step(const double *__restrict__ r0, const double *__restrict__ r1,
                                                 const double *__restrict__ corr, const double *__restrict__ xprev,
                                                 const int *__restrict__ sys, const unsigned short *__restrict__ code,
                                                 long ncell, double *__restrict__ x, double *__restrict__ ratio) {
  const int p = blockIdx.x, s = sys[p];
  const long off = ncell * s;
  double rw = 0.0, ww = 0.0, rr = 0.0;
  for (long c = threadIdx.x; c < ncell; c += blockDim.x) {
    if (code[c] & 0x8000) continue;
    const double a = r0[off + c], w = a - r1[off + c];
    rw = fma(a, w, rw);
    ww = fma(w, w, ww);
    rr = fma(a, a, rr);
  }
  double trw, tww, trr;
  block_sum2<double>(rw, ww, trw, tww);
  trr = block_sum1<double>(rr);
  __shared__ double salpha;
  if (threadIdx.x == 0) {
    const double al = tww > 0.0 ? trw / tww : 0.0;
    salpha = al;
    ratio[p] = trr > 0.0 ? sqrt(fmax(0.0, trr - al * trw) / trr) : 1.0;
  }
  __syncthreads();
  const double al = salpha;
  for (long c = threadIdx.x; c < ncell; c += blockDim.x) x[off + c] = fma(al, corr[off + c], xprev[off + c]);
}

// training pair of recorded plane q: the target D (x - x_prev) / RMS(r0) and its squared norm
__global__ void __launch_bounds__(256) k_gn_target(const double *__restrict__ xnew, const double *__restrict__ xprev,
                                                   const float *__restrict__ rms, const int *__restrict__ sys,
                                                   const unsigned short *__restrict__ code, const double *__restrict__ shift,
                                                   const double *__restrict__ w01, const double *__restrict__ cc,
                                                   long ncell, float *__restrict__ tgt, float *__restrict__ tnorm) {
  const int p = blockIdx.x, s = sys[p];
  double acc = 0.0;
  const double m = rms[p];
  for (long c = threadIdx.x; c < ncell; c += blockDim.x) {
    float v = 0.f;
    if (m > 0.0 && !(code[c] & 0x8000))
      v = (float)((xnew[ncell * s + c] - xprev[ncell * s + c]) * gn_diag(shift, w01, cc, s, c) / m);
    tgt[(long)p * ncell + c] = v;
    acc += (double)v * v;
  }
  const double t = block_sum1<double>(acc);
  if (threadIdx.x == 0) tnorm[p] = (float)t;
}

// BF16 network input of recorded planes idx[0..nb) (channel 0 the stored residual, channel 1 lambda)
__global__ void k_gn_gather(const float *__restrict__ rec_x, const float *__restrict__ rec_lam, const int *__restrict__ idx,
                            long ncell, int H, int W, __nv_bfloat16 *__restrict__ x0) {
  const int p = blockIdx.y, q = idx[p];
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  const float v = rec_x[(long)q * ncell + c];
  const int h = (int)(c / W), w = (int)(c - (long)h * W);
  __nv_bfloat16 *o = x0 + act_idx(p, 0, h, w, H, W);
  o[0] = __float2bfloat16(v);
  o[1] = __float2bfloat16(v != 0.f || rec_lam[q] != 0.f ? rec_lam[q] : 0.f);
  for (int ch = 2; ch < 8; ch++) o[ch] = __float2bfloat16(0.f);
  __nv_bfloat16 *o2 = x0 + act_idx(p, 8, h, w, H, W);
  for (int ch = 0; ch < 8; ch++) o2[ch] = __float2bfloat16(0.f);
}

// loss (1/B) sum_p |y3 - t|^2 / |t|^2 per plane and its gradient on channel 0 (other channels 0)
__global__ void __launch_bounds__(256) k_gn_loss(const float *__restrict__ y3, const float *__restrict__ tgt,
                                                 const float *__restrict__ tnorm, const int *__restrict__ idx, int nb,
                                                 long ncell, float *__restrict__ d3, float *__restrict__ lpart) {
  const int p = blockIdx.x, q = idx[p];
  const float tn = tnorm[q];
  const float sc = tn > 0.f ? 2.f / ((float)nb * tn) : 0.f;
  double acc = 0.0;
  for (long c = threadIdx.x; c < ncell; c += blockDim.x) {
    const float e = y3[(long)p * GC * ncell + c] - tgt[(long)q * ncell + c];
    d3[(long)p * GC * ncell + c] = sc * e;
    for (int ch = 1; ch < GC; ch++) d3[(long)p * GC * ncell + ch * ncell + c] = 0.f;
    acc += (double)e * e;
  }
  const double t = block_sum1<double>(acc);
  if (threadIdx.x == 0) lpart[p] = tn > 0.f ? (float)(t / tn) / (float)nb : 0.f;
}

// ReLU backward in place: d *= (y > 0)
__global__ void k_gn_relu_back(float *__restrict__ d, const float *__restrict__ y, long n) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && !(y[i] > 0.f)) d[i] = 0.f;
}

// weight and bias gradients of one layer: dW[co][ci][dy][dx] = sum d[co](h,w) x[ci](h+dy-1, w+dx-1),
// db[co] = sum d[co]; one CTA per (co, ci), fixed-order block reduction
__global__ void __launch_bounds__(256) k_gn_dw(const float *__restrict__ d, const __nv_bfloat16 *__restrict__ x, int nb,
                                               int H, int W, float *__restrict__ dw, float *__restrict__ db) {
  const int co = blockIdx.x, ci = blockIdx.y;
  const long plane = (long)H * W;
  float acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  float accb = 0.f;
  for (long e = threadIdx.x; e < (long)nb * plane; e += blockDim.x) {
    const int p = (int)(e / plane);
    const long px = e - (long)p * plane;
    const int h = (int)(px / W), w = (int)(px - (long)h * W);
    const float g = d[(long)p * GC * plane + co * plane + px];
    if (g == 0.f) continue;
    accb += g;
#pragma unroll
    for (int q = 0; q < 9; q++) {
      const int hh = h + q / 3 - 1, ww = w + q % 3 - 1;
      if (hh >= 0 && hh < H && ww >= 0 && ww < W) acc[q] = fmaf(g, __bfloat162float(x[act_idx(p, ci, hh, ww, H, W)]), acc[q]);
    }
  }
  for (int q = 0; q < 9; q++) {
    const double t = block_sum1<double>((double)acc[q]);
    if (threadIdx.x == 0) dw[((co * GC + ci) * 9) + q] = (float)t;
  }
  const double tb = block_sum1<double>((double)accb);
  if (threadIdx.x == 0 && ci == 0) db[co] = (float)tb;
}

// input gradient of one layer: dx[ci](h, w) = sum_{co,dy,dx} W[co][ci][dy][dx] d[co](h-dy+1, w-dx+1)
__global__ void __launch_bounds__(256) k_gn_dx(const float *__restrict__ d, const float *__restrict__ wts, int nb,
                                               int H, int W, float *__restrict__ dx) {
  const long plane = (long)H * W;
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)nb * GC * plane) return;
  const int p = (int)(e / (GC * plane));
  const long rem = e - (long)p * GC * plane;
  const int ci = (int)(rem / plane);
  const long px = rem - (long)ci * plane;
  const int h = (int)(px / W), w = (int)(px - (long)h * W);
  float acc = 0.f;
  for (int co = 0; co < GC; co++) {
    const float *ds = d + (long)p * GC * plane + (long)co * plane;
    const float *wc = wts + (co * GC + ci) * 9;
#pragma unroll
    for (int q = 0; q < 9; q++) {  // the BF16 weights the forward multiplied with
      const int hh = h - (q / 3 - 1), ww = w - (q % 3 - 1);
      if (hh >= 0 && hh < H && ww >= 0 && ww < W)
        acc = fmaf(__bfloat162float(__float2bfloat16(wc[q])), ds[(long)hh * W + ww], acc);
    }
  }
  dx[e] = acc;
}

__global__ void k_gn_adam(float *__restrict__ w, float *__restrict__ m, float *__restrict__ v,
                          const float *__restrict__ g, int n, float lr, float b1, float b2, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  m[i] = b1 * m[i] + (1.f - b1) * gi;
  v[i] = b2 * v[i] + (1.f - b2) * gi * gi;
  w[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + 1e-8f);
}

// ---------------------------------------------------------------- host side
struct GuessNet {
  // parameters (FP32 masters), Adam moments and gradients, layer by layer: weights then biases
  float *par = nullptr, *m = nullptr, *v = nullptr, *g = nullptr;
  int adam_t = 0;
  int nplanes = 0, H = 0, W = 0;  // batch buffers for nplanes planes of H x W
  __nv_bfloat16 *xb[GL] = {};     // inputs of the layers (BF16)
  float *y[GL] = {};              // outputs (FP32)
  float *d[GL] = {};              // gradients of the outputs
  float *lpart = nullptr, *rms = nullptr;
  int *err = nullptr, *idx = nullptr;
  std::vector<void *> mem;
  void *alloc(size_t bytes) {
    void *p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, bytes);
    mem.push_back(p);
    return p;
  }
  ~GuessNet() { for (void *p : mem) cudaFree(p); }
  float *w(int l) { return par + l * (GWN + GC); }
  float *b(int l) { return par + l * (GWN + GC) + GWN; }
  float *gw(int l) { return g + l * (GWN + GC); }
  float *gbias(int l) { return g + l * (GWN + GC) + GWN; }
  static constexpr int NPAR = GL * (GWN + GC);

  int init(unsigned seed) {
    par = (float *)alloc(NPAR * 4); m = (float *)alloc(NPAR * 4); v = (float *)alloc(NPAR * 4); g = (float *)alloc(NPAR * 4);
    err = (int *)alloc(sizeof(int));
    if (!par || !m || !v || !g || !err) { set_error("device allocation failed (network)"); return SNAC_ERR_NOMEM; }
    // He-style initialisation of the weights (fan-in 9 * 16), zero biases; the last layer starts small
    std::mt19937 rng(seed);
    std::normal_distribution<float> nd(0.f, 1.f);
    std::vector<float> h(NPAR, 0.f);
    for (int l = 0; l < GL; l++) {
      const float sc = (l == GL - 1 ? 0.1f : 1.f) * std::sqrt(2.f / (9.f * GC));
      for (int i = 0; i < GWN; i++) h[l * (GWN + GC) + i] = sc * nd(rng);
    }
    SNAC_CUDA(cudaMemcpy(par, h.data(), NPAR * 4, cudaMemcpyHostToDevice));
    adam_t = 0;
    return SNAC_OK;
  }
  int ensure(int np, int h, int wd) {
    if (np <= nplanes && h == H && wd == W) return SNAC_OK;
    const long n = (long)np * GC * h * wd;
    for (int l = 0; l < GL; l++) {
      xb[l] = (__nv_bfloat16 *)alloc(n * 2);
      y[l] = (float *)alloc(n * 4);
      d[l] = (float *)alloc(n * 4);
      if (!xb[l] || !y[l] || !d[l]) { set_error("device allocation failed (network activations)"); return SNAC_ERR_NOMEM; }
    }
    lpart = (float *)alloc(np * 4);
    rms = (float *)alloc(np * 4);
    idx = (int *)alloc(np * 4);
    if (!lpart || !rms || !idx) { set_error("device allocation failed (network batch)"); return SNAC_ERR_NOMEM; }
    nplanes = np; H = h; W = wd;
    return SNAC_OK;
  }
  // forward of np planes whose BF16 input is in xb[0]; the output is y[GL-1].  Training keeps the FP32
  // outputs of every layer (the backward reads them); inference writes only the BF16 inputs of the next
  // layers and channel 0 of the last output (the correction)
  int forward(int np, bool train, cudaStream_t st) {
    for (int l = 0; l < GL; l++) {
      const bool last = l + 1 == GL;
      __nv_bfloat16 *next = last ? nullptr : xb[l + 1];
      float *out = train || last ? y[l] : nullptr;
      SNAC_TRY(launch_conv3x3_tc(xb[l], np, H, W, w(l), b(l), last ? 0 : 1, out, train ? GC : 1, next, err, st));
    }
    return SNAC_OK;
  }
  // gradients of all parameters given d[GL-1] (the loss gradient of the output)
  int backward(int np, cudaStream_t st) {
    const long n = (long)np * GC * H * W;
    for (int l = GL - 1; l >= 0; l--) {
      if (l + 1 < GL) {
        k_gn_relu_back<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d[l], y[l], n), ::snac::count_launch();
      }
      k_gn_dw<<<dim3(GC, GC), 256, 0, st>>>(d[l], xb[l], np, H, W, gw(l), gbias(l)), ::snac::count_launch();
      if (l > 0)
        k_gn_dx<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d[l], w(l), np, H, W, d[l - 1]), ::snac::count_launch();
    }
    SNAC_CUDA(cudaGetLastError());
    return SNAC_OK;
  }
  int adam(float lr, cudaStream_t st) {
    adam_t++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)adam_t), c2 = 1.f - std::pow(b2, (float)adam_t);
    k_gn_adam<<<(NPAR + 255) / 256, 256, 0, st>>>(par, m, v, g, NPAR, lr, b1, b2, c1, c2), ::snac::count_launch();
    SNAC_CUDA(cudaGetLastError());
    return SNAC_OK;
  }
  int check_err() {
    int e = 0;
    SNAC_CUDA(cudaMemcpy(&e, err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) { set_error("tensor-core accumulator wait timed out"); return SNAC_ERR_TIMEOUT; }
    return SNAC_OK;
  }
};

}  // namespace snac

using namespace snac;

// forward + backward of the network on host data (the gradient check): x nb x 16 x H x W (FP32, rounded
// to BF16), target nb x H x W, tnorm per plane, params NPAR (layer by layer: 16x16x3x3 weights, 16 biases);
// returns the loss and the gradients of every parameter
int snac_guess_grad(const float *x, const float *target, int nb, int H, int W, const float *params, float *grads,
                    double *loss) {
  if (!x || !target || !params || !grads || nb < 1 || H < 1 || W < 1) { set_error("snac_guess_grad: bad argument"); return SNAC_ERR_ARG; }
  GuessNet net;
  SNAC_TRY(net.init(1));
  SNAC_TRY(net.ensure(nb, H, W));
  const long plane = (long)H * W, n = (long)nb * GC * plane;
  SNAC_CUDA(cudaMemcpy(net.par, params, GuessNet::NPAR * 4, cudaMemcpyHostToDevice));
  std::vector<__nv_bfloat16> xb(n);
  for (int p = 0; p < nb; p++)
    for (int c = 0; c < GC; c++)
      for (int h = 0; h < H; h++)
        for (int w = 0; w < W; w++)
          xb[act_idx(p, c, h, w, H, W)] = __float2bfloat16(x[(((long)p * GC + c) * H + h) * W + w]);
  SNAC_CUDA(cudaMemcpy(net.xb[0], xb.data(), n * 2, cudaMemcpyHostToDevice));
  float *tg = (float *)net.alloc(nb * plane * 4), *tn = (float *)net.alloc(nb * 4);
  if (!tg || !tn) { set_error("device allocation failed"); return SNAC_ERR_NOMEM; }
  std::vector<float> tnh(nb, 0.f);
  for (int p = 0; p < nb; p++) {
    double s = 0.0;
    for (long c = 0; c < plane; c++) s += (double)target[p * plane + c] * target[p * plane + c];
    tnh[p] = (float)s;
  }
  SNAC_CUDA(cudaMemcpy(tg, target, nb * plane * 4, cudaMemcpyHostToDevice));
  SNAC_CUDA(cudaMemcpy(tn, tnh.data(), nb * 4, cudaMemcpyHostToDevice));
  std::vector<int> id(nb);
  for (int p = 0; p < nb; p++) id[p] = p;
  SNAC_CUDA(cudaMemcpy(net.idx, id.data(), nb * 4, cudaMemcpyHostToDevice));
  SNAC_TRY(net.forward(nb, true, 0));
  k_gn_loss<<<nb, 256>>>(net.y[GL - 1], tg, tn, net.idx, nb, plane, net.d[GL - 1], net.lpart), ::snac::count_launch();
  SNAC_TRY(net.backward(nb, 0));
  SNAC_CUDA(cudaDeviceSynchronize());
  SNAC_TRY(net.check_err());
  SNAC_CUDA(cudaMemcpy(grads, net.g, GuessNet::NPAR * 4, cudaMemcpyDeviceToHost));
  std::vector<float> lp(nb);
  SNAC_CUDA(cudaMemcpy(lp.data(), net.lpart, nb * 4, cudaMemcpyDeviceToHost));
  double L = 0.0;
  for (float v : lp) L += v;
  if (loss) *loss = L;
  return SNAC_OK;
}

// ---------------------------------------------------------------- the guess in the pressure solve
namespace snac {

struct GuessState {
  int mode = 0;  // 0 off, 1 record training pairs, 2 apply the network
  GuessNet net;
  bool net_init = false;
  long ncell = 0;
  int nsys = 0, H = 0, W = 0;
  double lam_scale = 1.0;
  double *r = nullptr, *xprev = nullptr;  // residual of x_prev, copy of x_prev (box layout, FP64)
  double *r1 = nullptr, *corr = nullptr;  // residual of the trial guess, the correction (mode 2)
  double *ratio = nullptr;                // per system: residual after the guess / before it
  float *xf = nullptr, *rms = nullptr;    // normalised residual planes and their RMS, this solve
  float *tmp_t = nullptr, *tmp_tn = nullptr;
  int *sys = nullptr;                     // 0..nsys-1
  // recorded pairs (a ring): normalised residual, target, scaled eigenvalue, |target|^2
  float *rec_x = nullptr, *rec_t = nullptr, *rec_lam = nullptr, *rec_tn = nullptr;
  int cap = 0, count = 0, next = 0;
  std::vector<float> lam_host;
  std::mt19937 rng{12345};
  // measure (mode 2): the residual after the network's correction relative to the one before it, over the
  // systems the network corrected in the last solve (median and largest)
  int measure = 0;
  double ratio_median = 0.0, ratio_max = 0.0;
  Guess3 *g3 = nullptr;  // the 3-D solve's U-Net and its recorded crops
  std::vector<void *> mem;
  void *alloc(size_t bytes) {
    void *p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    cudaMemset(p, 0, bytes);
    mem.push_back(p);
    return p;
  }
  ~GuessState() {
    guess3_destroy(g3);
    for (void *p : mem) cudaFree(p);
  }
};

void guess_destroy(GuessState *g) { delete g; }

static int guess_setup(PoissonSolver &S, GuessState &g) {
  if (g.r) return SNAC_OK;
  const MgProblem &P = S.P;
  g.ncell = P.L[0].ncell;
  g.nsys = P.nsys;
  g.W = P.L[0].n[0];
  g.H = P.L[0].n[1];
  const long nv = g.ncell * g.nsys;
  g.r = (double *)g.alloc(nv * 8);
  g.xprev = (double *)g.alloc(nv * 8);
  g.xf = (float *)g.alloc(nv * 4);
  g.rms = (float *)g.alloc(g.nsys * 4);
  g.sys = (int *)g.alloc(g.nsys * 4);
  g.tmp_t = (float *)g.alloc(nv * 4);
  g.r1 = (double *)g.alloc(nv * 8);
  g.corr = (double *)g.alloc(nv * 8);
  g.ratio = (double *)g.alloc(g.nsys * 8);
  g.tmp_tn = (float *)g.alloc(g.nsys * 4);
  g.cap = std::max(g.nsys, std::min(1024, 32 * g.nsys));
  g.rec_x = (float *)g.alloc((size_t)g.cap * g.ncell * 4);
  g.rec_t = (float *)g.alloc((size_t)g.cap * g.ncell * 4);
  g.rec_lam = (float *)g.alloc(g.cap * 4);
  g.rec_tn = (float *)g.alloc(g.cap * 4);
  if (!g.r || !g.xprev || !g.xf || !g.rms || !g.sys || !g.tmp_t || !g.tmp_tn || !g.rec_x || !g.rec_t || !g.rec_lam ||
      !g.rec_tn || !g.r1 || !g.corr || !g.ratio) {
    set_error("device allocation failed (learned guess)");
    return SNAC_ERR_NOMEM;
  }
  std::vector<int> ids(g.nsys);
  for (int q = 0; q < g.nsys; q++) ids[q] = q;
  SNAC_CUDA(cudaMemcpy(g.sys, ids.data(), g.nsys * 4, cudaMemcpyHostToDevice));
  double mx = 0.0;
  for (double v : S.lambda) mx = std::max(mx, std::fabs(v));
  g.lam_scale = mx > 0.0 ? mx : 1.0;
  g.lam_host.resize(g.nsys);
  for (int q = 0; q < g.nsys; q++) g.lam_host[q] = (float)(S.lambda[q] / g.lam_scale);
  if (!g.net_init) { SNAC_TRY(g.net.init(7)); g.net_init = true; }
  return SNAC_OK;
}

// before the solve: r0 = b - A x_prev and its normalised planes; mode 2 also moves x_prev by the guess
int guess_before(Domain &d, PoissonSolver &S, cudaStream_t st) {
  GuessState *g = d.guess;
  if (!g || g->mode == 0) return SNAC_OK;
  if (S.mode3d) {
    if (!g->g3) g->g3 = guess3_create();
    double ratio = 0.0;
    SNAC_TRY(guess3_before(S, *g->g3, g->mode, g->measure, &ratio, st));
    if (g->mode == 2 && g->measure) g->ratio_median = g->ratio_max = ratio;
    return SNAC_OK;
  }
  SNAC_TRY(guess_setup(S, *g));
  const MgProblem &P = S.P;
  const int stride = mg_partial_stride(P);
  SNAC_TRY(plane_resid<double>(P, P.shift, nullptr, S.box_x, S.box_b, g->r, S.W64.part0, nullptr, stride, st));
  SNAC_CUDA(cudaMemcpyAsync(g->xprev, S.box_x, (size_t)g->ncell * g->nsys * 8, cudaMemcpyDeviceToDevice, st));
  __nv_bfloat16 *x0 = nullptr;
  if (g->mode == 2) {
    SNAC_TRY(g->net.ensure(g->nsys, g->H, g->W));
    x0 = g->net.xb[0];
  }
  k_gn_input<<<g->nsys, 256, 0, st>>>(g->r, P.L[0].code, P.shift, g->lam_scale, P.singular, g->sys, g->ncell, g->H,
                                      g->W, x0, g->rms, g->mode == 1 ? g->xf : nullptr), ::snac::count_launch();
  if (g->mode == 2) {
    SNAC_TRY(g->net.forward(g->nsys, false, st));
    const MgLevelD &L = P.L[0];
    const dim3 ga((unsigned)((g->ncell + 255) / 256), (unsigned)g->nsys);
    k_gn_corr<<<ga, 256, 0, st>>>(g->net.y[GL - 1], g->rms, g->sys, L.code, P.shift, L.w01, L.cc, g->ncell, g->xprev,
                                  g->corr, S.box_x), ::snac::count_launch();
    SNAC_TRY(plane_resid<double>(P, P.shift, nullptr, S.box_x, S.box_b, g->r1, S.W64.part0, nullptr, stride, st));
    k_gn_step<<<g->nsys, 256, 0, st>>>(g->r, g->r1, g->corr, g->xprev, g->sys, L.code, g->ncell, S.box_x, g->ratio),
        ::snac::count_launch();
    if (g->measure) {
      std::vector<double> ratio(g->nsys), rms(g->nsys);
      std::vector<float> rmsf(g->nsys);
      SNAC_CUDA(cudaMemcpyAsync(ratio.data(), g->ratio, g->nsys * 8, cudaMemcpyDeviceToHost, st));
      SNAC_CUDA(cudaMemcpyAsync(rmsf.data(), g->rms, g->nsys * 4, cudaMemcpyDeviceToHost, st));
      SNAC_CUDA(cudaStreamSynchronize(st));
      std::vector<double> v;
      for (int q = 0; q < g->nsys; q++)
        if (rmsf[q] != 0.f) v.push_back(ratio[q]);  // singular and already-solved systems are left alone
      std::sort(v.begin(), v.end());
      g->ratio_median = v.empty() ? 0.0 : v[v.size() / 2];
      g->ratio_max = v.empty() ? 0.0 : v.back();
    }
  }
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

// after the solve (mode 1): the targets D (x - x_prev) / RMS(r0) of every system go into the ring with
// their residual planes
int guess_after(Domain &d, PoissonSolver &S, cudaStream_t st) {
  GuessState *g = d.guess;
  if (!g || g->mode != 1) return SNAC_OK;
  if (S.mode3d) return g->g3 ? guess3_after(S, *g->g3, st) : SNAC_OK;
  const MgProblem &P = S.P;
  const MgLevelD &L = P.L[0];
  k_gn_target<<<g->nsys, 256, 0, st>>>(S.box_x, g->xprev, g->rms, g->sys, L.code, P.shift, L.w01, L.cc, g->ncell,
                                       g->tmp_t, g->tmp_tn), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  int done = 0;
  while (done < g->nsys) {
    const int k = std::min(g->nsys - done, g->cap - g->next);
    const size_t pb = (size_t)g->ncell * 4;
    SNAC_CUDA(cudaMemcpyAsync(g->rec_x + (size_t)g->next * g->ncell, g->xf + (size_t)done * g->ncell, k * pb, cudaMemcpyDeviceToDevice, st));
    SNAC_CUDA(cudaMemcpyAsync(g->rec_t + (size_t)g->next * g->ncell, g->tmp_t + (size_t)done * g->ncell, k * pb, cudaMemcpyDeviceToDevice, st));
    SNAC_CUDA(cudaMemcpyAsync(g->rec_tn + g->next, g->tmp_tn + done, k * 4, cudaMemcpyDeviceToDevice, st));
    SNAC_CUDA(cudaMemcpy(g->rec_lam + g->next, g->lam_host.data() + done, k * 4, cudaMemcpyHostToDevice));
    g->next = (g->next + k) % g->cap;
    done += k;
  }
  g->count = std::min(g->cap, g->count + g->nsys);
  return SNAC_OK;
}

}  // namespace snac

namespace snac {
int guess_get_mode(const Domain &d) { return d.guess ? d.guess->mode : 0; }
void guess_set_mode(Domain &d, int mode) {
  if (d.guess) d.guess->mode = mode;
}
}  // namespace snac

int snac_guess_mode(int mode) {
  Domain *d = domain();
  if (!d) { set_error("snac_guess_mode: no domain (call snac_init first)"); return SNAC_ERR_STATE; }
  if (mode < 0 || mode > 2) { set_error("snac_guess_mode: mode must be 0, 1 or 2"); return SNAC_ERR_ARG; }
  if (!d->guess) d->guess = new GuessState();
  d->guess->mode = mode;
  return SNAC_OK;
}

int snac_guess_measure(int on, double *ratio_median, double *ratio_max) {
  Domain *d = domain();
  if (!d || !d->guess) { set_error("snac_guess_measure: the learned guess is not set up"); return SNAC_ERR_STATE; }
  d->guess->measure = on ? 1 : 0;
  if (ratio_median) *ratio_median = d->guess->ratio_median;
  if (ratio_max) *ratio_max = d->guess->ratio_max;
  return SNAC_OK;
}

int snac_guess_train(int iters, double lr, double *loss_first, double *loss_last, int *pairs) {
  Domain *d = domain();
  if (d && d->guess && d->ps->mode3d) {
    if (!d->guess->g3) { set_error("snac_guess_train: no recorded pairs"); return SNAC_ERR_STATE; }
    return guess3_train(*d->guess->g3, iters, lr, loss_first, loss_last, pairs, d->st);
  }
  if (!d || !d->guess || d->guess->count == 0) { set_error("snac_guess_train: no recorded pairs"); return SNAC_ERR_STATE; }
  GuessState &g = *d->guess;
  cudaStream_t st = d->st;
  SNAC_TRY(g.net.ensure(std::max(GB, g.nsys), g.H, g.W));
  std::uniform_int_distribution<int> pick(0, g.count - 1);
  double lf = 0.0, ll = 0.0;
  int nf = 0, nl = 0;
  const int avg = std::min(10, std::max(1, iters / 2));
  std::vector<float> lp(GB);
  for (int it = 0; it < iters; it++) {
    int ids[GB];
    for (int q = 0; q < GB; q++) ids[q] = pick(g.rng);
    SNAC_CUDA(cudaMemcpyAsync(g.net.idx, ids, sizeof(ids), cudaMemcpyHostToDevice, st));
    k_gn_gather<<<dim3((unsigned)((g.ncell + 255) / 256), GB), 256, 0, st>>>(g.rec_x, g.rec_lam, g.net.idx, g.ncell,
                                                                           g.H, g.W, g.net.xb[0]), ::snac::count_launch();
    SNAC_TRY(g.net.forward(GB, true, st));
    k_gn_loss<<<GB, 256, 0, st>>>(g.net.y[GL - 1], g.rec_t, g.rec_tn, g.net.idx, GB, g.ncell, g.net.d[GL - 1], g.net.lpart), ::snac::count_launch();
    SNAC_TRY(g.net.backward(GB, st));
    SNAC_TRY(g.net.adam((float)lr, st));
    if (it < avg || it >= iters - avg) {
      SNAC_CUDA(cudaMemcpyAsync(lp.data(), g.net.lpart, GB * 4, cudaMemcpyDeviceToHost, st));
      SNAC_CUDA(cudaStreamSynchronize(st));
      double L = 0.0;
      for (float v : lp) L += v;
      if (it < avg) { lf += L; nf++; }
      if (it >= iters - avg) { ll += L; nl++; }
    }
  }
  SNAC_CUDA(cudaStreamSynchronize(st));
  SNAC_TRY(g.net.check_err());
  if (loss_first) *loss_first = nf ? lf / nf : 0.0;
  if (loss_last) *loss_last = nl ? ll / nl : 0.0;
  if (pairs) *pairs = g.count;
  return SNAC_OK;
}
