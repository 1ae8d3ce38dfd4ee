// k_cnn.cu -- dense 3x3 convolutions on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// The convolution of a 16-channel BF16 image with 16 output channels is an implicit GEMM per CTA:
// 128 pixels of one image row (M = 128) times K = 9 x 16 (the 3x3 taps of 16 channels) times N = 16.
// The CTA builds the nine 128 x 16 A blocks (im2col of its pixels) and the nine 16 x 16 B blocks (the
// weights of one tap) in shared memory in the no-swizzle K-major core-matrix layout (8 rows x 16 bytes
// per core matrix), one thread issues the nine tcgen05.mma.kind::f16 (BF16 inputs, FP32 accumulation)
// into a 128-lane x 16-column TMEM accumulator, tcgen05.commit signals an mbarrier, and every warp
// reads its 32 lanes back with tcgen05.ld for the epilogue (bias, optional ReLU).  The wait on the
// mbarrier has an iteration limit; past it the kernel records an error and returns without reading TMEM.
#include <cuda_bf16.h>

#include <cstdint>
#include <vector>

#include "snac_host.h"

namespace snac {

namespace {

constexpr int CNN_C = 16;        // channels in and out of a tensor-core layer
constexpr int CNN_M = 128;       // pixels per CTA (one row segment)
constexpr int CNN_TAPS = 9;
constexpr uint32_t TMEM_COLS = 32;  // allocation unit (power of two >= 32); 16 columns are used

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor (tcgen05): start >> 4, leading-dimension (K) byte offset >> 4, stride
// (M/N) byte offset >> 4, descriptor version 1 at bit 46, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both K-major, N >> 3, M >> 4
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// byte offset of element (row r, k) in a rows x 16 K-major block of core matrices: core (r/8, k/8) at
// ((r/8) * 2 + k/8) * 128, row r%8 at 16 bytes, element k%8 at 2 bytes (LBO 128, SBO 256)
__device__ __forceinline__ int core_off(int r, int k) { return (((r >> 3) * 2 + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1); }

}  // namespace

// y[p][co][h][w] = act(bias[co] + sum_{ci,dy,dx} w[co][ci][dy][dx] x[p][ci][h+dy-1][w+dx-1]) with zero
// padding; x BF16, weights given in FP32 and rounded to BF16 here; y FP32 for the first ny output channels
// (none when y is null) and the BF16 copy of all 16 when yb
__global__ void __launch_bounds__(CNN_M) k_conv3x3_tc(const __nv_bfloat16 *__restrict__ x, int H, int W,
                                                      const float *__restrict__ wts, const float *__restrict__ bias,
                                                      int relu, float *__restrict__ y, int ny,
                                                      __nv_bfloat16 *__restrict__ yb, int *__restrict__ err) {
  __shared__ __align__(128) unsigned char sa[CNN_TAPS * CNN_M * CNN_C * 2];  // 36 KB of A blocks
  __shared__ __align__(128) unsigned char sb[CNN_TAPS * CNN_C * CNN_C * 2];  // 4.5 KB of B blocks
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int w0 = blockIdx.x * CNN_M, h = blockIdx.y, p = blockIdx.z;
  const long plane = (long)H * W;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&mbar)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  // B blocks: tap q = dy*3+dx, row n = output channel, k = input channel
  for (int e = t; e < CNN_TAPS * CNN_C * CNN_C; e += CNN_M) {
    const int k = e % CNN_C, n = (e / CNN_C) % CNN_C, q = e / (CNN_C * CNN_C);
    const float wv = wts[((n * CNN_C + k) * 3 + q / 3) * 3 + q % 3];
    *reinterpret_cast<__nv_bfloat16 *>(sb + q * (CNN_C * CNN_C * 2) + core_off(n, k)) = __float2bfloat16(wv);
  }
  __syncthreads();
  // A blocks: thread t fills row t (pixel w0 + t) of every tap, zero outside the image
  for (int q = 0; q < CNN_TAPS; q++) {
    const int hh = h + q / 3 - 1, ww = w0 + t + q % 3 - 1;
    const bool in = hh >= 0 && hh < H && ww >= 0 && ww < W;
    unsigned char *blk = sa + q * (CNN_M * CNN_C * 2);
    for (int c = 0; c < CNN_C; c++) {
      const __nv_bfloat16 v = in ? x[(long)p * CNN_C * plane + (long)c * plane + (long)hh * W + ww] : __float2bfloat16(0.f);
      *reinterpret_cast<__nv_bfloat16 *>(blk + core_off(t, c)) = v;
    }
  }
  // the operands were written by the generic proxy and are read by the tensor core (async proxy)
  asm volatile("fence.proxy.async.shared::cta;");
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t dtmem = tmem_base;
  if (t == 0) {
    constexpr uint32_t idesc = idesc_bf16(CNN_M, CNN_C);
    for (int q = 0; q < CNN_TAPS; q++) {
      const uint64_t ad = smem_desc(smem_u32(sa + q * (CNN_M * CNN_C * 2)), 128, 256);
      const uint64_t bd = smem_desc(smem_u32(sb + q * (CNN_C * CNN_C * 2)), 128, 256);
      const uint32_t acc = q > 0 ? 1u : 0u;
      asm volatile(
          "{\n .reg .pred pa;\n setp.ne.b32 pa, %4, 0;\n"
          " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, pa;\n}\n" ::"r"(dtmem),
          "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(&mbar)));
  }
  // bounded wait for the accumulator (phase 0)
  uint32_t done = 0;
  for (long it = 0; it < (1L << 24) && !done; it++) {
    asm volatile(
        "{\n .reg .pred pw;\n mbarrier.try_wait.parity.shared::cta.b64 pw, [%1], %2;\n selp.u32 %0, 1, 0, pw;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(&mbar)), "r"(0));
  }
  asm volatile("tcgen05.fence::after_thread_sync;");
  done = __all_sync(0xffffffffu, done);  // tcgen05.ld is warp-collective
  if (done) {
    uint32_t r[16];
    const uint32_t taddr = dtmem + ((uint32_t)(warp * 32) << 16);
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
    const int m = warp * 32 + lane, ww = w0 + m;
    if (ww < W) {
      for (int n = 0; n < CNN_C; n++) {
        float v = __uint_as_float(r[n]) + bias[n];
        if (relu) v = fmaxf(v, 0.f);
        const long o = (long)p * CNN_C * plane + (long)n * plane + (long)h * W + ww;
        if (y && n < ny) y[o] = v;
        if (yb) yb[o] = __float2bfloat16(v);
      }
    }
  } else if (lane == 0) {
    atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(dtmem), "r"(TMEM_COLS));
}

int launch_conv3x3_tc(const __nv_bfloat16 *x, int nplanes, int H, int W, const float *wts, const float *bias, int relu,
                      float *y, int ny, __nv_bfloat16 *yb, int *err, cudaStream_t st) {
  const dim3 g((unsigned)((W + CNN_M - 1) / CNN_M), (unsigned)H, (unsigned)nplanes);
  k_conv3x3_tc<<<g, CNN_M, 0, st>>>(x, H, W, wts, bias, relu, y, ny, yb, err), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  return SNAC_OK;
}

}  // namespace snac

using namespace snac;

// test entry: one layer on host arrays (x: nplanes x 16 x H x W FP32, rounded to BF16 on the way in)
int snac_cnn_conv3x3(const float *x, int nplanes, int H, int W, const float *wts, const float *bias, int relu,
                     float *y) {
  if (!x || !wts || !bias || !y || nplanes < 1 || H < 1 || W < 1) { set_error("snac_cnn_conv3x3: bad argument"); return SNAC_ERR_ARG; }
  const size_t n = (size_t)nplanes * 16 * H * W;
  std::vector<__nv_bfloat16> xb(n);
  for (size_t i = 0; i < n; i++) xb[i] = __float2bfloat16(x[i]);
  __nv_bfloat16 *dx = nullptr;
  float *dw = nullptr, *db = nullptr, *dy = nullptr;
  int *derr = nullptr;
  int rc = SNAC_OK;
  auto fail = [&](const char *what) { set_error("snac_cnn_conv3x3: %s", what); rc = SNAC_ERR_CUDA; };
  if (cudaMalloc(&dx, n * 2) != cudaSuccess || cudaMalloc(&dw, 16 * 16 * 9 * 4) != cudaSuccess ||
      cudaMalloc(&db, 16 * 4) != cudaSuccess || cudaMalloc(&dy, n * 4) != cudaSuccess ||
      cudaMalloc(&derr, sizeof(int)) != cudaSuccess) {
    fail("device allocation failed");
  } else {
    cudaMemcpy(dx, xb.data(), n * 2, cudaMemcpyHostToDevice);
    cudaMemcpy(dw, wts, 16 * 16 * 9 * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(db, bias, 16 * 4, cudaMemcpyHostToDevice);
    cudaMemset(derr, 0, sizeof(int));
    rc = launch_conv3x3_tc(dx, nplanes, H, W, dw, db, relu, dy, CNN_C, nullptr, derr, 0);
    if (rc == SNAC_OK) {
      if (cudaDeviceSynchronize() != cudaSuccess) fail(cudaGetErrorString(cudaGetLastError()));
      else {
        int e = 0;
        cudaMemcpy(&e, derr, sizeof(int), cudaMemcpyDeviceToHost);
        if (e) { set_error("snac_cnn_conv3x3: tensor-core accumulator wait timed out"); rc = SNAC_ERR_TIMEOUT; }
        else cudaMemcpy(y, dy, n * 4, cudaMemcpyDeviceToHost);
      }
    }
  }
  cudaFree(dx); cudaFree(dw); cudaFree(db); cudaFree(dy); cudaFree(derr);
  return rc;
}
