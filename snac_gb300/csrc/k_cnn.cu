// k_cnn.cu -- dense 3x3 convolutions on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// The convolution of a 16-channel BF16 image with 16 output channels is an implicit GEMM per row segment:
// 128 pixels of one image row (M = 128) times K = 9 x 16 (the 3x3 taps of 16 channels) times N = 16.
// Activations are stored per row as two 8-channel halves of 16-byte pixel records (act_idx), so the three
// input rows a segment needs, staged in shared memory with 16-byte loads, already are the A operands of
// the nine taps in the no-swizzle K-major core-matrix layout: a tap's horizontal offset is a 16-byte
// offset of the descriptor's start address (rows of a core matrix are consecutive pixels, 16 bytes
// apart; the two K halves are one staged half-row apart).  The weights (B, 16 x 16 per tap) are converted
// to BF16 once per CTA; the CTAs are persistent and loop over row segments with one TMEM accumulator
// (128 lanes x 16 columns), one elected thread issuing the nine tcgen05.mma.kind::f16 (BF16 inputs, FP32
// accumulation) and tcgen05.commit signalling an mbarrier whose phase alternates per segment.  Every warp
// reads its 32 lanes back with tcgen05.ld for the epilogue (bias, optional ReLU).  The mbarrier wait has
// an iteration limit; past it the kernel records an error, waits (bounded) for the MMAs in flight, frees
// its TMEM and returns.
#include <cuda_bf16.h>

#include <algorithm>
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
// padding; x BF16 in the act_idx layout, weights given in FP32 and rounded to BF16 here; y FP32 (planar
// [p][co][h][w]) for the first ny output channels (none when y is null) and yb BF16 (act_idx) of all 16
constexpr int CNN_ROW = (CNN_M + 2) * 16;  // bytes of one staged half-row (130 pixel records)

constexpr long MBAR_POLLS = 1L << 24;  // polls of an mbarrier wait before it gives up

__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, long limit) {
  uint32_t done = 0;
  for (long it = 0; it < limit && !done; it++) {
    asm volatile(
        "{\n .reg .pred pw;\n mbarrier.try_wait.parity.shared::cta.b64 pw, [%1], %2;\n selp.u32 %0, 1, 0, pw;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity));
  }
  return done != 0;
}

__global__ void __launch_bounds__(CNN_M) k_conv3x3_tc(const __nv_bfloat16 *__restrict__ x, int np, int H, int W,
                                                      const float *__restrict__ wts, const float *__restrict__ bias,
                                                      int relu, float *__restrict__ y, int ny,
                                                      __nv_bfloat16 *__restrict__ yb, int *__restrict__ err,
                                                      long poll_limit) {
  __shared__ __align__(128) unsigned char sa[3 * 2 * CNN_ROW];               // 12.2 KB: rows h-1..h+1, halves
  __shared__ __align__(128) unsigned char sb[CNN_TAPS * CNN_C * CNN_C * 2];  // 4.5 KB of B blocks
  __shared__ float sbias[CNN_C];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&mbar)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  // B blocks: tap q = dy*3+dx, row n = output channel, k = input channel (K-major core matrices)
  for (int e = t; e < CNN_TAPS * CNN_C * CNN_C; e += CNN_M) {
    const int k = e % CNN_C, n = (e / CNN_C) % CNN_C, q = e / (CNN_C * CNN_C);
    const float wv = wts[((n * CNN_C + k) * 3 + q / 3) * 3 + q % 3];
    *reinterpret_cast<__nv_bfloat16 *>(sb + q * (CNN_C * CNN_C * 2) + core_off(n, k)) = __float2bfloat16(wv);
  }
  if (t < CNN_C) sbias[t] = bias[t];
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t dtmem = tmem_base, bar = smem_u32(&mbar);
  const int nseg = (W + CNN_M - 1) / CNN_M;
  const long total = (long)np * H * nseg;
  uint32_t phase = 0;
  bool failed = false;
  for (long seg = blockIdx.x; seg < total; seg += gridDim.x) {
    const int ws = (int)(seg % nseg);
    const long ph = seg / nseg;
    const int h = (int)(ph % H), p = (int)(ph / H);
    const int w0 = ws * CNN_M;
    // stage rows h-1, h, h+1 (zero outside the image): 3 x 2 halves x 130 records of 16 bytes
    for (int e = t; e < 3 * 2 * (CNN_M + 2); e += CNN_M) {
      const int r = e / (2 * (CNN_M + 2)), rem = e - r * 2 * (CNN_M + 2);
      const int kh = rem / (CNN_M + 2), q = rem - kh * (CNN_M + 2);
      const int hh = h + r - 1, ww = w0 - 1 + q;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (hh >= 0 && hh < H && ww >= 0 && ww < W) v = *reinterpret_cast<const uint4 *>(x + act_idx(p, kh * 8, hh, ww, H, W));
      *reinterpret_cast<uint4 *>(sa + (r * 2 + kh) * CNN_ROW + q * 16) = v;
    }
    // the operands were written by the generic proxy and are read by the tensor core (async proxy)
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (t == 0) {
      constexpr uint32_t idesc = idesc_bf16(CNN_M, CNN_C);
      for (int q = 0; q < CNN_TAPS; q++) {
        const int dy = q / 3, dx = q % 3;
        // pixel rows 16 bytes apart (8-row core matrices 128 B apart), K halves one staged half-row apart
        const uint64_t ad = smem_desc(smem_u32(sa + dy * 2 * CNN_ROW + dx * 16), CNN_ROW, 128);
        const uint64_t bd = smem_desc(smem_u32(sb + q * (CNN_C * CNN_C * 2)), 128, 256);
        const uint32_t acc = q > 0 ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred pa;\n setp.ne.b32 pa, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, pa;\n}\n" ::"r"(dtmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar));
    }
    const bool got = mbar_wait_bounded(bar, phase, poll_limit);
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (!__syncthreads_and(got ? 1 : 0)) {  // the accumulator did not arrive in time
      if (t == 0) atomicExch(err, 1);
      failed = true;
      break;
    }
    phase ^= 1u;
    uint32_t rr[16];
    const uint32_t taddr = dtmem + ((uint32_t)(warp * 32) << 16);
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(rr[0]), "=r"(rr[1]), "=r"(rr[2]), "=r"(rr[3]), "=r"(rr[4]), "=r"(rr[5]), "=r"(rr[6]), "=r"(rr[7]),
          "=r"(rr[8]), "=r"(rr[9]), "=r"(rr[10]), "=r"(rr[11]), "=r"(rr[12]), "=r"(rr[13]), "=r"(rr[14]), "=r"(rr[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
    const int ww = w0 + warp * 32 + lane;
    if (ww < W) {
      float v[CNN_C];
#pragma unroll
      for (int n = 0; n < CNN_C; n++) {
        v[n] = __uint_as_float(rr[n]) + sbias[n];
        if (relu) v[n] = fmaxf(v[n], 0.f);
      }
      if (yb) {
#pragma unroll
        for (int kh = 0; kh < 2; kh++) {
          __align__(16) __nv_bfloat16 o[8];
#pragma unroll
          for (int c = 0; c < 8; c++) o[c] = __float2bfloat16(v[kh * 8 + c]);
          *reinterpret_cast<uint4 *>(yb + act_idx(p, kh * 8, h, ww, H, W)) = *reinterpret_cast<const uint4 *>(o);
        }
      }
      if (y) {
        const long plane = (long)H * W;
        for (int n = 0; n < ny && n < CNN_C; n++) y[((long)p * CNN_C + n) * plane + (long)h * W + ww] = v[n];
      }
    }
    // the next segment's MMAs overwrite the accumulator after the barrier that follows its staging
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();  // every thread has finished with the staged rows and the accumulator
  }
  // let the MMAs in flight finish before freeing TMEM: always the full bound, whatever the main wait's limit
  if (failed) mbar_wait_bounded(bar, phase, MBAR_POLLS);
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(dtmem), "r"(TMEM_COLS));
}

// polls of the accumulator wait in the launches that follow (snac_cnn_set_poll_limit; testing only)
static long g_poll_limit = MBAR_POLLS;

int launch_conv3x3_tc(const __nv_bfloat16 *x, int nplanes, int H, int W, const float *wts, const float *bias, int relu,
                      float *y, int ny, __nv_bfloat16 *yb, int *err, cudaStream_t st) {
  int dev = 0, nsm = 0;  // the current device's multiprocessors (an attribute query, no synchronisation)
  SNAC_CUDA(cudaGetDevice(&dev));
  SNAC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const long total = (long)nplanes * H * ((W + CNN_M - 1) / CNN_M);
  const int grid = (int)std::min<long>(total, (long)nsm * 8);  // persistent CTAs, 8 per SM
  k_conv3x3_tc<<<grid, CNN_M, 0, st>>>(x, nplanes, H, W, wts, bias, relu, y, ny, yb, err, g_poll_limit),
      ::snac::count_launch();
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
  for (int p = 0; p < nplanes; p++)
    for (int c = 0; c < 16; c++)
      for (int h = 0; h < H; h++)
        for (int w = 0; w < W; w++)
          xb[act_idx(p, c, h, w, H, W)] = __float2bfloat16(x[(((size_t)p * 16 + c) * H + h) * W + w]);
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

int snac_cnn_set_poll_limit(long polls) {
  snac::g_poll_limit = polls < 0 ? snac::MBAR_POLLS : polls;
  return SNAC_OK;
}
