// k_probe.cu -- arithmetic-throughput probe used as the compute roofline of the FP64 kernels.
//
// The FP64 stencils of this library are bound by the FP64 pipe on GB300, not by
// HBM; the peak they are compared with is measured here with a dependent-free
// FMA stream (8 independent chains per thread, all SMs), in FP64 and in FP32.
#include "snac_internal.h"

namespace snac {

template <typename T>
__global__ void k_fma_stream(T *out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  const T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == (T)12345.678) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains alive
}

template <typename T>
static int probe(double *gflops) {
  int dev = 0, sms = 0;
  SNAC_CUDA(cudaGetDevice(&dev));
  SNAC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int threads = 256, blocks = sms * 8, iters = 1 << 14;
  T *out = nullptr;
  SNAC_CUDA(cudaMalloc(&out, (size_t)threads * blocks * sizeof(T)));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_stream<T><<<blocks, threads>>>(out, iters / 16, (T)0.999999, (T)1e-7), ::snac::count_launch();  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 3; r++) {
    cudaEventRecord(e0);
    k_fma_stream<T><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7), ::snac::count_launch();
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = ms < best ? ms : best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaError_t e = cudaGetLastError();
  cudaFree(out);
  if (e != cudaSuccess) return cuda_fail(e, "k_fma_stream", __FILE__, __LINE__);
  *gflops = 2.0 * 8.0 * (double)iters * threads * blocks / (best * 1e-3) / 1e9;
  return SNAC_OK;
}

}  // namespace snac

extern "C" int snac_probe_peaks(double *fp64_gflops, double *fp32_gflops) {
  SNAC_TRY(snac::probe<double>(fp64_gflops));
  SNAC_TRY(snac::probe<float>(fp32_gflops));
  return SNAC_OK;
}
