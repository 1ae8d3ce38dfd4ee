// noalloc.cu -- divergence check (chkdiv.f90:8-44) that allocates no device memory.
//
// Who needs it: a driver that owns every device array itself and must not
// allocate inside its time loop -- for instance SNaC's Fortran main program
// with its fields put on the GPU once, up front, by OpenACC or CUDA Fortran data
// regions, checking the divergence every icheck steps.  The regular
// snac_chkdiv allocates a partial-sum buffer on each call; a cudaMalloc /
// cudaFree pair there synchronises the whole device and can fail outright when
// the caller has already claimed nearly all of the GPU's memory.
// snac_chkdiv_noalloc reads the caller's device arrays, returns the two
// scalars through host pointers, and keeps its only scratch -- one (sum, max)
// pair per CTA plus the final pair -- in a fixed array that lives in the
// library's own device memory.
//
// Limits and contract:
//   * scratch: SNAC_NOALLOC_CTAS = 8192 (sum, max) pairs plus one final pair,
//     128 KiB, resident on every GPU that loads the library until the process
//     exits; each CTA walks its share of the block's 32x4x2 tiles in a fixed
//     order, so any block works up to 2^31 - 1 interior cells (and 2^31 - 65
//     along one axis); larger blocks are rejected with SNAC_ERR_ARG;
//   * the first call on a device looks the array's device address up with
//     cudaGetSymbolAddress, with that device current; make the first call
//     before any stream capture begins;
//   * every call uses the same array and leaves its last results in it: calls
//     whose kernels overlap on the GPU (different streams with no ordering
//     between them) race on the array and return wrong values.
#include <mutex>

#include "snac_internal.h"

namespace snac {

namespace {

constexpr int NTX = 32, NTY = 4, NTZ = 2;      // tile of one CTA pass
constexpr int NCTA = 8192;                      // SNAC_NOALLOC_CTAS
constexpr long MAX_CELLS = 2147483647L;         // 2^31 - 1 interior cells per block
constexpr long MAX_EXTENT = 2147483647L - 64;   // cells along one axis (the 1-D metric arrays have n + 2)

static __device__ __align__(256) double g_scratch[2 * NCTA + 2];

constexpr int MAX_DEVICES = 64;
std::mutex g_mtx;
double *g_addr[MAX_DEVICES] = {nullptr};

// device address of g_scratch on the current device, looked up once per device
int scratch_address(double **out) {
  int dev = 0;
  SNAC_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= MAX_DEVICES) {
    set_error("snac_chkdiv_noalloc: device ordinal %d unsupported", dev);
    return SNAC_ERR_ARG;
  }
  std::lock_guard<std::mutex> lk(g_mtx);
  if (!g_addr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_scratch)", __FILE__, __LINE__);
    g_addr[dev] = (double *)p;
  }
  *out = g_addr[dev];
  return SNAC_OK;
}

// chkdiv.f90:24-43: CTA c accumulates tiles c, c+gridDim.x, ... (fixed order per thread)
__global__ void __launch_bounds__(NTX * NTY * NTZ)
k_chkdiv_noalloc(int nx, int ny, int nz, long tx, long ty, long ntiles, const double *__restrict__ u,
                 const double *__restrict__ v, const double *__restrict__ w, const double *__restrict__ dxf,
                 const double *__restrict__ dyf, const double *__restrict__ dzf, double rvol,
                 double *__restrict__ part) {
  const long sy = (long)nx + 2, sz = ((long)nx + 2) * ((long)ny + 2);
  double s = 0.0, m = 0.0;
  for (long t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const long bx = t % tx, by = (t / tx) % ty, bz = t / (tx * ty);
    // cell coordinates and the halo'd index in 64-bit arithmetic: an extent near 2^31 stays exact
    const long i = bx * NTX + threadIdx.x, j = by * NTY + threadIdx.y, k = bz * NTZ + threadIdx.z;
    if (i < nx && j < ny && k < nz) {
      const long c = (i + 1) + sy * (j + 1) + sz * (k + 1);
      const double div = (w[c] - w[c - sz]) / dzf[k + 1] + (v[c] - v[c - sy]) / dyf[j + 1] + (u[c] - u[c - 1]) / dxf[i + 1];
      double a = fabs(div);
      if (!(a == a)) a = __longlong_as_double(0x7ff0000000000000ll);  // NaN -> +Inf, survives fmax
      m = fmax(m, a);
      s += div * dxf[i + 1] * dyf[j + 1] * dzf[k + 1] * rvol;
    }
  }
  __shared__ double ss[NTX * NTY * NTZ / 32], sm[NTX * NTY * NTZ / 32];
  const int tid = threadIdx.x + NTX * (threadIdx.y + NTY * threadIdx.z);
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_down_sync(0xffffffffu, s, o);
    m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  }
  if ((tid & 31) == 0) { ss[tid >> 5] = s; sm[tid >> 5] = m; }
  __syncthreads();
  if (tid == 0) {
    double S = 0.0, M = 0.0;
    for (int q = 0; q < NTX * NTY * NTZ / 32; q++) { S += ss[q]; M = fmax(M, sm[q]); }
    part[2 * blockIdx.x] = S;
    part[2 * blockIdx.x + 1] = M;
  }
}

// fixed-order final pass over the CTA pairs: one warp, lane-strided then a shuffle tree
__global__ void k_chkdiv_noalloc_final(const double *__restrict__ part, int nparts, double *__restrict__ out) {
  const int l = threadIdx.x;
  double s = 0.0, m = 0.0;
  for (int q = l; q < nparts; q += 32) { s += part[2 * q]; m = fmax(m, part[2 * q + 1]); }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_down_sync(0xffffffffu, s, o);
    m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  }
  if (l == 0) { out[0] = s; out[1] = m; }
}

}  // namespace
}  // namespace snac

using namespace snac;

extern "C" int snac_chkdiv_noalloc(const int lo[3], const int hi[3], const double *dxf, const double *dyf,
                                   const double *dzf, const double *u, const double *v, const double *w, double vol,
                                   void *stream, double *divtot, double *divmax) {
  if (!lo || !hi || !dxf || !dyf || !dzf || !u || !v || !w || !divtot || !divmax) {
    set_error("snac_chkdiv_noalloc: null argument");
    return SNAC_ERR_ARG;
  }
  const long nx = (long)hi[0] - lo[0] + 1, ny = (long)hi[1] - lo[1] + 1, nz = (long)hi[2] - lo[2] + 1;
  if (nx < 1 || ny < 1 || nz < 1) {
    set_error("snac_chkdiv_noalloc: hi < lo");
    return SNAC_ERR_ARG;
  }
  if (nx > MAX_EXTENT || ny > MAX_EXTENT || nz > MAX_EXTENT || nx * ny * nz > MAX_CELLS) {
    set_error("snac_chkdiv_noalloc: block of %ld x %ld x %ld cells exceeds the limit of %ld cells (%ld along "
              "one axis); use snac_chkdiv", nx, ny, nz, MAX_CELLS, MAX_EXTENT);
    return SNAC_ERR_ARG;
  }
  const long tx = (nx + NTX - 1) / NTX, ty = (ny + NTY - 1) / NTY, tz = (nz + NTZ - 1) / NTZ;
  const long ntiles = tx * ty * tz;
  const int nparts = (int)(ntiles < NCTA ? ntiles : NCTA);
  double *scratch = nullptr;
  SNAC_TRY(scratch_address(&scratch));
  cudaStream_t st = (cudaStream_t)stream;
  k_chkdiv_noalloc<<<nparts, dim3(NTX, NTY, NTZ), 0, st>>>((int)nx, (int)ny, (int)nz, tx, ty, ntiles, u, v, w, dxf, dyf,
                                                            dzf, 1.0 / vol, scratch), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  double *fin = scratch + 2 * NCTA;
  k_chkdiv_noalloc_final<<<1, 32, 0, st>>>(scratch, nparts, fin), ::snac::count_launch();
  SNAC_CUDA(cudaGetLastError());
  double r[2];
  SNAC_CUDA(cudaMemcpyAsync(r, fin, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  SNAC_CUDA(cudaStreamSynchronize(st));
  *divtot = r[0];
  *divmax = r[1];
  return SNAC_OK;
}
