// snac_internal.h -- shared device structures of snac_gb300 (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <array>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "snac_gpu.h"

namespace snac {

// every kernel launch site appends ", count_launch()" to its launch expression
void count_launch();

// Programmatic dependent launch of the solver's inner-loop kernels (snac_options.pdl; on by default): the
// launch lets the next kernel's CTAs be scheduled while this one drains, and every kernel launched this way
// calls pdl_enter() before its first access to data an earlier kernel writes (griddepcontrol.wait waits for
// the previous grid's completion and its memory), so only set-up work on constant tables overlaps.
extern int g_pdl;
// A kernel launched by launch_k waits here for the grid before it (and its memory), then lets the next one be
// scheduled; a no-op for a kernel launched without the programmatic-serialization attribute.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
template <typename... K, typename... A>
inline cudaError_t launch_k(void (*kern)(K...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, A &&...args) {
  count_launch();
  if (!g_pdl) {
    kern<<<grid, block, smem, st>>>(static_cast<K>(args)...);
    return cudaGetLastError();
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, static_cast<K>(args)...);
}

void set_error(const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what, const char *file, int line);
// SNAC_DEBUG=1 in the environment: every traced phase syncs the device and logs to stderr
void trace(const char *what, cudaStream_t st);

#define SNAC_CUDA(x)                                                      \
  do {                                                                    \
    cudaError_t e_ = (x);                                                 \
    if (e_ != cudaSuccess) return snac::cuda_fail(e_, #x, __FILE__, __LINE__); \
  } while (0)
#define SNAC_TRY(x)                  \
  do {                               \
    int r_ = (x);                    \
    if (r_ != SNAC_OK) return r_;    \
  } while (0)

// Per-axis stencil coefficients, all (n+2) long, element q+1 holds index q (q = -1..n).
// The reference divides by the spacings in every cell (mom.f90, scal.f90); here
// the divisions are hoisted into these 1-D tables so the FP64 pipe only sees
// adds and FMAs in the 3-D loops.
enum AxisArr {
  AX_DC = 0,  // d?c (centre-to-centre spacing)
  AX_DF,      // d?f (face-to-face spacing)
  AX_RC,      // 1/dc
  AX_RF,      // 1/df
  AX_A,       // 0.25/dc
  AX_E0,      // 0.25*df(q)/dc(q)
  AX_E1,      // 0.25*df(q+1)/dc(q)
  AX_SP,      // 1/(dc(q)*df(q+1))   staggered-component diffusion, + side
  AX_SM,      // 1/(dc(q)*df(q))     staggered-component diffusion, - side
  AX_CP,      // 1/(df(q)*dc(q))     centred-component diffusion, + side
  AX_CM,      // 1/(df(q)*dc(q-1))   centred-component diffusion, - side
  AX_NARR
};

struct DBlock {
  int n[3];                    // interior extents
  int lo[3];                   // global lower bounds (initmpi placement)
  double *u, *v, *w, *p, *pp;  // halo'd (n+2)^3 arrays
  double *s[SNAC_MAX_SCAL];    // halo'd scalars
  double *ru, *rv, *rw;        // RK storage dudtrko.. (interior)
  double *rs[SNAC_MAX_SCAL];   // dsdtrko (interior)
  double *nu, *nv, *nw;        // new velocity of a stage: halo'd in the domain layer (swapped with u, v, w after
                               // the stage), interior in the per-block path (written back)
  double *ns;                  // interior scratch for scalars
  const double *ax[3];         // AxisArr tables per axis: ax[a][AX_*(n+2) + q + 1]
  unsigned long long *bchk;    // bounds-check build: the flag the device checks record into (null otherwise)
};

// Bounds-check build (compiled with -DSNAC_BOUNDS_CHECK, libsnac_gb300_checked.so): kernels validate the cells
// and table entries they address against the block's extents; the first failure is recorded in the flag as
// (kernel id, i, j, k) and the access is skipped, so nothing outside an array is touched; the host turns a
// set flag into SNAC_ERR_BOUNDS.  In the normal build every check is a constant true.
enum BchkKernel { BK_TILE = 1, BK_AXIS, BK_EXCHANGE_DST, BK_EXCHANGE_SRC, BK_SETBC, BK_INFLOW, BK_PROBE, BK_NKIND };
#ifdef SNAC_BOUNDS_CHECK
__device__ inline void bchk_record(unsigned long long *f, int kid, int i, int j, int k) {
  if (!f) return;
  const unsigned long long v = (1ull << 63) | ((unsigned long long)(kid & 0x7FFF) << 48) |
                               ((unsigned long long)((i + 32768) & 0xFFFF) << 32) |
                               ((unsigned long long)((j + 32768) & 0xFFFF) << 16) | (unsigned long long)((k + 32768) & 0xFFFF);
  atomicCAS(f, 0ull, v);
}
// (i, j, k) within [lo, n_a - 1 + hi] on every axis of B
__device__ inline bool bchk(const DBlock &B, int kid, int i, int j, int k, int lo, int hi) {
  const bool ok = i >= lo && i <= B.n[0] - 1 + hi && j >= lo && j <= B.n[1] - 1 + hi && k >= lo && k <= B.n[2] - 1 + hi;
  if (!ok) bchk_record(B.bchk, kid, i, j, k);
  return ok;
}
#else
__device__ __forceinline__ bool bchk(const DBlock &, int, int, int, int, int, int) { return true; }
#endif

__host__ __device__ inline long hidx(int i, int j, int k, int nx, int ny) {
  return (long)(i + 1) + (long)(nx + 2) * ((long)(j + 1) + (long)(ny + 2) * (long)(k + 1));
}
__host__ __device__ inline long iidx(int i, int j, int k, int nx, int ny) {
  return (long)i + (long)nx * ((long)j + (long)ny * (long)k);
}
__device__ inline double AX(const DBlock &B, int a, int which, int q) {
#ifdef SNAC_BOUNDS_CHECK
  if (a < 0 || a > 2 || which < 0 || which >= AX_NARR || q < -1 || q > B.n[a]) {
    bchk_record(B.bchk, BK_AXIS, a, which, q);
    return 0.0;
  }
#endif
  return B.ax[a][which * (B.n[a] + 2) + q + 1];
}
// the library's bounds flag (null in the normal build) and its host check: SNAC_ERR_BOUNDS with the kernel and
// cell of the first failure, the flag cleared (bchk.cu)
unsigned long long *bounds_flag();
int bounds_check(cudaStream_t st);

// a tile of one block: x = block, y,z,w = i0,j0,k0 (0-based interior)
typedef int4 Tile;

struct RkMomParams {
  double f1, f2, f12;
  double bforce[3];
  double gb[3];       // f12*gacc*beta*0.5 (Boussinesq)
  double visc;
  int impdiff, boussinesq;
  int halo_out;       // 1: nu, nv, nw are halo'd (index as u); 0: interior
};

struct RkScalParams {
  double f1, f2, f12, alpha, ssource;
  int impdiff, sidx;
};

// kernel launchers (k_stencil.cu)
int launch_rk_mom(const DBlock *dB, const Tile *dT, int ntiles, const RkMomParams &prm, cudaStream_t st);
int launch_rk_mom_writeback(const DBlock *dB, const Tile *dT, int ntiles, cudaStream_t st);
// the six halo planes of u, v, w copied into nu, nv, nw (before the two trade places)
int launch_uvw_halo_copy(const DBlock *dB, int nblocks, int maxplane, cudaStream_t st);
int launch_rk_scal(const DBlock *dB, const Tile *dT, int ntiles, const RkScalParams &prm, double *part,
                   cudaStream_t st);
int launch_rk_scal_writeback(const DBlock *dB, const Tile *dT, int ntiles, int sidx, cudaStream_t st);
int launch_bulk_forcing_s(const DBlock *dB, const Tile *dT, int ntiles, int sidx, double scalf, double inv_vol,
                          const double *red, cudaStream_t st);
int launch_fillps(const DBlock *dB, const Tile *dT, int ntiles, double dt, int fft_axis, cudaStream_t st);
int launch_correc(const DBlock *dB, const Tile *dT, int ntiles, double dt, cudaStream_t st);
int launch_updt_pressure(const DBlock *dB, const Tile *dT, int ntiles, double alpha, int impdiff, cudaStream_t st);
// reductions: per-tile partials written to `part` (2 doubles per tile), then a fixed-order final pass
int launch_chkdt_partial(const DBlock *dB, const Tile *dT, int ntiles, double *part, cudaStream_t st);
int launch_chkdiv_partial(const DBlock *dB, const Tile *dT, int ntiles, double vol, double *part, cudaStream_t st);
int launch_ke_partial(const DBlock *dB, const Tile *dT, int ntiles, double *part, cudaStream_t st);
int launch_out1d(const double *f, const int n[3], int idir, const double *wa, const double *wb, double lprod,
                 double *prof, cudaStream_t st);
int launch_bulk_partial(const DBlock *dB, const Tile *dT, int ntiles, int sidx, double *part, cudaStream_t st);
int launch_updt_rhs(int nx, int ny, int nz, const int isb[6], const double *rx, const double *ry, const double *rz,
                    double *p, cudaStream_t st);
int launch_reduce_final(const double *part, int ntiles, double *out, cudaStream_t st);  // out[0]=sum part[2t], out[1]=max part[2t+1]

// tile shape of the stencil kernels
constexpr int TX = 32, TY = 4, TZ = 2;
std::vector<Tile> make_tiles(const std::vector<std::array<int, 3>> &sizes, int tx, int ty, int tz);

}  // namespace snac
