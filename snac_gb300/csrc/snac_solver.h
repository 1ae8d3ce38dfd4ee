// snac_solver.h -- batched multigrid solver and transforms (device side).
//
// The linear systems are the ones solver.f90 assembles for HYPRE
// (init_matrix_3d, init_matrix_2d + init_n_2d_matrices): all blocks placed in
// the global index space of initmpi.f90:50-103, which is the solver "box"
// (cells outside every block are inactive).  In plane mode (FFT_AXIS set) the
// box holds one 2-D system per wavenumber, stored [system][i1][i0], i0 fastest;
// in 3-D mode it holds one system [i2][i1][i0].
#pragma once
#include "snac_internal.h"

namespace snac {

constexpr int MG_MAXLEV = 16;
constexpr int MG_DENSE_MAX = 256;    // coarsest level solved with a dense inverse when it has at most this many cells
constexpr int MG_CHUNK = 256;        // cells of one system per CTA in level-0 vector kernels

// one multigrid level, device pointers; real-typed arrays exist in FP64 and FP32
struct MgLevelD {
  int n[3];
  long ncell;
  int coarsened[3];                  // axes halved from the previous (finer) level
  const unsigned short *code;        // per cell: bit 15 inactive; bits (2*(2a+s)).. fold type of face (a,s)
  const double *cc, *cp[3], *W[3];
  const float *ccf, *cpf[3], *Wf[3];
  const double *w01;                 // plane mode: W0(i) * W1(j) per cell (weight of the wavenumber shift)
  const float *w01f;
  double *x, *b, *r;                 // ncell*nsys, FP64 path
  float *xf, *bf, *rf;               // ncell*nsys, FP32 path
  double *xp;                        // plane mode: pre-smoothed x of the tiled smoother (read while x is written)
  float *xpf;
  const double *dinv;                // coarsest: ncell^2 per system
  const float *dinvf;
  const double *invd;                // plane mode: 1 / diagonal per system and cell (0 for inactive cells)
  const float *invdf;
  // 3-D mode, FP32 V-cycles (MgProblem::sep): the couplings are products of 1-D factors, cp[a] of an unfolded
  // face between cells q and q+1 along a = caf[a][q] * Wf[b][q_b] * Wf[c][q_c] (b, c the other axes)
  const float *caf[3];
};

struct MgProblem {
  int mode3d;
  int periodic[3];
  int nsys;
  int nlev;
  int nu;                            // smoothing sweeps per side on levels < lnu
  int nu_coarse;                     // and on levels >= lnu
  int lnu;
  MgLevelD L[MG_MAXLEV];
  const double *shift;               // per system (lambda_k), device
  const float *shiftf;
  const int *singular;               // per system, device
  int fused;                         // bits: 1/4 tiled plane smoother FP32/FP64, 2/8 one-CTA coarse tail FP32/FP64
  int cta_level[2];                  // first level run by k_vcycle_coarse / k_vcycle_coarse3d ([0] FP32, [1] FP64); nlev = none
  int nsm;                           // multiprocessors of the device (sizes the system batches)
  int tile_shape;                    // FP32 smoother tile: 0 auto, 1..4 = 8x2, 8x3, 16x2, 16x3 (warps x rows)
  int tile_inv;                      // FP32 tiled smoother: 1 / diagonal formed in registers instead of read
  int tile_restrict;                 // FP32 tiled pre-smoother also restricts its residual (no separate pass)
  int waves;                         // waves of CTAs per batched plane launch
  int red_batch;                     // the reducing plane kernels batch systems (0: one system per CTA)
  int any_singular;                  // some system is singular (pure Neumann, zero shift)
  const int *sing_list;              // device: indices of the singular systems (nsing of them)
  int nsing;
  long nact0;                        // active cells of one system on level 0
  int sep;                           // 3-D mode: every level's couplings factor into 1-D tables (caf), which the
                                     // FP32 V-cycle and Krylov kernels use instead of the per-cell arrays
};
// smoothing sweeps per side of the V-cycle on level l
__host__ __device__ inline int mg_nu(const MgProblem &P, int l) { return l >= P.lnu ? P.nu_coarse : P.nu; }


struct MgGeom;
// fused kernels (k_mg_fused.cu)
bool tile2d_ok(const MgProblem &P, int l, int prec);
bool tile2d_geometry_ok(const MgProblem &P, int l);  // tile2d_ok before the level's arrays exist
int tile2d_max_parts(const MgLevelD &L);
int tile2d_shape_index(const MgProblem &P, int l);
// part_bx: partials of b.x of the stored cells (post-smoother, mode 1); for the singular systems also those
// of x and of b in part_x and part_b
template <typename T>
int launch_rbgs_tile2d(const MgProblem &P, int l, const int *active, int first_color, int mode, T *x, const T *b,
                       const T *xin, const T *xc, double *part_bx, double *part_x, double *part_b, int part_stride,
                       int *nchunk, cudaStream_t st);
// FP32 pre-smoother of level l (xp out) that also writes the restricted residual bc of level l + 1 and, when
// xcz is given, zeroes that level's x (the separate restriction pass folded in; the same values)
template <typename T>
int launch_rbgs_tile2d_restrict(const MgProblem &P, int l, const int *active, T *xp, const T *b, T *bc, T *xcz,
                                cudaStream_t st);
template <typename T>
size_t coarse_smem_bytes(const MgProblem &P, int l0);
struct MgGeom;
template <typename T>
size_t coarse3d_smem_bytes(const MgProblem &P, int l0);
template <typename T>
int launch_vcycle_coarse3d(const MgProblem &P, const MgGeom &G, int l0, const T *shift, const int *active, T *x,
                           const T *b, cudaStream_t st);
// dynamic shared memory of the one-CTA coarse V-cycles (227 KB at most per CTA): the plane kernel keeps 8 KB
// of static shared memory for its dense coarsest solve, the 3-D kernel a few bytes
constexpr size_t MG_SMEM_OPT_IN = 226 * 1024;      // opt-in limit set on every kernel that needs more than 48 KB
constexpr size_t MG_COARSE_SMEM_MAX = 218 * 1024;
constexpr size_t MG_COARSE3D_SMEM_MAX = 226 * 1024;
// 3-D mode, default start of the one-CTA coarse V-cycle: the finest level of at most this many cells (about
// four per thread); a finer level is swept faster by the level-by-level kernels, which spread over the GPU
// (L-shaped box 288 x 288 x 96: 65.8 ms per step from its 1,944-cell level, 71.7 ms from the 15,552-cell one)
constexpr long MG_COARSE3D_CELLS = 4096;
template <typename T>
int launch_vcycle_coarse(const MgProblem &P, int l0, const T *shift, const int *active, T *x, const T *b,
                         cudaStream_t st);

// plane-mode kernels batched over systems (k_mg_plane.cu)
int plane_batch(const MgProblem &P, long ctas_per_system, int per_sm);
int plane_nchunk(const MgLevelD &L);
int plane_resid_nchunk(const MgLevelD &L, int prec);
template <typename T> int plane_sweep(const MgProblem &P, int l, const T *shift, const int *active, int color, T *x,
                                      const T *b, cudaStream_t st);
template <typename T> int plane_restrict(const MgProblem &P, int l, const T *shift, const int *active, const T *xf,
                                         const T *bf, T *bc, T *xc, cudaStream_t st);
template <typename T> int plane_prolong(const MgProblem &P, int l, const int *active, T *xf, const T *xc,
                                        cudaStream_t st);
int plane_make_invd(MgProblem &P, double *const *out, float *const *outf, cudaStream_t st);

// kernels (k_mg.cu) -- T = double or float
template <typename T> int mg_vcycle(const MgProblem &P, int l, const int *active, cudaStream_t st);
int mg_set_active(int nsys, int *active, const int *src, cudaStream_t st);
int mg_partial_stride(const MgProblem &P);  // capacity of one system's row of partial sums

}  // namespace snac
