// snac_host.h -- host-side state of snac_gb300 (not part of the C ABI).
#pragma once
#include <memory>
#include <string>
#include <vector>

#include "snac_bound.h"
#include "snac_mgk.h"
#include "snac_solver.h"

namespace snac {

// device view of one host argument of a reference-signature call
struct ArgArray {
  const void *host = nullptr;
  void *dev = nullptr;
  size_t bytes = 0;
  bool owned = false, copy_out = false;
  int bind(const void *h, size_t nbytes, bool in, bool out);
  int finish();
  ~ArgArray();
};

// one block given by reference arguments (lo, hi, metric arrays)
struct OneBlock {
  DBlock hb{};
  DBlock *dblk = nullptr;
  double *dax = nullptr;
  Tile *dtiles = nullptr;
  int ntiles = 0;
  std::vector<void *> temps;
  int setup(const int lo[3], const int hi[3], const double *dxc, const double *dxf, const double *dyc,
            const double *dyf, const double *dzc, const double *dzf, bool halo_tiles);
  int upload();
  int scratch(size_t bytes, double **p);
  size_t halo_bytes() const;
  size_t interior_bytes() const;
  ~OneBlock();
};

std::vector<double> axis_tables(const double *dc, const double *df, int n);

// set-up results for one block (initmpi + initgrid + bound_grid + init_bc_rhs)
struct HostBlock {
  int ng[3], lo[3], hi[3];
  int nb[3][2], is_bound[3][2];
  snac_block_desc desc;
  std::vector<double> g[3][4];   // per axis: dc, df, c, f over lo-1..hi+1
  std::vector<double> rhsp[3];   // pressure BC planes
  std::vector<double> dl[3];     // dl(0:1,idir) of main.f90:725-727
  int inflow[3][2] = {};         // is_bound_inflow (main.f90:596)
  std::vector<double> vin[3][2][3];  // inflow planes u_in%x.. per axis, side, component over the halo'd plane
};

// the field a solver is built for: the pressure, or (IMPDIFF Helmholtz problems) velocity component c
// (HF_U + c) or scalar s (HF_S0 + s)
enum { HF_P = -1, HF_U = 0, HF_S0 = 3 };
char field_cbc(const HostBlock &H, int field, int p, int side);
double field_bc(const HostBlock &H, int field, int p, int side);
inline int field_centered(int field, int p) { return !(field >= HF_U && field < HF_S0 && field == p); }
// last solved index along p: one less at a wall along a velocity component's own direction
inline int field_hi(const HostBlock &H, int field, int p) {
  return H.hi[p] - ((!field_centered(field, p) && H.is_bound[p][1]) ? 1 : 0);
}

struct HelmBlk;  // per-block tables of a Helmholtz solver (k_helm.cu)
struct GuessState;  // the learned initial guess (k_guess.cu)
// BF16 activations of the guess network: plane p, row h, channel half c/8, pixel w, 8 channels of 2 bytes
// (each pixel's half is one 16-byte record; the tensor-core convolution reads the records as its operands)
__host__ __device__ inline long act_idx(int p, int c, int h, int w, int H, int W) {
  return ((((long)p * H + h) * 2 + (c >> 3)) * W + w) * 8 + (c & 7);
}
void guess_destroy(GuessState *g);
// the learned guess of the 3-D solve (k_unet.cu): a U-Net, crops of the solves as training pairs
struct Guess3;
// cuTensorMapEncodeTiled from the driver (k_tma.cu; null when unavailable)
void *tma_encode_fn();
Guess3 *guess3_create();
void guess3_destroy(Guess3 *g);

// the device multigrid problem plus its host-side construction data
struct PoissonSolver {
  int field = HF_P;                  // what the solver is built for
  int helm = 0;                      // Helmholtz problem: never singular, iterative coarsest level
  HelmBlk *d_hb = nullptr;           // Helmholtz solvers: per-block extents, offsets and BC planes (device)
  int mode3d = 0, ax[3] = {0, 1, 2}, periodic[3] = {0, 0, 0}, nsys = 1, lo_min[3] = {0, 0, 0};
  int fft_axis = 0, nfft = 0, kind_fwd = -1, kind_bwd = -1;
  double normfft = 1.0;
  int use_fft = 0;                   // 1: radix-2 FFT for power-of-two R2HC/HC2R; 2: mixed-radix (2, 3, 4, 5)
                                     // FFT of length nfft_c for every kind; 0: dense r2r matrices
  double *d_tw = nullptr;            // use_fft 1: FFT twiddles exp(-2 pi i k/n), k < n/2 (complex)
  double *d_gt_fwd = nullptr, *d_gt_bwd = nullptr;  // use_fft 2: tables of the forward / backward kind
  int nfft_c = 0, fft_nst = 0, fft_rad[16] = {};    // use_fft 2: complex length and its radices
  double *d_mat_fwd = nullptr, *d_mat_bwd = nullptr;  // dense r2r matrices (n x n)
  // transform line tiles (k_fft.cu), built once per solver: (block, first line) per CTA, box offsets of the
  // blocks, per block the solved extents along the two other axes (lines outside them are transformed in
  // place but not solved) and, 3-D mode, the box offsets
  int2 *d_lt = nullptr, *d_boff = nullptr;
  int2 *d_lext = nullptr;
  int4 *d_boff3 = nullptr;
  int nlt = 0, lt_lp = 0, tabs_ready = 0;
  double *invd_tab[MG_MAXLEV] = {};  // plane mode: 1/diagonal tables (remade when a Helmholtz shift changes)
  float *invd_tabf[MG_MAXLEV] = {};
  double *d_lambda = nullptr;        // Helmholtz with a transform: lambda_k / dl^2 (the shift is lambda_k + alphai)
  std::vector<double> lambda;
  int precision = 0;
  int inner_iters = 5;               // mixed path: FP32 Krylov iterations per refinement step
  int use_graph = 0;                 // mixed path: replay each refinement step's FP32 solve as a CUDA graph
  cudaGraphExec_t inner_exec = nullptr;
  long long inner_nodes = 0;         // kernel launches in that graph
  // mixed path: refinement steps run without reading the active count back, up to the number the previous
  // solve of this solver needed; each step's residual counts go to their own slot, read once at the end
  static constexpr int SPEC_MAX = 8;
  int spec_outer = 0;
  int *d_ocount = nullptr, *h_ocount = nullptr;  // 2 * SPEC_MAX ints (device, pinned host)
  double inner_tol = 1e-6;           // mixed path: relative tolerance of the FP32 solve
  int refine_steps = -1;             // mixed path: FP32 refinement steps before the systems still above the
                                     // tolerance finish with FP64 PCG (-1: FP32 refinement to convergence)
  bool adapt_inner = true;           // mixed path: each system's inner solve stops once its outer residual
                                     // would be within a tenth of the tolerance (never beyond inner_tol)
  double tol = 1e-12;
  int maxiter = 200;
  MgProblem P{};
  long ncell0 = 0, nact0 = 0;
  double *box_b = nullptr, *box_x = nullptr;  // rhs, solution / warm start (po)
  CgWork W64{}, W32{};
  int *active_outer = nullptr;
  SysScal *sc_outer = nullptr;
  double *r64 = nullptr;
  float *box_e32 = nullptr;  // FP32 correction of the mixed path
  std::vector<void *> allocs;
  int last_iters = 0;
  int last_polish = 0;               // mixed path: FP64 PCG iterations that finished the last solve
  double last_res = 0.0;
  int host_levels = 0;
  long host_coarse_cells = 0;
  ~PoissonSolver();
  void *alloc(size_t bytes);
};

struct TmaMaps;                     // tensor maps of the TMA-staged kernels (k_tma.cu)
constexpr int TMA_MAX_BLOCKS = 16;  // blocks the TMA-staged kernels take (more: the plain kernels run)

struct Domain {
  snac_case c{};
  snac_options opt{};
  int nblocks = 0;
  std::vector<HostBlock> hb;
  int periods[3] = {0, 0, 0}, is_periodic[3] = {0, 0, 0};
  double vol_all = 0.0;
  std::vector<DBlock> db;
  DBlock *d_db = nullptr;            // the block table the kernels read: d_db_set[uvw_par]
  // the momentum stage writes the new velocity into nu, nv, nw (halo'd) and the two buffers then trade places:
  // the two block tables (u, v, w and nu, nv, nw swapped) are uploaded once and uvw_par selects one
  DBlock *d_db_set[2] = {nullptr, nullptr};
  int uvw_par = 0;
  Tile *d_tiles = nullptr, *d_tiles_halo = nullptr;
  int ntiles = 0, ntiles_halo = 0;
  FaceLink *d_links[3] = {nullptr, nullptr, nullptr};
  InflowFace *d_inflow[3][2] = {};   // inflow faces per axis and side, blocks in order
  int ninflow[3][2] = {}, inflow_plane[3][2] = {};
  int nlinks[3] = {0, 0, 0}, maxplane[3] = {0, 0, 0};
  // boundary-condition tables: [kind][axis]; kinds 0 bounduvw, 1 bounduvw(is_correc), 2 p, 3 pp, 4+s scalar s
  BcEntry *d_bc[4 + SNAC_MAX_SCAL][3] = {};
  int nbc[4 + SNAC_MAX_SCAL][3] = {};
  int *d_flds = nullptr;             // field lists: [0..2] = u,v,w; [3] = p; [4] = pp; [5+s] = scalar s
  double *d_rhsp = nullptr;          // concatenated pressure BC planes
  std::vector<size_t> rhsp_off;      // per block: offsets of x,y,z planes
  double *d_part = nullptr, *d_red = nullptr, *h_red = nullptr;
  std::unique_ptr<PoissonSolver> ps;
  std::unique_ptr<PoissonSolver> hs[3 + SNAC_MAX_SCAL];  // IMPDIFF: Helmholtz solvers of u, v, w, scalars
  GuessState *guess = nullptr;       // learned initial guess of the pressure solve (off unless requested)
  TmaMaps *tma = nullptr;            // TMA-staged fillps: tensor maps, tile list, CTAs, error flag (null: n/a)
  TmaMaps *tma_alt = nullptr;        // the maps of the swapped buffers (uvw_par 1)
  int4 *tma_tiles = nullptr;
  int tma_ntiles = 0, tma_ctas = 0;
  int *tma_err = nullptr;
  double dt = 0.0, time = 0.0;
  int istep = 0;
  int last_solve_iters = 0, solves = 0;
  double last_solve_res = 0.0;
  int last_helm_iters = 0;
  double last_helm_res = 0.0;
  bool helm_not_converged = false;
  cudaStream_t st = nullptr;
  cudaStream_t st_copy = nullptr;   // second stream for batched host copies (created on first use)
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double device_ms = 0.0;
  std::vector<void *> allocs;
  void *alloc(size_t bytes);
  ~Domain();
};

Domain *domain();
int solver_create(Domain &d, PoissonSolver &S, bool upload = true, int field = HF_P);
// IMPDIFF (solve_helmholtz.f90:109-138): S.field <- solution of (A + alphai V) x = alphai V field + BC planes
int solver_solve_helmholtz(Domain &d, PoissonSolver &S, double alphai);
int helm_upload_tables(Domain &d, PoissonSolver &S, const std::vector<std::vector<double>> (&planes)[3]);
int helm_rhs(Domain &d, PoissonSolver &S, double alphai, cudaStream_t st);
int helm_shift(PoissonSolver &S, double alphai, cudaStream_t st);
int helm_io(Domain &d, PoissonSolver &S, double *box, int to_box, cudaStream_t st);
int solver_solve_pressure(Domain &d, PoissonSolver &S);
int tma_setup(Domain &d);
void tma_destroy(Domain &d);
int launch_fillps_tma(Domain &d, double dt, int *done);
int tma_check(Domain &d);
int guess_before(Domain &d, PoissonSolver &S, cudaStream_t st);
int guess_after(Domain &d, PoissonSolver &S, cudaStream_t st);
int guess3_before(PoissonSolver &S, Guess3 &g, int mode, int measure, double *ratio, cudaStream_t st);
int guess3_after(PoissonSolver &S, Guess3 &g, cudaStream_t st);
int guess3_train(Guess3 &g, int iters, double lr, double *loss_first, double *loss_last, int *pairs, cudaStream_t st);
// mode of the learned guess (0 when it was never set up); set only changes an existing guess state
int guess_get_mode(const Domain &d);
void guess_set_mode(Domain &d, int mode);

// transforms (k_fft.cu)
int fft_forward_to_box(Domain &d, PoissonSolver &S, cudaStream_t st);
int fft_backward_from_box(Domain &d, PoissonSolver &S, cudaStream_t st);
int box_gather(Domain &d, PoissonSolver &S, cudaStream_t st);
int box_scatter(Domain &d, PoissonSolver &S, cudaStream_t st);
int r2r_array(int kind, int idir, const int nn[3], int q, double *darr, cudaStream_t st);
std::vector<double> r2r_matrix(int kind, int n);
void find_fft(char a, char b, int is_centered, int *kf, int *kb, double norm[2]);
int eigenvalues(int n, char a, char b, int is_centered, double *lambda);
void initgrid(int lo, int hi, int gt, double gr, double lmin, double lmax, double *drc, double *drf, double *rc,
              double *rf);

}  // namespace snac
