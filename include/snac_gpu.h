/*
 * snac_gpu.h -- C ABI of snac_gb300, a GB300 (sm_103a) implementation of
 * SNaC's per-time-step hot path.
 *
 * Every entry point is plain C (extern "C", pointers and sizes, no C++ or
 * torch types) so that SNaC's Fortran driver can bind it with
 * iso_c_binding.  Each declaration names the reference interface it replaces
 * (paths relative to the SNaC source tree).
 *
 * Two layers:
 *   1. Reference-signature calls (snac_rk_mom, snac_fillps, ...): the same
 *      argument lists as the Fortran subroutines, one block at a time, on the
 *      caller's host arrays.  Arrays registered with snac_register() are used
 *      through their device mirror without copies; unregistered arrays are
 *      copied to the device and back around the call.
 *   2. Domain calls (snac_init, snac_*_all, snac_step): all blocks of a case
 *      resident in HBM, the block-to-block halo exchange done on the device,
 *      the Poisson solve, and whole RK3 steps driven by the library.
 *
 * Array conventions follow the reference's Fortran declarations:
 *   halo'd field   f(lo(1)-1:hi(1)+1, lo(2)-1:hi(2)+1, lo(3)-1:hi(3)+1), x fastest;
 *   RK storage     dudtrko(lo(1):hi(1), lo(2):hi(2), lo(3):hi(3));
 *   1-D metrics    dxc(lo(1)-1:hi(1)+1), passed as a pointer to element lo(1)-1;
 *   BC planes      rhsx(lo(2):hi(2),lo(3):hi(3),0:1), rhsy(lo(1):hi(1),lo(3):hi(3),0:1),
 *                  rhsz(lo(1):hi(1),lo(2):hi(2),0:1);
 *   logical(0:1,3) arguments are int[3][2] (side fastest), 0 = .false.
 *
 * Errors: every function returns SNAC_OK (0) or one of the SNAC_ERR_* codes;
 * snac_last_error() returns a message for the last failure.  There is no CPU
 * fallback: without a usable CUDA device the calls fail with SNAC_ERR_CUDA.
 */
#ifndef SNAC_GPU_H
#define SNAC_GPU_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

#define SNAC_MAX_SCAL 4

enum {
  SNAC_OK = 0,
  SNAC_ERR_ARG = 1,            /* invalid argument or inconsistent input */
  SNAC_ERR_CUDA = 2,           /* CUDA runtime error (no device, launch failure, ...) */
  SNAC_ERR_NOT_CONVERGED = 3,  /* a Poisson/Helmholtz solve hit maxiter above tolerance */
  SNAC_ERR_NAN = 4,            /* NaN/Inf detected in a reduction */
  SNAC_ERR_TIMEOUT = 5,        /* a bounded device-side wait gave up */
  SNAC_ERR_BOUNDS = 6,         /* a device-side bounds check fired */
  SNAC_ERR_STATE = 7,          /* call out of order (e.g. snac_step before snac_init) */
  SNAC_ERR_UNSUPPORTED = 8,    /* input the library does not implement */
  SNAC_ERR_NOMEM = 9,          /* device allocation failed */
  SNAC_ERR_IO = 10             /* a checkpoint file could not be opened, read or written, or has the wrong size */
};

/* field identifiers for the domain layer */
enum {
  SNAC_U = 0, SNAC_V = 1, SNAC_W = 2, SNAC_P = 3, SNAC_PP = 4, SNAC_PO = 5,
  SNAC_DUDTRKO = 6, SNAC_DVDTRKO = 7, SNAC_DWDTRKO = 8,
  SNAC_S0 = 9,                       /* scalar s: SNAC_S0 + s, s < SNAC_MAX_SCAL */
  SNAC_DSDTRKO0 = 20                 /* scalar RK storage: SNAC_DSDTRKO0 + s */
};

/* grid arrays for snac_get_grid */
enum { SNAC_G_DXC = 0, SNAC_G_DXF = 1, SNAC_G_XC = 2, SNAC_G_XF = 3 };

/* r2r transform kinds, FFTW's unnormalised definitions (fftw.f90:9-29) */
enum { SNAC_R2HC = 0, SNAC_HC2R = 1, SNAC_REDFT00 = 3, SNAC_REDFT01 = 4, SNAC_REDFT10 = 5,
       SNAC_REDFT11 = 6, SNAC_RODFT00 = 7, SNAC_RODFT01 = 8, SNAC_RODFT10 = 9, SNAC_RODFT11 = 10 };

/* One entry of the &blocks namelist (param.f90:332-360, docs/INFO_INPUT.md).
 * cbcvel[comp][dir][side] = block_cbcvel(side,dir,comp,ib); a friend link 'F'
 * carries the 1-based id of the neighbouring block in the value array. */
typedef struct snac_block_desc {
  int    ng[3];
  double lmin[3], lmax[3];
  int    gt[3];
  double gr[3];
  char   cbcvel[3][3][2];
  double bcvel[3][3][2];
  char   cbcpre[3][2];
  double bcpre[3][2];
  char   cbcscal[SNAC_MAX_SCAL][3][2];
  double bcscal[SNAC_MAX_SCAL][3][2];
  const double *grid_file[3];  /* optional grid/grid_?_b_###.bin: rf,rc,drf,drc over lo..hi (4*ng) */
  int    inflow_type[3][2];    /* block_inflow_type (param.f90:84): 0 none, 1 Poiseuille, 2 Kovasznay; active on a
                                  physical boundary whose normal velocity component is 'D' (main.f90:596) */
} snac_block_desc;

/* &dns, &scalar and &hypre namelists (param.f90:342-355) plus the build flags */
typedef struct snac_case {
  int    nblocks;
  double visci, cfl, dtmax, dt_f;
  double bforce[3], gacc[3], beta;
  int    nscal;
  double alphai[SNAC_MAX_SCAL], ssource[SNAC_MAX_SCAL], scalf[SNAC_MAX_SCAL];
  int    is_sforced[SNAC_MAX_SCAL];
  int    icheck;
  int    fft_axis;    /* 0: 3-D solve; 1,2,3: FFT_AXIS (transform along x/y/z) */
  int    impdiff;     /* _IMPDIFF */
  int    boussinesq;  /* _BOUSSINESQ_BUOYANCY */
  double tol;         /* relative residual ||r||/||b|| of every solve (hypre_tol) */
  int    maxiter;     /* iteration cap of every solve (hypre_maxiter) */
} snac_case;

/* Library options with no counterpart in the reference. */
typedef struct snac_options {
  int precision;      /* 0: FP64 multigrid-preconditioned CG; 1: FP32 V-cycles inside FP64 iterative refinement */
  int use_graph;      /* 1: replay each mixed-precision refinement step (FP32 PCG with its V-cycles) as a
                         CUDA graph captured once per solver */
  int nu;             /* smoothing sweeps before/after each coarse correction (0 = default 2) */
  int device;         /* CUDA device ordinal */
  int nu_coarse;      /* smoothing sweeps per side on multigrid levels mg_lnu and coarser (0 = default: 1 with a
                         transform axis, nu for a 3-D solve) */
  /* mixed-precision solve (precision 1); 0 selects the default everywhere */
  int inner_iters;    /* FP32 Krylov iterations per refinement step (default 5) */
  double inner_tol;   /* relative reduction at which a system's FP32 solve stops (default 1e-6) */
  int inner_adapt;    /* 1 (default): a system's FP32 solve also stops once its outer residual would be within a
                         tenth of the tolerance; -1: off */
  int refine_steps;   /* n > 0: FP32 refinement steps after which the systems still above the tolerance finish
                         with FP64 conjugate-gradient iterations; default (0 or -1): FP32 refinement steps
                         until converged */
  /* multigrid kernels (plane systems: tiled smoother, one-CTA coarse V-cycle) */
  int mg_fuse;        /* bits: 1 tiled FP32 smoother, 2 one-CTA coarse V-cycle FP32, 4 tiled FP64 smoother,
                         8 one-CTA coarse V-cycle FP64 (default 11); -1: one kernel per sweep */
  int mg_cta_level;   /* finest level the one-CTA coarse V-cycle may start at (default: the finest that fits;
                         with the 3-D solve, and for the FP32 plane systems with the tiled smoother on, the
                         finest that fits with at most 4096 cells) */
  int mg_tile;        /* FP32 smoother tile, warps x rows per warp: 1 8x2, 2 8x3, 3 16x2, 4 16x3, 5 8x4, 6 16x4
                         (default: the shape among the first four with the fewest tile rows, the three-row
                         shapes' rows counted twice for their halved occupancy) */
  int mg_waves;       /* waves of CTAs per batched plane launch (default 2) */
  int mg_red_batch;   /* -1: the reducing plane kernels run one system per CTA (default: batched) */
  int mg_lnu;         /* first multigrid level that uses nu_coarse (default 2) */
  int tma;            /* -1: the fillps pass reads its fields directly instead of through TMA-staged tiles
                         (default: TMA where the blocks allow it: even x extents, at most 16 blocks) */
  int pdl;            /* -1: the solver's inner-loop kernels launch without programmatic dependent launch
                         (default: with it, each kernel's set-up overlapping the previous kernel's tail) */
  int mg_inv;         /* 1: the FP32 tiled smoother forms 1 / diagonal of each system in registers from the cell's
                         coefficients and the system's shift instead of reading the per-system table (the same
                         values); default: the table */
  int mg_restrict;    /* -1: the FP32 tiled pre-smoother of levels 0 and 1 leaves the residual restriction to a
                         separate pass over the level; default: it restricts the residual of its own output cells
                         (the same values, one pass fewer per level and V-cycle) */
} snac_options;

typedef struct snac_step_stats {
  int    istep;
  double time, dt;
  int    solve_iters_max;     /* largest iteration count of the last step's solves */
  double solve_residual_max;  /* largest final relative residual of the last step's solves */
  int    solves;              /* solves run in the last step */
  double device_ms;           /* device time of the last snac_step call (CUDA events on the library stream) */
  int    helm_iters_max;      /* IMPDIFF: largest iteration count of the last step's Helmholtz solves */
  double helm_residual_max;   /* IMPDIFF: largest final relative residual of those solves */
} snac_step_stats;

/* param.f90:88-240: reads dns.nml (&dns, &scalar, &hypre) and blocks.nml (&blocks) with the reference's
 * defaults into c and blocks[0..nblocks-1] (room for max_blocks).  The reference's build flags are
 * arguments: fft_axis (FFT_AXIS 0..3), impdiff (_IMPDIFF), boussinesq (_BOUSSINESQ_BUOYANCY).  Host only;
 * grid files and block_dims (the MPI split of a block) are not read. */
int snac_read_namelists(const char *dns_path, const char *blocks_path, int fft_axis, int impdiff, int boussinesq,
                        snac_case *c, snac_block_desc *blocks, int max_blocks);

/* ---------------------------------------------------------------- errors, diagnostics */
const char *snac_last_error(void);
int snac_device_count(int *n);
/* No counterpart in the reference: measured FMA throughput of the device (GFLOP/s, 2 flops per FMA),
 * the compute roofline of the FP64 kernels. */
int snac_probe_peaks(double *fp64_gflops, double *fp32_gflops);
/* No counterpart in the reference: time every launch of one kernel class with CUDA events on the
 * library stream (1 rk_mom, 2 red-black smoother, 3 residual+restriction, 4/5 forward/backward
 * transform, 6 Krylov operator apply, 7 fillps, 8 correc, 9 one-CTA coarse V-cycle, 10 whole pressure
 * solve; 0 = off).  Selecting resets the record. */
int snac_profile_kernel(int kernel_class);
int snac_profile_read(int *launches, double *total_ms);
/* No counterpart in the reference: number of kernels this library has launched since it was loaded
 * (a host-side counter incremented at every launch site). */
int snac_launch_count(long long *n);
/* No counterpart in the reference: time `reps` launches of the FP32 tiled pre-smoother on level `level`
 * of the pressure solver of the current domain as its V-cycles run it (restricting its residual unless
 * snac_options.mg_restrict is -1), all systems active, with CUDA events on the library stream.  Returns
 * the mean time per launch and its algorithmic bytes (b, 1/diagonal read, x written: 12 bytes per cell and
 * system; with the restriction also 4 bytes per coarse cell and system written).  The solver's level
 * buffers are overwritten. */
int snac_bench_smoother(int level, int reps, double *ms_per_launch, double *bytes_per_launch);

/* ---------------------------------------------------------------- host mirrors */
/* Keep a device mirror of a host array of `bytes` bytes (contents uploaded). */
int snac_register(void *host, size_t bytes);
int snac_unregister(void *host);
int snac_update_device(void *host);      /* host -> mirror */
int snac_update_host(void *host);        /* mirror -> host */

/* ---------------------------------------------------------------- reference-signature calls */
/* rk.f90:7-128 (rk_mom) with mom.f90:112-386; s1 = scalars(1)%val (may be NULL unless boussinesq) */
int snac_rk_mom(const double rkpar[2], const int lo[3], const int hi[3],
                const double *dxc, const double *dxf, const double *dyc, const double *dyf,
                const double *dzc, const double *dzf, double dt, const double bforce[3],
                const double gacc[3], double beta, const double *s1, double visc,
                double *u, double *v, double *w, const double *p,
                double *dudtrko, double *dvdtrko, double *dwdtrko, int impdiff, int boussinesq);
/* rk.f90:130-204 (rk_scal) with scal.f90:89-179; f receives scalf - bulk mean when is_forced */
int snac_rk_scal(const double rkpar[2], const int lo[3], const int hi[3],
                 const double *dxc, const double *dxf, const double *dyc, const double *dyf,
                 const double *dzc, const double *dzf, double dt, double alpha, double vol_all,
                 const double *u, const double *v, const double *w, int is_forced, double scalf,
                 double ssource, double *dsdtrko, double *s, double *f, int impdiff);
/* fillps.f90:7-54; fft_axis selects the _FFT_X/_Y/_Z weighting */
int snac_fillps(const int lo[3], const int hi[3], const double *dxf, const double *dyf,
                const double *dzf, double dt, const double *u, const double *v, const double *w,
                double *p, int fft_axis);
/* correc.f90:7-48 */
int snac_correc(const int lo[3], const int hi[3], const double *dxc, const double *dyc,
                const double *dzc, double dt, const double *p, double *u, double *v, double *w);
/* updt_pressure.f90:7-47 */
int snac_updt_pressure(const int lo[3], const int hi[3], const double *dxc, const double *dxf,
                       const double *dyc, const double *dyf, const double *dzc, const double *dzf,
                       double alpha, const double *pp, double *p, int impdiff);
/* bound.f90:543-585 */
int snac_updt_rhs(const int lo[3], const int hi[3], const int is_bound[3][2],
                  const double *rhsx, const double *rhsy, const double *rhsz, double *p);
/* chkdt.f90:8-56 for one block/rank; visc is the value passed by main.f90:660 (max(visc,alpha_max)) */
int snac_chkdt(const int lo[3], const int hi[3], const double *dxc, const double *dxf,
               const double *dyc, const double *dyf, const double *dzc, const double *dzf,
               double visc, const double *u, const double *v, const double *w, int impdiff,
               double *dtmax);
/* chkdiv.f90:8-44 for one block/rank (the MPI reductions are the caller's when several blocks) */
int snac_chkdiv(const int lo[3], const int hi[3], const double *dxf, const double *dyf,
                const double *dzf, const double *u, const double *v, const double *w, double vol,
                double *divtot, double *divmax);
/* No counterpart in the reference.  snac_chkdiv for callers that must not allocate device memory
 * (e.g. a driver whose fields were placed on the GPU up front and that checks the divergence inside
 * its time loop, where cudaMalloc/cudaFree would synchronise the device or fail on a full GPU):
 * u, v, w (halo'd) and dxf, dyf, dzf ((n+2) entries) are DEVICE pointers, stream is a cudaStream_t
 * (NULL = default stream), divtot/divmax are host pointers.  Scratch is a fixed 128 KiB device array
 * owned by the library (held on every GPU that loads it until exit); blocks above 2^31-1 cells, or
 * above 2^31-65 cells along one axis, are rejected with SNAC_ERR_ARG.  The first call on a device resolves the array's address with that
 * device current -- make it before any stream capture; calls that overlap on the GPU race on the
 * shared array. */
int snac_chkdiv_noalloc(const int lo[3], const int hi[3], const double *dxf, const double *dyf,
                        const double *dzf, const double *u, const double *v, const double *w, double vol,
                        void *stream, double *divtot, double *divmax);
/* bound.f90:8-66 (bounduvw) for one block on the caller's arrays, with the reference's argument list:
 * cbc[c][d][s] and bc[c][d][s] are the reference's cbc(s,d,c) and bc(s,d,c) of velocity component c along
 * direction d, is_bound[d][s] and nb[d][s] its is_bound(s,d) and nb(s,d).  The halo exchange (updthalo,
 * bound.f90:587-650) is made on the device for every side whose neighbour nb[d][s] is `myrank` itself (a
 * periodic direction this rank spans alone), in the reference's x, y, z order; sides whose neighbour is another
 * rank are the caller's MPI exchange (their ghost planes are left untouched), and the MPI datatypes `halos`
 * of the reference have no counterpart here.  Then set_bc on every face with is_bound, face by face in the
 * reference's order, the wall-normal component skipped when is_correc.  Metrics (n+2 entries from lo-1) and
 * u, v, w (halo'd) are host arrays, registered (device mirror) or copied around the call. */
int snac_bounduvw(const char cbc[3][3][2], const int lo[3], const int hi[3], const double bc[3][3][2], int is_correc,
                  const int is_bound[3][2], const int nb[3][2], int myrank, const double *dxc, const double *dxf,
                  const double *dyc, const double *dyf, const double *dzc, const double *dzf, double *u, double *v,
                  double *w);
/* bound.f90:68-106 (boundp) for one block, as snac_bounduvw for the centred field p (cbc[d][s], bc[d][s] are
 * cbc(s,d), bc(s,d)). */
int snac_boundp(const char cbc[3][2], const int lo[3], const int hi[3], const double bc[3][2], const int is_bound[3][2],
                const int nb[3][2], int myrank, const double *dxc, const double *dyc, const double *dzc, double *p);
/* post.f90:8-156 for one block, with the reference's argument lists: n the interior extents, the metrics
 * (n+2 entries from lo-1) and the halo'd velocity ux, uy, uz as host arrays (registered mirrors or copied
 * around the call); outputs interior (n).  cmpt_vorticity (post.f90:8-53): the three vorticity components at
 * the cell centres; cmpt_strain_rate (post.f90:55-98): S_ij S_ij; cmpt_rotation_rate (post.f90:100-139):
 * W_ij W_ij; cmpt_q_criterion (post.f90:141-156): Q = (ens - str) / 2. */
int snac_cmpt_vorticity(const int n[3], const double *dxc, const double *dyc, const double *dzc, const double *ux,
                        const double *uy, const double *uz, double *vox, double *voy, double *voz);
int snac_cmpt_strain_rate(const int n[3], const double *dxc, const double *dyc, const double *dzc, const double *dxf,
                          const double *dyf, const double *dzf, const double *ux, const double *uy, const double *uz,
                          double *str);
int snac_cmpt_rotation_rate(const int n[3], const double *dxc, const double *dyc, const double *dzc, const double *ux,
                            const double *uy, const double *uz, double *ens);
int snac_cmpt_q_criterion(const int n[3], const double *ens, const double *str, double *qcr);
/* No counterpart in the reference (which computes the two rates into arrays first): the Q criterion of one block
 * straight from the velocity in one pass, the same values as the three calls above. */
int snac_q_criterion(const int n[3], const double *dxc, const double *dyc, const double *dzc, const double *dxf,
                     const double *dyf, const double *dzf, const double *ux, const double *uy, const double *uz,
                     double *qcr);
/* bound.f90:108-248 (set_bc) on one face of one halo'd array */
int snac_set_bc(char ctype, int ibound, const int lo[3], const int hi[3], int idir, int centered,
                double rvalue, double dr, double *p);
/* fft.f90:85-94 (fft): in-place unnormalised r2r of kind along axis idir (1..3) of an
 * interior array arr(n(1),n(2),n(3)), over the first n(idir)-q points (q = 0 or 1, fft.f90:32) */
int snac_fft(int kind, int idir, const int n[3], int q, double *arr);
/* fft.f90:96-149 and 151-189 */
int snac_find_fft(const char bc[2], int is_centered, int *kind_fwd, int *kind_bwd, double norm[2]);
int snac_eigenvalues(int n, const char bc[2], int is_centered, double *lambda);
/* initgrid.f90:9-83: arrays over lo-1..hi+1 */
int snac_initgrid(int lo, int hi, int gt, double gr, double lmin, double lmax,
                  double *drc, double *drf, double *rc, double *rf);

/* ---------------------------------------------------------------- domain layer */
/* read_input + initmpi + initgrid/bound_grid + init_bc_rhs + solver set-up (main.f90:188-886) */
int snac_init(const snac_case *c, const snac_block_desc *blocks, const snac_options *opt);
/* The host part of snac_init without a device (placement, grids, operator assembly, multigrid
 * hierarchy): validates an input and returns the number of multigrid levels and the cells of the
 * coarsest level.  Reference counterpart: the sanity checks of sanity.f90 / initmpi.f90:150-237. */
int snac_check_case(const snac_case *c, const snac_block_desc *blocks, int *levels, long *coarse_cells);
int snac_finalize(void);
int snac_block_geometry(int ib, int lo[3], int hi[3], int nb[3][2], int is_bound[3][2]);
int snac_get_grid(int ib, int axis, int which, double *out);         /* (ng+2) values */
int snac_set_field(int ib, int field, const double *host);
int snac_get_field(int ib, int field, double *host);
/* n fields at once (block ib[q], field kind field[q], host array host[q]): the copies are issued on two
 * streams (two copy engines) and the call returns when all are complete */
int snac_set_fields(int n, const int *ib, const int *field, const double *const *host);
int snac_get_fields(int n, const int *ib, const int *field, double *const *host);
double snac_vol_all(void);
/* the per-stage routines of main.f90:906-1043 on every block */
int snac_rk_mom_all(int irk);                     /* rk_mom for all blocks with the current dt */
int snac_bounduvw_all(int is_correc);             /* bound.f90:8-66 */
int snac_boundp_all(int field);
/* inflow (bound.f90:438-477) on every block's inflow faces: the normal component set on the boundary face
 * (skipped when is_correc), the tangential ones mirrored about the face value */
int snac_inflow_all(int is_correc);                   /* bound.f90:68-106 (SNAC_P, SNAC_PP, scalars) */
int snac_fillps_all(double dtrk);                 /* fillps.f90 */
/* solve_impdiff_field (solve_helmholtz.f90:32-138, called at main.f90:919-934 and 961-978) of one field of every
 * block: field SNAC_U, SNAC_V, SNAC_W or SNAC_S0 + s is replaced by the solution of the IMPDIFF Helmholtz problem
 * (A + alphai_new V) phi = alphai_new V phi + BC planes, warm-started from the previous solution of that field's
 * solver, with the transform along FFT_AXIS when there is one.  alphai_old is accepted for the reference's
 * argument list: the shift of each solve is set from alphai_new alone (the reference adds alphai_new -
 * alphai_old to the matrix it keeps).  Needs a domain set up with IMPDIFF; SNAC_ERR_NOT_CONVERGED as for
 * the pressure solve. */
int snac_impdiff_solve(int field, double alphai_new, double alphai_old);
int snac_updt_rhs_all(void);                      /* bound.f90:543-585 with the pressure BC planes */
int snac_solve_pressure(void);                    /* fft + solve_n_helmholtz_2d + fft + normfft, or solve_helmholtz */
int snac_correc_all(double dtrk);                 /* correc.f90 */
int snac_updt_pressure_all(double alpha);         /* updt_pressure.f90 */
int snac_chkdt_all(double *dt_cfl);               /* chkdt.f90 incl. the MPI reductions */
int snac_chkdiv_all(double *divtot, double *divmax);
int snac_kinetic_energy(double *ke);
/* checkpoints, load_one (load.f90:92-160) as main.f90:544-553 (read) and 1107-1115 (write) call it: for
 * block b (1-based) and field f the file "<prefix>_b_<b as %03d>_<f>.bin", f = u, v, w, p, s_001..,
 * each the block's interior ng(1) x ng(2) x ng(3) FP64 values in Fortran order followed by
 * [time, istep] as two FP64 values.  prefix is e.g. "data/fld" (is_overwrite_save) or "data/fld_0001000".
 * Loading checks every file's size (the reference's abort becomes SNAC_ERR_IO), replaces the interiors
 * and sets time and istep; ghost cells are left to the caller's bounduvw/boundp, as in main.f90:562-568. */
int snac_checkpoint_save(const char *prefix);
int snac_checkpoint_load(const char *prefix);

/* out1d (output.f90:34-125) as out1d.h90 calls it: the average of field f of block ib over the planes
 * normal to idir (1..3), each field with its own spacings and coordinates (u: dxc,dyf,dzf at xf,yc,zc;
 * v: dxf,dyc,dzf at xc,yf,zc; w: dxf,dyf,dzc at xc,yc,zf; p, pp and scalars: dxf,dyf,dzf at xc,yc,zc),
 * divided by the block's lengths.  coord and prof receive ng(idir) values. */
int snac_out1d(int ib, int field, int idir, double *coord, double *prof);
/* the same profile written as the reference's text file: one line per index in format (2E15.7) */
int snac_out1d_write(const char *fname, int ib, int field, int idir);
/* out3d (output.f90:227-257): the interior of field f of block ib in Fortran order, FP64, no header */
int snac_out3d_write(const char *fname, int ib, int field);

/* No counterpart in the reference: one dense 3x3 convolution layer of the learned initial guess on the
 * tensor cores (tcgen05, BF16 inputs, FP32 accumulation): y = act(bias + w * x) over nplanes images of
 * 16 channels x H x W (x rounded to BF16, zero padding, act = ReLU when relu != 0), weights w[16][16][3][3]. */
int snac_cnn_conv3x3(const float *x, int nplanes, int H, int W, const float *w, const float *bias, int relu,
                     float *y);
/* No counterpart in the reference: a testing hook for the convolution's bounded wait on its tensor-core
 * accumulator.  The launches that follow poll the accumulator's mbarrier at most `polls` times (negative:
 * the default, 2^24); a wait that runs out makes the call return SNAC_ERR_TIMEOUT after the kernel has let the
 * MMAs in flight finish (with the full bound) and freed its tensor memory, so the context stays usable. */
int snac_cnn_set_poll_limit(long polls);

/* No counterpart in the reference: forward and backward of the learned-guess network (three 3x3 layers of
 * 16 channels, ReLU between them) on host data, for checking its gradients: x nb x 16 x H x W, target
 * nb x H x W, params 3 x (16*16*9 weights + 16 biases); returns the loss
 * (1/nb) sum_p |y_p - t_p|^2 / |t_p|^2 and its gradient with respect to every parameter. */
int snac_guess_grad(const float *x, const float *target, int nb, int H, int W, const float *params, float *grads,
                    double *loss);

/* Open and outflow boundaries of one block (bound.f90:250-541; the reference's main.f90 does not call them).
 * idir 1..3, ibound 0/1; u, v, w, p halo'd (lo-1:hi+1)^3; a traction plane tr (tr_x, tr_y, tr_z for idir 1, 2,
 * 3) is (lo_t1-1:hi_t1+1, lo_t2-1:hi_t2+1, 0:1), t1 < t2 the two other axes.  Fortran (ibound, idir) arrays are
 * [idir-1][ibound] here, dlc(0:1, ibound, idir) is dlc[idir-1][ibound][0:1]. */
/* set_open_bc_uvw (bound.f90:250-328) */
int snac_set_open_bc_uvw(int ibound, const int lo[3], const int hi[3], int idir, double visc, double dr, double *u,
                         double *v, double *w, const double *p, double *tr);
/* set_open_bc_p (bound.f90:330-375) */
int snac_set_open_bc_p(int ibound, const int lo[3], const int hi[3], int idir, const double drc[2], double drf,
                       double alpha, double *p);
/* cmpt_estimated_traction (bound.f90:377-436) */
int snac_cmpt_estimated_traction(int ibound, const int lo[3], const int hi[3], int idir, double visc, double dr,
                                 const double *u, const double *v, const double *w, const double *p, double *tr);
/* outflow (bound.f90:479-515) */
int snac_outflow(const int is_outflow_bound[3][2], const int is_estimated_traction[3][2], const int lo[3],
                 const int hi[3], const double dl[3][2], const double dl_h[3][2], double visc, double *u, double *v,
                 double *w, double *p, double *tr_x, double *tr_y, double *tr_z);
/* outflow_p (bound.f90:517-541) */
int snac_outflow_p(const int is_outflow_bound[3][2], const int lo[3], const int hi[3], const double dlc[3][2][2],
                   const double dlf[3][2], double alpha, double *p);

/* No counterpart in the reference (the stand-in for compute-sanitizer and the reference's -fcheck=all debug
 * build): snac_bounds_checked is 1 in the bounds-check build (libsnac_gb300_checked.so, compiled with
 * -DSNAC_BOUNDS_CHECK), where the stencil, halo-exchange, boundary-condition and inflow kernels validate the
 * cells and 1-D table entries they address against their block and skip an access outside it; the entry
 * points that run kernels then return SNAC_ERR_BOUNDS naming the kernel and the cell.  snac_bounds_selftest
 * launches a check that fails by design (no access is made) and returns what the host check reports:
 * SNAC_ERR_BOUNDS in that build, SNAC_ERR_UNSUPPORTED in the normal one. */
int snac_bounds_checked(void);
int snac_bounds_selftest(void);

/* No counterpart in the reference: the three-level U-Net of the learned guess of the 3-D pressure solve
 * (about 180k parameters: conv 3x3x3 16->16, pool, 16->32, pool, 32->64, [up | skip] 96->32, [up | skip]
 * 48->16, head 1x1x1 16->1; BF16 tensor-core operands, FP32 accumulation).  snac_unet_nparams gives the
 * parameter count.  snac_unet_forward runs it on host data: x nb x 2 x n2 x n1 x n0 (residual, live mask
 * 0/1), params as the oracle lays them out; out nb x n2 x n1 x n0.  snac_unet_grad also returns the loss
 * (1/nb) sum_b sum_live (out - t)^2 / sum_live t^2 and its gradient with respect to every parameter.
 * snac_unet_set_poll_limit is the testing hook of the convolutions' bounded accumulator wait (as
 * snac_cnn_set_poll_limit). */
int snac_unet_nparams(void);
int snac_unet_forward(const float *x, int nb, int n0, int n1, int n2, const float *params, float *out);
int snac_unet_grad(const float *x, const float *target, int nb, int n0, int n1, int n2, const float *params,
                   float *grads, double *loss);
int snac_unet_set_poll_limit(long polls);

/* No counterpart in the reference: the learned initial guess of the pressure solve.  mode 0 off;
 * 1 every pressure solve of snac_step records training pairs (the residual of the previous solution and
 * the diagonally scaled correction the solve made: whole wavenumber planes with a transform axis, random
 * 32^3 crops with the 3-D solve); 2 every solve starts from the previous solution plus the network's
 * correction, scaled by the step that minimises the residual (the multigrid then iterates to the same
 * tolerance).  With a transform axis the network is the plane network of snac_guess_grad, with the 3-D
 * solve the U-Net of snac_unet_forward. */
int snac_guess_mode(int mode);
/* trains the network on the recorded pairs on the GPU: iters Adam steps at learning rate lr (16-plane
 * batches; 3-D solve: 4 crops); returns the mean batch loss of the first and last few steps and the number
 * of recorded pairs */
int snac_guess_train(int iters, double lr, double *loss_first, double *loss_last, int *pairs);
/* with on != 0 every guided solve also measures |b - A x0| / |b - A x_prev| per non-singular system; returns
 * the median and largest ratio of the last guided solve */
int snac_guess_measure(int on, double *ratio_median, double *ratio_max);

/* No counterpart in the reference (HYPRE's PFMG settings are fixed in the input): picks the solver settings
 * for this case by timing.  Every candidate (the plain FP64 solve, or the mixed solve with 4, 5 or 6 FP32
 * Krylov iterations per refinement step; one or two smoothing sweeps per side on levels 2 and coarser with
 * a transform axis) rebuilds the solvers and runs 1 + steps RK3 steps from a snapshot of the state; all
 * solve to the same tolerance, and candidates whose solves do not converge are dropped.  The state (fields, RK storage, time, dt, step count and the solvers' warm starts) is
 * then restored and the solvers are rebuilt with the fastest candidate. */
typedef struct snac_tune_result {
  int precision;        /* chosen solve: 0 plain FP64, 1 mixed (as snac_options.precision) */
  int inner_iters;      /* chosen FP32 Krylov iterations per refinement step (mixed solve) */
  int nu_coarse;        /* chosen smoothing sweeps per side on levels 2 and coarser */
  double ms_per_step;   /* device time per step of the chosen candidate */
  double ms_before;     /* device time per step of the settings in use before the call */
  int ncand;            /* candidates timed */
  int mg_tile;          /* chosen FP32 smoother tile of level 0 (as snac_options.mg_tile; 0 without a plane solve) */
  int mg_waves;         /* chosen waves of CTAs per batched plane launch */
  int mg_cta_level;     /* first level of the one-CTA coarse V-cycle of the chosen solve */
  int refine_steps;     /* mixed solve: FP32 refinement steps before FP64 finishing (-1: FP32 to convergence) */
} snac_tune_result;
int snac_autotune(int steps, snac_tune_result *out);
/* No counterpart in the reference: a host-side fault injector for testing snac_autotune's error paths.  The
 * next snac_autotune call fails with SNAC_ERR_STATE right after rebuilding the solvers of candidate
 * `candidate` (0-based; -1 clears), which must leave the settings, the solvers and the state as they were
 * before the call.  Nothing on the device is made to fail. */
int snac_tune_inject_failure(int candidate);

/* whole RK3 steps, main.f90:893-1069 (dt from chkdt every icheck steps) */
int snac_step(int nsteps);
int snac_get_stats(snac_step_stats *st);
int snac_set_dt(double dt);
int snac_get_dt(double *dt);

#ifdef __cplusplus
}
#endif
#endif
