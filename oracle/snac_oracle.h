/*
 * snac_oracle.h -- CPU restatement of SNaC's per-time-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity oracle and the timed
 * CPU baseline; it is never linked into, loaded by, or called from the
 * snac_gb300 product path.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py may load it.
 *
 * Every routine states the reference file:line it restates (paths relative to
 * the SNaC source tree).  The reference is Fortran 2008 + MPI + HYPRE + FFTW;
 * none of those toolchains/libraries exist on the build or GPU machines, so
 * the reference cannot be compiled and this C restatement is the oracle.
 * HYPRE (unpinned master) and FFTW3 (unpinned distro package) are replaced by:
 *   - direct O(n^2) evaluations of FFTW's documented, unnormalised r2r kinds
 *     (R2HC/HC2R, REDFT00/01/10/11, RODFT00/01/10/11);
 *   - a preconditioned conjugate-gradient solve (multigrid V-cycle
 *     preconditioner) of the exact linear systems the reference assembles in
 *     solver.f90 (init_matrix_3d / init_matrix_2d / init_n_2d_matrices),
 *     iterated to a relative residual far below HYPRE's, so only HYPRE's
 *     converged answer -- not its iterates -- is reproduced.
 *
 * Array conventions (identical to the reference's Fortran declarations):
 *   halo'd field  f(lo(1)-1:hi(1)+1, lo(2)-1:hi(2)+1, lo(3)-1:hi(3)+1), x fastest;
 *   RK storage    dudtrko(lo(1):hi(1), lo(2):hi(2), lo(3):hi(3));
 *   1-D metric    dxc(lo(1)-1:hi(1)+1)  -- pointer to element lo(1)-1;
 *   BC planes     rhsx(lo(2):hi(2),lo(3):hi(3),0:1) etc.
 * Character BC arrays cbc(0:1,3) are stored side-fastest: cbc[dir][side].
 */
#ifndef SNAC_ORACLE_H
#define SNAC_ORACLE_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

#define OR_MAX_SCAL 4

/* per-block input, mirrors the &blocks namelist entries (param.f90:332-360) */
typedef struct or_block_desc {
  int    ng[3];
  double lmin[3], lmax[3];
  int    gt[3];
  double gr[3];
  char   cbcvel[3][3][2];          /* block_cbcvel(0:1,1:3,1:3,ib): [comp][dir][side] */
  double bcvel[3][3][2];
  char   cbcpre[3][2];             /* block_cbcpre(0:1,1:3,ib) */
  double bcpre[3][2];
  char   cbcscal[OR_MAX_SCAL][3][2];
  double bcscal[OR_MAX_SCAL][3][2];
  const double *grid_file[3];      /* optional grid/grid_?_b_###.bin contents: rf,rc,drf,drc (4*ng) */
  int    inflow_type[3][2];        /* block_inflow_type(0:1,1:3,ib): 0 none, 1 Poiseuille, 2 Kovasznay */
} or_block_desc;

/* global input, mirrors &dns/&scalar/&hypre (param.f90:342-355) + build flags */
typedef struct or_case {
  int    nblocks;
  double visci, cfl, dtmax, dt_f;
  double bforce[3], gacc[3], beta;
  int    nscal;
  double alphai[OR_MAX_SCAL], ssource[OR_MAX_SCAL], scalf[OR_MAX_SCAL];
  int    is_sforced[OR_MAX_SCAL];
  int    icheck;
  int    fft_axis;                 /* 0: 3-D solve; 1,2,3: _FFT_X/_FFT_Y/_FFT_Z */
  int    impdiff;                  /* _IMPDIFF */
  int    boussinesq;               /* _BOUSSINESQ_BUOYANCY */
  double tol;                      /* relative residual of every Poisson/Helmholtz solve */
  int    maxiter;
} or_case;

/* ---------------- per-block hot-path routines (reference signatures) ---- */
void or_rk_mom(const double rkpar[2], const int lo[3], const int hi[3],
               const double *dxc, const double *dxf, const double *dyc, const double *dyf,
               const double *dzc, const double *dzf, double dt, const double bforce[3],
               const double gacc[3], double beta, const double *s1, double visc,
               double *u, double *v, double *w, const double *p,
               double *dudtrko, double *dvdtrko, double *dwdtrko,
               int impdiff, int boussinesq);
void or_rk_scal(const double rkpar[2], const int lo[3], const int hi[3],
                const double *dxc, const double *dxf, const double *dyc, const double *dyf,
                const double *dzc, const double *dzf, double dt, double alpha, double vol_all,
                const double *u, const double *v, const double *w,
                int is_forced, double scalf, double ssource, double *dsdtrko, double *s,
                double *f, int impdiff);
void or_bulk_forcing_s(const int lo[3], const int hi[3], int is_forced, double ff, double *s);
void or_fillps(const int lo[3], const int hi[3], const double *dxf, const double *dyf,
               const double *dzf, double dt, const double *u, const double *v, const double *w,
               double *p, int fft_axis);
void or_correc(const int lo[3], const int hi[3], const double *dxc, const double *dyc,
               const double *dzc, double dt, const double *p, double *u, double *v, double *w);
void or_updt_pressure(const int lo[3], const int hi[3], const double *dxc, const double *dxf,
                      const double *dyc, const double *dyf, const double *dzc, const double *dzf,
                      double alpha, const double *pp, double *p, int impdiff);
/* local parts of chkdt/chkdiv (before MPI_ALLREDUCE) */
void or_chkdt_local(const int lo[3], const int hi[3], const double *dxc, const double *dxf,
                    const double *dyc, const double *dyf, const double *dzc, const double *dzf,
                    const double *u, const double *v, const double *w, double *dti, double *dlmin);
void or_chkdiv_local(const int lo[3], const int hi[3], const double *dxf, const double *dyf,
                     const double *dzf, const double *u, const double *v, const double *w,
                     double vol, double *divtot, double *divmax);
void or_updt_rhs(const int lo[3], const int hi[3], const int is_bound[3][2],
                 const double *rhsx, const double *rhsy, const double *rhsz, double *p);
void or_set_bc(char ctype, int ibound, const int lo[3], const int hi[3], int idir,
               int centered, double rvalue, double dr, double *p);
void or_bounduvw_block(const char cbc[3][3][2], const int lo[3], const int hi[3], const double bc[3][3][2],
                       int is_correc, const int is_bound[3][2], const int nb[3][2], int myrank,
                       const double *dxc, const double *dxf, const double *dyc, const double *dyf,
                       const double *dzc, const double *dzf, double *u, double *v, double *w);
void or_boundp_block(const char cbc[3][2], const int lo[3], const int hi[3], const double bc[3][2],
                     const int is_bound[3][2], const int nb[3][2], int myrank, const double *dxc,
                     const double *dyc, const double *dzc, double *p);
void or_cmpt_vorticity(const int n[3], const double *dxc, const double *dyc, const double *dzc, const double *ux,
                       const double *uy, const double *uz, double *vox, double *voy, double *voz);
void or_cmpt_strain_rate(const int n[3], const double *dxc, const double *dyc, const double *dzc, const double *dxf,
                         const double *dyf, const double *dzf, const double *ux, const double *uy, const double *uz,
                         double *str);
void or_cmpt_rotation_rate(const int n[3], const double *dxc, const double *dyc, const double *dzc, const double *ux,
                           const double *uy, const double *uz, double *ens);
void or_cmpt_q_criterion(const int n[3], const double *ens, const double *str, double *qcr);
/* open / outflow boundaries, bound.f90:250-541 (traction planes (lo_t1-1:hi_t1+1, lo_t2-1:hi_t2+1, 0:1)) */
void or_set_open_bc_uvw(int ibound, const int lo[3], const int hi[3], int idir, double visc, double dr, double *u,
                        double *v, double *w, const double *p, double *tr);
void or_set_open_bc_p(int ibound, const int lo[3], const int hi[3], int idir, const double drc[2], double drf,
                      double alpha, double *p);
void or_cmpt_estimated_traction(int ibound, const int lo[3], const int hi[3], int idir, double visc, double dr,
                                const double *u, const double *v, const double *w, const double *p, double *tr);
void or_outflow(const int is_outflow_bound[3][2], const int is_estimated_traction[3][2], const int lo[3],
                const int hi[3], const double dl[3][2], const double dl_h[3][2], double visc, double *u, double *v,
                double *w, double *p, double *tr_x, double *tr_y, double *tr_z);
void or_outflow_p(const int is_outflow_bound[3][2], const int lo[3], const int hi[3], const double dlc[3][2][2],
                  const double dlf[3][2], double alpha, double *p);
void or_init_bc_rhs(const char cbc[3][2], const double bc[3][2], const double dl[3][2],
                    const int is_bound[3][2], const int is_centered[3], const int lo[3],
                    const int hi[3], const int periods[3],
                    const double *dx1, const double *dx2, const double *dy1, const double *dy2,
                    const double *dz1, const double *dz2,
                    double *rhsx, double *rhsy, double *rhsz,
                    const double *bcx, const double *bcy, const double *bcz, int fft_axis);

/* ---------------- transforms (fft.f90) ---------------------------------- */
enum { OR_R2HC = 0, OR_HC2R = 1, OR_REDFT00 = 3, OR_REDFT01 = 4, OR_REDFT10 = 5,
       OR_REDFT11 = 6, OR_RODFT00 = 7, OR_RODFT01 = 8, OR_RODFT10 = 9, OR_RODFT11 = 10 };
void or_find_fft(const char bc[2], int is_centered, int *kind_fwd, int *kind_bwd, double norm[2]);
int  or_eigenvalues(int n, const char bc[2], int is_centered, double *lambda);
void or_r2r(int kind, int n, const double *in, double *out);
void or_r2r_lines(int kind, int n, int howmany, long stride, long dist, double *arr);

/* ---------------- setup (initgrid.f90, initmpi.f90) --------------------- */
void or_initgrid(int lo, int hi, int gt, double gr, double lmin, double lmax,
                 double *drc, double *drf, double *rc, double *rf);
int  or_place_blocks(int nblocks, const or_block_desc *blocks, int (*lo_g)[3]);

/* ---------------- domain: all blocks on one process -------------------- */
typedef struct or_domain or_domain;
enum { OR_U = 0, OR_V, OR_W, OR_P, OR_PP, OR_PO, OR_DUDTRKO, OR_DVDTRKO, OR_DWDTRKO,
       OR_S0, OR_S1, OR_S2, OR_S3, OR_DSDTRKO0 = 20, OR_NFIELDS = 32 };
enum { OR_G_DXC = 0, OR_G_DXF, OR_G_XC, OR_G_XF };

or_domain *or_create(const or_case *c, const or_block_desc *blocks, char *err, int errlen);
void   or_destroy(or_domain *d);
int    or_block_geometry(const or_domain *d, int ib, int lo[3], int hi[3], int nb[3][2],
                         int is_bound[3][2]);
double *or_field(or_domain *d, int ib, int kind);        /* NULL if not allocated */
double *or_grid(or_domain *d, int ib, int axis, int which); /* (n+2) entries, lo-1..hi+1 */
double  or_vol_all(const or_domain *d);
void   or_bounduvw(or_domain *d, int is_correc);
void   or_boundp(or_domain *d, int kind);
void   or_inflow(or_domain *d, int is_correc);              /* bound.f90:438-477 on every inflow face */
/* load_one (load.f90:92-160) per block and field: "<prefix>_b_%03d_{u,v,w,p,s_%03d}.bin"; 0 ok, -1 i/o error,
   -2 a file of the wrong size */
int    or_checkpoint_save(or_domain *d, const char *prefix);
int    or_checkpoint_load(or_domain *d, const char *prefix);
void   or_time_istep(const or_domain *d, double *time, int *istep);
/* out1d (output.f90:34-125) with out1d.h90's spacings/coordinates per field; writes n(idir) values, and
   the reference's text file when fname is not NULL (format 2E15.7) */
int    or_out1d(or_domain *d, int ib, int kind, int idir, double *coord, double *prof, const char *fname);
void   or_fortran_e15_7(double v, char *out);  /* Fortran Ew.d, w = 15, d = 7 */
void   or_fillps_all(or_domain *d, double dtrk);
int    or_impdiff_solve(or_domain *d, int field, double alphai);
void   or_updt_rhs_all(or_domain *d);
int    or_solve_pressure(or_domain *d);                   /* pp <- solution, po updated */
void   or_correc_all(or_domain *d, double dtrk);
void   or_updt_pressure_all(or_domain *d, double alpha);
double or_chkdt(or_domain *d);                            /* dt_cfl, incl. MPI reductions */
void   or_chkdiv(or_domain *d, double *divtot, double *divmax);
double or_kinetic_energy(or_domain *d);
/* whole RK3 steps, main.f90:893-1069 (dt from chkdt every icheck steps) */
int    or_step(or_domain *d, int nsteps);
double or_dt(const or_domain *d);
void   or_set_dt(or_domain *d, double dt);
int    or_istep(const or_domain *d);
double or_time(const or_domain *d);
/* solver statistics of the last solve */
int    or_last_iterations(const or_domain *d);
double or_last_residual(const or_domain *d);
void   or_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
