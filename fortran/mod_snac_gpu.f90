! mod_snac_gpu.f90 -- iso_c_binding interfaces of libsnac_gb300 (include/snac_gpu.h) for SNaC's Fortran
! driver: the reference-signature calls (one block, the driver's own arrays), the per-block boundary routines,
! and the domain-level calls that replace the MPI halo exchange and the HYPRE/FFTW solves.  Not compiled on the
! machines this library is built on (no Fortran compiler there); it follows the C header declaration by
! declaration.
module mod_snac_gpu
  use, intrinsic :: iso_c_binding
  use, intrinsic :: iso_fortran_env, only: stderr => error_unit
  implicit none
  ! field kinds (enum of snac_gpu.h)
  integer(c_int), parameter :: SNAC_U = 0, SNAC_V = 1, SNAC_W = 2, SNAC_P = 3, SNAC_PP = 4, SNAC_S0 = 9
  integer(c_int), parameter :: SNAC_MAX_SCAL = 4
  ! the arguments of snac_init: the same members in the same order as the C structs (the C arrays' dimensions
  ! reversed, so side and direction run fastest as in the reference's block_cbcvel(side,dir,comp))
  ! one &blocks entry (param.f90:332-360); a friend link 'F' carries the neighbour's 1-based id in the value
  type, bind(C) :: snac_block_desc
    integer(c_int)         :: ng(3)
    real(c_double)         :: lmin(3), lmax(3)
    integer(c_int)         :: gt(3)
    real(c_double)         :: gr(3)
    character(kind=c_char) :: cbcvel(2,3,3)
    real(c_double)         :: bcvel(2,3,3)
    character(kind=c_char) :: cbcpre(2,3)
    real(c_double)         :: bcpre(2,3)
    character(kind=c_char) :: cbcscal(2,3,SNAC_MAX_SCAL)
    real(c_double)         :: bcscal(2,3,SNAC_MAX_SCAL)
    type(c_ptr)            :: grid_file(3)       ! c_loc of grid/grid_?_b_###.bin contents, or c_null_ptr
    integer(c_int)         :: inflow_type(2,3)
  end type
  ! &dns, &scalar and &hypre (param.f90:342-355) plus the build flags
  type, bind(C) :: snac_case
    integer(c_int) :: nblocks
    real(c_double) :: visci, cfl, dtmax, dt_f
    real(c_double) :: bforce(3), gacc(3), beta
    integer(c_int) :: nscal
    real(c_double) :: alphai(SNAC_MAX_SCAL), ssource(SNAC_MAX_SCAL), scalf(SNAC_MAX_SCAL)
    integer(c_int) :: is_sforced(SNAC_MAX_SCAL)
    integer(c_int) :: icheck
    integer(c_int) :: fft_axis                   ! 0: 3-D solve; 1, 2, 3: FFT_AXIS
    integer(c_int) :: impdiff                    ! _IMPDIFF
    integer(c_int) :: boussinesq                 ! _BOUSSINESQ_BUOYANCY
    real(c_double) :: tol                        ! hypre_tol
    integer(c_int) :: maxiter                    ! hypre_maxiter
  end type
  ! library options (no reference counterpart); zero selects each default
  type, bind(C) :: snac_options
    integer(c_int) :: precision = 1              ! 0 plain FP64 multigrid-PCG, 1 FP32 V-cycles in FP64 refinement
    integer(c_int) :: use_graph = 1              ! replay each refinement step as a CUDA graph
    integer(c_int) :: nu = 0
    integer(c_int) :: device = 0
    integer(c_int) :: nu_coarse = 0
    integer(c_int) :: inner_iters = 0
    real(c_double) :: inner_tol = 0
    integer(c_int) :: inner_adapt = 0
    integer(c_int) :: refine_steps = 0
    integer(c_int) :: mg_fuse = 0
    integer(c_int) :: mg_cta_level = 0
    integer(c_int) :: mg_tile = 0
    integer(c_int) :: mg_waves = 0
    integer(c_int) :: mg_red_batch = 0
    integer(c_int) :: mg_lnu = 0
    integer(c_int) :: tma = 0
    integer(c_int) :: pdl = 0
    integer(c_int) :: mg_inv = 0
    integer(c_int) :: mg_restrict = 0
  end type
  interface
    ! rk.f90:7-128 -- u,v,w,p halo'd; dudtrko interior; s1 = scalars(1)%val or c_null_ptr
    integer(c_int) function snac_rk_mom(rkpar,lo,hi,dxc,dxf,dyc,dyf,dzc,dzf,dt,bforce,gacc,beta,s1,visc, &
                                        u,v,w,p,dudtrko,dvdtrko,dwdtrko,impdiff,boussinesq) bind(C,name='snac_rk_mom')
      import
      real(c_double), intent(in) :: rkpar(2), bforce(3), gacc(3)
      integer(c_int), intent(in) :: lo(3), hi(3)
      real(c_double), intent(in) :: dxc(*), dxf(*), dyc(*), dyf(*), dzc(*), dzf(*)
      real(c_double), value :: dt, beta, visc
      type(c_ptr), value :: s1
      real(c_double) :: u(*), v(*), w(*), p(*), dudtrko(*), dvdtrko(*), dwdtrko(*)
      integer(c_int), value :: impdiff, boussinesq
    end function
    ! rk.f90:130-204 (rk_scal) + scal.f90:89-179; f = scalf - bulk mean when is_forced
    integer(c_int) function snac_rk_scal(rkpar,lo,hi,dxc,dxf,dyc,dyf,dzc,dzf,dt,alpha,vol_all,u,v,w, &
                                         is_forced,scalf,ssource,dsdtrko,s,f,impdiff) bind(C,name='snac_rk_scal')
      import
      real(c_double), intent(in) :: rkpar(2)
      integer(c_int), intent(in) :: lo(3), hi(3)
      real(c_double), intent(in) :: dxc(*), dxf(*), dyc(*), dyf(*), dzc(*), dzf(*), u(*), v(*), w(*)
      real(c_double), value :: dt, alpha, vol_all, scalf, ssource
      integer(c_int), value :: is_forced, impdiff
      real(c_double) :: dsdtrko(*), s(*), f
    end function
    ! fillps.f90:7-54 (fft_axis 0..3 selects the _FFT_X/_Y/_Z weighting)
    integer(c_int) function snac_fillps(lo,hi,dxf,dyf,dzf,dt,u,v,w,p,fft_axis) bind(C,name='snac_fillps')
      import
      integer(c_int), intent(in) :: lo(3), hi(3)
      real(c_double), intent(in) :: dxf(*), dyf(*), dzf(*), u(*), v(*), w(*)
      real(c_double), value :: dt
      real(c_double) :: p(*)
      integer(c_int), value :: fft_axis
    end function
    ! correc.f90:7-48
    integer(c_int) function snac_correc(lo,hi,dxc,dyc,dzc,dt,p,u,v,w) bind(C,name='snac_correc')
      import
      integer(c_int), intent(in) :: lo(3), hi(3)
      real(c_double), intent(in) :: dxc(*), dyc(*), dzc(*), p(*)
      real(c_double), value :: dt
      real(c_double) :: u(*), v(*), w(*)
    end function
    ! updt_pressure.f90:7-47
    integer(c_int) function snac_updt_pressure(lo,hi,dxc,dxf,dyc,dyf,dzc,dzf,alpha,pp,p,impdiff) &
                   bind(C,name='snac_updt_pressure')
      import
      integer(c_int), intent(in) :: lo(3), hi(3)
      real(c_double), intent(in) :: dxc(*), dxf(*), dyc(*), dyf(*), dzc(*), dzf(*), pp(*)
      real(c_double), value :: alpha
      real(c_double) :: p(*)
      integer(c_int), value :: impdiff
    end function
    ! bound.f90:543-585; is_bound(0:1,3) as integer (side fastest)
    integer(c_int) function snac_updt_rhs(lo,hi,is_bound,rhsx,rhsy,rhsz,p) bind(C,name='snac_updt_rhs')
      import
      integer(c_int), intent(in) :: lo(3), hi(3), is_bound(0:1,3)
      real(c_double), intent(in) :: rhsx(*), rhsy(*), rhsz(*)
      real(c_double) :: p(*)
    end function
    ! chkdt.f90:8-56 (one block); the MPI_ALLREDUCE stays in the caller
    integer(c_int) function snac_chkdt(lo,hi,dxc,dxf,dyc,dyf,dzc,dzf,visc,u,v,w,impdiff,dtmax) &
                   bind(C,name='snac_chkdt')
      import
      integer(c_int), intent(in) :: lo(3), hi(3)
      real(c_double), intent(in) :: dxc(*), dxf(*), dyc(*), dyf(*), dzc(*), dzf(*), u(*), v(*), w(*)
      real(c_double), value :: visc
      integer(c_int), value :: impdiff
      real(c_double), intent(out) :: dtmax
    end function
    ! chkdiv.f90:8-44 (one block); the MPI reductions stay in the caller
    integer(c_int) function snac_chkdiv(lo,hi,dxf,dyf,dzf,u,v,w,vol,divtot,divmax) bind(C,name='snac_chkdiv')
      import
      integer(c_int), intent(in) :: lo(3), hi(3)
      real(c_double), intent(in) :: dxf(*), dyf(*), dzf(*), u(*), v(*), w(*)
      real(c_double), value :: vol
      real(c_double), intent(out) :: divtot, divmax
    end function
    ! bound.f90:108-248 (set_bc) on one face of one array
    integer(c_int) function snac_set_bc(ctype,ibound,lo,hi,idir,centered,rvalue,dr,p) bind(C,name='snac_set_bc')
      import
      character(kind=c_char), value :: ctype
      integer(c_int), value :: ibound, idir, centered
      integer(c_int), intent(in) :: lo(3), hi(3)
      real(c_double), value :: rvalue, dr
      real(c_double) :: p(*)
    end function
    ! fft.f90:85-94; kind from snac_find_fft (fft.f90:96-149)
    integer(c_int) function snac_fft(kind,idir,n,q,arr) bind(C,name='snac_fft')
      import
      integer(c_int), value :: kind, idir, q
      integer(c_int), intent(in) :: n(3)
      real(c_double) :: arr(*)
    end function
    ! host mirrors: keep a device copy of a Fortran array (no copies inside the time loop)
    integer(c_int) function snac_register(host,bytes) bind(C,name='snac_register')
      import
      type(c_ptr), value :: host
      integer(c_size_t), value :: bytes
    end function
    integer(c_int) function snac_update_host(host) bind(C,name='snac_update_host')
      import
      type(c_ptr), value :: host
    end function
    integer(c_int) function snac_update_device(host) bind(C,name='snac_update_device')
      import
      type(c_ptr), value :: host
    end function
    function snac_last_error() bind(C,name='snac_last_error')
      import
      type(c_ptr) :: snac_last_error
    end function
    ! bound.f90:8-66 (bounduvw) for one block: halo faces whose neighbour is this rank exchanged on the device,
    ! the others left to the driver's MPI exchange; cbc(0:1,3,3), bc(0:1,3,3), is_bound/nb(0:1,3) as integers
    integer(c_int) function snac_bounduvw(cbc,lo,hi,bc,is_correc,is_bound,nb,myrank,dxc,dxf,dyc,dyf,dzc,dzf, &
                                          u,v,w) bind(C,name='snac_bounduvw')
      import
      character(kind=c_char), intent(in) :: cbc(0:1,3,3)
      integer(c_int), intent(in) :: lo(3), hi(3), is_bound(0:1,3), nb(0:1,3)
      real(c_double), intent(in) :: bc(0:1,3,3), dxc(*), dxf(*), dyc(*), dyf(*), dzc(*), dzf(*)
      integer(c_int), value :: is_correc, myrank
      real(c_double) :: u(*), v(*), w(*)
    end function
    ! bound.f90:68-106 (boundp) for one block
    integer(c_int) function snac_boundp(cbc,lo,hi,bc,is_bound,nb,myrank,dxc,dyc,dzc,p) bind(C,name='snac_boundp')
      import
      character(kind=c_char), intent(in) :: cbc(0:1,3)
      integer(c_int), intent(in) :: lo(3), hi(3), is_bound(0:1,3), nb(0:1,3)
      real(c_double), intent(in) :: bc(0:1,3), dxc(*), dyc(*), dzc(*)
      integer(c_int), value :: myrank
      real(c_double) :: p(*)
    end function
    ! open / outflow boundaries of one block (bound.f90:250-541); logical masks passed as 0/1 integers
    integer(c_int) function snac_set_open_bc_uvw(ibound,lo,hi,idir,visc,dr,u,v,w,p,tr) bind(C,name='snac_set_open_bc_uvw')
      import
      integer(c_int), value :: ibound, idir
      integer(c_int), intent(in) :: lo(3), hi(3)
      real(c_double), value :: visc, dr
      real(c_double) :: u(*), v(*), w(*), tr(*)
      real(c_double), intent(in) :: p(*)
    end function
    integer(c_int) function snac_set_open_bc_p(ibound,lo,hi,idir,drc,drf,alpha,p) bind(C,name='snac_set_open_bc_p')
      import
      integer(c_int), value :: ibound, idir
      integer(c_int), intent(in) :: lo(3), hi(3)
      real(c_double), intent(in) :: drc(0:1)
      real(c_double), value :: drf, alpha
      real(c_double) :: p(*)
    end function
    integer(c_int) function snac_cmpt_estimated_traction(ibound,lo,hi,idir,visc,dr,u,v,w,p,tr) &
        bind(C,name='snac_cmpt_estimated_traction')
      import
      integer(c_int), value :: ibound, idir
      integer(c_int), intent(in) :: lo(3), hi(3)
      real(c_double), value :: visc, dr
      real(c_double), intent(in) :: u(*), v(*), w(*), p(*)
      real(c_double) :: tr(*)
    end function
    integer(c_int) function snac_outflow(is_outflow_bound,is_estimated_traction,lo,hi,dl,dl_h,visc,u,v,w,p, &
        tr_x,tr_y,tr_z) bind(C,name='snac_outflow')
      import
      integer(c_int), intent(in) :: is_outflow_bound(0:1,3), is_estimated_traction(0:1,3), lo(3), hi(3)
      real(c_double), intent(in) :: dl(0:1,3), dl_h(0:1,3)
      real(c_double), value :: visc
      real(c_double) :: u(*), v(*), w(*), p(*), tr_x(*), tr_y(*), tr_z(*)
    end function
    integer(c_int) function snac_outflow_p(is_outflow_bound,lo,hi,dlc,dlf,alpha,p) bind(C,name='snac_outflow_p')
      import
      integer(c_int), intent(in) :: is_outflow_bound(0:1,3), lo(3), hi(3)
      real(c_double), intent(in) :: dlc(0:1,0:1,3), dlf(0:1,3)
      real(c_double), value :: alpha
      real(c_double) :: p(*)
    end function
    ! domain layer: every block placed, gridded and resident on the GPU, solvers built (initmpi.f90, initgrid.f90,
    ! solver.f90 set-up); nblocks entries in blocks
    integer(c_int) function snac_init(c,blocks,opt) bind(C,name='snac_init')
      import
      type(snac_case), intent(in) :: c
      type(snac_block_desc), intent(in) :: blocks(*)
      type(snac_options), intent(in) :: opt
    end function
    ! domain layer (all blocks resident on the GPU after snac_init): the per-stage routines of main.f90:906-1043
    integer(c_int) function snac_rk_mom_all(irk) bind(C,name='snac_rk_mom_all')
      import
      integer(c_int), value :: irk
    end function
    integer(c_int) function snac_bounduvw_all(is_correc) bind(C,name='snac_bounduvw_all')
      import
      integer(c_int), value :: is_correc
    end function
    integer(c_int) function snac_boundp_all(field) bind(C,name='snac_boundp_all')
      import
      integer(c_int), value :: field
    end function
    integer(c_int) function snac_fillps_all(dtrk) bind(C,name='snac_fillps_all')
      import
      real(c_double), value :: dtrk
    end function
    ! solve_impdiff_field (solve_helmholtz.f90:32-138) of one field: SNAC_U, SNAC_V, SNAC_W or SNAC_S0 + s
    integer(c_int) function snac_impdiff_solve(field,alphai_new,alphai_old) bind(C,name='snac_impdiff_solve')
      import
      integer(c_int), value :: field
      real(c_double), value :: alphai_new, alphai_old
    end function
    integer(c_int) function snac_updt_rhs_all() bind(C,name='snac_updt_rhs_all')
      import
    end function
    integer(c_int) function snac_solve_pressure() bind(C,name='snac_solve_pressure')
      import
    end function
    integer(c_int) function snac_correc_all(dtrk) bind(C,name='snac_correc_all')
      import
      real(c_double), value :: dtrk
    end function
    integer(c_int) function snac_updt_pressure_all(alpha) bind(C,name='snac_updt_pressure_all')
      import
      real(c_double), value :: alpha
    end function
    integer(c_int) function snac_chkdt_all(dt_cfl) bind(C,name='snac_chkdt_all')
      import
      real(c_double), intent(out) :: dt_cfl
    end function
    integer(c_int) function snac_chkdiv_all(divtot,divmax) bind(C,name='snac_chkdiv_all')
      import
      real(c_double), intent(out) :: divtot, divmax
    end function
    ! whole RK3 steps (main.f90:893-1069)
    integer(c_int) function snac_step(nsteps) bind(C,name='snac_step')
      import
      integer(c_int), value :: nsteps
    end function
    ! copies between the driver's arrays and the resident fields of block ib (field kinds of snac_gpu.h)
    integer(c_int) function snac_set_field(ib,field,host) bind(C,name='snac_set_field')
      import
      integer(c_int), value :: ib, field
      real(c_double), intent(in) :: host(*)
    end function
    integer(c_int) function snac_get_field(ib,field,host) bind(C,name='snac_get_field')
      import
      integer(c_int), value :: ib, field
      real(c_double) :: host(*)
    end function
    integer(c_int) function snac_finalize() bind(C,name='snac_finalize')
      import
    end function
  end interface
contains
  subroutine snac_check(ierr)
    integer(c_int), intent(in) :: ierr
    if(ierr /= 0) then
      write(stderr,*) 'ERROR: snac_gb300 call failed with code ', ierr
      error stop
    end if
  end subroutine
end module mod_snac_gpu
