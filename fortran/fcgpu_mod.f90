! fcgpu_mod.f90 -- ISO_C_BINDING module that lets freeCappuccino call libfcgpu.so in
! place of its pressure-correction routines.
!
! Not compiled in this repository: the image it is built in has no Fortran compiler.
! It is meant to be added to the reference's src/ and compiled with its other modules
! (it uses the reference's modules types, parameters, geometry, sparse_matrix,
! variables and title_mod), then linked with
!   -L$FCG/freecappuccino_gb300/_build -lfcgpu -Wl,-rpath,$FCG/freecappuccino_gb300/_build
!
! The interfaces follow include/fcgpu.h one for one (argument order, value / reference
! passing, 1-based index arrays).  The subroutines at the end have the names and
! argument lists of the reference routines they replace, so that their callers keep
! their call lines:
!   laplacian(mu,phi)   fvm_laplacian.f90:1
!   bpres(p,istage)     bpres.f90:3
!   dpcg(fi,ifi)        dpcg.f90:3
!   iccg(fi,ifi)        iccg.f90:3
!   bicgstab(fi,ifi)    bicgstab.f90:1
! The reference's own files for these routines then drop out of its build.  Every call
! returns a status: a non-zero status stops the run with the library's message, which is
! the reference's own reaction to bad input.  On a mesh with O-C grid cuts (noc > 0)
! laplacian, bpres, dpcg, iccg and bicgstab carry the pairs (ar, al through the array
! aoc); the face-flux calls take flmass followed by fmoc in one array.
module fcgpu
  use iso_c_binding
  implicit none
  private
  public :: fcg_init, fcg_finish, laplacian, bpres, dpcg, iccg, bicgstab, dpcg_mixed, &
            fcg_check, fcg_ctx

  type(c_ptr), save :: fcg_ctx = c_null_ptr

  ! include/fcgpu.h: fcg_mesh_desc
  type, bind(c) :: fcg_mesh_desc
    integer(c_int) :: numCells, numFaces, numInnerFaces
    integer(c_int) :: ninl, nout, nsym, nwal, npru
    integer(c_int) :: iInletFacesStart, iOutletFacesStart, iSymmetryFacesStart, &
                      iWallFacesStart, iPressOutletFacesStart, noc
    type(c_ptr) :: owner, neighbour, arx, ary, arz, xf, yf, zf, xc, yc, zc, vol, facint
    integer(c_int) :: ncyc, iOCFacesStart
    type(c_ptr) :: ijlFace, ijrFace
  end type

  ! With O-C grid cuts (noc > 0) the library takes a matrix as one array: the CSR values
  ! a(1:nnz), then ar(1:noc), then al(1:noc) (module sparse_matrix's ar, al).
  real(c_double), allocatable, save :: aoc(:)

  ! include/fcgpu.h: fcg_solve_report
  type, bind(c) :: fcg_solve_report
    real(c_double) :: res0, resl
    integer(c_int) :: iters, converged
    real(c_double) :: l2_rel, seconds
  end type

  ! include/fcgpu.h: fcg_flow_fields (addresses of the calcp fields)
  type, bind(c), public :: fcg_flow_fields
    type(c_ptr) :: u, v, w, p, dUdxi, dVdxi, dWdxi, dPdxi, apu, apv, apw, den
  end type

  interface
    function fcg_last_error(ctx) bind(c) result(msg)
      import; type(c_ptr), value :: ctx; type(c_ptr) :: msg
    end function
    integer(c_int) function fcg_create(ctx, device) bind(c)
      import; type(c_ptr) :: ctx; integer(c_int), value :: device
    end function
    integer(c_int) function fcg_destroy(ctx) bind(c)
      import; type(c_ptr), value :: ctx
    end function
    integer(c_int) function fcg_bind_mesh(ctx, m) bind(c)
      import; type(c_ptr), value :: ctx; type(fcg_mesh_desc) :: m
    end function
    integer(c_int) function fcg_create_csr(ctx, ioffset, ja, diag, spn, snp) bind(c)
      import; type(c_ptr), value :: ctx
      integer(c_int) :: ioffset(*), ja(*), diag(*), spn(*), snp(*)
    end function
    integer(c_int) function fcg_laplacian(ctx, mu, phi, a, su) bind(c)
      import; type(c_ptr), value :: ctx; real(c_double) :: mu(*), phi(*), a(*), su(*)
    end function
    integer(c_int) function fcg_facefluxmass(ctx, f, a, su, flmass) bind(c)
      import; type(c_ptr), value :: ctx; type(fcg_flow_fields) :: f
      real(c_double) :: a(*), su(*), flmass(*)
    end function
    integer(c_int) function fcg_fluxmc(ctx, dPdxi, apu, den, su, flmass) bind(c)
      import; type(c_ptr), value :: ctx
      real(c_double) :: dPdxi(*), apu(*), den(*), su(*), flmass(*)
    end function
    integer(c_int) function fcg_flux_correct(ctx, a, pp, flmass) bind(c)
      import; type(c_ptr), value :: ctx; real(c_double) :: a(*), pp(*), flmass(*)
    end function
    integer(c_int) function fcg_correct_fields(ctx, dPdxi, apu, apv, apw, pp, urf, pRefCell, &
                                               u, v, w, p) bind(c)
      import; type(c_ptr), value :: ctx
      real(c_double) :: dPdxi(*), apu(*), apv(*), apw(*), pp(*), u(*), v(*), w(*), p(*)
      real(c_double), value :: urf; integer(c_int), value :: pRefCell
    end function
    integer(c_int) function fcg_grad(ctx, phi, dphidxi, method, nigrad) bind(c)
      import; type(c_ptr), value :: ctx; real(c_double) :: phi(*), dphidxi(*)
      integer(c_int), value :: method, nigrad
    end function
    integer(c_int) function fcg_grad_lsq_matrix(ctx, dmat) bind(c)
      import; type(c_ptr), value :: ctx; real(c_double) :: dmat(*)
    end function
    integer(c_int) function fcg_bpres(ctx, p, dpdxi, istage) bind(c)
      import; type(c_ptr), value :: ctx; real(c_double) :: p(*), dpdxi(*)
      integer(c_int), value :: istage
    end function
    integer(c_int) function fcg_dpcg(ctx, a, su, fi, res, sor, nsw, resor, rep) bind(c)
      import; type(c_ptr), value :: ctx; real(c_double) :: a(*), su(*), fi(*), res(*)
      real(c_double), value :: sor; integer(c_int), value :: nsw
      real(c_double) :: resor; type(fcg_solve_report) :: rep
    end function
    integer(c_int) function fcg_iccg(ctx, a, su, fi, res, sor, nsw, resor, rep) bind(c)
      import; type(c_ptr), value :: ctx; real(c_double) :: a(*), su(*), fi(*), res(*)
      real(c_double), value :: sor; integer(c_int), value :: nsw
      real(c_double) :: resor; type(fcg_solve_report) :: rep
    end function
    integer(c_int) function fcg_bicgstab(ctx, a, su, fi, res, sor, nsw, resor, rep) bind(c)
      import; type(c_ptr), value :: ctx; real(c_double) :: a(*), su(*), fi(*), res(*)
      real(c_double), value :: sor; integer(c_int), value :: nsw
      real(c_double) :: resor; type(fcg_solve_report) :: rep
    end function
    integer(c_int) function fcg_dpcg_mixed(ctx, a, su, fi, res, sor, nsw, resor, rep) bind(c)
      import; type(c_ptr), value :: ctx; real(c_double) :: a(*), su(*), fi(*), res(*)
      real(c_double), value :: sor; integer(c_int), value :: nsw
      real(c_double) :: resor; type(fcg_solve_report) :: rep
    end function
    function c_strlen(s) bind(c, name='strlen') result(n)
      import; type(c_ptr), value :: s; integer(c_size_t) :: n
    end function
  end interface

  ! status of the last fcg_* call of this module (0 = FCG_OK)
  integer(c_int), public, save :: fcg_status = 0

contains

  ! Stops the run with the library's message when a call failed.
  subroutine fcg_check(rc, where)
    integer(c_int), intent(in) :: rc
    character(*), intent(in) :: where
    character(kind=c_char), pointer :: chars(:)
    type(c_ptr) :: msg
    integer :: n
    fcg_status = rc
    if (rc == 0) return
    msg = fcg_last_error(fcg_ctx)
    if (c_associated(msg)) then
      n = int(c_strlen(msg))
      call c_f_pointer(msg, chars, [n])
      write(6,'(4a)') 'fcgpu: ', where, ' failed: ', transfer(chars(1:n), repeat(' ', n))
    else
      write(6,'(3a,i0)') 'fcgpu: ', where, ' failed with status ', rc
    end if
    stop 1
  end subroutine

  ! Once, after mesh_geometry (mesh_geometry_and_topology.f90:310) and before the time
  ! loop; replaces create_CSR_matrix_from_mesh_data (sparse_matrix.f90:42-172).  The
  ! Fortran CSR arrays stay authoritative: the library writes them (bit-exact).
  subroutine fcg_init(device)
    use geometry
    use sparse_matrix
    integer, intent(in), optional :: device
    type(fcg_mesh_desc), target, save :: m
    integer(c_int) :: dev
    type(c_ptr) :: pl, pr
    dev = 0
    if (present(device)) dev = device
    call fcg_check(fcg_create(fcg_ctx, dev), 'fcg_create')
    pl = c_null_ptr
    pr = c_null_ptr
    if (noc > 0) then  ! noc = noc + ncyc after mesh_geometry (:1163)
      pl = c_loc(ijlFace)
      pr = c_loc(ijrFace)
      allocate(aoc(nnz + 2*noc))
    end if
    m = fcg_mesh_desc(numCells, numFaces, numInnerFaces, ninl, nout, nsym, nwal, npru, &
        iInletFacesStart, iOutletFacesStart, iSymmetryFacesStart, iWallFacesStart,     &
        iPressOutletFacesStart, noc, c_loc(owner), c_loc(neighbour), c_loc(arx),       &
        c_loc(ary), c_loc(arz), c_loc(xf), c_loc(yf), c_loc(zf), c_loc(xc), c_loc(yc), &
        c_loc(zc), c_loc(vol), c_loc(facint), ncyc, iOCFacesStart, pl, pr)
    call fcg_check(fcg_bind_mesh(fcg_ctx, m), 'fcg_bind_mesh')
    allocate(ioffset(numCells+1), ja(nnz), diag(numCells), a(nnz))
    allocate(icell_jcell_csr_value_index(numInnerFaces), jcell_icell_csr_value_index(numInnerFaces))
    call fcg_check(fcg_create_csr(fcg_ctx, ioffset, ja, diag, icell_jcell_csr_value_index, &
                                  jcell_icell_csr_value_index), 'fcg_create_csr')
  end subroutine

  subroutine fcg_finish
    if (c_associated(fcg_ctx)) call fcg_check(fcg_destroy(fcg_ctx), 'fcg_destroy')
    fcg_ctx = c_null_ptr
    if (allocated(aoc)) deallocate(aoc)
  end subroutine

  ! laplacian(mu,phi) (fvm_laplacian.f90:1-163): writes the module arrays a and su.
  ! With O-C pairs also ar and al (:67-86).
  subroutine laplacian(mu, phi)
    use types; use geometry, only: numCells, numTotal, noc
    use sparse_matrix, only: a, su, ar, al, nnz
    real(dp), dimension(numCells), intent(in) :: mu
    real(dp), dimension(numTotal), intent(in) :: phi
    if (noc == 0) then
      call fcg_check(fcg_laplacian(fcg_ctx, mu, phi, a, su), 'laplacian')
    else
      call fcg_check(fcg_laplacian(fcg_ctx, mu, phi, aoc, su), 'laplacian')
      a(1:nnz) = aoc(1:nnz)
      ar(1:noc) = aoc(nnz+1:nnz+noc)
      al(1:noc) = aoc(nnz+noc+1:nnz+2*noc)
    end if
  end subroutine

  ! aoc = [a, ar, al] for a solve on a mesh with O-C pairs.
  subroutine pack_oc
    use geometry, only: noc; use sparse_matrix, only: a, ar, al, nnz
    aoc(1:nnz) = a(1:nnz)
    aoc(nnz+1:nnz+noc) = ar(1:noc)
    aoc(nnz+noc+1:nnz+2*noc) = al(1:noc)
  end subroutine

  ! bpres(p,istage) (bpres.f90:3-152), with the module gradient dPdxi(3,numCells).
  subroutine bpres(p, istage)
    use types; use geometry, only: numTotal; use variables, only: dPdxi
    real(dp), dimension(numTotal) :: p
    integer, intent(in) :: istage
    call fcg_check(fcg_bpres(fcg_ctx, p, dPdxi, int(istage, c_int)), 'bpres')
  end subroutine

  ! The solvers: same arguments and module state as dpcg/iccg/bicgstab, same stop test
  ! resl/(res0+small) < sor(ifi), resor(ifi) set, and the reference's log line.
  subroutine dpcg(fi, ifi)
    use types; use parameters; use sparse_matrix; use title_mod; use geometry, only: noc
    real(dp), intent(inout) :: fi(*)
    integer, intent(in) :: ifi
    type(fcg_solve_report) :: rep
    if (noc == 0) then
      call fcg_check(fcg_dpcg(fcg_ctx, a, su, fi, res, sor(ifi), int(nsw(ifi), c_int), &
                              resor(ifi), rep), 'dpcg')
    else
      call pack_oc
      call fcg_check(fcg_dpcg(fcg_ctx, aoc, su, fi, res, sor(ifi), int(nsw(ifi), c_int), &
                              resor(ifi), rep), 'dpcg')
    end if
    call solver_log('PCG(Jacobi):  ', ifi, rep)
  end subroutine

  subroutine iccg(fi, ifi)
    use types; use parameters; use sparse_matrix; use title_mod; use geometry, only: noc
    real(dp), intent(inout) :: fi(*)
    integer, intent(in) :: ifi
    type(fcg_solve_report) :: rep
    if (noc == 0) then
      call fcg_check(fcg_iccg(fcg_ctx, a, su, fi, res, sor(ifi), int(nsw(ifi), c_int), &
                              resor(ifi), rep), 'iccg')
    else
      call pack_oc
      call fcg_check(fcg_iccg(fcg_ctx, aoc, su, fi, res, sor(ifi), int(nsw(ifi), c_int), &
                              resor(ifi), rep), 'iccg')
    end if
    call solver_log('  PCG(IC0):  ', ifi, rep)
  end subroutine

  subroutine bicgstab(fi, ifi)
    use types; use parameters; use sparse_matrix; use title_mod; use geometry, only: noc
    real(dp), intent(inout) :: fi(*)
    integer, intent(in) :: ifi
    type(fcg_solve_report) :: rep
    if (noc == 0) then
      call fcg_check(fcg_bicgstab(fcg_ctx, a, su, fi, res, sor(ifi), int(nsw(ifi), c_int), &
                                  resor(ifi), rep), 'bicgstab')
    else
      call pack_oc
      call fcg_check(fcg_bicgstab(fcg_ctx, aoc, su, fi, res, sor(ifi), int(nsw(ifi), c_int), &
                                  resor(ifi), rep), 'bicgstab')
    end if
    call solver_log('  BiCGStab(ILU(0)):  ', ifi, rep)
  end subroutine

  ! dpcg with FP32 sweeps under FP64 reliable updates (no reference counterpart; the
  ! same stop test on the true FP64 residual), a drop-in for dpcg(fi,ifi).
  subroutine dpcg_mixed(fi, ifi)
    use types; use parameters; use sparse_matrix; use title_mod
    real(dp), intent(inout) :: fi(*)
    integer, intent(in) :: ifi
    type(fcg_solve_report) :: rep
    call fcg_check(fcg_dpcg_mixed(fcg_ctx, a, su, fi, res, sor(ifi), int(nsw(ifi), c_int), &
                                  resor(ifi), rep), 'dpcg_mixed')
    call solver_log('PCG(Jacobi, FP32 sweeps):  ', ifi, rep)
  end subroutine

  ! The reference's per-solve line (dpcg.f90:150, iccg.f90:328, bicgstab.f90:227).
  subroutine solver_log(name, ifi, rep)
    use title_mod
    character(*), intent(in) :: name
    integer, intent(in) :: ifi
    type(fcg_solve_report), intent(in) :: rep
    write(6,'(4a,1PE10.3,a,1PE10.3,a,I0)') name, 'Solving for ', trim(chvarSolver(ifi)), &
      ', Initial residual = ', rep%res0, ', Final residual = ', rep%resl, &
      ', No Iterations ', rep%iters
  end subroutine

end module fcgpu
