! fibmd_gpu_mod: ISO_C_BINDING interface of libfibmd_gpu for a Fortran host.
!
! The reference's driver calls its hot path as module subroutines from
! onestep (src/timeint.f90:158-242); a GPU build of bin/mdrun2 uses this
! module instead: fibmd_gpu_create / upload / nlist after init
! (src/main.f90:45-65), fibmd_gpu_steps in place of the TI loop's onestep
! calls, fibmd_gpu_download at dump steps before writeatoms / writerestart
! (src/out.f90:34-100), and fibmd_gpu_set_atom after knock
! (src/knock.f90:21-55). Every binding follows include/fibmd_gpu.h; the
! type fibmd_params has the C struct's fields in order (bind(C) gives the
! same layout and padding). Per-atom arrays are the reference's
! column-major X(Natm,3) arrays; atom indices are 1-based.
!
! Build: gfortran -c fibmd_gpu_mod.f90, link the host with
! -L<package dir> -lfibmd_gpu.
module fibmd_gpu_mod
  use iso_c_binding
  implicit none

  ! status codes
  integer(c_int), parameter :: FIBMD_OK = 0, FIBMD_EINVAL = 1, FIBMD_ECUDA = 2, &
       FIBMD_EOVERFLOW = 3, FIBMD_ENAN = 4, FIBMD_ETIMEOUT = 5, FIBMD_ESTATE = 6, &
       FIBMD_ENOMEM = 7, FIBMD_ETABLE = 8
  ! modes and precisions
  integer(c_int), parameter :: FIBMD_MODE_REF = 0, FIBMD_MODE_SPEC = 1
  integer(c_int), parameter :: FIBMD_PREC_FP64 = 0, FIBMD_PREC_MIXED = 1
  ! spec-mode per-atom tags
  integer(c_int32_t), parameter :: FIBMD_TAG_FROZEN = 1, FIBMD_TAG_THERMO = 2, &
       FIBMD_TAG_REMOVED = 4
  ! why fibmd_gpu_steps returned (bits)
  integer(c_int), parameter :: FIBMD_STOP_MAXSTEPS = 1, FIBMD_STOP_DUMP = 2, &
       FIBMD_STOP_DONE = 4, FIBMD_STOP_REGIME = 8

  type, bind(C) :: fibmd_params
     integer(c_int) :: abi_version, mode, precision, Natm, Nsg, Nlj
     real(c_double) :: Lb(3)
     real(c_double) :: A, B, psi, qsi, al, gamma
     real(c_double) :: lambdaSi, lambdaGe, epsSi, epsGe, sigmaSi, sigmaGe
     real(c_double) :: massSi, massGe, massGa
     real(c_double) :: ZSi, ZGe, ZGa
     real(c_double) :: Amol, Bmol, Cmol, alpha_mol, beta_mol, gamma_mol
     real(c_double) :: kB, eps0, ec, ao
     real(c_double) :: listfac
     integer(c_int) :: Ntable
     real(c_double) :: Ts_i, Ts_r
     real(c_double) :: Ttar1
     real(c_double) :: ke_limit_1
     real(c_double) :: Tau_i, Tau_r
     real(c_double) :: Teps
     integer(c_int) :: ntlist_i, ntlist_r, atlist_i, atlist_r, dslist_i, dslist_r
     integer(c_int) :: atm_out_i, atm_out_r, res_out
     real(c_double) :: outz(4), atomz(2), ionz, knockz
     real(c_double) :: sidewidth
     real(c_double) :: dti
     real(c_double) :: dt_max
     real(c_double) :: dx_max
     real(c_double) :: tau_spec
     real(c_double) :: remove_z
     real(c_double) :: mixed_mol_fp64_r
     real(c_double) :: list_skin
     integer(c_int) :: max_sw_nbrs
     integer(c_int) :: max_mol_pairs
     integer(c_int) :: reserved(8)
  end type fibmd_params

  ! one replica of a batched ensemble (fibmd_gpu_batch_create)
  type, bind(C) :: fibmd_replica
     integer(c_int) :: natm, nsg
     real(c_double) :: Lb(3)
     real(c_double) :: remove_z
     integer(c_int) :: reserved(4)
  end type fibmd_replica

  interface
     integer(c_int) function fibmd_gpu_abi_version() bind(C)
       import
     end function fibmd_gpu_abi_version

     integer(c_int) function fibmd_gpu_params_size() bind(C)
       import
     end function fibmd_gpu_params_size

     integer(c_int) function fibmd_gpu_params_default(p) bind(C)
       import
       type(fibmd_params) :: p
     end function fibmd_gpu_params_default

     integer(c_int) function fibmd_gpu_create(p, ctx) bind(C)
       import
       type(fibmd_params) :: p
       type(c_ptr) :: ctx
     end function fibmd_gpu_create

     subroutine fibmd_gpu_destroy(ctx) bind(C)
       import
       type(c_ptr), value :: ctx
     end subroutine fibmd_gpu_destroy

     integer(c_int) function fibmd_gpu_last_error(ctx, buf, len) bind(C)
       import
       type(c_ptr), value :: ctx
       character(kind=c_char) :: buf(*)
       integer(c_int), value :: len
     end function fibmd_gpu_last_error

     integer(c_int) function fibmd_gpu_upload(ctx, X, V, F, Xi, mass, atype, xsides) bind(C)
       import
       type(c_ptr), value :: ctx
       real(c_double) :: X(*), V(*), Xi(*), mass(*)
       real(c_double), optional :: F(*)
       integer(c_int) :: atype(*), xsides(*)
     end function fibmd_gpu_upload

     integer(c_int) function fibmd_gpu_download(ctx, X, V, F) bind(C)
       import
       type(c_ptr), value :: ctx
       real(c_double), optional :: X(*), V(*), F(*)
     end function fibmd_gpu_download

     integer(c_int) function fibmd_gpu_set_tags(ctx, tags) bind(C)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t) :: tags(*)
     end function fibmd_gpu_set_tags

     integer(c_int) function fibmd_gpu_get_tags(ctx, tags) bind(C)
       import
       type(c_ptr), value :: ctx
       integer(c_int32_t) :: tags(*)
     end function fibmd_gpu_get_tags

     integer(c_int) function fibmd_gpu_set_atom(ctx, i, x, v) bind(C)
       import
       type(c_ptr), value :: ctx
       integer(c_int), value :: i
       real(c_double) :: x(3), v(3)
     end function fibmd_gpu_set_atom

     integer(c_int) function fibmd_gpu_set_impact(ctx, impact) bind(C)
       import
       type(c_ptr), value :: ctx
       integer(c_int), value :: impact
     end function fibmd_gpu_set_impact

     integer(c_int) function fibmd_gpu_ionrun(ctx, tic) bind(C)
       import
       type(c_ptr), value :: ctx
       integer(c_int), value :: tic
     end function fibmd_gpu_ionrun

     integer(c_int) function fibmd_gpu_set_tau(ctx, tau) bind(C)
       import
       type(c_ptr), value :: ctx
       real(c_double), value :: tau
     end function fibmd_gpu_set_tau

     integer(c_int) function fibmd_gpu_nlist(ctx) bind(C)
       import
       type(c_ptr), value :: ctx
     end function fibmd_gpu_nlist

     integer(c_int) function fibmd_gpu_force(ctx, F, u, Utot) bind(C)
       import
       type(c_ptr), value :: ctx
       real(c_double) :: F(*)
       real(c_double), optional :: u(*), Utot
     end function fibmd_gpu_force

     integer(c_int) function fibmd_gpu_steps(ctx, whichctrl, max_steps, lt, time, temp, &
                                              reason) bind(C)
       import
       type(c_ptr), value :: ctx
       integer(c_int), value :: whichctrl
       integer(c_long_long), value :: max_steps
       integer(c_long_long) :: lt
       real(c_double) :: time, temp
       integer(c_int) :: reason
     end function fibmd_gpu_steps

     integer(c_int) function fibmd_gpu_temperature(ctx, T) bind(C)
       import
       type(c_ptr), value :: ctx
       real(c_double) :: T
     end function fibmd_gpu_temperature

     integer(c_int) function fibmd_gpu_timers(ctx, at, nt, ds, f, counts4, reset) bind(C)
       import
       type(c_ptr), value :: ctx
       real(c_double) :: at, nt, ds, f
       integer(c_long_long) :: counts4(4)
       integer(c_int), value :: reset
     end function fibmd_gpu_timers

     integer(c_int) function fibmd_gpu_set_option(ctx, key, value) bind(C)
       import
       type(c_ptr), value :: ctx
       character(kind=c_char) :: key(*)
       real(c_double), value :: value
     end function fibmd_gpu_set_option

     integer(c_int) function fibmd_gpu_get_option(ctx, key, value) bind(C)
       import
       type(c_ptr), value :: ctx
       character(kind=c_char) :: key(*)
       real(c_double) :: value
     end function fibmd_gpu_get_option

     integer(c_int) function fibmd_gpu_regime(ctx, Ts, tic) bind(C)
       import
       type(c_ptr), value :: ctx
       real(c_double) :: Ts
       integer(c_int) :: tic
     end function fibmd_gpu_regime

     integer(c_int) function fibmd_gpu_xyz_frame(ctx, xyz_A, ke_eV) bind(C)
       import
       type(c_ptr), value :: ctx
       real(c_double) :: xyz_A(*), ke_eV(*)
     end function fibmd_gpu_xyz_frame

     integer(c_int) function fibmd_gpu_list_counts(ctx, n_sw_full, n_mol_full, n_triplets) &
          bind(C)
       import
       type(c_ptr), value :: ctx
       integer(c_long_long) :: n_sw_full, n_mol_full, n_triplets
     end function fibmd_gpu_list_counts

     integer(c_int) function fibmd_gpu_get_pairs(ctx, kind, n, ij, cap) bind(C)
       import
       type(c_ptr), value :: ctx
       integer(c_int), value :: kind, cap
       integer(c_int) :: n
       integer(c_int) :: ij(*)
     end function fibmd_gpu_get_pairs

     integer(c_int) function fibmd_gpu_get_triplets(ctx, n, ijk, cap) bind(C)
       import
       type(c_ptr), value :: ctx
       integer(c_long_long) :: n
       integer(c_int) :: ijk(*)
       integer(c_long_long), value :: cap
     end function fibmd_gpu_get_triplets

     integer(c_int) function fibmd_gpu_phase_times(ctx, seconds7, counts7, reset) bind(C)
       import
       type(c_ptr), value :: ctx
       real(c_double) :: seconds7(7)
       integer(c_long_long) :: counts7(7)
       integer(c_int), value :: reset
     end function fibmd_gpu_phase_times

     integer(c_int) function fibmd_gpu_kernel_time(ctx, force_kernel_s, launches, reset) bind(C)
       import
       type(c_ptr), value :: ctx
       real(c_double) :: force_kernel_s
       integer(c_long_long) :: launches
       integer(c_int), value :: reset
     end function fibmd_gpu_kernel_time

     integer(c_int) function fibmd_gpu_pipe_peaks(fp64_tflops, fp32_tflops) bind(C)
       import
       real(c_double) :: fp64_tflops, fp32_tflops
     end function fibmd_gpu_pipe_peaks

     integer(c_int) function fibmd_gpu_work_counters(ctx, counts) bind(C)
       import
       type(c_ptr), value :: ctx
       integer(c_long_long) :: counts(6)
     end function fibmd_gpu_work_counters

     ! virial W(6) = xx yy zz xy xz yz (J) and the per-atom shares w_atom(natm,6)
     integer(c_int) function fibmd_gpu_virial(ctx, w, w_atom) bind(C)
       import
       type(c_ptr), value :: ctx
       real(c_double) :: w(6)
       real(c_double) :: w_atom(*)
     end function fibmd_gpu_virial

     ! successive impacts on the device: ion_atoms 1-based, x/v (nimp,3)
     integer(c_int) function fibmd_gpu_dose(ctx, nimp, ion_atoms, x, v, steps, relax_s, &
          removed_after, ions_removed_after, time_after, steps_after) bind(C)
       import
       type(c_ptr), value :: ctx
       integer(c_int), value :: nimp
       integer(c_int) :: ion_atoms(*)
       real(c_double) :: x(*), v(*)
       integer(c_long_long), value :: steps
       real(c_double), value :: relax_s
       integer(c_int), optional :: removed_after(*), ions_removed_after(*)
       real(c_double), optional :: time_after(*)
       integer(c_long_long), optional :: steps_after(*)
     end function fibmd_gpu_dose

     integer(c_int) function fibmd_gpu_batch_create(p, nrep, reps, ctx) bind(C)
       import
       type(fibmd_params) :: p
       integer(c_int), value :: nrep
       type(fibmd_replica) :: reps(*)
       type(c_ptr) :: ctx
     end function fibmd_gpu_batch_create

     integer(c_int) function fibmd_gpu_batch_layout(ctx, nrep, offsets) bind(C)
       import
       type(c_ptr), value :: ctx
       integer(c_int) :: nrep
       integer(c_int) :: offsets(*)
     end function fibmd_gpu_batch_layout

     integer(c_int) function fibmd_gpu_batch_scalars(ctx, time, dt, removed) bind(C)
       import
       type(c_ptr), value :: ctx
       real(c_double) :: time(*), dt(*)
       integer(c_int) :: removed(*)
     end function fibmd_gpu_batch_scalars

     integer(c_int) function fibmd_gpu_impact_stats(ctx, surface_z, displaced_m, sputtered, &
          displaced, ion_depth) bind(C)
       import
       type(c_ptr), value :: ctx
       real(c_double) :: surface_z(*)
       real(c_double), value :: displaced_m
       integer(c_int) :: sputtered(*), displaced(*)
       real(c_double) :: ion_depth(*)
     end function fibmd_gpu_impact_stats
  end interface

contains

  ! Stops with the library's message when rc is not FIBMD_OK (the reference
  ! prints and goes on for list overflows, src/si.f90:264-272; a host that
  ! wants that passes fatal = .false.).
  subroutine fibmd_check(rc, ctx, what, fatal)
    integer(c_int), intent(in) :: rc
    type(c_ptr), intent(in) :: ctx
    character(len=*), intent(in) :: what
    logical, intent(in), optional :: fatal
    character(kind=c_char) :: buf(512)
    integer(c_int) :: st
    integer :: k
    character(len=512) :: msg
    if (rc == FIBMD_OK) return
    buf = c_null_char
    st = fibmd_gpu_last_error(ctx, buf, 512_c_int)
    msg = ' '
    do k = 1, 511
       if (buf(k) == c_null_char) exit
       msg(k:k) = buf(k)
    end do
    write (*, '(A,A,I0,A,A)') what, ': fibmd status ', rc, ': ', trim(msg)
    if (.not. present(fatal)) then
       stop 1
    else if (fatal) then
       stop 1
    end if
  end subroutine fibmd_check

end module fibmd_gpu_mod
