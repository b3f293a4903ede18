! Fortran binding of the mpcmd C ABI (include/mpcmd.h) with iso_c_binding.
!
! A Fortran driver of the reference (collective_code/main_pattern.f95,
! selkov_code/Main_SelkovDimer.f90) uses this module to run its time step on
! one GPU: it fills an mpcmd_config from the values it reads from its input
! deck, creates a context, uploads its module arrays once, calls mpcmd_step
! (or mpcmd_run) in the main loop and downloads the arrays only when it writes
! output or a restart file.  Every function returns an mpcmd_status; the
! helper mpcmd_check stops the program with the library's error text on a
! nonzero status, which is what the reference's module subroutines would do
! if they reported errors at all.
!
! Not compiled in this repository's tests: neither the development container
! nor the GPU box has a Fortran compiler.  The type and interfaces follow the
! C declarations field by field (int32_t -> integer(c_int32_t), int64_t ->
! integer(c_int64_t), uint64_t -> integer(c_int64_t), double -> real(c_double)).
module mpcmd_shim
  use, intrinsic :: iso_c_binding
  implicit none
  private

  integer(c_int), parameter, public :: MPCMD_OK = 0
  integer(c_int32_t), parameter, public :: MPCMD_GEOM_WALLS = 0, MPCMD_GEOM_PERIODIC = 1
  integer(c_int32_t), parameter, public :: MPCMD_KIN_NONE = 0, MPCMD_KIN_SIMPLE = 1, MPCMD_KIN_SELKOV = 2
  integer(c_int32_t), parameter, public :: MPCMD_EXCL_PARTICLE = 0, MPCMD_EXCL_CELLS = 1
  integer(c_int32_t), parameter, public :: MPCMD_CAT_DETERMINISTIC = 0, MPCMD_CAT_PROBABILISTIC = 1
  integer(c_int32_t), parameter, public :: MPCMD_PREC_FP32 = 32, MPCMD_PREC_FP64 = 64
  integer(c_int32_t), parameter, public :: MPCMD_VARIANT_MOTOR = 0, MPCMD_VARIANT_ROTOR = 1
  integer(c_int32_t), parameter, public :: MPCMD_LAYOUT_RANDOM = 0, MPCMD_LAYOUT_GRID = 1, MPCMD_LAYOUT_LINE = 2

  ! struct mpcmd_config
  type, bind(C), public :: mpcmd_config
    integer(c_int32_t) :: lx, ly, lz
    integer(c_int32_t) :: geometry
    integer(c_int32_t) :: n_dimers
    integer(c_int32_t) :: kinetics
    integer(c_int32_t) :: exclusion
    integer(c_int32_t) :: catalysis
    integer(c_int32_t) :: rotation_sense
    integer(c_int32_t) :: mpc_every
    integer(c_int32_t) :: sort_every
    integer(c_int32_t) :: react_box_type
    integer(c_int32_t) :: react_dir
    integer(c_int32_t) :: cell_capacity
    integer(c_int32_t) :: max_neighbour
    integer(c_int32_t) :: rattle_max_iter
    integer(c_int32_t) :: init_plane
    integer(c_int32_t) :: pad0
    integer(c_int64_t) :: n_solvent
    integer(c_int64_t) :: seed
    integer(c_int64_t) :: init_count(4)
    real(c_double) :: mass(4)
    real(c_double) :: eps_c(4)
    real(c_double) :: eps_n(4)
    real(c_double) :: rc, rn, dcn
    real(c_double) :: mc, mn
    real(c_double) :: rw, ew
    real(c_double) :: rm_delta, em
    real(c_double) :: rp_ab, rp_ba
    real(c_double) :: kT, skin, rot_angle, md_dt, mpc_dt
    real(c_double) :: k(6)
    integer(c_int32_t) :: precision
    integer(c_int32_t) :: shell_capacity
    integer(c_int32_t) :: variant
    integer(c_int32_t) :: layout
    integer(c_int32_t) :: layout_rows, layout_cols
    integer(c_int32_t) :: owner_tags
    integer(c_int32_t) :: reserved
    real(c_double) :: tether_k, tether_z
    real(c_double) :: layout_sep
  end type mpcmd_config

  ! struct mpcmd_conc_params
  type, bind(C), public :: mpcmd_conc_params
    real(c_double) :: x_slab, y_slab, z_slab
    real(c_double) :: half_width
    real(c_double) :: x_width, y_width, z_width
  end type mpcmd_conc_params

  ! struct mpcmd_obs
  type, bind(C), public :: mpcmd_obs
    real(c_double) :: momentum(3)
    real(c_double) :: solvent_momentum(3)
    real(c_double) :: kinetic_solvent, kinetic_dimer, potential
    integer(c_int64_t) :: species_count(4)
    integer(c_int64_t) :: n_inside, n_pairs
    integer(c_int32_t) :: time_count, time_penetrate
    integer(c_int64_t) :: cstep
  end type mpcmd_obs

  public :: mpcmd_create, mpcmd_destroy, mpcmd_error_string, mpcmd_upload_state, mpcmd_download_state
  public :: mpcmd_set_step, mpcmd_initial, mpcmd_prepare, mpcmd_prepare_restart, mpcmd_step, mpcmd_evolve, mpcmd_run
  public :: mpcmd_sort, mpcmd_rebuild_lists, mpcmd_distribute, mpcmd_mpc_rotation, mpcmd_reaction
  public :: mpcmd_observables, mpcmd_checkpoint, mpcmd_restore, mpcmd_set_cell_order
  public :: mpcmd_concentration, mpcmd_dimer_axes, mpcmd_set_anchors, mpcmd_get_anchors
  public :: mpcmd_set_owner_tags, mpcmd_get_owner_tags
  public :: mpcmd_check

  interface
    ! int mpcmd_create(const mpcmd_config*, mpcmd_ctx**)
    integer(c_int) function mpcmd_create(cfg, ctx) bind(C, name="mpcmd_create")
      import :: c_int, c_ptr, mpcmd_config
      type(mpcmd_config), intent(in) :: cfg
      type(c_ptr), intent(out) :: ctx
    end function
    integer(c_int) function mpcmd_destroy(ctx) bind(C, name="mpcmd_destroy")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    type(c_ptr) function mpcmd_error_string(status) bind(C, name="mpcmd_error_string")
      import :: c_int, c_ptr
      integer(c_int), value :: status
    end function
    ! Host arrays in the reference layout: Xsol..VZsol(NT), flag(NT) as
    ! integer(4), dimer arrays as dpos(3, 2*numdims) (x, y, z of sphere s =
    ! 2k + i contiguous), i.e. the transpose of Xdim(k, i) .. Zdim(k, i).
    integer(c_int) function mpcmd_upload_state(ctx, x, y, z, vx, vy, vz, flag, dpos, dvel, dforce) &
        bind(C, name="mpcmd_upload_state")
      import :: c_int, c_ptr, c_double, c_int32_t
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: x(*), y(*), z(*), vx(*), vy(*), vz(*)
      integer(c_int32_t), intent(in) :: flag(*)
      real(c_double), intent(in) :: dpos(*), dvel(*), dforce(*)
    end function
    integer(c_int) function mpcmd_download_state(ctx, x, y, z, vx, vy, vz, flag, dpos, dvel, dforce) &
        bind(C, name="mpcmd_download_state")
      import :: c_int, c_ptr, c_double, c_int32_t
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: x(*), y(*), z(*), vx(*), vy(*), vz(*)
      integer(c_int32_t), intent(out) :: flag(*)
      real(c_double), intent(out) :: dpos(*), dvel(*), dforce(*)
    end function
    ! motorCM of rotational_code/2d_array (main_rotation.f95:89), [3, numdims]
    integer(c_int) function mpcmd_set_anchors(ctx, anchors) bind(C, name="mpcmd_set_anchors")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(in) :: anchors(*)
    end function
    integer(c_int) function mpcmd_get_anchors(ctx, anchors) bind(C, name="mpcmd_get_anchors")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), intent(out) :: anchors(*)
    end function
    ! type_B of rotational_code/linear_periodic_no_ci (global_mod.f95:72), [NT]
    integer(c_int) function mpcmd_set_owner_tags(ctx, type_b) bind(C, name="mpcmd_set_owner_tags")
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), intent(in) :: type_b(*)
    end function
    integer(c_int) function mpcmd_get_owner_tags(ctx, type_b) bind(C, name="mpcmd_get_owner_tags")
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), intent(out) :: type_b(*)
    end function
    integer(c_int) function mpcmd_set_cell_order(ctx, order, n) bind(C, name="mpcmd_set_cell_order")
      import :: c_int, c_ptr, c_int32_t, c_int64_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), intent(in) :: order(*)
      integer(c_int64_t), value :: n
    end function
    integer(c_int) function mpcmd_set_step(ctx, cstep, time_count) bind(C, name="mpcmd_set_step")
      import :: c_int, c_ptr, c_int64_t, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int64_t), value :: cstep
      integer(c_int32_t), value :: time_count
    end function
    integer(c_int) function mpcmd_initial(ctx) bind(C, name="mpcmd_initial")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mpcmd_prepare(ctx) bind(C, name="mpcmd_prepare")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mpcmd_prepare_restart(ctx) bind(C, name="mpcmd_prepare_restart")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mpcmd_step(ctx) bind(C, name="mpcmd_step")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mpcmd_evolve(ctx) bind(C, name="mpcmd_evolve")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mpcmd_run(ctx, nsteps) bind(C, name="mpcmd_run")
      import :: c_int, c_ptr, c_int64_t
      type(c_ptr), value :: ctx
      integer(c_int64_t), value :: nsteps
    end function
    integer(c_int) function mpcmd_sort(ctx) bind(C, name="mpcmd_sort")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mpcmd_rebuild_lists(ctx) bind(C, name="mpcmd_rebuild_lists")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mpcmd_distribute(ctx) bind(C, name="mpcmd_distribute")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mpcmd_mpc_rotation(ctx) bind(C, name="mpcmd_mpc_rotation")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mpcmd_reaction(ctx) bind(C, name="mpcmd_reaction")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx
    end function
    integer(c_int) function mpcmd_observables(ctx, obs) bind(C, name="mpcmd_observables")
      import :: c_int, c_ptr, mpcmd_obs
      type(c_ptr), value :: ctx
      type(mpcmd_obs), intent(out) :: obs
    end function
    ! output_mod.f95:482-575: totals(4) = TotA, TotB, ConcA, ConcB; the 1D and 2D
    ! fields in the reference's own array order (concA1d(nx), concA2d_xy(nx,ny) ...)
    integer(c_int) function mpcmd_concentration(ctx, p, totals, c1d_a, c1d_b, xy_a, xy_b, xz_a, xz_b, &
        yz_a, yz_b) bind(C, name="mpcmd_concentration")
      import :: c_int, c_ptr, c_double, mpcmd_conc_params
      type(c_ptr), value :: ctx
      type(mpcmd_conc_params), intent(in) :: p
      real(c_double), intent(out) :: totals(*), c1d_a(*), c1d_b(*), xy_a(*), xy_b(*)
      real(c_double), intent(out) :: xz_a(*), xz_b(*), yz_a(*), yz_b(*)
    end function
    ! nucvec(3, numdims): output_mod.f95:826-846 with normalize = 0
    integer(c_int) function mpcmd_dimer_axes(ctx, normalize, nucvec, vdot) bind(C, name="mpcmd_dimer_axes")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      integer(c_int), value :: normalize
      real(c_double), intent(out) :: nucvec(*), vdot(*)
    end function
    integer(c_int) function mpcmd_checkpoint(ctx, path) bind(C, name="mpcmd_checkpoint")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: ctx
      character(kind=c_char), intent(in) :: path(*)
    end function
    integer(c_int) function mpcmd_restore(ctx, path) bind(C, name="mpcmd_restore")
      import :: c_int, c_ptr, c_char
      type(c_ptr), value :: ctx
      character(kind=c_char), intent(in) :: path(*)
    end function
  end interface

contains

  ! Stop with the library's error text when a call did not return MPCMD_OK.
  subroutine mpcmd_check(status, what)
    integer(c_int), intent(in) :: status
    character(len=*), intent(in) :: what
    character(kind=c_char), pointer :: msg(:)
    integer :: n
    if (status == MPCMD_OK) return
    call c_f_pointer(mpcmd_error_string(status), msg, [256])
    n = 0
    do while (n < 256)
      if (msg(n + 1) == c_null_char) exit
      n = n + 1
    end do
    write(*, '(a, a, a, i0, a, 256a)') 'mpcmd: ', what, ' failed (', status, '): ', msg(1:n)
    error stop 1
  end subroutine mpcmd_check

end module mpcmd_shim
