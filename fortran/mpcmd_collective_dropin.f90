! Drop-in modules for collective_code/main_pattern.f95: evolve_mod,
! distribute_mod, mpc_rotation_mod, reaction_mod, sort_hilbert_mod and
! neighbour_list_mod with the reference's module and subroutine names and
! dummy-argument lists (evolve_mod.f95:6-12, distribute_mod.f95:6-8,
! mpc_rotation_mod.f95:6-7, reaction_mod.f95:8, sort_hilbert_mod.f95:6,
! neighbour_list_mod.f95:6 and :63-64).  The driver compiles unchanged: link
! these modules (and mpcmd_shim.f90, libmpcmd.so) in place of the
! reference's evolve_mod.f95, forces_mod.f95, distribute_mod.f95,
! mpc_rotation_mod.f95, reaction_mod.f95, sort_hilbert_mod.f95 and
! neighbour_list_mod.f95; initial_mod, restart_mod, reactive_grid_mod,
! output_mod, global_mod and mtmod stay the reference's.
!
! Where the state lives.  The first evolve call creates one GPU context from
! its arguments (box, particle and dimer counts, masses, radii, LJ strengths,
! wall and motor-motor terms, catalytic probabilities, skin, MD step, MPC
! interval, sort interval, reactive floor), uploads the driver's arrays
! (after initial or restart) and prepares the lists on the device; from then
! on the device state is the authoritative copy.  The host arrays are
! brought up to date at every collision step, by the routine that owns each
! array in the reference's call sequence (main_pattern.f95:212-224): evolve
! writes the positions, the dimer arrays, TPotential, time_count and
! time_penetrate; mpc_rotation the velocities; reaction_simple the species.
! Between collision steps the host arrays hold the last collision step's
! state; the output cadences of the input decks (Freq1..Freq4) are multiples
! of MPCtstep.  The per-cell tables (tACellN, sBCellN, VXCM, NewCellN, UVX,
! ...), the neighbour lists and the pair forces stay on the device: in the
! reference only these routines read them.
!
! Random numbers.  The contract stream of the library replaces the
! per-thread MT19937 streams (mt, mti are accepted and not used); its key is
! derived from the uploaded initial state, so a run is reproducible from its
! input deck.
!
! Not compiled in this repository: there is no Fortran compiler on the
! development machine or on the GPU hosts.  The plain-C driver
! fortran/mpcmd_driver.c runs the same call sequence through the C ABI and
! is checked against the oracle.
module mpcmd_dropin_state
  use, intrinsic :: iso_c_binding
  use mpcmd_shim
  implicit none
  private
  public :: dropin_ctx, dropin_ready, dropin_start, dropin_download, dropin_obs, dropin_collision
  public :: dropin_precision, current_angle, current_mpct, current_k1

  type(c_ptr), save :: dropin_ctx = c_null_ptr
  logical, save :: dropin_ready = .false.
  ! working precision of the device state (MPCMD_PREC_FP64 for parity runs)
  integer(c_int32_t), save :: dropin_precision = MPCMD_PREC_FP32
  real(c_double), save :: cur_angle = -1.0_c_double, cur_k1 = -1.0_c_double, cur_mpct = -1.0_c_double
  integer, save :: nspheres = 0

  interface
    integer(c_int) function c_download(ctx, x, y, z, vx, vy, vz, flag, dpos, dvel, dforce) &
        bind(C, name="mpcmd_download_state")
      import :: c_int, c_ptr
      type(c_ptr), value :: ctx, x, y, z, vx, vy, vz, flag, dpos, dvel, dforce
    end function
    integer(c_int) function c_set_collision(ctx, angle, mpc_dt, k) bind(C, name="mpcmd_set_collision")
      import :: c_int, c_ptr, c_double
      type(c_ptr), value :: ctx
      real(c_double), value :: angle, mpc_dt
      real(c_double), intent(in) :: k(6)
    end function
    integer(c_int) function c_set_reactive_grid(ctx, table) bind(C, name="mpcmd_set_reactive_grid")
      import :: c_int, c_ptr, c_int32_t
      type(c_ptr), value :: ctx
      integer(c_int32_t), intent(in) :: table(*)
    end function
  end interface

contains

  ! Context from the arguments of the first evolve call, the driver's arrays
  ! uploaded, lists prepared (restart_mod.f95's force evaluation when the run
  ! starts from a restart, cstep > 1).
  subroutine dropin_start(cstep, NT, MDt, MPCtstep, numdims, Ma, Mb, Ms, Mc, Mn, Dcn, Box, Rc, Rn, EaC, EbC, &
                          EsC, EaN, EbN, EsN, Rw, Ew, Rm_delta, Em, RPab, RPba, flag, xsol, ysol, zsol, &
                          vxsol, vysol, vzsol, xdim, ydim, zdim, vxdim, vydim, vzdim, fxdim, fydim, fzdim, &
                          skinrad, max_nb, sort_step, react_box, react_dir)
    integer(4), intent(in) :: cstep, NT, MPCtstep, numdims, sort_step, react_dir, max_nb
    real(8), intent(in) :: MDt, Ma, Mb, Ms, Mc, Mn, Dcn, Box(:), Rc, Rn, EaC, EbC, EsC, EaN, EbN, EsN
    real(8), intent(in) :: Rw, Ew, Rm_delta, Em, RPab, RPba, skinrad
    integer(4), intent(in) :: flag(:), react_box(:)
    real(8), intent(in) :: xsol(:), ysol(:), zsol(:), vxsol(:), vysol(:), vzsol(:)
    real(8), intent(in) :: xdim(:,:), ydim(:,:), zdim(:,:), vxdim(:,:), vydim(:,:), vzdim(:,:)
    real(8), intent(in) :: fxdim(:,:), fydim(:,:), fzdim(:,:)
    type(mpcmd_config) :: cfg
    real(c_double), allocatable :: dpos(:,:), dvel(:,:), dfrc(:,:)
    integer(c_int32_t), allocatable :: iflag(:), table(:)
    integer :: k, i
    integer(c_int64_t) :: key
    cfg%lx = int(Box(1), c_int32_t); cfg%ly = int(Box(2), c_int32_t); cfg%lz = int(Box(3), c_int32_t)
    cfg%geometry = MPCMD_GEOM_WALLS
    cfg%n_dimers = numdims
    cfg%kinetics = MPCMD_KIN_SIMPLE
    cfg%exclusion = MPCMD_EXCL_PARTICLE
    cfg%catalysis = MPCMD_CAT_DETERMINISTIC
    cfg%rotation_sense = 1
    cfg%mpc_every = MPCtstep
    cfg%sort_every = sort_step
    cfg%react_box_type = 1          ! replaced by the driver's react_box table below
    cfg%react_dir = react_dir
    cfg%cell_capacity = 100         ! MaxA (global_mod.f95:114-116)
    cfg%max_neighbour = max_nb
    cfg%rattle_max_iter = 100000
    cfg%init_plane = 0
    cfg%pad0 = 0
    cfg%n_solvent = NT
    ! contract-stream key from the initial state's bits
    key = transfer(xsol(1), key)
    key = ieor(key, ishft(transfer(vxsol(1), key), 1))
    cfg%seed = key
    cfg%init_count = [int(NT, c_int64_t), 0_c_int64_t, 0_c_int64_t, 0_c_int64_t]
    cfg%mass = [Ma, Mb, Ms, 1.0_c_double]
    cfg%eps_c = [EaC, EbC, EsC, 0.0_c_double]
    cfg%eps_n = [EaN, EbN, EsN, 0.0_c_double]
    cfg%rc = Rc; cfg%rn = Rn; cfg%dcn = Dcn; cfg%mc = Mc; cfg%mn = Mn
    cfg%rw = Rw; cfg%ew = Ew; cfg%rm_delta = Rm_delta; cfg%em = Em
    cfg%rp_ab = RPab; cfg%rp_ba = RPba
    cfg%kT = 1.0_c_double           ! initial velocities are the driver's (initial_mod / restart_mod)
    cfg%skin = skinrad
    cfg%rot_angle = 2.0_c_double * acos(-1.0_c_double) / 3.0_c_double   ! set by mpc_rotation before the first collision
    cfg%md_dt = MDt
    cfg%mpc_dt = MDt * MPCtstep
    cfg%k = 0.0_c_double            ! set by reaction_simple before the first reaction
    cfg%precision = dropin_precision
    cfg%shell_capacity = 0
    cfg%variant = MPCMD_VARIANT_MOTOR
    cfg%layout = MPCMD_LAYOUT_RANDOM
    cfg%layout_rows = 0; cfg%layout_cols = 0
    cfg%owner_tags = 0; cfg%reserved = 0
    cfg%tether_k = 0.0_c_double; cfg%tether_z = 0.0_c_double; cfg%layout_sep = 0.0_c_double
    call mpcmd_check(mpcmd_create(cfg, dropin_ctx), 'create')
    cur_angle = cfg%rot_angle; cur_mpct = cfg%mpc_dt; cur_k1 = 0.0_c_double
    allocate(table(size(react_box)))
    table = int(react_box, c_int32_t)
    call mpcmd_check(c_set_reactive_grid(dropin_ctx, table), 'set_reactive_grid')
    nspheres = 2 * numdims
    allocate(dpos(3, nspheres), dvel(3, nspheres), dfrc(3, nspheres), iflag(NT))
    do k = 1, numdims
      do i = 1, 2
        dpos(:, 2 * (k - 1) + i) = [xdim(k, i), ydim(k, i), zdim(k, i)]
        dvel(:, 2 * (k - 1) + i) = [vxdim(k, i), vydim(k, i), vzdim(k, i)]
        dfrc(:, 2 * (k - 1) + i) = [fxdim(k, i), fydim(k, i), fzdim(k, i)]
      end do
    end do
    iflag = int(flag, c_int32_t)
    call mpcmd_check(mpcmd_upload_state(dropin_ctx, xsol, ysol, zsol, vxsol, vysol, vzsol, iflag, dpos, dvel, dfrc), &
                     'upload_state')
    ! the step before this one is the state's step
    call mpcmd_check(mpcmd_set_step(dropin_ctx, int(cstep - 1, c_int64_t), 0_c_int32_t), 'set_step')
    if (cstep - 1 == 0) then
      call mpcmd_check(mpcmd_prepare(dropin_ctx), 'prepare')
    else
      call mpcmd_check(mpcmd_prepare_restart(dropin_ctx), 'prepare_restart')
    end if
    dropin_ready = .true.
  end subroutine dropin_start

  ! Collision angle and the reaction's interval and rate as the driver passes them.
  subroutine dropin_collision(angle, mpct, k1)
    real(8), intent(in) :: angle, mpct, k1
    real(c_double) :: k(6)
    if (angle == cur_angle .and. mpct == cur_mpct .and. k1 == cur_k1) return
    k = 0.0_c_double
    k(1) = k1
    call mpcmd_check(c_set_collision(dropin_ctx, angle, mpct, k), 'set_collision')
    cur_angle = angle; cur_mpct = mpct; cur_k1 = k1
  end subroutine dropin_collision

  ! Selected host arrays from the device (c_null_ptr: not wanted).
  subroutine dropin_download(x, y, z, vx, vy, vz, flag, dpos, dvel, dforce)
    type(c_ptr), intent(in) :: x, y, z, vx, vy, vz, flag, dpos, dvel, dforce
    call mpcmd_check(c_download(dropin_ctx, x, y, z, vx, vy, vz, flag, dpos, dvel, dforce), 'download_state')
  end subroutine dropin_download

  real(8) function current_angle()
    current_angle = cur_angle
  end function current_angle

  real(8) function current_mpct()
    current_mpct = cur_mpct
  end function current_mpct

  real(8) function current_k1()
    current_k1 = cur_k1
  end function current_k1

  subroutine dropin_obs(obs)
    type(mpcmd_obs), intent(out) :: obs
    call mpcmd_check(mpcmd_observables(dropin_ctx, obs), 'observables')
  end subroutine dropin_obs

end module mpcmd_dropin_state


module evolve_mod
  use, intrinsic :: iso_c_binding
  use mpcmd_shim
  use mpcmd_dropin_state
  implicit none
contains

! evolve_mod.f95:6-732: one MD step of every particle and dimer on the device.
subroutine evolve(cstep,time,NT,MDt,MPCtstep,numdims,Ma,Mb,Ms,Mc,Mn,Dcn,Box,cutoff,Rc,Rn,EaC,EbC,EsC,EaN,EbN,EsN,&
                  Rw,Ew,Rm_delta,Em,RPab,RPba,sphere,flag,xsol,Ysol,Zsol,VXsol,VYsol,VZsol,Xdim,&
                  Ydim,Zdim,VXdim,VYdim,VZdim,FXdim,FYdim,FZdim,motorCM,TPotential,Potential,FpairX,&
                  FpairY,FpairZ,skinrad,max_solvent_dist,neighbour_num,neighbour,time_count,&
                  time_penetrate,outside_particle_num,outside_particle,inside_particle_num,inside_particle,&
                  vol,sort_step,react_box,react_dir)
implicit none
integer, parameter :: sp = selected_real_kind(6,37)
integer, parameter :: dp = selected_real_kind(15,307)
integer(kind=sp) :: cstep
integer(kind=dp) :: time
integer(kind=sp) , intent(in) :: NT
real(kind=dp) , intent(in) :: MDt
integer(kind=sp) :: MPCtstep
integer , intent(in) :: numdims
real(kind=dp) , intent(in) :: Ma, Mb, Ms, Mc, Mn, Dcn
real(kind=dp) , dimension(:), intent(in) :: Box
real(kind=dp) , intent(in) :: cutoff, Rc, Rn, EaC, EbC, EsC, EaN, EbN, EsN, Rw, Ew, Rm_delta, Em, RPab, RPba
integer , dimension(:) , intent(in) :: sphere
integer(kind=sp) , dimension(:), intent(inout), target, contiguous :: flag
real(kind=dp) , dimension(:) , intent(inout), target, contiguous :: Xsol, Ysol, Zsol
real(kind=dp) , dimension(:,:) , intent(inout) :: Xdim, Ydim, Zdim
real(kind=dp) , dimension(:) , intent(inout), target, contiguous :: VXsol, VYsol, VZsol
real(kind=dp) , dimension(:,:) , intent(inout) :: VXdim, VYdim, VZdim, FXdim, FYdim, FZdim
real(kind=dp) , dimension(:,:) , intent(in) :: motorCM
real(kind=dp) , intent(out) :: TPotential
real(kind=dp) , dimension(:,:,:) , intent(inout) :: Potential, FpairX, FpairY, FpairZ
integer(kind=dp) , dimension(:,:) , intent(inout) :: neighbour_num
integer(kind=dp) , dimension(:,:,:) , intent(inout) :: neighbour
real(kind=dp) , intent(in) :: skinrad
real(kind=dp) , dimension(:) , intent(inout) :: max_solvent_dist
integer , intent(inout) :: time_count
integer , intent(inout) :: time_penetrate
integer(kind=dp) , intent(inout) :: outside_particle_num
integer(kind=dp) , dimension(:) , intent(inout) :: outside_particle
integer(kind=dp) :: vol
integer :: sort_step
integer(kind=dp) , intent(inout) :: inside_particle_num
integer(kind=dp) , dimension(:) , intent(inout) :: inside_particle
integer , dimension(:) , intent(in) :: react_box
integer , intent(in) :: react_dir
real(c_double), dimension(:,:), allocatable, target :: dpos, dvel, dfrc
type(mpcmd_obs) :: obs
integer :: k, i

if (.not. dropin_ready) then
  call dropin_start(cstep, NT, MDt, MPCtstep, numdims, Ma, Mb, Ms, Mc, Mn, Dcn, Box, Rc, Rn, EaC, EbC, EsC, &
                    EaN, EbN, EsN, Rw, Ew, Rm_delta, Em, RPab, RPba, flag, Xsol, Ysol, Zsol, VXsol, VYsol, VZsol, &
                    Xdim, Ydim, Zdim, VXdim, VYdim, VZdim, FXdim, FYdim, FZdim, skinrad, size(neighbour, 3), &
                    sort_step, react_box, react_dir)
end if
call mpcmd_check(mpcmd_evolve(dropin_ctx), 'evolve')
TPotential = 0.0_dp
if (mod(cstep, MPCtstep) == 0) then
  ! every particle is at this step: positions, dimers and the step counters to the host
  allocate(dpos(3, 2 * numdims), dvel(3, 2 * numdims), dfrc(3, 2 * numdims))
  call dropin_download(c_loc(Xsol), c_loc(Ysol), c_loc(Zsol), c_null_ptr, c_null_ptr, c_null_ptr, &
                       c_null_ptr, c_loc(dpos), c_loc(dvel), c_loc(dfrc))
  do k = 1, numdims
    do i = 1, 2
      Xdim(k, i) = dpos(1, 2 * (k - 1) + i); Ydim(k, i) = dpos(2, 2 * (k - 1) + i); Zdim(k, i) = dpos(3, 2 * (k - 1) + i)
      VXdim(k, i) = dvel(1, 2 * (k - 1) + i); VYdim(k, i) = dvel(2, 2 * (k - 1) + i); VZdim(k, i) = dvel(3, 2 * (k - 1) + i)
      FXdim(k, i) = dfrc(1, 2 * (k - 1) + i); FYdim(k, i) = dfrc(2, 2 * (k - 1) + i); FZdim(k, i) = dfrc(3, 2 * (k - 1) + i)
    end do
  end do
  call dropin_obs(obs)
  TPotential = obs%potential
  time_count = obs%time_count
  time_penetrate = obs%time_penetrate
end if
end subroutine evolve

end module evolve_mod


module distribute_mod
  use, intrinsic :: iso_c_binding
  use mpcmd_shim
  use mpcmd_dropin_state
  implicit none
contains

! distribute_mod.f95:6-205: the per-species cell lists of the bulk solvent,
! kept on the device for reaction_simple.
subroutine distribute(NT,numdims,cutoff,Rc,Rn,flag,Xsol,Ysol,Zsol,Xdim,Ydim,Zdim,Box,tACellN,tBCellN,tSCellN, &
                      sACellN,sBCellN,sSCellN,cutoffC2,cutoffN2,cstep,outside_particle_num,outside_particle,&
                      inside_particle_num,inside_particle)
implicit none
integer, parameter :: sp = selected_real_kind(6,37)
integer, parameter :: dp = selected_real_kind(15,307)
integer(kind=sp) , intent(in) :: NT
integer , intent(in) :: numdims
integer(kind=sp) , dimension(:), intent(in) :: flag
real(kind=dp) , dimension(:) , intent(in) :: Xsol, Ysol, Zsol
real(kind=dp) , dimension(:,:) , intent(in) :: Xdim, Ydim, Zdim
real(kind=dp) , dimension(:) , intent(in) :: Box
integer(kind=dp) , dimension(:), intent(out) :: tACellN, tBCellN, tSCellN
integer(kind=dp) , dimension(:,:), intent(out) :: sACellN, sBCellN, sSCellN
real(kind=dp) , intent(in) :: cutoff, Rc, Rn, cutoffC2, cutoffN2
integer(kind=sp) :: cstep
integer(kind=dp) , intent(inout) :: outside_particle_num
integer(kind=dp) , dimension(:) , intent(inout) :: outside_particle
integer(kind=dp) , intent(inout) :: inside_particle_num
integer(kind=dp) , dimension(:) , intent(inout) :: inside_particle
call mpcmd_check(mpcmd_distribute(dropin_ctx), 'distribute')
end subroutine distribute

end module distribute_mod


module mpc_rotation_mod
  use, intrinsic :: iso_c_binding
  use mpcmd_shim
  use mpcmd_dropin_state
  implicit none
contains

! mpc_rotation_mod.f95:6-239: the SRD collision of every particle; the
! rotated velocities to the host.
subroutine mpc_rotation(NT,rotang,numcell,a0,Box,Xsol,Ysol,Zsol,VXsol,VYsol,VZsol,VXCM,VYCM,VZCM, &
                        tCellShift,NewCellN,UVX,UVY,UVZ,mt,mti)
implicit none
integer, parameter :: sp = selected_real_kind(6,37)
integer, parameter :: dp = selected_real_kind(15,307)
integer(kind=sp) , intent(in) :: NT
real(kind=dp) , intent(in) :: rotang
integer(kind=dp) , intent(in) :: numcell
real(kind=dp) , intent(in) :: a0
real(kind=dp) , dimension(:) , intent(in) :: Box
real(kind=dp) , dimension(:) , intent(in) :: Xsol, Ysol, Zsol
real(kind=dp) , dimension(:) , intent(inout), target, contiguous :: VXsol, VYsol, VZsol
real(kind=dp) , dimension(:) , intent(inout) :: VXCM, VYCM, VZCM, tCellShift
integer(kind=dp) , dimension(:) , intent(inout) :: NewCellN
real(kind=dp) , dimension(:) , intent(inout) :: UVX, UVY, UVZ
integer , dimension(:,:) , intent(inout) :: mt
integer , dimension(:) , intent(inout) :: mti
call dropin_collision(rotang, current_mpct(), current_k1())
call mpcmd_check(mpcmd_mpc_rotation(dropin_ctx), 'mpc_rotation')
call dropin_download(c_null_ptr, c_null_ptr, c_null_ptr, c_loc(VXsol), c_loc(VYsol), c_loc(VZsol), &
                     c_null_ptr, c_null_ptr, c_null_ptr, c_null_ptr)
end subroutine mpc_rotation

end module mpc_rotation_mod


module reaction_mod
  use, intrinsic :: iso_c_binding
  use mpcmd_shim
  use mpcmd_dropin_state
  implicit none
contains

! reaction_mod.f95:8-66: the bulk B -> A reaction of every cell; the species
! to the host.
subroutine reaction_simple(MPCt,numcell,k1,flag,tBCellN,sBCellN,mt,mti)
implicit none
integer, parameter :: sp = selected_real_kind(6,37)
integer, parameter :: dp = selected_real_kind(15,307)
integer(kind=dp) , intent(in) :: numcell
real(kind=dp) , intent(in) :: MPCt
real(kind=dp) , intent(in) :: k1
integer(kind=sp) , dimension(:), intent(inout), target, contiguous :: flag
integer(kind=dp) , dimension(:), intent(in) :: tBCellN
integer(kind=dp) , dimension(:,:), intent(in) :: sBCellN
integer , dimension(:,:) , intent(inout) :: mt
integer , dimension(:) , intent(inout) :: mti
call dropin_collision(current_angle(), MPCt, k1)
call mpcmd_check(mpcmd_reaction(dropin_ctx), 'reaction')
call dropin_download(c_null_ptr, c_null_ptr, c_null_ptr, c_null_ptr, c_null_ptr, c_null_ptr, &
                     c_loc(flag), c_null_ptr, c_null_ptr, c_null_ptr)
end subroutine reaction_simple

end module reaction_mod


module sort_hilbert_mod
  use, intrinsic :: iso_c_binding
  use mpcmd_shim
  use mpcmd_dropin_state
  implicit none
contains

! sort_hilbert_mod.f95:6-98.  The driver calls it at initialisation only
! (evolve sorts inside the rebuild on sort steps); before the device state
! exists there is nothing to sort on the device, which sorts at its first
! prepare (the same stable cell order); afterwards the device sorts.
subroutine sort_hilbert(vol,NT,box,xsol,ysol,zsol,flag,vxsol,vysol,vzsol)
implicit none
integer, parameter :: sp = selected_real_kind(6,37)
integer, parameter :: dp = selected_real_kind(15,307)
integer(kind=dp) , intent(in) :: vol
integer(kind=sp) , intent(in) :: NT
real(kind=dp) , dimension(:) , intent(in) :: box
real(kind=dp) , dimension(:) , intent(inout) :: xsol, ysol, zsol
integer , dimension(:) , intent(inout) :: flag
real(kind=dp) , dimension(:) , intent(inout) :: vxsol, vysol, vzsol
if (dropin_ready) call mpcmd_check(mpcmd_sort(dropin_ctx), 'sort')
end subroutine sort_hilbert

end module sort_hilbert_mod


module neighbour_list_mod
  use, intrinsic :: iso_c_binding
  use mpcmd_shim
  use mpcmd_dropin_state
  implicit none
contains

! neighbour_list_mod.f95:6-59 and :63-184.  The lists live on the device,
! built by the first evolve (prepare) and by every rebuild; the driver's
! calls at initialisation find no device state yet and return.
subroutine neighbour_list(NT,Box,cutoff,skinrad,Xsol,Ysol,Zsol,Xdim,Ydim,Zdim,neighbour_num,neighbour)
implicit none
integer, parameter :: sp = selected_real_kind(6,37)
integer, parameter :: dp = selected_real_kind(15,307)
integer(kind=sp) , intent(in) :: NT
real(kind=dp) , dimension(:) , intent(in) :: Box
real(kind=dp) , intent(in) :: cutoff, skinrad
real(kind=dp) , dimension(:) , intent(in) :: Xsol, Ysol, Zsol
real(kind=dp) , intent(in) :: Xdim, Ydim, Zdim
integer(kind=dp) , intent(out) :: neighbour_num
integer(kind=dp) , dimension(:) , intent(out) :: neighbour
neighbour_num = 0
if (dropin_ready) call mpcmd_check(mpcmd_rebuild_lists(dropin_ctx), 'rebuild_lists')
end subroutine neighbour_list

subroutine inout_particle_list(NT,box,cutoffC,cutoffN,skinrad,xsol,ysol,zsol,xdim,ydim,zdim,&
outside_particle_num,outside_particle,inside_particle_num,inside_particle,numdims)
implicit none
integer, parameter :: sp = selected_real_kind(6,37)
integer, parameter :: dp = selected_real_kind(15,307)
integer(kind=sp) , intent(in) :: NT
real(kind=dp) , dimension(:) , intent(in) :: box
real(kind=dp) , intent(in) :: cutoffC, cutoffN, skinrad
real(kind=dp) , dimension(:) , intent(in) :: xsol, ysol, zsol
real(kind=dp) , dimension(:,:) , intent(in) :: xdim, ydim, zdim
integer(kind=dp) , intent(inout) :: outside_particle_num
integer(kind=dp) , dimension(:) , intent(inout) :: outside_particle
integer(kind=dp) , intent(inout) :: inside_particle_num
integer(kind=dp) , dimension(:) , intent(inout) :: inside_particle
integer , intent(in) :: numdims
end subroutine inout_particle_list

end module neighbour_list_mod
