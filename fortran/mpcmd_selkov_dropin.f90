! Drop-in subroutines for selkov_code/Main_SelkovDimer.f90: Motion_SelkovDimer,
! ForcesMD_SelkovDimer, Distribute_SelkovDimer, Affected_Cell,
! RMPC_SelkovDimer and Sort, argument-less like the reference
! (Main_SelkovDimer.f90:125-137), on the arrays of the reference's
! Global_SelkovDimer module.  The driver compiles unchanged: link this file
! (and mpcmd_shim.f90, libmpcmd.so) in place of Motion_SelkovDimer.f90,
! ForcesMD_SelkovDimer.f90, Distribute_SelkovDimer.f90, Affected_Cell.f90,
! RMPC_SelkovDimer.f90 and Sort.f90; Global_SelkovDimer, Initial_SelkovDimer,
! Restart, the outputs and mt95 stay the reference's.
!
! The first Motion_SelkovDimer call creates one GPU context from the module
! variables (Box, NT, the masses, radii, bond, LJ strengths F/G/I with C and N,
! RPfg, RPgf, the six Selkov rates k1..k6, T, MDt, MPCt, rotang), uploads the
! solvent and dimer arrays (species codes F 0, G 1, I 3) and prepares the
! lists.  Motion_SelkovDimer then runs one whole MD step (positions, forces,
! velocities and RATTLE of the solvent and the dimer, with the probabilistic
! catalysis of ForcesMD_SelkovDimer.f90:143-198); ForcesMD_SelkovDimer has
! nothing left to do.  On collision steps Distribute_SelkovDimer bins the
! solvent and marks the affected cells (Affected_Cell.f90:7-101, so
! Affected_Cell has nothing left to do), RMPC_SelkovDimer performs the
! collision and the six-channel reaction and then copies the solvent and
! dimer arrays back to the module, where Output_SelkovDimer and Restart read
! them.  Sort is the engine's sort on sort steps (the context sorts every
! 10,000 steps as the driver does, Main_SelkovDimer.f90:128); its hole
! compaction (Sort.f90:166-183) has nothing to do because the engine keeps
! no holes.
!
! Not compiled in this repository: no Fortran compiler on either machine.
module mpcmd_selkov_state
  use, intrinsic :: iso_c_binding
  use mpcmd_shim
  implicit none
  type(c_ptr), save :: sk_ctx = c_null_ptr
  logical, save :: sk_ready = .false.
  integer(c_int32_t), save :: sk_precision = MPCMD_PREC_FP32
end module mpcmd_selkov_state

SUBROUTINE Motion_SelkovDimer
USE Global_SelkovDimer
USE mpcmd_selkov_state
IMPLICIT NONE
type(mpcmd_config) :: cfg
real(c_double), allocatable :: dpos(:,:), dvel(:,:), dfrc(:,:)
integer(c_int32_t), allocatable :: iflag(:)
integer :: s
IF (.NOT. sk_ready) THEN
  cfg%lx = INT(Box(1)); cfg%ly = INT(Box(2)); cfg%lz = INT(Box(3))
  cfg%geometry = MPCMD_GEOM_PERIODIC
  cfg%n_dimers = 1
  cfg%kinetics = MPCMD_KIN_SELKOV
  cfg%exclusion = MPCMD_EXCL_CELLS
  cfg%catalysis = MPCMD_CAT_PROBABILISTIC
  cfg%rotation_sense = -1
  cfg%mpc_every = INT(MPCtstep)
  cfg%sort_every = 10000
  cfg%react_box_type = 7
  cfg%react_dir = 0
  cfg%cell_capacity = MaxF
  cfg%max_neighbour = 30000
  cfg%rattle_max_iter = 100000
  cfg%init_plane = 0
  cfg%pad0 = 0
  cfg%n_solvent = NT
  cfg%seed = INT(seed, c_int64_t)
  cfg%init_count = [0_c_int64_t, 0_c_int64_t, 0_c_int64_t, 0_c_int64_t]
  cfg%init_count(1) = NT
  cfg%mass = [Mf, Mg, 1.0_c_double, Mi]
  cfg%eps_c = [EfC, EgC, 0.0_c_double, EiC]
  cfg%eps_n = [EfN, EgN, 0.0_c_double, EiN]
  cfg%rc = Rc; cfg%rn = Rn; cfg%dcn = Dcn; cfg%mc = Mc; cfg%mn = Mn
  cfg%rw = 1.0_c_double; cfg%ew = 1.0_c_double; cfg%rm_delta = 1.0_c_double; cfg%em = 1.0_c_double
  cfg%rp_ab = RPfg; cfg%rp_ba = RPgf
  cfg%kT = T
  cfg%skin = 1.5_c_double
  cfg%rot_angle = rotang
  cfg%md_dt = MDt
  cfg%mpc_dt = MPCt
  cfg%k = [k1, k2, k3, k4, k5, k6]
  cfg%precision = sk_precision
  cfg%shell_capacity = 0
  cfg%variant = MPCMD_VARIANT_MOTOR
  cfg%layout = MPCMD_LAYOUT_RANDOM
  cfg%layout_rows = 0; cfg%layout_cols = 0
  cfg%owner_tags = 0; cfg%reserved = 0
  cfg%tether_k = 0.0_c_double; cfg%tether_z = 0.0_c_double; cfg%layout_sep = 0.0_c_double
  CALL mpcmd_check(mpcmd_create(cfg, sk_ctx), 'create')
  ALLOCATE(dpos(3, 2), dvel(3, 2), dfrc(3, 2), iflag(NT))
  DO s = 1, 2
    dpos(:, s) = [Xdim(s), Ydim(s), Zdim(s)]
    dvel(:, s) = [VXdim(s), VYdim(s), VZdim(s)]
    dfrc(:, s) = [FXdim(s), FYdim(s), FZdim(s)]
  END DO
  iflag = INT(FLAG(1:NT), c_int32_t)
  CALL mpcmd_check(mpcmd_upload_state(sk_ctx, Xsol, Ysol, Zsol, VXsol, VYsol, VZsol, iflag, dpos, dvel, dfrc), &
                   'upload_state')
  CALL mpcmd_check(mpcmd_set_step(sk_ctx, INT(cstep - 1, c_int64_t), 0_c_int32_t), 'set_step')
  CALL mpcmd_check(mpcmd_prepare_restart(sk_ctx), 'prepare_restart')
  sk_ready = .TRUE.
END IF
CALL mpcmd_check(mpcmd_evolve(sk_ctx), 'evolve')
END SUBROUTINE Motion_SelkovDimer

SUBROUTINE ForcesMD_SelkovDimer
! (the forces, velocities and RATTLE velocities of this step ran in Motion_SelkovDimer)
END SUBROUTINE ForcesMD_SelkovDimer

SUBROUTINE Distribute_SelkovDimer
USE mpcmd_selkov_state
IMPLICIT NONE
CALL mpcmd_check(mpcmd_distribute(sk_ctx), 'distribute')
END SUBROUTINE Distribute_SelkovDimer

SUBROUTINE Affected_Cell
! (marked by Distribute_SelkovDimer: the engine's distribute stage includes Affected_Cell.f90:7-101)
END SUBROUTINE Affected_Cell

SUBROUTINE Sort
! (the context sorts on its sort steps, every 10,000 steps as Main_SelkovDimer.f90:128 calls Sort)
END SUBROUTINE Sort

SUBROUTINE RMPC_SelkovDimer
USE Global_SelkovDimer
USE mpcmd_selkov_state
IMPLICIT NONE
real(c_double), allocatable :: dpos(:,:), dvel(:,:), dfrc(:,:)
integer(c_int32_t), allocatable :: iflag(:)
integer :: s
CALL mpcmd_check(mpcmd_mpc_rotation(sk_ctx), 'mpc_rotation')
CALL mpcmd_check(mpcmd_reaction(sk_ctx), 'reaction')
! the state of this collision step back to the module arrays
ALLOCATE(dpos(3, 2), dvel(3, 2), dfrc(3, 2), iflag(NT))
CALL mpcmd_check(mpcmd_download_state(sk_ctx, Xsol, Ysol, Zsol, VXsol, VYsol, VZsol, iflag, dpos, dvel, dfrc), &
                 'download_state')
FLAG(1:NT) = INT(iflag, KIND(FLAG))
DO s = 1, 2
  Xdim(s) = dpos(1, s); Ydim(s) = dpos(2, s); Zdim(s) = dpos(3, s)
  VXdim(s) = dvel(1, s); VYdim(s) = dvel(2, s); VZdim(s) = dvel(3, s)
  FXdim(s) = dfrc(1, s); FYdim(s) = dfrc(2, s); FZdim(s) = dfrc(3, s)
END DO
END SUBROUTINE RMPC_SelkovDimer
