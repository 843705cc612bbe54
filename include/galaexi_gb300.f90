!==================================================================================================
! MOD_GB300: Fortran 2003 ISO_C_BINDING interface to libgalaexi_gb300 (include/galaexi_gb300.h).
!
! The module a GALAEXI maintainer adds to the reference's host code so that its DG operator and
! time stepper call the GB300 kernels through the C ABI:
!   DGTimeDerivative_weakForm(t)   (src/dg/dg.f90:255)             -> dg_rhs
!   TimeStepByLSERKW2(t)           (src/timedisc/timestep.f90:49)  -> dg_lserk_step
!   CALCTIMESTEP(errType)          (src/timedisc/calctimestep.f90:98) -> dg_calc_timestep
! Device arrays are passed by address (C_DEVLOC of the CUDA Fortran device arrays, TYPE(C_PTR)
! VALUE here); host arrays (mesh, metrics, BC tables) in the reference's own Fortran layouts with
! 1-based IDs.  Every function returns 0 or a negative DG_ERR_* status; dg_last_error() gives the
! text.  Only standard ISO_C_BINDING is used: any Fortran 2003 compiler can build this file; the
! CUDA Fortran side (C_DEVLOC) is in the calling code.
!==================================================================================================
MODULE MOD_GB300
USE ISO_C_BINDING
IMPLICIT NONE

! status codes (include/galaexi_gb300.h)
INTEGER(C_INT), PARAMETER :: DG_OK              =  0
INTEGER(C_INT), PARAMETER :: DG_ERR_ARG         = -1
INTEGER(C_INT), PARAMETER :: DG_ERR_ALLOC       = -2
INTEGER(C_INT), PARAMETER :: DG_ERR_CUDA        = -3
INTEGER(C_INT), PARAMETER :: DG_ERR_NAN         = -4
INTEGER(C_INT), PARAMETER :: DG_ERR_TIMEOUT     = -5
INTEGER(C_INT), PARAMETER :: DG_ERR_UNSUPPORTED = -6

! option values of dg_config (the reference's NodeType, RIEMANN, SPLIT_DG, PP_Lifting and FilterType
! numbering) and the other constants of the header
INTEGER(C_INT), PARAMETER :: DG_NODETYPE_GAUSS         = 1
INTEGER(C_INT), PARAMETER :: DG_NODETYPE_GAUSS_LOBATTO = 2
INTEGER(C_INT), PARAMETER :: DG_RIEMANN_LF             = 0
INTEGER(C_INT), PARAMETER :: DG_RIEMANN_ROE            = 1
INTEGER(C_INT), PARAMETER :: DG_RIEMANN_ROEL2          = 2
INTEGER(C_INT), PARAMETER :: DG_RIEMANN_ROEENTROPYFIX  = 3
INTEGER(C_INT), PARAMETER :: DG_RIEMANN_HLL            = 4
INTEGER(C_INT), PARAMETER :: DG_RIEMANN_HLLC           = 5
INTEGER(C_INT), PARAMETER :: DG_RIEMANN_HLLE           = 6
INTEGER(C_INT), PARAMETER :: DG_RIEMANN_HLLEM          = 7
INTEGER(C_INT), PARAMETER :: DG_RIEMANN_AVERAGE        = 8
INTEGER(C_INT), PARAMETER :: DG_SPLIT_NONE             = -1
INTEGER(C_INT), PARAMETER :: DG_SPLIT_SD               = 0
INTEGER(C_INT), PARAMETER :: DG_SPLIT_MO               = 1
INTEGER(C_INT), PARAMETER :: DG_SPLIT_DU               = 2
INTEGER(C_INT), PARAMETER :: DG_SPLIT_KG               = 3
INTEGER(C_INT), PARAMETER :: DG_SPLIT_PI               = 4
INTEGER(C_INT), PARAMETER :: DG_LIFTING_BR1            = 1
INTEGER(C_INT), PARAMETER :: DG_LIFTING_BR2            = 2
INTEGER(C_INT), PARAMETER :: DG_PRECISION_FP64         = 0
INTEGER(C_INT), PARAMETER :: DG_PRECISION_MIXED        = 1
INTEGER(C_INT), PARAMETER :: DG_FILTER_NONE            = 0
INTEGER(C_INT), PARAMETER :: DG_FILTER_CUTOFF          = 1
INTEGER(C_INT), PARAMETER :: DG_FILTER_MODAL           = 2
INTEGER(C_INT), PARAMETER :: DG_FILTER_LAF             = 3
INTEGER(C_INT), PARAMETER :: DG_MAX_N                  = 9
INTEGER(C_INT), PARAMETER :: DG_NOALLOC_MAX_ELEMS      = 524288
INTEGER(C_INT), PARAMETER :: DG_EXACTFUNC_CONST        = 1
INTEGER(C_INT), PARAMETER :: DG_EXACTFUNC_SHU_VORTEX   = 7
INTEGER(C_INT), PARAMETER :: DG_EXACTFUNC_TGV          = 100

! run-time configuration: the C struct dg_config field by field
TYPE, BIND(C) :: dg_config
  INTEGER(C_INT) :: N, node_type, parabolic, riemann, split_dg, lifting
  INTEGER(C_INT) :: do_weak_lifting, do_conservative_lifting
  REAL(C_DOUBLE) :: eta_br2, kappa, R, Pr, mu0
  INTEGER(C_INT) :: precision
  INTEGER(C_INT) :: filter_type, n_filter
  REAL(C_DOUBLE) :: hest_filter_param(3), laf_alpha
END TYPE dg_config

INTERFACE
  SUBROUTINE dg_config_default(cfg) BIND(C,NAME='dg_config_default')
    IMPORT :: dg_config
    TYPE(dg_config), INTENT(OUT) :: cfg
  END SUBROUTINE dg_config_default

  ! ini_text: NUL-terminated key = value lines (the reference's parameter file syntax)
  INTEGER(C_INT) FUNCTION dg_config_from_ini(ini_text, cfg) BIND(C,NAME='dg_config_from_ini')
    IMPORT :: C_INT, C_CHAR, dg_config
    CHARACTER(KIND=C_CHAR), INTENT(IN) :: ini_text(*)
    TYPE(dg_config), INTENT(INOUT) :: cfg
  END FUNCTION dg_config_from_ini

  INTEGER(C_INT) FUNCTION dg_ctx_create(cfg, ctx) BIND(C,NAME='dg_ctx_create')
    IMPORT :: C_INT, C_PTR, dg_config
    TYPE(dg_config), INTENT(IN) :: cfg
    TYPE(C_PTR), INTENT(OUT) :: ctx
  END FUNCTION dg_ctx_create

  INTEGER(C_INT) FUNCTION dg_ctx_destroy(ctx) BIND(C,NAME='dg_ctx_destroy')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: ctx
  END FUNCTION dg_ctx_destroy

  ! Metrics_fTilde(3,0:N,0:N,0:N,nElems) ... sJ(0:N,0:N,0:N,nElems), NormVec/TangVec1/TangVec2(3,0:N,0:N,nSides),
  ! SurfElem(0:N,0:N,nSides), ElemToSide(3,6,nElems), SideToElem(5,nSides); int32 with 1-based IDs
  INTEGER(C_INT) FUNCTION dg_set_mesh(ctx, nElems, nSides, nBCSides, Mf, Mg, Mh, sJ, nv, t1, t2, se, E2S, S2E) &
                                      BIND(C,NAME='dg_set_mesh')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: ctx
    INTEGER(C_INT), VALUE :: nElems, nSides, nBCSides
    REAL(C_DOUBLE), INTENT(IN) :: Mf(*), Mg(*), Mh(*), sJ(*), nv(*), t1(*), t2(*), se(*)
    INTEGER(C_INT), INTENT(IN) :: E2S(*), S2E(*)
  END FUNCTION dg_set_mesh

  ! BCSides(BC_TYPE,1:nBCSides), BCSides(BC_STATE,1:nBCSides), RefStatePrim rows as read (rho,u,v,w,p)
  INTEGER(C_INT) FUNCTION dg_set_boundaries(ctx, bc_type, bc_state, nRefState, refstate) &
                                            BIND(C,NAME='dg_set_boundaries')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: ctx
    INTEGER(C_INT), INTENT(IN) :: bc_type(*), bc_state(*)
    INTEGER(C_INT), VALUE :: nRefState
    REAL(C_DOUBLE), INTENT(IN) :: refstate(5,*)
  END FUNCTION dg_set_boundaries

  ! DGTimeDerivative_weakForm(t): d_Ut = R(d_U), device arrays (5,0:N,0:N,0:N,nElems)
  INTEGER(C_INT) FUNCTION dg_rhs(ctx, t, d_U, d_Ut, stream) BIND(C,NAME='dg_rhs')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: ctx, d_U, d_Ut, stream
    REAL(C_DOUBLE), VALUE :: t
  END FUNCTION dg_rhs

  ! TimeStepByLSERKW2(t): one Carpenter-Kennedy RK4-5 step of d_U with the caller's Ut_tmp register
  INTEGER(C_INT) FUNCTION dg_lserk_step(ctx, t, dt, d_U, d_Ut_tmp, stream) BIND(C,NAME='dg_lserk_step')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: ctx, d_U, d_Ut_tmp, stream
    REAL(C_DOUBLE), VALUE :: t, dt
  END FUNCTION dg_lserk_step

  INTEGER(C_INT) FUNCTION dg_lserk_steps(ctx, t, dt, nSteps, d_U, d_Ut_tmp, stream) BIND(C,NAME='dg_lserk_steps')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: ctx, d_U, d_Ut_tmp, stream
    REAL(C_DOUBLE), VALUE :: t, dt
    INTEGER(C_INT), VALUE :: nSteps
  END FUNCTION dg_lserk_steps

  ! CALCTIMESTEP with the FillCFL_DFL scaling; returns DG_ERR_NAN for a bad state (the reference's errType)
  INTEGER(C_INT) FUNCTION dg_calc_timestep(ctx, d_U, cfl, dfl, dt, stream) BIND(C,NAME='dg_calc_timestep')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: ctx, d_U, stream
    REAL(C_DOUBLE), VALUE :: cfl, dfl
    REAL(C_DOUBLE), INTENT(OUT) :: dt
  END FUNCTION dg_calc_timestep

  INTEGER(C_INT) FUNCTION dg_check_state(ctx, d_U, bad_count, stream) BIND(C,NAME='dg_check_state')
    IMPORT :: C_INT, C_PTR, C_LONG_LONG
    TYPE(C_PTR), VALUE :: ctx, d_U, stream
    INTEGER(C_LONG_LONG), INTENT(OUT) :: bad_count
  END FUNCTION dg_check_state

  ! the lifting module arrays GradUx/GradUy/GradUz(5,0:N,0:N,0:N,nElems) of the last operator call
  INTEGER(C_INT) FUNCTION dg_get_gradients(ctx, d_gradUx, d_gradUy, d_gradUz, stream) &
                                           BIND(C,NAME='dg_get_gradients')
    IMPORT :: C_INT, C_PTR
    TYPE(C_PTR), VALUE :: ctx, d_gradUx, d_gradUy, d_gradUz, stream
  END FUNCTION dg_get_gradients

  ! discrete adjoint (no counterpart in the reference): d_Ubar = (dR/dU)^T d_Utbar, mu_bar = <d_Utbar, dR/dmu>
  INTEGER(C_INT) FUNCTION dg_rhs_vjp(ctx, t, d_U, d_Utbar, d_Ubar, mu_bar, stream) BIND(C,NAME='dg_rhs_vjp')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: ctx, d_U, d_Utbar, d_Ubar, stream
    REAL(C_DOUBLE), VALUE :: t
    REAL(C_DOUBLE), INTENT(OUT) :: mu_bar
  END FUNCTION dg_rhs_vjp

  ! kinetic-energy objective of the end state of nSteps LSERK steps and its gradient w.r.t. the start
  ! state and mu, with checkpoints in at most budget_bytes of device memory; d_U_final may be C_NULL_PTR
  INTEGER(C_INT) FUNCTION dg_adjoint_window(ctx, t0, dt, nSteps, d_U0, budget_bytes, J, d_dJdU0, dJdmu, &
                                            d_U_final, stream) BIND(C,NAME='dg_adjoint_window')
    IMPORT :: C_INT, C_PTR, C_DOUBLE, C_SIZE_T
    TYPE(C_PTR), VALUE :: ctx, d_U0, d_dJdU0, d_U_final, stream
    REAL(C_DOUBLE), VALUE :: t0, dt
    INTEGER(C_INT), VALUE :: nSteps
    INTEGER(C_SIZE_T), VALUE :: budget_bytes
    REAL(C_DOUBLE), INTENT(OUT) :: J, dJdmu
  END FUNCTION dg_adjoint_window

  ! NUL-terminated description of the last error on the calling thread (C_F_POINTER to read it)
  TYPE(C_PTR) FUNCTION dg_last_error() BIND(C,NAME='dg_last_error')
    IMPORT :: C_PTR
  END FUNCTION dg_last_error

  ! ---- further operator entry points ----------------------------------------------------------
  ! per-element LAF filter state (LAF_lim, LAF_eRatio, LAF_r) after the last operator call, host arrays
  INTEGER(C_INT) FUNCTION dg_laf_state(ctx, lim, eRatio, r) BIND(C,NAME='dg_laf_state')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: ctx
    REAL(C_DOUBLE), INTENT(OUT) :: lim(*), eRatio(*), r(*)
  END FUNCTION dg_laf_state

  ! CALCTIMESTEP without a context and without any allocation (scratch: a static device array of the
  ! library, at most DG_NOALLOC_MAX_ELEMS elements), for callers whose device memory belongs to
  ! nvfortran's allocator; the caller's device U, Metrics_f/g/hTilde and sJ
  INTEGER(C_INT) FUNCTION dg_calc_timestep_noalloc(N, node_type, nElems, parabolic, kappa, mu0, Pr, d_U, d_Mf, &
                                                   d_Mg, d_Mh, d_sJ, cfl, dfl, dt, stream) &
                                                   BIND(C,NAME='dg_calc_timestep_noalloc')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    INTEGER(C_INT), VALUE :: N, node_type, nElems, parabolic
    REAL(C_DOUBLE), VALUE :: kappa, mu0, Pr, cfl, dfl
    TYPE(C_PTR), VALUE :: d_U, d_Mf, d_Mg, d_Mh, d_sJ, stream
    REAL(C_DOUBLE), INTENT(OUT) :: dt
  END FUNCTION dg_calc_timestep_noalloc

  ! mass, momentum (3), total energy and kinetic energy integrals of d_U (host out6(6))
  INTEGER(C_INT) FUNCTION dg_integrals(ctx, d_U, out6, stream) BIND(C,NAME='dg_integrals')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: ctx, d_U, stream
    REAL(C_DOUBLE), INTENT(OUT) :: out6(6)
  END FUNCTION dg_integrals

  INTEGER(C_INT) FUNCTION dg_kinetic_energy(ctx, d_U, J, d_dJdU, stream) BIND(C,NAME='dg_kinetic_energy')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: ctx, d_U, d_dJdU, stream
    REAL(C_DOUBLE), INTENT(OUT) :: J
  END FUNCTION dg_kinetic_energy

  ! tangent-linear operator and stepper (no counterpart in the reference)
  INTEGER(C_INT) FUNCTION dg_rhs_jvp(ctx, t, d_U, d_Udot, mu_dot, d_Ut, d_Utdot, stream) BIND(C,NAME='dg_rhs_jvp')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: ctx, d_U, d_Udot, d_Ut, d_Utdot, stream
    REAL(C_DOUBLE), VALUE :: t, mu_dot
  END FUNCTION dg_rhs_jvp

  INTEGER(C_INT) FUNCTION dg_tlm_steps(ctx, t, dt, nSteps, d_U, d_Udot, mu_dot, d_Ut_tmp, stream) &
                                       BIND(C,NAME='dg_tlm_steps')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: ctx, d_U, d_Udot, d_Ut_tmp, stream
    REAL(C_DOUBLE), VALUE :: t, dt, mu_dot
    INTEGER(C_INT), VALUE :: nSteps
  END FUNCTION dg_tlm_steps

  ! the adjoint window in two calls: record (checkpoint plan 1, 2 or 3 within budget_bytes), then reverse
  INTEGER(C_INT) FUNCTION dg_adjoint_forward(ctx, t0, dt, nSteps, d_U0, d_U_final, budget_bytes, plan, stream) &
                                             BIND(C,NAME='dg_adjoint_forward')
    IMPORT :: C_INT, C_PTR, C_DOUBLE, C_SIZE_T
    TYPE(C_PTR), VALUE :: ctx, d_U0, d_U_final, stream
    REAL(C_DOUBLE), VALUE :: t0, dt
    INTEGER(C_INT), VALUE :: nSteps
    INTEGER(C_SIZE_T), VALUE :: budget_bytes
    INTEGER(C_INT), INTENT(OUT) :: plan
  END FUNCTION dg_adjoint_forward

  INTEGER(C_INT) FUNCTION dg_adjoint_scratch_bytes(ctx, nbytes) BIND(C,NAME='dg_adjoint_scratch_bytes')
    IMPORT :: C_INT, C_PTR, C_SIZE_T
    TYPE(C_PTR), VALUE :: ctx
    INTEGER(C_SIZE_T), INTENT(OUT) :: nbytes
  END FUNCTION dg_adjoint_scratch_bytes

  INTEGER(C_INT) FUNCTION dg_adjoint_reverse(ctx, d_Ubar, mu_bar, stream) BIND(C,NAME='dg_adjoint_reverse')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: ctx, d_Ubar, stream
    REAL(C_DOUBLE), INTENT(OUT) :: mu_bar
  END FUNCTION dg_adjoint_reverse

  ! reference pressure of the mixed form (p' = p - p_ref in the FP32 momentum pressure terms)
  INTEGER(C_INT) FUNCTION dg_set_pressure_offset(ctx, p_ref) BIND(C,NAME='dg_set_pressure_offset')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: ctx
    REAL(C_DOUBLE), VALUE :: p_ref
  END FUNCTION dg_set_pressure_offset

  ! measurement: CUDA-event times of (prolong, lift, face, volume, stage) in ms_out(5); FMA peak in GFLOP/s
  INTEGER(C_INT) FUNCTION dg_profile_stage(ctx, d_U, d_Ut_tmp, dt, reps, ms_out, stream) &
                                           BIND(C,NAME='dg_profile_stage')
    IMPORT :: C_INT, C_PTR, C_DOUBLE
    TYPE(C_PTR), VALUE :: ctx, d_U, d_Ut_tmp, stream
    REAL(C_DOUBLE), VALUE :: dt
    INTEGER(C_INT), VALUE :: reps
    REAL(C_DOUBLE), INTENT(OUT) :: ms_out(5)
  END FUNCTION dg_profile_stage

  INTEGER(C_INT) FUNCTION dg_measure_fma_peak(precision, gflops) BIND(C,NAME='dg_measure_fma_peak')
    IMPORT :: C_INT, C_DOUBLE
    INTEGER(C_INT), VALUE :: precision
    REAL(C_DOUBLE), INTENT(OUT) :: gflops
  END FUNCTION dg_measure_fma_peak

  INTEGER(C_INT) FUNCTION dg_selftest_bulk_wait(polls, seconds) BIND(C,NAME='dg_selftest_bulk_wait')
    IMPORT :: C_INT, C_LONG_LONG, C_DOUBLE
    INTEGER(C_LONG_LONG), VALUE :: polls
    REAL(C_DOUBLE), INTENT(OUT) :: seconds
  END FUNCTION dg_selftest_bulk_wait

  INTEGER(C_LONG_LONG) FUNCTION dg_kernel_launch_count(ctx) BIND(C,NAME='dg_kernel_launch_count')
    IMPORT :: C_LONG_LONG, C_PTR
    TYPE(C_PTR), VALUE :: ctx
  END FUNCTION dg_kernel_launch_count

  ! ---- files and host-side set-up (strings NUL-terminated: TRIM(path)//C_NULL_CHAR) -------------
  INTEGER(C_INT) FUNCTION dg_mesh_hopr_sizes(path, nElems, nSides, nBCSides, NGeo) BIND(C,NAME='dg_mesh_hopr_sizes')
    IMPORT :: C_INT, C_CHAR
    CHARACTER(KIND=C_CHAR), INTENT(IN) :: path(*)
    INTEGER(C_INT), INTENT(OUT) :: nElems, nSides, nBCSides, NGeo
  END FUNCTION dg_mesh_hopr_sizes

  ! BCNames (nBCs x name_len characters) and BCType(4,nBCs) of a HOPR mesh file
  INTEGER(C_INT) FUNCTION dg_mesh_hopr_bcs(path, nBCs, names, name_len, bc_type) BIND(C,NAME='dg_mesh_hopr_bcs')
    IMPORT :: C_INT, C_CHAR
    CHARACTER(KIND=C_CHAR), INTENT(IN) :: path(*)
    INTEGER(C_INT), INTENT(OUT) :: nBCs
    CHARACTER(KIND=C_CHAR), INTENT(OUT) :: names(*)
    INTEGER(C_INT), VALUE :: name_len
    INTEGER(C_INT), INTENT(OUT) :: bc_type(*)
  END FUNCTION dg_mesh_hopr_bcs

  ! a dataset (attribute = 0) or root attribute (attribute = 1) of an HDF5 file: dims(8), slowest first
  INTEGER(C_INT) FUNCTION dg_h5_read(path, dset, attribute, ndims, dims, values, cap, str, str_len) &
                                     BIND(C,NAME='dg_h5_read')
    IMPORT :: C_INT, C_CHAR, C_DOUBLE, C_LONG_LONG
    CHARACTER(KIND=C_CHAR), INTENT(IN) :: path(*), dset(*)
    INTEGER(C_INT), VALUE :: attribute, str_len
    INTEGER(C_INT), INTENT(OUT) :: ndims
    INTEGER(C_LONG_LONG), INTENT(OUT) :: dims(8)
    REAL(C_DOUBLE), INTENT(OUT) :: values(*)
    INTEGER(C_LONG_LONG), VALUE :: cap
    CHARACTER(KIND=C_CHAR), INTENT(OUT) :: str(*)
  END FUNCTION dg_h5_read

  ! WriteState: a FLEXI state file with DG_Solution(5,0:N,0:N,0:N,nElems) from the host array U
  INTEGER(C_INT) FUNCTION dg_write_state(path, project, mesh_file, N, node_type, t, nElems, U) &
                                         BIND(C,NAME='dg_write_state')
    IMPORT :: C_INT, C_CHAR, C_DOUBLE
    CHARACTER(KIND=C_CHAR), INTENT(IN) :: path(*), project(*), mesh_file(*), node_type(*)
    INTEGER(C_INT), VALUE :: N, nElems
    REAL(C_DOUBLE), VALUE :: t
    REAL(C_DOUBLE), INTENT(IN) :: U(*)
  END FUNCTION dg_write_state

  ! ReadMesh + CalcMetrics of a HOPR mesh file: the arrays of dg_set_mesh, Elem_xGP and the BC indices
  INTEGER(C_INT) FUNCTION dg_mesh_hopr(path, N, node_type, xgp, Mf, Mg, Mh, sJ, nv, t1, t2, se, E2S, S2E, BCIndex) &
                                       BIND(C,NAME='dg_mesh_hopr')
    IMPORT :: C_INT, C_CHAR, C_DOUBLE
    CHARACTER(KIND=C_CHAR), INTENT(IN) :: path(*)
    INTEGER(C_INT), VALUE :: N, node_type
    REAL(C_DOUBLE), INTENT(OUT) :: xgp(*), Mf(*), Mg(*), Mh(*), sJ(*), nv(*), t1(*), t2(*), se(*)
    INTEGER(C_INT), INTENT(OUT) :: E2S(*), S2E(*), BCIndex(*)
  END FUNCTION dg_mesh_hopr

  ! InitInterpolationBasis + InitDGbasis: nodes, weights and the 1D operators ((0:N,0:N) column-major)
  INTEGER(C_INT) FUNCTION dg_basis(N, node_type, xGP, wGP, wBary, L_minus, L_plus, D, D_hat_T, L_hat_minus, &
                                   L_hat_plus, DVolSurf) BIND(C,NAME='dg_basis')
    IMPORT :: C_INT, C_DOUBLE
    INTEGER(C_INT), VALUE :: N, node_type
    REAL(C_DOUBLE), INTENT(OUT) :: xGP(*), wGP(*), wBary(*), L_minus(*), L_plus(*), D(*), D_hat_T(*)
    REAL(C_DOUBLE), INTENT(OUT) :: L_hat_minus(*), L_hat_plus(*), DVolSurf(*)
  END FUNCTION dg_basis

  INTEGER(C_INT) FUNCTION dg_mesh_cartesian_sizes(nx, ny, nz, nElems, nSides) BIND(C,NAME='dg_mesh_cartesian_sizes')
    IMPORT :: C_INT
    INTEGER(C_INT), VALUE :: nx, ny, nz
    INTEGER(C_INT), INTENT(OUT) :: nElems, nSides
  END FUNCTION dg_mesh_cartesian_sizes

  ! a periodic box [x0,x1] of nx*ny*nz elements of mapping degree NGeo, optionally displaced (deform_amp), in the
  ! dg_set_mesh layouts plus NodeCoords(3,0:NGeo,0:NGeo,0:NGeo,nElems) and Elem_xGP
  INTEGER(C_INT) FUNCTION dg_mesh_cartesian(N, node_type, NGeo, nx, ny, nz, x0, x1, deform_amp, nodes, xgp, Mf, Mg, &
                                            Mh, sJ, nv, t1, t2, se, E2S, S2E) BIND(C,NAME='dg_mesh_cartesian')
    IMPORT :: C_INT, C_DOUBLE
    INTEGER(C_INT), VALUE :: N, node_type, NGeo, nx, ny, nz
    REAL(C_DOUBLE), INTENT(IN) :: x0(3), x1(3)
    REAL(C_DOUBLE), VALUE :: deform_amp
    REAL(C_DOUBLE), INTENT(OUT) :: nodes(*), xgp(*), Mf(*), Mg(*), Mh(*), sJ(*), nv(*), t1(*), t2(*), se(*)
    INTEGER(C_INT), INTENT(OUT) :: E2S(*), S2E(*)
  END FUNCTION dg_mesh_cartesian

  ! FillIni: U(5,nNodes) at the node coordinates xgp(3,nNodes) for DG_EXACTFUNC_* and its parameters
  INTEGER(C_INT) FUNCTION dg_fill_ini(exactfunc, params, nParams, nNodes, xgp, kappa, R, t, U) &
                                      BIND(C,NAME='dg_fill_ini')
    IMPORT :: C_INT, C_DOUBLE, C_LONG_LONG
    INTEGER(C_INT), VALUE :: exactfunc, nParams
    REAL(C_DOUBLE), INTENT(IN) :: params(*), xgp(*)
    INTEGER(C_LONG_LONG), VALUE :: nNodes
    REAL(C_DOUBLE), VALUE :: kappa, R, t
    REAL(C_DOUBLE), INTENT(OUT) :: U(*)
  END FUNCTION dg_fill_ini
END INTERFACE

! the operator context of this process (one per host thread and stream)
TYPE(C_PTR) :: gb300_ctx = C_NULL_PTR

END MODULE MOD_GB300
