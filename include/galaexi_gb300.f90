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
END INTERFACE

! the operator context of this process (one per host thread and stream)
TYPE(C_PTR) :: gb300_ctx = C_NULL_PTR

END MODULE MOD_GB300
