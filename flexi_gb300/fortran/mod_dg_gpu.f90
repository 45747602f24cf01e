!==================================================================================================================================
! MOD_DG_GPU: the FLEXI side of libflexigpu.so.
!
! Part 1 binds every function of the C ABI (include/flexi_gpu.h) with ISO_C_BINDING: the three structs as BIND(C) derived
! types, every entry point as a BIND(C) interface (handles and opaque pointers as TYPE(C_PTR), VALUE; arrays and scalars
! written by the library by reference; strings as NUL-terminated CHARACTER(KIND=C_CHAR) arrays; outputs the library accepts
! as NULL as OPTIONAL dummies, which an absent actual argument passes as NULL).
!
! Part 2 is the shim a FLEXI build adds to use it: InitDG_GPU hands the module arrays of MOD_Mesh_Vars / MOD_DG_Vars over
! once after InitFlexi (flexilib.f90), DGTimeDerivative_GPU replaces DGTimeDerivative_weakForm (dg.f90:221),
! TimeStepByLSERKW2_GPU is the target of the TimeStep procedure pointer (timestep.f90:37-39,64), CalcTimeStep_GPU
! replaces CALCTIMESTEP inside EvalTimeStep (timedisc_func.f90:443), TimeDiscSteps_GPU runs the TimeDisc loop body on the
! device (timedisc.f90:190-212), GetState_GPU copies U back before WriteState/Analyze, FinalizeDG_GPU frees the handle.
! Compiled as part of FLEXI (flexi.h preprocessor macros, -fdefault-real-8: REAL is C_DOUBLE).
!==================================================================================================================================
#include "flexi.h"

MODULE MOD_DG_GPU
USE ISO_C_BINDING
IMPLICIT NONE
PRIVATE

!----------------------------------------------------------------------------------------------------------------------------------
! Part 1: the C ABI
!----------------------------------------------------------------------------------------------------------------------------------
INTEGER(C_INT),PARAMETER,PUBLIC :: FG_OK=0, FG_ERR_CONFIG=1, FG_ERR_MESH=2, FG_ERR_CUDA=3, FG_ERR_STATE=4, FG_ERR_NAN=5, &
                                   FG_ERR_DT=6, FG_ERR_DTKILL=7

TYPE, BIND(C), PUBLIC :: fg_config
  INTEGER(C_INT)  :: N, NodeType, Riemann, RiemannBC, Lifting, doWeakLifting, doConservativeLifting, SplitDG
  REAL(C_DOUBLE)  :: etaBR2, etaBR2_wall, kappa, R, Pr, mu0, CFLScale, DFLScale
  INTEGER(C_INT)  :: doTCSource
  REAL(C_DOUBLE)  :: dpdx
  INTEGER(C_INT)  :: TimeDiscMethod, OverintegrationType, NUnder, IniExactFunc
  REAL(C_DOUBLE)  :: AdvVel(3), IniFrequency, IniAmplitude
  REAL(C_DOUBLE)  :: TEnd, Analyze_dt, dtmin, dtkill
  INTEGER(C_INT)  :: nCalcTimeStepMax, maxIter
  REAL(C_DOUBLE)  :: RiemannPhiFactor
END TYPE fg_config

TYPE, BIND(C), PUBLIC :: fg_timedisc_state
  REAL(C_DOUBLE)       :: t, dt, dtMin
  INTEGER(C_LONG_LONG) :: iter
  INTEGER(C_INT)       :: atAnalyze, finished, nDtLimited
END TYPE fg_timedisc_state

TYPE, BIND(C), PUBLIC :: fg_device_mesh
  INTEGER(C_INT) :: nElems, nSides, nBCSides
  TYPE(C_PTR)    :: elemSide, sideElem, metr, sJ, geo, bcType, bcTwall
END TYPE fg_device_mesh

INTERFACE
  INTEGER(C_INT) FUNCTION fg_config_default(cfg) BIND(C,NAME='fg_config_default')
    IMPORT; TYPE(fg_config) :: cfg
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_config_from_ini(ini_text, cfg) BIND(C,NAME='fg_config_from_ini')
    IMPORT; CHARACTER(KIND=C_CHAR) :: ini_text(*); TYPE(fg_config) :: cfg
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_create(cfg, h) BIND(C,NAME='fg_create')
    IMPORT; TYPE(fg_config) :: cfg; TYPE(C_PTR) :: h
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_destroy(h) BIND(C,NAME='fg_destroy')
    IMPORT; TYPE(C_PTR), VALUE :: h
  END FUNCTION
  TYPE(C_PTR) FUNCTION fg_last_error(h) BIND(C,NAME='fg_last_error')
    IMPORT; TYPE(C_PTR), VALUE :: h
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_build_mesh(h, nElems, NGeo, NodeCoords, ElemNb, nBCs, BoundaryType, nRefStates, RefStatePrim, &
                                        ElemInst) BIND(C,NAME='fg_build_mesh')
    IMPORT; TYPE(C_PTR), VALUE :: h; INTEGER(C_INT), VALUE :: nElems, NGeo
    REAL(C_DOUBLE) :: NodeCoords(*); INTEGER(C_INT) :: ElemNb(*)
    INTEGER(C_INT), VALUE :: nBCs; INTEGER(C_INT) :: BoundaryType(*)
    INTEGER(C_INT), VALUE :: nRefStates; REAL(C_DOUBLE) :: RefStatePrim(*)
    INTEGER(C_INT), OPTIONAL :: ElemInst(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_build_mesh_mortar(h, nElems, NGeo, NodeCoords, ElemNb, nBCs, BoundaryType, nRefStates, &
                                               RefStatePrim, ElemInst, nMortars, Mortars) BIND(C,NAME='fg_build_mesh_mortar')
    IMPORT; TYPE(C_PTR), VALUE :: h; INTEGER(C_INT), VALUE :: nElems, NGeo
    REAL(C_DOUBLE) :: NodeCoords(*); INTEGER(C_INT) :: ElemNb(*)
    INTEGER(C_INT), VALUE :: nBCs; INTEGER(C_INT) :: BoundaryType(*)
    INTEGER(C_INT), VALUE :: nRefStates; REAL(C_DOUBLE) :: RefStatePrim(*)
    INTEGER(C_INT), OPTIONAL :: ElemInst(*)
    INTEGER(C_INT), VALUE :: nMortars; INTEGER(C_INT), OPTIONAL :: Mortars(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_set_mesh(h, nElems, nSides, nBCSides, SideToElem, ElemToSide, BC, nBCs, BoundaryType, nRefStates, &
                                      RefStatePrim, Metrics_fTilde, Metrics_gTilde, Metrics_hTilde, sJ, NormVec, TangVec1, &
                                      TangVec2, SurfElem) BIND(C,NAME='fg_set_mesh')
    IMPORT; TYPE(C_PTR), VALUE :: h; INTEGER(C_INT), VALUE :: nElems, nSides, nBCSides
    INTEGER(C_INT) :: SideToElem(*), ElemToSide(*), BC(*)
    INTEGER(C_INT), VALUE :: nBCs; INTEGER(C_INT) :: BoundaryType(*)
    INTEGER(C_INT), VALUE :: nRefStates; REAL(C_DOUBLE) :: RefStatePrim(*)
    REAL(C_DOUBLE) :: Metrics_fTilde(*), Metrics_gTilde(*), Metrics_hTilde(*), sJ(*)
    REAL(C_DOUBLE) :: NormVec(*), TangVec1(*), TangVec2(*), SurfElem(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_set_mesh_mortar(h, nElems, nSides, nBCSides, SideToElem, ElemToSide, BC, nBCs, BoundaryType, &
                                             nRefStates, RefStatePrim, Metrics_fTilde, Metrics_gTilde, Metrics_hTilde, sJ, &
                                             NormVec, TangVec1, TangVec2, SurfElem, nMortars, MortarType, MortarInfo) &
                                             BIND(C,NAME='fg_set_mesh_mortar')
    IMPORT; TYPE(C_PTR), VALUE :: h; INTEGER(C_INT), VALUE :: nElems, nSides, nBCSides
    INTEGER(C_INT) :: SideToElem(*), ElemToSide(*), BC(*)
    INTEGER(C_INT), VALUE :: nBCs; INTEGER(C_INT) :: BoundaryType(*)
    INTEGER(C_INT), VALUE :: nRefStates; REAL(C_DOUBLE) :: RefStatePrim(*)
    REAL(C_DOUBLE) :: Metrics_fTilde(*), Metrics_gTilde(*), Metrics_hTilde(*), sJ(*)
    REAL(C_DOUBLE) :: NormVec(*), TangVec1(*), TangVec2(*), SurfElem(*)
    INTEGER(C_INT), VALUE :: nMortars; INTEGER(C_INT) :: MortarType(*), MortarInfo(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_set_face_metrics(h, Ja_Face, Ja_slave) BIND(C,NAME='fg_set_face_metrics')
    IMPORT; TYPE(C_PTR), VALUE :: h; REAL(C_DOUBLE) :: Ja_Face(*), Ja_slave(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_overintegrate_state(h) BIND(C,NAME='fg_overintegrate_state')
    IMPORT; TYPE(C_PTR), VALUE :: h
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_lserk_table(method, stages, A, b, c, cflAlpha, relativeDFL) BIND(C,NAME='fg_lserk_table')
    IMPORT; INTEGER(C_INT), VALUE :: method; INTEGER(C_INT) :: stages
    REAL(C_DOUBLE) :: A(*), b(*), c(*), cflAlpha(*), relativeDFL
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_get_config(h, cfg) BIND(C,NAME='fg_get_config')
    IMPORT; TYPE(C_PTR), VALUE :: h; TYPE(fg_config) :: cfg
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_hopr_sizes(path, sizes) BIND(C,NAME='fg_hopr_sizes')
    IMPORT; CHARACTER(KIND=C_CHAR) :: path(*); INTEGER(C_INT) :: sizes(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_hopr_read(path, NodeCoords, ElemNb, BoundaryType, BCNames, Mortars) BIND(C,NAME='fg_hopr_read')
    IMPORT; CHARACTER(KIND=C_CHAR) :: path(*); REAL(C_DOUBLE) :: NodeCoords(*); INTEGER(C_INT) :: ElemNb(*), BoundaryType(*)
    CHARACTER(KIND=C_CHAR), OPTIONAL :: BCNames(*); INTEGER(C_INT), OPTIONAL :: Mortars(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_write_state(h, path, projectName, meshFile, time) BIND(C,NAME='fg_write_state')
    IMPORT; TYPE(C_PTR), VALUE :: h; CHARACTER(KIND=C_CHAR) :: path(*), projectName(*), meshFile(*); REAL(C_DOUBLE), VALUE :: time
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_read_state(h, path, time) BIND(C,NAME='fg_read_state')
    IMPORT; TYPE(C_PTR), VALUE :: h; CHARACTER(KIND=C_CHAR) :: path(*); REAL(C_DOUBLE) :: time
  END FUNCTION
  TYPE(C_PTR) FUNCTION fg_io_last_error() BIND(C,NAME='fg_io_last_error')
    IMPORT
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_set_instance_mu0(h, nInst, mu0) BIND(C,NAME='fg_set_instance_mu0')
    IMPORT; TYPE(C_PTR), VALUE :: h; INTEGER(C_INT), VALUE :: nInst; REAL(C_DOUBLE) :: mu0(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_get_elem_xgp(h, Elem_xGP) BIND(C,NAME='fg_get_elem_xgp')
    IMPORT; TYPE(C_PTR), VALUE :: h; REAL(C_DOUBLE) :: Elem_xGP(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_get_sizes(h, sizes) BIND(C,NAME='fg_get_sizes')
    IMPORT; TYPE(C_PTR), VALUE :: h; INTEGER(C_INT) :: sizes(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_get_mesh_array(h, which, arr) BIND(C,NAME='fg_get_mesh_array')
    IMPORT; TYPE(C_PTR), VALUE :: h; INTEGER(C_INT), VALUE :: which; REAL(C_DOUBLE) :: arr(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_get_side_to_elem(h, SideToElem) BIND(C,NAME='fg_get_side_to_elem')
    IMPORT; TYPE(C_PTR), VALUE :: h; INTEGER(C_INT) :: SideToElem(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_set_state(h, U) BIND(C,NAME='fg_set_state')
    IMPORT; TYPE(C_PTR), VALUE :: h; REAL(C_DOUBLE) :: U(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_get_state(h, U) BIND(C,NAME='fg_get_state')
    IMPORT; TYPE(C_PTR), VALUE :: h; REAL(C_DOUBLE) :: U(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_state_device_ptr(h, dptr) BIND(C,NAME='fg_state_device_ptr')
    IMPORT; TYPE(C_PTR), VALUE :: h; TYPE(C_PTR) :: dptr
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_time_derivative(h, t, Ut) BIND(C,NAME='fg_time_derivative')
    IMPORT; TYPE(C_PTR), VALUE :: h; REAL(C_DOUBLE), VALUE :: t; REAL(C_DOUBLE), OPTIONAL :: Ut(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_calc_timestep(h, dt, errType) BIND(C,NAME='fg_calc_timestep')
    IMPORT; TYPE(C_PTR), VALUE :: h; REAL(C_DOUBLE) :: dt(*); INTEGER(C_INT) :: errType
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_get_dt_elem(h, dtConv, dtVisc) BIND(C,NAME='fg_get_dt_elem')
    IMPORT; TYPE(C_PTR), VALUE :: h; REAL(C_DOUBLE) :: dtConv(*), dtVisc(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_timestep_lserkw2(h, t, dt) BIND(C,NAME='fg_timestep_lserkw2')
    IMPORT; TYPE(C_PTR), VALUE :: h; REAL(C_DOUBLE) :: t; REAL(C_DOUBLE), VALUE :: dt
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_run(h, nSteps, t) BIND(C,NAME='fg_run')
    IMPORT; TYPE(C_PTR), VALUE :: h; INTEGER(C_INT), VALUE :: nSteps; REAL(C_DOUBLE), OPTIONAL :: t(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_run_to_host(h, nSteps, t, U) BIND(C,NAME='fg_run_to_host')
    IMPORT; TYPE(C_PTR), VALUE :: h; INTEGER(C_INT), VALUE :: nSteps; REAL(C_DOUBLE) :: t(*); REAL(C_DOUBLE) :: U(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_get_timedisc_state(h, nInst, state) BIND(C,NAME='fg_get_timedisc_state')
    IMPORT; TYPE(C_PTR), VALUE :: h; INTEGER(C_INT), VALUE :: nInst; TYPE(fg_timedisc_state) :: state(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_set_time(h, t) BIND(C,NAME='fg_set_time')
    IMPORT; TYPE(C_PTR), VALUE :: h; REAL(C_DOUBLE) :: t(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_get_gradients(h, gx, gy, gz) BIND(C,NAME='fg_get_gradients')
    IMPORT; TYPE(C_PTR), VALUE :: h; REAL(C_DOUBLE), OPTIONAL :: gx(*), gy(*), gz(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_get_stream(h, stream) BIND(C,NAME='fg_get_stream')
    IMPORT; TYPE(C_PTR), VALUE :: h; TYPE(C_PTR) :: stream
  END FUNCTION
  INTEGER(C_LONG_LONG) FUNCTION fg_launch_count(h) BIND(C,NAME='fg_launch_count')
    IMPORT; TYPE(C_PTR), VALUE :: h
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_debug_array(h, name, arr, count) BIND(C,NAME='fg_debug_array')
    IMPORT; TYPE(C_PTR), VALUE :: h; CHARACTER(KIND=C_CHAR) :: name(*); TYPE(C_PTR), VALUE :: arr; INTEGER(C_LONG_LONG) :: count
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_profile_enable(h, on) BIND(C,NAME='fg_profile_enable')
    IMPORT; TYPE(C_PTR), VALUE :: h; INTEGER(C_INT), VALUE :: on
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_profile_read(h, ms, counts) BIND(C,NAME='fg_profile_read')
    IMPORT; TYPE(C_PTR), VALUE :: h; REAL(C_DOUBLE) :: ms(*); INTEGER(C_LONG_LONG) :: counts(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_set_elem_mu_scale(h, scale) BIND(C,NAME='fg_set_elem_mu_scale')
    IMPORT; TYPE(C_PTR), VALUE :: h; REAL(C_DOUBLE), OPTIONAL :: scale(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_vjp_time_derivative(h, t, W, V, muScaleBar) BIND(C,NAME='fg_vjp_time_derivative')
    IMPORT; TYPE(C_PTR), VALUE :: h; REAL(C_DOUBLE), VALUE :: t; REAL(C_DOUBLE) :: W(*), V(*)
    REAL(C_DOUBLE), OPTIONAL :: muScaleBar(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_jvp_time_derivative(h, t, V, JV, fdOrder, epsMethod, scaleps) BIND(C,NAME='fg_jvp_time_derivative')
    IMPORT; TYPE(C_PTR), VALUE :: h; REAL(C_DOUBLE), VALUE :: t; REAL(C_DOUBLE) :: V(*), JV(*)
    INTEGER(C_INT), VALUE :: fdOrder, epsMethod; REAL(C_DOUBLE), VALUE :: scaleps
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_adjoint_forward(h, nSteps, dt, ckptEvery) BIND(C,NAME='fg_adjoint_forward')
    IMPORT; TYPE(C_PTR), VALUE :: h; INTEGER(C_INT), VALUE :: nSteps; REAL(C_DOUBLE), VALUE :: dt
    INTEGER(C_INT), VALUE :: ckptEvery
  END FUNCTION
  INTEGER(C_LONG_LONG) FUNCTION fg_adjoint_recomputed_steps(h) BIND(C,NAME='fg_adjoint_recomputed_steps')
    IMPORT; TYPE(C_PTR), VALUE :: h
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_adjoint_reverse(h, UbarT, Ubar0, muScaleBar, forceBar) BIND(C,NAME='fg_adjoint_reverse')
    IMPORT; TYPE(C_PTR), VALUE :: h; REAL(C_DOUBLE) :: UbarT(*)
    REAL(C_DOUBLE), OPTIONAL :: Ubar0(*), muScaleBar(*), forceBar(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_set_body_force_field(h, F) BIND(C,NAME='fg_set_body_force_field')
    IMPORT; TYPE(C_PTR), VALUE :: h; REAL(C_DOUBLE), OPTIONAL :: F(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_wall_shear(h, J, dJdU) BIND(C,NAME='fg_wall_shear')
    IMPORT; TYPE(C_PTR), VALUE :: h; REAL(C_DOUBLE) :: J; REAL(C_DOUBLE), OPTIONAL :: dJdU(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_autotune(h, reps, report) BIND(C,NAME='fg_autotune')
    IMPORT; TYPE(C_PTR), VALUE :: h; INTEGER(C_INT), VALUE :: reps; REAL(C_DOUBLE), OPTIONAL :: report(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_autotune_choice(h, choice) BIND(C,NAME='fg_autotune_choice')
    IMPORT; TYPE(C_PTR), VALUE :: h; INTEGER(C_INT) :: choice(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_set_launch_shapes(h, epbPrep, epbLift, epbVol, fluxBlock) BIND(C,NAME='fg_set_launch_shapes')
    IMPORT; TYPE(C_PTR), VALUE :: h; INTEGER(C_INT), VALUE :: epbPrep, epbLift, epbVol, fluxBlock
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_probe_fp64_pipe(rates) BIND(C,NAME='fg_probe_fp64_pipe')
    IMPORT; REAL(C_DOUBLE) :: rates(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_probe_fp64(tflops) BIND(C,NAME='fg_probe_fp64')
    IMPORT; REAL(C_DOUBLE) :: tflops
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_probe_fp64_tensor(rates) BIND(C,NAME='fg_probe_fp64_tensor')
    IMPORT; REAL(C_DOUBLE) :: rates(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_probe_fp64_lanes(ms) BIND(C,NAME='fg_probe_fp64_lanes')
    IMPORT; REAL(C_DOUBLE) :: ms(*)
  END FUNCTION
  INTEGER(C_INT) FUNCTION fg_time_derivative_noalloc(cfg, mesh, U, Ut, stream) BIND(C,NAME='fg_time_derivative_noalloc')
    IMPORT; TYPE(fg_config) :: cfg; TYPE(fg_device_mesh) :: mesh; TYPE(C_PTR), VALUE :: U, Ut, stream
  END FUNCTION
  ! C library: length of a NUL-terminated message
  INTEGER(C_SIZE_T) FUNCTION c_strlen(s) BIND(C,NAME='strlen')
    IMPORT; TYPE(C_PTR), VALUE :: s
  END FUNCTION
END INTERFACE

PUBLIC :: fg_config_default, fg_config_from_ini, fg_create, fg_destroy, fg_last_error, fg_build_mesh, fg_build_mesh_mortar
PUBLIC :: fg_set_mesh, fg_set_mesh_mortar, fg_set_face_metrics, fg_overintegrate_state, fg_lserk_table, fg_get_config
PUBLIC :: fg_hopr_sizes, fg_hopr_read, fg_write_state, fg_read_state, fg_io_last_error, fg_set_instance_mu0, fg_get_elem_xgp
PUBLIC :: fg_get_sizes, fg_get_mesh_array, fg_get_side_to_elem, fg_set_state, fg_get_state, fg_state_device_ptr
PUBLIC :: fg_time_derivative, fg_calc_timestep, fg_get_dt_elem, fg_timestep_lserkw2, fg_run, fg_run_to_host, fg_get_timedisc_state
PUBLIC :: fg_set_time
PUBLIC :: fg_get_gradients, fg_get_stream, fg_launch_count, fg_debug_array, fg_profile_enable, fg_profile_read
PUBLIC :: fg_set_elem_mu_scale, fg_vjp_time_derivative, fg_jvp_time_derivative, fg_adjoint_forward, fg_adjoint_recomputed_steps
PUBLIC :: fg_adjoint_reverse, fg_set_body_force_field, fg_wall_shear, fg_autotune, fg_autotune_choice, fg_set_launch_shapes
PUBLIC :: fg_probe_fp64_pipe, fg_probe_fp64, fg_probe_fp64_tensor, fg_probe_fp64_lanes, fg_time_derivative_noalloc

!----------------------------------------------------------------------------------------------------------------------------------
! Part 2: the FLEXI shim
!----------------------------------------------------------------------------------------------------------------------------------
TYPE(C_PTR)    :: gpu = C_NULL_PTR   !< the solver handle (one rank, one GPU)
LOGICAL,PUBLIC :: useGPU = .FALSE.   !< set by InitDG_GPU once the handle holds mesh and state

PUBLIC :: InitDG_GPU, DGTimeDerivative_GPU, TimeStepByLSERKW2_GPU, CalcTimeStep_GPU, TimeDiscSteps_GPU, TimeDiscStepsToHost_GPU
PUBLIC :: GetState_GPU
PUBLIC :: FinalizeDG_GPU, GPUErrorMessage

CONTAINS

!==================================================================================================================================
!> The library's message for the last failed call on the handle (empty when none)
!==================================================================================================================================
FUNCTION GPUErrorMessage() RESULT(msg)
CHARACTER(LEN=512)              :: msg
TYPE(C_PTR)                     :: p
CHARACTER(KIND=C_CHAR),POINTER  :: c(:)
INTEGER                         :: i, nChar
msg = ''
p = fg_last_error(gpu)
IF (.NOT.C_ASSOCIATED(p)) RETURN
nChar = INT(MIN(c_strlen(p), INT(LEN(msg), C_SIZE_T)))
CALL C_F_POINTER(p, c, [nChar])
DO i = 1, nChar
  msg(i:i) = c(i)
END DO
END FUNCTION GPUErrorMessage

!==================================================================================================================================
!> Abort (globals.f90:177) with the library's message when a call did not return FG_OK
!==================================================================================================================================
SUBROUTINE CheckGPU(rc, what)
USE MOD_Globals, ONLY: Abort
INTEGER(C_INT),INTENT(IN)   :: rc
CHARACTER(LEN=*),INTENT(IN) :: what
IF (rc.EQ.FG_OK) RETURN
CALL Abort(__STAMP__, 'GPU '//what//': '//TRIM(GPUErrorMessage()), IntInfo=INT(rc))
END SUBROUTINE CheckGPU

!==================================================================================================================================
!> Called at the end of InitFlexi (flexilib.f90): the ini keys of this path and the processed mesh arrays of MOD_Mesh_Vars
!> (FLEXI keeps its own InitMesh), then the initial state.
!==================================================================================================================================
SUBROUTINE InitDG_GPU()
USE MOD_PreProc,              ONLY: PP_N
USE MOD_Mesh_Vars,            ONLY: nElems, nSides, nBCSides, nBCs, SideToElem, ElemToSide, BC, BoundaryType
USE MOD_Mesh_Vars,            ONLY: Metrics_fTilde, Metrics_gTilde, Metrics_hTilde, sJ, NormVec, TangVec1, TangVec2, SurfElem
USE MOD_Mesh_Vars,            ONLY: nMortarInnerSides, MortarType, MortarInfo
#if PP_EntropyVars == 1
USE MOD_Mesh_Vars,            ONLY: Ja_Face, Ja_slave
#endif
USE MOD_Equation_Vars,        ONLY: RefStatePrim, nRefState, IniExactFunc
USE MOD_Exactfunc_Vars,       ONLY: AdvVel, IniFrequency, IniAmplitude
USE MOD_EOS_Vars,             ONLY: Kappa, R, Pr, mu0
USE MOD_Lifting_Vars,         ONLY: etaBR2, etaBR2_wall, doWeakLifting, doConservativeLifting
USE MOD_Overintegration_Vars, ONLY: OverintegrationType, NUnder
USE MOD_TimeDisc_Vars,        ONLY: CFLScale_Readin, DFLScale_Readin, TimeDiscMethod, tEnd, dt_dynmin, dt_kill
USE MOD_TimeDisc_Vars,        ONLY: nCalcTimeStepMax, maxIter
USE MOD_Analyze_Vars,         ONLY: analyze_dt
USE MOD_DG_Vars,              ONLY: U
USE MOD_ReadInTools,          ONLY: GETINTFROMSTR
TYPE(fg_config) :: cfg
CALL CheckGPU(fg_config_default(cfg), 'config')
cfg%N         = PP_N
cfg%NodeType  = PP_NodeType
cfg%Lifting   = PP_Lifting
cfg%Riemann   = GETINTFROMSTR('Riemann')
cfg%RiemannBC = GETINTFROMSTR('RiemannBC')
#ifdef SPLIT_DG
cfg%SplitDG   = GETINTFROMSTR('SplitDG')
#else
cfg%SplitDG   = -1
#endif
cfg%doWeakLifting         = MERGE(1, 0, doWeakLifting)
cfg%doConservativeLifting = MERGE(1, 0, doConservativeLifting)
cfg%etaBR2      = etaBR2
cfg%etaBR2_wall = etaBR2_wall
cfg%kappa = Kappa
cfg%R     = R
cfg%Pr    = Pr
cfg%mu0   = mu0
cfg%CFLScale = CFLScale_Readin(0)   ! the unscaled ini values: the library applies FillCFL_DFL itself
cfg%DFLScale = DFLScale_Readin(0)
SELECT CASE (TRIM(TimeDiscMethod))  ! the low-storage schemes of TimeStepByLSERKW2 (timedisc_vars.f90:123-133)
CASE('carpenterrk4-5');  cfg%TimeDiscMethod = 0
CASE('standardrk3-3');   cfg%TimeDiscMethod = 1
CASE('niegemannrk4-14'); cfg%TimeDiscMethod = 2
CASE('toulorgerk4-8c');  cfg%TimeDiscMethod = 3
CASE('toulorgerk3-7c');  cfg%TimeDiscMethod = 4
CASE('toulorgerk4-8f');  cfg%TimeDiscMethod = 5
CASE DEFAULT;            cfg%TimeDiscMethod = -1  ! fg_create refuses other schemes: FLEXI keeps its CPU path
END SELECT
cfg%OverintegrationType = OverintegrationType
cfg%NUnder              = NUnder
cfg%IniExactFunc        = IniExactFunc         ! CalcSource of exact function 4 (exactfunc.f90)
cfg%AdvVel              = AdvVel
cfg%IniFrequency        = IniFrequency
cfg%IniAmplitude        = IniAmplitude
cfg%TEnd                = tEnd                 ! UpdateTimeStep control of TimeDiscSteps_GPU
cfg%Analyze_dt          = analyze_dt
cfg%dtmin               = dt_dynmin
cfg%dtkill              = dt_kill
cfg%nCalcTimeStepMax    = nCalcTimeStepMax
cfg%maxIter             = INT(MIN(maxIter, INT(HUGE(cfg%maxIter), KIND(maxIter))), C_INT)
IF (fg_create(cfg, gpu).NE.FG_OK) RETURN      ! unsupported configuration: FLEXI keeps its CPU path
IF (nMortarInnerSides.GT.0) THEN  ! one rank: every mortar is an inner mortar
  CALL CheckGPU(fg_set_mesh_mortar(gpu, nElems, nSides, nBCSides, SideToElem, ElemToSide, BC, nBCs, BoundaryType, nRefState, &
                                   RefStatePrim, Metrics_fTilde(:,:,:,:,:,0), Metrics_gTilde(:,:,:,:,:,0),                   &
                                   Metrics_hTilde(:,:,:,:,:,0), sJ(:,:,:,:,0), NormVec(:,:,:,0,:), TangVec1(:,:,:,0,:),      &
                                   TangVec2(:,:,:,0,:), SurfElem(:,:,0,:), nMortarInnerSides, MortarType, MortarInfo), 'mesh')
ELSE
  CALL CheckGPU(fg_set_mesh(gpu, nElems, nSides, nBCSides, SideToElem, ElemToSide, BC, nBCs, BoundaryType, nRefState,        &
                            RefStatePrim, Metrics_fTilde(:,:,:,:,:,0), Metrics_gTilde(:,:,:,:,:,0), Metrics_hTilde(:,:,:,:,:,0), &
                            sJ(:,:,:,:,0), NormVec(:,:,:,0,:), TangVec1(:,:,:,0,:), TangVec2(:,:,:,0,:), SurfElem(:,:,0,:)),  &
                'mesh')
END IF
#if PP_EntropyVars == 1
CALL CheckGPU(fg_set_face_metrics(gpu, Ja_Face, Ja_slave), 'face metrics')  ! split form on Gauss nodes
#endif
CALL CheckGPU(fg_set_state(gpu, U), 'state')
useGPU = .TRUE.
END SUBROUTINE InitDG_GPU

!==================================================================================================================================
!> Replaces the body of DGTimeDerivative_weakForm (dg.f90:221): Ut of the current U
!==================================================================================================================================
SUBROUTINE DGTimeDerivative_GPU(t)
USE MOD_DG_Vars, ONLY: U, Ut
REAL,INTENT(IN) :: t
CALL CheckGPU(fg_set_state(gpu, U), 'state')
CALL CheckGPU(fg_time_derivative(gpu, t, Ut), 'DGTimeDerivative_weakForm')
END SUBROUTINE DGTimeDerivative_GPU

!==================================================================================================================================
!> TimeStep => TimeStepByLSERKW2_GPU (timestep.f90:37-39,64): U stays on the device between steps
!==================================================================================================================================
SUBROUTINE TimeStepByLSERKW2_GPU(t)
USE MOD_TimeDisc_Vars, ONLY: dt
REAL,INTENT(INOUT) :: t
REAL(C_DOUBLE)     :: tt
tt = t
CALL CheckGPU(fg_timestep_lserkw2(gpu, tt, dt), 'TimeStepByLSERKW2')
END SUBROUTINE TimeStepByLSERKW2_GPU

!==================================================================================================================================
!> CALCTIMESTEP (calctimestep.f90:89) on the device state, called by EvalTimeStep in place of CalcTimeStep
!==================================================================================================================================
FUNCTION CalcTimeStep_GPU(errType) RESULT(dtOut)
INTEGER,INTENT(OUT) :: errType
REAL                :: dtOut
REAL(C_DOUBLE)      :: dtv(1)
INTEGER(C_INT)      :: e
CALL CheckGPU(fg_calc_timestep(gpu, dtv, e), 'CALCTIMESTEP')
dtOut   = dtv(1)
errType = e
END FUNCTION CalcTimeStep_GPU

!==================================================================================================================================
!> Up to nSteps passes of the TimeDisc loop body (timedisc.f90:190-212) on the device without host synchronisation, with
!> UpdateTimeStep's clipping to the next analysis time and to tEnd: returns after the step that reaches an analysis time
!> (doAnalyze) or tEnd / maxIter (doFinalize), with t, dt and iter updated; the caller then runs AnalyzeTimeStep's analysis
!> on the state copied back by GetState_GPU.
!==================================================================================================================================
SUBROUTINE TimeDiscSteps_GPU(nSteps, doAnalyze, doFinalize)
USE MOD_TimeDisc_Vars, ONLY: t, dt, iter
INTEGER,INTENT(IN)      :: nSteps
LOGICAL,INTENT(OUT)     :: doAnalyze, doFinalize
TYPE(fg_timedisc_state) :: st(1)
CALL CheckGPU(fg_run(gpu, INT(nSteps, C_INT)), 'TimeDisc')
CALL CheckGPU(fg_get_timedisc_state(gpu, 1_C_INT, st), 'TimeDisc state')
t          = st(1)%t
dt         = st(1)%dt
iter       = st(1)%iter
doAnalyze  = st(1)%atAnalyze.NE.0
doFinalize = st(1)%finished.NE.0
END SUBROUTINE TimeDiscSteps_GPU

!==================================================================================================================================
!> TimeDiscSteps_GPU and GetState_GPU in one call: the copy of the state into U overlaps the last stage of the last step
!==================================================================================================================================
SUBROUTINE TimeDiscStepsToHost_GPU(nSteps, doAnalyze, doFinalize)
USE MOD_DG_Vars,       ONLY: U
USE MOD_TimeDisc_Vars, ONLY: t, dt, iter
INTEGER,INTENT(IN)      :: nSteps
LOGICAL,INTENT(OUT)     :: doAnalyze, doFinalize
TYPE(fg_timedisc_state) :: st(1)
REAL(C_DOUBLE)          :: tInst(1)
CALL CheckGPU(fg_run_to_host(gpu, INT(nSteps, C_INT), tInst, U), 'TimeDisc')
CALL CheckGPU(fg_get_timedisc_state(gpu, 1_C_INT, st), 'TimeDisc state')
t          = st(1)%t
dt         = st(1)%dt
iter       = st(1)%iter
doAnalyze  = st(1)%atAnalyze.NE.0
doFinalize = st(1)%finished.NE.0
END SUBROUTINE TimeDiscStepsToHost_GPU

!==================================================================================================================================
!> Copies the device state into U (before WriteState / Analyze) and, optionally, the lifted gradients
!==================================================================================================================================
SUBROUTINE GetState_GPU()
USE MOD_DG_Vars, ONLY: U
CALL CheckGPU(fg_get_state(gpu, U), 'state')
END SUBROUTINE GetState_GPU

!==================================================================================================================================
!> Frees the handle (FinalizeFlexi)
!==================================================================================================================================
SUBROUTINE FinalizeDG_GPU()
INTEGER(C_INT) :: rc
IF (C_ASSOCIATED(gpu)) rc = fg_destroy(gpu)
gpu    = C_NULL_PTR
useGPU = .FALSE.
END SUBROUTINE FinalizeDG_GPU

END MODULE MOD_DG_GPU
