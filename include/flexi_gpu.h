/*
 * flexi_gpu.h -- C ABI of libflexigpu.so, a GB300 (sm_103a) implementation of FLEXI's DGSEM
 * right-hand side and low-storage Runge-Kutta stepper for the compressible Navier-Stokes equations.
 *
 * FLEXI (v25.10) has no C interface for this path; its entry points are Fortran module procedures
 * operating on module arrays. Each function below names the reference procedure it replaces
 * (path:line inside the FLEXI source tree). Arrays crossing this interface use FLEXI's Fortran
 * layouts, e.g. U(1:5,0:N,0:N,0:N,1:nElems), and are host pointers borrowed for the duration of the
 * call unless stated otherwise. The library copies them into its own device-resident layouts.
 *
 * Every function returns 0 on success or a positive FG_ERR_* code; fg_last_error() gives a message.
 * Device-side failures (NaN density, non-finite time step) are recorded in a sticky error word that
 * the host reads after each step; nothing traps or aborts.
 */
#ifndef FLEXI_GPU_H
#define FLEXI_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define FG_OK 0
#define FG_ERR_CONFIG 1    /* invalid or unsupported configuration */
#define FG_ERR_MESH 2      /* mesh could not be processed */
#define FG_ERR_CUDA 3      /* CUDA runtime error */
#define FG_ERR_STATE 4     /* call order violated (e.g. no mesh yet) */
#define FG_ERR_NAN 5       /* NaN density found (calctimestep.f90 errType 1) */
#define FG_ERR_DT 6        /* non-finite time step (errType 2/3) */
#define FG_ERR_DTKILL 7    /* time step below dtkill (timedisc_func.f90:EvalTimeStep, "Critical Kill timestep reached") */

/* Riemann solver ids: the integer values of riemann.f90:44-58 (CH, IR and AVERAGE need the split form; the other
 * solvers run with both forms, the HLL family with the split form as an extension of the reference) */
#define FG_RIEMANN_SAME (-1)
#define FG_RIEMANN_AVERAGE 0
#define FG_RIEMANN_LF 1
#define FG_RIEMANN_HLLC 2
#define FG_RIEMANN_ROE 3
#define FG_RIEMANN_HLL 4
#define FG_RIEMANN_HLLE 5
#define FG_RIEMANN_HLLEM 6
#define FG_RIEMANN_CH 7
#define FG_RIEMANN_IR 8
#define FG_RIEMANN_ROEL2 32
#define FG_RIEMANN_ROEENTROPYFIX 33
#define FG_RIEMANN_ROEENTROPYGSHOCKFIX 34
/* SplitDG ids: splitflux.f90:63-69; -1 selects the weak (non-split) form */
#define FG_SPLIT_NONE (-1)
#define FG_SPLIT_SD 0
#define FG_SPLIT_MO 1
#define FG_SPLIT_DU 2
#define FG_SPLIT_KG 3
#define FG_SPLIT_PI 4
#define FG_SPLIT_CH 5
#define FG_SPLIT_IR 6
#define FG_NODE_GAUSS 1
#define FG_NODE_GAUSS_LOBATTO 2

/* Parameters of parameter_flexi.ini for this path (same meaning and defaults as the reference):
 *   N (interpolation.f90:59), NodeType (CMake FLEXI_NODETYPE), Riemann/RiemannBC (riemann.f90:91-115),
 *   Lifting 1=BR1 / 2=BR2 (CMake FLEXI_LIFTING), doWeakLifting, doConservativeLifting, etaBR2,
 *   etaBR2_wall (lifting.f90:61-83), SplitDG (splitflux.f90:77), kappa, R, Pr, mu0 (eos.f90:84-90),
 *   CFLScale, DFLScale (timedisc_func.f90:463-527), TimeDiscMethod (0 = CarpenterRK4-5, 1..5 the other low-storage schemes),
 *   the channel body force of testcase/channel (doTCSource, dpdx), and the time-loop control of TimeDisc
 *   (TEnd, Analyze_dt, dtmin, dtkill, nCalcTimeStepMax, maxIter: timedisc_func.f90:51-61, analyze.f90:49-52). */
typedef struct fg_config {
  int N;
  int NodeType;
  int Riemann;
  int RiemannBC;
  int Lifting;
  int doWeakLifting;
  int doConservativeLifting;
  int SplitDG;
  double etaBR2;
  double etaBR2_wall;
  double kappa;
  double R;
  double Pr;
  double mu0;
  double CFLScale;
  double DFLScale;
  int doTCSource;
  double dpdx;
  int TimeDiscMethod;       /* timedisc_vars.f90 low-storage schemes (TimeStepByLSERKW2): 0 carpenterrk4-5, 1 standardrk3-3,
                               2 niegemannrk4-14, 3 toulorgerk4-8c, 4 toulorgerk3-7c, 5 toulorgerk4-8f */
  int OverintegrationType;  /* overintegration.f90: 0 none, 1 cut-off filter of J u_t, 2 conservative cut-off */
  int NUnder;               /* filter degree of OverintegrationType 1/2 (-1: N) */
  int IniExactFunc;         /* exactfunc.f90: 4 (oblique sine wave) adds its source, CalcSource CASE(4); others: no source */
  double AdvVel[3];         /* AdvVel of exact function 4 (its wave speed is 2 pi AdvVel(1)) */
  double IniFrequency;      /* IniFrequency (default 1) */
  double IniAmplitude;      /* IniAmplitude (default 0.1) */
  /* time-loop control of fg_run (timedisc_func.f90:UpdateTimeStep/EvalTimeStep, timedisc.f90:190-212) */
  double TEnd;              /* end time: the step that reaches it is clipped to it, later steps do not advance (default +inf: none) */
  double Analyze_dt;        /* analysis interval: steps are clipped to the analysis times t0 + k Analyze_dt (<= 0: TEnd, analyze.f90:127) */
  double dtmin;             /* time steps below dtmin are raised to it (default -1: off) */
  double dtkill;            /* a time step below dtkill stops the run with FG_ERR_DTKILL (default -1: off) */
  int nCalcTimeStepMax;     /* NCalcTimeStepMax: CALCTIMESTEP at least every nCalcTimeStepMax steps, fewer when dt varies (default 1) */
  int maxIter;              /* maxIter: an instance stops after this many steps (default -1: no limit) */
  double RiemannPhiFactor;  /* RiemannPhiFactor of RoeEntropyGShockFix (riemann.f90:131, default 5) */
} fg_config;

typedef struct fg_handle fg_handle;

/* Defaults of the reference (Riemann=RoeEntropyFix, SplitDG=PI, Lifting=BR1, etaBR2=2, kappa=1.4,
 * R=287.058, Pr=0.72, mu0=0, CFLScale=DFLScale=0.9, CarpenterRK4-5, no overintegration, Analyze_dt=0,
 * dtmin=dtkill=-1, nCalcTimeStepMax=1, maxIter=-1); TEnd (mandatory in the reference) defaults to +inf. */
int fg_config_default(fg_config* cfg);

/* Parses the keys above from parameter_flexi.ini text (readintools.f90:read_options syntax:
 * "key = value", "!" comments, case-insensitive keys, string values for Riemann/SplitDG/NodeType/
 * TimeDiscMethod/OverintegrationType). Unknown keys are ignored. */
int fg_config_from_ini(const char* ini_text, fg_config* cfg);

/* Creates a solver on the current CUDA device. Replaces InitDG/InitLifting/InitTimeDisc
 * (dg.f90:InitDG, lifting.f90:InitLifting, timedisc_func.f90:InitTimeDisc). */
int fg_create(const fg_config* cfg, fg_handle** out);
int fg_destroy(fg_handle* h);
const char* fg_last_error(const fg_handle* h);

/* Mesh from raw element data -- what InitMesh (mesh.f90:82) builds from a HOPR mesh file:
 * NodeCoords(3,0:NGeo,0:NGeo,0:NGeo,nElems) on equidistant points (mesh_readin.f90:ReadMesh),
 * ElemNb(3,6,nElems) = (neighbour element 1-based or 0, neighbour local side, BC index) per local side
 * in FLEXI's local side numbering (flexi.h:90-95), BoundaryType(2,nBCs) = (type, state),
 * RefStatePrim(6,nRefStates). ElemInst(nElems) (nullable) assigns elements to independent ensemble
 * instances (0-based). Sides, orientation flips and curl-form metrics are computed here
 * (prepare_mesh.f90, mappings.f90, metrics.f90:CalcMetrics/CalcSurfMetrics). */
int fg_build_mesh(fg_handle* h, int nElems, int NGeo, const double* NodeCoords, const int* ElemNb, int nBCs, const int* BoundaryType,
                  int nRefStates, const double* RefStatePrim, const int* ElemInst);

/* fg_build_mesh for meshes with mortar interfaces (non-conforming 1->4 / 1->2 element faces): ElemNb holds
 * -1 for every big and small mortar side, and Mortars(15,nMortars) = (big element 1-based, its local side,
 * MortarType 1: 1->4, 2: 1->2 in eta, 3: 1->2 in xi, then per small side: element, local side, 0) as
 * fg_hopr_read returns it -- the content of mesh_readin.f90:ReadMesh's MortarType/MortarInfo
 * (mesh_vars.f90:122-126), with the small-side metrics of mortar_metrics.f90:Mortar_CalcSurfMetrics and
 * the operators of mortar.f90:InitMortar. */
int fg_build_mesh_mortar(fg_handle* h, int nElems, int NGeo, const double* NodeCoords, const int* ElemNb, int nBCs, const int* BoundaryType,
                         int nRefStates, const double* RefStatePrim, const int* ElemInst, int nMortars, const int* Mortars);

/* Drop-in mesh: the arrays of MOD_Mesh_Vars (mesh_vars.f90:34-160) after FLEXI's own InitMesh,
 * SideToElem(5,nSides), ElemToSide(2,6,nElems), BC(nBCSides), Metrics_fTilde/gTilde/hTilde
 * (3,0:N,0:N,0:N,nElems), sJ(0:N,0:N,0:N,nElems), NormVec/TangVec1/TangVec2(3,0:N,0:N,nSides),
 * SurfElem(0:N,0:N,nSides). Single rank: no MPI or mortar sides. */
int fg_set_mesh(fg_handle* h, int nElems, int nSides, int nBCSides, const int* SideToElem, const int* ElemToSide, const int* BC, int nBCs,
                const int* BoundaryType, int nRefStates, const double* RefStatePrim, const double* Metrics_fTilde,
                const double* Metrics_gTilde, const double* Metrics_hTilde, const double* sJ, const double* NormVec,
                const double* TangVec1, const double* TangVec2, const double* SurfElem);

/* fg_set_mesh for meshes with mortar interfaces: also MortarType(2,nSides) and MortarInfo(2,4,nMortars)
 * (mesh_vars.f90:158-159, nMortars = nMortarInnerSides; single rank, no MPI mortars). The small sides'
 * metrics are FLEXI's own (mortar_metrics.f90). The library renumbers the sides (conforming, then small,
 * then big: fg_get_side_to_elem reports its order); fg_set_face_metrics still takes FLEXI's numbering. */
int fg_set_mesh_mortar(fg_handle* h, int nElems, int nSides, int nBCSides, const int* SideToElem, const int* ElemToSide, const int* BC,
                       int nBCs, const int* BoundaryType, int nRefStates, const double* RefStatePrim, const double* Metrics_fTilde,
                       const double* Metrics_gTilde, const double* Metrics_hTilde, const double* sJ, const double* NormVec,
                       const double* TangVec1, const double* TangVec2, const double* SurfElem, int nMortars, const int* MortarType,
                       const int* MortarInfo);

/* Face metrics of the split form on Gauss nodes, FLEXI's Ja_Face(3,3,0:N,0:N,nSides) and
 * Ja_slave(3,3,0:N,0:N,nSides) (MOD_Mesh_Vars, filled by metrics.f90:CalcSurfMetrics; used by
 * surfint.t90:90-140). Optional after fg_set_mesh, which otherwise evaluates the normal-direction volume
 * metrics at the faces (identical up to round-off). Only row NormalDir of each side is read. */
int fg_set_face_metrics(fg_handle* h, const double* Ja_Face, const double* Ja_slave);

/* Overintegration of the state before the first time step (timedisc.f90:115-123; InitTimeDisc/TimeDisc do
 * it once after the initial condition or restart): OverintegrationType 1 filters U with the modal cut-off,
 * 2 applies the conservative cut-off to J U. No-op without overintegration. */
int fg_overintegrate_state(fg_handle* h);

/* The coefficients of low-storage scheme `method` (TimeDiscMethod code, timedisc_vars.f90:137-457): stage count,
 * RKA(2:s), RKb(1:s), RKc(2:s) at 1-based indices of 21-element arrays, CFLScaleAlpha(1:15) for Gauss then
 * Gauss-Lobatto nodes (30 values) and RelativeDFL; any output may be NULL but `stages`. */
int fg_lserk_table(int method, int* stages, double* A, double* b, double* c, double* cflAlpha, double* relativeDFL);

/* The configuration the handle was created with. */
int fg_get_config(const fg_handle* h, fg_config* out);

/* HOPR mesh files (the file part of mesh_readin.f90:ReadMesh/ReadBCs, datasets ElemInfo, SideInfo,
 * NodeCoords, BCType, BCNames, attribute Ngeo), read without the HDF5 library (contiguous datasets of the
 * classic file format, as HOPR writes them). fg_hopr_sizes: out[0]=nElems, out[1]=NGeo, out[2]=nBCs,
 * out[3]=nMortars. fg_hopr_read fills the inputs of fg_build_mesh: NodeCoords(3,0:NGeo,0:NGeo,0:NGeo,nElems),
 * ElemNb(3,6,nElems) (neighbour element, its local side, BC index; BC sides of types other than 0/1/100
 * are boundaries, mesh_readin.f90:398-456; -1 for the big and small sides of a mortar),
 * BoundaryType(2,nBCs) = (BCType(1), BCType(3)), BCNames (nBCs x 256 chars, NUL-terminated; may be NULL)
 * and Mortars(15,nMortars) (big element, its local side, mortar type 1: 1->4, 2: 1->2 in eta, 3: 1->2 in
 * xi, then per small side: small element, its local side, 0; may be NULL without mortars). Hexahedra only.
 * Errors in fg_io_last_error(). */
int fg_hopr_sizes(const char* path, int* out);
int fg_hopr_read(const char* path, double* NodeCoords, int* ElemNb, int* BoundaryType, char* BCNames, int* Mortars);

/* FLEXI state files (hdf5_output.f90:WriteState): dataset DG_Solution(1:5,0:N,0:N,0:N,nElems) and the
 * header attributes (VarNames, Program, File_Type, Project_Name, File_Version, N, Dimension, Time,
 * MeshFile, NextFile, NodeType, NComputation, TIME). fg_read_state loads DG_Solution of a file with the
 * same N, node type and element count (the restart of restart.f90 without interpolation) and returns its
 * Time. Errors in fg_io_last_error(). */
int fg_write_state(fg_handle* h, const char* path, const char* projectName, const char* meshFile, double time);
int fg_read_state(fg_handle* h, const char* path, double* time);
const char* fg_io_last_error(void);

/* Per-instance viscosity (ensembles); default: cfg.mu0 for every instance. */
int fg_set_instance_mu0(fg_handle* h, int nInst, const double* mu0);

/* Solution coordinates Elem_xGP(3,0:N,0:N,0:N,nElems) (metrics.f90:BuildCoords), fg_build_mesh only. */
int fg_get_elem_xgp(fg_handle* h, double* Elem_xGP);
/* Sizes: out[0]=nElems, out[1]=nSides, out[2]=nBCSides, out[3]=N, out[4]=nInstances. */
int fg_get_sizes(const fg_handle* h, int* out);
/* Processed metrics in FLEXI layouts, for comparison with FLEXI's own arrays:
 * which 0..2 = Metrics_f/g/hTilde, 3 = sJ, 4..6 = NormVec/TangVec1/TangVec2 of the master sides,
 * 7 = SurfElem (side order of this library, see fg_get_side_to_elem). */
int fg_get_mesh_array(fg_handle* h, int which, double* out);
/* SideToElem(5,nSides) of this library's side numbering (FLEXI conventions, 1-based). */
int fg_get_side_to_elem(fg_handle* h, int* out);

/* Solution U(1:5,0:N,0:N,0:N,1:nElems), Fortran layout. */
int fg_set_state(fg_handle* h, const double* U);
int fg_get_state(fg_handle* h, double* U);
/* Device pointer of the state in this library's layout [elem][var][k][j][i] (zero-copy access). */
int fg_state_device_ptr(fg_handle* h, double** dptr);

/* DGTimeDerivative_weakForm(t) (dg.f90:221): Ut(1:5,0:N,0:N,0:N,1:nElems) of the current state.
 * Ut may be NULL (result stays on the device). */
int fg_time_derivative(fg_handle* h, double t, double* Ut);

/* CALCTIMESTEP (calctimestep.f90:89): dt = min over elements of the convective and viscous limits,
 * per instance; dt[0] is instance 0. errType as in the reference (0 ok, 1 NaN density, 2/3 NaN dt). */
int fg_calc_timestep(fg_handle* h, double* dt, int* errType);

/* Per-element time-step limits of the last CALCTIMESTEP (calctimestep.f90:dtElem): convective limit
 * CFL*2/sum(lambda_conv) and viscous limit DFL*4/sum(lambda_visc) (+inf when mu0 = 0), nElems each. */
int fg_get_dt_elem(fg_handle* h, double* dtConv, double* dtVisc);

/* TimeStepByLSERKW2 (timestep.f90:82) with the low-storage scheme of cfg.TimeDiscMethod (timedisc_vars.f90:137-457):
 * advances the state by dt (all instances use the same dt here); t is advanced by dt. Includes CalcForcing
 * (testcase/channel/testcase.f90:262) when the channel body force is active. */
int fg_timestep_lserkw2(fg_handle* h, double* t, double dt);

/* TimeDisc loop body (timedisc.f90:190-212) for nSteps steps without host synchronisation:
 * UpdateTimeStep (timedisc_func.f90:215-268, per instance, on the device: CALCTIMESTEP, dtmin/dtkill of
 * EvalTimeStep :433-454, clipping to the next analysis time and to TEnd with the dt/100 stretch, the
 * nCalcTimeStepMax reuse of dt), CalcForcing, TimeStepByLSERKW2; the step sequence is captured once into a
 * CUDA graph and replayed. An instance whose step ends on an analysis time (doAnalyze) holds there for the
 * rest of the call and continues on the next call; one that reached TEnd or maxIter (doFinalize) no longer
 * advances (fg_set_time starts a new run); fg_get_timedisc_state reports which. A time step below dtkill stops the
 * instance that found it at its state then, the other instances after at most one more step, and returns FG_ERR_DTKILL. t[inst] (nullable) receives the
 * per-instance times, which start at 0 on the first call and continue on later calls. */
int fg_run(fg_handle* h, int nSteps, double* t);

/* fg_run followed by fg_get_state: nSteps steps of the TimeDisc loop, then U(t_end) into the host array U in the
 * Fortran layout (the reference's state after the loop, e.g. for WriteStateToHDF5 at an analysis time). The copy
 * overlaps the last stage: its volume kernel, which writes the final state, runs over element chunks, and each
 * chunk is copied to U while the later ones compute. Results are bitwise those of fg_run + fg_get_state; U is
 * written only up to the return (pinned host memory gives the full copy rate). */
int fg_run_to_host(fg_handle* h, int nSteps, double* t, double* U);

/* Per-instance state of the time loop (the reference's t, dt, dt_Min(DT_MIN), iter, doAnalyze, doFinalize,
 * nDtLimited of timedisc_vars.f90). */
typedef struct fg_timedisc_state {
  double t;          /* time */
  double dt;         /* time step of the last step */
  double dtMin;      /* dt_Min(DT_MIN): the last CALCTIMESTEP time step, after dtmin */
  long long iter;    /* steps since the handle's creation or the last fg_set_time */
  int atAnalyze;     /* the last step ended on an analysis time (the next fg_run continues) */
  int finished;      /* TEnd or maxIter reached (doFinalize) */
  int nDtLimited;    /* steps whose time step was raised to dtmin */
} fg_timedisc_state;
int fg_get_timedisc_state(fg_handle* h, int nInst, fg_timedisc_state* out);

/* Sets the device-side time of every instance (t[nInst]), the time fg_run and fg_adjoint_forward start from
 * (the restart time of a FLEXI run), and starts the time loop afresh there (InitTimeStep, timedisc.f90:105-112:
 * next analysis time min(t + Analyze_dt, TEnd), step counter 0, no held or finished instance). */
int fg_set_time(fg_handle* h, const double* t);

/* Lifted gradients of the last right-hand side, gradUx/gradUy/gradUz(4,0:N,0:N,0:N,nElems) of the
 * lifting variables (v1,v2,v3,T) (lifting_vars.f90, PP_OPTLIFT layout). */
int fg_get_gradients(fg_handle* h, double* gx, double* gy, double* gz);

/* CUDA stream the handle launches on (cudaStream_t as void*). */
int fg_get_stream(fg_handle* h, void** stream);

/* Number of kernel launches issued by the last fg_run / fg_timestep_lserkw2 / fg_time_derivative call. */
long long fg_launch_count(const fg_handle* h);

/* Copies one of the handle's device arrays to host memory for inspection, in the device layout:
 * "U","Ut","prim","grad","metr","sJ","metAdv","metVisc","mu0","dt","dtElem","geo","bcTwall" (double), "elemInst",
 * "elemSide","sideElem","bcType" (int). *count receives the number of elements; out may be NULL to query it. */
int fg_debug_array(fg_handle* h, const char* name, void* out, long long* count);

/* Per-kernel CUDA-event timing of later launches on the handle's stream; while enabled, fg_run issues
 * the kernels directly instead of replaying the captured graph. fg_profile_read returns, per kernel
 * class (0 prep, 1 lift, 2 flux, 3 volume+update, 4 time step, 5 other), the summed milliseconds and
 * the launch counts since the previous read, and resets them (class 5 includes the mortar kernels). */
int fg_profile_enable(fg_handle* h, int on);
int fg_profile_read(fg_handle* h, double* ms, long long* counts);

/* ---- Differentiation ---------------------------------------------------------------------------------
 * Per-element viscosity multiplier: element e uses mu0 (of its instance) x scale[e] in its volume viscous
 * flux, its own half of the viscous side fluxes and its viscous time-step limit; NULL resets all to 1.
 * No counterpart in the reference (the parameter of a gradient study). */
int fg_set_elem_mu_scale(fg_handle* h, const double* scale);

/* Adjoint of DGTimeDerivative_weakForm (dg.f90:221) at the current state: V = (dUt/dU)^T W, with W and V
 * in the layout of U (host arrays), and optionally muScaleBar[nElems] = d<W, Ut>/d(scale). The transposed
 * Jacobian is that of the discrete operator the GPU evaluates (the reference's implicit solver only forms
 * J V by finite differences, implicit.f90:MatrixVector). t is unused (the exact-function source does not
 * depend on U; the LSERK adjoint recomputes its steps at the forward's stage times). The bulk velocity of a
 * channel body force is held fixed.
 * Supported: weak form and every split form (SD, PI, MO, DU, KG, CH, IR) on Gauss and Gauss-Lobatto nodes (on Gauss nodes
 * with the transposed entropy-variable prolongation and split-Gauss surface term), N <= 7, every Riemann solver (LF, HLLC,
 * Roe, RoeEntropyFix, RoeL2, RoeEntropyGShockFix, HLL, HLLE, HLLEM; with the split form the flux average, CH and IR),
 * strong BR1/BR2 lifting, both overintegration types (the transposed filter), walls 3/4, mortar interfaces
 * (transposed U_Mortar and Flux_Mortar, fillmortar.t90). */
int fg_vjp_time_derivative(fg_handle* h, double t, const double* W, double* V, double* muScaleBar);

/* J V of DGTimeDerivative_weakForm at the current state by the matrix-free finite difference of the
 * reference's implicit solver (implicit.f90:483-531, MatrixVector without its V - alpha dt term; step size
 * of InitImplicit, implicit.f90:141-163): fdOrder 1 (one-sided) or 2 (central), epsMethod 1 (Qin, Ludlow,
 * Shaw: sqrt(eps) scaleps/|V|) or 2 (Knoll, Keyes: additionally sqrt(1+|U|)); the reference defaults are
 * fdOrder 1, epsMethod 2, scaleps 1. V and JV have the layout of U; the state is left unchanged. */
int fg_jvp_time_derivative(fg_handle* h, double t, const double* V, double* JV, int fdOrder, int epsMethod, double scaleps);

/* Adjoint of TimeStepByLSERKW2 (timestep.f90:82) over nSteps steps of fixed dt (the time step is not
 * differentiated), in two calls. fg_adjoint_forward advances the state by nSteps steps and keeps a device
 * checkpoint of U every ckptEvery steps. fg_adjoint_reverse takes UbarT = dL/dU(t_end) (layout of U) and
 * returns Ubar0 = dL/dU(t_0) and muScaleBar[nElems] = dL/d(viscosity multipliers), both optional: per
 * segment it recomputes the stage states from the checkpoint and runs the transposed stages in reverse.
 * Device memory: (nSteps/ckptEvery + 5 ckptEvery + 3) states; when it takes at most half of the free
 * device memory, the forward intermediates of the 5 ckptEvery stages of a segment are kept as well (about
 * 8 states per stage), so that the adjoint right-hand sides skip their recomputation (environment variable
 * FLEXI_GB300_ADJOINT_RECOMPUTE=1 forces the recomputing path). The state is left at t_end. No counterpart
 * in the reference. */
int fg_adjoint_forward(fg_handle* h, int nSteps, double dt, int ckptEvery);
/* ckptEvery < 0 selects binomial checkpointing (Griewank's revolve schedule) with -ckptEvery snapshot
 * states in device memory instead of uniform checkpoints: horizons of C(s + r, s) steps need s + 1
 * snapshots and r forward repetitions, so long horizons fit in a fixed memory budget. A binomial reverse
 * sweep reuses the snapshot slots and needs a new fg_adjoint_forward before the next sweep. */
/* Forward steps the last fg_adjoint_reverse re-ran (the recomputation cost of its schedule). */
long long fg_adjoint_recomputed_steps(const fg_handle* h);
/* forceBar(0:N,0:N,0:N,nElems) (optional) = dL/d(body-force field of fg_set_body_force_field). With the channel
 * body force or a body-force field, the dependence of each step's bulk velocity on its start state is
 * included. */
int fg_adjoint_reverse(fg_handle* h, const double* UbarT, double* Ubar0, double* muScaleBar, double* forceBar);

/* Additional x-momentum body-force field F(0:N,0:N,0:N,nElems) with the form of the channel forcing
 * (testcase/channel/testcase.f90:361-362): Ut(MOM1) += F, Ut(ENER) += F * BulkVel (after the Jacobian);
 * NULL sets it to zero. No counterpart in the reference (the parameter of a gradient study). */
int fg_set_body_force_field(fg_handle* h, const double* F);

/* Mean wall shear of the current state: J = sum over wall side points of the x-momentum viscous flux through
 * the wall times SurfElem, divided by the wall area (the lifted face gradients of the master side, as in
 * GetBoundaryFlux). dJdU (optional, layout of U) = dJ/dU through the lifting. No counterpart in the
 * reference. */
int fg_wall_shear(fg_handle* h, double* J, double* dJdU);

/* Autotuner (no counterpart in the reference): times, on the handle's mesh and current state with CUDA
 * events over reps launches each, the candidate launch shapes -- elements per CTA of the prep, lifting and
 * weak-form volume kernels (default and one alternative, N=3 and N=5) and the block size of the side
 * kernel (64/128/256) -- and keeps the fastest for all later launches (the captured time loop is captured
 * again). report[9] (optional) = ms per launch of prep default/alternative, lift default/alternative,
 * volume default/alternative, side kernel 64/128/256 (NaN where not a candidate); the state is unchanged. */
int fg_autotune(fg_handle* h, int reps, double* report);
/* Shapes in use: out[0..2] = elements per CTA of prep, lifting, weak-form volume; out[3] = side-kernel block. */
int fg_autotune_choice(const fg_handle* h, int* out);
/* Sets the shapes explicitly (each element count the default or the alternative of this N, as
 * fg_autotune_choice reports them; side block 64/128/256), e.g. to reproduce a tuned run. */
int fg_set_launch_shapes(fg_handle* h, int epbPrep, int epbLift, int epbVol, int fluxBlock);

/* FP64 pipe probes of the current device (no counterpart in the reference): the rate an arithmetic FP64 instruction
 * stream attains, next to which the roofline of these FP64-bound kernels is read. fg_probe_fp64_pipe: rates[0..3] = DFMA,
 * DADD, DMUL alone and the three mixed, in T thread-instructions per second (independent chains on every SM).
 * fg_probe_fp64: 2 x the DFMA rate (TFLOP/s). */
int fg_probe_fp64_pipe(double* rates);
int fg_probe_fp64(double* tflops);
/* FP64 tensor-core throughput of the current device, TFLOP/s: rates[0] = mma.sync m8n8k4 f64 alone (two independent
 * accumulator chains per warp), rates[1] = the same interleaved with eight independent DFMA chains per thread (MMA
 * and DFMA flops together). If rates[1] is not above the larger of rates[0] and 2 x the DFMA rate, the two share the
 * FP64 units. No counterpart in the reference. */
int fg_probe_fp64_tensor(double* rates);
/* Time (ms) of the same DFMA chains run by 32, 16, 8, 4 and 1 active lanes of every warp (ms[0..4]): equal times mean
 * the FP64 pipe spends the same issue time on a warp instruction whatever its active lanes, so idle lanes of FP64 code
 * are lost pipe time. No counterpart in the reference. */
int fg_probe_fp64_lanes(double* ms);

/* ---- Allocation-free right-hand side (no counterpart in the reference) ----------------------------
 * For callers that cannot allocate device memory: host codes whose device memory all comes from their
 * own pool or caching allocator, and time loops that must not allocate once they run. Everything is
 * caller-owned DEVICE memory in the library's device layouts (n = N+1 nodes per direction, n2 = n*n,
 * n3 = n*n*n); the layouts are those fg_debug_array returns for "U", "metr", "sJ", "geo", "elemSide",
 * "sideElem", "bcType", "bcTwall". BC sides are sides 0..nBCSides-1, as in FLEXI. */
typedef struct fg_device_mesh {
  int nElems, nSides, nBCSides;
  const int* elemSide;    /* [nElems][6]: 8*sideID + flip per local side ZETA-,ETA-,XI+,ETA+,XI-,ZETA+ (flip 0: master) */
  const int* sideElem;    /* [nSides][4]: master elem, master local side, slave elem (-1 on BC sides), 8*slave local side + flip */
  const double* metr;     /* [nElems][9][n3]: Metrics_fTilde(1:3), Metrics_gTilde(1:3), Metrics_hTilde(1:3) */
  const double* sJ;       /* [nElems][n3]: 1/J */
  const double* geo;      /* [nSides][10][n2]: NormVec(3), TangVec1(3), TangVec2(3), SurfElem */
  const int* bcType;      /* [nBCSides]: FLEXI BC type of each BC side, 3 (adiabatic wall) or 4 (isothermal wall) */
  const double* bcTwall;  /* [nBCSides]: wall temperature of each BC side (isothermal walls) */
} fg_device_mesh;

/* The device tables of fg_device_mesh are not checked: they must describe a valid mesh as this library builds it (as
 * fg_debug_array returns them from a handle), with side and element ids in range and bcType 3 or 4 only; other values
 * make the kernels read or write out of bounds or apply neither wall condition. */

/* Largest scratch the allocation-free call can use: 64 MiB of static device memory, held by every
 * device that loads the library (e.g. 343 elements at N=7, ~2500 elements at N=3). */
#define FG_NOALLOC_SCRATCH_BYTES (64ull << 20)

/* Ut = DGTimeDerivative_weakForm(U) for one instance with viscosity cfg->mu0, like fg_time_derivative
 * but handle-free and allocation-free: U and Ut are DEVICE arrays [nElems][5][n3], the launches are
 * asynchronous on `stream` (cudaStream_t as void*, NULL = legacy default stream). All intermediate
 * arrays live in one static __device__ scratch array of FG_NOALLOC_SCRATCH_BYTES; the call clears what
 * must start at zero (sticky error word, instance ids) itself on the stream. The first call on each
 * device, with that device current, looks up the scratch address and sets the kernels' shared-memory
 * limits: make it before any stream capture. That set-up belongs to the CUDA context it ran in and is
 * redone by the first call in a later context of the device (e.g. after cudaDeviceReset); host threads
 * making first calls together are serialised on it. Calls that overlap on the GPU (other streams, or host
 * threads without ordering) race on the shared scratch. The call reports no NaN (it runs no CALCTIMESTEP)
 * and no asynchronous kernel fault (check the stream); it refuses to run, leaving the error in place, when a
 * CUDA error of earlier work is pending on the calling thread. Meshes needing more scratch, and configurations
 * the kernels do not cover (N > 7, weak or conservative lifting, body force, overintegration, split form
 * off Gauss-Lobatto nodes or with N not in {1,3,7}), are rejected before any launch, with the reason in
 * fg_last_error(NULL). No cudaMalloc, cudaFree or other device allocation is made. */
int fg_time_derivative_noalloc(const fg_config* cfg, const fg_device_mesh* mesh, const double* U, double* Ut, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* FLEXI_GPU_H */
