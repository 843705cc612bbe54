/*
 * galaexi_gb300 -- C ABI of the GB300-native DGSEM right-hand side and its
 * low-storage Runge-Kutta stepper.
 *
 * This boundary replaces the module-global operator of GALAEXI:
 *   DGTimeDerivative_weakForm(t)        src/dg/dg.f90:255-425
 *   TimeStepByLSERKW2(t)                src/timedisc/timestep.f90:49-120
 *   CALCTIMESTEP(errType)               src/equations/navierstokes/calctimestep.f90:98-186
 *   InitDGbasis / InitMesh device copies src/dg/dg.f90:181-242, src/mesh/mesh.f90:307-451
 * The reference works on module-global device arrays (MOD_DG_Vars, MOD_Mesh_Vars,
 * MOD_Lifting_Vars); here the same arrays are passed explicitly, in the
 * reference's Fortran (column-major) layouts:
 *   U, Ut           (nVar=5, 0:N, 0:N, 0:N, nElems)   conservative state / time derivative
 *   Metrics_f/g/hTilde (3, 0:N, 0:N, 0:N, nElems)     contravariant metric terms J*a^i
 *   sJ              (0:N, 0:N, 0:N, nElems)           inverse Jacobian
 *   NormVec/TangVec1/TangVec2 (3, 0:N, 0:N, nSides)   master-side face frame
 *   SurfElem        (0:N, 0:N, nSides)                surface element
 *   ElemToSide      (3, 6, nElems)  int32, 1-based IDs (E2S_SIDE_ID, E2S_FLIP, E2S_IS_MASTER)
 *   SideToElem      (5, nSides)     int32, 1-based IDs, -1 where absent
 * All functions return 0 on success or a negative DG_ERR_* status; none of them
 * aborts the process or traps on the device.  dg_last_error() describes the
 * most recent failure of the calling thread.
 *
 * Ownership: the caller owns U, Ut and Ut_tmp (device pointers, FP64); the
 * context owns copies of metrics, connectivity and all scratch, sized once in
 * dg_set_mesh.  dg_rhs / dg_lserk_step allocate nothing.
 * Threading: one context per host thread and stream; calls are asynchronous
 * on the given stream except dg_calc_timestep and dg_check_state, which
 * return one host scalar each.
 */
#ifndef GALAEXI_GB300_H
#define GALAEXI_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define DG_OK               0
#define DG_ERR_ARG         -1   /* invalid argument or call order            */
#define DG_ERR_ALLOC       -2   /* device allocation failed                  */
#define DG_ERR_CUDA        -3   /* a CUDA runtime call failed                */
#define DG_ERR_NAN         -4   /* NaN, Inf or non-positive density/pressure */
#define DG_ERR_TIMEOUT     -5   /* a bounded device wait gave up             */
#define DG_ERR_UNSUPPORTED -6   /* option combination not built              */

/* ---- option values (ini keys of the reference, see dg_config) ----------- */
/* NodeType: PP_NodeType of the reference build (src/CMakeLists.txt) */
#define DG_NODETYPE_GAUSS          1
#define DG_NODETYPE_GAUSS_LOBATTO  2
/* Riemann: the RIEMANN macro numbering of src/equations/navierstokes/riemann.f90:69-87 */
#define DG_RIEMANN_LF              0
#define DG_RIEMANN_ROE             1
#define DG_RIEMANN_ROEL2           2
#define DG_RIEMANN_ROEENTROPYFIX   3
#define DG_RIEMANN_HLL             4
#define DG_RIEMANN_HLLC            5
#define DG_RIEMANN_HLLE            6
#define DG_RIEMANN_HLLEM           7
#define DG_RIEMANN_AVERAGE         8   /* Riemann_FluxAverage, split form only (riemann.f90:1239) */
/* SplitDG: the SPLIT_DG macro numbering of splitflux.f90:36-66; -1 = weak form */
#define DG_SPLIT_NONE             -1
#define DG_SPLIT_SD                0
#define DG_SPLIT_MO                1
#define DG_SPLIT_DU                2
#define DG_SPLIT_KG                3
#define DG_SPLIT_PI                4
/* Lifting: PP_Lifting (src/dg/lifting/lifting.f90:26-32) */
#define DG_LIFTING_BR1             1
#define DG_LIFTING_BR2             2
/* precision form of the bulk operator */
#define DG_PRECISION_FP64          0   /* plain FP64 everywhere                              */
#define DG_PRECISION_MIXED         1   /* FP32 volume/face/lifting/surface work, FP64 U, RK,
                                          metric precompute, CFL reduction and integrals     */

/* Run-time configuration.  Field names follow the reference's ini keys
 * (N, NodeType, Riemann, SplitDG, kappa, R, Pr, mu0, doWeakLifting,
 * doConservativeLifting, etaBR2); in GALAEXI several of them are compile-time
 * macros, here all are run-time. */
typedef struct dg_config {
  int    N;                     /* polynomial degree, 1..DG_MAX_N                     */
  int    node_type;             /* DG_NODETYPE_*                                      */
  int    parabolic;             /* 0: Euler, 1: Navier-Stokes (constant mu0)          */
  int    riemann;               /* DG_RIEMANN_*                                       */
  int    split_dg;              /* DG_SPLIT_*; split forms need Gauss-Lobatto nodes   */
  int    lifting;               /* DG_LIFTING_*                                       */
  int    do_weak_lifting;       /* doWeakLifting (BR1)                                */
  int    do_conservative_lifting; /* doConservativeLifting (BR1, strong form)         */
  double eta_br2;               /* etaBR2                                             */
  double kappa, R, Pr, mu0;     /* EOS_Vars (idealgas/eos.f90:191-203)                */
  int    precision;             /* DG_PRECISION_*                                     */
  /* filter of the solution at the start of every operator call (filter.f90:100-311) */
  int    filter_type;           /* DG_FILTER_* (FilterType)                           */
  int    n_filter;              /* NFilter: highest kept mode (cut-off, LAF)          */
  double hest_filter_param[3];  /* HestFilterParam (alpha, s, cut-off mode), modal    */
  double laf_alpha;             /* LAF_alpha                                          */
} dg_config;

/* FilterType (filter.f90:40-43) */
#define DG_FILTER_NONE   0
#define DG_FILTER_CUTOFF 1
#define DG_FILTER_MODAL  2
#define DG_FILTER_LAF    3

#define DG_MAX_N 9

typedef struct dg_ctx dg_ctx;

/* Fill *cfg with the reference's defaults (N=3, Gauss-Lobatto, Euler, LF,
 * weak form, BR1 strong non-conservative, kappa=1.4, R=287.058, Pr=0.72,
 * mu0=0, etaBR2=2, FP64). */
void dg_config_default(dg_config* cfg);

/* Parse ini text (key = value lines, '!' comments, case-insensitive keys and
 * string values) into *cfg, starting from the values already in *cfg.
 * Recognised keys: N, NodeType, Riemann, SplitDG, Lifting, Parabolic, kappa, R, Pr,
 * mu0, doWeakLifting, doConservativeLifting, etaBR2, Precision, FilterType, NFilter,
 * HestFilterParam, LAF_alpha.  Replaces the
 * GET* calls of src/readintools/readintools.f90:1021-1229 for these keys. */
int dg_config_from_ini(const char* ini_text, dg_config* cfg);

/* Create a context: builds D, D^T, D_hat^T, L+-, L_hat+-, DVolSurf
 * (InitDGbasis, src/dg/dg.f90:181-242) and uploads them. */
int dg_ctx_create(const dg_config* cfg, dg_ctx** ctx);
int dg_ctx_destroy(dg_ctx* ctx);

/* Upload mesh data (host pointers, layouts above) and size all scratch.
 * Replaces the device copies of InitMesh (src/mesh/mesh.f90:307-451) and
 * InitCalctimestep (calctimestep.f90:51-92).  Periodic and inner faces are
 * resolved in-kernel.  As in the reference's side order, the first nBCSides sides
 * are boundary sides with a master element only; a mesh with nBCSides > 0 needs
 * dg_set_boundaries before the operator is used. */
int dg_set_mesh(dg_ctx* ctx, int nElems, int nSides, int nBCSides,
                const double* metrics_f, const double* metrics_g, const double* metrics_h,
                const double* sJ,
                const double* normvec, const double* tangvec1, const double* tangvec2,
                const double* surfelem,
                const int* elem_to_side, const int* side_to_elem);

/* Boundary conditions of the BC sides: the reference's BCSides(BC_TYPE, BC_STATE) per side and
 * its RefStates (InitBC, equations/navierstokes/idealgas/getboundaryflux.f90:87-256).
 * bc_type[s], bc_state[s] for s < nBCSides: type 2 (Dirichlet, RefState), 3 (adiabatic wall),
 * 4 (isothermal wall, RefState temperature), 9 / 91 (slip walls), 23 (outflow, RefState u = Mach
 * number), 24 / 25 (pressure / subsonic outflow, RefState p), 27 (subsonic inflow); bc_state is
 * the 1-based RefState index (ignored for 3, 9, 91).  refstate: nRefState x 5 RefState rows as in
 * the parameter file, (rho, u, v, w, p); a state used by type 27 is (Tt, alpha, beta, -, pt) with
 * the angles in degrees and is turned into the inflow direction as InitBC does.
 * Other BC types return DG_ERR_UNSUPPORTED. */
int dg_set_boundaries(dg_ctx* ctx, const int* bc_type, const int* bc_state, int nRefState, const double* refstate);

/* Ut = DGTimeDerivative_weakForm(U) at time t (src/dg/dg.f90:255-425).
 * d_U, d_Ut: device FP64 arrays (5,0:N,0:N,0:N,nElems); stream: cudaStream_t or NULL.
 * With a filter configured (FilterType > 0) d_U is first filtered in place, as the reference's
 * step 1 does (dg.f90:330); otherwise it is only read. */
int dg_rhs(dg_ctx* ctx, double t, double* d_U, double* d_Ut, void* stream);

/* Per-element state of the LAF filter after the last operator call (Filter_LAF,
 * filter.f90:318-474; written as element data LAF_lim, LAF_eRatio, LAF_r by the reference):
 * host arrays of nElems values, any may be NULL.  DG_ERR_ARG unless FilterType is LAF. */
int dg_laf_state(dg_ctx* ctx, double* lim, double* eRatio, double* r);

/* One Carpenter-Kennedy RK4-5 low-storage step (TimeStepByLSERKW2,
 * timestep.f90:49-120, coefficients timedisc_vars.f90:213-227), updating
 * d_U in place; d_Ut_tmp is the caller-owned second register (zero it before
 * the first step, as the reference does). */
int dg_lserk_step(dg_ctx* ctx, double t, double dt, double* d_U, double* d_Ut_tmp, void* stream);

/* Several steps of fixed dt in one call (the same arithmetic as repeated
 * dg_lserk_step calls). */
int dg_lserk_steps(dg_ctx* ctx, double t, double dt, int nSteps, double* d_U, double* d_Ut_tmp,
                   void* stream);

/* dt = min over elements of CFLScale*2/lambda_conv and DFLScale*4/lambda_visc
 * (CALCTIMESTEP, calctimestep.f90:98-296).  cfl_scale / dfl_scale are the
 * ini values CFLScale / DFLScale; the N- and node-type-dependent scaling of
 * FillCFL_DFL (timedisc_func.f90:480-550, Carpenter RK4-5 tables) is applied
 * inside.  Synchronises the stream.  Returns DG_ERR_NAN if the state holds a
 * NaN or a non-positive density or pressure. */
int dg_calc_timestep(dg_ctx* ctx, const double* d_U, double cfl_scale, double dfl_scale,
                     double* dt_out, void* stream);

/* Allocation-free time step (no counterpart in the reference).
 *
 * Some callers cannot allocate device memory: a host code whose device arrays all belong to another
 * runtime's allocator (GALAEXI's CUDA Fortran arrays live in nvfortran's heap), a process that must
 * keep a fixed device-memory budget once its time loop has started, or a loop that cannot afford the
 * device-wide synchronisation cudaMalloc/cudaFree may imply.  For them this entry point computes the
 * same dt as dg_calc_timestep without a context and without any allocation: the caller passes the
 * state and the metric arrays it already holds on the device, in the reference layouts
 * U(5,0:N,0:N,0:N,nElems), Metrics_f/g/hTilde(3,0:N,0:N,0:N,nElems), sJ(0:N,0:N,0:N,nElems), and the
 * scratch comes from a static device array of the library (DG_NOALLOC_MAX_ELEMS eigenvalue pairs,
 * 8 MiB, held on every GPU that loads the library until the process exits).
 *   - nElems above DG_NOALLOC_MAX_ELEMS is rejected with DG_ERR_ARG.
 *   - Each call looks up the device address of the static array in the current device's context
 *     (cudaGetSymbolAddress): call it with the device that holds the arrays current.
 *   - Every call uses the same static array; the previous call's contents stay in it (the error
 *     counter is cleared at the start of each call).  Calls whose work overlaps on the GPU (other
 *     streams, other host threads) race on that array: serialise them.
 * Copies dt to the host and synchronises the stream; returns DG_ERR_NAN for NaN/Inf or non-positive
 * density/pressure. */
#define DG_NOALLOC_MAX_ELEMS (1 << 19)
int dg_calc_timestep_noalloc(int N, int node_type, int nElems, int parabolic, double kappa, double mu0, double Pr,
                             const double* d_U, const double* d_metrics_f, const double* d_metrics_g,
                             const double* d_metrics_h, const double* d_sJ, double cfl_scale, double dfl_scale,
                             double* dt_out, void* stream);

/* Scan the state for NaN/Inf or non-positive density/pressure; *bad_count
 * receives the number of bad nodes.  Synchronises the stream. */
int dg_check_state(dg_ctx* ctx, const double* d_U, long long* bad_count, void* stream);

/* Lifted gradients of the last RHS evaluation (dg_rhs or the last stage of dg_lserk_step[s]):
 * the reference's GradUx/GradUy/GradUz(PP_nVarLifting=5, 0:N,0:N,0:N, nElems) module arrays
 * (lifting_vars.f90), lifting variables (rho, u, v, w, T) = LIFT_DENS..LIFT_TEMP (eos.h:136-142),
 * which the reference's analysis routines read (testcase/taylorgreenvortex/testcase.f90:283-510).
 * Each output is a device array of 5*(N+1)^3*nElems doubles; the mixed form converts from FP32.
 * DG_ERR_UNSUPPORTED for a non-parabolic operator, DG_ERR_ARG before the first RHS on the mesh. */
int dg_get_gradients(dg_ctx* ctx, double* d_gradUx, double* d_gradUy, double* d_gradUz, void* stream);

/* Volume integrals of the state in FP64 on the solution nodes (quadrature weights w_i w_j w_k / sJ,
 * as the reference's analysis integrates, analyze.f90:383-484): out6 = {mass, x-, y-, z-momentum,
 * total energy, kinetic energy 0.5|m|^2/rho}.  Synchronises the stream.  No counterpart as one call
 * in the reference (its testcase analysis computes these on the host). */
int dg_integrals(dg_ctx* ctx, const double* d_U, double* out6, void* stream);

/* Kinetic-energy objective J = sum w_i w_j w_k / sJ * 0.5|m|^2/rho and, if d_dJdU is not null, its
 * gradient dJ/dU (device array in the state layout).  Synchronises the stream. */
int dg_kinetic_energy(dg_ctx* ctx, const double* d_U, double* J, double* d_dJdU, void* stream);

/* ---- tangent-linear and adjoint operators (FP64 form; no counterpart in the reference) ---------
 * Supported: Gauss or Gauss-Lobatto nodes, weak form or split form PI / KG, every Riemann solver,
 * Euler or Navier-Stokes, periodic meshes and meshes with boundary sides (every BC type of
 * dg_set_boundaries), no solution filter; the adjoint with BR1 lifting in strong form.  The
 * tangent-linear operator also takes BR1 in weak or conservative form and BR2.  Others return
 * DG_ERR_UNSUPPORTED.
 *
 * dg_rhs_jvp: Ut = R(U) (if d_Ut is not null) and Utdot = dR/dU . Udot + dR/dmu . mu_dot, the exact
 * linearisation of the operator (forward-mode dual numbers through the same kernels).
 * dg_tlm_steps: nSteps LSERK steps of U and of its tangent Udot (fixed dt). */
int dg_rhs_jvp(dg_ctx* ctx, double t, const double* d_U, const double* d_Udot, double mu_dot, double* d_Ut,
               double* d_Utdot, void* stream);
int dg_tlm_steps(dg_ctx* ctx, double t, double dt, int nSteps, double* d_U, double* d_Udot, double mu_dot,
                 double* d_Ut_tmp, void* stream);

/* dg_rhs_vjp: d_Ubar = (dR/dU)^T d_Utbar at d_U, and *mu_bar = <d_Utbar, dR/dmu> (if not null). */
int dg_rhs_vjp(dg_ctx* ctx, double t, const double* d_U, const double* d_Utbar, double* d_Ubar, double* mu_bar,
               void* stream);

/* Discrete adjoint of nSteps LSERK-W2 steps with fixed dt from d_U0.
 * dg_adjoint_forward runs the window and records checkpoints in device memory of at most
 * budget_bytes: every stage input if that fits (plan 1), else segment starts every k steps plus the
 * stage inputs of one segment but its first (which is the segment start), recomputed during the
 * reverse sweep (plan 2, one extra forward sweep over all segments but the last), else segment starts plus the step starts of one segment plus one
 * step's stage inputs (plan 3, two extra sweeps); the last segment's checkpoints are recorded by the
 * forward run itself.  *plan_out (if not null) receives the plan.  d_U_final (if not null) receives
 * the end state.
 * dg_adjoint_reverse: on entry d_Ubar holds dJ/dU(t_end); on exit dJ/dU(t0); *mu_bar = dJ/dmu.
 * Consumes the recorded window.
 * dg_adjoint_window: both, for J = the kinetic-energy integral of the end state (dg_kinetic_energy);
 * writes J, dJ/dU0 and dJ/dmu. */
int dg_adjoint_forward(dg_ctx* ctx, double t0, double dt, int nSteps, const double* d_U0, double* d_U_final,
                       size_t budget_bytes, int* plan_out, void* stream);
/* Device memory (bytes) that the adjoint entry points still allocate besides the checkpoints: its
 * work states and scratch, for sizing budget_bytes against the free memory.  d_U_final may alias
 * d_U0 (the start state is read once, at the start). */
int dg_adjoint_scratch_bytes(dg_ctx* ctx, size_t* bytes);
int dg_adjoint_reverse(dg_ctx* ctx, double* d_Ubar, double* mu_bar, void* stream);
int dg_adjoint_window(dg_ctx* ctx, double t0, double dt, int nSteps, const double* d_U0, size_t budget_bytes,
                      double* J, double* d_dJdU0, double* dJdmu, double* d_U_final, void* stream);

/* Reference pressure of the mixed form (no counterpart in the reference).  With p_ref > 0 the FP32
 * bulk works with p' = p - p_ref (formed in FP64 from the FP64 state) in the momentum pressure terms
 * of the volume and surface fluxes.  The constant p_ref drops out of the operator for
 * free-stream-preserving metrics, so results are unchanged in exact arithmetic, while low-Mach
 * pressure differences keep FP32 precision.  Ignored by the FP64 form.  Default 0. */
int dg_set_pressure_offset(dg_ctx* ctx, double p_ref);

/* Measurement utilities (no counterpart in the reference).
 * dg_profile_stage: run `reps` LSERK stages on d_U / d_Ut_tmp (modified in place) with CUDA events
 * around each kernel; ms_out[0..4] = average ms of (prolong, lift, face, volume, whole stage).
 * dg_measure_fma_peak: FMA-chain microkernel on the current device; precision 0 = FP64, 1 = FP32;
 * *gflops receives the achieved FLOP rate (FMA = 2 flops). */
int dg_profile_stage(dg_ctx* ctx, double* d_U, double* d_Ut_tmp, double dt, int reps, double* ms_out, void* stream);
int dg_measure_fma_peak(int precision, double* gflops);

/* Self-test of the bounded waits of the kernels that stage data by bulk copies (no counterpart in
 * the reference).  Launches one block that arms a shared-memory barrier for 16 bytes that no copy
 * delivers and waits for it with `polls` polls, as those kernels wait for their copies; the wait runs
 * out, the block records the timeout and returns.  Returns DG_ERR_TIMEOUT (the status those kernels'
 * callers report) with *seconds = the duration of the wait, DG_OK if the wait completed (which
 * would be a defect), or an error code. */
int dg_selftest_bulk_wait(long long polls, double* seconds);

/* Number of kernels this context launched since creation (for accounting). */
long long dg_kernel_launch_count(const dg_ctx* ctx);

/* Description of the last error on the calling thread. */
const char* dg_last_error(void);

/* ---- HOPR mesh files (HDF5): ReadMesh + BuildCoords + CalcMetrics (mesh_readin.f90:204-470,
 * metrics.f90:85-789) without MPI and mortars --------------------------------------------------
 * dg_mesh_hopr_sizes: element/side counts of the file (BC sides counted in nSides; periodic sides
 * are connected sides, not BC sides).  dg_mesh_hopr: the arrays of dg_mesh_cartesian for N and the
 * node type, computed from the file's NGeo node coordinates; BC sides come first (1..nBCSides) and
 * BCIndex[0..nBCSides-1] (if not null) receives their BC index into the file's BCNames/BCType. */
int dg_mesh_hopr_sizes(const char* path, int* nElems, int* nSides, int* nBCSides, int* NGeo);
/* The file's boundary table (ReadBCs, mesh_readin.f90:78-189): *nBCs, and if not null the names
 * (nBCs x name_len bytes, NUL-terminated, trailing blanks trimmed) and BCType rows (nBCs x 4:
 * type, curve index, state, periodic vector index). */
int dg_mesh_hopr_bcs(const char* path, int* nBCs, char* names, int name_len, int* bc_type);
/* A dataset (attribute = 0) or root attribute (attribute = 1) of an HDF5 file such as a FLEXI state
 * file (DG_Solution, Time, N, NodeType, MeshFile; ReadState, restart.f90): *ndims and dims[0..7]
 * (slowest first); numbers as doubles into out (if not null; cap >= element count); a string's first
 * element into str (str_len bytes, NUL-terminated). */
int dg_h5_read(const char* path, const char* name, int attribute, int* ndims, long long* dims, double* out,
               long long cap, char* str, int str_len);
/* A FLEXI state file (WriteState, io_hdf5/hdf5_output.f90:84-211): the dataset DG_Solution
 * (5,0:N,0:N,0:N,nElems) from the host array U, and the root attributes File_Type = 'State',
 * Project_Name, File_Version, Program, VarNames, N, Dimension, Time, MeshFile, NextFile, NodeType
 * ('GAUSS' or 'GAUSS-LOBATTO').  The file is written without libhdf5 (HDF5 superblock version 0,
 * the structures of the reference's own state files). */
int dg_write_state(const char* path, const char* project, const char* mesh_file, int N, const char* node_type,
                   double time, int nElems, const double* U);
int dg_mesh_hopr(const char* path, int N, int node_type, double* elem_xgp, double* metrics_f, double* metrics_g,
                 double* metrics_h, double* sJ, double* nvec, double* t1, double* t2, double* surfelem,
                 int* elem_to_side, int* side_to_elem, int* BCIndex);

/* ---- host-side mesh and state set-up (stand-ins for HOPR + ReadMesh) ------ */

/* Basis of the reference (InitInterpolationBasis + InitDGbasis): arrays of
 * length N+1 or (N+1)^2 (column-major (0:N,0:N)).  Any output may be NULL. */
int dg_basis(int N, int node_type, double* xGP, double* wGP, double* wBary,
             double* L_minus, double* L_plus, double* D, double* D_hat_T,
             double* L_hat_minus, double* L_hat_plus, double* DVolSurf);

/* Sizes of a periodic Cartesian box of nx*ny*nz hexahedra. */
int dg_mesh_cartesian_sizes(int nx, int ny, int nz, int* nElems, int* nSides);

/* Build a periodic box [x0,x1]^3 with nx*ny*nz elements.  Each element's mapping is
 * given, as in a HOPR mesh file, by node coordinates on NGeo+1 equidistant points per
 * direction, optionally displaced by x_i += deform_amp * sin(2 pi xh) sin(2 pi yh)
 * sin(2 pi zh) with (xh,yh,zh) the coordinates normalised to [0,1] (the node
 * displacement of the reference's meshdeform, mesh.f90:224-234).  deform_amp = 0:
 * affine box, with the exact (constant) metric terms and the exact node positions
 * Elem_xGP; otherwise BuildCoords + CalcMetrics + CalcSurfMetrics of the reference
 * (metrics.f90:85-750: curl form on the Chebyshev-Gauss-Lobatto points, the
 * Jacobian on 3 NGeo nodes projected to N) on the node coordinates.  Outputs in the
 * layouts of dg_set_mesh plus NodeCoords(3,0:NGeo,0:NGeo,0:NGeo,nElems) and
 * Elem_xGP(3,0:N,0:N,0:N,nElems) (either may be NULL).  Every element is master of
 * its XI_PLUS, ETA_PLUS and ZETA_PLUS sides.  A displacement that folds an element
 * (scaled Jacobian below 0.01, the reference's abort criterion) is DG_ERR_ARG. */
int dg_mesh_cartesian(int N, int node_type, int NGeo, int nx, int ny, int nz,
                      const double* x0, const double* x1, double deform_amp,
                      double* node_coords, double* elem_xgp,
                      double* metrics_f, double* metrics_g, double* metrics_h, double* sJ,
                      double* normvec, double* tangvec1, double* tangvec2, double* surfelem,
                      int* elem_to_side, int* side_to_elem);

/* Initial states at the nodes (FillIni, src/dg/dg.f90:432-456).  xgp: (3,nNodes), U: (5,nNodes).
 *   DG_EXACTFUNC_CONST      params: RefState (rho,u,v,w,p)
 *   DG_EXACTFUNC_SHU_VORTEX params: RefState(5), IniCenter(3), IniAxis(3), IniAmplitude, IniHalfwidth
 *                           (IniExactFunc=7, idealgas/exactfunc.f90:482-502; t advects the centre)
 *   DG_EXACTFUNC_TGV        params: rho0, U0, MachNumber, IniConstDens (0/1)
 *                           (testcase/taylorgreenvortex/testcase.f90:145-149,220-262) */
#define DG_EXACTFUNC_CONST       1
#define DG_EXACTFUNC_SHU_VORTEX  7
#define DG_EXACTFUNC_TGV       100
int dg_fill_ini(int exactfunc, const double* params, int nParams, long long nNodes, const double* xgp,
                double kappa, double R, double t, double* U);

#ifdef __cplusplus
}
#endif
#endif /* GALAEXI_GB300_H */
