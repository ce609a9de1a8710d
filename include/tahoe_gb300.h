/*
 * tahoe_gb300 -- C ABI of the GB300 implicit hex8 solid path.
 *
 * The entry points below are what a Tahoe host build binds when a deck
 * selects the GPU element group and the GPU matrix/solver type.  They replace
 * the per-element virtual calls and the CPU global-matrix classes of the
 * reference; each declaration names the reference interface it stands in for
 * (paths relative to the Tahoe source tree).
 *
 * Conventions
 *   - every entry point returns an int status: TG_OK (0) or a negative
 *     TG_ERR_* code; nothing throws across the ABI and no kernel traps;
 *   - equation numbers are the reference's: 1-based, node-major/dof-minor,
 *     <= 0 for prescribed dofs (NodeManagerT::SetEquationNumbers);
 *   - "nodal" arrays are nnd*3 doubles, node-major (x,y,z per node);
 *     "equation" arrays are neq doubles indexed by equation number - 1;
 *   - one CUDA stream per context; a context is not thread-safe.
 */
#ifndef TAHOE_GB300_H
#define TAHOE_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tg_context tg_context;

enum tg_status {
  TG_OK = 0,
  TG_ERR_ARG = -1,            /* bad argument or call order */
  TG_ERR_CUDA = -2,           /* CUDA runtime error (text in tg_last_error) */
  TG_ERR_OOM = -3,            /* device allocation failed */
  TG_ERR_BAD_JACOBIAN = -4,   /* det J <= 0 or J <= 0 (ExceptionT::kBadJacobianDet) */
  TG_ERR_NAN = -5,            /* non-finite residual or Krylov scalar */
  TG_ERR_NOT_CONVERGED = -6,  /* iteration limit hit (NLSolver kFailed) */
  TG_ERR_DIVERGED = -7,       /* relative error above divergence tolerance */
  TG_ERR_CAPACITY = -8        /* size above a fixed capacity */
};

enum tg_formulation { TG_SMALL_STRAIN = 0, TG_TOTAL_LAGRANGIAN = 1, TG_UPDATED_LAGRANGIAN = 2 };
enum tg_strain_displacement { TG_STRAIN_STANDARD = 0, TG_STRAIN_BBAR = 1 };

enum tg_material_kind {
  TG_MAT_SS_HOOKEAN = 0,  /* small_strain_StVenant / small_strain_Hookean: {E,nu} or C[36] row-major */
  TG_MAT_SS_J2 = 1,       /* small_strain_StVenant_J2: {E, nu, a, b[, elastic_iterations]} */
  TG_MAT_FS_SIMO = 2,     /* Simo_isotropic: {mu, kappa} */
  TG_MAT_FS_STVENANT = 3  /* large_strain_StVenant: {E, nu} */
};

/* TG_FP64: plain form (FP64 tangent, FP64 CSR, FP64 PCG).
 * TG_MIXED: FP32 element tangent, FP32 CSR and inner PCG vectors, FP64
 *           residual, FP64 Krylov dot products/norms and FP64 Newton test. */
enum tg_precision { TG_FP64 = 0, TG_MIXED = 1 };
enum tg_precond { TG_PRECOND_JACOBI = 0, TG_PRECOND_BLOCK_JACOBI = 1 };

/* J2 integration-point flags (J2SSC0HardeningT.h:32-34) plus "never yielded"
 * (the reference leaves such ElementCardT storage unallocated). */
enum tg_j2_flag { TG_J2_PLASTIC = 0, TG_J2_ELASTIC = 1, TG_J2_RESET = 3, TG_J2_UNALLOCATED = 7 };

/* ---- context ------------------------------------------------------------ */

/* Creates a context on a CUDA device (one stream).  Stands in for the
 * construction of an element group + global matrix (ElementListT::NewElement,
 * ElementListT.cpp:649; SolverT::SetGlobalMatrix, SolverT.cpp:1073). */
int tg_create(tg_context** ctx, int device);
int tg_destroy(tg_context* ctx);
/* text of the last error on this context (never NULL) */
const char* tg_last_error(const tg_context* ctx);
/* number of kernels this library launched on the context so far (graph
 * launches count every kernel node they run) */
long long tg_launch_count(const tg_context* ctx);

/* ---- mesh, equations, materials ---------------------------------------- */

/* Uploads the element block: coordinates as structure-of-arrays
 * (x[0..nnd), y[..], z[..]), hex8 connectivity (nel*8, 0-based, reference
 * node order HexahedronT.cpp:23-25) and the equation array (nnd*3).
 * Replaces ContinuumElementT::TakeParameterList geometry set-up
 * (ContinuumElementT.cpp:1330) + ElementBaseT::Equations (ElementBaseT.cpp:196)
 * + GlobalMatrixT::AddEquationSet/Initialize (MSRMatrixT.cpp:35-57). */
int tg_mesh_upload(tg_context* ctx, int nnd, const double* coords_soa, int nel, const int* conn,
                   const int* eqnos);
/* small_strain / total_lagrangian / updated_lagrangian (ElementListT.cpp:738,
 * 752; UpdatedLagrangianT.cpp:94-171: gradients and integration weight of the
 * current configuration, the same weak form as total_lagrangian) */
int tg_element_set(tg_context* ctx, int formulation);
/* strain_displacement option of small_strain (SmallStrainT.cpp:46-91,
 * 327-421): TG_STRAIN_STANDARD, or TG_STRAIN_BBAR for the mean-dilatation
 * B-bar of SolidElementT::Set_B_bar (SolidElementT.cpp:956-1044); ignored by
 * total_lagrangian */
int tg_element_strain_displacement(tg_context* ctx, int option);
/* material of element block `block` (SSSolidMatList3DT.cpp:199-207,
 * FSSolidMatList3DT.cpp:409-415) */
int tg_material_set(tg_context* ctx, int block, int kind, const double* params, int nparams);
/* block index of every element (nel ints); default all 0 */
int tg_element_blocks(tg_context* ctx, const int* block_of_element);

/* Scalar CSR structure over the active equations, rows and columns 0-based
 * equation indices, columns sorted.  upper_only keeps col >= row (the MSR
 * symmetric pattern of MSRBuilderT::GenerateMSR, MSRBuilderT.cpp:134, with
 * the diagonal stored in-row).  Call with row_ptr == NULL to get *nnz. */
int tg_pattern_build(tg_context* ctx, int upper_only, int* row_ptr, int* col_idx, long long* nnz);
/* The same structure computed on the host from the mesh alone (no context,
 * no GPU): the node graph of the connectivity (conn: nel*8, 0-based) that
 * tg_mesh_upload builds, expanded over the equations `eqnos` (nnd*3) exactly
 * as tg_pattern_build does -- MSRBuilderT::GenerateMSR (MSRBuilderT.cpp:134)
 * over GraphT::MakeGraph's node graph.  Call with row_ptr == NULL to get *nnz. */
int tg_pattern_build_host(int nnd, int nel, const int* conn, const int* eqnos, int upper_only, int* row_ptr,
                          int* col_idx, long long* nnz);
/* number of active equations / structural block nonzeros */
int tg_sizes(const tg_context* ctx, int* neq, long long* block_nnz);

/* ---- state, loads -------------------------------------------------------- */

/* nodal displacement (nnd*3), host <-> device */
int tg_set_displacement(tg_context* ctx, const double* u_nodal);
int tg_get_displacement(tg_context* ctx, double* u_nodal);
/* prescribed values at `n` dofs (index node*3+dof) -- FieldT::InitStep /
 * ConsistentKBC (FieldT.cpp:261-322) */
int tg_set_prescribed(tg_context* ctx, int n, const int* dof_index, const double* values);
/* reference nodal external force (nnd*3) and its current load factor:
 * Fext = factor * f (force_BC and traction nodal forces; ScheduleT value) */
int tg_set_external_force(tg_context* ctx, const double* f_nodal);
int tg_set_load_factor(tg_context* ctx, double factor);
/* consistent nodal forces of uniform Cartesian tractions on hex8 facets in
 * the reference configuration (ContinuumElementT::ApplyTractionBC,
 * ContinuumElementT.cpp:514-665); host-only helper, accumulates into f_nodal */
int tg_traction_forces(int nnd, const double* coords_soa, int nel, const int* conn, int nfacets,
                       const int* elem, const int* facet, const double* traction3, double* f_nodal);
/* group iteration number seen by history materials (SolverT fNumIteration,
 * SolverT.cpp:148; read by J2SSKStV::s_ij, J2SSKStV.cpp:69) */
int tg_set_iteration(tg_context* ctx, int iteration);

/* ---- element group: residual and tangent -------------------------------- */

/* R = Fext - Fint(u) on the active equations in FP64 (SolidElementT::
 * ElementRHSDriver, SolidElementT.cpp:1166, + SolverT::AssembleRHS,
 * SolverT.cpp:446).  R_out (neq) may be NULL (kept on the device); norm_out
 * receives ||R||_2 (SolverT::Residual, SolverT.cpp:848). */
int tg_form_residual(tg_context* ctx, double* R_out, double* norm_out);
/* the same in the arithmetic of a Newton driver of the given precision:
 * TG_FP64 as tg_form_residual; TG_MIXED forms the element forces of a
 * total-Lagrangian group whose blocks are all Simo in double-float arithmetic
 * on the FP32 pipe (pairs of floats, 48 significant bits: the error bounds of
 * the FP64 operations with 2^-48 for 2^-53, FP32's exponent range), the
 * other groups in FP64.  The gather, R and its norm stay FP64. */
int tg_form_residual_precision(tg_context* ctx, int precision, double* R_out, double* norm_out);
/* element stiffness + deterministic CSR assembly + preconditioner in the
 * given precision, device resident (SolidElementT::ElementLHSDriver,
 * SolidElementT.cpp:1100 + MSRMatrixT::Assemble, MSRMatrixT.cpp:66) */
int tg_form_tangent(tg_context* ctx, int precision);
/* assembled values of the last tangent on the tg_pattern_build structure
 * (MSRMatrixT::GenerateRCV, MSRMatrixT.cpp:474, for parity dumps) */
int tg_get_tangent_csr(tg_context* ctx, int upper_only, double* vals);
/* element matrices/internal forces of elements [first, first+count) at the
 * current u, FP64 (Ke 24x24 row-major, fint 24), for parity dumps */
int tg_element_dump(tg_context* ctx, int first, int count, double* Ke, double* fint);

/* ---- Krylov solve and update ------------------------------------------- */

/* Solves K du = rhs with (block-)Jacobi PCG on the last tangent.  rhs == NULL
 * uses the device residual of tg_form_residual; du == NULL keeps the result
 * on the device for tg_apply_update.  Replaces GlobalMatrixT::Solve
 * (GlobalMatrixT.cpp:77) with the Krylov solve of the spec path. */
int tg_pcg_solve(tg_context* ctx, const double* rhs, double* du, double rel_tol, int max_it, int precond,
                 int* iterations, double* rel_res);
/* u += du on the active dofs (FEManagerT::Update -> FieldT::ApplyUpdate,
 * FieldT.cpp:531-563) */
int tg_apply_update(tg_context* ctx);

/* Same solve as tg_pcg_solve for callers that cannot allocate device memory
 * (hosts that reserve all device memory up front, or whose request path must
 * not enter the CUDA allocator).  No counterpart in the reference.  rhs and du
 * are DEVICE pointers (neq doubles each).  Allocates nothing: work vectors,
 * partial sums and scalars live in one static device array of 8 MiB held by
 * every GPU that loads the library, which limits the mesh to 32,768 nodes
 * (larger meshes get TG_ERR_CAPACITY).  The first call on a device looks up
 * that array's address, so make it before any stream capture; the address is
 * cached per device for the life of the process and assumes the device's
 * primary context (do not call it after cudaDeviceReset or under another
 * driver context).  All calls on a device share the array: calls that overlap
 * on the GPU race.  The solve reads the full matrix storage: a tangent formed
 * for the push storage alone (tg_pcg_form 3; the default picks it only on
 * meshes of a million block nonzeros and more, above this call's limit) has
 * its full storage assembled, and allocated if it never was, by the first
 * call. */
int tg_pcg_solve_noalloc(tg_context* ctx, const double* rhs_device, double* du_device, double rel_tol, int max_it,
                         int precond, int* iterations, double* rel_res);

/* ---- history ------------------------------------------------------------ */

/* J2 history update after a converged step / reset after a failed one
 * (ContinuumElementT::CloseStep/ResetStep, ContinuumElementT.cpp:148,178;
 * J2SSC0HardeningT::Update/Reset, J2SSC0HardeningT.cpp:204,244) */
int tg_close_step(tg_context* ctx);
int tg_reset_step(tg_context* ctx);
/* Nodal stresses of the .run output at the current state (no history
 * written): SolidElementT::ComputeOutput (SolidElementT.cpp:1540-1570) --
 * Cauchy stress at the integration points extrapolated to the element nodes
 * (HexahedronT::SetExtrapolation, HexahedronT.cpp:2071) and averaged over the
 * elements sharing a node (GroupAverageT.cpp:40-56).  out: nnd*6, Voigt
 * [11,22,33,23,13,12].  Call before tg_close_step, as the reference writes
 * output before the element groups close the step. */
int tg_nodal_stress(tg_context* ctx, double* out);
/* Nodal material output of the small-strain J2 material (alpha, von Mises
 * stress, pressure; J2SSKStV::ComputeOutput, J2SSKStV.cpp:181-207), point
 * values extrapolated and averaged as the stresses; out: nnd*3.  Alpha is
 * zero at points of other materials; von Mises stress and pressure are
 * formed from their stress. */
int tg_nodal_material_output(tg_context* ctx, double* out);
/* per-integration-point flags (nel*8, tg_j2_flag) -- the active set */
int tg_get_active_set(tg_context* ctx, signed char* flags);
/* equivalent plastic strain alpha (nel*8) and plastic strain (nel*8*6) */
int tg_get_j2_state(tg_context* ctx, double* alpha, double* eps_p);

/* ---- Newton (NLSolver) --------------------------------------------------- */

typedef struct tg_newton_params {
  double rel_tol;       /* NLSolver rel_tolerance */
  double abs_tol;       /* NLSolver abs_tolerance */
  double div_tol;       /* NLSolver divergence_tolerance */
  int max_iterations;   /* NLSolver max_iterations */
  int precision;        /* tg_precision: TG_MIXED runs FP32 tangents and Krylov
                           vectors with FP64 scalars, and residuals in the
                           arithmetic of tg_form_residual_precision */
  int precond;          /* tg_precond */
  double lin_rel_tol;   /* inner PCG relative tolerance */
  int lin_max_it;       /* inner PCG iteration cap */
} tg_newton_params;

typedef struct tg_newton_report {
  int iterations;       /* Newton iterations taken */
  int pcg_iterations;   /* total inner PCG iterations */
  double error0;        /* ||R|| at the first residual */
  double error;         /* ||R|| at exit */
  double ms_residual, ms_tangent, ms_solve; /* device time by phase */
} tg_newton_report;

/* One Newton iteration of NLSolver::Solve's loop body (NLSolver.cpp:137-188):
 * tangent + assembly, PCG on the device residual, u += du, iteration + 1, new
 * residual.  *norm receives the new ||R||; *pcg_iterations the inner count. */
int tg_newton_iteration(tg_context* ctx, const tg_newton_params* params, double* norm, int* pcg_iterations);

/* Load-step predictor for prescribed displacements: with u at the last
 * converged state and the step's load factor set, solves
 * K(u) du = R(u) - K(u)[du_p] for the free dofs (du_p = new - current values
 * at the n prescribed dofs), then sets u_p to the new values and u_f += du_f.
 * The reference applies the jump to the prescribed dofs alone before the
 * first residual (FieldT::InitStep, FieldT.cpp:261-322), which is fine for its
 * direct solvers but can leave an indefinite first tangent that breaks CG on
 * fine finite-strain meshes; the converged step is the same either way.
 * History variables are not modified. */
int tg_predict_prescribed(tg_context* ctx, int n, const int* dof_index, const double* values,
                          const tg_newton_params* params, int* pcg_iterations);

/* Restart image of the state a step sequence resumes from (the role of
 * ElementBaseT/ContinuumElementT::WriteRestart/ReadRestart,
 * ElementBaseT.cpp:299-345, and the nodal field's restart data): the
 * displacements and every J2 history array, in a versioned host buffer of
 * tg_state_size bytes.  Loading checks the version and that the mesh sizes
 * and materials match; the caller restores time and load factor. */
int tg_state_size(tg_context* ctx, long long* bytes);
int tg_state_save(tg_context* ctx, void* buffer, long long bytes);
int tg_state_load(tg_context* ctx, const void* buffer, long long bytes);
/* Device snapshot of the displacement and residual, and its restore: the
 * last-converged-state reset of FEManagerT::ResetStep (FEManagerT.cpp:247-262)
 * used for step cuts; also lets a caller repeat an identical iteration. */
int tg_checkpoint(tg_context* ctx);
int tg_rollback(tg_context* ctx);

/* One load step of NLSolver::Solve (NLSolver.cpp:57-262) with its exit test
 * (NLSolver::ExitIteration, NLSolver.cpp:675-755): the caller has applied the
 * step's prescribed values and load factor.  Iteration numbers run from -1
 * as in SolverT::InitStep.  Does not close the step. */
int tg_newton_solve(tg_context* ctx, const tg_newton_params* params, tg_newton_report* report);

/* ---- batched FE^2 micro-solves ------------------------------------------ */

/* A batch of independent RVEs uploaded as one disconnected mesh: RVE r owns
 * nodes [node_off[r], node_off[r+1]) and elements [elem_off[r],
 * elem_off[r+1]) (nseg+1 entries each, host arrays).  No reference
 * counterpart: the reference has no FE^2 driver; each RVE is an ordinary
 * element group with affine prescribed boundary displacement
 * (MappedPeriodicT / kinematic_BC). */
int tg_set_segments(tg_context* ctx, int nseg, const int* node_off, const int* elem_off);
/* ||R_r||_2 of the last residual restricted to each RVE (nseg doubles) */
int tg_segment_residual_norms(tg_context* ctx, double* norms);
/* volume-averaged first Piola stress of each RVE from the last residual
 * evaluation: P_r = (1/V0_r) sum over its element nodes of fint (x) X, equal
 * at equilibrium to the reaction sum sum_{boundary a} f_a (x) X_a; P is
 * nseg*9 row-major (P_iJ), vol0 the reference volumes (NULL: no division) */
int tg_segment_average_stress(tg_context* ctx, const double* vol0, double* P);
/* Newton over the whole batch with NLSolver's exit test (NLSolver.cpp:675-755)
 * applied to every RVE, relative to that RVE's first residual.  With per-RVE
 * Krylov solves (tg_segment_solver, default) every RVE runs its own PCG over
 * the shared matrix stream; an RVE that has converged, diverged, reached the
 * iteration limit or whose PCG broke down is frozen and reported on its own,
 * and the others continue.  seg_rel (nseg, may be NULL) receives each RVE's
 * final relative residual, seg_status (nseg, may be NULL) TG_OK or the RVE's
 * failure code; the return is TG_OK when every RVE converged, else the first
 * RVE failure code (CUDA and argument errors end the batch). */
int tg_newton_solve_segmented(tg_context* ctx, const tg_newton_params* params, tg_newton_report* report,
                              double* seg_rel, int* seg_status);
/* Krylov solves of a segmented batch: per_rve = 1 (default) one PCG per RVE
 * (own scaling, alpha, beta, tolerance relative to its own residual,
 * convergence and breakdown; the solution of an RVE does not depend on the
 * batch it shares, bitwise), per_rve = 0 one PCG over the whole batch (shared
 * scalars, one tolerance).  No reference counterpart (FE^2 batching). */
int tg_segment_solver(tg_context* ctx, int per_rve);
/* Consistent macro tangent dP/dF of every RVE at the current (converged)
 * state, by static condensation onto the prescribed boundary dofs: for each
 * of the nine unit perturbations dF = e_k (x) e_L the interior response
 * K_ii du_i = -K_ib (dF X)_b is solved (PCG with params' precision,
 * preconditioner, lin_rel_tol, lin_max_it) and dP = (1/V0) sum_a (K du)_a (x)
 * X_a.  C is nseg*81 doubles, C[s*81 + (3j+J)*9 + (3k+L)] = dP_jJ/dF_kL;
 * vol0 as for tg_segment_average_stress.  The nine solves run as one
 * multi-vector PCG over the whole batch: each right-hand side stops when its
 * residual norm over the batch falls below lin_rel_tol times its initial
 * norm over the batch (not per RVE), so an RVE's tangent in a batch agrees
 * with the same RVE's tangent computed alone to about lin_rel_tol times the
 * batch's spread of RVE sizes (1e-5 at lin_rel_tol 1e-7 in the tests).  No
 * reference counterpart (FE^2 is not in the reference; the definition is
 * checked against finite differences of the averaged stress). */
int tg_segment_macro_tangent(tg_context* ctx, const tg_newton_params* params, const double* vol0, double* C,
                             int* pcg_iterations);

/* ---- resident templates and composed batch meshes ----------------------
 * No reference counterpart (serving side of the FE^2 batch): a mesh used
 * over and over (one RVE size) is registered once; its pattern, contribution
 * map and tiles stay on the device.  A batch mesh is then composed on the
 * device as the disjoint union of instances, instance i becoming segment i,
 * with the same structure tg_mesh_upload would build for the concatenated
 * mesh.  Templates live until tg_destroy; the context's materials and
 * formulation apply to composed meshes as to uploaded ones. */
/* template: coordinates SoA, 0-based connectivity, equation numbers as for
 * tg_mesh_upload (ascending node-major from 1, prescribed <= 0), element
 * blocks (NULL: all 0); returns its id */
int tg_template_add(tg_context* ctx, int nnd, const double* coords_soa, int nel, const int* conn, const int* eqnos,
                    const int* block_of_element, int* template_id);
/* replaces the mesh by count instances (template ids in order; <= 65535);
 * state (displacement, loads, history) starts at zero */
int tg_mesh_compose(tg_context* ctx, int count, const int* template_ids);
/* every prescribed dof of segment s set to the affine field (F_s - I) X
 * (F: nseg row-major 3x3): the per-node kinematic_BC values an affine
 * (MappedPeriodicT-style) boundary condition would give */
int tg_set_affine_prescribed(tg_context* ctx, const double* F);
/* tg_predict_prescribed with the affine field of tg_set_affine_prescribed as
 * the new prescribed values */
int tg_predict_affine(tg_context* ctx, const double* F, const tg_newton_params* params, int* pcg_iterations);

/* ---- served RVE stream ---------------------------------------------------
 * The request loop of configuration 5 inside the library (no reference
 * counterpart; the serving side of the FE^2 batch, SURVEY's tg_serve_submit /
 * poll).  Requests are RVEs of side n (the benchmark RVE: n x n x n hex8 unit
 * cube, centred spherical inclusion r = 0.3 with ten times the matrix's Simo
 * neo-Hookean moduli, affine boundary displacement (F - I) X).  lanes host
 * threads each own a context (one CUDA stream, resident templates); a free
 * lane takes the arrived requests in order while the batch stays within
 * max_batch, the device-memory budget of every batch in flight
 * (budget_bytes) and the latency target target_batch_ms (predicted batch
 * time from a model fitted to the lanes' own batches; 0 disables it), and
 * solves them with tg_predict_affine + tg_newton_solve_segmented (an RVE that
 * fails fails alone; a batch-level failure is retried request by request).
 * The server is thread-safe: submit and poll from any thread. */
typedef struct tg_server tg_server;
int tg_serve_create(tg_server** server, int device, int lanes, int max_batch, double budget_bytes, int precision,
                    int precond, double rel_tol, double lin_rel_tol, double target_batch_ms);
/* queues one request (F: 3x3 row-major); *request_id numbers requests from 0 */
int tg_serve_submit(tg_server* server, int n, const double* F, long long* request_id);
/* TG_OK with the averaged first Piola stress P (9, row-major), the request's
 * status and its latency (submission to completion, ms) once it is done;
 * 1 while it is pending */
int tg_serve_poll(tg_server* server, long long request_id, double* P, int* status, double* latency_ms);
/* blocks until every submitted request is done */
int tg_serve_wait(tg_server* server);
/* out[0..5]: batches, mean batch size, most lanes busy at once, requests
 * retried alone, predicted ms of a 1,000-element batch, completed requests */
int tg_serve_stats(tg_server* server, double* out, int n);
const char* tg_serve_error(const tg_server* server);
/* finishes queued requests, joins the lanes and releases their contexts */
int tg_serve_destroy(tg_server* server);

/* ---- measurement and tuning helpers (no reference counterpart) ---------- */

/* Shape of the streamed PCG matrix product: row tiles of at most tile_blocks
 * block nonzeros (the unit of the tile-contiguous matrix storage) staged
 * through a ring of `stages` (2 or 3) shared-memory buffers.  Defaults
 * 640 / 2.  Changing the tile size drops the assembled tangent. */
int tg_spmv_config(tg_context* ctx, int tile_blocks, int stages);
/* stage release of the streamed product: 0 (default) every CTA waits at a
 * barrier after each staged tile; 1 each warp releases the stage on an
 * mbarrier and moves on (results are bitwise the same) */
int tg_spmv_release(tg_context* ctx, int per_warp);
/* Recurrences and matrix storage of the single-vector PCG (both
 * precisions).  form = 1: the single-reduction form of Chronopoulos & Gear on
 * the full block storage -- per iteration one product kernel (w = A u, CTA
 * partials of u.w) and
 * one vector kernel whose CTAs each form the iteration's scalars from the
 * partials and run one fused pass over p, s, x, r, u; no grid barrier and no
 * atomic in either kernel; each kernel launches with a programmatic
 * dependency on the one before, so its independent prologue (the product's
 * first matrix tiles, the vector kernel's node vectors) overlaps the
 * previous kernel's last CTAs.  form = 2: the same without programmatic
 * dependencies.  form = 0: the textbook recurrences (product with a
 * last-block reduction; vector update with a grid barrier between its two
 * passes).  All solve the same (block-)Jacobi CG system to the same
 * tolerance; forms 1 and 2 take bitwise the same iterates, form 0 differs
 * from them by rounding.  form = 3: form 1 on the symmetric push storage -- the product streams the upper node blocks only (about 55 % of
 * the full storage's bytes) and stores each off-diagonal block's transposed
 * product in a slot of its lower row, which the vector kernel adds in a fixed
 * order (bitwise repeatable; it differs from form 1 by rounding).  The
 * storage is built on the device on first use after a mesh change and its
 * values are copied from every new assembly.  form = -1 (default): form 3
 * on meshes of at least one million block nonzeros, form 1 below (where the
 * one-time build of the push storage is not amortised).  The symmetric
 * format of tg_spmv_symmetric, segmented batches and the no-allocation entry
 * point use their own kernels. */
int tg_pcg_form(tg_context* ctx, int form);
/* the form the next single-vector solve runs on the current mesh (0..3) */
int tg_pcg_form_get(const tg_context* ctx, int* form);
/* L2 priorities of the streamed matrix.  bytes >= 0: the leading whole
 * tiles within `bytes` of the matrix storage are copied with evict_last
 * (kept in the L2 from one product to the next) and the rest with
 * evict_first (streamed past the PCG vectors, which then stay L2-resident
 * across the iterations); default 16 MiB.  bytes = -1: plain bulk copies.
 * A cache hint only: results are bitwise the same for every value. */
int tg_spmv_l2_keep(tg_context* ctx, long long bytes);
/* Storage the single-vector PCG product streams: on = 0 (default) the full
 * block storage; on = 1, 2, 3 the symmetric format -- the upper node blocks
 * only, each lower block read as the transpose of its upper twin (the
 * symmetric MSR storage of MSRMatrixT.cpp:104-175 applied as in
 * MSRMatrixT::Multx, MSRMatrixT.cpp:385-420), about 0.63 of the full
 * storage's DRAM bytes -- with three launch shapes for the autotuner: 1 two
 * staged tiles at 80 registers, 2 two staged tiles at 64, 3 three staged
 * tiles at 80.  Meshes composed from templates always use the full storage.
 * tile_blocks: upper blocks per streamed tile (0 keeps the current value,
 * default 512).  The results equal the full-storage product up to the order
 * of the FP sums. */
int tg_spmv_symmetric(tg_context* ctx, int on, int tile_blocks);
/* elements per CTA of the tangent kernel: 2, 4 or 8 (default 8); element
 * matrices are bitwise the same for every choice */
int tg_tangent_config(tg_context* ctx, int elems_per_block);
/* the current launch shapes (any pointer may be NULL) */
int tg_tuning_get(const tg_context* ctx, int* tile_blocks, int* stages, int* tangent_elems_per_block);

/* CUDA events on the context stream around caller-defined work */
int tg_timer_start(tg_context* ctx);
int tg_timer_stop(tg_context* ctx, double* ms);
/* average device time of `reps` standalone launches of one hot kernel on the
 * current state: 0 PCG product, 1 PCG vector kernel, each launch timed right
 * after an untimed product launch as in the solve (the kernels of the form
 * the single-vector solve runs, tg_pcg_form), 2 element tangent, 3 assembly,
 * 4 element residual (+gather) in FP64, 5 the same in the mixed form's
 * arithmetic (tg_form_residual_precision) */
int tg_time_kernel(tg_context* ctx, int which, int reps, double* ms_per_launch);

#ifdef __cplusplus
}
#endif
#endif /* TAHOE_GB300_H */
