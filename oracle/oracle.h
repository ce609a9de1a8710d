/*
 * CPU oracle for the Tahoe implicit hex8 solid path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain FP64 C++ restatement of the
 * reference algorithms (shape functions, kinematics, materials, element
 * residual/stiffness, equation numbering, MSR sparsity and assembly, Krylov
 * and Newton solvers).  Only the tests, the smoke check and the CPU-baseline
 * leg of the benchmark may load it; the product library never links it.
 *
 * Parity pin: the oracle is checked against the golden nodal outputs that the
 * reference's own regression suite commits (benchmark_XML level.0/level.1
 * `.run` files, extracted into tests/golden by tests/golden/make_golden.py).
 *
 * Conventions (identical to the reference):
 *   - Voigt order [11,22,33,23,13,12]; strains carry tensor shear components,
 *     the 6x6 moduli act on engineering shear (dSymMatrixT::A_ijkl_B_kl).
 *   - hex8 node order and Gauss points: toolbox/src/geometry/HexahedronT.cpp:23-25,
 *     1540-1548 (8 points at +-1/sqrt(3) in node order, weight 1).
 *   - equation numbers 1-based, node-major / dof-minor, prescribed dofs -1
 *     (tahoe/src/nodes/NodeManagerT.cpp:712-760, FieldT.h:48-50).
 */
#ifndef TAHOE_ORACLE_H
#define TAHOE_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* formulations */
enum { ORC_SMALL_STRAIN = 0, ORC_TOTAL_LAGRANGIAN = 1, ORC_UPDATED_LAGRANGIAN = 2 };

/* material kinds (parameter layout in oracle.cpp: orc_set_material) */
enum {
  ORC_MAT_SS_HOOKEAN = 0,  /* small_strain_StVenant / small_strain_Hookean: p = C(36) col-major */
  ORC_MAT_SS_J2 = 1,       /* small_strain_StVenant_J2: p = {E, nu, a (slope), b (yield)} */
  ORC_MAT_FS_SIMO = 2,     /* Simo_isotropic: p = {mu, kappa} */
  ORC_MAT_FS_STVENANT = 3  /* large_strain_StVenant: p = {E, nu} */
};

/* J2 flags (J2SSC0HardeningT.h:32-34) plus a marker for unallocated cards */
enum { ORC_J2_PLASTIC = 0, ORC_J2_ELASTIC = 1, ORC_J2_RESET = 3, ORC_J2_UNALLOCATED = 7 };

void* orc_model_create(int nnd, const double* X, int nel, const int* conn);
void orc_model_free(void* m);
int orc_set_formulation(void* m, int form);
/* small strain only: 1 = B-bar strain-displacement (SmallStrainT
 * strain_displacement="B-bar", mean dilatation, SmallStrainT.cpp:337-421) */
int orc_set_bbar(void* m, int on);
int orc_set_material(void* m, int block, int kind, const double* p, int np);
int orc_set_element_blocks(void* m, const int* block_of_element);
int orc_set_schedule(void* m, int npts, const double* x, const double* y);
int orc_add_kbc(void* m, int node, int dof, double value, int scheduled);
/* rigid turn of `nodes` about coordinate axis `axis` (0..2) through `point`,
 * theta = rate * t (TorsionKBCT) */
int orc_add_torsion(void* m, int axis, double rate, const double* point, int nnodes, const int* nodes);
int orc_add_force(void* m, int node, int dof, double value);
int orc_add_traction(void* m, int elem, int facet, const double* t3);
int orc_set_threads(void* m, int nthreads);

/* equations: returns number of active equations; eqnos is nnd*3 */
int orc_equations(void* m, int* eqnos);
/* MSR structure (MSRBuilderT::GenerateMSR): bindx[0..n] row starts (offset n+1),
 * then sorted 0-based off-diagonal columns.  Returns length; writes when
 * bindx != NULL and cap is large enough. */
long long orc_msr_pattern(void* m, int upper_only, int* bindx, long long cap);

/* element level (uses the model's material/formulation and J2 state) */
int orc_element(void* m, int e, const double* u_nodal, int iteration, double* Ke, double* fint);

/* global residual (R = Fext - Fint on active eqs) at time t and, when
 * val != NULL, the MSR (upper, symmetric) tangent values aligned with bindx. */
int orc_form(void* m, const double* u_nodal, double t, int iteration, double* R, double* val);

/* MSR symmetric product (MSRMatrixT::Multx). */
int orc_msr_multx(void* m, const double* val, const double* x, double* y);

/* Jacobi PCG on the assembled MSR matrix; returns iterations (<0 on failure). */
int orc_pcg(void* m, const double* val, const double* b, double* x, double rel_tol, int max_it,
            double* rel_res);

/* R = Fext - Fint at the held displacement (kept for orc_newton_iteration). */
int orc_residual(void* m, double t, int iteration, double* norm);
/* One Newton iteration from the held displacement and residual: tangent +
 * MSR assembly, Jacobi CG to lin_tol, u += du, new residual at
 * iteration + 1 (*norm).  times (may be NULL): seconds of the tangent pass,
 * the CG and the residual pass.  The CG runs on orc_set_threads threads. */
int orc_newton_iteration(void* m, double t, int iteration, double lin_tol, int max_it, int* pcg_its, double* norm,
                         double* times);
/* Prescribed-increment predictor to time t: K(u) du_f = R(u) - K(u)[du_p]
 * on the free dofs (Jacobi CG to lin_tol), then u_p = new values, u_f += du_f. */
int orc_predict(void* m, double t, double lin_tol, int max_it, int* pcg_its);

/* Newton (NLSolver) over nsteps load steps with time step dt.
 * solver: 0 dense Cholesky, 1 Jacobi PCG (lin_tol).  u_hist: nsteps*nnd*3
 * nodal displacements after each converged step; its_hist: Newton iterations
 * per step.  Returns 0 on success, step index+1 of the first failure otherwise. */
int orc_run(void* m, int nsteps, double dt, double rel_tol, double abs_tol, int max_its,
            double div_tol, int solver, double lin_tol, double* u_hist, int* its_hist);
/* orc_run inside TimeManagerT's step sequence with load-step cuts (a failed
 * step is reset and retried at half the step, at most max_cuts halvings in
 * force; the step is doubled back after quick_count quick convergences of
 * fewer than quick_iter iterations).  u_hist / its_hist at the original
 * steps k*dt; *cuts_out = cuts made.  0, or the failing original step. */
int orc_run_cuts(void* m, int nsteps, double dt, double rel_tol, double abs_tol, int max_its, double div_tol,
                 int solver, double lin_tol, int max_cuts, int quick_iter, int quick_count, double* u_hist,
                 int* its_hist, int* cuts_out, double* s_hist, double* m_hist);
/* nodal stresses of the .run output (extrapolated from the integration
 * points, averaged over elements; nnd*6, Voigt [11,22,33,23,13,12]) at u with
 * the current history; s_hist of orc_run_cuts holds them per original step */
int orc_nodal_stress(void* m, const double* u, int iteration, double* out);
/* J2 material output (alpha, von Mises, pressure; J2SSKStV::ComputeOutput)
 * extrapolated and averaged the same way (nnd*3); m_hist of orc_run_cuts
 * holds it per original step */
int orc_nodal_material_output(void* m, const double* u, int iteration, double* out);

/* J2 state after the last converged step (nel*8 each; alpha per IP). */
int orc_j2_state(void* m, signed char* flags, double* alpha, double* eps_p);
/* reactions (Fint at every dof, nnd*3) at the current displacement */
int orc_nodal_internal_force(void* m, const double* u_nodal, int iteration, double* f);
/* the displacement currently held by the model (nnd*3) */
int orc_get_u(void* m, double* u);
int orc_set_u(void* m, const double* u);
/* J2 step bookkeeping (exposed for stepwise parity tests) */
int orc_close_step(void* m);

#ifdef __cplusplus
}
#endif
#endif
