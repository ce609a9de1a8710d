/* GPUCSRMatrixT -- a Tahoe global matrix whose solve is the GB300 library's
 * (block-)Jacobi PCG on the tangent a GPUSolidElementT group formed on the
 * device.
 *
 * Register under SolverT::NewSub("matrix_type_choice")
 * (tahoe/src/solvers/SolverT.cpp:577-700) and SolverT::SetGlobalMatrix
 * (:1073-1300), reading linear_tolerance, max_iterations and preconditioner
 * ("jacobi" -> TG_PRECOND_JACOBI, "block_jacobi" -> TG_PRECOND_BLOCK_JACOBI)
 * from the deck's <GPU_CSR_matrix .../> element, and hand it the element
 * group's context (SetContext) once the group is set up.  Element matrices
 * are not assembled here: the library assembles the tangent itself.
 * Header-only; the Tahoe build links libtahoe_gb300.so. */
#ifndef TAHOE_GB300_GPU_CSR_MATRIX_T_H_
#define TAHOE_GB300_GPU_CSR_MATRIX_T_H_

#include "ExceptionT.h"
#include "GlobalMatrixT.h"
#include "dArrayT.h"
#include "tahoe_gb300.h"

namespace Tahoe {

class GPUCSRMatrixT : public GlobalMatrixT {
 public:
  GPUCSRMatrixT(ostream& out, int check_code, const CommunicatorT& comm, tg_context* ctx, double lin_tol,
                int max_it, int precond)
      : GlobalMatrixT(out, check_code, comm), fCtx(ctx), fTol(lin_tol), fMaxIt(max_it), fPrecond(precond) {}
  GPUCSRMatrixT(const GPUCSRMatrixT& source)
      : GlobalMatrixT(source), fCtx(source.fCtx), fTol(source.fTol), fMaxIt(source.fMaxIt),
        fPrecond(source.fPrecond) {}

  void SetContext(tg_context* ctx) { fCtx = ctx; }
  int LastIterations(void) const { return fIterations; }

  /* the structure was uploaded with the group (tg_mesh_upload) */
  virtual void AddEquationSet(const iArray2DT&) {}
  virtual void AddEquationSet(const RaggedArray2DT<int>&) {}
  /* the tangent is assembled on the device (tg_form_tangent) */
  virtual void Assemble(const ElementMatrixT&, const ArrayT<int>&) {}
  virtual void Assemble(const ElementMatrixT&, const ArrayT<int>&, const ArrayT<int>&) {}
  virtual void Assemble(const nArrayT<double>&, const ArrayT<int>&) {}

  virtual EquationNumberScopeT EquationNumberScope(void) const { return kLocal; }
  virtual bool RenumberEquations(void) const { return false; }  // the reference numbering is kept
  virtual GlobalT::SystemTypeT MatrixType(void) const { return GlobalT::kSymmetric; }
  virtual GlobalMatrixT* Clone(void) const { return new GPUCSRMatrixT(*this); }

  virtual void PrintAllPivots(void) const {}
  virtual void PrintZeroPivots(void) const {}
  virtual void PrintLHS(bool) const {}

 protected:
  virtual void Factorize(void) {}
  /* result: right-hand side in, solution out (GlobalMatrixT::Solve) */
  virtual void BackSubstitute(dArrayT& result) {
    if (!fCtx) ExceptionT::GeneralFail("GPUCSRMatrixT::BackSubstitute", "no device context");
    double rr = 0.0;
    const int s = tg_pcg_solve(fCtx, result.Pointer(), result.Pointer(), fTol, fMaxIt, fPrecond, &fIterations, &rr);
    // an iteration limit is reported, not fatal: Newton continues inexactly
    if (s != TG_OK && s != TG_ERR_NOT_CONVERGED)
      ExceptionT::GeneralFail("GPUCSRMatrixT::BackSubstitute", "%s", tg_last_error(fCtx));
  }

 private:
  tg_context* fCtx;
  double fTol;
  int fMaxIt, fPrecond;
  int fIterations = 0;
};

}  // namespace Tahoe

#endif
