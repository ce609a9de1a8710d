/* GPUSolidElementT -- a Tahoe element group whose residual and tangent are
 * formed by the GB300 library (include/tahoe_gb300.h).
 *
 * A template over Tahoe's own concrete solid elements (SmallStrainT,
 * TotalLagrangianT, UpdatedLagrangianT): deck parsing, the material list,
 * output and restart stay Tahoe's; the element loops move to the device.
 * Register the three instantiations in ElementListT::NewElement
 * (tahoe/src/elements/ElementListT.cpp:649, beside small_strain :738 and
 * total_lagrangian :752) under the names small_strain_gpu,
 * total_lagrangian_gpu and updated_lagrangian_gpu.  Header-only; the Tahoe
 * build links libtahoe_gb300.so. */
#ifndef TAHOE_GB300_GPU_SOLID_ELEMENT_T_H_
#define TAHOE_GB300_GPU_SOLID_ELEMENT_T_H_

#include <vector>

#include "ElementSupportT.h"
#include "ExceptionT.h"
#include "FieldT.h"
#include "SolidElementT.h"
#include "dArray2DT.h"
#include "dArrayT.h"
#include "iArray2DT.h"
#include "iArrayT.h"
#include "tahoe_gb300.h"

namespace Tahoe {

template <class ElementT>
class GPUSolidElementT : public ElementT {
 public:
  /* formulation: TG_SMALL_STRAIN, TG_TOTAL_LAGRANGIAN or
   * TG_UPDATED_LAGRANGIAN, matching ElementT; precision: TG_MIXED (FP32
   * tangent and PCG, double-float or FP64 residual, tg_form_residual_precision)
   * or TG_FP64 */
  GPUSolidElementT(const ElementSupportT& support, int formulation, int precision = TG_MIXED)
      : ElementT(support), fForm(formulation), fPrecision(precision) {
    if (tg_create(&fCtx, 0) != TG_OK) ExceptionT::GeneralFail("GPUSolidElementT", "no CUDA device");
  }
  virtual ~GPUSolidElementT(void) { tg_destroy(fCtx); }

  /* After ElementT::TakeParameterList: the group's geometry (one hex8 block),
   * the field's equation numbers and the block's material (kind and
   * parameters as tg_material_set takes them, read from the group's
   * material list by the caller). */
  void UploadGroup(int material_kind, const double* params, int nparams) {
    const dArray2DT& X = this->ElementSupport().InitialCoordinates();
    const int nnd = X.MajorDim();
    std::vector<double> soa(3 * (size_t)nnd);
    for (int n = 0; n < nnd; ++n)
      for (int d = 0; d < 3; ++d) soa[(size_t)d * nnd + n] = X(n, d);
    const iArray2DT& conn = *(this->fConnectivities[0]);  // nel x 8, 0-based nodes
    const iArray2DT& eq = this->Field().Equations();      // nnd x 3 equation numbers
    Check(tg_mesh_upload(fCtx, nnd, soa.data(), conn.MajorDim(), conn.Pointer(), eq.Pointer()));
    Check(tg_element_set(fCtx, fForm));
    Check(tg_material_set(fCtx, 0, material_kind, params, nparams));
    // the group's residual covers every active equation of the field
    const int neq = this->Field().NumEquations();
    fR.Dimension(neq);
    fEqAll.Dimension(neq);
    for (int k = 0; k < neq; ++k) fEqAll[k] = k + 1;
  }

  /* SolidElementT::RHSDriver: the whole group's internal forces on the
   * device, in the arithmetic of the group's precision (TG_MIXED: the
   * double-float element forces of a total-Lagrangian Simo group).  No
   * external force is uploaded to the library, so its residual is -Fint;
   * Tahoe's nodal and traction forces are assembled by their own managers as
   * before. */
  virtual void RHSDriver(void) {
    Check(tg_set_iteration(fCtx, this->IterationNumber()));
    double norm = 0.0;
    const int s = tg_form_residual_precision(fCtx, fPrecision, fR.Pointer(), &norm);
    if (s == TG_ERR_BAD_JACOBIAN) ExceptionT::BadJacobianDet("GPUSolidElementT::RHSDriver");
    Check(s);
    this->ElementSupport().AssembleRHS(this->Group(), fR, fEqAll);
  }

  /* SolidElementT::LHSDriver: element stiffness, assembly and the
   * preconditioner stay on the device (GPUCSRMatrixT solves with them) */
  virtual void LHSDriver(GlobalT::SystemTypeT) { Check(tg_form_tangent(fCtx, fPrecision)); }

  virtual void CloseStep(void) {
    ElementT::CloseStep();
    Check(tg_close_step(fCtx));
  }
  virtual GlobalT::RelaxCodeT ResetStep(void) {
    Check(tg_reset_step(fCtx));
    return ElementT::ResetStep();
  }

  tg_context* Context(void) { return fCtx; }

 private:
  void Check(int s) const {
    if (s != TG_OK) ExceptionT::GeneralFail("GPUSolidElementT", "%s", tg_last_error(fCtx));
  }
  tg_context* fCtx = nullptr;
  int fForm, fPrecision;
  dArrayT fR;
  iArrayT fEqAll;
};

}  // namespace Tahoe

#endif
