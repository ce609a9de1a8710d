"""The Tahoe-side bindings compiled against Tahoe's own headers.

include/tahoe/GPUSolidElementT.h (the element group over SmallStrainT,
TotalLagrangianT and UpdatedLagrangianT) and include/tahoe/GPUCSRMatrixT.h
(the global matrix) are what a maintainer adds to a Tahoe tree.  This test
runs `g++ -fsyntax-only` on a unit that instantiates the element binding for
all three elements and constructs both classes (so neither is abstract),
with the reference's source directories on the include path -- the same
declarations a Tahoe build compiles them against.  It needs the reference
source tree (TAHOE_REFERENCE_DIR, or a checkout named `reference` beside this
repository) and g++; without them it is skipped.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

UNIT = r'''
#include "GPUSolidElementT.h"
#include "GPUCSRMatrixT.h"
#include "SmallStrainT.h"
#include "TotalLagrangianT.h"
#include "UpdatedLagrangianT.h"
namespace Tahoe {
template class GPUSolidElementT<SmallStrainT>;
template class GPUSolidElementT<TotalLagrangianT>;
template class GPUSolidElementT<UpdatedLagrangianT>;
ElementBaseT* make_small(const ElementSupportT& s) { return new GPUSolidElementT<SmallStrainT>(s, TG_SMALL_STRAIN); }
ElementBaseT* make_total(const ElementSupportT& s) {
  return new GPUSolidElementT<TotalLagrangianT>(s, TG_TOTAL_LAGRANGIAN, TG_FP64);
}
ElementBaseT* make_updated(const ElementSupportT& s) {
  return new GPUSolidElementT<UpdatedLagrangianT>(s, TG_UPDATED_LAGRANGIAN);
}
GlobalMatrixT* make_matrix(ostream& out, const CommunicatorT& comm) {
  return new GPUCSRMatrixT(out, 0, comm, nullptr, 1e-4, 20000, TG_PRECOND_JACOBI);
}
}
'''


def _reference():
    for cand in (os.environ.get("TAHOE_REFERENCE_DIR"), os.path.join(os.path.dirname(ROOT), "reference")):
        if cand and os.path.isdir(os.path.join(cand, "tahoe", "src")) and os.path.isdir(os.path.join(cand, "toolbox", "src")):
            return cand
    return None


def test_bindings_compile_against_tahoe_headers(tmp_path):
    ref = _reference()
    if ref is None:
        pytest.skip("no Tahoe source tree to compile the bindings against")
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    incs = []
    for top in (os.path.join(ref, "tahoe", "src"), os.path.join(ref, "toolbox", "src")):
        for d, _, _ in os.walk(top):
            incs.append("-I" + d)
    unit = tmp_path / "bindings.cpp"
    unit.write_text(UNIT)
    cmd = [gxx, "-std=c++11", "-fsyntax-only", "-w", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "include", "tahoe")] + incs + [str(unit)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-4000:]
