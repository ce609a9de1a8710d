// Driver for the reference's own MSR structure builder (MSRBuilderT,
// toolbox/src/graph/MSRBuilderT.cpp), compiled from the reference's sources
// by oracle/build.py into oracle/_ref/ref_msr.  Test infrastructure: it lets
// the sparsity tests compare the library's pattern with the reference's code
// itself, not only with the oracle's restatement of it.
//
// Input (binary, little-endian int32): upper_only, nel, nen, neq, then the
// nel x nen element equation numbers (1-based, < 1 inactive) -- what
// MSRMatrixT::AddEquationSet hands the builder (MSRMatrixT.cpp:53).
// Output (binary int32): length, then the MSR array of
// MSRBuilderT::SetMSRData for active rows 1..neq (MSRMatrixT::SetMSRData,
// MSRMatrixT.cpp:633-649): neq+1 row pointers into the off-diagonal
// columns, then the 0-based off-diagonal columns of every row, ascending.
#include <cstdio>
#include <vector>

#include "MSRBuilderT.h"
#include "iArray2DT.h"
#include "iArrayT.h"

using namespace Tahoe;

static bool get(FILE* f, void* p, size_t n) { return fread(p, 4, n, f) == n; }

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  FILE* in = fopen(argv[1], "rb");
  if (!in) return 2;
  int hdr[4];
  if (!get(in, hdr, 4)) return 2;
  const int upper = hdr[0], nel = hdr[1], nen = hdr[2], neq = hdr[3];
  iArray2DT eq(nel, nen);
  if (!get(in, eq.Pointer(), (size_t)nel * nen)) return 2;
  fclose(in);
  MSRBuilderT builder(upper != 0);
  builder.AddGroup(eq);
  iArrayT rows(neq);
  for (int i = 0; i < neq; ++i) rows[i] = i + 1;
  iArrayT bindx;
  builder.SetMSRData(rows, bindx);
  FILE* out = fopen(argv[2], "wb");
  if (!out) return 2;
  const int len = bindx.Length();
  fwrite(&len, 4, 1, out);
  fwrite(bindx.Pointer(), 4, (size_t)len, out);
  fclose(out);
  return 0;
}
