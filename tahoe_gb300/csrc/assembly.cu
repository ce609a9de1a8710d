// Deterministic, atomic-free global assembly on sm_103a.
//
// The global tangent is CSR over 3x3 node blocks (rows = nodes).  Values live
// in tile-contiguous storage: each row tile of the streamed product holds its
// row pointers, column indices and nine value planes (entry k of every block)
// in one contiguous range, so a warp writing consecutive blocks of a row
// issues unit-stride stores and the product streams the matrix sequentially.  Every block gathers
// its element contributions through the destination-sorted map built on the
// host (ascending element order), so the sum order is fixed and the result is
// bitwise repeatable.  Element blocks are stored as three 16-byte (FP32) or
// 32-byte (FP64) aligned rows, so a contribution is three vector loads.  Rows of prescribed dofs are zeroed; restricted to the
// active rows and columns the values are the reference's "active equations
// only" assembly (MSRMatrixT::Assemble, MSRMatrixT.cpp:96-143).  The diagonal block's (block-)Jacobi inverse is
// produced in the same pass (DiagonalMatrixT, DiagonalMatrixT.cpp:91,313):
// minv[0 .. 9*nnd) holds the Jacobi inverse, minv[9*nnd .. 18*nnd) the 3x3
// block-Jacobi inverse, so the solve can pick either, and the Jacobi
// inverse's diagonal follows as one padded 4-vector per node
// (minv_diag_offset).
#include <type_traits>

#include "tg_internal.h"

namespace tg {

namespace {

__device__ __forceinline__ int upper_slot(int a, int b) { return a * 8 - a * (a - 1) / 2 + (b - a); }

// The value of global block j: its element contributions in the
// destination-sorted order, rows of prescribed dofs zeroed (columns are kept,
// so a product with a prescribed-increment vector gives the coupling
// K_fp du_p; PCG vectors are zero at prescribed dofs, so the kept columns
// never enter the solve).
template <typename T>
__device__ __forceinline__ void block_value(int j, uint8_t mI, const int* __restrict__ cptr,
                                            const int* __restrict__ contrib, const T* __restrict__ Ke, T acc[9]) {
  using V4 = typename std::conditional<sizeof(T) == 4, float4, double4_32a>::type;
#pragma unroll
  for (int k = 0; k < 9; ++k) acc[k] = T(0);
  const int c1 = cptr[j + 1];
  for (int c = cptr[j]; c < c1; ++c) {
    const int code = contrib[c];
    const int e = code >> 6, a = (code >> 3) & 7, b = code & 7;
    // the element block's three padded rows: one aligned vector load each
    const V4* src = reinterpret_cast<const V4*>(
        Ke + ((long long)e * kSlots + (a <= b ? upper_slot(a, b) : upper_slot(b, a))) * kKeBlock);
    const V4 k0 = src[0], k1 = src[1], k2 = src[2];
    const T m[9] = {k0.x, k0.y, k0.z, k1.x, k1.y, k1.z, k2.x, k2.y, k2.z};
    if (a <= b) {
#pragma unroll
      for (int k = 0; k < 9; ++k) acc[k] += m[k];
    } else {
#pragma unroll
      for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 3; ++q) acc[p * 3 + q] += m[q * 3 + p];
    }
  }
#pragma unroll
  for (int p = 0; p < 3; ++p)
    if (!((mI >> p) & 1))
#pragma unroll
      for (int q = 0; q < 3; ++q) acc[p * 3 + q] = T(0);
}

// (block-)Jacobi inverse of row I's diagonal block; inactive dofs get
// identity in the inverse's input and zero in its output.
template <typename T>
__device__ __forceinline__ void write_inverses(int I, int nnd, uint8_t mI, const T acc[9], T* __restrict__ minv) {
  using V4 = typename std::conditional<sizeof(T) == 4, float4, double4_32a>::type;
  T A[9];
#pragma unroll
  for (int p = 0; p < 3; ++p)
#pragma unroll
    for (int q = 0; q < 3; ++q)
      A[p * 3 + q] = (((mI >> p) & 1) && ((mI >> q) & 1)) ? acc[p * 3 + q] : (p == q ? T(1) : T(0));
  // Jacobi: inverse diagonal; block-Jacobi: inverse of the 3x3 block
  T B[9], Dg[9];
  const T d = A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
              A[2] * (A[3] * A[7] - A[4] * A[6]);
  const T id = T(1) / d;
  B[0] = (A[4] * A[8] - A[5] * A[7]) * id;
  B[1] = (A[2] * A[7] - A[1] * A[8]) * id;
  B[2] = (A[1] * A[5] - A[2] * A[4]) * id;
  B[3] = (A[5] * A[6] - A[3] * A[8]) * id;
  B[4] = (A[0] * A[8] - A[2] * A[6]) * id;
  B[5] = (A[2] * A[3] - A[0] * A[5]) * id;
  B[6] = (A[3] * A[7] - A[4] * A[6]) * id;
  B[7] = (A[1] * A[6] - A[0] * A[7]) * id;
  B[8] = (A[0] * A[4] - A[1] * A[3]) * id;
#pragma unroll
  for (int k = 0; k < 9; ++k) Dg[k] = T(0);
  Dg[0] = T(1) / A[0];
  Dg[4] = T(1) / A[4];
  Dg[8] = T(1) / A[8];
#pragma unroll
  for (int p = 0; p < 3; ++p)
#pragma unroll
    for (int q = 0; q < 3; ++q)
      if (!((mI >> p) & 1) || !((mI >> q) & 1)) {
        B[p * 3 + q] = T(0);
        Dg[p * 3 + q] = T(0);
      }
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    minv[(long long)I * 9 + k] = Dg[k];
    minv[((long long)nnd + I) * 9 + k] = B[k];
  }
  V4 dv;
  dv.x = Dg[0];
  dv.y = Dg[4];
  dv.z = Dg[8];
  dv.w = T(0);
  reinterpret_cast<V4*>(minv + minv_diag_offset(nnd))[I] = dv;
}

template <typename T>
__global__ void __launch_bounds__(256) assemble_kernel(int nnd, const int* __restrict__ rowptr,
                                                       const int* __restrict__ col,
                                                       const int* __restrict__ cptr,
                                                       const int* __restrict__ contrib, const T* __restrict__ Ke,
                                                       const uint8_t* __restrict__ mask, unsigned char* __restrict__ blob,
                                                       const long long* __restrict__ blob_off,
                                                       const int* __restrict__ row_tile, T* __restrict__ minv) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; I < nnd; I += warps) {
    const uint8_t mI = mask[I];
    const int r0 = rowptr[I], r1 = rowptr[I + 1];
    // this row's value planes in its tile of the tile-contiguous storage
    unsigned char* base = blob + blob_off[row_tile[I]];
    const int* hdr = reinterpret_cast<const int*>(base);
    const int trow0 = hdr[0], tnrows = hdr[1], tnb = hdr[2], ps = hdr[3];
    T* planes = reinterpret_cast<T*>(base + 16 + 4 * ceil4(tnrows + 1) + 4 * ceil4(tnb));
    const int tb0 = rowptr[trow0];
    for (int j = r0 + lane; j < r1; j += 32) {
      T acc[9];
      block_value<T>(j, mI, cptr, contrib, Ke, acc);
#pragma unroll
      for (int k = 0; k < 9; ++k) planes[(long long)k * ps + (j - tb0)] = acc[k];
      if (col[j] == I) write_inverses<T>(I, nnd, mI, acc, minv);
    }
  }
}

// The same for the upper blocks only, written straight into the symmetric
// push storage's tiles (when the solve streams that storage, the full one
// is assembled only on demand): 16 lanes per row (an upper row holds about
// 14 blocks, the row's diagonal first), values bitwise those of the full
// assembly.
template <typename T>
__global__ void __launch_bounds__(256) assemble_upper_kernel(
    int nnd, const int* __restrict__ rowptr, const int* __restrict__ diag, const int* __restrict__ urow,
    const int* __restrict__ tile_row, const int* __restrict__ row_tile, const long long* __restrict__ off,
    unsigned char* __restrict__ pblob, const int* __restrict__ cptr, const int* __restrict__ contrib,
    const T* __restrict__ Ke, const uint8_t* __restrict__ mask, T* __restrict__ minv) {
  const int sub = threadIdx.x & 15;
  const int groups = (gridDim.x * blockDim.x) >> 4;
  for (int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 4; I < nnd; I += groups) {
    const uint8_t mI = mask[I];
    const int t = row_tile[I];
    const int r0 = tile_row[t], nrows = tile_row[t + 1] - r0;
    const int k0 = urow[r0], nb = urow[tile_row[t + 1]] - k0, ps = ceil4(nb);
    T* planes = reinterpret_cast<T*>(pblob + off[t] + 16 + 4 * ceil4(nrows + 1) + 8 * ceil4(nb));
    const int jd = diag[I], je = rowptr[I + 1], kr = urow[I] - k0;
    for (int j = jd + sub; j < je; j += 16) {
      T acc[9];
      block_value<T>(j, mI, cptr, contrib, Ke, acc);
#pragma unroll
      for (int k = 0; k < 9; ++k) planes[(long long)k * ps + kr + (j - jd)] = acc[k];
      if (j == jd) write_inverses<T>(I, nnd, mI, acc, minv);
    }
  }
}

__global__ void set_prescribed_kernel(int n, const int* __restrict__ idx, const double* __restrict__ val,
                                      double4_32a* __restrict__ u) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int node = idx[k] / 3, d = idx[k] % 3;
  double* p = reinterpret_cast<double*>(u + node);
  p[d] = val[k];
}

// u += du / scale (the PCG ran on a scaled right-hand side)
template <typename V>
__global__ void apply_update_kernel(int nnd, const V* __restrict__ du, const PcgScalars* __restrict__ sc,
                                    double4_32a* __restrict__ u) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnd) return;
  const double us = sc->unscale;
  const V d = du[n];
  double4_32a x = u[n];
  x.x += us * (double)d.x;
  x.y += us * (double)d.y;
  x.z += us * (double)d.z;
  u[n] = x;
}

__global__ void xyz_to_nodal_kernel(int nnd, const double* __restrict__ xyz, double4_32a* __restrict__ u) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnd) return;
  u[n] = make_double4_32a(xyz[3LL * n], xyz[3LL * n + 1], xyz[3LL * n + 2], 0.0);
}

__global__ void nodal_to_xyz_kernel(int nnd, const double4_32a* __restrict__ u, double* __restrict__ xyz) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnd) return;
  const double4_32a v = u[n];
  xyz[3LL * n] = v.x;
  xyz[3LL * n + 1] = v.y;
  xyz[3LL * n + 2] = v.z;
}

__global__ void gather_eq_kernel(int neq, const int* __restrict__ slot, const double4_32a* __restrict__ nodal,
                                 double* __restrict__ eq) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= neq) return;
  const int s = slot[k];
  eq[k] = reinterpret_cast<const double*>(nodal)[s];
}

__global__ void scatter_eq_kernel(int neq, const int* __restrict__ slot, const double* __restrict__ eq,
                                  double4_32a* __restrict__ nodal) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= neq) return;
  reinterpret_cast<double*>(nodal)[slot[k]] = eq[k];
}

// Structure part of the tile-contiguous storage: one CTA per tile writes the
// header, the local row pointers and the column indices from the global CSR.
__global__ void blob_structure_kernel(int ntiles, const int* __restrict__ tile_row, const int* __restrict__ rowptr,
                                      const int* __restrict__ col, const long long* __restrict__ off, int elem,
                                      unsigned char* __restrict__ blob) {
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int r0 = tile_row[t], r1 = tile_row[t + 1];
    const int b0 = rowptr[r0], nb = rowptr[r1] - b0, nrows = r1 - r0;
    int* hdr = reinterpret_cast<int*>(blob + off[t]);
    if (threadIdx.x == 0) {
      hdr[0] = r0;
      hdr[1] = nrows;
      hdr[2] = nb;
      hdr[3] = (int)((((long long)nb * elem + 15) / 16 * 16) / elem);
    }
    int* rp = hdr + 4;
    for (int i = threadIdx.x; i <= nrows; i += blockDim.x) rp[i] = rowptr[r0 + i] - b0;
    int* cl = rp + ceil4(nrows + 1);
    for (int j = threadIdx.x; j < nb; j += blockDim.x) cl[j] = col[b0 + j];
  }
}

}  // namespace

int launch_blob_structure(Context* c, int precision) {
  const bool f32 = precision == TG_MIXED;
  const int grid = std::min(c->ntiles, c->num_sms * 16);
  blob_structure_kernel<<<std::max(grid, 1), 128, 0, c->stream>>>(c->ntiles, c->d_tile_row, c->d_rowptr, c->d_col,
                                                                  f32 ? c->d_blob_off32 : c->d_blob_off64,
                                                                  f32 ? 4 : 8, f32 ? c->d_blob32 : c->d_blob64);
  c->launches++;
  return ok(c, cudaGetLastError(), "blob_structure_kernel") ? TG_OK : TG_ERR_CUDA;
}

int launch_assemble(Context* c, int precision) {
  // persistent grid: every CTA resident, so the rows in flight are one
  // contiguous window of the row order and an element block read for one
  // row is still in L2 when the neighbouring rows read it
  const int warps_per_block = 8;
  int per_sm = 0;
  if (!ok(c, precision == TG_MIXED
                 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, assemble_kernel<float>, 256, 0)
                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, assemble_kernel<double>, 256, 0),
          "occupancy"))
    return TG_ERR_CUDA;
  int grid = (c->nnd + warps_per_block - 1) / warps_per_block;
  grid = std::max(1, std::min(grid, c->num_sms * std::max(per_sm, 1)));
  if (precision == TG_MIXED)
    assemble_kernel<float><<<grid, 256, 0, c->stream>>>(c->nnd, c->d_rowptr, c->d_col, c->d_contrib_ptr,
                                                        c->d_contrib, c->d_Ke32, c->d_mask, c->d_blob32,
                                                        c->d_blob_off32, c->d_row_tile, c->d_minv32);
  else
    assemble_kernel<double><<<grid, 256, 0, c->stream>>>(c->nnd, c->d_rowptr, c->d_col, c->d_contrib_ptr,
                                                         c->d_contrib, c->d_Ke64, c->d_mask, c->d_blob64,
                                                         c->d_blob_off64, c->d_row_tile, c->d_minv64);
  c->launches++;
  return ok(c, cudaGetLastError(), "assemble_kernel") ? TG_OK : TG_ERR_CUDA;
}

// Upper blocks into the push storage (its structure built first); the
// push storage's values are then those of the current tangent.
int launch_assemble_upper(Context* c, int precision) {
  int s = push_structure(c, precision);
  if (s) return s;
  PushStore& ps = c->push;
  const bool f32 = precision == TG_MIXED;
  int per_sm = 0;
  if (!ok(c, f32 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, assemble_upper_kernel<float>, 256, 0)
                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, assemble_upper_kernel<double>, 256, 0),
          "occupancy"))
    return TG_ERR_CUDA;
  const int rows_per_block = 16;
  int grid = (c->nnd + rows_per_block - 1) / rows_per_block;
  grid = std::max(1, std::min(grid, c->num_sms * std::max(per_sm, 1)));
  if (f32)
    assemble_upper_kernel<float><<<grid, 256, 0, c->stream>>>(c->nnd, c->d_rowptr, ps.d_diag, ps.d_urow,
                                                              ps.d_tile_row, ps.d_row_tile, ps.d_off32, ps.d_blob32,
                                                              c->d_contrib_ptr, c->d_contrib, c->d_Ke32, c->d_mask,
                                                              c->d_minv32);
  else
    assemble_upper_kernel<double><<<grid, 256, 0, c->stream>>>(c->nnd, c->d_rowptr, ps.d_diag, ps.d_urow,
                                                               ps.d_tile_row, ps.d_row_tile, ps.d_off64, ps.d_blob64,
                                                               c->d_contrib_ptr, c->d_contrib, c->d_Ke64, c->d_mask,
                                                               c->d_minv64);
  c->launches++;
  return ok(c, cudaGetLastError(), "assemble_upper_kernel") ? TG_OK : TG_ERR_CUDA;
}

// The full storage of the current tangent, assembled from its element
// blocks (still on the device) when the tangent went to the push storage
// only.
int ensure_full_assembly(Context* c) {
  const int precision = c->tangent_precision;
  if (precision != TG_MIXED && precision != TG_FP64) return TG_OK;
  long long& serial = precision == TG_MIXED ? c->full_serial32 : c->full_serial64;
  if (serial == c->tangent_serial) return TG_OK;
  int s = ensure_blob(c, precision);
  if (!s) s = launch_assemble(c, precision);
  if (!s) serial = c->tangent_serial;
  return s;
}

int launch_set_prescribed(Context* c, int n, const int* d_idx, const double* d_val) {
  if (n <= 0) return TG_OK;
  set_prescribed_kernel<<<(n + 255) / 256, 256, 0, c->stream>>>(n, d_idx, d_val, c->d_u);
  c->launches++;
  return ok(c, cudaGetLastError(), "set_prescribed_kernel") ? TG_OK : TG_ERR_CUDA;
}

int launch_apply_update(Context* c) {
  const int grid = (c->nnd + 255) / 256;
  if (c->pcg_vec_precision == TG_MIXED)
    apply_update_kernel<float4><<<grid, 256, 0, c->stream>>>(c->nnd, (const float4*)c->d_x, c->d_pcg, c->d_u);
  else
    apply_update_kernel<double4_32a><<<grid, 256, 0, c->stream>>>(c->nnd, (const double4_32a*)c->d_x, c->d_pcg, c->d_u);
  c->launches++;
  return ok(c, cudaGetLastError(), "apply_update_kernel") ? TG_OK : TG_ERR_CUDA;
}

int launch_xyz_to_nodal(Context* c, const double* d_xyz, double4_32a* d_nodal) {
  xyz_to_nodal_kernel<<<(c->nnd + 255) / 256, 256, 0, c->stream>>>(c->nnd, d_xyz, d_nodal);
  c->launches++;
  return ok(c, cudaGetLastError(), "xyz_to_nodal_kernel") ? TG_OK : TG_ERR_CUDA;
}

int launch_nodal_to_xyz(Context* c, const double4_32a* d_nodal, double* d_xyz) {
  nodal_to_xyz_kernel<<<(c->nnd + 255) / 256, 256, 0, c->stream>>>(c->nnd, d_nodal, d_xyz);
  c->launches++;
  return ok(c, cudaGetLastError(), "nodal_to_xyz_kernel") ? TG_OK : TG_ERR_CUDA;
}

int launch_gather_eq(Context* c, const double4_32a* d_nodal, double* d_eq) {
  if (c->neq == 0) return TG_OK;
  gather_eq_kernel<<<(c->neq + 255) / 256, 256, 0, c->stream>>>(c->neq, c->d_eq_slot, d_nodal, d_eq);
  c->launches++;
  return ok(c, cudaGetLastError(), "gather_eq_kernel") ? TG_OK : TG_ERR_CUDA;
}

int launch_scatter_eq(Context* c, const double* d_eq, double4_32a* d_nodal) {
  if (c->neq == 0) return TG_OK;
  scatter_eq_kernel<<<(c->neq + 255) / 256, 256, 0, c->stream>>>(c->neq, c->d_eq_slot, d_eq, d_nodal);
  c->launches++;
  return ok(c, cudaGetLastError(), "scatter_eq_kernel") ? TG_OK : TG_ERR_CUDA;
}

}  // namespace tg
