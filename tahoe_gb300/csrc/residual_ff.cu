// Element internal forces of a total-Lagrangian Simo group in double-float
// arithmetic on the FP32 pipe (TotalLagrangianT::FormKd,
// TotalLagrangianT.cpp:107, with SimoIso3D::s_ij, SimoIso3D.cpp:102-135).
//
// The FP64 residual kernel is bound by GB300's FP64 pipe, which issues at a
// small fraction of the FP32 rate.  Here every value is a double-float
// (ff.cuh: about 48 significant bits, error bounds of the FP64 operations
// with 2^-48 in place of 2^-53), so the forces carry the accuracy a Newton
// residual needs (a relative floor near 1e-14 of the element forces, far
// below the Newton tolerances) at FP32 throughput.  Converting the nodal
// displacements in and the nodal forces out are the only FP64 operations.
//
// One CTA handles 32 elements, one thread per (element, Gauss point), in two
// phases over shared memory:
//   1. thread (e, p): F = I + sum_a u_a (x) dN_a/dX at point p, the cofactor
//      matrix C = J F^-T, J = det F, the Simo Cauchy stress
//      sigma = mu J^-1 dev(J^(-2/3) b) + kappa/2 (J - 1/J) I, and
//      Q_p = w_p det(dX/dxi) sigma C (w J sigma F^-T: the first Piola-Kirchhoff
//      stress times the point weight) into shared memory;
//   2. thread (e, a): f_a = sum_p Q_p dN_a/dX(p), the force on node a as a sum
//      over the element's points (no shuffle reduction).
// The reference-configuration gradients dN_a/dX and w det J come from the
// per-mesh double-float geometry planes (25 planes of nel*8 float2), or for
// a batch mesh composed from resident templates from the templates' planes
// (one pool; each element indexes its template element's points).
#include "ff.cuh"
#include "tg_internal.h"

namespace tg {

namespace {

using ff::dfloat;

constexpr int kFFElems = 32;                 // elements per CTA
constexpr int kFFThreads = kFFElems * 8;     // one thread per (element, point)
constexpr int kGRow = kFFThreads + 1;        // padded row of the gradient tile (conflict-free phase 2)
constexpr size_t kFFSmem = sizeof(float2) * (24 * kGRow + 9 * kFFThreads + kFFThreads * 3);

// three CTAs per SM (80 registers, no spills; 24 warps): measured on the
// 64^3 block at 0.41 ms against 0.46 ms with two CTAs per SM and 0.50 ms with
// one CTA of 64 elements; 16-element CTAs at six per SM time the same
__global__ void __launch_bounds__(kFFThreads, 3)
    residual_tl_ff_kernel(const int* __restrict__ conn, const int8_t* __restrict__ blk, int nel,
                          const double4_32a* __restrict__ u, MatTable mt, const float2* __restrict__ geo,
                          const int* __restrict__ src, long long gstride, double4_32a* __restrict__ fint,
                          int* status) {
  extern __shared__ float2 ff_smem[];
  float2* sG = ff_smem;                    // [24][kGRow]: dN_a/dX_l of every point, row l*8+a
  float2* sQ = sG + 24 * kGRow;            // [9][kFFThreads]: Q of every point
  float2* sU = sQ + 9 * kFFThreads;        // [kFFThreads][3]: u of every (element, node)
  const int tid = threadIdx.x;
  const int le = tid >> 3, p = tid & 7;
  const int e = blockIdx.x * kFFElems + le;
  const bool valid = e < nel;
  // this thread's point in the planes: its own, or its element's in the
  // template pool
  const long long k = valid ? (src ? (long long)src[e] * 8 + p : (long long)e * 8 + p) : 0;

  // stage the gradients (coalesced rows) and the element displacements
#pragma unroll 8
  for (int row = 0; row < 24; ++row) sG[row * kGRow + tid] = valid ? geo[row * gstride + k] : make_float2(0.f, 0.f);
  dfloat wdet = ff::make(0.f, 0.f);
  if (valid) {
    wdet = ff::from_float2(geo[24 * gstride + k]);
    const double4_32a un = u[conn[(long long)e * 8 + p]];
    sU[tid * 3 + 0] = ff::to_float2(ff::from_double(un.x));
    sU[tid * 3 + 1] = ff::to_float2(ff::from_double(un.y));
    sU[tid * 3 + 2] = ff::to_float2(ff::from_double(un.z));
  }
  __syncthreads();

  // phase 1: point p of element e
  dfloat Q[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) Q[i] = ff::make(0.f, 0.f);
  if (valid) {
    ff::Dot H[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) H[i] = ff::dot_zero();
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      const float2* ua = sU + (le * 8 + a) * 3;
      const dfloat u0 = ff::from_float2(ua[0]), u1 = ff::from_float2(ua[1]), u2 = ff::from_float2(ua[2]);
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const dfloat g = ff::from_float2(sG[(j * 8 + a) * kGRow + tid]);
        ff::dot_fma(H[0 * 3 + j], u0, g);
        ff::dot_fma(H[1 * 3 + j], u1, g);
        ff::dot_fma(H[2 * 3 + j], u2, g);
      }
    }
    dfloat F[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) F[i] = ff::dot_value(H[i]);
    F[0] = ff::add(F[0], 1.0f);
    F[4] = ff::add(F[4], 1.0f);
    F[8] = ff::add(F[8], 1.0f);
    // cofactors C_kl = dJ/dF_kl (C = J F^-T)
    auto cof = [&](int a, int b, int c2, int d) {
      ff::Dot t = ff::dot_zero();
      ff::dot_fma(t, F[a], F[b]);
      ff::dot_fms(t, F[c2], F[d]);
      return ff::dot_value(t);
    };
    dfloat C[9];
    C[0] = cof(4, 8, 5, 7);
    C[1] = cof(5, 6, 3, 8);
    C[2] = cof(3, 7, 4, 6);
    C[3] = cof(2, 7, 1, 8);
    C[4] = cof(0, 8, 2, 6);
    C[5] = cof(1, 6, 0, 7);
    C[6] = cof(1, 5, 2, 4);
    C[7] = cof(2, 3, 0, 5);
    C[8] = cof(0, 4, 1, 3);
    ff::Dot tJ = ff::dot_zero();
    ff::dot_fma(tJ, F[0], C[0]);
    ff::dot_fma(tJ, F[1], C[1]);
    ff::dot_fma(tJ, F[2], C[2]);
    const dfloat J = ff::dot_value(tJ);
    // the element's material, read with constant indices from the parameter
    // space (a dynamic index would copy the table to local memory)
    const int bi = blk ? blk[e] : 0;
    double mu = mt.m[0].mu, kappa = mt.m[0].kappa;
#pragma unroll
    for (int b = 1; b < kMaxBlocks; ++b)
      if (bi == b) {
        mu = mt.m[b].mu;
        kappa = mt.m[b].kappa;
      }
    if (!(J.hi > 0.f) || !(wdet.hi > 0.f)) {
      atomicOr(status, kStatusBadJacobian);
    } else {
      const dfloat invJ = ff::rcp(J);
      const dfloat y = ff::rcbrt(J);      // J^(-1/3)
      const dfloat sc = ff::mul(y, y);    // J^(-2/3)
      // b = F F^T, Voigt [11,22,33,23,13,12]
      auto row_dot = [&](int r, int s) {
        ff::Dot t = ff::dot_zero();
        ff::dot_fma(t, F[r * 3 + 0], F[s * 3 + 0]);
        ff::dot_fma(t, F[r * 3 + 1], F[s * 3 + 1]);
        ff::dot_fma(t, F[r * 3 + 2], F[s * 3 + 2]);
        return ff::dot_value(t);
      };
      const dfloat b0 = row_dot(0, 0), b1 = row_dot(1, 1), b2 = row_dot(2, 2);
      const dfloat b3 = row_dot(1, 2), b4 = row_dot(0, 2), b5 = row_dot(0, 1);
      const dfloat mean = ff::mul(ff::add(ff::add(b0, b1), b2), ff::from_double(1.0 / 3.0));
      // sigma = mu J^-1 J^(-2/3) dev(b) + kappa/2 (J - 1/J) I, times w det(dX/dxi)
      const dfloat coef = ff::mul(ff::mul(ff::mul(ff::from_double(mu), invJ), sc), wdet);
      const dfloat dU = ff::mul(ff::mul(ff::sub(J, invJ), ff::from_double(0.5 * kappa)), wdet);
      const dfloat s0 = ff::add(ff::mul(coef, ff::sub(b0, mean)), dU);
      const dfloat s1 = ff::add(ff::mul(coef, ff::sub(b1, mean)), dU);
      const dfloat s2 = ff::add(ff::mul(coef, ff::sub(b2, mean)), dU);
      const dfloat s3 = ff::mul(coef, b3), s4 = ff::mul(coef, b4), s5 = ff::mul(coef, b5);
      const dfloat sm[9] = {s0, s5, s4, s5, s1, s3, s4, s3, s2};
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int l = 0; l < 3; ++l) {
          ff::Dot t = ff::dot_zero();
          ff::dot_fma(t, sm[i * 3 + 0], C[0 * 3 + l]);
          ff::dot_fma(t, sm[i * 3 + 1], C[1 * 3 + l]);
          ff::dot_fma(t, sm[i * 3 + 2], C[2 * 3 + l]);
          Q[i * 3 + l] = ff::dot_value(t);
        }
    }
  }
#pragma unroll
  for (int i = 0; i < 9; ++i) sQ[i * kFFThreads + tid] = ff::to_float2(Q[i]);
  __syncthreads();

  // phase 2: node a = p of element e, summed over the element's points
  if (valid) {
    const int a = p;
    ff::Dot f[3] = {ff::dot_zero(), ff::dot_zero(), ff::dot_zero()};
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int t = le * 8 + q;
      dfloat g[3];
#pragma unroll
      for (int l = 0; l < 3; ++l) g[l] = ff::from_float2(sG[(l * 8 + a) * kGRow + t]);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int l = 0; l < 3; ++l) ff::dot_fma(f[i], ff::from_float2(sQ[(i * 3 + l) * kFFThreads + t]), g[l]);
    }
    fint[(long long)e * 8 + a] = make_double4_32a(ff::to_double(ff::dot_value(f[0])),
                                                  ff::to_double(ff::dot_value(f[1])),
                                                  ff::to_double(ff::dot_value(f[2])), 0.0);
  }
}

}  // namespace

int launch_residual_ff(Context* c, const float2* d_geo_ff, const int* src, long long gstride) {
  static_assert(kFFSmem <= 227 * 1024, "shared memory of the double-float residual");
  if (!ok(c, cudaFuncSetAttribute(residual_tl_ff_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFFSmem),
          "residual_tl_ff_kernel smem"))
    return TG_ERR_CUDA;
  const int grid = (c->nel + kFFElems - 1) / kFFElems;
  residual_tl_ff_kernel<<<grid, kFFThreads, kFFSmem, c->stream>>>(c->d_conn, c->d_block, c->nel, c->d_u, c->mats,
                                                                   d_geo_ff, src, gstride, c->d_fint, c->d_status);
  c->launches++;
  return ok(c, cudaGetLastError(), "residual_tl_ff_kernel") ? TG_OK : TG_ERR_CUDA;
}

}  // namespace tg
