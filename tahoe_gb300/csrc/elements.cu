// Element group kernels of the hex8 implicit path on sm_103a.
//
//  * residual_kernel  (FP64): one thread per Gauss point, 8 lanes per element.
//    Kinematics, material stress (with J2 return mapping and history writes)
//    and the element internal force, reduced over the 8 points with an
//    in-register shuffle reduce-scatter so lane a ends with node a's force.
//    SmallStrainT::FormKd (SmallStrainT.cpp:255), TotalLagrangianT::FormKd
//    (TotalLagrangianT.cpp:107).
//  * gather_residual_kernel: R = factor*Fext - sum of element forces per node,
//    in the fixed node->element incidence order (no atomics), fused with the
//    FP64 norm (SolverT::Residual, SolverT.cpp:848).
//  * tangent_kernel<T>: 8 elements per CTA.  64 threads stage per-point
//    gradients, moduli and stress in shared memory; then one thread per
//    upper node-pair block (36 per element) integrates its 3x3 block of
//    B^T c B (+ geometric stiffness for TL) over the 8 points.
//    SmallStrainT::FormStiffness (SmallStrainT.cpp:285), TotalLagrangianT::
//    FormStiffness (TotalLagrangianT.cpp:40), Set_B (SolidElementT.cpp:854).
//
// Conventions: Voigt [11,22,33,23,13,12]; strain vectors hold tensor shear,
// 6x6 moduli act on engineering shear.  Hex8 node/Gauss-point order of
// HexahedronT.cpp:23-25,1540-1548.
#include <cmath>

#include <type_traits>

#include "ff.cuh"
#include "tg_internal.h"

namespace tg {

namespace {

constexpr double kSqrt23 = 0.81649658092772603273;  // sqrt(2/3)
constexpr int kOutPerPoint = 9;  // output pass: stress (6) + J2 material output (3)
constexpr double kYieldTol = 1.0e-10;                // J2SSC0HardeningT.cpp:17
constexpr double kGauss = 0.57735026918962576451;    // 1/sqrt(3)

// node sign patterns of HexahedronT.cpp:23-25
__host__ __device__ constexpr double sr(int a) { return (((a + 1) >> 1) & 1) ? 1.0 : -1.0; }
__host__ __device__ constexpr double ss(int a) { return ((a >> 1) & 1) ? 1.0 : -1.0; }
__host__ __device__ constexpr double st(int a) { return ((a >> 2) & 1) ? 1.0 : -1.0; }

// reference-domain derivatives of N_a at Gauss point ip (ParentDomainT)
template <typename T>
__device__ __forceinline__ void ref_grad(int ip, T dN[3][8]) {
  const T r = T(kGauss) * T(sr(ip)), s = T(kGauss) * T(ss(ip)), t = T(kGauss) * T(st(ip));
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const T fr = T(1) + r * T(sr(a)), fs = T(1) + s * T(ss(a)), ft = T(1) + t * T(st(a));
    dN[0][a] = T(0.125) * T(sr(a)) * fs * ft;
    dN[1][a] = T(0.125) * T(ss(a)) * fr * ft;
    dN[2][a] = T(0.125) * T(st(a)) * fr * fs;
  }
}

template <typename T>
__device__ __forceinline__ T det3(const T A[9]) {
  return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
         A[2] * (A[3] * A[7] - A[4] * A[6]);
}
template <typename T>
__device__ __forceinline__ void inv3(const T A[9], T d, T B[9]) {
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
}

// Jacobian, det and spatial gradients g[l][a] = dN_a/dX_l at one point
// (ParentDomainT::ComputeDNa, ParentDomainT.cpp:426-470).
template <typename T>
__device__ __forceinline__ T point_gradients(const T (*Xe)[3], int ip, T g[3][8]) {
  T dN[3][8];
  ref_grad<T>(ip, dN);
  T J[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      T acc = T(0);
#pragma unroll
      for (int a = 0; a < 8; ++a) acc += Xe[a][i] * dN[k][a];
      J[i * 3 + k] = acc;
    }
  const T d = det3(J);
  T Ji[9];
  inv3(J, d, Ji);
#pragma unroll
  for (int l = 0; l < 3; ++l)
#pragma unroll
    for (int a = 0; a < 8; ++a)
      g[l][a] = Ji[0 * 3 + l] * dN[0][a] + Ji[1 * 3 + l] * dN[1][a] + Ji[2 * 3 + l] * dN[2][a];
  return d;
}

// The same for the current configuration x = X + u (updated Lagrangian):
// gradients dN/dx and det(dx/dxi), no coordinate array formed.
template <typename T>
__device__ __forceinline__ T point_gradients_current(const T (*Xe)[3], const T (*Ue)[3], int ip, T g[3][8]) {
  T dN[3][8];
  ref_grad<T>(ip, dN);
  T J[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      T acc = T(0);
#pragma unroll
      for (int a = 0; a < 8; ++a) acc += (Xe[a][i] + Ue[a][i]) * dN[k][a];
      J[i * 3 + k] = acc;
    }
  const T d = det3(J);
  T Ji[9];
  inv3(J, d, Ji);
#pragma unroll
  for (int l = 0; l < 3; ++l)
#pragma unroll
    for (int a = 0; a < 8; ++a)
      g[l][a] = Ji[0 * 3 + l] * dN[0][a] + Ji[1 * 3 + l] * dN[1][a] + Ji[2 * 3 + l] * dN[2][a];
  return d;
}

template <typename T>
__device__ __forceinline__ void hooke(const double* C, const T e[6], T s[6]) {
#pragma unroll
  for (int i = 0; i < 6; ++i)
    s[i] = T(C[i * 6 + 0]) * e[0] + T(C[i * 6 + 1]) * e[1] + T(C[i * 6 + 2]) * e[2] +
           T(2) * (T(C[i * 6 + 3]) * e[3] + T(C[i * 6 + 4]) * e[4] + T(C[i * 6 + 5]) * e[5]);
}
template <typename T>
__device__ __forceinline__ T sym_dot(const T a[6], const T b[6]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + T(2) * (a[3] * b[3] + a[4] * b[4] + a[5] * b[5]);
}
template <typename T>
__device__ __forceinline__ void deviatoric(const T a[6], T d[6]) {
  const T m = (a[0] + a[1] + a[2]) / T(3);
  d[0] = a[0] - m;
  d[1] = a[1] - m;
  d[2] = a[2] - m;
  d[3] = a[3];
  d[4] = a[4];
  d[5] = a[5];
}

// J = sqrt(det b), 1/J and J^(-2/3) = (det b)^(-1/3) of the Simo model.
// In FP64 without the library's FP64 sqrt, pow and division (GB300 issues
// FP64 at a small fraction of the FP32 rate, and pow is an FP64 log and exp):
// FP32 estimates of (det b)^(-1/2) and (det b)^(-1/3) refined by Newton's
// method on r^-2 = d (r <- r (3 - d r^2) / 2) and y^-3 = d
// (y <- y (4 - d y^3) / 3), two steps each -- the error of an estimate good
// to 2^-24 squares with every step, to FP64 rounding after two.  Outside
// the range of FP32 the library functions are used.  In FP32 the library
// functions throughout.
__device__ __forceinline__ void simo_roots(double d, double& J, double& invJ, double& sc) {
  if (d > 1e-30 && d < 1e30) {
    double r = (double)rsqrtf((float)d);
    r = r * (1.5 - 0.5 * d * r * r);
    r = r * (1.5 - 0.5 * d * r * r);
    double y = (double)rcbrtf((float)d);
    y = y * (4.0 - d * (y * y * y)) * (1.0 / 3.0);
    y = y * (4.0 - d * (y * y * y)) * (1.0 / 3.0);
    invJ = r;
    J = d * r;
    sc = y;
  } else {
    J = sqrt(d);
    invJ = 1.0 / J;
    sc = pow(J, -2.0 / 3.0);
  }
}
__device__ __forceinline__ void simo_roots(float d, float& J, float& invJ, float& sc) {
  J = sqrtf(d);
  invJ = 1.0f / J;
  sc = powf(J, -2.0f / 3.0f);
}

// SimoIso3D Cauchy stress and spatial moduli (SimoIso3D.cpp:16-53,102-135;
// U(J) = kappa/2 (1/2 (J^2-1) - ln J), SimoIso3D.h:88-101).
template <typename T>
__device__ __forceinline__ bool simo(const MatParams& m, const T F[9], T s[6], T* D) {
  T b[6];
  b[0] = F[0] * F[0] + F[1] * F[1] + F[2] * F[2];
  b[1] = F[3] * F[3] + F[4] * F[4] + F[5] * F[5];
  b[2] = F[6] * F[6] + F[7] * F[7] + F[8] * F[8];
  b[3] = F[3] * F[6] + F[4] * F[7] + F[5] * F[8];
  b[4] = F[0] * F[6] + F[1] * F[7] + F[2] * F[8];
  b[5] = F[0] * F[3] + F[1] * F[4] + F[2] * F[5];
  const T detb = b[0] * (b[1] * b[2] - b[3] * b[3]) - b[5] * (b[5] * b[2] - b[3] * b[4]) +
                 b[4] * (b[5] * b[3] - b[1] * b[4]);
  if (!(detb > T(0))) return false;
  T J, invJ, sc;
  simo_roots(detb, J, invJ, sc);
  T bb[6], dev[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) bb[k] = sc * b[k];
  deviatoric(bb, dev);
  const T mu = T(m.mu), kappa = T(m.kappa);
  const T dU = T(0.5) * kappa * (J - invJ);
  const T ddU = T(0.5) * kappa * (T(1) + invJ * invJ);
  const T muJ = mu * invJ;
#pragma unroll
  for (int k = 0; k < 6; ++k) s[k] = muJ * dev[k];
  s[0] += dU;
  s[1] += dU;
  s[2] += dU;
  if (D) {
    const T mubar = mu * (bb[0] + bb[1] + bb[2]) * invJ * T(1.0 / 3.0);
    const T c1 = dU + J * ddU;
    const T c4 = T(-2.0 / 3.0) * mu * invJ;
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        T v = T(0);
        if (i < 3 && j < 3) v += c1 + T(2) * mubar * (i == j ? T(2.0 / 3.0) : T(-1.0 / 3.0));
        if (i == j) v += T(-2) * dU * (i < 3 ? T(1) : T(0.5)) + (i >= 3 ? T(2) * mubar * T(0.5) : T(0));
        const T Ii = i < 3 ? T(1) : T(0), Ij = j < 3 ? T(1) : T(0);
        v += c4 * (dev[i] * Ij + Ii * dev[j]);
        D[i * 6 + j] = v;
      }
  }
  return true;
}

__host__ __device__ constexpr int vgt(int i, int j) {
  return i == j ? i : ((i + j) == 1 ? 5 : ((i + j) == 2 ? 4 : 3));
}

// large_strain_StVenant: S = C:E, sigma = F S F^T / J, c = push-forward(C)/J
// (FDHookeanMatT.cpp s_ij/c_ijkl with FDKStV isotropic C).
template <typename T>
__device__ __forceinline__ bool stvenant(const MatParams& m, const T F[9], T s[6], T* D) {
  T Cg[9];
#pragma unroll
  for (int I = 0; I < 3; ++I)
#pragma unroll
    for (int J = 0; J < 3; ++J) Cg[I * 3 + J] = F[I] * F[J] + F[3 + I] * F[3 + J] + F[6 + I] * F[6 + J];
  T E[6] = {T(0.5) * (Cg[0] - T(1)), T(0.5) * (Cg[4] - T(1)), T(0.5) * (Cg[8] - T(1)),
            T(0.5) * Cg[5],          T(0.5) * Cg[2],          T(0.5) * Cg[1]};
  T S6[6];
  hooke<T>(m.C, E, S6);
  const T S[9] = {S6[0], S6[5], S6[4], S6[5], S6[1], S6[3], S6[4], S6[3], S6[2]};
  const T J = det3(F);
  if (!(J > T(0))) return false;
  T FS[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int K = 0; K < 3; ++K) FS[i * 3 + K] = F[i * 3 + 0] * S[0 * 3 + K] + F[i * 3 + 1] * S[1 * 3 + K] + F[i * 3 + 2] * S[2 * 3 + K];
  T sig[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      sig[i * 3 + j] = (FS[i * 3 + 0] * F[j * 3 + 0] + FS[i * 3 + 1] * F[j * 3 + 1] + FS[i * 3 + 2] * F[j * 3 + 2]) / J;
  s[0] = sig[0]; s[1] = sig[4]; s[2] = sig[8]; s[3] = sig[5]; s[4] = sig[2]; s[5] = sig[1];
  if (D) {
    const int pi[6] = {0, 1, 2, 1, 0, 0}, pj[6] = {0, 1, 2, 2, 2, 1};
    for (int A = 0; A < 6; ++A)
      for (int B = A; B < 6; ++B) {
        const int i = pi[A], j = pj[A], k = pi[B], l = pj[B];
        T acc = T(0);
        for (int I = 0; I < 3; ++I)
          for (int JJ = 0; JJ < 3; ++JJ) {
            const T fij = F[i * 3 + I] * F[j * 3 + JJ];
            for (int K = 0; K < 3; ++K)
              for (int L = 0; L < 3; ++L)
                acc += fij * F[k * 3 + K] * F[l * 3 + L] * T(m.C[vgt(I, JJ) * 6 + vgt(K, L)]);
          }
        D[A * 6 + B] = acc / J;
        D[B * 6 + A] = acc / J;
      }
  }
  return true;
}

// J2 consistent moduli C + ModuliCorrection (J2SSC0HardeningT.cpp:148-176)
template <typename T>
__device__ __forceinline__ void j2_moduli(const MatParams& m, bool plastic, double dgamma, double norm,
                                          const T nh[6], T D[36]) {
#pragma unroll
  for (int k = 0; k < 36; ++k) D[k] = T(m.C[k]);
  if (plastic) {
    const T mu = T(m.mu);
    const T th = T(2.0 * m.mu * dgamma / norm);
    const T tb = T(3.0 / (3.0 + m.hard_a / m.mu)) - th;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) D[i * 6 + j] += T(-2) * mu * th * (i == j ? T(2.0 / 3.0) : T(-1.0 / 3.0));
#pragma unroll
    for (int i = 3; i < 6; ++i) D[i * 6 + i] += T(-2) * mu * th * T(0.5);
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = 0; j < 6; ++j) D[i * 6 + j] += T(-2) * mu * tb * nh[i] * nh[j];
  }
}

// ---------------------------------------------------------------------------
// residual
// ---------------------------------------------------------------------------
constexpr int kResElems = 32;  // elements per CTA (256 threads)

struct J2View {
  int8_t* flags;
  int8_t* alloc;
  double* alpha;
  double* dgamma;
  double* norm;
  double* epsp;
  double* nhat;
  long long nip;
};

__global__ void __launch_bounds__(256) residual_kernel(const double* __restrict__ X, int nnd,
                                                       const int* __restrict__ conn, const int8_t* __restrict__ blk,
                                                       int nel, const double4_32a* __restrict__ u, MatTable mt,
                                                       J2View j2, int iteration, int commit_state,
                                                       double4_32a* __restrict__ fint, int* status,
                                                       double* __restrict__ ip_sig,
                                                       const double* __restrict__ geo,
                                                       const int* __restrict__ geo_src, long long gstride) {
  __shared__ double sX[kResElems][8][3];
  __shared__ double sU[kResElems][8][3];
  const int tid = threadIdx.x;
  const int le = tid >> 3, ip = tid & 7;
  const int e = blockIdx.x * kResElems + le;
  const bool valid = e < nel;
  if (valid) {
    const int n = conn[e * 8 + ip];
    if (!geo || mt.formulation == TG_UPDATED_LAGRANGIAN) {
      sX[le][ip][0] = X[n];
      sX[le][ip][1] = X[nnd + n];
      sX[le][ip][2] = X[2 * nnd + n];
    }
    const double4_32a un = u[n];
    sU[le][ip][0] = un.x;
    sU[le][ip][1] = un.y;
    sU[le][ip][2] = un.z;
  }
  __syncthreads();

  double f[8][3];
#pragma unroll
  for (int a = 0; a < 8; ++a) f[a][0] = f[a][1] = f[a][2] = 0.0;
  bool bad = false;
  const int bi = (valid && blk) ? blk[e] : 0;
  const MatParams& m = mt.m[bi];
  // J2 element-level "allocation" vote must be warp-uniform: evaluate the
  // yield predicate for every lane (invalid lanes vote false).
  bool yield_vote = false;
  double eps[6] = {0, 0, 0, 0, 0, 0};
  double g[3][8];
  double wdet = 0.0;
  if (valid) {
    if (geo) {
      // reference-configuration gradients and w det J, formed once per mesh
      // (or per template of a composed mesh)
      const long long k = (geo_src ? (long long)geo_src[e] : (long long)e) * 8 + ip;
#pragma unroll
      for (int l = 0; l < 3; ++l)
#pragma unroll
        for (int a = 0; a < 8; ++a) g[l][a] = geo[(l * 8 + a) * gstride + k];
      wdet = geo[24 * gstride + k];
    } else {
      wdet = point_gradients<double>(sX[le], ip, g);  // weight 1 (HexahedronT.cpp:1545)
    }
    if (!(wdet > 0.0)) bad = true;
  }
  // B-bar: element-mean shape-function gradients (SmallStrainT::SetMeanGradient,
  // SmallStrainT.cpp:404-421), summed over the element's 8 lanes
  const bool bbar = mt.bbar && mt.formulation == TG_SMALL_STRAIN;  // uniform
  double mean[3][8];
  if (bbar) {
    const bool use = valid && !bad;
    double vol = use ? wdet : 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
      for (int a = 0; a < 8; ++a) mean[d][a] = use ? wdet * g[d][a] : 0.0;
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
      vol += __shfl_xor_sync(0xffffffffu, vol, o);
#pragma unroll
      for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int a = 0; a < 8; ++a) mean[d][a] += __shfl_xor_sync(0xffffffffu, mean[d][a], o);
    }
    const double iv = vol > 0.0 ? 1.0 / vol : 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
      for (int a = 0; a < 8; ++a) mean[d][a] *= iv;
  }
  const bool is_j2 = valid && m.kind == TG_MAT_SS_J2;
  bool j2_alloc = false;
  double alpha_h = 0.0, alpha_out = 0.0;  // history alpha; alpha written by the output pass
  double rel[6] = {0, 0, 0, 0, 0, 0};
  double ftr = 0.0, nr = 0.0;
  const long long gid = (long long)e * 8 + ip;
  if (valid && !bad && mt.formulation == TG_SMALL_STRAIN) {
    double H[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        double acc = 0.0;
#pragma unroll
        for (int a = 0; a < 8; ++a) acc += sU[le][a][i] * g[j][a];
        H[i * 3 + j] = acc;
      }
    eps[0] = H[0];
    eps[1] = H[4];
    eps[2] = H[8];
    eps[3] = 0.5 * (H[5] + H[7]);
    eps[4] = 0.5 * (H[2] + H[6]);
    eps[5] = 0.5 * (H[1] + H[3]);
    if (bbar) {
      // Hughes (4.5.11-16): the point dilatation replaced by the element mean
      double th = 0.0;
#pragma unroll
      for (int a = 0; a < 8; ++a)
        th += mean[0][a] * sU[le][a][0] + mean[1][a] * sU[le][a][1] + mean[2][a] * sU[le][a][2];
      const double dv = (th - (H[0] + H[4] + H[8])) / 3.0;
      eps[0] += dv;
      eps[1] += dv;
      eps[2] += dv;
    }
    if (is_j2) {
      j2_alloc = j2.alloc[e] != 0;
      if (j2_alloc)
#pragma unroll
        for (int k = 0; k < 6; ++k) eps[k] -= j2.epsp[k * j2.nip + gid];
      if (iteration > m.elastic_its - 2) {
        double dev[6];
        deviatoric(eps, dev);
#pragma unroll
        for (int k = 0; k < 6; ++k) rel[k] = 2.0 * m.mu * dev[k];
        nr = sqrt(sym_dot(rel, rel));
        const double alpha = j2_alloc ? j2.alpha[gid] : 0.0;
        alpha_h = alpha;
        ftr = nr - kSqrt23 * (m.hard_a * alpha + m.hard_b);
        yield_vote = ftr > kYieldTol;
      }
    }
  }
  // element-wide OR over the 8 lanes of this element
  const unsigned ballot = __ballot_sync(0xffffffffu, yield_vote);
  const unsigned group = (ballot >> ((threadIdx.x & 31) & ~7)) & 0xffu;

  if (valid && !bad) {
    double s[6];
    if (mt.formulation == TG_SMALL_STRAIN) {
      hooke<double>(m.C, eps, s);  // eps holds the elastic strain here
      if (is_j2 && iteration > m.elastic_its - 2) {
        // J2SSC0HardeningT::StressCorrection (:68-145) + PlasticLoading (:302-346)
        const bool now_alloc = j2_alloc || group != 0u;
        if (now_alloc) {
          const bool plastic = ftr > kYieldTol;
          double dg = 0.0;
          if (plastic) {
            dg = 0.5 * ftr / (m.mu + m.hard_a / 3.0);
#pragma unroll
            for (int k = 0; k < 6; ++k) s[k] += -2.0 * m.mu * dg * (rel[k] / nr);
          }
          // J2SSKStV::ComputeOutput (J2SSKStV.cpp:181-207): alpha with the
          // pending increment of a plastic point
          alpha_out = alpha_h + (plastic ? kSqrt23 * dg : 0.0);
          if (commit_state) {
            j2.flags[gid] = plastic ? (int8_t)TG_J2_PLASTIC : (int8_t)TG_J2_ELASTIC;
            j2.dgamma[gid] = dg;
            if (plastic) {
              j2.norm[gid] = nr;
#pragma unroll
              for (int k = 0; k < 6; ++k) j2.nhat[k * j2.nip + gid] = rel[k] / nr;
            }
            if (!j2_alloc && ip == 0) j2.alloc[e] = 1;
          }
        }
      }
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        f[a][0] = wdet * (g[0][a] * s[0] + g[2][a] * s[4] + g[1][a] * s[5]);
        f[a][1] = wdet * (g[1][a] * s[1] + g[2][a] * s[3] + g[0][a] * s[5]);
        f[a][2] = wdet * (g[2][a] * s[2] + g[1][a] * s[3] + g[0][a] * s[4]);
      }
      if (bbar) {
        // B-bar^T sigma: the normal rows carry (mean_a - grad_a)/3
        const double tr = wdet * (s[0] + s[1] + s[2]) / 3.0;
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
          for (int d = 0; d < 3; ++d) f[a][d] += tr * (mean[d][a] - g[d][a]);
      }
    } else {
      double F[9];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          double acc = (i == j) ? 1.0 : 0.0;
#pragma unroll
          for (int a = 0; a < 8; ++a) acc += sU[le][a][i] * g[j][a];
          F[i * 3 + j] = acc;
        }
      const double J = det3(F);
      bool okm = J > 0.0;
      if (okm) okm = (m.kind == TG_MAT_FS_SIMO) ? simo<double>(m, F, s, nullptr) : stvenant<double>(m, F, s, nullptr);
      const double sm[9] = {s[0], s[5], s[4], s[5], s[1], s[3], s[4], s[3], s[2]};
      if (!okm) {
        bad = true;
      } else if (mt.formulation == TG_UPDATED_LAGRANGIAN) {
        // UpdatedLagrangianT::FormKd (UpdatedLagrangianT.cpp:145-171): the
        // shape functions of the current configuration x = X + u give dN/dx
        // directly; f_a,i = w det(dx/dxi) sigma_ij dN_a/dx_j
        // (the reference gradients are no longer needed: g takes dN/dx)
        const double wc = point_gradients_current<double>(sX[le], sU[le], ip, g);  // weight 1
        if (!(wc > 0.0)) {
          bad = true;
        } else {
#pragma unroll
          for (int a = 0; a < 8; ++a)
#pragma unroll
            for (int i = 0; i < 3; ++i)
              f[a][i] = wc * (sm[i * 3 + 0] * g[0][a] + sm[i * 3 + 1] * g[1][a] + sm[i * 3 + 2] * g[2][a]);
        }
      } else {
        double Fi[9];
        inv3(F, J, Fi);
        const double scale = wdet * J;
        // f_a,i = w J sigma_ij dN_a/dx_j with dN_a/dx = F^-T dN_a/dX:
        // Q = w J sigma F^-T (w times the first Piola-Kirchhoff stress) once
        // per point, then f_a = Q dN_a/dX (72 FP64 FMA instead of 168)
        double Q[9];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int l = 0; l < 3; ++l)
            Q[i * 3 + l] = scale * (sm[i * 3 + 0] * Fi[l * 3 + 0] + sm[i * 3 + 1] * Fi[l * 3 + 1] + sm[i * 3 + 2] * Fi[l * 3 + 2]);
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
          for (int i = 0; i < 3; ++i) f[a][i] = Q[i * 3 + 0] * g[0][a] + Q[i * 3 + 1] * g[1][a] + Q[i * 3 + 2] * g[2][a];
      }
    }
    if (ip_sig) {
      // output pass: the point's Cauchy stress (SolidElementT::ComputeOutput)
      // and the J2 material output (alpha, von Mises, pressure;
      // J2SSKStV::ComputeOutput, J2SSKStV.cpp:181-207)
      double* o = ip_sig + ((long long)e * 8 + ip) * kOutPerPoint;
#pragma unroll
      for (int k = 0; k < 6; ++k) o[k] = bad ? 0.0 : s[k];
      const double p = (s[0] + s[1] + s[2]) / 3.0;
      const double d0 = s[0] - p, d1 = s[1] - p, d2 = s[2] - p;
      double i2 = s[3] * s[3] + s[4] * s[4] + s[5] * s[5] - d0 * d1 - d1 * d2 - d2 * d0;
      i2 = i2 < 0.0 ? 0.0 : i2;
      o[6] = bad ? 0.0 : alpha_out;
      o[7] = bad ? 0.0 : sqrt(3.0 * i2);
      o[8] = bad ? 0.0 : p;
    }
  }
  if (bad) {
    atomicOr(status, kStatusBadJacobian);
#pragma unroll
    for (int a = 0; a < 8; ++a) f[a][0] = f[a][1] = f[a][2] = 0.0;
  }

  // reduce-scatter over the 8 points of the element: lane ip ends with node ip
  double h[4][3];
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const double keep = (ip & 4) ? f[4 + j][i] : f[j][i];
      const double send = (ip & 4) ? f[j][i] : f[4 + j][i];
      h[j][i] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
  double q[2][3];
#pragma unroll
  for (int j = 0; j < 2; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const double keep = (ip & 2) ? h[2 + j][i] : h[j][i];
      const double send = (ip & 2) ? h[j][i] : h[2 + j][i];
      q[j][i] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
    }
  double r[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const double keep = (ip & 1) ? q[1][i] : q[0][i];
    const double send = (ip & 1) ? q[0][i] : q[1][i];
    r[i] = keep + __shfl_xor_sync(0xffffffffu, send, 1);
  }
  if (valid) fint[(long long)e * 8 + ip] = make_double4_32a(r[0], r[1], r[2], 0.0);
}

// R[node] = factor*Fext - sum_k fint[k] over incident (e,a), active dofs only;
// partial sums of R.R reduced with a last-block-done pass (fixed order).
__global__ void __launch_bounds__(256) gather_residual_kernel(
    int nnd, const int* __restrict__ nptr, const int* __restrict__ nlist, const double4_32a* __restrict__ fint,
    const double4_32a* __restrict__ fext, double factor, const uint8_t* __restrict__ mask, double4_32a* __restrict__ R,
    double* partials, ResidScalars* sc) {
  double local = 0.0;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nnd; n += gridDim.x * blockDim.x) {
    const double4_32a fe = fext[n];
    double rx = factor * fe.x, ry = factor * fe.y, rz = factor * fe.z;
    for (int k = nptr[n]; k < nptr[n + 1]; ++k) {
      const double4_32a v = fint[nlist[k]];
      rx -= v.x;
      ry -= v.y;
      rz -= v.z;
    }
    const uint8_t mk = mask[n];
    rx = (mk & 1) ? rx : 0.0;
    ry = (mk & 2) ? ry : 0.0;
    rz = (mk & 4) ? rz : 0.0;
    R[n] = make_double4_32a(rx, ry, rz, 0.0);
    local += rx * rx + ry * ry + rz * rz;
  }
  // block reduction (fixed tree)
  __shared__ double red[256];
  red[threadIdx.x] = local;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  __shared__ bool last;
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = red[0];
    __threadfence();
    const unsigned prev = atomicAdd(&sc->count, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    __threadfence();
    double acc = 0.0;
    for (int b = threadIdx.x; b < gridDim.x; b += blockDim.x) acc += ((volatile double*)partials)[b];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      sc->norm2 = red[0];
      sc->count = 0u;
    }
  }
}

// ---------------------------------------------------------------------------
// tangent
// ---------------------------------------------------------------------------
// elements per CTA (kTanElems by default; 2 and 4 selectable through
// tg_tangent_config); one thread per upper node-pair block of each element
constexpr int kTanElems = 8;

__device__ __forceinline__ void slot_pair(int slot, int& a, int& b) {
  int start = 0;
  a = 0;
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int len = 8 - r;
    if (slot >= start && slot < start + len) {
      a = r;
      b = r + (slot - start);
    }
    start += len;
  }
}

// UL: the updated-Lagrangian gradients and weight (compiled only into the
// instantiation that needs them, so the other formulations keep their
// register budget)
constexpr int kTanH = 21;  // per (point, node): D B_b (18 values) and sigma grad N_b (3)
// Per-element stride of the h_b tile: 64 x kTanH values and 64 bytes, so the
// tiles of consecutive elements start 16 banks apart.  A warp of the slot
// phase holds lanes of two elements (36 slots each); with a stride of a
// multiple of 32 banks, lanes of both reading the same node b collided.
template <typename T>
__host__ __device__ constexpr int tan_h_stride() {
  return 64 * kTanH + 64 / (int)sizeof(T);
}

// CTAs per SM the FP32 tangent is compiled for (72 registers at 8 elements
// per CTA, a few spilled): the per-point phase runs on 64 of the 288 threads
// while the others wait at its barrier, so resident CTAs, whose phases
// interleave, set the throughput.  Measured on the 64^3 block: 0.60 ms at two
// CTAs per SM, 0.49 ms at three; the per-point phase kept in registers (its
// moduli formed in shared memory instead, to avoid the spills: 0.52 ms); 7
// elements per CTA at 80 registers: 0.57 ms.  The FP64 tangent keeps the
// compiler's choice.
template <typename T>
constexpr int kTanMinBlocks = sizeof(T) == 4 ? 3 : 1;

template <typename T, int kTanElems, bool UL>
__global__ void __launch_bounds__(kTanElems * kSlots, kTanMinBlocks<T>) tangent_kernel(const double* __restrict__ X, int nnd,
                                                              const int* __restrict__ conn,
                                                              const int8_t* __restrict__ blk, int nel,
                                                              const double4_32a* __restrict__ u, MatTable mt,
                                                              J2View j2, T* __restrict__ Ke, int* status) {
  __shared__ T sX[kTanElems][8][3];
  __shared__ T sU[kTanElems][8][3];
  // per point spatial gradients; the ninth point row is padding that puts
  // consecutive elements 24 banks apart (see tan_h_stride)
  __shared__ T sG[kTanElems][9][3][8];
  __shared__ T sD[kTanElems][8][36];    // per point moduli (scaled)
  __shared__ T sS[kTanElems][8][6];     // per point Cauchy stress (scaled, TL only)
  __shared__ T sW[kTanElems][8];        // per point w det J (B-bar mean gradients)
  __shared__ T sM[kTanElems][3][8];     // element-mean gradients (B-bar)
  // dynamic: per element (stride tan_h_stride) [8 points][8 nodes][kTanH]
  // per-node products h_b
  extern __shared__ __align__(16) unsigned char tan_dyn[];
  const int tid = threadIdx.x;
  const int e0 = blockIdx.x * kTanElems;

  if (tid < kTanElems * 8) {
    const int le = tid >> 3, a = tid & 7;
    const int e = e0 + le;
    if (e < nel) {
      const int n0 = conn[e * 8];
      const int n = conn[e * 8 + a];
      // local origin at node 0 keeps FP32 coordinate differences accurate
      sX[le][a][0] = T(X[n] - X[n0]);
      sX[le][a][1] = T(X[nnd + n] - X[nnd + n0]);
      sX[le][a][2] = T(X[2 * nnd + n] - X[2 * nnd + n0]);
      const double4_32a un = u[n];
      sU[le][a][0] = T(un.x);
      sU[le][a][1] = T(un.y);
      sU[le][a][2] = T(un.z);
    }
  }
  __syncthreads();
  if (tid < kTanElems * 8) {
    const int le = tid >> 3, ip = tid & 7;
    const int e = e0 + le;
    if (e < nel) {
      const MatParams& m = mt.m[blk ? blk[e] : 0];
      T g[3][8];
      const T detj = point_gradients<T>(sX[le], ip, g);
      T D[36];
      T s[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
      T scale = detj;
      bool okm = detj > T(0);
      if (mt.formulation == TG_SMALL_STRAIN) {
        if (m.kind == TG_MAT_SS_J2) {
          const long long gid = (long long)e * 8 + ip;
          const bool plastic = j2.alloc[e] != 0 && j2.flags[gid] == TG_J2_PLASTIC;
          T nh[6];
#pragma unroll
          for (int k = 0; k < 6; ++k) nh[k] = plastic ? T(j2.nhat[k * j2.nip + gid]) : T(0);
          j2_moduli<T>(m, plastic, plastic ? j2.dgamma[gid] : 0.0, plastic ? j2.norm[gid] : 1.0, nh, D);
        } else {
#pragma unroll
          for (int k = 0; k < 36; ++k) D[k] = T(m.C[k]);
        }
#pragma unroll
        for (int l = 0; l < 3; ++l)
#pragma unroll
          for (int a = 0; a < 8; ++a) sG[le][ip][l][a] = g[l][a];
      } else {
        T F[9];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            T acc = (i == j) ? T(1) : T(0);
#pragma unroll
            for (int a = 0; a < 8; ++a) acc += sU[le][a][i] * g[j][a];
            F[i * 3 + j] = acc;
          }
        const T J = det3(F);
        okm = okm && J > T(0);
        if (okm) okm = (m.kind == TG_MAT_FS_SIMO) ? simo<T>(m, F, s, D) : stvenant<T>(m, F, s, D);
        if (UL && okm) {
          // UpdatedLagrangianT::FormStiffness (UpdatedLagrangianT.cpp:94-142):
          // gradients and integration weight of the current configuration
          // (coordinates relative to node 0: the gradients see differences)
          const T detc = point_gradients_current<T>(sX[le], sU[le], ip, g);
          okm = detc > T(0);
#pragma unroll
          for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int a = 0; a < 8; ++a) sG[le][ip][k][a] = g[k][a];
          scale = detc;
        } else if (okm) {
          T Fi[9];
          inv3(F, J, Fi);
#pragma unroll
          for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int a = 0; a < 8; ++a)
              sG[le][ip][k][a] = g[0][a] * Fi[0 * 3 + k] + g[1][a] * Fi[1 * 3 + k] + g[2][a] * Fi[2 * 3 + k];
          scale = detj * J;
        }
      }
      if (!okm) {
        atomicOr(status, kStatusBadJacobian);
        scale = T(0);
#pragma unroll
        for (int l = 0; l < 3; ++l)
#pragma unroll
          for (int a = 0; a < 8; ++a) sG[le][ip][l][a] = T(0);
#pragma unroll
        for (int k = 0; k < 36; ++k) D[k] = T(0);
      }
#pragma unroll
      for (int k = 0; k < 36; ++k) sD[le][ip][k] = scale * D[k];
#pragma unroll
      for (int k = 0; k < 6; ++k) sS[le][ip][k] = scale * s[k];
      sW[le][ip] = okm ? detj : T(0);
    }
  }
  __syncthreads();
  const bool bbar = mt.bbar && mt.formulation == TG_SMALL_STRAIN;
  if (bbar) {
    // element-mean gradients (SmallStrainT::SetMeanGradient, :404-421)
    if (tid < kTanElems * 8) {
      const int le = tid >> 3, a = tid & 7;
      if (e0 + le < nel) {
        T vol = T(0), m0 = T(0), m1 = T(0), m2 = T(0);
#pragma unroll
        for (int ip = 0; ip < 8; ++ip) {
          const T w = sW[le][ip];
          vol += w;
          m0 += w * sG[le][ip][0][a];
          m1 += w * sG[le][ip][1][a];
          m2 += w * sG[le][ip][2][a];
        }
        const T iv = vol > T(0) ? T(1) / vol : T(0);
        sM[le][0][a] = m0 * iv;
        sM[le][1][a] = m1 * iv;
        sM[le][2][a] = m2 * iv;
      }
    }
    __syncthreads();
  }

  // Per (element, point, node b), once: h_b = D B_b (6 x 3; with the B-bar
  // correction of node b's columns) and the geometric term's sigma grad N_b
  // (3).  Every node-pair slot (a, b) then only contracts with node a's
  // gradients: the h_b a slot used to form for itself are shared by the
  // slots of the same b (54 of the ~93 FMA a slot spent per point).
  const bool tl = mt.formulation != TG_SMALL_STRAIN;  // geometric stiffness (TL and UL)
  T* const sH = reinterpret_cast<T*>(tan_dyn);
  auto h_at = [&](int el, int ip, int b) { return sH + el * tan_h_stride<T>() + (ip * 8 + b) * kTanH; };
  for (int item = tid; item < kTanElems * 64; item += blockDim.x) {
    const int hl = item >> 6, ip = (item >> 3) & 7, b = item & 7;
    if (e0 + hl >= nel) continue;
    const T gb[3] = {sG[hl][ip][0][b], sG[hl][ip][1][b], sG[hl][ip][2][b]};
    const T* D = sD[hl][ip];
    // h[V][j] = sum_n D[V][vgt(j,n)] gb[n]
    T h[6][3];
#pragma unroll
    for (int V = 0; V < 6; ++V)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        h[V][j] = D[V * 6 + vgt(j, 0)] * gb[0] + D[V * 6 + vgt(j, 1)] * gb[1] + D[V * 6 + vgt(j, 2)] * gb[2];
    if (bbar) {
      // B-bar columns: normal rows plus f = (mean - grad)/3 (Hughes 4.5.11-16)
      const T fb[3] = {(sM[hl][0][b] - gb[0]) / T(3), (sM[hl][1][b] - gb[1]) / T(3), (sM[hl][2][b] - gb[2]) / T(3)};
#pragma unroll
      for (int V = 0; V < 6; ++V) {
        const T ds = D[V * 6 + 0] + D[V * 6 + 1] + D[V * 6 + 2];
#pragma unroll
        for (int j = 0; j < 3; ++j) h[V][j] += fb[j] * ds;
      }
    }
    T* out = h_at(hl, ip, b);
#pragma unroll
    for (int V = 0; V < 6; ++V)
#pragma unroll
      for (int j = 0; j < 3; ++j) out[V * 3 + j] = h[V][j];
    if (tl) {
      const T* sp = sS[hl][ip];
      out[18] = sp[0] * gb[0] + sp[5] * gb[1] + sp[4] * gb[2];
      out[19] = sp[5] * gb[0] + sp[1] * gb[1] + sp[3] * gb[2];
      out[20] = sp[4] * gb[0] + sp[3] * gb[1] + sp[2] * gb[2];
    }
  }
  __syncthreads();

  const int le = tid / kSlots, slot = tid - le * kSlots;
  const int e = e0 + le;
  if (e >= nel) return;
  int a, b;
  slot_pair(slot, a, b);
  T K[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) K[k] = T(0);
  for (int ip = 0; ip < 8; ++ip) {
    const T ga[3] = {sG[le][ip][0][a], sG[le][ip][1][a], sG[le][ip][2][a]};
    const T* h = h_at(le, ip, b);
    // K(i,j) += sum_m ga[m] h[vgt(i,m)][j]
    if (bbar) {
      const T fa[3] = {(sM[le][0][a] - ga[0]) / T(3), (sM[le][1][a] - ga[1]) / T(3), (sM[le][2][a] - ga[2]) / T(3)};
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) K[i * 3 + j] += fa[i] * (h[0 * 3 + j] + h[1 * 3 + j] + h[2 * 3 + j]);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        K[i * 3 + j] += ga[0] * h[vgt(i, 0) * 3 + j] + ga[1] * h[vgt(i, 1) * 3 + j] + ga[2] * h[vgt(i, 2) * 3 + j];
    if (tl) {
      const T geo = ga[0] * h[18] + ga[1] * h[19] + ga[2] * h[20];
      K[0] += geo;
      K[4] += geo;
      K[8] += geo;
    }
  }
  // three padded rows, one aligned vector store each
  using V4 = typename std::conditional<sizeof(T) == 4, float4, double4_32a>::type;
  V4* out = reinterpret_cast<V4*>(Ke + ((long long)e * kSlots + slot) * kKeBlock);
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    V4 row;
    row.x = K[p * 3 + 0];
    row.y = K[p * 3 + 1];
    row.z = K[p * 3 + 2];
    row.w = T(0);
    out[p] = row;
  }
}

// J2 history update / reset (J2SSC0HardeningT::Update/Reset, :204-250);
// one thread per element.
__global__ void j2_close_kernel(int nel, J2View j2, int reset) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel || !j2.alloc[e]) return;
  const long long base = (long long)e * 8;
  if (reset) {
    for (int ip = 0; ip < 8; ++ip) j2.flags[base + ip] = TG_J2_RESET;
    return;
  }
  if (j2.flags[base] == TG_J2_RESET) {
    for (int ip = 0; ip < 8; ++ip) j2.flags[base + ip] = TG_J2_ELASTIC;
    return;
  }
  for (int ip = 0; ip < 8; ++ip) {
    const long long gid = base + ip;
    if (j2.flags[gid] == TG_J2_PLASTIC) {
      j2.flags[gid] = TG_J2_RESET;
      const double dg = j2.dgamma[gid];
      j2.alpha[gid] += kSqrt23 * dg;
      for (int k = 0; k < 6; ++k) j2.epsp[k * j2.nip + gid] += dg * j2.nhat[k * j2.nip + gid];
    }
  }
}

J2View j2view(Context* c) {
  J2View v;
  v.flags = c->d_j2_flags;
  v.alloc = c->d_j2_alloc;
  v.alpha = c->d_j2_alpha;
  v.dgamma = c->d_j2_dgamma;
  v.norm = c->d_j2_norm;
  v.epsp = c->d_j2_epsp;
  v.nhat = c->d_j2_nhat;
  v.nip = (long long)c->nel * 8;
  return v;
}

// Reference-configuration shape-function gradients and w det J of every
// point (the element geometry does not change over a mesh's life: the
// residual reads them instead of re-forming Jacobians on the FP64 pipe).
// Formed in FP64 and stored as FP64 planes, or as double-float planes
// (float2 hi, lo) for the double-float residual.
__device__ __forceinline__ void put_geo(double* p, double v) { *p = v; }
__device__ __forceinline__ void put_geo(float2* p, double v) { *p = ff::to_float2(ff::from_double(v)); }

// Planes of `stride` points, this mesh's points from `off` on.
template <typename G>
__global__ void geometry_kernel(const double* __restrict__ X, int nnd, const int* __restrict__ conn, int nel,
                                G* __restrict__ geo, long long stride, long long off) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nip = (long long)nel * 8;
  if (k >= nip) return;
  const long long e = k >> 3;
  const int ip = (int)(k & 7);
  double Xe[8][3];
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const int n = conn[e * 8 + a];
    Xe[a][0] = X[n];
    Xe[a][1] = X[nnd + n];
    Xe[a][2] = X[2 * nnd + n];
  }
  double g[3][8];
  const double d = point_gradients<double>(Xe, ip, g);
#pragma unroll
  for (int l = 0; l < 3; ++l)
#pragma unroll
    for (int a = 0; a < 8; ++a) put_geo(&geo[(l * 8 + a) * stride + off + k], g[l][a]);
  put_geo(&geo[24 * stride + off + k], d);
}

}  // namespace

template <typename G>
int launch_geometry(Context* c, const double* X, int nnd, const int* conn, int nel, G* geo, long long stride,
                    long long off) {
  const long long nip = (long long)nel * 8;
  geometry_kernel<G><<<(unsigned)((nip + 255) / 256), 256, 0, c->stream>>>(X, nnd, conn, nel, geo, stride, off);
  c->launches++;
  return ok(c, cudaGetLastError(), "geometry_kernel") ? TG_OK : TG_ERR_CUDA;
}
template int launch_geometry<float2>(Context*, const double*, int, const int*, int, float2*, long long, long long);
template int launch_geometry<double>(Context*, const double*, int, const int*, int, double*, long long, long long);

namespace {

// the geometry planes of the mesh, formed on first use after a mesh change;
// without room for them the slot stays empty and the caller goes without
template <typename G>
int geometry_planes(Context* c, G*& slot) {
  if (slot) return TG_OK;
  const size_t n = (size_t)c->nel * 8 * kGeoPlanes;
  G* g = nullptr;
  if (cudaMallocAsync((void**)&g, n * sizeof(G), c->stream) == cudaSuccess &&
      cudaStreamSynchronize(c->stream) == cudaSuccess) {
    c->allocations.push_back(g);
    const int s = launch_geometry<G>(c, c->d_X, c->nnd, c->d_conn, c->nel, g, (long long)c->nel * 8, 0);
    if (s) return s;
    slot = g;
  } else {
    cudaGetLastError();
  }
  return TG_OK;
}

// The double-float residual covers the total-Lagrangian Simo group (every
// block Simo); the other formulations and materials keep the FP64 kernel.
bool ff_residual_applies(const Context* c) {
  if (c->mats.formulation != TG_TOTAL_LAGRANGIAN || c->nel <= 0) return false;
  const int nb = c->have_blocks ? c->mats.nblocks : 1;
  for (int b = 0; b < nb; ++b)
    if (c->mats.m[b].kind != TG_MAT_FS_SIMO) return false;
  return true;
}

int residual_impl(Context* c, int commit_state, double* d_ip_sig = nullptr, int arith = kResidualFP64) {
  if (arith == kResidualDoubleFloat && !d_ip_sig && ff_residual_applies(c)) {
    if (c->composed && c->d_elem_src) {
      // a batch mesh reads its templates' planes
      const int s = template_geometry_pool<float2>(c, c->tpl_geo_ff);
      if (s) return s;
      if (c->tpl_geo_ff.d)
        return launch_residual_ff(c, (const float2*)c->tpl_geo_ff.d, c->d_elem_src, c->tpl_geo_ff.elems * 8);
    }
    const int s = geometry_planes(c, c->d_geo_ff);
    if (s) return s;
    if (c->d_geo_ff) return launch_residual_ff(c, c->d_geo_ff, nullptr, (long long)c->nel * 8);
  }
  // a batch mesh reads its templates' planes; without room for the planes
  // the kernel forms the gradients itself (bitwise the same values)
  const double* geo = nullptr;
  const int* geo_src = nullptr;
  long long gstride = (long long)c->nel * 8;
  if (c->composed && c->d_elem_src) {
    const int s = template_geometry_pool<double>(c, c->tpl_geo64);
    if (s) return s;
    if (c->tpl_geo64.d) {
      geo = (const double*)c->tpl_geo64.d;
      geo_src = c->d_elem_src;
      gstride = c->tpl_geo64.elems * 8;
    }
  }
  if (!geo) {
    const int s = geometry_planes(c, c->d_geo);
    if (s) return s;
    geo = c->d_geo;
  }
  const int grid = (c->nel + kResElems - 1) / kResElems;
  residual_kernel<<<grid, 256, 0, c->stream>>>(c->d_X, c->nnd, c->d_conn, c->d_block, c->nel, c->d_u, c->mats,
                                               j2view(c), c->iteration, commit_state, c->d_fint, c->d_status,
                                               d_ip_sig, geo, geo_src, gstride);
  c->launches++;
  return ok(c, cudaGetLastError(), "residual_kernel") ? TG_OK : TG_ERR_CUDA;
}

}  // namespace

int launch_residual_commit(Context* c, int commit, int arith);
int launch_residual(Context* c, int arith) { return launch_residual_commit(c, 1, arith); }
int launch_residual_nocommit(Context* c, int arith) { return launch_residual_commit(c, 0, arith); }

int launch_residual_commit(Context* c, int commit, int arith) {
  int s = residual_impl(c, commit, nullptr, arith);
  if (s) return s;
  const int grid = std::min((c->nnd + 255) / 256, c->partials_cap);
  gather_residual_kernel<<<grid, 256, 0, c->stream>>>(c->nnd, c->d_node_elem_ptr, c->d_node_elem, c->d_fint,
                                                      c->d_fext, c->load_factor, c->d_mask, c->d_R, c->d_partials,
                                                      c->d_resid);
  c->launches++;
  return ok(c, cudaGetLastError(), "gather_residual_kernel") ? TG_OK : TG_ERR_CUDA;
}

namespace {
// Nodal output stress: every incident element's point stresses extrapolated
// to the node with the hex8 smoothing matrix (HexahedronT::SetExtrapolation,
// HexahedronT.cpp:2071-2140: (1 + sqrt3 s_a . t_p)/8 for node signs s_a and
// point signs t_p), averaged over the incident elements (GroupAverageT).
__global__ void nodal_stress_kernel(int nnd, const int* __restrict__ nptr, const int* __restrict__ nlist,
                                    const double* __restrict__ ip_sig, double* __restrict__ out) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnd) return;
  const double r3 = 1.7320508075688772;  // sqrt(3)
  double acc[kOutPerPoint];
#pragma unroll
  for (int c = 0; c < kOutPerPoint; ++c) acc[c] = 0.0;
  const int k0 = nptr[n], k1 = nptr[n + 1];
  for (int k = k0; k < k1; ++k) {
    const int code = nlist[k];
    const long long e = code >> 3;
    const int a = code & 7;
    const int sa0 = (a == 1 || a == 2 || a == 5 || a == 6) ? 1 : -1;
    const int sa1 = (a == 2 || a == 3 || a == 6 || a == 7) ? 1 : -1;
    const int sa2 = a >= 4 ? 1 : -1;
    for (int p = 0; p < 8; ++p) {
      const int sp0 = (p == 1 || p == 2 || p == 5 || p == 6) ? 1 : -1;
      const int sp1 = (p == 2 || p == 3 || p == 6 || p == 7) ? 1 : -1;
      const int sp2 = p >= 4 ? 1 : -1;
      const double w = 0.125 * (1.0 + r3 * (double)(sa0 * sp0 + sa1 * sp1 + sa2 * sp2));
      const double* sg = ip_sig + (e * 8 + p) * kOutPerPoint;
#pragma unroll
      for (int c = 0; c < kOutPerPoint; ++c) acc[c] += w * sg[c];
    }
  }
  const double inv = k1 > k0 ? 1.0 / (double)(k1 - k0) : 0.0;
#pragma unroll
  for (int c = 0; c < kOutPerPoint; ++c) out[(long long)n * kOutPerPoint + c] = acc[c] * inv;
}
}  // namespace

int launch_nodal_stress(Context* c, double* d_ip_sig, double* d_out) {
  int s = residual_impl(c, 0, d_ip_sig);
  if (s) return s;
  nodal_stress_kernel<<<(c->nnd + 255) / 256, 256, 0, c->stream>>>(c->nnd, c->d_node_elem_ptr, c->d_node_elem,
                                                                    d_ip_sig, d_out);
  c->launches++;
  return ok(c, cudaGetLastError(), "nodal_stress_kernel") ? TG_OK : TG_ERR_CUDA;
}

template <typename T, int EPB, bool UL>
void launch_tangent_t(Context* c, T* Ke) {
  const int grid = (c->nel + EPB - 1) / EPB;
  const size_t dyn = (size_t)EPB * tan_h_stride<T>() * sizeof(T);
  // the per-node products exceed the default dynamic shared memory for some
  // shapes; the attribute belongs to the function on the current device
  // (the same value for every caller), set at every launch -- a tangent is
  // formed once per Newton iteration
  cudaFuncSetAttribute(tangent_kernel<T, EPB, UL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
  // three CTAs of 8 elements hold about 190 KB of shared memory
  cudaFuncSetAttribute(tangent_kernel<T, EPB, UL>, cudaFuncAttributePreferredSharedMemoryCarveout,
                       cudaSharedmemCarveoutMaxShared);
  tangent_kernel<T, EPB, UL><<<grid, EPB * kSlots, dyn, c->stream>>>(
      c->d_X, c->nnd, c->d_conn, c->d_block, c->nel, c->d_u, c->mats, j2view(c), Ke, c->d_status);
}

template <int EPB, bool UL>
void launch_tangent_form(Context* c, int precision) {
  if (precision == TG_MIXED)
    launch_tangent_t<float, EPB, UL>(c, c->d_Ke32);
  else
    launch_tangent_t<double, EPB, UL>(c, c->d_Ke64);
}

template <int EPB>
void launch_tangent_epb(Context* c, int precision) {
  if (c->mats.formulation == TG_UPDATED_LAGRANGIAN)
    launch_tangent_form<EPB, true>(c, precision);
  else
    launch_tangent_form<EPB, false>(c, precision);
}

int launch_tangent(Context* c, int precision) {
  switch (c->tangent_epb) {
    case 2: launch_tangent_epb<2>(c, precision); break;
    case 4: launch_tangent_epb<4>(c, precision); break;
    default: launch_tangent_epb<kTanElems>(c, precision); break;
  }
  c->launches++;
  return ok(c, cudaGetLastError(), "tangent_kernel") ? TG_OK : TG_ERR_CUDA;
}

// FP64 element matrices (full 24x24) and forces for a range of elements,
// without committing history (parity dumps).
namespace {
__global__ void expand_ke_kernel(int first, int count, const double* __restrict__ Ke, const double4_32a* __restrict__ fint,
                                 double* __restrict__ outK, double* __restrict__ outF) {
  const int k = blockIdx.x;
  if (k >= count) return;
  const int e = first + k;
  for (int t = threadIdx.x; t < 576; t += blockDim.x) {
    const int p = t / 24, q = t % 24;
    const int a = p / 3, i = p % 3, b = q / 3, j = q % 3;
    const int lo = a < b ? a : b, hi = a < b ? b : a;
    const int slot = lo * 8 - lo * (lo - 1) / 2 + (hi - lo);
    const double* blkp = Ke + ((long long)e * kSlots + slot) * kKeBlock;
    outK[(long long)k * 576 + t] = (a <= b) ? blkp[i * 4 + j] : blkp[j * 4 + i];
  }
  if (threadIdx.x < 24) {
    const int a = threadIdx.x / 3, i = threadIdx.x % 3;
    const double4_32a v = fint[(long long)e * 8 + a];
    outF[(long long)k * 24 + threadIdx.x] = i == 0 ? v.x : (i == 1 ? v.y : v.z);
  }
}
}  // namespace

int launch_element_dump(Context* c, int first, int count, double* dKe, double* dfint) {
  // the FP64 element blocks are re-formed here at the current state: a full
  // storage the current FP64 tangent has not built yet is built first, from
  // that tangent's blocks
  int s = c->tangent_precision == TG_FP64 ? ensure_full_assembly(c) : TG_OK;
  if (!s) s = residual_impl(c, 0);
  if (s) return s;
  s = launch_tangent(c, TG_FP64);
  if (s) return s;
  expand_ke_kernel<<<count, 256, 0, c->stream>>>(first, count, c->d_Ke64, c->d_fint, dKe, dfint);
  c->launches++;
  return ok(c, cudaGetLastError(), "expand_ke_kernel") ? TG_OK : TG_ERR_CUDA;
}

int launch_close_step(Context* c, int reset) {
  if (!c->has_j2) return TG_OK;
  j2_close_kernel<<<(c->nel + 255) / 256, 256, 0, c->stream>>>(c->nel, j2view(c), reset);
  c->launches++;
  return ok(c, cudaGetLastError(), "j2_close_kernel") ? TG_OK : TG_ERR_CUDA;
}

}  // namespace tg
