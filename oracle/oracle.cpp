/*
 * CPU oracle for the Tahoe implicit hex8 solid path -- TEST INFRASTRUCTURE.
 *
 * A plain FP64 restatement of the reference algorithms, written for clarity
 * rather than speed.  The CUDA library's results are tested against it:
 * only tests, the smoke check and the benchmark's CPU-baseline leg use it.  Each routine
 * names the reference function it restates (paths relative to the Tahoe
 * source tree).
 */
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace {

/* toolbox/src/geometry/HexahedronT.cpp:23-25 */
const double kRa[8] = {-1.0, 1.0, 1.0, -1.0, -1.0, 1.0, 1.0, -1.0};
const double kSa[8] = {-1.0, -1.0, 1.0, 1.0, -1.0, -1.0, 1.0, 1.0};
const double kTa[8] = {-1.0, -1.0, -1.0, -1.0, 1.0, 1.0, 1.0, 1.0};
/* HexahedronT::NodesOnFacet, HexahedronT.cpp:1913-1918 */
const int kFacetNodes[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4},
                               {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}};
const double kSqrt23 = std::sqrt(2.0 / 3.0);
const double kYieldTol = 1.0e-10; /* J2SSC0HardeningT.cpp:17 */

/* Voigt index of tensor pair (i,j): [11,22,33,23,13,12] */
inline int voigt(int i, int j) {
  if (i == j) return i;
  int s = i + j; /* 1:(0,1)->5, 2:(0,2)->4, 3:(1,2)->3 */
  return s == 1 ? 5 : (s == 2 ? 4 : 3);
}

/* reference-domain gradients at the 8 Gauss points:
 * HexahedronT::SetLocalShape (HexahedronT.cpp:1492-1548) + EvaluateShapeFunctions */
struct RefShape {
  double dN[8][3][8]; /* [ip][xi_k][node] */
  double w[8];
  RefShape() {
    const double g = 1.0 / std::sqrt(3.0);
    for (int ip = 0; ip < 8; ++ip) {
      double r = g * kRa[ip], s = g * kSa[ip], t = g * kTa[ip];
      w[ip] = 1.0;
      for (int a = 0; a < 8; ++a) {
        double fr = 1.0 + r * kRa[a], fs = 1.0 + s * kSa[a], ft = 1.0 + t * kTa[a];
        dN[ip][0][a] = 0.125 * kRa[a] * fs * ft;
        dN[ip][1][a] = 0.125 * kSa[a] * fr * ft;
        dN[ip][2][a] = 0.125 * kTa[a] * fr * fs;
      }
    }
  }
};
const RefShape& ref_shape() {
  static RefShape s;
  return s;
}

double det3(const double A[9]) { /* row-major A[i*3+j] */
  return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
         A[2] * (A[3] * A[7] - A[4] * A[6]);
}
void inv3(const double A[9], double d, double B[9]) {
  B[0] = (A[4] * A[8] - A[5] * A[7]) / d;
  B[1] = (A[2] * A[7] - A[1] * A[8]) / d;
  B[2] = (A[1] * A[5] - A[2] * A[4]) / d;
  B[3] = (A[5] * A[6] - A[3] * A[8]) / d;
  B[4] = (A[0] * A[8] - A[2] * A[6]) / d;
  B[5] = (A[2] * A[3] - A[0] * A[5]) / d;
  B[6] = (A[3] * A[7] - A[4] * A[6]) / d;
  B[7] = (A[1] * A[6] - A[0] * A[7]) / d;
  B[8] = (A[0] * A[4] - A[1] * A[3]) / d;
}

/* isotropic 6x6 moduli (IsotropicT::ComputeModuli, IsotropicT.cpp:153-165) */
void iso_moduli(double mu, double lambda, double C[36]) {
  std::fill(C, C + 36, 0.0);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) C[i * 6 + j] = lambda;
  for (int i = 0; i < 3; ++i) C[i * 6 + i] = lambda + 2.0 * mu;
  for (int i = 3; i < 6; ++i) C[i * 6 + i] = mu;
}

/* sigma = C : eps with tensor-shear strain (dSymMatrixT::A_ijkl_B_kl) */
void hooke(const double C[36], const double e[6], double s[6]) {
  for (int i = 0; i < 6; ++i)
    s[i] = C[i * 6 + 0] * e[0] + C[i * 6 + 1] * e[1] + C[i * 6 + 2] * e[2] +
           2.0 * (C[i * 6 + 3] * e[3] + C[i * 6 + 4] * e[4] + C[i * 6 + 5] * e[5]);
}

void deviatoric(const double a[6], double d[6]) {
  double m = (a[0] + a[1] + a[2]) / 3.0;
  d[0] = a[0] - m;
  d[1] = a[1] - m;
  d[2] = a[2] - m;
  d[3] = a[3];
  d[4] = a[4];
  d[5] = a[5];
}
/* dSymMatrixT::ScalarProduct (dSymMatrixT.cpp:304-321) */
double sym_dot(const double a[6], const double b[6]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + 2.0 * (a[3] * b[3] + a[4] * b[4] + a[5] * b[5]);
}

struct Material {
  int kind = ORC_MAT_SS_HOOKEAN;
  double C[36] = {0};
  double mu = 0, kappa = 0, lambda = 0;
  double hard_a = 0, hard_b = 0; /* K(alpha) = a*alpha + b (LinearT) */
  int elastic_its = 0;           /* parameter value; compared as (it > value-2) */
};

/* J2 history per element (ElementCardT layout of J2SSC0HardeningT::LoadData,
 * J2SSC0HardeningT.cpp:277-299): plastic strain, unit normal, beta, internal */
struct J2Card {
  bool allocated = false;
  signed char flags[8];
  double eps_p[8][6];
  double nhat[8][6];
  double alpha[8], norm[8], dgamma[8], ftrial[8];
  void allocate() { /* AllocateElement, J2SSC0HardeningT.cpp:179-200 */
    allocated = true;
    for (int i = 0; i < 8; ++i) {
      flags[i] = ORC_J2_ELASTIC;
      alpha[i] = norm[i] = dgamma[i] = ftrial[i] = 0.0;
      for (int k = 0; k < 6; ++k) eps_p[i][k] = nhat[i][k] = 0.0;
    }
  }
};

/* J2SSC0HardeningT::PlasticLoading for an allocated card (:302-346) */
bool j2_plastic_loading(const Material& m, J2Card& c, int ip, const double e_el[6]) {
  double dev[6], rel[6];
  deviatoric(e_el, dev);
  for (int k = 0; k < 6; ++k) rel[k] = 2.0 * m.mu * dev[k]; /* beta == 0 */
  double f = std::sqrt(sym_dot(rel, rel)) - kSqrt23 * (m.hard_a * c.alpha[ip] + m.hard_b);
  c.ftrial[ip] = f;
  if (f > kYieldTol) {
    double nrm = std::sqrt(sym_dot(rel, rel));
    c.norm[ip] = nrm;
    for (int k = 0; k < 6; ++k) c.nhat[ip][k] = rel[k] / nrm;
    c.flags[ip] = ORC_J2_PLASTIC;
    return true;
  }
  c.flags[ip] = ORC_J2_ELASTIC;
  return false;
}

/* J2SSKStV::s_ij (J2SSKStV.cpp:58-84) with StressCorrection
 * (J2SSC0HardeningT.cpp:68-145), linear hardening branch. */
void j2_stress(const Material& m, J2Card& c, int ip, const double e_tot[6], int iteration,
               double s[6]) {
  double e_el[6];
  for (int k = 0; k < 6; ++k) e_el[k] = c.allocated ? e_tot[k] - c.eps_p[ip][k] : e_tot[k];
  hooke(m.C, e_el, s);
  if (iteration > m.elastic_its - 2) {
    bool plastic;
    if (!c.allocated) {
      double dev[6], rel[6];
      deviatoric(e_el, dev);
      for (int k = 0; k < 6; ++k) rel[k] = 2.0 * m.mu * dev[k];
      plastic = std::sqrt(sym_dot(rel, rel)) - kSqrt23 * m.hard_b > kYieldTol;
      if (plastic) {
        c.allocate();
        j2_plastic_loading(m, c, ip, e_el);
      }
    } else {
      j2_plastic_loading(m, c, ip, e_el);
    }
    if (c.allocated) {
      if (c.ftrial[ip] > kYieldTol) {
        double dg = 0.5 * c.ftrial[ip] / (m.mu + m.hard_a / 3.0);
        c.dgamma[ip] = dg;
        for (int k = 0; k < 6; ++k) s[k] += -2.0 * m.mu * dg * c.nhat[ip][k];
      } else {
        c.dgamma[ip] = 0.0;
      }
    }
  }
}

/* J2SSKStV::c_ijkl = C + ModuliCorrection (J2SSC0HardeningT.cpp:148-176) */
void j2_moduli(const Material& m, const J2Card& c, int ip, double D[36]) {
  std::memcpy(D, m.C, sizeof(double) * 36);
  if (c.allocated && c.flags[ip] == ORC_J2_PLASTIC) {
    double th = 2.0 * m.mu * c.dgamma[ip] / c.norm[ip];
    double tb = 3.0 / (3.0 + m.hard_a / m.mu) - th;
    /* -2 mu th * I_dev (ReducedIndexDeviatoric) */
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) D[i * 6 + j] += -2.0 * m.mu * th * (i == j ? 2.0 / 3.0 : -1.0 / 3.0);
    for (int i = 3; i < 6; ++i) D[i * 6 + i] += -2.0 * m.mu * th * 0.5;
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) D[i * 6 + j] += -2.0 * m.mu * tb * c.nhat[ip][i] * c.nhat[ip][j];
  }
}

/* J2SSC0HardeningT::Update (:204-241) */
void j2_update(J2Card& c) {
  if (!c.allocated) return;
  if (c.flags[0] == ORC_J2_RESET) {
    for (int i = 0; i < 8; ++i) c.flags[i] = ORC_J2_ELASTIC;
    return;
  }
  for (int ip = 0; ip < 8; ++ip)
    if (c.flags[ip] == ORC_J2_PLASTIC) {
      c.flags[ip] = ORC_J2_RESET;
      c.alpha[ip] += kSqrt23 * c.dgamma[ip];
      for (int k = 0; k < 6; ++k) c.eps_p[ip][k] += c.dgamma[ip] * c.nhat[ip][k];
    }
}

/* SimoIso3D::s_ij / c_ijkl (SimoIso3D.cpp:16-53, 102-135; U(J) from SimoIso3D.h:88-101) */
void simo(const Material& m, const double F[9], double s[6], double D[36]) {
  double b[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      b[i * 3 + j] = F[i * 3 + 0] * F[j * 3 + 0] + F[i * 3 + 1] * F[j * 3 + 1] + F[i * 3 + 2] * F[j * 3 + 2];
  double J = std::sqrt(det3(b));
  double sc = std::pow(J, -2.0 / 3.0);
  double bb[6] = {sc * b[0], sc * b[4], sc * b[8], sc * b[5], sc * b[2], sc * b[1]};
  double dU = 0.5 * m.kappa * (J - 1.0 / J);
  double ddU = 0.5 * m.kappa * (1.0 + 1.0 / (J * J));
  double dev[6];
  deviatoric(bb, dev);
  for (int k = 0; k < 6; ++k) s[k] = m.mu / J * dev[k];
  for (int k = 0; k < 3; ++k) s[k] += dU;
  if (D) {
    std::fill(D, D + 36, 0.0);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) D[i * 6 + j] += dU + J * ddU;
    for (int i = 0; i < 6; ++i) D[i * 6 + i] += -2.0 * dU * (i < 3 ? 1.0 : 0.5);
    double mubar = m.mu * (bb[0] + bb[1] + bb[2]) / (J * 3.0);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) D[i * 6 + j] += 2.0 * mubar * (i == j ? 2.0 / 3.0 : -1.0 / 3.0);
    for (int i = 3; i < 6; ++i) D[i * 6 + i] += 2.0 * mubar * 0.5;
    double sd[6];
    for (int k = 0; k < 6; ++k) sd[k] = m.mu * dev[k];
    const double I[6] = {1, 1, 1, 0, 0, 0};
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j)
        D[i * 6 + j] += -4.0 / (J * 3.0) * 0.5 * (sd[i] * I[j] + I[i] * sd[j]);
  }
}

/* FDHookeanMatT::s_ij / c_ijkl with isotropic C (FDHookeanMatT.cpp, FDKStV.cpp):
 * S = C:E, sigma = F S F^T / J, c = push-forward(C) / J */
void stvenant(const Material& m, const double F[9], double s[6], double D[36]) {
  double Cg[9];
  for (int I = 0; I < 3; ++I)
    for (int Jj = 0; Jj < 3; ++Jj)
      Cg[I * 3 + Jj] = F[0 * 3 + I] * F[0 * 3 + Jj] + F[1 * 3 + I] * F[1 * 3 + Jj] + F[2 * 3 + I] * F[2 * 3 + Jj];
  double E[6] = {0.5 * (Cg[0] - 1.0), 0.5 * (Cg[4] - 1.0), 0.5 * (Cg[8] - 1.0), 0.5 * Cg[5], 0.5 * Cg[2], 0.5 * Cg[1]};
  double S6[6];
  hooke(m.C, E, S6);
  double S[9] = {S6[0], S6[5], S6[4], S6[5], S6[1], S6[3], S6[4], S6[3], S6[2]};
  double J = det3(F);
  double sig[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double a = 0;
      for (int I = 0; I < 3; ++I)
        for (int Jj = 0; Jj < 3; ++Jj) a += F[i * 3 + I] * S[I * 3 + Jj] * F[j * 3 + Jj];
      sig[i * 3 + j] = a / J;
    }
  s[0] = sig[0]; s[1] = sig[4]; s[2] = sig[8]; s[3] = sig[5]; s[4] = sig[2]; s[5] = sig[1];
  if (D) {
    const int pi[6] = {0, 1, 2, 1, 0, 0}, pj[6] = {0, 1, 2, 2, 2, 1};
    for (int A = 0; A < 6; ++A)
      for (int B = 0; B < 6; ++B) {
        int i = pi[A], j = pj[A], k = pi[B], l = pj[B];
        double a = 0;
        for (int I = 0; I < 3; ++I)
          for (int Jj = 0; Jj < 3; ++Jj)
            for (int K = 0; K < 3; ++K)
              for (int L = 0; L < 3; ++L)
                a += F[i * 3 + I] * F[j * 3 + Jj] * F[k * 3 + K] * F[l * 3 + L] *
                     m.C[voigt(I, Jj) * 6 + voigt(K, L)];
        D[A * 6 + B] = a / J;
      }
  }
}

struct KBC {
  int node, dof;
  double value;
  bool scheduled;
  int torsion = -1;  /* >= 0: the dof follows torsion controller [torsion] */
};
/* TorsionKBCT (TorsionKBCT.cpp:39-99, 148-180): the nodes turn rigidly about
 * an axis through `point` by theta = rate * t; the two dofs across the axis
 * are prescribed, the one along it is free. */
struct Torsion {
  int axis;
  double rate;
  double point[3];
};
struct Force {
  int node, dof;
  double value;
};
struct Traction {
  int elem, facet;
  double t[3];
};

struct Model {
  int nnd = 0, nel = 0;
  std::vector<double> X;  /* nnd*3 */
  std::vector<int> conn;  /* nel*8 */
  std::vector<int> block; /* nel */
  int form = ORC_SMALL_STRAIN;
  bool bbar = false; /* small strain with B-bar (SmallStrainT kMeanDilBbar) */
  std::vector<Material> mats;
  std::vector<double> sx, sy; /* schedule */
  std::vector<KBC> kbc;
  std::vector<Torsion> torsions;
  std::vector<Force> forces;
  std::vector<Traction> tractions;
  int nthreads = 1;
  /* derived */
  std::vector<int> eqnos; /* nnd*3 */
  int neq = -1;
  std::vector<int> bindx; /* MSR upper (symmetric) */
  std::vector<J2Card> j2;
  std::vector<double> u; /* nnd*3 current */
  std::vector<double> Rcur; /* residual at u (orc_residual / orc_newton_iteration) */
  std::vector<double> Kval; /* MSR values of the last tangent of orc_newton_iteration */

  const Material& mat(int e) const { return mats[block.empty() ? 0 : block[e]]; }
  double schedule(double t) const { /* PiecewiseLinearT::function (:179-188) */
    if (sx.empty()) return 1.0;
    if (t <= sx[0]) return sy[0];
    for (size_t i = 1; i < sx.size(); ++i)
      if (t < sx[i]) return sy[i - 1] + (t - sx[i - 1]) * (sy[i] - sy[i - 1]) / (sx[i] - sx[i - 1]);
    return sy.back();
  }
};

/* FieldT::InitEquations + NodeManagerT::SetEquationNumbers (NodeManagerT.cpp:712-760) */
void set_equations(Model& M) {
  M.eqnos.assign(M.nnd * 3, 0);
  for (const KBC& k : M.kbc) M.eqnos[k.node * 3 + k.dof] = -1;
  int n = 0;
  for (int i = 0; i < M.nnd * 3; ++i)
    if (M.eqnos[i] >= 0) M.eqnos[i] = ++n;
  M.neq = n;
}

/* MSRBuilderT::SetMSRData/GenerateMSR (MSRBuilderT.cpp:16-175) over the
 * equation graph of the element connectivities (GraphT::MakeGraph). */
void build_msr(const Model& M, bool upper, std::vector<int>& bindx) {
  int n = M.neq;
  std::vector<std::vector<int>> adj(n);
  for (int e = 0; e < M.nel; ++e) {
    int eq[24], k = 0;
    for (int a = 0; a < 8; ++a)
      for (int d = 0; d < 3; ++d) eq[k++] = M.eqnos[M.conn[e * 8 + a] * 3 + d];
    for (int i = 0; i < 24; ++i) {
      if (eq[i] <= 0) continue;
      for (int j = 0; j < 24; ++j) {
        if (eq[j] <= 0 || eq[j] == eq[i]) continue;
        if (upper && eq[j] < eq[i]) continue;
        adj[eq[i] - 1].push_back(eq[j] - 1);
      }
    }
  }
  size_t tot = 0;
  for (auto& r : adj) {
    std::sort(r.begin(), r.end());
    r.erase(std::unique(r.begin(), r.end()), r.end());
    tot += r.size();
  }
  bindx.assign(tot + n + 1, 0);
  bindx[0] = n + 1;
  size_t p = n + 1;
  for (int i = 0; i < n; ++i) {
    for (int c : adj[i]) bindx[p++] = c;
    bindx[i + 1] = bindx[i] + (int)adj[i].size();
  }
}

struct ElemOut {
  double Ke[576];
  double fint[24];
  double sig[8][6]; /* Cauchy stress per integration point (residual pass) */
  double mat[8][3]; /* J2 material output per point: alpha, von Mises, pressure */
};

/* element geometry at one IP: ParentDomainT::ComputeDNa (ParentDomainT.cpp:426-470);
 * returns det J, fills dN/dX [3][8]. */
double ip_gradients(const double* Xe, int ip, double dNdx[3][8]) {
  const RefShape& S = ref_shape();
  double Jm[9] = {0};
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) {
      double a = 0;
      for (int n = 0; n < 8; ++n) a += Xe[n * 3 + i] * S.dN[ip][k][n];
      Jm[i * 3 + k] = a;
    }
  double d = det3(Jm);
  if (!(d > 0.0)) return d;
  double Ji[9];
  inv3(Jm, d, Ji);
  for (int l = 0; l < 3; ++l)
    for (int n = 0; n < 8; ++n)
      dNdx[l][n] = Ji[0 * 3 + l] * S.dN[ip][0][n] + Ji[1 * 3 + l] * S.dN[ip][1][n] + Ji[2 * 3 + l] * S.dN[ip][2][n];
  return d;
}

/* B^T D B accumulation with B from SolidElementT::Set_B (SolidElementT.cpp:889-918) */
/* strain-displacement matrix, Voigt rows [11,22,33,23,13,12] with
 * engineering shear (SolidElementT::Set_B, SolidElementT.cpp:854-920) */
void set_b(const double g[3][8], double B[6][24]) {
  std::memset(B, 0, sizeof(double) * 6 * 24);
  for (int a = 0; a < 8; ++a) {
    B[0][3 * a] = g[0][a];
    B[4][3 * a] = g[2][a];
    B[5][3 * a] = g[1][a];
    B[1][3 * a + 1] = g[1][a];
    B[3][3 * a + 1] = g[2][a];
    B[5][3 * a + 1] = g[0][a];
    B[2][3 * a + 2] = g[2][a];
    B[3][3 * a + 2] = g[1][a];
    B[4][3 * a + 2] = g[0][a];
  }
}

/* B-bar of Hughes (4.5.11-16) (SolidElementT::Set_B_bar,
 * SolidElementT.cpp:956-1044): the normal rows of node a's columns take
 * (mean_a - grad_a)/3 added, the element-mean dilatation replacing the
 * point dilatation. */
void set_b_bar(const double g[3][8], const double mean[3][8], double B[6][24]) {
  set_b(g, B);
  for (int a = 0; a < 8; ++a)
    for (int d = 0; d < 3; ++d) {
      const double f = (mean[d][a] - g[d][a]) / 3.0;
      for (int r = 0; r < 3; ++r) B[r][3 * a + d] += f;
    }
}

void add_btdb_b(const double B[6][24], const double D[36], double scale, double* Ke) {
  double DB[6][24];
  for (int i = 0; i < 6; ++i)
    for (int q = 0; q < 24; ++q) {
      double a = 0;
      for (int k = 0; k < 6; ++k) a += D[i * 6 + k] * B[k][q];
      DB[i][q] = a;
    }
  for (int p = 0; p < 24; ++p)
    for (int q = 0; q < 24; ++q) {
      double a = 0;
      for (int k = 0; k < 6; ++k) a += B[k][p] * DB[k][q];
      Ke[p * 24 + q] += scale * a;
    }
}

void add_btdb(const double g[3][8], const double D[36], double scale, double* Ke) {
  double B[6][24];
  set_b(g, B);
  add_btdb_b(B, D, scale, Ke);
}

/* Element Ke and internal force.  Small strain: SmallStrainT::FormKd/FormStiffness
 * (SmallStrainT.cpp:255-324).  Total Lagrangian: TotalLagrangianT::FormKd/
 * FormStiffness (TotalLagrangianT.cpp:40-144).  Updated Lagrangian:
 * UpdatedLagrangianT::FormKd/FormStiffness (UpdatedLagrangianT.cpp:94-171),
 * the same weak form evaluated on the current configuration.  Returns 0, or -1 on a
 * non-positive Jacobian (ExceptionT::BadJacobianDet). */
int element(Model& M, int e, const double* u, int iteration, bool wantK, ElemOut& out,
            bool update_state) {
  const RefShape& S = ref_shape();
  double Xe[24], ue[24];
  for (int a = 0; a < 8; ++a) {
    int n = M.conn[e * 8 + a];
    for (int d = 0; d < 3; ++d) {
      Xe[a * 3 + d] = M.X[n * 3 + d];
      ue[a * 3 + d] = u[n * 3 + d];
    }
  }
  const Material& m = M.mat(e);
  std::fill(out.Ke, out.Ke + 576, 0.0);
  std::fill(out.fint, out.fint + 24, 0.0);
  J2Card scratch;
  J2Card* card = nullptr;
  if (m.kind == ORC_MAT_SS_J2) {
    if (update_state) card = &M.j2[e];
    else { scratch = M.j2[e]; card = &scratch; }
  }
  /* B-bar: mean shape-function gradients over the element
   * (SmallStrainT::SetMeanGradient, SmallStrainT.cpp:404-421) */
  const bool bbar = M.bbar && M.form == ORC_SMALL_STRAIN;
  double mean[3][8] = {{0}};
  if (bbar) {
    double vol = 0.0;
    for (int ip = 0; ip < 8; ++ip) {
      double g[3][8];
      const double detj = ip_gradients(Xe, ip, g);
      if (!(detj > 0.0)) return -1;
      const double wdet = S.w[ip] * detj;
      vol += wdet;
      for (int d = 0; d < 3; ++d)
        for (int a = 0; a < 8; ++a) mean[d][a] += wdet * g[d][a];
    }
    for (int d = 0; d < 3; ++d)
      for (int a = 0; a < 8; ++a) mean[d][a] /= vol;
  }
  for (int ip = 0; ip < 8; ++ip) {
    double g[3][8];
    double detj = ip_gradients(Xe, ip, g);
    if (!(detj > 0.0)) return -1;
    double wdet = S.w[ip] * detj;
    double s[6], D[36];
    if (M.form == ORC_SMALL_STRAIN) {
      double B[6][24];
      if (bbar) set_b_bar(g, mean, B);
      else set_b(g, B);
      /* strain = B u, shear halved to tensor components */
      double eps[6];
      for (int r = 0; r < 6; ++r) {
        double a = 0;
        for (int q = 0; q < 24; ++q) a += B[r][q] * ue[q];
        eps[r] = r < 3 ? a : 0.5 * a;
      }
      if (m.kind == ORC_MAT_SS_J2) {
        /* the tangent reads the state left by the last residual evaluation
         * (FormStiffness calls only c_ijkl) */
        if (wantK) j2_moduli(m, *card, ip, D);
        else j2_stress(m, *card, ip, eps, iteration, s);
      } else {
        hooke(m.C, eps, s);
        std::memcpy(D, m.C, sizeof(D));
      }
      if (!wantK) {
        std::memcpy(out.sig[ip], s, sizeof(double) * 6);
        /* J2SSKStV::ComputeOutput (J2SSKStV.cpp:181-207) */
        const double p = (s[0] + s[1] + s[2]) / 3.0;
        double dv[3] = {s[0] - p, s[1] - p, s[2] - p};
        double i2 = s[3] * s[3] + s[4] * s[4] + s[5] * s[5] - dv[0] * dv[1] - dv[1] * dv[2] - dv[2] * dv[0];
        if (i2 < 0.0) i2 = 0.0;
        double al = 0.0;
        if (card && card->allocated)
          al = card->alpha[ip] + (card->flags[ip] == ORC_J2_PLASTIC ? std::sqrt(2.0 / 3.0) * card->dgamma[ip] : 0.0);
        out.mat[ip][0] = al;
        out.mat[ip][1] = std::sqrt(3.0 * i2);
        out.mat[ip][2] = p;
      }
      if (wantK) {
        add_btdb_b(B, D, wdet, out.Ke);
      } else {
        /* fint = B^T sigma (SmallStrainT::FormKd) */
        for (int q = 0; q < 24; ++q) {
          double a = 0;
          for (int r = 0; r < 6; ++r) a += B[r][q] * s[r];
          out.fint[q] += wdet * a;
        }
      }
    } else {
      double F[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double a = (i == j) ? 1.0 : 0.0;
          for (int n = 0; n < 8; ++n) a += ue[n * 3 + i] * g[j][n];
          F[i * 3 + j] = a;
        }
      double J = det3(F);
      if (!(J > 0.0)) return -1;
      if (m.kind == ORC_MAT_FS_SIMO) simo(m, F, s, wantK ? D : nullptr);
      else stvenant(m, F, s, wantK ? D : nullptr);
      if (!wantK) {
        std::memcpy(out.sig[ip], s, sizeof(double) * 6);
        const double p = (s[0] + s[1] + s[2]) / 3.0;
        double dv[3] = {s[0] - p, s[1] - p, s[2] - p};
        double i2 = s[3] * s[3] + s[4] * s[4] + s[5] * s[5] - dv[0] * dv[1] - dv[1] * dv[2] - dv[2] * dv[0];
        if (i2 < 0.0) i2 = 0.0;
        out.mat[ip][0] = 0.0;
        out.mat[ip][1] = std::sqrt(3.0 * i2);
        out.mat[ip][2] = p;
      }
      double gx[3][8];
      double scale;
      if (M.form == ORC_UPDATED_LAGRANGIAN) {
        /* UpdatedLagrangianT::SetGlobalShape / FormStiffness / FormKd
         * (UpdatedLagrangianT.cpp:84-171): the shape functions of the
         * current configuration x = X + u give dN/dx directly, and the
         * integration runs over the current volume (w det dx/dxi) */
        double xe[24];
        for (int k = 0; k < 24; ++k) xe[k] = Xe[k] + ue[k];
        const double detc = ip_gradients(xe, ip, gx);
        if (!(detc > 0.0)) return -1;
        scale = S.w[ip] * detc;
      } else {
        double Fi[9];
        inv3(F, J, Fi);
        /* spatial gradients dN/dx_k = sum_J dN/dX_J Finv(J,k) */
        for (int k = 0; k < 3; ++k)
          for (int n = 0; n < 8; ++n)
            gx[k][n] = g[0][n] * Fi[0 * 3 + k] + g[1][n] * Fi[1 * 3 + k] + g[2][n] * Fi[2 * 3 + k];
        scale = wdet * J;
      }
      if (wantK) {
        add_btdb(gx, D, scale, out.Ke);
        double sm[9] = {s[0], s[5], s[4], s[5], s[1], s[3], s[4], s[3], s[2]};
        for (int a = 0; a < 8; ++a)
          for (int b = 0; b < 8; ++b) {
            double gab = 0;
            for (int i = 0; i < 3; ++i)
              for (int j = 0; j < 3; ++j) gab += gx[i][a] * sm[i * 3 + j] * gx[j][b];
            for (int d = 0; d < 3; ++d) out.Ke[(a * 3 + d) * 24 + b * 3 + d] += scale * gab;
          }
      } else {
        double sm[9] = {s[0], s[5], s[4], s[5], s[1], s[3], s[4], s[3], s[2]};
        for (int a = 0; a < 8; ++a)
          for (int i = 0; i < 3; ++i) {
            double v = 0;
            for (int j = 0; j < 3; ++j) v += sm[i * 3 + j] * gx[j][a];
            out.fint[a * 3 + i] += scale * v;
          }
      }
    }
  }
  return 0;
}

/* external force at time t: nodal forces (force_BC) and tractions
 * (ContinuumElementT::ApplyTractionBC, ContinuumElementT.cpp:514-665; reference
 * coordinates, 2x2 Gauss on the facet) */
void external_force(const Model& M, double t, std::vector<double>& f) {
  f.assign(M.nnd * 3, 0.0);
  double sc = M.schedule(t);
  for (const Force& F : M.forces) f[F.node * 3 + F.dof] += sc * F.value;
  const double g = 1.0 / std::sqrt(3.0);
  const double qr[4] = {-g, g, g, -g}, qs[4] = {-g, -g, g, g};
  const double nr[4] = {-1, 1, 1, -1}, ns[4] = {-1, -1, 1, 1};
  for (const Traction& T : M.tractions) {
    int nodes[4];
    for (int k = 0; k < 4; ++k) nodes[k] = M.conn[T.elem * 8 + kFacetNodes[T.facet][k]];
    for (int q = 0; q < 4; ++q) {
      double Na[4], dr[4], ds[4];
      for (int k = 0; k < 4; ++k) {
        Na[k] = 0.25 * (1 + qr[q] * nr[k]) * (1 + qs[q] * ns[k]);
        dr[k] = 0.25 * nr[k] * (1 + qs[q] * ns[k]);
        ds[k] = 0.25 * ns[k] * (1 + qr[q] * nr[k]);
      }
      double m1[3] = {0, 0, 0}, m2[3] = {0, 0, 0};
      for (int k = 0; k < 4; ++k)
        for (int d = 0; d < 3; ++d) {
          m1[d] += M.X[nodes[k] * 3 + d] * dr[k];
          m2[d] += M.X[nodes[k] * 3 + d] * ds[k];
        }
      double n3[3] = {m1[1] * m2[2] - m1[2] * m2[1], m1[2] * m2[0] - m1[0] * m2[2], m1[0] * m2[1] - m1[1] * m2[0]};
      double jw = std::sqrt(n3[0] * n3[0] + n3[1] * n3[1] + n3[2] * n3[2]);
      for (int k = 0; k < 4; ++k)
        for (int d = 0; d < 3; ++d) f[nodes[k] * 3 + d] += sc * jw * T.t[d] * Na[k];
    }
  }
}

/* locate (row, col) in MSR upper structure; returns value index */
long msr_find(const std::vector<int>& bindx, int row, int col) {
  if (row == col) return row;
  int lo = bindx[row], hi = bindx[row + 1];
  const int* p = std::lower_bound(bindx.data() + lo, bindx.data() + hi, col);
  if (p == bindx.data() + hi || *p != col) return -1;
  return p - bindx.data();
}

/* global residual and (optionally) MSR tangent; element loop of
 * SolidElementT::ElementRHSDriver / ElementLHSDriver with assembly of
 * MSRMatrixT::Assemble (symmetric, MSRMatrixT.cpp:96-143).  Element
 * formation is spread over M.nthreads threads; assembly is serial. */
int form(Model& M, const double* u, double t, int iteration, double* R, double* val,
         const double* v_nodal = nullptr, double* Kv = nullptr) {
  const int nth = std::max(1, M.nthreads);
  if (R) {
    std::vector<double> fext;
    external_force(M, t, fext);
    for (int i = 0; i < M.nnd * 3; ++i)
      if (M.eqnos[i] > 0) R[M.eqnos[i] - 1] = fext[i];
  }
  if (val) std::fill(val, val + M.bindx.size(), 0.0);
  const int chunk = 2048;
  std::vector<ElemOut> buf(chunk);
  std::vector<int> status(chunk);
  for (int e0 = 0; e0 < M.nel; e0 += chunk) {
    int ne = std::min(chunk, M.nel - e0);
    for (int pass = 0; pass < 2; ++pass) {
      bool wantK = pass == 1;
      if (wantK && !val) continue;
      if (!wantK && !R) continue;
      /* threads touch disjoint elements (and disjoint J2 cards) */
      auto work = [&](int tid) {
        for (int k = tid; k < ne; k += nth)
          status[k] = element(M, e0 + k, u, iteration, wantK, buf[k], !wantK);
      };
      if (nth == 1) {
        work(0);
      } else {
        std::vector<std::thread> th;
        for (int i = 0; i < nth; ++i) th.emplace_back(work, i);
        for (auto& x : th) x.join();
      }
      for (int k = 0; k < ne; ++k) {
        if (status[k]) return -1;
        int e = e0 + k;
        int eq[24];
        for (int a = 0; a < 8; ++a)
          for (int d = 0; d < 3; ++d) eq[a * 3 + d] = M.eqnos[M.conn[e * 8 + a] * 3 + d];
        if (!wantK) {
          for (int p = 0; p < 24; ++p)
            if (eq[p] > 0) R[eq[p] - 1] -= buf[k].fint[p];
        } else {
          if (Kv) {
            /* the element tangent applied to a nodal vector, on the active
             * rows (all columns: the coupling to prescribed dofs included) */
            double ve[24];
            for (int a = 0; a < 8; ++a)
              for (int d = 0; d < 3; ++d) ve[a * 3 + d] = v_nodal[M.conn[e * 8 + a] * 3 + d];
            for (int p = 0; p < 24; ++p) {
              if (eq[p] <= 0) continue;
              double a = 0.0;
              for (int q = 0; q < 24; ++q) a += buf[k].Ke[p * 24 + q] * ve[q];
              Kv[eq[p] - 1] += a;
            }
          }
          for (int p = 0; p < 24; ++p) {
            if (eq[p] <= 0) continue;
            for (int q = 0; q < 24; ++q) {
              if (eq[q] <= 0 || eq[q] < eq[p]) continue;
              if (eq[q] == eq[p] && q < p) continue;
              double v = buf[k].Ke[p * 24 + q];
              if (eq[p] == eq[q] && p != q) v *= 2.0;
              long idx = msr_find(M.bindx, eq[p] - 1, eq[q] - 1);
              if (idx < 0) return -2;
              val[idx] += v;
            }
          }
        }
      }
    }
  }
  return 0;
}

/* MSRMatrixT::Multx (MSRMatrixT.cpp:385-420), symmetric upper storage */
void msr_multx(const Model& M, const double* val, const double* x, double* y) {
  int n = M.neq;
  std::fill(y, y + n, 0.0);
  for (int r = 0; r < n; ++r) {
    y[r] += val[r] * x[r];
    for (int j = M.bindx[r]; j < M.bindx[r + 1]; ++j) {
      int c = M.bindx[j];
      y[r] += val[j] * x[c];
      y[c] += val[j] * x[r];
    }
  }
}

/* Jacobi-preconditioned CG (DiagonalMatrixT Jacobi scaling as M^-1) */
int pcg(const Model& M, const double* val, const double* b, double* x, double tol, int maxit,
        double* relres) {
  int n = M.neq;
  std::vector<double> r(n), z(n), p(n), q(n), minv(n);
  for (int i = 0; i < n; ++i) minv[i] = 1.0 / val[i];
  msr_multx(M, val, x, q.data());
  double bb = 0, rz = 0;
  for (int i = 0; i < n; ++i) {
    r[i] = b[i] - q[i];
    z[i] = minv[i] * r[i];
    p[i] = z[i];
    bb += b[i] * b[i];
    rz += r[i] * z[i];
  }
  double bn = std::sqrt(bb);
  if (bn == 0.0) { if (relres) *relres = 0; return 0; }
  for (int it = 1; it <= maxit; ++it) {
    msr_multx(M, val, p.data(), q.data());
    double pq = 0;
    for (int i = 0; i < n; ++i) pq += p[i] * q[i];
    double alpha = rz / pq;
    double rr = 0, rzn = 0;
    for (int i = 0; i < n; ++i) {
      x[i] += alpha * p[i];
      r[i] -= alpha * q[i];
      z[i] = minv[i] * r[i];
      rr += r[i] * r[i];
      rzn += r[i] * z[i];
    }
    double rel = std::sqrt(rr) / bn;
    if (relres) *relres = rel;
    if (rel < tol) return it;
    double beta = rzn / rz;
    rz = rzn;
    for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
  }
  return -maxit;
}

/* Spin barrier of the oracle's worker threads (generation counter). */
struct SpinBarrier {
  std::atomic<int> count{0};
  std::atomic<int> gen{0};
  int n;
  explicit SpinBarrier(int n_) : n(n_) {}
  void wait() {
    const int g = gen.load(std::memory_order_acquire);
    if (count.fetch_add(1, std::memory_order_acq_rel) == n - 1) {
      count.store(0, std::memory_order_relaxed);
      gen.store(g + 1, std::memory_order_release);
    } else {
      while (gen.load(std::memory_order_acquire) == g) std::this_thread::yield();
    }
  }
};

/* The same Jacobi CG as pcg() on M.nthreads threads, for the CPU baseline
 * and large oracle runs.  The rows are split into contiguous ranges of
 * about equal stored length; the symmetric MSR product (MSRMatrixT::Multx,
 * MSRMatrixT.cpp:385-420) runs per range, a row's transposed contributions
 * to rows of later ranges going into a per-thread spill buffer that the
 * owners of those rows add, in thread order, after a barrier.  Dot products
 * are summed per thread and then over threads in a fixed order, so every
 * thread takes the same decisions and the result does not depend on timing.
 * Same stopping rule as pcg(): ||r|| / ||b|| < tol. */
int pcg_mt(const Model& M, const double* val, const double* b, double* x, double tol, int maxit,
           double* relres) {
  const int n = M.neq;
  const int nth = std::max(1, std::min(M.nthreads, n / 2048));
  if (nth <= 1) return pcg(M, val, b, x, tol, maxit, relres);
  const std::vector<int>& bx = M.bindx;
  std::vector<int> lo(nth + 1, n);
  {
    const long long total = (long long)n + (bx[n] - bx[0]);
    long long acc = 0;
    int t = 1;
    lo[0] = 0;
    for (int r = 0; r < n && t < nth; ++r) {
      acc += 1 + (bx[r + 1] - bx[r]);
      if (acc * nth >= total * t) lo[t++] = r + 1;
    }
    for (; t < nth; ++t) lo[t] = n;
  }
  std::vector<int> spill_len(nth, 0);
  for (int t = 0; t < nth; ++t) {
    int hi = lo[t + 1];
    for (int r = lo[t]; r < lo[t + 1]; ++r)
      if (bx[r + 1] > bx[r]) hi = std::max(hi, bx[bx[r + 1] - 1] + 1);
    spill_len[t] = hi - lo[t + 1];
  }
  std::vector<std::vector<double>> spill(nth);
  for (int t = 0; t < nth; ++t) spill[t].assign(spill_len[t], 0.0);
  std::vector<double> r(n), z(n), p(n), q(n), minv(n);
  std::vector<double> part_a(nth), part_b(nth), part_c(nth);
  SpinBarrier bar(nth);
  int result = -maxit;
  double rel_out = 0.0;
  /* y = A v over the rows of thread t (spill of later rows kept aside) */
  auto product = [&](int t, const double* v, double* y) {
    const int a = lo[t], e = lo[t + 1];
    std::vector<double>& sp = spill[t];
    std::fill(sp.begin(), sp.end(), 0.0);
    for (int i = a; i < e; ++i) y[i] = 0.0;
    for (int i = a; i < e; ++i) {
      const double vi = v[i];
      double s_ = val[i] * vi;
      for (int j = bx[i]; j < bx[i + 1]; ++j) {
        const int c = bx[j];
        const double w = val[j];
        s_ += w * v[c];
        if (c < e) y[c] += w * vi;
        else sp[c - e] += w * vi;
      }
      y[i] += s_;
    }
  };
  /* add the spills of earlier threads that fall on thread t's rows */
  auto add_spills = [&](int t, double* y) {
    const int a = lo[t], e = lo[t + 1];
    for (int s2 = 0; s2 < t; ++s2) {
      const int base = lo[s2 + 1], len = spill_len[s2];
      const int i0 = std::max(a, base), i1 = std::min(e, base + len);
      for (int i = i0; i < i1; ++i) y[i] += spill[s2][i - base];
    }
  };
  auto total = [&](const std::vector<double>& part) {
    double s_ = 0.0;
    for (int t = 0; t < nth; ++t) s_ += part[t];
    return s_;
  };
  auto worker = [&](int t) {
    const int a = lo[t], e = lo[t + 1];
    for (int i = a; i < e; ++i) minv[i] = 1.0 / val[i];
    product(t, x, q.data());
    bar.wait();
    add_spills(t, q.data());
    double bb = 0.0, rz_ = 0.0;
    for (int i = a; i < e; ++i) {
      r[i] = b[i] - q[i];
      z[i] = minv[i] * r[i];
      p[i] = z[i];
      bb += b[i] * b[i];
      rz_ += r[i] * z[i];
    }
    part_a[t] = bb;
    part_b[t] = rz_;
    bar.wait();
    const double bn = std::sqrt(total(part_a));
    double rz = total(part_b);
    bar.wait();  /* part_a / part_b are rewritten below */
    if (bn == 0.0) {
      if (t == 0) {
        result = 0;
        rel_out = 0.0;
      }
      return;
    }
    for (int it = 1; it <= maxit; ++it) {
      product(t, p.data(), q.data());
      bar.wait();
      add_spills(t, q.data());
      double pq = 0.0;
      for (int i = a; i < e; ++i) pq += p[i] * q[i];
      part_c[t] = pq;
      bar.wait();
      const double alpha = rz / total(part_c);
      double rr = 0.0, rzn = 0.0;
      for (int i = a; i < e; ++i) {
        x[i] += alpha * p[i];
        r[i] -= alpha * q[i];
        z[i] = minv[i] * r[i];
        rr += r[i] * r[i];
        rzn += r[i] * z[i];
      }
      part_a[t] = rr;
      part_b[t] = rzn;
      bar.wait();
      const double rel = std::sqrt(total(part_a)) / bn;
      const double rz_new = total(part_b);
      if (t == 0) rel_out = rel;
      if (rel < tol) {
        if (t == 0) result = it;
        return;
      }
      const double beta = rz_new / rz;
      rz = rz_new;
      for (int i = a; i < e; ++i) p[i] = z[i] + beta * p[i];
      bar.wait();  /* p complete before the next product; totals read */
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nth; ++t) th.emplace_back(worker, t);
  worker(0);
  for (auto& w : th) w.join();
  if (relres) *relres = rel_out;
  return result;
}

/* Jacobi CG on the model's thread count (serial when it is 1). */
int pcg_any(const Model& M, const double* val, const double* b, double* x, double tol, int maxit, double* relres) {
  return M.nthreads > 1 ? pcg_mt(M, val, b, x, tol, maxit, relres) : pcg(M, val, b, x, tol, maxit, relres);
}

/* dense LU (partial pivoting) solve of the MSR system: stands in for the
 * reference's direct profile / SPOOLES factorisations on small decks, which
 * accept symmetric indefinite tangents */
int dense_solve(const Model& M, const double* val, const double* b, double* x) {
  int n = M.neq;
  std::vector<double> A((size_t)n * n, 0.0);
  for (int r = 0; r < n; ++r) {
    A[(size_t)r * n + r] = val[r];
    for (int j = M.bindx[r]; j < M.bindx[r + 1]; ++j) {
      int c = M.bindx[j];
      A[(size_t)r * n + c] = A[(size_t)c * n + r] = val[j];
    }
  }
  std::vector<double> y(b, b + n);
  for (int k = 0; k < n; ++k) {
    int piv = k;
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(A[(size_t)i * n + k]) > std::fabs(A[(size_t)piv * n + k])) piv = i;
    if (A[(size_t)piv * n + k] == 0.0) return -1;
    if (piv != k) {
      for (int j = 0; j < n; ++j) std::swap(A[(size_t)k * n + j], A[(size_t)piv * n + j]);
      std::swap(y[k], y[piv]);
    }
    const double d = A[(size_t)k * n + k];
    for (int i = k + 1; i < n; ++i) {
      const double l = A[(size_t)i * n + k] / d;
      if (l == 0.0) continue;
      A[(size_t)i * n + k] = l;
      for (int j = k + 1; j < n; ++j) A[(size_t)i * n + j] -= l * A[(size_t)k * n + j];
      y[i] -= l * y[k];
    }
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = y[i];
    for (int j = i + 1; j < n; ++j) s -= A[(size_t)i * n + j] * x[j];
    x[i] = s / A[(size_t)i * n + i];
  }
  return 0;
}

void ensure_setup(Model& M) {
  if (M.neq < 0) {
    set_equations(M);
    build_msr(M, true, M.bindx);
    M.j2.assign(M.nel, J2Card());
    M.u.assign(M.nnd * 3, 0.0);
  }
}

}  // namespace

extern "C" {

void* orc_model_create(int nnd, const double* X, int nel, const int* conn) {
  Model* M = new Model;
  M->nnd = nnd;
  M->nel = nel;
  M->X.assign(X, X + nnd * 3);
  M->conn.assign(conn, conn + nel * 8);
  M->mats.resize(1);
  return M;
}
void orc_model_free(void* m) { delete static_cast<Model*>(m); }
int orc_set_formulation(void* m, int form) {
  static_cast<Model*>(m)->form = form;
  return 0;
}
int orc_set_bbar(void* m, int on) {
  static_cast<Model*>(m)->bbar = on != 0;
  return 0;
}
/* parameters:
 *  SS_HOOKEAN: 36 values (row-major 6x6) or {E, nu}
 *  SS_J2: {E, nu, a, b[, elastic_iterations]}
 *  FS_SIMO: {mu, kappa}
 *  FS_STVENANT: {E, nu} */
int orc_set_material(void* m, int block, int kind, const double* p, int np) {
  Model* M = static_cast<Model*>(m);
  if (block < 0) return -1;
  if ((int)M->mats.size() <= block) M->mats.resize(block + 1);
  Material& mt = M->mats[block];
  mt.kind = kind;
  auto set_E_nu = [&](double E, double nu) { /* IsotropicT::Set_E_nu (:32-44) */
    mt.mu = 0.5 * E / (1.0 + nu);
    mt.lambda = 2.0 * mt.mu * nu / (1.0 - 2.0 * nu);
    mt.kappa = mt.lambda + 2.0 / 3.0 * mt.mu;
    iso_moduli(mt.mu, mt.lambda, mt.C);
  };
  switch (kind) {
    case ORC_MAT_SS_HOOKEAN:
      if (np == 36) std::memcpy(mt.C, p, sizeof(mt.C));
      else if (np == 2) set_E_nu(p[0], p[1]);
      else return -1;
      break;
    case ORC_MAT_SS_J2:
      if (np < 4) return -1;
      set_E_nu(p[0], p[1]);
      mt.hard_a = p[2];
      mt.hard_b = p[3];
      mt.elastic_its = np > 4 ? (int)p[4] : 0;
      break;
    case ORC_MAT_FS_SIMO: /* IsotropicT::Set_mu_kappa (:46-57) */
      if (np != 2) return -1;
      mt.mu = p[0];
      mt.kappa = p[1];
      break;
    case ORC_MAT_FS_STVENANT:
      if (np != 2) return -1;
      set_E_nu(p[0], p[1]);
      break;
    default:
      return -1;
  }
  return 0;
}
int orc_set_element_blocks(void* m, const int* b) {
  Model* M = static_cast<Model*>(m);
  M->block.assign(b, b + M->nel);
  return 0;
}
int orc_set_schedule(void* m, int n, const double* x, const double* y) {
  Model* M = static_cast<Model*>(m);
  M->sx.assign(x, x + n);
  M->sy.assign(y, y + n);
  return 0;
}
int orc_add_torsion(void* m, int axis, double rate, const double* point, int nnodes, const int* nodes) {
  Model* M = static_cast<Model*>(m);
  if (axis < 0 || axis > 2 || nnodes < 0) return -1;
  const int t = (int)M->torsions.size();
  M->torsions.push_back({axis, rate, {point[0], point[1], point[2]}});
  const int across[3][2] = {{1, 2}, {2, 0}, {0, 1}};  /* the dofs turned about each axis */
  for (int i = 0; i < nnodes; ++i)
    for (int j = 0; j < 2; ++j) {
      KBC k{nodes[i], across[axis][j], 0.0, false};
      k.torsion = t;
      M->kbc.push_back(k);
    }
  return 0;
}
int orc_add_kbc(void* m, int node, int dof, double value, int scheduled) {
  static_cast<Model*>(m)->kbc.push_back({node, dof, value, scheduled != 0});
  return 0;
}
int orc_add_force(void* m, int node, int dof, double value) {
  static_cast<Model*>(m)->forces.push_back({node, dof, value});
  return 0;
}
int orc_add_traction(void* m, int elem, int facet, const double* t) {
  static_cast<Model*>(m)->tractions.push_back({elem, facet, {t[0], t[1], t[2]}});
  return 0;
}
int orc_set_threads(void* m, int n) {
  static_cast<Model*>(m)->nthreads = n;
  return 0;
}
int orc_equations(void* m, int* eqnos) {
  Model* M = static_cast<Model*>(m);
  ensure_setup(*M);
  if (eqnos) std::memcpy(eqnos, M->eqnos.data(), sizeof(int) * M->nnd * 3);
  return M->neq;
}
long long orc_msr_pattern(void* m, int upper_only, int* bindx, long long cap) {
  Model* M = static_cast<Model*>(m);
  ensure_setup(*M);
  std::vector<int> tmp;
  const std::vector<int>* b = &M->bindx;
  if (!upper_only) {
    build_msr(*M, false, tmp);
    b = &tmp;
  }
  if (bindx && cap >= (long long)b->size()) std::memcpy(bindx, b->data(), sizeof(int) * b->size());
  return (long long)b->size();
}
int orc_element(void* m, int e, const double* u, int iteration, double* Ke, double* fint) {
  Model* M = static_cast<Model*>(m);
  ensure_setup(*M);
  ElemOut o;
  int s = element(*M, e, u, iteration, true, o, false);
  if (s) return s;
  if (Ke) std::memcpy(Ke, o.Ke, sizeof(o.Ke));
  s = element(*M, e, u, iteration, false, o, false);
  if (fint) std::memcpy(fint, o.fint, sizeof(o.fint));
  return s;
}
int orc_form(void* m, const double* u, double t, int iteration, double* R, double* val) {
  Model* M = static_cast<Model*>(m);
  ensure_setup(*M);
  return form(*M, u, t, iteration, R, val);
}
int orc_msr_multx(void* m, const double* val, const double* x, double* y) {
  Model* M = static_cast<Model*>(m);
  ensure_setup(*M);
  msr_multx(*M, val, x, y);
  return 0;
}
int orc_pcg(void* m, const double* val, const double* b, double* x, double tol, int maxit,
            double* relres) {
  Model* M = static_cast<Model*>(m);
  ensure_setup(*M);
  return pcg_any(*M, val, b, x, tol, maxit, relres);
}

static double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static double norm2(const std::vector<double>& v) {
  double a = 0.0;
  for (double x : v) a += x * x;
  return std::sqrt(a);
}

/* R = Fext - Fint at the held displacement (SolverT::Residual after
 * FEManagerT::FormRHS), kept for the next orc_newton_iteration. */
int orc_residual(void* m, double t, int iteration, double* norm) {
  Model* M = static_cast<Model*>(m);
  ensure_setup(*M);
  M->Rcur.assign(M->neq, 0.0);
  if (form(*M, M->u.data(), t, iteration, M->Rcur.data(), nullptr)) return -1;
  if (norm) *norm = norm2(M->Rcur);
  return 0;
}

/* One iteration of NLSolver::Solve's loop (NLSolver.cpp:137-188) from the
 * held displacement and residual: tangent + MSR assembly, Jacobi CG to
 * lin_tol, u += du, new residual (iteration + 1).  times[3] receives the
 * seconds of the tangent pass, the CG and the residual pass. */
int orc_newton_iteration(void* m, double t, int iteration, double lin_tol, int max_it, int* pcg_its, double* norm,
                         double* times) {
  Model* M = static_cast<Model*>(m);
  ensure_setup(*M);
  if ((int)M->Rcur.size() != M->neq) return -1;
  const int n = M->neq;
  M->Kval.assign(M->bindx.size(), 0.0);
  double t0 = now_s();
  if (form(*M, M->u.data(), t, iteration, nullptr, M->Kval.data())) return -1;
  double t1 = now_s();
  std::vector<double> du(n, 0.0);
  const int its = pcg_any(*M, M->Kval.data(), M->Rcur.data(), du.data(), lin_tol, max_it, nullptr);
  double t2 = now_s();
  if (its < 0) return -2;
  for (int i = 0; i < M->nnd * 3; ++i)
    if (M->eqnos[i] > 0) M->u[i] += du[M->eqnos[i] - 1];
  if (form(*M, M->u.data(), t, iteration + 1, M->Rcur.data(), nullptr)) return -1;
  double t3 = now_s();
  if (pcg_its) *pcg_its = its;
  if (norm) *norm = norm2(M->Rcur);
  if (times) {
    times[0] = t1 - t0;
    times[1] = t2 - t1;
    times[2] = t3 - t2;
  }
  return 0;
}

static void apply_kbc(Model& M, double t);

/* Prescribed-increment predictor of a load step (the GPU path's
 * tg_predict_prescribed): with u at the last converged state and du_p the
 * jump of the prescribed values to time t, solves
 * K(u) du_f = R(u) - K(u) [du_p] on the free dofs (Jacobi CG to lin_tol),
 * then sets u_p to the new values and u_f += du_f.  History is untouched. */
int orc_predict(void* m, double t, double lin_tol, int max_it, int* pcg_its) {
  Model* M = static_cast<Model*>(m);
  ensure_setup(*M);
  const int n = M->neq;
  const std::vector<double> u_old = M->u;
  apply_kbc(*M, t);
  std::vector<double> dup(M->nnd * 3, 0.0);
  for (int i = 0; i < M->nnd * 3; ++i)
    if (M->eqnos[i] <= 0) dup[i] = M->u[i] - u_old[i];
  const std::vector<double> u_new_p = M->u;
  M->u = u_old;
  std::vector<double> R(n, 0.0), Kv(n, 0.0), val(M->bindx.size(), 0.0);
  if (form(*M, M->u.data(), t, -1, R.data(), val.data(), dup.data(), Kv.data())) return -1;
  for (int i = 0; i < n; ++i) R[i] -= Kv[i];
  std::vector<double> du(n, 0.0);
  const int its = pcg_any(*M, val.data(), R.data(), du.data(), lin_tol, max_it, nullptr);
  if (its < 0) return -2;
  for (int i = 0; i < M->nnd * 3; ++i) {
    if (M->eqnos[i] > 0) M->u[i] += du[M->eqnos[i] - 1];
    else M->u[i] = u_new_p[i];
  }
  if (pcg_its) *pcg_its = its;
  return 0;
}

/* Prescribed displacements at the start of the step ending at time t
 * (FieldT::InitStep): schedule x value for ordinary cards; for torsion cards
 * the rigid turn of the node's initial position (TorsionKBCT::InitStep), the
 * in-plane radius vector rotated by theta = rate * t about the axis. */
static void apply_kbc(Model& M, double t) {
  const double sc = M.schedule(t);
  for (const KBC& k : M.kbc) {
    double v = k.scheduled ? sc * k.value : 0.0;
    if (k.torsion >= 0) {
      const Torsion& T = M.torsions[k.torsion];
      double a[3] = {0.0, 0.0, 0.0};
      a[T.axis] = 1.0;
      const double* X = &M.X[(size_t)k.node * 3];
      double d[3], r[3];
      for (int i = 0; i < 3; ++i) d[i] = X[i] - T.point[i];
      const double along = d[0] * a[0] + d[1] * a[1] + d[2] * a[2];
      for (int i = 0; i < 3; ++i) r[i] = d[i] - along * a[i];
      const double rad = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
      v = 0.0;
      if (std::fabs(rad) > 1.0e-12) {
        const double th = T.rate * t;
        double e1[3], e2[3];
        for (int i = 0; i < 3; ++i) e1[i] = r[i] / rad;
        e2[0] = a[1] * e1[2] - a[2] * e1[1];
        e2[1] = a[2] * e1[0] - a[0] * e1[2];
        e2[2] = a[0] * e1[1] - a[1] * e1[0];
        /* new position: the foot on the axis plus the turned radius */
        const int i = k.dof;
        const double x = (X[i] - r[i]) + rad * std::cos(th) * e1[i] + rad * std::sin(th) * e2[i];
        v = x - X[i];
      }
    }
    M.u[(size_t)k.node * 3 + k.dof] = v;
  }
}

/* NLSolver::Solve (NLSolver.cpp:57-262) + ExitIteration (:675-755) over load
 * steps; prescribed displacements applied at step start (FieldT::InitStep);
 * J2 history closed after each converged step (ContinuumElementT::CloseStep). */
int orc_run(void* m, int nsteps, double dt, double rel_tol, double abs_tol, int max_its,
            double div_tol, int solver, double lin_tol, double* u_hist, int* its_hist) {
  Model* M = static_cast<Model*>(m);
  ensure_setup(*M);
  int n = M->neq;
  std::vector<double> R(n), du(n), val(M->bindx.size());
  for (int step = 1; step <= nsteps; ++step) {
    double t = step * dt;
    apply_kbc(*M, t);
    int iteration = -1;
    if (form(*M, M->u.data(), t, iteration, R.data(), nullptr)) return step;
    double err0 = 0;
    for (double v : R) err0 += v * v;
    err0 = std::sqrt(err0);
    bool converged = err0 < abs_tol;
    int its = 0;
    while (!converged) {
      if (form(*M, M->u.data(), t, iteration, nullptr, val.data())) return step;
      std::fill(du.begin(), du.end(), 0.0);
      int s = (solver == 0) ? dense_solve(*M, val.data(), R.data(), du.data())
                            : (pcg_any(*M, val.data(), R.data(), du.data(), lin_tol, 100000, nullptr) < 0 ? -1 : 0);
      if (s) return step;
      for (int i = 0; i < M->nnd * 3; ++i)
        if (M->eqnos[i] > 0) M->u[i] += du[M->eqnos[i] - 1];
      ++iteration;
      ++its;
      if (form(*M, M->u.data(), t, iteration, R.data(), nullptr)) return step;
      double err = 0;
      for (double v : R) err += v * v;
      err = std::sqrt(err);
      double rel = err / err0;
      if (rel > div_tol) return step;
      if (rel < rel_tol || err < abs_tol) converged = true;
      else if (iteration >= max_its) return step;
    }
    for (J2Card& c : M->j2) j2_update(c);
    if (u_hist) std::memcpy(u_hist + (size_t)(step - 1) * M->nnd * 3, M->u.data(), sizeof(double) * M->nnd * 3);
    if (its_hist) its_hist[step - 1] = its;
  }
  return 0;
}

namespace {
/* Nodal stresses as written to the .run output (SolidElementT::ComputeOutput,
 * SolidElementT.cpp:1540-1570): Cauchy stress at every integration point
 * extrapolated to the element's nodes with the hex8 smoothing matrix of
 * HexahedronT::SetExtrapolation (HexahedronT.cpp:2071-2140, entries
 * (1 + sqrt3 * s_a . t_p)/8 for node signs s_a and point signs t_p), then
 * averaged over the elements sharing each node (GroupAverageT,
 * GroupAverageT.cpp:40-56).  Voigt order [11,22,33,23,13,12]. */
int nodal_output(Model& M, const double* u, int iteration, double* out, int what) {
  /* what: 0 stresses (nnd*6), 1 J2 material output alpha/VM/pressure (nnd*3) */
  static const int sg[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                               {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
  const double r3 = std::sqrt(3.0);
  const int nv = what == 0 ? 6 : 3;
  std::vector<int> count(M.nnd, 0);
  std::fill(out, out + (size_t)M.nnd * nv, 0.0);
  ElemOut o;
  for (int e = 0; e < M.nel; ++e) {
    if (element(M, e, u, iteration, false, o, false)) return -1;
    for (int a = 0; a < 8; ++a) {
      const int n = M.conn[e * 8 + a];
      ++count[n];
      for (int p = 0; p < 8; ++p) {
        const double w = 0.125 * (1.0 + r3 * (sg[a][0] * sg[p][0] + sg[a][1] * sg[p][1] + sg[a][2] * sg[p][2]));
        const double* v = what == 0 ? o.sig[p] : o.mat[p];
        for (int c = 0; c < nv; ++c) out[(size_t)n * nv + c] += w * v[c];
      }
    }
  }
  for (int n = 0; n < M.nnd; ++n)
    if (count[n])
      for (int c = 0; c < nv; ++c) out[(size_t)n * nv + c] /= count[n];
  return 0;
}
int nodal_stress(Model& M, const double* u, int iteration, double* out) { return nodal_output(M, u, iteration, out, 0); }
}  // namespace

namespace {
/* One load step of NLSolver::Solve at time t from the current state; its =
 * Newton iterations made.  0 converged, else failure (state not restored). */
int newton_step(Model* M, double t, double rel_tol, double abs_tol, int max_its, double div_tol, int solver,
                double lin_tol, int* its_out) {
  const int n = M->neq;
  std::vector<double> R(n), du(n), val(M->bindx.size());
  apply_kbc(*M, t);
  int iteration = -1, its = 0;
  *its_out = 0;
  if (form(*M, M->u.data(), t, iteration, R.data(), nullptr)) return 1;
  double err0 = 0;
  for (double v : R) err0 += v * v;
  err0 = std::sqrt(err0);
  bool converged = err0 < abs_tol;
  while (!converged) {
    if (form(*M, M->u.data(), t, iteration, nullptr, val.data())) return 1;
    std::fill(du.begin(), du.end(), 0.0);
    int s = (solver == 0) ? dense_solve(*M, val.data(), R.data(), du.data())
                          : (pcg_any(*M, val.data(), R.data(), du.data(), lin_tol, 100000, nullptr) < 0 ? -1 : 0);
    if (s) return 1;
    for (int i = 0; i < M->nnd * 3; ++i)
      if (M->eqnos[i] > 0) M->u[i] += du[M->eqnos[i] - 1];
    ++iteration;
    *its_out = ++its;
    if (form(*M, M->u.data(), t, iteration, R.data(), nullptr)) return 1;
    double err = 0;
    for (double v : R) err += v * v;
    err = std::sqrt(err);
    const double rel = err / err0;
    if (!(rel <= div_tol)) return 1;
    if (rel < rel_tol || err < abs_tol) converged = true;
    else if (iteration >= max_its) return 1;
  }
  return 0;
}
}  // namespace

/* The load-step sequence of TimeManagerT with step cuts around NLSolver
 * (TimeManagerT::Step/DecreaseLoadStep/IncreaseLoadStep/DoDecreaseStep/
 * DoIncreaseStep, TimeManagerT.cpp:55-150,350-375; NLSolver::DoConverged,
 * NLSolver.cpp:517-539; FEManagerT::ResetStep restoring the last converged
 * state, J2SSC0HardeningT::Reset).  A failed step is reset and retried at
 * half the time step while fewer than max_cuts halvings are in force; after
 * quick_count consecutive steps converged with fewer than quick_iter
 * iterations (NLSolver's iteration counter, -1 based) the step is doubled
 * back at an even step number.  u_hist / its_hist are written at the original
 * step times k*dt (its: Newton iterations summed over the sub-steps);
 * *cuts_out counts the cuts made.  Returns 0, or the 1-based original step
 * that failed with no cut left. */
int orc_run_cuts(void* m, int nsteps, double dt, double rel_tol, double abs_tol, int max_its, double div_tol,
                 int solver, double lin_tol, int max_cuts, int quick_iter, int quick_count, double* u_hist,
                 int* its_hist, int* cuts_out, double* s_hist, double* m_hist) {
  Model* M = static_cast<Model*>(m);
  ensure_setup(*M);
  enum { kSame, kDecrease, kIncrease };
  int step_num = 0, num_steps = nsteps, cuts = 0, status = kSame, quick = 0, total_cuts = 0, its_acc = 0;
  double tstep = dt, t = 0.0;
  std::vector<double> u0;
  if (cuts_out) *cuts_out = 0;
  while (step_num < num_steps) {
    if (status == kDecrease) {
      ++cuts;
      tstep /= 2;
      num_steps *= 2;
      step_num *= 2;
    } else if (status == kIncrease) {
      --cuts;
      tstep *= 2;
      num_steps /= 2;
      step_num /= 2;
    }
    status = kSame;
    ++step_num;
    t += tstep;
    u0 = M->u;
    int its = 0;
    const int s = newton_step(M, t, rel_tol, abs_tol, max_its, div_tol, solver, lin_tol, &its);
    its_acc += its;
    if (s) {
      /* ResetStep: last converged displacements, J2 flags "reset" */
      M->u = u0;
      for (J2Card& c : M->j2)
        if (c.allocated)
          for (int ip = 0; ip < 8; ++ip) c.flags[ip] = ORC_J2_RESET;
      t -= tstep;
      --step_num;
      if (cuts >= max_cuts) return (int)std::floor(t / dt + 1e-9) + 1;
      status = kDecrease;
      ++total_cuts;
      if (cuts_out) *cuts_out = total_cuts;
      continue;
    }
    const double kk = std::round(t / dt);
    const bool at_output = std::fabs(t - kk * dt) <= 1e-9 * dt && kk >= 1;
    /* output before the element groups close the step (FEManagerT::CloseStep,
     * FEManagerT.cpp:625-645) */
    if (at_output && s_hist && nodal_stress(*M, M->u.data(), its - 1, s_hist + (size_t)(kk - 1) * M->nnd * 6))
      return (int)kk;
    if (at_output && m_hist &&
        nodal_output(*M, M->u.data(), its - 1, m_hist + (size_t)(kk - 1) * M->nnd * 3, 1))
      return (int)kk;
    for (J2Card& c : M->j2) j2_update(c);
    /* NLSolver::DoConverged: fNumIteration is its - 1 here */
    if (quick_iter > 1 && its - 1 < quick_iter) {
      if (++quick >= quick_count && cuts > 0 && step_num % 2 == 0 && num_steps % 2 == 0 && step_num < num_steps) {
        status = kIncrease;
        quick = 0;
      }
    } else {
      quick = 0;
    }
    const double k = std::round(t / dt);
    if (std::fabs(t - k * dt) <= 1e-9 * dt && k >= 1) {
      if (u_hist) std::memcpy(u_hist + (size_t)(k - 1) * M->nnd * 3, M->u.data(), sizeof(double) * M->nnd * 3);
      if (its_hist) its_hist[(size_t)k - 1] = its_acc;
      its_acc = 0;
    }
  }
  return 0;
}


int orc_nodal_stress(void* m, const double* u, int iteration, double* out) {
  Model* M = static_cast<Model*>(m);
  ensure_setup(*M);
  return nodal_stress(*M, u, iteration, out);
}
int orc_nodal_material_output(void* m, const double* u, int iteration, double* out) {
  Model* M = static_cast<Model*>(m);
  ensure_setup(*M);
  return nodal_output(*M, u, iteration, out, 1);
}

int orc_j2_state(void* m, signed char* flags, double* alpha, double* eps_p) {
  Model* M = static_cast<Model*>(m);
  ensure_setup(*M);
  for (int e = 0; e < M->nel; ++e) {
    const J2Card& c = M->j2[e];
    for (int ip = 0; ip < 8; ++ip) {
      if (flags) flags[e * 8 + ip] = c.allocated ? c.flags[ip] : (signed char)ORC_J2_UNALLOCATED;
      if (alpha) alpha[e * 8 + ip] = c.allocated ? c.alpha[ip] : 0.0;
      if (eps_p)
        for (int k = 0; k < 6; ++k) eps_p[(e * 8 + ip) * 6 + k] = c.allocated ? c.eps_p[ip][k] : 0.0;
    }
  }
  return 0;
}
int orc_nodal_internal_force(void* m, const double* u, int iteration, double* f) {
  Model* M = static_cast<Model*>(m);
  ensure_setup(*M);
  std::fill(f, f + M->nnd * 3, 0.0);
  ElemOut o;
  for (int e = 0; e < M->nel; ++e) {
    if (element(*M, e, u, iteration, false, o, false)) return -1;
    for (int a = 0; a < 8; ++a)
      for (int d = 0; d < 3; ++d) f[M->conn[e * 8 + a] * 3 + d] += o.fint[a * 3 + d];
  }
  return 0;
}
int orc_get_u(void* m, double* u) {
  Model* M = static_cast<Model*>(m);
  ensure_setup(*M);
  std::memcpy(u, M->u.data(), sizeof(double) * M->nnd * 3);
  return 0;
}
int orc_set_u(void* m, const double* u) {
  Model* M = static_cast<Model*>(m);
  ensure_setup(*M);
  std::memcpy(M->u.data(), u, sizeof(double) * M->nnd * 3);
  return 0;
}
int orc_close_step(void* m) {
  Model* M = static_cast<Model*>(m);
  ensure_setup(*M);
  for (J2Card& c : M->j2) j2_update(c);
  return 0;
}

}  // extern "C"
