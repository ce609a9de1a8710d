// Tangent formation, Krylov entry points, history management and the Newton
// driver of the tahoe_gb300 C ABI.  The Newton loop mirrors NLSolver::Solve
// (tahoe/src/solvers/NLSolver.cpp:57-262) and its exit test
// NLSolver::ExitIteration (:675-755); all vectors stay on the device and the
// host reads back one residual norm per iteration plus the PCG flag per
// graph chunk.
#include <algorithm>
#include <string>
#include <cmath>
#include <cstring>
#include <vector>

#include "tg_internal.h"

namespace tg {

int launch_gather_solution(Context* c, double* d_eq);

namespace {

int set_device(Context* c) { return ok(c, cudaSetDevice(c->device), "cudaSetDevice") ? TG_OK : TG_ERR_CUDA; }

// A copy ordered after everything queued on the context stream, complete on
// return (a plain cudaMemcpy runs on the legacy stream, which does not wait
// for the context's non-blocking stream).
bool copy_sync(Context* c, void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, const char* what) {
  return ok(c, cudaMemcpyAsync(dst, src, bytes, kind, c->stream), what) &&
         ok(c, cudaStreamSynchronize(c->stream), what);
}

int check_status(Context* c) {
  if (!ok(c, cudaMemcpyAsync(c->h_status, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "status") ||
      !ok(c, cudaStreamSynchronize(c->stream), "sync"))
    return TG_ERR_CUDA;
  const int st = *c->h_status;
  if (!st) return TG_OK;
  cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream);
  cudaStreamSynchronize(c->stream);
  if (st & kStatusBadJacobian) {
    c->err = "non-positive Jacobian determinant";
    return TG_ERR_BAD_JACOBIAN;
  }
  c->err = "non-finite value";
  return TG_ERR_NAN;
}

// arithmetic of the residuals a Newton driver forms: the mixed-precision
// form's are double-float (48 significant bits, on the FP32 pipe), the FP64
// form's are FP64
int residual_arith(const tg_newton_params* P) {
  return P->precision == TG_MIXED ? kResidualDoubleFloat : kResidualFP64;
}

// residual on the device; returns its norm
int residual_norm(Context* c, double* norm, int arith) {
  int s = launch_residual(c, arith);
  if (s) return s;
  if (!ok(c, cudaMemcpyAsync(c->h_resid, c->d_resid, sizeof(ResidScalars), cudaMemcpyDeviceToHost, c->stream), "norm"))
    return TG_ERR_CUDA;
  s = check_status(c);
  if (s) return s;
  const double n2 = c->h_resid->norm2;
  if (!std::isfinite(n2)) {
    c->err = "non-finite residual";
    return TG_ERR_NAN;
  }
  *norm = std::sqrt(n2);
  return TG_OK;
}

struct PhaseTimer {
  cudaEvent_t a = nullptr, b = nullptr;
  explicit PhaseTimer(bool on) {
    if (on) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
    }
  }
  ~PhaseTimer() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
  void start(cudaStream_t s) {
    if (a) cudaEventRecord(a, s);
  }
  double stop(cudaStream_t s) {
    if (!a) return 0.0;
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
  }
};

}  // namespace

int form_tangent(Context* c, int precision) {
  const size_t keN = (size_t)c->nel * kKeStride;
  if (precision == TG_MIXED) {
    if (!c->d_Ke32 && !dalloc(c, &c->d_Ke32, keN)) return TG_ERR_OOM;
    if (!c->d_minv32 && !dalloc(c, &c->d_minv32, minv_values(c->nnd))) return TG_ERR_OOM;
  } else {
    if (!c->d_Ke64 && !dalloc(c, &c->d_Ke64, keN)) return TG_ERR_OOM;
    if (!c->d_minv64 && !dalloc(c, &c->d_minv64, minv_values(c->nnd))) return TG_ERR_OOM;
  }
  int s = launch_tangent(c, precision);
  if (!s && push_solve(c)) {
    // the solve streams the push storage: its upper blocks are assembled
    // straight into it, the full storage only when something reads it
    s = launch_assemble_upper(c, precision);
    if (!s) {
      ++c->tangent_serial;
      (precision == TG_MIXED ? c->push.serial32 : c->push.serial64) = c->tangent_serial;
    }
  } else if (!s) {
    s = ensure_blob(c, precision);
    if (!s) s = launch_assemble(c, precision);
    if (!s) {
      ++c->tangent_serial;
      (precision == TG_MIXED ? c->full_serial32 : c->full_serial64) = c->tangent_serial;
    }
    // the symmetric stream format of the single-vector product
    if (!s && sym_active(c)) s = sym_convert(c, precision);
  }
  if (!s) s = check_status(c);
  if (!s) c->tangent_precision = precision;
  return s;
}

}  // namespace tg

using namespace tg;

extern "C" {

int tg_get_tangent_csr(tg_context* c, int upper_only, double* vals) {
  if (!c || !vals || c->tangent_precision < 0) return TG_ERR_ARG;
  if (set_device(c) || ensure_host_mesh(c)) return TG_ERR_CUDA;
  {
    const int sf = ensure_full_assembly(c);
    if (sf) return sf;
  }
  // decode the tile-contiguous storage: tile t, local block jl, plane k
  const bool f32 = c->tangent_precision == TG_MIXED;
  const std::vector<long long>& off = f32 ? c->h_blob_off32 : c->h_blob_off64;
  std::vector<unsigned char> h((size_t)off[c->ntiles]);
  if (!copy_sync(c, h.data(), f32 ? c->d_blob32 : c->d_blob64, h.size(), cudaMemcpyDeviceToHost, "blob"))
    return TG_ERR_CUDA;
  auto value = [&](int I, int k, int pq) -> double {
    int t = 0;
    {
      const auto& tr = c->h_tile_row;
      t = (int)(std::upper_bound(tr.begin(), tr.end(), I) - tr.begin()) - 1;
    }
    const unsigned char* base = h.data() + off[t];
    const int* hdr = reinterpret_cast<const int*>(base);
    const int nrows = hdr[1], nb = hdr[2], ps = hdr[3];
    const int jl = k - c->h_rowptr[hdr[0]];
    const unsigned char* planes = base + 16 + 4 * ceil4(nrows + 1) + 4 * ceil4(nb);
    return f32 ? (double)reinterpret_cast<const float*>(planes)[(size_t)pq * ps + jl]
               : reinterpret_cast<const double*>(planes)[(size_t)pq * ps + jl];
  };
  const int* eq = c->h_eqnos.data();
  long long count = 0;
  for (int I = 0; I < c->nnd; ++I)
    for (int p = 0; p < 3; ++p) {
      const int r = eq[I * 3 + p];
      if (r <= 0) continue;
      for (int k = c->h_rowptr[I]; k < c->h_rowptr[I + 1]; ++k) {
        const int J = c->h_col[k];
        for (int q = 0; q < 3; ++q) {
          const int cc = eq[J * 3 + q];
          if (cc <= 0 || (upper_only && cc < r)) continue;
          vals[count++] = value(I, k, p * 3 + q);
        }
      }
    }
  return TG_OK;
}

int tg_element_dump(tg_context* c, int first, int count, double* Ke, double* fint) {
  if (!c || first < 0 || count <= 0 || first + count > c->nel || !Ke || !fint) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  if (!c->d_Ke64 && !dalloc(c, &c->d_Ke64, (size_t)c->nel * kKeStride)) return TG_ERR_OOM;
  double *dK = nullptr, *dF = nullptr;
  if (!ok(c, cudaMallocAsync((void**)&dK, sizeof(double) * 576 * count, c->stream), "alloc") ||
      !ok(c, cudaMallocAsync((void**)&dF, sizeof(double) * 24 * count, c->stream), "alloc")) {
    if (dK) cudaFreeAsync(dK, c->stream);
    return TG_ERR_OOM;
  }
  int s = launch_element_dump(c, first, count, dK, dF);
  if (!s && (!ok(c, cudaMemcpyAsync(Ke, dK, sizeof(double) * 576 * count, cudaMemcpyDeviceToHost, c->stream), "K") ||
             !ok(c, cudaMemcpyAsync(fint, dF, sizeof(double) * 24 * count, cudaMemcpyDeviceToHost, c->stream), "F")))
    s = TG_ERR_CUDA;
  if (!s) s = check_status(c);
  cudaFreeAsync(dK, c->stream);
  cudaFreeAsync(dF, c->stream);
  cudaStreamSynchronize(c->stream);
  return s;
}

int tg_pcg_solve(tg_context* c, const double* rhs, double* du, double rel_tol, int max_it, int precond, int* iters,
                 double* rel_res) {
  if (!c || c->nnd <= 0 || max_it <= 0 || rel_tol <= 0.0) return TG_ERR_ARG;
  if (precond != TG_PRECOND_JACOBI && precond != TG_PRECOND_BLOCK_JACOBI) return TG_ERR_ARG;
  if (c->tangent_precision < 0) {
    c->err = "tg_pcg_solve: form the tangent first";
    return TG_ERR_ARG;
  }
  if (set_device(c)) return TG_ERR_CUDA;
  const double4_32a* d_rhs = c->d_R;
  double4_32a* tmp = nullptr;
  double* d_eq = nullptr;
  int s = TG_OK;
  if (rhs || du) {
    if (!ok(c, cudaMallocAsync((void**)&d_eq, sizeof(double) * std::max(c->neq, 1), c->stream), "alloc"))
      return TG_ERR_OOM;
  }
  if (rhs) {
    if (!ok(c, cudaMallocAsync((void**)&tmp, sizeof(double4_32a) * c->nnd, c->stream), "alloc") ||
        !ok(c, cudaMemsetAsync(tmp, 0, sizeof(double4_32a) * c->nnd, c->stream), "memset") ||
        !ok(c, cudaMemcpyAsync(d_eq, rhs, sizeof(double) * c->neq, cudaMemcpyHostToDevice, c->stream), "rhs"))
      s = TG_ERR_CUDA;
    if (!s) s = launch_scatter_eq(c, d_eq, tmp);
    d_rhs = tmp;
  }
  if (!s) s = pcg_solve(c, d_rhs, rel_tol, max_it, precond, iters, rel_res);
  int s2 = TG_OK;
  if (du && (s == TG_OK || s == TG_ERR_NOT_CONVERGED)) {
    s2 = launch_gather_solution(c, d_eq);
    if (!s2 && !ok(c, cudaMemcpyAsync(du, d_eq, sizeof(double) * c->neq, cudaMemcpyDeviceToHost, c->stream), "du"))
      s2 = TG_ERR_CUDA;
  }
  if (tmp) cudaFreeAsync(tmp, c->stream);
  if (d_eq) cudaFreeAsync(d_eq, c->stream);
  cudaStreamSynchronize(c->stream);
  return s ? s : s2;
}

int tg_apply_update(tg_context* c) {
  if (!c || !c->have_du) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  int s = launch_apply_update(c);
  if (!s && !ok(c, cudaStreamSynchronize(c->stream), "sync")) s = TG_ERR_CUDA;
  return s;
}

int tg_close_step(tg_context* c) {
  if (!c) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  int s = launch_close_step(c, 0);
  if (!s && !ok(c, cudaStreamSynchronize(c->stream), "sync")) s = TG_ERR_CUDA;
  return s;
}

int tg_reset_step(tg_context* c) {
  if (!c) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  int s = launch_close_step(c, 1);
  if (!s && !ok(c, cudaStreamSynchronize(c->stream), "sync")) s = TG_ERR_CUDA;
  return s;
}

namespace {
// nodal output values (nnd x 9: stress, then alpha, von Mises, pressure)
int nodal_output(tg_context* c, std::vector<double>& h) {
  double *d_ip = nullptr, *d_out = nullptr;
  if (!ok(c, cudaMallocAsync((void**)&d_ip, sizeof(double) * 72 * (size_t)c->nel, c->stream), "alloc") ||
      !ok(c, cudaMallocAsync((void**)&d_out, sizeof(double) * 9 * (size_t)c->nnd, c->stream), "alloc"))
    return TG_ERR_OOM;
  h.resize((size_t)c->nnd * 9);
  int s = launch_nodal_stress(c, d_ip, d_out);
  if (!s) s = check_status(c);
  if (!s && !copy_sync(c, h.data(), d_out, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, "output"))
    s = TG_ERR_CUDA;
  cudaFreeAsync(d_ip, c->stream);
  cudaFreeAsync(d_out, c->stream);
  if (!ok(c, cudaStreamSynchronize(c->stream), "sync") && !s) s = TG_ERR_CUDA;
  return s;
}
}  // namespace

int tg_nodal_stress(tg_context* c, double* out) {
  if (!c || !out || c->nnd <= 0) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  std::vector<double> h;
  const int s = nodal_output(c, h);
  if (!s)
    for (int n = 0; n < c->nnd; ++n)
      for (int k = 0; k < 6; ++k) out[(size_t)n * 6 + k] = h[(size_t)n * 9 + k];
  return s;
}

int tg_nodal_material_output(tg_context* c, double* out) {
  if (!c || !out || c->nnd <= 0) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  std::vector<double> h;
  const int s = nodal_output(c, h);
  if (!s)
    for (int n = 0; n < c->nnd; ++n)
      for (int k = 0; k < 3; ++k) out[(size_t)n * 3 + k] = h[(size_t)n * 9 + 6 + k];
  return s;
}

// Restart snapshot: a versioned host image of the state needed to resume a
// step sequence bitwise -- displacements and the J2 history arrays (flags,
// allocation, alpha, dgamma, |s|, plastic strain, unit normal).
namespace {
struct StateHeader {
  char magic[8];  // "TGSTATE"
  int version, nnd, nel, has_j2;
  long long bytes;
};
constexpr int kStateVersion = 1;

struct StatePart {
  void* dev;
  size_t bytes;
};

std::vector<StatePart> state_parts(tg_context* c) {
  const size_t nip = (size_t)c->nel * 8;
  std::vector<StatePart> p = {{c->d_u, sizeof(double4_32a) * c->nnd}};
  if (c->has_j2) {
    p.push_back({c->d_j2_flags, nip});
    p.push_back({c->d_j2_alloc, (size_t)c->nel});
    p.push_back({c->d_j2_alpha, sizeof(double) * nip});
    p.push_back({c->d_j2_dgamma, sizeof(double) * nip});
    p.push_back({c->d_j2_norm, sizeof(double) * nip});
    p.push_back({c->d_j2_epsp, sizeof(double) * nip * 6});
    p.push_back({c->d_j2_nhat, sizeof(double) * nip * 6});
  }
  return p;
}

long long state_bytes(tg_context* c) {
  long long b = sizeof(StateHeader);
  for (const StatePart& q : state_parts(c)) b += (long long)((q.bytes + 15) / 16 * 16);
  return b;
}
}  // namespace

int tg_state_size(tg_context* c, long long* bytes) {
  if (!c || !bytes || c->nnd <= 0) return TG_ERR_ARG;
  *bytes = state_bytes(c);
  return TG_OK;
}

int tg_state_save(tg_context* c, void* buf, long long bytes) {
  if (!c || !buf || c->nnd <= 0 || bytes < state_bytes(c)) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  StateHeader h;
  std::memset(&h, 0, sizeof(h));
  std::memcpy(h.magic, "TGSTATE", 8);
  h.version = kStateVersion;
  h.nnd = c->nnd;
  h.nel = c->nel;
  h.has_j2 = c->has_j2 ? 1 : 0;
  h.bytes = state_bytes(c);
  unsigned char* out = static_cast<unsigned char*>(buf);
  std::memcpy(out, &h, sizeof(h));
  size_t off = sizeof(h);
  for (const StatePart& q : state_parts(c)) {
    if (!ok(c, cudaMemcpyAsync(out + off, q.dev, q.bytes, cudaMemcpyDeviceToHost, c->stream), "state")) return TG_ERR_CUDA;
    off += (q.bytes + 15) / 16 * 16;
  }
  return ok(c, cudaStreamSynchronize(c->stream), "sync") ? TG_OK : TG_ERR_CUDA;
}

int tg_state_load(tg_context* c, const void* buf, long long bytes) {
  if (!c || !buf || c->nnd <= 0 || bytes < (long long)sizeof(StateHeader)) return TG_ERR_ARG;
  StateHeader h;
  std::memcpy(&h, buf, sizeof(h));
  if (std::memcmp(h.magic, "TGSTATE", 8) != 0 || h.version != kStateVersion) {
    c->err = "not a state image of this library version";
    return TG_ERR_ARG;
  }
  if (h.nnd != c->nnd || h.nel != c->nel || h.has_j2 != (c->has_j2 ? 1 : 0) || h.bytes != state_bytes(c) ||
      bytes < h.bytes) {
    c->err = "state image does not match the mesh and materials of this context";
    return TG_ERR_ARG;
  }
  if (set_device(c)) return TG_ERR_CUDA;
  const unsigned char* in = static_cast<const unsigned char*>(buf);
  size_t off = sizeof(h);
  for (const StatePart& q : state_parts(c)) {
    if (!ok(c, cudaMemcpyAsync(q.dev, in + off, q.bytes, cudaMemcpyHostToDevice, c->stream), "state")) return TG_ERR_CUDA;
    off += (q.bytes + 15) / 16 * 16;
  }
  c->have_du = false;
  // the device snapshot predates the loaded state: a rollback must not bring
  // it back (the caller checkpoints again once the residual is formed)
  c->ckpt_valid = false;
  return ok(c, cudaStreamSynchronize(c->stream), "sync") ? TG_OK : TG_ERR_CUDA;
}

int tg_get_active_set(tg_context* c, signed char* flags) {
  if (!c || !flags || c->nel <= 0) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  return copy_sync(c, flags, c->d_j2_flags, (size_t)c->nel * 8, cudaMemcpyDeviceToHost, "flags") ? TG_OK
                                                                                                    : TG_ERR_CUDA;
}

int tg_get_j2_state(tg_context* c, double* alpha, double* eps_p) {
  if (!c || c->nel <= 0) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  const size_t nip = (size_t)c->nel * 8;
  if (alpha && !copy_sync(c, alpha, c->d_j2_alpha, sizeof(double) * nip, cudaMemcpyDeviceToHost, "alpha"))
    return TG_ERR_CUDA;
  if (eps_p) {
    std::vector<double> h(nip * 6);
    if (!copy_sync(c, h.data(), c->d_j2_epsp, sizeof(double) * nip * 6, cudaMemcpyDeviceToHost, "epsp"))
      return TG_ERR_CUDA;
    for (size_t g = 0; g < nip; ++g)
      for (int k = 0; k < 6; ++k) eps_p[g * 6 + k] = h[k * nip + g];
  }
  return TG_OK;
}

namespace {
// NLSolver::Solve loop body: tangent, solve, update, residual (NLSolver.cpp:137-188)
int newton_iteration(Context* c, const tg_newton_params* P, double* err, int* its, tg_newton_report* r,
                     PhaseTimer* tm) {
  if (tm) tm->start(c->stream);
  int s = form_tangent(c, P->precision);
  if (tm) r->ms_tangent += tm->stop(c->stream);
  if (s) return s;
  double rr = 0.0;
  *its = 0;
  if (tm) tm->start(c->stream);
  s = pcg_solve(c, c->d_R, P->lin_rel_tol, P->lin_max_it, P->precond, its, &rr);
  if (s == TG_ERR_NOT_CONVERGED) s = TG_OK;  // inexact Newton step; the outer test decides
  if (!s) s = launch_apply_update(c);
  if (tm) r->ms_solve += tm->stop(c->stream);
  if (s) return s;
  c->iteration += 1;
  if (tm) tm->start(c->stream);
  s = residual_norm(c, err, residual_arith(P));
  if (tm) r->ms_residual += tm->stop(c->stream);
  return s;
}
}  // namespace

int tg_newton_iteration(tg_context* c, const tg_newton_params* P, double* norm, int* pcg_iterations) {
  if (!c || !P || c->nnd <= 0) return TG_ERR_ARG;
  if (P->precision != TG_FP64 && P->precision != TG_MIXED) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  tg_newton_report r;
  std::memset(&r, 0, sizeof(r));
  double err = 0.0;
  int its = 0;
  int s = newton_iteration(c, P, &err, &its, &r, nullptr);
  if (norm) *norm = err;
  if (pcg_iterations) *pcg_iterations = its;
  return s;
}
}  // extern "C"

namespace {
int predict(tg_context* c, int n, const int* idx, const double* val, const double* F, const tg_newton_params* P,
            int* pcg_iterations);
}  // namespace

extern "C" {

int tg_newton_solve(tg_context* c, const tg_newton_params* P, tg_newton_report* rep) {
  if (!c || !P || c->nnd <= 0) return TG_ERR_ARG;
  if (P->precision != TG_FP64 && P->precision != TG_MIXED) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  tg_newton_report r;
  std::memset(&r, 0, sizeof(r));
  PhaseTimer tm(rep != nullptr);
  // SolverT::InitStep: iteration -1 for the first residual
  c->iteration = -1;
  tm.start(c->stream);
  double err0 = 0.0;
  int s = residual_norm(c, &err0, residual_arith(P));
  r.ms_residual += tm.stop(c->stream);
  r.error0 = r.error = err0;
  if (s) {
    if (rep) *rep = r;
    return s;
  }
  bool converged = err0 < P->abs_tol;  // "hit on first try"
  while (!converged) {
    double err = 0.0;
    int its = 0;
    s = newton_iteration(c, P, &err, &its, &r, rep ? &tm : nullptr);
    r.pcg_iterations += its;
    if (s) break;
    ++r.iterations;
    r.error = err;
    const double rel = err / err0;
    if (rel > P->div_tol) {
      c->err = "diverging solution";
      s = TG_ERR_DIVERGED;
      break;
    }
    if (rel < P->rel_tol || err < P->abs_tol) {
      converged = true;
    } else if (c->iteration >= P->max_iterations) {
      c->err = "max iterations hit";
      s = TG_ERR_NOT_CONVERGED;
      break;
    }
  }
  if (rep) *rep = r;
  return s;
}

int tg_predict_prescribed(tg_context* c, int n, const int* idx, const double* val, const tg_newton_params* P,
                          int* pcg_iterations) {
  if (!c || !P || n < 0 || (n > 0 && (!idx || !val)) || c->nnd <= 0) return TG_ERR_ARG;
  if (P->precision != TG_FP64 && P->precision != TG_MIXED) return TG_ERR_ARG;
  for (int k = 0; k < n; ++k)
    if (idx[k] < 0 || idx[k] >= c->nnd * 3) return TG_ERR_ARG;
  return predict(c, n, idx, val, nullptr, P, pcg_iterations);
}

int tg_predict_affine(tg_context* c, const double* F, const tg_newton_params* P, int* pcg_iterations) {
  if (!c || !P || !F || c->nnd <= 0 || c->nseg <= 0) return TG_ERR_ARG;
  if (P->precision != TG_FP64 && P->precision != TG_MIXED) return TG_ERR_ARG;
  return predict(c, 0, nullptr, nullptr, F, P, pcg_iterations);
}

}  // extern "C"

namespace {
// The prescribed-increment predictor: the new prescribed values are either
// n (dof, value) pairs or, with F given, the affine field (F_s - I) X of every
// segment on its prescribed dofs.
int predict(tg_context* c, int n, const int* idx, const double* val, const double* F, const tg_newton_params* P,
            int* pcg_iterations) {
  if (set_device(c)) return TG_ERR_CUDA;
  if (pcg_iterations) *pcg_iterations = 0;
  // R(u_old) without committing history, tangent at u_old
  int s = launch_residual_nocommit(c, residual_arith(P));
  if (!s) s = check_status(c);
  if (!s) s = form_tangent(c, P->precision);
  if (s) return s;
  double4_32a *d_old = nullptr, *d_v = nullptr;
  int* d_idx = nullptr;
  double* d_val = nullptr;
  const size_t nb = sizeof(double4_32a) * c->nnd;
  const size_t nval = F ? (size_t)9 * c->nseg : (size_t)std::max(n, 1);
  if (!ok(c, cudaMallocAsync((void**)&d_old, nb, c->stream), "alloc") ||
      !ok(c, cudaMallocAsync((void**)&d_v, nb, c->stream), "alloc") ||
      !ok(c, cudaMallocAsync((void**)&d_idx, sizeof(int) * std::max(n, 1), c->stream), "alloc") ||
      !ok(c, cudaMallocAsync((void**)&d_val, sizeof(double) * nval, c->stream), "alloc"))
    return TG_ERR_OOM;
  if (!ok(c, cudaMemcpyAsync(d_old, c->d_u, nb, cudaMemcpyDeviceToDevice, c->stream), "copy") ||
      (n > 0 && (!ok(c, cudaMemcpyAsync(d_idx, idx, sizeof(int) * n, cudaMemcpyHostToDevice, c->stream), "idx") ||
                 !ok(c, cudaMemcpyAsync(d_val, val, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream), "val"))) ||
      (F && !ok(c, cudaMemcpyAsync(d_val, F, sizeof(double) * nval, cudaMemcpyHostToDevice, c->stream), "F")))
    s = TG_ERR_CUDA;
  // u now carries the new prescribed values
  if (!s) s = F ? launch_affine_prescribed(c, d_val) : launch_set_prescribed(c, n, d_idx, d_val);
  if (!s) s = launch_diff(c, c->d_u, d_old, d_v);         // v = du_p (zero on free dofs)
  if (!s) s = launch_lift_rhs(c, d_v, d_old);             // rhs = R - K v (d_old is free after the diff)
  int its = 0;
  double rr = 0.0;
  if (!s) {
    s = pcg_solve(c, d_old, P->lin_rel_tol, P->lin_max_it, P->precond, &its, &rr);
    if (s == TG_ERR_NOT_CONVERGED) s = TG_OK;
  }
  if (!s) s = launch_apply_update(c);
  cudaFreeAsync(d_old, c->stream);
  cudaFreeAsync(d_v, c->stream);
  cudaFreeAsync(d_idx, c->stream);
  cudaFreeAsync(d_val, c->stream);
  if (!ok(c, cudaStreamSynchronize(c->stream), "sync") && !s) s = TG_ERR_CUDA;
  if (pcg_iterations) *pcg_iterations = its;
  return s;
}
}  // namespace

extern "C" {

int tg_set_segments(tg_context* c, int nseg, const int* node_off, const int* elem_off) {
  if (!c || nseg <= 0 || !node_off || !elem_off || c->nnd <= 0) return TG_ERR_ARG;
  if (node_off[0] != 0 || node_off[nseg] != c->nnd || elem_off[0] != 0 || elem_off[nseg] != c->nel) return TG_ERR_ARG;
  for (int s = 0; s < nseg; ++s)
    if (node_off[s + 1] < node_off[s] || elem_off[s + 1] < elem_off[s]) return TG_ERR_ARG;
  if (set_device(c) || ensure_host_mesh(c)) return TG_ERR_CUDA;
  // elements of RVE s may only reference nodes of RVE s
  for (int s = 0; s < nseg; ++s)
    for (long long k = (long long)elem_off[s] * 8; k < (long long)elem_off[s + 1] * 8; ++k)
      if (c->h_conn[k] < node_off[s] || c->h_conn[k] >= node_off[s + 1]) {
        c->err = "element of RVE " + std::to_string(s) + " references a node outside it";
        return TG_ERR_ARG;
      }
  if (set_device(c)) return TG_ERR_CUDA;
  for (void** p : {(void**)&c->d_seg_node, (void**)&c->d_seg_elem, (void**)&c->d_seg_out}) {
    if (*p) dfree(c, *p);
    *p = nullptr;
  }
  seg_free(c);  // the per-RVE solve's chunks follow the partition
  c->nseg = nseg;
  c->h_seg_node.assign(node_off, node_off + nseg + 1);
  c->h_seg_elem.assign(elem_off, elem_off + nseg + 1);
  if (!dalloc(c, &c->d_seg_node, (size_t)nseg + 1) || !dalloc(c, &c->d_seg_elem, (size_t)nseg + 1) ||
      !dalloc(c, &c->d_seg_out, (size_t)nseg * 9))
    return TG_ERR_OOM;
  return copy_sync(c, c->d_seg_node, node_off, sizeof(int) * (nseg + 1), cudaMemcpyHostToDevice, "seg") &&
                 copy_sync(c, c->d_seg_elem, elem_off, sizeof(int) * (nseg + 1), cudaMemcpyHostToDevice, "seg")
             ? TG_OK
             : TG_ERR_CUDA;
}

int tg_segment_residual_norms(tg_context* c, double* norms) {
  if (!c || !norms || c->nseg <= 0) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  int s = launch_segment_norms(c, c->nseg, c->d_seg_node, c->d_seg_out);
  if (!s && (!ok(c, cudaMemcpyAsync(norms, c->d_seg_out, sizeof(double) * c->nseg, cudaMemcpyDeviceToHost, c->stream),
                 "norms") ||
             !ok(c, cudaStreamSynchronize(c->stream), "sync")))
    s = TG_ERR_CUDA;
  if (!s)
    for (int i = 0; i < c->nseg; ++i) norms[i] = std::sqrt(norms[i]);
  return s;
}

int tg_segment_average_stress(tg_context* c, const double* vol0, double* P) {
  if (!c || !P || c->nseg <= 0) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  int s = launch_segment_stress(c, c->nseg, c->d_seg_elem, c->d_seg_out);
  if (!s &&
      (!ok(c, cudaMemcpyAsync(P, c->d_seg_out, sizeof(double) * 9 * c->nseg, cudaMemcpyDeviceToHost, c->stream), "P") ||
       !ok(c, cudaStreamSynchronize(c->stream), "sync")))
    s = TG_ERR_CUDA;
  if (!s && vol0)
    for (int i = 0; i < c->nseg; ++i)
      for (int k = 0; k < 9; ++k) P[i * 9 + k] /= vol0[i];
  return s;
}

int tg_segment_macro_tangent(tg_context* c, const tg_newton_params* P, const double* vol0, double* C,
                             int* pcg_iterations) {
  if (!c || !P || !C || c->nseg <= 0 || c->nnd <= 0) return TG_ERR_ARG;
  if (P->precision != TG_FP64 && P->precision != TG_MIXED) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  if (pcg_iterations) *pcg_iterations = 0;
  // tangent at the current (converged) state
  int s = form_tangent(c, P->precision);
  if (s) return s;
  double *d_vol = nullptr, *d_C = nullptr;
  if (!ok(c, cudaMallocAsync((void**)&d_C, sizeof(double) * 81 * c->nseg, c->stream), "alloc") ||
      (vol0 && !ok(c, cudaMallocAsync((void**)&d_vol, sizeof(double) * c->nseg, c->stream), "alloc")))
    return TG_ERR_OOM;
  if (vol0 && !ok(c, cudaMemcpyAsync(d_vol, vol0, sizeof(double) * c->nseg, cudaMemcpyHostToDevice, c->stream), "vol"))
    s = TG_ERR_CUDA;
  int total = 0;
  // columns kL: boundary perturbations v = dF X with dF = e_k (x) e_L,
  // interior responses K_ii du_i = -K_ib v_b (nine right-hand sides, one
  // multi-vector PCG), dP = (1/V0) sum_a (K w)_a (x) X_a with w = v + du
  if (!s) s = macro_tangent_mrhs(c, P->precision, P->precond, P->lin_rel_tol, P->lin_max_it, d_vol, d_C, &total);
  if (!s && !ok(c, cudaMemcpyAsync(C, d_C, sizeof(double) * 81 * c->nseg, cudaMemcpyDeviceToHost, c->stream), "C"))
    s = TG_ERR_CUDA;
  for (void* p : {(void*)d_C, (void*)d_vol})
    if (p) cudaFreeAsync(p, c->stream);
  if (!ok(c, cudaStreamSynchronize(c->stream), "sync") && !s) s = TG_ERR_CUDA;
  if (pcg_iterations) *pcg_iterations = total;
  return s;
}

int tg_newton_solve_segmented(tg_context* c, const tg_newton_params* P, tg_newton_report* rep, double* seg_rel,
                              int* seg_status) {
  if (!c || !P || c->nseg <= 0) return TG_ERR_ARG;
  if (P->precision != TG_FP64 && P->precision != TG_MIXED) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  tg_newton_report r;
  std::memset(&r, 0, sizeof(r));
  PhaseTimer tm(rep != nullptr);
  c->iteration = -1;
  const int ns = c->nseg;
  std::vector<double> n0(ns), nk(ns);
  double err0 = 0.0;
  tm.start(c->stream);
  int s = residual_norm(c, &err0, residual_arith(P));
  if (!s) s = tg_segment_residual_norms(c, n0.data());
  r.ms_residual += tm.stop(c->stream);
  r.error0 = r.error = err0;
  nk = n0;
  // NLSolver::ExitIteration per RVE (NLSolver.cpp:675-755): converged when
  // rel < rel_tol or the absolute norm < abs_tol, diverged when rel >
  // div_tol, failed at the iteration limit.
  const int kRunning = 1;
  std::vector<int> state(ns, kRunning);  // kRunning, TG_OK, or the RVE's failure code
  auto converged = [&](int i) {
    const double rel = n0[i] > 0.0 ? nk[i] / n0[i] : 0.0;
    return rel < P->rel_tol || nk[i] < P->abs_tol;
  };
  for (int i = 0; i < ns; ++i)
    if (n0[i] < P->abs_tol) state[i] = TG_OK;  // "hit on first try"
  const bool per_rve = c->seg_pcg_mode != 0;
  auto running = [&]() {
    int k = 0;
    for (int v : state) k += v == kRunning ? 1 : 0;
    return k;
  };
  while (!s && running() > 0) {
    // with per-RVE Krylov solves an RVE that has converged or failed is
    // frozen (no further update) and fails alone; the batch-wide solve
    // updates every RVE until all have converged
    if (per_rve) {
      c->seg_active.assign(ns, 0);
      for (int i = 0; i < ns; ++i) c->seg_active[i] = state[i] == kRunning ? 1 : 0;
      c->seg_tolerate = true;
    }
    double err = 0.0;
    int its = 0;
    s = newton_iteration(c, P, &err, &its, &r, rep ? &tm : nullptr);
    c->seg_tolerate = false;
    r.pcg_iterations += its;
    if (s) break;
    ++r.iterations;
    r.error = err;
    s = tg_segment_residual_norms(c, nk.data());
    if (s) break;
    if (per_rve) {
      for (int i = 0; i < ns; ++i) {
        if (state[i] != kRunning) continue;
        const double rel = n0[i] > 0.0 ? nk[i] / n0[i] : 0.0;
        if ((int)c->seg_status.size() == ns && c->seg_status[i] == TG_ERR_NAN) state[i] = TG_ERR_NAN;
        else if (converged(i)) state[i] = TG_OK;
        else if (rel > P->div_tol) state[i] = TG_ERR_DIVERGED;
        else if (c->iteration >= P->max_iterations) state[i] = TG_ERR_NOT_CONVERGED;
      }
    } else {
      double worst = 0.0;
      bool all = true;
      for (int i = 0; i < ns; ++i) {
        all = all && converged(i);
        if (n0[i] > 0.0) worst = std::max(worst, nk[i] / n0[i]);
      }
      if (all) {
        std::fill(state.begin(), state.end(), (int)TG_OK);
      } else if (worst > P->div_tol) {
        c->err = "diverging RVE";
        s = TG_ERR_DIVERGED;
      } else if (c->iteration >= P->max_iterations) {
        c->err = "max iterations hit";
        s = TG_ERR_NOT_CONVERGED;
      }
    }
  }
  c->seg_active.clear();
  int failed = 0, first_fail = TG_OK;
  for (int i = 0; i < ns; ++i) {
    if (state[i] == kRunning) state[i] = s;
    if (state[i] != TG_OK) {
      ++failed;
      if (first_fail == TG_OK) first_fail = state[i];
    }
  }
  if (seg_rel)
    for (int i = 0; i < ns; ++i) seg_rel[i] = n0[i] > 0.0 ? nk[i] / n0[i] : 0.0;
  if (seg_status)
    for (int i = 0; i < ns; ++i) seg_status[i] = state[i];
  if (rep) *rep = r;
  if (s) return s;
  if (failed) {
    c->err = std::to_string(failed) + " of " + std::to_string(ns) + " RVEs failed (status per RVE)";
    return first_fail;
  }
  return TG_OK;
}

int tg_checkpoint(tg_context* c) {
  if (!c || c->nnd <= 0) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  if (!c->d_u_ckpt && (!dalloc(c, &c->d_u_ckpt, (size_t)c->nnd) || !dalloc(c, &c->d_R_ckpt, (size_t)c->nnd)))
    return TG_ERR_OOM;
  const size_t n = sizeof(double4_32a) * c->nnd;
  if (!ok(c, cudaMemcpyAsync(c->d_u_ckpt, c->d_u, n, cudaMemcpyDeviceToDevice, c->stream), "ckpt") ||
      !ok(c, cudaMemcpyAsync(c->d_R_ckpt, c->d_R, n, cudaMemcpyDeviceToDevice, c->stream), "ckpt"))
    return TG_ERR_CUDA;
  c->ckpt_valid = true;
  return TG_OK;
}

int tg_rollback(tg_context* c) {
  if (!c) return TG_ERR_ARG;
  if (!c->d_u_ckpt || !c->ckpt_valid) {
    c->err = "tg_rollback: no checkpoint of the current state (take one with tg_checkpoint)";
    return TG_ERR_ARG;
  }
  const size_t n = sizeof(double4_32a) * c->nnd;
  return ok(c, cudaMemcpyAsync(c->d_u, c->d_u_ckpt, n, cudaMemcpyDeviceToDevice, c->stream), "rollback") &&
                 ok(c, cudaMemcpyAsync(c->d_R, c->d_R_ckpt, n, cudaMemcpyDeviceToDevice, c->stream), "rollback")
             ? TG_OK
             : TG_ERR_CUDA;
}

int tg_timer_start(tg_context* c) {
  if (!c) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  if (!c->ev_a && (!ok(c, cudaEventCreate(&c->ev_a), "event") || !ok(c, cudaEventCreate(&c->ev_b), "event")))
    return TG_ERR_CUDA;
  return ok(c, cudaEventRecord(c->ev_a, c->stream), "event") ? TG_OK : TG_ERR_CUDA;
}

int tg_timer_stop(tg_context* c, double* ms) {
  if (!c || !c->ev_a || !ms) return TG_ERR_ARG;
  float e = 0.f;
  if (!ok(c, cudaEventRecord(c->ev_b, c->stream), "event") || !ok(c, cudaEventSynchronize(c->ev_b), "event") ||
      !ok(c, cudaEventElapsedTime(&e, c->ev_a, c->ev_b), "event"))
    return TG_ERR_CUDA;
  *ms = e;
  return TG_OK;
}

int tg_time_kernel(tg_context* c, int which, int reps, double* ms) {
  if (!c || reps <= 0 || !ms || which < 0 || which > 5) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  if (which <= 1) return time_pcg_kernel(c, which, reps, ms);
  if ((which == 2 || which == 3) && c->tangent_precision < 0) {
    c->err = "form a tangent first (its precision is the one timed)";
    return TG_ERR_ARG;
  }
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  double total = 0.0;
  int s = TG_OK;
  for (int r = 0; r < reps && !s; ++r) {
    cudaEventRecord(a, c->stream);
    if (which == 2) s = launch_tangent(c, c->tangent_precision);
    else if (which == 3) {
      // the assembly the solve uses (the values do not change: the same
      // element blocks, the same order)
      if (push_solve(c)) {
        s = launch_assemble_upper(c, c->tangent_precision);
      } else {
        s = ensure_blob(c, c->tangent_precision);
        if (!s) s = launch_assemble(c, c->tangent_precision);
        if (!s) (c->tangent_precision == TG_MIXED ? c->full_serial32 : c->full_serial64) = c->tangent_serial;
        if (!s && sym_active(c)) s = sym_convert(c, c->tangent_precision);
      }
    }
    else s = launch_residual(c, which == 5 ? kResidualDoubleFloat : kResidualFP64);
    cudaEventRecord(b, c->stream);
    cudaEventSynchronize(b);
    float e = 0.f;
    cudaEventElapsedTime(&e, a, b);
    total += e;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (!s) s = check_status(c);
  *ms = total / reps;
  return s;
}

}  // extern "C"
