// Single-reduction PCG on the streamed node-block matrix, sm_103a.
//
// (Block-)Jacobi CG in the single-reduction form of Chronopoulos & Gear
// (J. Comput. Appl. Math. 25 (1989) 153-168), two kernels per iteration and
// no grid-wide synchronisation inside either of them:
//
//   product  w = A u; each CTA writes its partial of u.w
//            (pcg_spmv_kernel with CTA partials only)
//   vector   every CTA forms delta = u.w, gamma = r.u and r.r from the CTA
//            partials of the two kernels before it (visible through the
//            kernel boundary), in the same fixed order in every CTA; tests
//            convergence; forms beta = gamma / gamma_old and
//            alpha = gamma / (delta - beta gamma / alpha_old); and runs one
//            pass p = u + beta p, s = w + beta s (s = A p by recurrence),
//            x += alpha p, r -= alpha s, u = M^-1 r with its CTA partials of
//            the next r.u and r.r
//
// A kernel boundary inside a CUDA graph costs well under a microsecond on
// GB300, while a software grid barrier or a last-block reduction costs
// several (arrival atomics, fences and a second round trip for the values),
// and the textbook recurrences need two reductions with a dependent vector
// pass between them.  Here both reductions ride on the kernel boundaries and
// every CTA repeats the short sums of the partials itself.
//
// State hand-off without races: a vector kernel reads the iteration state
// from scalars[0] and its CTA 0 writes the next state to scalars[1]; the
// next product kernel copies scalars[1] to scalars[0] before anything reads
// it.  The partials of r.u and r.r alternate between two buffers by
// iteration parity, so a kernel never overwrites partials its own CTAs are
// still summing.  Convergence of an update is seen by the next vector
// kernel, which then leaves every vector as it is.
//
// This solves the same system as the textbook two-kernel form in krylov.cu
// (NLSolver_NK's Krylov solve with DiagonalMatrixT::BackSubstitute as
// preconditioner and MSRMatrixT::Multx as product, NLSolver_NK.cpp:121,
// DiagonalMatrixT.cpp:313, MSRMatrixT.cpp:385) to the same tolerance; the
// iterates differ from the textbook recurrences' by rounding.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "krylov_common.cuh"

namespace tg {

namespace {

constexpr int kCgChunk = 16;       // iterations per graph replay
constexpr int kCgThreads = 256;
constexpr int kDeltaCap = 2048;    // product CTAs (the persistent product grid is far smaller)
constexpr int kVecCap = 1024;      // vector-kernel CTAs
// partials (doubles): product u.w at [0, kDeltaCap); then two buffers of
// {r.u [kVecCap], r.r [kVecCap]}
constexpr int kCgPartials = kDeltaCap + 4 * kVecCap;

// One node per thread per pass: with 4 (FP32) or 2 (FP64) CTAs of 256
// threads per SM, 1024 / 512 nodes are in flight per SM, enough to cover the
// L2 latency of the vector pass (its vectors stay L2-resident).
template <typename T>
struct CgUnroll {
  static constexpr int value = 1;
  static constexpr int ctas_per_sm = sizeof(T) == 4 ? 4 : 2;
};

template <typename T>
__global__ void __launch_bounds__(kCgThreads, CgUnroll<T>::ctas_per_sm) pcg_cg_vector_kernel(
    int nnd, const T* __restrict__ minv, typename Vec4<T>::type* __restrict__ x,
    typename Vec4<T>::type* __restrict__ r, typename Vec4<T>::type* __restrict__ u,
    typename Vec4<T>::type* __restrict__ p, typename Vec4<T>::type* __restrict__ s,
    const typename Vec4<T>::type* __restrict__ w, const double* __restrict__ dpart, int ndp, double* vpart,
    PcgScalars* sc) {
  using V = typename Vec4<T>::type;
  using P = typename Partial<T>::type;
  constexpr int U = CgUnroll<T>::value;
  __shared__ double coef[2];  // alpha, beta
  __shared__ int go;
  if (((volatile PcgScalars*)sc)->done) return;
  const int it = sc->iters;  // updates done so far: the same in every CTA (scalars[0] is not written here)
  const P* dp = reinterpret_cast<const P*>(dpart);
  const P* prev = reinterpret_cast<const P*>(vpart + kDeltaCap + (size_t)(it & 1) * 2 * kVecCap);
  P* next = reinterpret_cast<P*>(vpart + kDeltaCap + (size_t)((it + 1) & 1) * 2 * kVecCap);
  {
    // totals of the product's u.w and the last vector kernel's r.u, r.r:
    // thread-strided sums in a fixed order, then the fixed block tree, in
    // the accumulator's arithmetic (compensated FP32 in the FP32 form)
    Acc<T> a[3];
    for (int b = threadIdx.x; b < ndp; b += blockDim.x) acc_merge(a[0], dp[b]);
    if (it > 0)
      for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
        acc_merge(a[1], prev[b]);
        acc_merge(a[2], prev[kVecCap + b]);
      }
    P tot[3];
    block_total_acc<T, 3>(a, tot);
    if (threadIdx.x == 0) {
      PcgScalars o = *sc;
      const double delta = partial_value(tot[0]);
      const double gamma = it > 0 ? partial_value(tot[1]) : o.rz;
      const double rr = it > 0 ? partial_value(tot[2]) : o.rr;
      int done = 0, fail = 0;
      double alpha = 0.0, beta = 0.0;
      if (!isfinite(gamma) || !isfinite(rr)) {
        done = 2;
        fail = 4;
      } else if (it > 0 && rr <= o.tol2 * o.rr0) {
        done = 1;
      } else if (it >= o.max_it) {
        done = 3;
      } else {
        double den = delta;
        if (it > 0) {
          beta = gamma / o.rz;  // o.rz, o.alpha: the last update's gamma and alpha
          den = delta - beta * gamma / o.alpha;
        }
        if (!(den > 0.0) || !isfinite(den)) {
          done = 2;
          fail = isfinite(den) ? 2 : 3;
        } else {
          alpha = gamma / den;
        }
      }
      coef[0] = alpha;
      coef[1] = beta;
      go = done == 0;
      if (blockIdx.x == 0) {
        o.pq = delta;
        o.rr = rr;
        if (done) {
          o.done = done;
          if (fail) o.fail = fail;
        } else {
          o.rz_old = o.rz;
          o.rz = gamma;
          o.alpha = alpha;
          o.beta = beta;
          o.iters = it + 1;
        }
        sc[1] = o;
      }
    }
    __syncthreads();
  }
  if (!go) return;
  const T a_ = T(coef[0]), b_ = T(coef[1]);
  const bool first = it == 0;
  Acc<T> acc[2];
  const int step = gridDim.x * blockDim.x * U;
  for (int base = blockIdx.x * blockDim.x * U + threadIdx.x; base < nnd; base += step) {
    V un[U], wn[U], pn[U], sn[U], xn[U], rn[U];
    T B[U][9];
#pragma unroll
    for (int k = 0; k < U; ++k) {
      const int n = base + k * blockDim.x;
      if (n < nnd) {
        un[k] = u[n];
        wn[k] = w[n];
        pn[k] = p[n];
        sn[k] = s[n];
        xn[k] = x[n];
        rn[k] = r[n];
#pragma unroll
        for (int m = 0; m < 9; ++m) B[k][m] = minv[(long long)n * 9 + m];
      }
    }
#pragma unroll
    for (int k = 0; k < U; ++k) {
      const int n = base + k * blockDim.x;
      if (n < nnd) {
        V pv, sv;
        if (first) {  // p = u, s = w (p and s hold nothing yet)
          pv = un[k];
          sv = wn[k];
        } else {
          pv = mk<V, T>(un[k].x + b_ * pn[k].x, un[k].y + b_ * pn[k].y, un[k].z + b_ * pn[k].z);
          sv = mk<V, T>(wn[k].x + b_ * sn[k].x, wn[k].y + b_ * sn[k].y, wn[k].z + b_ * sn[k].z);
        }
        const T rx = rn[k].x - a_ * sv.x, ry = rn[k].y - a_ * sv.y, rz = rn[k].z - a_ * sv.z;
        const T zx = B[k][0] * rx + B[k][1] * ry + B[k][2] * rz;
        const T zy = B[k][3] * rx + B[k][4] * ry + B[k][5] * rz;
        const T zz = B[k][6] * rx + B[k][7] * ry + B[k][8] * rz;
        p[n] = pv;
        s[n] = sv;
        x[n] = mk<V, T>(xn[k].x + a_ * pv.x, xn[k].y + a_ * pv.y, xn[k].z + a_ * pv.z);
        r[n] = mk<V, T>(rx, ry, rz);
        u[n] = mk<V, T>(zx, zy, zz);
        acc[0].add_prod(rx, zx);
        acc[0].add_prod(ry, zy);
        acc[0].add_prod(rz, zz);
        acc[1].add_prod(rx, rx);
        acc[1].add_prod(ry, ry);
        acc[1].add_prod(rz, rz);
      }
    }
  }
  P bt[2];
  block_total_acc<T, 2>(acc, bt);
  if (threadIdx.x == 0) {
    next[blockIdx.x] = bt[0];
    next[kVecCap + blockIdx.x] = bt[1];
  }
}

// as many CTAs as are resident at once (grid-stride over the nodes)
template <typename T>
int vec_grid(Context* c, int* grid) {
  int per_sm = 0;
  if (!ok(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pcg_cg_vector_kernel<T>, kCgThreads, 0),
          "occupancy"))
    return TG_ERR_CUDA;
  const int per = kCgThreads * CgUnroll<T>::value;
  *grid = std::max(1, std::min({(c->nnd + per - 1) / per, c->num_sms * std::max(per_sm, 1), kVecCap}));
  return TG_OK;
}

template <typename T>
int capture(Context* c, int precision, const T* minv) {
  using V = typename Vec4<T>::type;
  SpmvPlan plan;
  int s = spmv_plan(c, precision, plan);
  if (s) return s;
  if (plan.sym || plan.spmv > kDeltaCap) {
    c->err = "single-reduction PCG: product launch shape out of range";
    return TG_ERR_CAPACITY;
  }
  int nv = 0;
  s = vec_grid<T>(c, &nv);
  if (s) return s;
  cudaGraph_t graph;
  if (!ok(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture")) return TG_ERR_CUDA;
  cudaError_t le = cudaSuccess;
  for (int k = 0; k < kCgChunk && le == cudaSuccess; ++k) {
    spmv_run(c, precision, plan, c->d_z, c->d_q, c->d_partials, c->d_pcg, nullptr, 1);
    le = cudaGetLastError();
    if (le != cudaSuccess) break;
    pcg_cg_vector_kernel<T><<<nv, kCgThreads, 0, c->stream>>>(c->nnd, minv, (V*)c->d_x, (V*)c->d_r, (V*)c->d_z,
                                                              (V*)c->d_p, (V*)c->d_cg_s, (const V*)c->d_q,
                                                              c->d_partials, plan.spmv, c->d_partials, c->d_pcg);
    le = cudaGetLastError();
  }
  const cudaError_t ee = cudaStreamEndCapture(c->stream, &graph);
  if (!ok(c, le, "capture launch") || !ok(c, ee, "end capture")) {
    if (ee == cudaSuccess) cudaGraphDestroy(graph);
    return TG_ERR_CUDA;
  }
  cg_free(c);
  const cudaError_t e = cudaGraphInstantiate(&c->cg_graph, graph, 0);
  cudaGraphDestroy(graph);
  return ok(c, e, "graph instantiate") ? TG_OK : TG_ERR_CUDA;
}

template <typename T>
int solve_cg_t(Context* c, int precision, const double4_32a* d_rhs, double rel_tol, int max_it, int precond,
               int* iters, double* rel_res) {
  using V = typename Vec4<T>::type;
  static_assert(kCgPartials <= 8192, "partials buffer");
  if (c->partials_cap * 2 < kCgPartials) {
    c->err = "single-reduction PCG: partials buffer too small";
    return TG_ERR_CAPACITY;
  }
  int s = pcg_vectors(c, precision);
  if (s) return s;
  if (!c->d_cg_s || c->cg_s_precision != precision) {
    if (c->d_cg_s) dfree(c, c->d_cg_s);
    c->d_cg_s = nullptr;
    V* v = nullptr;
    if (!dalloc(c, &v, (size_t)c->nnd)) return TG_ERR_OOM;
    c->d_cg_s = v;
    c->cg_s_precision = precision;
    cg_free(c);
  }
  const T* minv_base = std::is_same<T, float>::value ? (const T*)c->d_minv32 : (const T*)c->d_minv64;
  const T* minv = minv_base + (precond == TG_PRECOND_BLOCK_JACOBI ? (long long)c->nnd * 9 : 0);
  s = pcg_start(c, precision, d_rhs, minv, rel_tol, max_it);
  if (s) return s;
  // the first product copies scalars[1] to scalars[0]: start them equal
  if (!ok(c, cudaMemcpyAsync(c->d_pcg + 1, c->d_pcg, sizeof(PcgScalars), cudaMemcpyDeviceToDevice, c->stream),
          "scalars"))
    return TG_ERR_CUDA;
  const int key = precision * 2 + (precond == TG_PRECOND_BLOCK_JACOBI ? 1 : 0);
  if (!c->cg_graph || c->cg_graph_key != key) {
    s = capture<T>(c, precision, minv);
    if (s) return s;
    c->cg_graph_key = key;
  }
  // each chunk's scalars go to alternating pinned mirrors; the host reads a
  // chunk's flag while the next chunk runs
  const int max_chunks = max_it / kCgChunk + 2;
  int last = 0;
  for (int k = 0; k < max_chunks; ++k) {
    if (!ok(c, cudaGraphLaunch(c->cg_graph, c->stream), "graph launch")) return TG_ERR_CUDA;
    c->launches += 2 * kCgChunk;
    last = k & 1;
    if (!ok(c, cudaMemcpyAsync(&c->h_pcg[last], c->d_pcg + 1, sizeof(PcgScalars), cudaMemcpyDeviceToHost,
                               c->stream),
            "copy") ||
        !ok(c, cudaEventRecord(c->ev_poll[last], c->stream), "event"))
      return TG_ERR_CUDA;
    if (k > 0) {
      if (!ok(c, cudaEventSynchronize(c->ev_poll[last ^ 1]), "pcg poll")) return TG_ERR_CUDA;
      if (c->h_pcg[last ^ 1].done) break;
    }
  }
  if (!ok(c, cudaStreamSynchronize(c->stream), "pcg sync")) return TG_ERR_CUDA;
  return pcg_finish(c, c->h_pcg[last], iters, rel_res);
}

}  // namespace

void cg_free(Context* c) {
  if (c->cg_graph) cudaGraphExecDestroy(c->cg_graph);
  c->cg_graph = nullptr;
  c->cg_graph_key = -1;
}

int pcg_solve_cg(Context* c, int precision, const double4_32a* d_rhs, double rel_tol, int max_it, int precond,
                 int* iters, double* rel_res) {
  if (precision == TG_MIXED) return solve_cg_t<float>(c, precision, d_rhs, rel_tol, max_it, precond, iters, rel_res);
  return solve_cg_t<double>(c, precision, d_rhs, rel_tol, max_it, precond, iters, rel_res);
}

}  // namespace tg
