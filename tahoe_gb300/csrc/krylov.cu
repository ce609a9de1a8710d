// (Block-)Jacobi preconditioned CG on the node-block CSR matrix, sm_103a.
//
// Each iteration is two kernels:
//   pcg_spmv_kernel   w = A z; q = w + beta q; p = z + beta p; partial p.q
//                     (uses A p = A z + beta A p_old, so the product runs on z,
//                     which is complete when the kernel starts)
//   pcg_update_kernel x += alpha p; r -= alpha q; z = M^-1 r; partial r.z, r.r
// Both end in a last-block-done reduction of their FP64 partial sums in a
// fixed order (bitwise repeatable, no floating-point atomics) that also
// computes alpha / beta and the convergence flag on the device.  Iterations
// run in chunks captured once in a CUDA graph; kernels return immediately
// once the flag is set, and the host polls the flag between chunks.
//
// Vectors are stored per node, padded to 4 lanes (float4 in the mixed form,
// double4_32a in the plain FP64 form).  Dot products and norms accumulate in
// FP64 in both forms.  This replaces the reference's Krylov/diagonal solve
// (NLSolver_NK::GMRES, NLSolver_NK.cpp:121; DiagonalMatrixT::BackSubstitute,
// DiagonalMatrixT.cpp:313; MSRMatrixT::Multx, MSRMatrixT.cpp:385).
#include <cmath>
#include <cstring>
#include <string>

#include "tg_internal.h"

namespace tg {

namespace {

constexpr int kChunk = 16;  // PCG iterations per graph replay

template <typename T> struct Vec4;
template <> struct Vec4<float> { using type = float4; };
template <> struct Vec4<double> { using type = double4_32a; };

template <typename V, typename T>
__device__ __forceinline__ V mk(T x, T y, T z) {
  V v;
  v.x = x;
  v.y = y;
  v.z = z;
  v.w = T(0);
  return v;
}

// block-wide sum of `nv` doubles; results valid in thread 0
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* sh /* NV*32 */) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[k * 32 + w] = v[k];
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double x = lane < nw ? sh[k * 32 + lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
      v[k] = x;
    }
  }
}

// last-block reduction of per-block partials (layout partials[k*gridDim + b]);
// returns true in the last block, with totals in `tot` on thread 0
template <int NV>
__device__ __forceinline__ bool last_block_total(double (&v)[NV], double* partials, unsigned int* counter,
                                                 double (&tot)[NV]) {
  __shared__ double sh[NV * 32];
  __shared__ bool last;
  block_sum<NV>(v, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) partials[k * gridDim.x + blockIdx.x] = v[k];
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double acc[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    acc[k] = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) acc[k] += ((volatile double*)partials)[k * gridDim.x + b];
  }
  __syncthreads();
  block_sum<NV>(acc, sh);
#pragma unroll
  for (int k = 0; k < NV; ++k) tot[k] = acc[k];
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

template <typename T>
__device__ __forceinline__ void apply_minv(const T* __restrict__ minv, int n, T rx, T ry, T rz, T& zx, T& zy, T& zz) {
  const T* B = minv + (long long)n * 9;
  zx = B[0] * rx + B[1] * ry + B[2] * rz;
  zy = B[3] * rx + B[4] * ry + B[5] * rz;
  zz = B[6] * rx + B[7] * ry + B[8] * rz;
}

template <typename T>
__global__ void __launch_bounds__(256) pcg_init_kernel(int nnd, const double4_32a* __restrict__ rhs,
                                                       const uint8_t* __restrict__ mask, const T* __restrict__ minv,
                                                       typename Vec4<T>::type* x, typename Vec4<T>::type* r,
                                                       typename Vec4<T>::type* z, typename Vec4<T>::type* p,
                                                       typename Vec4<T>::type* q, double* partials, PcgScalars* sc,
                                                       double tol, int max_it) {
  using V = typename Vec4<T>::type;
  double v[2] = {0.0, 0.0};
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nnd; n += gridDim.x * blockDim.x) {
    const double4_32a b = rhs[n];
    const uint8_t mk_ = mask[n];
    const T rx = (mk_ & 1) ? T(b.x) : T(0), ry = (mk_ & 2) ? T(b.y) : T(0), rz = (mk_ & 4) ? T(b.z) : T(0);
    T zx, zy, zz;
    apply_minv<T>(minv, n, rx, ry, rz, zx, zy, zz);
    x[n] = mk<V, T>(T(0), T(0), T(0));
    r[n] = mk<V, T>(rx, ry, rz);
    z[n] = mk<V, T>(zx, zy, zz);
    p[n] = mk<V, T>(T(0), T(0), T(0));
    q[n] = mk<V, T>(T(0), T(0), T(0));
    v[0] += (double)rx * zx + (double)ry * zy + (double)rz * zz;
    v[1] += (double)rx * rx + (double)ry * ry + (double)rz * rz;
  }
  double tot[2];
  if (last_block_total<2>(v, partials, &sc->count_b, tot) && threadIdx.x == 0) {
    sc->rz = tot[0];
    sc->rr = tot[1];
    sc->rr0 = tot[1];
    sc->beta = 0.0;
    sc->alpha = 0.0;
    sc->iters = 0;
    sc->tol2 = tol * tol;
    sc->max_it = max_it;
    sc->count_a = 0u;
    sc->fail = 0;
    sc->done = (tot[1] == 0.0) ? 1 : (isfinite(tot[0]) && isfinite(tot[1]) ? 0 : 2);
    if (sc->done == 2) sc->fail = 1;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) pcg_spmv_kernel(int nnd, const int* __restrict__ rowptr,
                                                       const int* __restrict__ col, const T* __restrict__ vals,
                                                       long long stride, const typename Vec4<T>::type* __restrict__ z,
                                                       typename Vec4<T>::type* __restrict__ p,
                                                       typename Vec4<T>::type* __restrict__ q, double* partials,
                                                       PcgScalars* sc) {
  using V = typename Vec4<T>::type;
  if (((volatile PcgScalars*)sc)->done) return;
  const T beta = T(sc->beta);
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  double v[1] = {0.0};
  for (int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; I < nnd; I += warps) {
    T a0 = T(0), a1 = T(0), a2 = T(0);
    const int r1 = rowptr[I + 1];
    for (int j = rowptr[I] + lane; j < r1; j += 32) {
      const V zj = z[col[j]];
      a0 += vals[0 * stride + j] * zj.x + vals[1 * stride + j] * zj.y + vals[2 * stride + j] * zj.z;
      a1 += vals[3 * stride + j] * zj.x + vals[4 * stride + j] * zj.y + vals[5 * stride + j] * zj.z;
      a2 += vals[6 * stride + j] * zj.x + vals[7 * stride + j] * zj.y + vals[8 * stride + j] * zj.z;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, o);
      a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if (lane == 0) {
      const V zi = z[I], pi = p[I], qi = q[I];
      const V qn = mk<V, T>(a0 + beta * qi.x, a1 + beta * qi.y, a2 + beta * qi.z);
      const V pn = mk<V, T>(zi.x + beta * pi.x, zi.y + beta * pi.y, zi.z + beta * pi.z);
      q[I] = qn;
      p[I] = pn;
      v[0] += (double)pn.x * qn.x + (double)pn.y * qn.y + (double)pn.z * qn.z;
    }
  }
  double tot[1];
  if (last_block_total<1>(v, partials, &sc->count_a, tot) && threadIdx.x == 0) {
    sc->pq = tot[0];
    if (!(tot[0] > 0.0) || !isfinite(tot[0])) {
      sc->done = 2;
      sc->fail = isfinite(tot[0]) ? 2 : 3;
    } else {
      sc->alpha = sc->rz / tot[0];
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(256) pcg_update_kernel(int nnd, const T* __restrict__ minv,
                                                         typename Vec4<T>::type* __restrict__ x,
                                                         typename Vec4<T>::type* __restrict__ r,
                                                         typename Vec4<T>::type* __restrict__ z,
                                                         const typename Vec4<T>::type* __restrict__ p,
                                                         const typename Vec4<T>::type* __restrict__ q,
                                                         double* partials, PcgScalars* sc) {
  using V = typename Vec4<T>::type;
  if (((volatile PcgScalars*)sc)->done) return;
  const T alpha = T(sc->alpha);
  double v[2] = {0.0, 0.0};
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nnd; n += gridDim.x * blockDim.x) {
    const V pn = p[n], qn = q[n];
    V xn = x[n], rn = r[n];
    xn.x += alpha * pn.x;
    xn.y += alpha * pn.y;
    xn.z += alpha * pn.z;
    rn.x -= alpha * qn.x;
    rn.y -= alpha * qn.y;
    rn.z -= alpha * qn.z;
    T zx, zy, zz;
    apply_minv<T>(minv, n, rn.x, rn.y, rn.z, zx, zy, zz);
    x[n] = xn;
    r[n] = rn;
    z[n] = mk<V, T>(zx, zy, zz);
    v[0] += (double)rn.x * zx + (double)rn.y * zy + (double)rn.z * zz;
    v[1] += (double)rn.x * rn.x + (double)rn.y * rn.y + (double)rn.z * rn.z;
  }
  double tot[2];
  if (last_block_total<2>(v, partials, &sc->count_b, tot) && threadIdx.x == 0) {
    const int it = sc->iters + 1;
    sc->iters = it;
    sc->beta = tot[0] / sc->rz;
    sc->rz = tot[0];
    sc->rr = tot[1];
    if (!isfinite(tot[0]) || !isfinite(tot[1])) {
      sc->done = 2;
      sc->fail = 4;
    }
    else if (tot[1] <= sc->tol2 * sc->rr0) sc->done = 1;
    else if (it >= sc->max_it) sc->done = 3;
  }
}

struct Grids {
  int spmv, vec;
};
Grids grids(const Context* c) {
  Grids g;
  g.spmv = std::min((c->nnd + 7) / 8, kNumSMs * 8);
  g.vec = std::min((c->nnd + 255) / 256, kNumSMs * 8);
  return g;
}

template <typename T>
int capture_chunk(Context* c, const T* minv) {
  using V = typename Vec4<T>::type;
  const Grids g = grids(c);
  const T* vals = std::is_same<T, float>::value ? (const T*)c->d_vals32 : (const T*)c->d_vals64;
  cudaGraph_t graph;
  if (!ok(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture")) return TG_ERR_CUDA;
  for (int k = 0; k < kChunk; ++k) {
    pcg_spmv_kernel<T><<<g.spmv, 256, 0, c->stream>>>(c->nnd, c->d_rowptr, c->d_col, vals, c->nnzb_pad,
                                                     (const V*)c->d_z, (V*)c->d_p, (V*)c->d_q, c->d_partials, c->d_pcg);
    pcg_update_kernel<T><<<g.vec, 256, 0, c->stream>>>(c->nnd, minv, (V*)c->d_x, (V*)c->d_r, (V*)c->d_z,
                                                      (const V*)c->d_p, (const V*)c->d_q, c->d_partials, c->d_pcg);
  }
  if (!ok(c, cudaStreamEndCapture(c->stream, &graph), "end capture")) return TG_ERR_CUDA;
  if (c->pcg_graph) cudaGraphExecDestroy(c->pcg_graph);
  c->pcg_graph = nullptr;
  cudaError_t e = cudaGraphInstantiate(&c->pcg_graph, graph, 0);
  cudaGraphDestroy(graph);
  return ok(c, e, "graph instantiate") ? TG_OK : TG_ERR_CUDA;
}

template <typename T>
int ensure_vectors(Context* c, int precision) {
  using V = typename Vec4<T>::type;
  if (c->pcg_vec_precision == precision) return TG_OK;
  for (void** pp : {&c->d_x, &c->d_r, &c->d_z, &c->d_p, &c->d_q}) {
    if (*pp) dfree(c, *pp);
    V* v = nullptr;
    if (!dalloc(c, &v, (size_t)c->nnd)) return TG_ERR_OOM;
    *pp = v;
  }
  c->pcg_vec_precision = precision;
  if (c->pcg_graph) {
    cudaGraphExecDestroy(c->pcg_graph);
    c->pcg_graph = nullptr;
  }
  c->pcg_graph_key = -1;
  return TG_OK;
}

template <typename T>
int solve_t(Context* c, const double4_32a* d_rhs, double rel_tol, int max_it, int precond, int* iters,
            double* rel_res) {
  using V = typename Vec4<T>::type;
  const int precision = std::is_same<T, float>::value ? TG_MIXED : TG_FP64;
  int s = ensure_vectors<T>(c, precision);
  if (s) return s;
  const T* minv_base = std::is_same<T, float>::value ? (const T*)c->d_minv32 : (const T*)c->d_minv64;
  const T* minv = minv_base + (precond == TG_PRECOND_BLOCK_JACOBI ? (long long)c->nnd * 9 : 0);
  const int key = precision * 2 + (precond == TG_PRECOND_BLOCK_JACOBI ? 1 : 0);
  const Grids g = grids(c);
  pcg_init_kernel<T><<<g.vec, 256, 0, c->stream>>>(c->nnd, d_rhs, c->d_mask, minv, (V*)c->d_x, (V*)c->d_r,
                                                  (V*)c->d_z, (V*)c->d_p, (V*)c->d_q, c->d_partials, c->d_pcg,
                                                  rel_tol, max_it);
  c->launches++;
  if (!ok(c, cudaGetLastError(), "pcg_init_kernel")) return TG_ERR_CUDA;
  if (c->pcg_graph_key != key || !c->pcg_graph) {
    s = capture_chunk<T>(c, minv);
    if (s) return s;
    c->pcg_graph_key = key;
  }
  const int max_chunks = max_it / kChunk + 2;
  for (int k = 0; k < max_chunks; ++k) {
    if (!ok(c, cudaGraphLaunch(c->pcg_graph, c->stream), "graph launch")) return TG_ERR_CUDA;
    c->launches += 2 * kChunk;
    if (!ok(c, cudaMemcpyAsync(c->h_pcg, c->d_pcg, sizeof(PcgScalars), cudaMemcpyDeviceToHost, c->stream), "copy"))
      return TG_ERR_CUDA;
    if (!ok(c, cudaStreamSynchronize(c->stream), "pcg sync")) return TG_ERR_CUDA;
    if (c->h_pcg->done) break;
  }
  const PcgScalars& h = *c->h_pcg;
  if (iters) *iters = h.iters;
  if (rel_res) *rel_res = h.rr0 > 0 ? std::sqrt(h.rr / h.rr0) : 0.0;
  c->have_du = true;
  if (h.done == 1) return TG_OK;
  if (h.done == 2) {
    static const char* why[] = {"", "non-finite initial residual", "p.Ap <= 0 (indefinite operator)",
                                "non-finite p.Ap", "non-finite r.z or r.r"};
    c->err = std::string("PCG breakdown: ") + why[h.fail >= 1 && h.fail <= 4 ? h.fail : 0] + " at iteration " +
             std::to_string(h.iters);
    return TG_ERR_NAN;
  }
  c->err = "PCG iteration limit reached";
  return TG_ERR_NOT_CONVERGED;
}

// rhs = R - K v on the node-block matrix (prescribed rows are zero in K and
// in R), accumulated in FP64 whatever the matrix precision
template <typename T>
__global__ void __launch_bounds__(256) lift_rhs_kernel(int nnd, const int* __restrict__ rowptr,
                                                       const int* __restrict__ col, const T* __restrict__ vals,
                                                       long long stride, const double4_32a* __restrict__ v,
                                                       const double4_32a* __restrict__ R, double4_32a* __restrict__ rhs) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; I < nnd; I += warps) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    const int r1 = rowptr[I + 1];
    for (int j = rowptr[I] + lane; j < r1; j += 32) {
      const double4_32a vj = v[col[j]];
      a0 += (double)vals[0 * stride + j] * vj.x + (double)vals[1 * stride + j] * vj.y + (double)vals[2 * stride + j] * vj.z;
      a1 += (double)vals[3 * stride + j] * vj.x + (double)vals[4 * stride + j] * vj.y + (double)vals[5 * stride + j] * vj.z;
      a2 += (double)vals[6 * stride + j] * vj.x + (double)vals[7 * stride + j] * vj.y + (double)vals[8 * stride + j] * vj.z;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, o);
      a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if (lane == 0) {
      const double4_32a r = R[I];
      rhs[I] = make_double4_32a(r.x - a0, r.y - a1, r.z - a2, 0.0);
    }
  }
}

__global__ void diff_kernel(int nnd, const double4_32a* __restrict__ a, const double4_32a* __restrict__ b,
                            double4_32a* __restrict__ out) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnd) return;
  const double4_32a x = a[n], y = b[n];
  out[n] = make_double4_32a(x.x - y.x, x.y - y.y, x.z - y.z, 0.0);
}

template <typename V>
__global__ void gather_solution_kernel(int neq, const int* __restrict__ slot, const V* __restrict__ x,
                                       double* __restrict__ eq) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= neq) return;
  const int s = slot[k];
  const V v = x[s >> 2];
  const int d = s & 3;
  eq[k] = (double)(d == 0 ? v.x : (d == 1 ? v.y : v.z));
}

}  // namespace

int launch_lift_rhs(Context* c, const double4_32a* d_v, double4_32a* d_rhs) {
  const Grids g = grids(c);
  if (c->tangent_precision == TG_MIXED)
    lift_rhs_kernel<float><<<g.spmv, 256, 0, c->stream>>>(c->nnd, c->d_rowptr, c->d_col, c->d_vals32, c->nnzb_pad,
                                                         d_v, c->d_R, d_rhs);
  else
    lift_rhs_kernel<double><<<g.spmv, 256, 0, c->stream>>>(c->nnd, c->d_rowptr, c->d_col, c->d_vals64, c->nnzb_pad,
                                                          d_v, c->d_R, d_rhs);
  c->launches++;
  return ok(c, cudaGetLastError(), "lift_rhs_kernel") ? TG_OK : TG_ERR_CUDA;
}

int launch_diff(Context* c, const double4_32a* a, const double4_32a* b, double4_32a* out) {
  diff_kernel<<<(c->nnd + 255) / 256, 256, 0, c->stream>>>(c->nnd, a, b, out);
  c->launches++;
  return ok(c, cudaGetLastError(), "diff_kernel") ? TG_OK : TG_ERR_CUDA;
}

int launch_gather_solution(Context* c, double* d_eq) {
  if (c->neq == 0) return TG_OK;
  const int grid = (c->neq + 255) / 256;
  if (c->pcg_vec_precision == TG_MIXED)
    gather_solution_kernel<float4><<<grid, 256, 0, c->stream>>>(c->neq, c->d_eq_slot, (const float4*)c->d_x, d_eq);
  else
    gather_solution_kernel<double4_32a><<<grid, 256, 0, c->stream>>>(c->neq, c->d_eq_slot, (const double4_32a*)c->d_x, d_eq);
  c->launches++;
  return ok(c, cudaGetLastError(), "gather_solution_kernel") ? TG_OK : TG_ERR_CUDA;
}

// Average device time of standalone launches of the two PCG kernels on the
// current tangent, with the scalars pinned so every launch does the same work
// (beta = alpha = 0: q = A z, p = z; x, r unchanged).
template <typename T>
int time_pcg_t(Context* c, int which, int reps, double* ms) {
  using V = typename Vec4<T>::type;
  const int precision = std::is_same<T, float>::value ? TG_MIXED : TG_FP64;
  int s = ensure_vectors<T>(c, precision);
  if (s) return s;
  const T* minv = std::is_same<T, float>::value ? (const T*)c->d_minv32 : (const T*)c->d_minv64;
  const T* vals = std::is_same<T, float>::value ? (const T*)c->d_vals32 : (const T*)c->d_vals64;
  const Grids g = grids(c);
  pcg_init_kernel<T><<<g.vec, 256, 0, c->stream>>>(c->nnd, c->d_R, c->d_mask, minv, (V*)c->d_x, (V*)c->d_r,
                                                  (V*)c->d_z, (V*)c->d_p, (V*)c->d_q, c->d_partials, c->d_pcg,
                                                  1e-30, 1 << 30);
  c->launches++;
  PcgScalars t;
  std::memset(&t, 0, sizeof(t));
  t.rz = t.rz_old = t.rr = t.rr0 = t.pq = 1.0;
  t.max_it = 1 << 30;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  double total = 0.0;
  for (int r = 0; r < reps; ++r) {
    cudaMemcpyAsync(c->d_pcg, &t, sizeof(t), cudaMemcpyHostToDevice, c->stream);
    cudaEventRecord(a, c->stream);
    if (which == 0)
      pcg_spmv_kernel<T><<<g.spmv, 256, 0, c->stream>>>(c->nnd, c->d_rowptr, c->d_col, vals, c->nnzb_pad,
                                                       (const V*)c->d_z, (V*)c->d_p, (V*)c->d_q, c->d_partials,
                                                       c->d_pcg);
    else
      pcg_update_kernel<T><<<g.vec, 256, 0, c->stream>>>(c->nnd, minv, (V*)c->d_x, (V*)c->d_r, (V*)c->d_z,
                                                        (const V*)c->d_p, (const V*)c->d_q, c->d_partials, c->d_pcg);
    cudaEventRecord(b, c->stream);
    c->launches++;
    cudaEventSynchronize(b);
    float e = 0.f;
    cudaEventElapsedTime(&e, a, b);
    total += e;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = total / reps;
  return ok(c, cudaGetLastError(), "time_pcg_kernel") ? TG_OK : TG_ERR_CUDA;
}

int time_pcg_kernel(Context* c, int which, int reps, double* ms) {
  if (c->tangent_precision == TG_MIXED) return time_pcg_t<float>(c, which, reps, ms);
  if (c->tangent_precision == TG_FP64) return time_pcg_t<double>(c, which, reps, ms);
  c->err = "form the tangent first";
  return TG_ERR_ARG;
}

int pcg_solve(Context* c, const double4_32a* d_rhs, double rel_tol, int max_it, int precond, int* iters,
              double* rel_res) {
  if (c->tangent_precision == TG_MIXED) return solve_t<float>(c, d_rhs, rel_tol, max_it, precond, iters, rel_res);
  if (c->tangent_precision == TG_FP64) return solve_t<double>(c, d_rhs, rel_tol, max_it, precond, iters, rel_res);
  c->err = "tg_pcg_solve: no tangent formed";
  return TG_ERR_ARG;
}

}  // namespace tg
