// (Block-)Jacobi preconditioned CG on the node-block CSR matrix, sm_103a.
//
// Each iteration is two kernels:
//   pcg_spmv_kernel   q = A p, partial p.q; the last CTA forms alpha (the
//                     product is exact each iteration: no recurrence for A p)
//   pcg_update_kernel x += alpha p; r -= alpha q; z = M^-1 r; partial r.z,
//                     r.r; a grid barrier (cooperative launch); every CTA
//                     then forms the same r.z and beta from the partials in
//                     the same order and updates its nodes' p = z + beta p in
//                     place, so the product gathers one vector per neighbour
// The reductions of FP64 partial sums run in a fixed order (bitwise
// repeatable, no floating-point atomics) and compute alpha / beta and the
// convergence flag on the device.  Iterations run in chunks captured once in
// a CUDA graph; kernels return immediately once the flag is set, and the host
// reads each chunk's flag while the next chunk runs.
//
// Vectors are stored per node, padded to 4 lanes (float4 in the mixed form,
// double4_32a in the plain FP64 form).  Dot products and norms accumulate in
// FP64 in both forms.  This replaces the reference's Krylov/diagonal solve
// (NLSolver_NK::GMRES, NLSolver_NK.cpp:121; DiagonalMatrixT::BackSubstitute,
// DiagonalMatrixT.cpp:313; MSRMatrixT::Multx, MSRMatrixT.cpp:385).
#include <cmath>
#include <cstring>
#include <string>

#include "krylov_common.cuh"

namespace tg {

namespace {

constexpr int kChunk = 16;  // PCG iterations per graph replay


// FP64 pre-pass: s = b.M^-1.b over active dofs; the solve then runs on
// b/sqrt(s) so the FP32 iterates stay O(1) whatever the residual magnitude
// (late Newton residuals sit at FP64 round-off, far below FP32 range when
// squared).
template <typename T>
__global__ void __launch_bounds__(256) pcg_scale_kernel(int nnd, const double4_32a* __restrict__ rhs,
                                                        const uint8_t* __restrict__ mask, const T* __restrict__ minv,
                                                        double* partials, PcgScalars* sc) {
  Acc<double> v[1];
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nnd; n += gridDim.x * blockDim.x) {
    const double4_32a b = rhs[n];
    const uint8_t m = mask[n];
    const double bx = (m & 1) ? b.x : 0.0, by = (m & 2) ? b.y : 0.0, bz = (m & 4) ? b.z : 0.0;
    const T* B = minv + (long long)n * 9;
    const double zx = (double)B[0] * bx + (double)B[1] * by + (double)B[2] * bz;
    const double zy = (double)B[3] * bx + (double)B[4] * by + (double)B[5] * bz;
    const double zz = (double)B[6] * bx + (double)B[7] * by + (double)B[8] * bz;
    v[0].add(bx * zx + by * zy + bz * zz);
  }
  double tot[1];
  if (last_block_total<double, 1>(v, partials, &sc->count_a, tot) && threadIdx.x == 0) {
    const double s = tot[0];
    const double sc_ = (s > 0.0 && isfinite(s)) ? 1.0 / sqrt(s) : 1.0;
    sc->scale = sc_;
    sc->unscale = 1.0 / sc_;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) pcg_init_kernel(int nnd, const double4_32a* __restrict__ rhs,
                                                       const uint8_t* __restrict__ mask, const T* __restrict__ minv,
                                                       typename Vec4<T>::type* x, typename Vec4<T>::type* r,
                                                       typename Vec4<T>::type* z, typename Vec4<T>::type* p,
                                                       typename Vec4<T>::type* q, double* partials, PcgScalars* sc,
                                                       double tol, int max_it) {
  using V = typename Vec4<T>::type;
  Acc<T> v[2];
  const double scale = sc->scale;
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nnd; n += gridDim.x * blockDim.x) {
    const double4_32a b = rhs[n];
    const uint8_t mk_ = mask[n];
    const T rx = (mk_ & 1) ? T(b.x * scale) : T(0), ry = (mk_ & 2) ? T(b.y * scale) : T(0),
            rz = (mk_ & 4) ? T(b.z * scale) : T(0);
    T zx, zy, zz;
    apply_minv<T>(minv, n, rx, ry, rz, zx, zy, zz);
    x[n] = mk<V, T>(T(0), T(0), T(0));
    r[n] = mk<V, T>(rx, ry, rz);
    z[n] = mk<V, T>(zx, zy, zz);
    p[n] = mk<V, T>(zx, zy, zz);  // first direction p = z
    q[n] = mk<V, T>(T(0), T(0), T(0));
    v[0].add_prod(rx, zx);
    v[0].add_prod(ry, zy);
    v[0].add_prod(rz, zz);
    v[1].add_prod(rx, rx);
    v[1].add_prod(ry, ry);
    v[1].add_prod(rz, rz);
  }
  double tot[2];
  if (last_block_total<T, 2>(v, partials, &sc->count_b, tot) && threadIdx.x == 0) {
    sc->rz = tot[0];
    sc->rr = tot[1];
    sc->rr0 = tot[1];
    sc->beta = 0.0;
    sc->alpha = 0.0;
    sc->iters = 0;
    sc->tol2 = tol * tol;
    sc->max_it = max_it;
    sc->count_a = 0u;
    sc->bar_count = 0u;
    sc->fail = 0;
    sc->done = (tot[1] == 0.0) ? 1 : (isfinite(tot[0]) && isfinite(tot[1]) ? 0 : 2);
    if (sc->done == 2) sc->fail = 1;
  }
}


// q = A p on a persistent grid.  Each CTA streams its row tiles through a ring of NST
// shared-memory stages: one bulk copy per tile (the tile-contiguous storage
// makes a tile one range), completing on the stage's mbarrier, is issued
// NST-1 tiles ahead while the CTA's warps compute the current tile: 8 lanes
// per row, 4 rows per warp at a time, each lane over every 8th block.  Every
// wait is bounded; a timeout sets an error flag, drains the copies in flight
// (bounded) and marks the solve broken down.
template <typename T, int NST>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 2) pcg_spmv_kernel(int ntiles, const long long* __restrict__ blob_off,
                                                       const unsigned char* __restrict__ blob, int cap,
                                                       const typename Vec4<T>::type* __restrict__ p,
                                                       typename Vec4<T>::type* __restrict__ q, double* partials,
                                                       PcgScalars* sc, int* status, double* node_dot,
                                                       int keep) {
  using V = typename Vec4<T>::type;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bars[NST];
  __shared__ int abort_flag;
  if (skip_launch(sc, 0)) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NST; ++k) mbar_init(&bars[k], 1);
    fence_mbar_init();
    abort_flag = 0;
  }
  __syncthreads();
  Acc<T> v[1];
  const int t0 = blockIdx.x, G = gridDim.x;
  uint64_t pol_last = 0, pol_first = 0;
  if (threadIdx.x == 0 && keep >= 0) {
    pol_last = l2_policy_evict_last();
    pol_first = l2_policy_evict_first();
  }
  auto issue = [&](int t, int stage) {
    const long long o0 = blob_off[t], o1 = blob_off[t + 1];
    const unsigned bytes = (unsigned)(o1 - o0);
    mbar_expect_tx(&bars[stage], bytes);
    stage_tile(smem + (size_t)stage * cap, blob + o0, bytes, &bars[stage], t, keep, pol_last, pol_first);
  };
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NST - 1; ++k)
      if (t0 + k * G < ntiles) issue(t0 + k * G, k);
  unsigned phases = 0u;  // bit k: parity of stage k's next completion
  int stuck = -1;
  int it = 0;
  for (int t = t0; t < ntiles; ++it, t += G) {
    const int s = it % NST;
    const int tn = t + (NST - 1) * G;
    if (threadIdx.x == 0 && tn < ntiles) {
      fence_async_smem();  // the stage was last read through generic loads
      issue(tn, (it + NST - 1) % NST);
    }
    if (!mbar_wait(&bars[s], (phases >> s) & 1u, kWaitLimit)) {
      if (lane == 0) atomicOr(&abort_flag, 1);
    }
    phases ^= 1u << s;
    __syncthreads();
    if (abort_flag) {
      stuck = s;
      break;
    }
    spmv_tile_rows<T>(smem + (size_t)s * cap, lane, warp, nwarps, p, q, v[0], node_dot);
    __syncthreads();  // stage s is free for the copy issued next iteration
  }
  if (stuck >= 0 && threadIdx.x == 0) {
    // a staged tile never completed: record it, drain the copies still in
    // flight (bounded waits) and leave the solve flagged as broken down
    atomicOr(status, kStatusWaitTimeout);
    for (int k = 0; k < NST; ++k) {
      const unsigned parity = ((phases >> k) & 1u) ^ (k == stuck ? 1u : 0u);
      mbar_wait(&bars[k], parity, kWaitLimit);  // bounded even when nothing is pending
    }
    sc->done = 2;
    sc->fail = 5;
  }
  // a segmented batch reduces the rows' own products per RVE instead
  if (node_dot) return;
  double tot[1];
  if (last_block_total<T, 1>(v, partials, &sc->count_a, tot) && threadIdx.x == 0) {
    sc->pq = tot[0];
    if (sc->done == 2) return;
    if (!(tot[0] > 0.0) || !isfinite(tot[0])) {
      sc->done = 2;
      sc->fail = isfinite(tot[0]) ? 2 : 3;
    } else {
      sc->alpha = sc->rz / tot[0];
    }
  }
}

// The same product with per-warp stage release: instead of a CTA barrier at
// the end of every tile, each warp arrives on the stage's "empty" mbarrier
// when its rows are done, and the producing thread waits on it (bounded)
// before the next bulk copy into that stage, so a warp that finishes a tile
// early moves on to the next staged tile.  Consumer reads are ordered before
// the next copy by the mbarrier release/acquire and a proxy fence.
template <typename T, int NST>
__global__ void __launch_bounds__(256) pcg_spmv_wr_kernel(int ntiles, const long long* __restrict__ blob_off,
                                                          const unsigned char* __restrict__ blob, int cap,
                                                          const typename Vec4<T>::type* __restrict__ p,
                                                          typename Vec4<T>::type* __restrict__ q, double* partials,
                                                          PcgScalars* sc, int* status, double* node_dot,
                                                          int keep) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t full[NST];
  __shared__ __align__(8) uint64_t empty[NST];
  __shared__ volatile int abort_flag;
  if (skip_launch(sc, 0)) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NST; ++k) {
      mbar_init(&full[k], 1);
      mbar_init(&empty[k], nwarps);
    }
    fence_mbar_init();
    abort_flag = 0;
  }
  __syncthreads();
  Acc<T> v[1];
  const int t0 = blockIdx.x, G = gridDim.x;
  // producer bookkeeping (thread 0): copies issued / completions seen per
  // stage, and the parity of the next "empty" completion per stage
  int issued[NST], seen[NST];
#pragma unroll
  for (int k = 0; k < NST; ++k) issued[k] = seen[k] = 0;
  unsigned eph = 0u;
  uint64_t pol_last = 0, pol_first = 0;
  if (threadIdx.x == 0 && keep >= 0) {
    pol_last = l2_policy_evict_last();
    pol_first = l2_policy_evict_first();
  }
  auto issue = [&](int t, int stage) {
    const long long o0 = blob_off[t], o1 = blob_off[t + 1];
    const unsigned bytes = (unsigned)(o1 - o0);
    mbar_expect_tx(&full[stage], bytes);
    stage_tile(smem + (size_t)stage * cap, blob + o0, bytes, &full[stage], t, keep, pol_last, pol_first);
  };
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NST - 1; ++k)
      if (t0 + k * G < ntiles) {
        issue(t0 + k * G, k);
        ++issued[k];
      }
  unsigned phases = 0u;  // parity of each stage's next "full" completion
  int it = 0;
  for (int t = t0; t < ntiles; ++it, t += G) {
    if (abort_flag) break;
    const int s = it % NST;
    const int tn = t + (NST - 1) * G;
    if (threadIdx.x == 0 && tn < ntiles) {
      const int sn = (it + NST - 1) % NST;
      bool free_ok = true;
      if (it >= 1) {  // stage sn held the tile of iteration it-1
        free_ok = mbar_wait(&empty[sn], (eph >> sn) & 1u, kWaitLimit);
        eph ^= 1u << sn;
      }
      if (free_ok) {
        fence_async_smem();
        issue(tn, sn);
        ++issued[sn];
      } else {
        abort_flag = 1;
      }
    }
    const bool got = mbar_wait(&full[s], (phases >> s) & 1u, kWaitLimit);
    phases ^= 1u << s;
    if (!got) {
      abort_flag = 1;
      break;
    }
    if (threadIdx.x == 0) ++seen[s];
    spmv_tile_rows<T>(smem + (size_t)s * cap, lane, warp, nwarps, p, q, v[0], node_dot);
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
  }
  __syncthreads();
  if (abort_flag && threadIdx.x == 0) {
    // a wait timed out: record it, drain the copies still in flight
    // (bounded) and leave the solve flagged as broken down
    atomicOr(status, kStatusWaitTimeout);
    for (int k = 0; k < NST; ++k)
      if (issued[k] > seen[k]) mbar_wait(&full[k], (unsigned)(seen[k] & 1), kWaitLimit);
    sc->done = 2;
    sc->fail = 5;
  }
  // a segmented batch reduces the rows' own products per RVE instead
  if (node_dot) return;
  double tot[1];
  if (last_block_total<T, 1>(v, partials, &sc->count_a, tot) && threadIdx.x == 0) {
    sc->pq = tot[0];
    if (sc->done == 2) return;
    if (!(tot[0] > 0.0) || !isfinite(tot[0])) {
      sc->done = 2;
      sc->fail = isfinite(tot[0]) ? 2 : 3;
    } else {
      sc->alpha = sc->rz / tot[0];
    }
  }
}

// Launched cooperatively (every CTA resident): the grid barrier between the
// two phases is bounded and, should it ever give up, the solve ends flagged
// as broken down instead of waiting.  Each thread takes its nodes
// n0, n0 + stride, ... four (FP32) or two (FP64) at a time with all their
// loads issued before any use (the partial sums keep that node order).
template <typename T>
__global__ void __launch_bounds__(256, 2) pcg_update_kernel(int nnd, const T* __restrict__ minv,
                                                            typename Vec4<T>::type* __restrict__ x,
                                                            typename Vec4<T>::type* __restrict__ r,
                                                            typename Vec4<T>::type* __restrict__ z,
                                                            typename Vec4<T>::type* __restrict__ p,
                                                            const typename Vec4<T>::type* __restrict__ q,
                                                            double* partials, PcgScalars* sc, int* status) {
  using V = typename Vec4<T>::type;
  constexpr int U = sizeof(T) == 4 ? 4 : 2;  // within 128 registers: two CTAs per SM
  __shared__ double totals[2];
  if (((volatile PcgScalars*)sc)->done) return;
  const T alpha = T(sc->alpha);
  const double rz_old = sc->rz;  // read before the barrier: CTA 0 replaces it after
  const int stride = gridDim.x * blockDim.x;
  const int n0 = blockIdx.x * blockDim.x + threadIdx.x;
  Acc<T> v[2];
  for (int base = n0; base < nnd; base += U * stride) {
    V pn[U], qn[U], xn[U], rn[U];
    T B[U][9];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int n = base + u * stride;
      if (n < nnd) {
        pn[u] = p[n];
        qn[u] = q[n];
        xn[u] = x[n];
        rn[u] = r[n];
#pragma unroll
        for (int k = 0; k < 9; ++k) B[u][k] = minv[(long long)n * 9 + k];
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int n = base + u * stride;
      if (n < nnd) {
        xn[u].x += alpha * pn[u].x;
        xn[u].y += alpha * pn[u].y;
        xn[u].z += alpha * pn[u].z;
        rn[u].x -= alpha * qn[u].x;
        rn[u].y -= alpha * qn[u].y;
        rn[u].z -= alpha * qn[u].z;
        const T zx = B[u][0] * rn[u].x + B[u][1] * rn[u].y + B[u][2] * rn[u].z;
        const T zy = B[u][3] * rn[u].x + B[u][4] * rn[u].y + B[u][5] * rn[u].z;
        const T zz = B[u][6] * rn[u].x + B[u][7] * rn[u].y + B[u][8] * rn[u].z;
        x[n] = xn[u];
        r[n] = rn[u];
        z[n] = mk<V, T>(zx, zy, zz);
        v[0].add_prod(rn[u].x, zx);
        v[0].add_prod(rn[u].y, zy);
        v[0].add_prod(rn[u].z, zz);
        v[1].add_prod(rn[u].x, rn[u].x);
        v[1].add_prod(rn[u].y, rn[u].y);
        v[1].add_prod(rn[u].z, rn[u].z);
      }
    }
  }
  {
    double bt[2];
    block_total<T, 2>(v, bt);
    if (threadIdx.x == 0) {
      partials[blockIdx.x] = bt[0];
      partials[gridDim.x + blockIdx.x] = bt[1];
    }
  }
  if (!grid_barrier(&sc->bar_count, kBarrierLimit)) {
    if (threadIdx.x == 0) {
      atomicOr(status, kStatusWaitTimeout);
      sc->fail = 5;
      atomicExch(&sc->done, 2);
    }
    return;
  }
  // every CTA forms the same totals from the partials, in the same order
  // (one warp: lane-strided sums, then a fixed shuffle tree)
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    double s0 = 0.0, s1 = 0.0;
#pragma unroll 4
    for (int b = lane; b < (int)gridDim.x; b += 32) {
      s0 += ((volatile double*)partials)[b];
      s1 += ((volatile double*)partials)[gridDim.x + b];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s0 += __shfl_xor_sync(0xffffffffu, s0, o);
      s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
    if (lane == 0) {
      totals[0] = s0;
      totals[1] = s1;
    }
  }
  __syncthreads();
  const double rz = totals[0], rr = totals[1];
  const double beta_d = rz / rz_old;
  const T beta = T(beta_d);
  // next search direction, in place: p = z + beta p
  for (int base = n0; base < nnd; base += U * stride) {
    V zn[U], pn[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int n = base + u * stride;
      if (n < nnd) {
        zn[u] = z[n];
        pn[u] = p[n];
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int n = base + u * stride;
      if (n < nnd)
        p[n] = mk<V, T>(zn[u].x + beta * pn[u].x, zn[u].y + beta * pn[u].y, zn[u].z + beta * pn[u].z);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const int it = sc->iters + 1;
    sc->iters = it;
    sc->beta = beta_d;
    sc->rz = rz;
    sc->rr = rr;
    int done = 0;
    if (!isfinite(rz) || !isfinite(rr)) {
      sc->fail = 4;
      done = 2;
    } else if (rr <= sc->tol2 * sc->rr0) {
      done = 1;
    } else if (it >= sc->max_it) {
      done = 3;
    }
    if (done) atomicCAS(&sc->done, 0, done);  // a barrier failure elsewhere keeps its flag
  }
}

using Grids = SpmvPlan;

// persistent grid for the streamed SpMV: as many CTAs as fit (shared memory
// bound), at most one per tile
template <typename T>
int blob_cap(const Context* c) {
  return (int)(((std::is_same<T, float>::value ? c->blob_cap32 : c->blob_cap64) + 127) / 128 * 128);
}
template <typename T, int NST>
int spmv_config_n(Context* c, Grids& g) {
  g.spmv_smem = (size_t)NST * blob_cap<T>(c);
  int optin = 0;
  if (!ok(c, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device), "attribute"))
    return TG_ERR_CUDA;
  if (g.spmv_smem + 1024 > (size_t)optin) {
    c->err = "SpMV tile ring does not fit in shared memory (reduce tile_blocks or stages)";
    return TG_ERR_CAPACITY;
  }
  auto kern = c->spmv_warp_release ? pcg_spmv_wr_kernel<T, NST> : pcg_spmv_kernel<T, NST>;
  // Both variants get the attribute (the scratch-vector solve always uses the
  // CTA-barrier kernel).  The attribute belongs to the function, not to this
  // context, and contexts with other meshes may configure and launch from
  // other threads at the same time, so it is always set to the largest
  // dynamic size the device allows (one value for every caller) rather than
  // to this mesh's ring.
  for (auto f : {pcg_spmv_kernel<T, NST>, pcg_spmv_wr_kernel<T, NST>}) {
    cudaFuncAttributes fa;
    if (!ok(c, cudaFuncGetAttributes(&fa, f), "function attributes") ||
        !ok(c, cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes),
            "smem attribute"))
      return TG_ERR_CUDA;
  }
  int per_sm = 0;
  if (!ok(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, g.spmv_smem), "occupancy"))
    return TG_ERR_CUDA;
  if (per_sm < 1) {
    c->err = "SpMV tile does not fit in shared memory";
    return TG_ERR_CAPACITY;
  }
  g.spmv = std::max(1, std::min(c->ntiles, c->num_sms * per_sm));
  g.warp_release = c->spmv_warp_release;
  // leading whole tiles within the bytes kept in L2
  g.keep = -1;
  if (c->l2_keep >= 0) {
    const std::vector<long long>& off = std::is_same<T, float>::value ? c->h_blob_off32 : c->h_blob_off64;
    int t = 0;
    while (t < c->ntiles && off[t + 1] <= c->l2_keep) ++t;
    g.keep = t;
  }
  return TG_OK;
}
template <typename T>
int spmv_config(Context* c, Grids& g) {
  if (sym_active(c)) {
    g.sym = true;
    return sym_config(c, std::is_same<T, float>::value ? TG_MIXED : TG_FP64, g.sl);
  }
  // the configured ring depth, or 8 stages when 16 do not fit (FP64 tiles)
  int optin = 0;
  if (!ok(c, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device), "attribute"))
    return TG_ERR_CUDA;
  g.stages = c->spmv_stages;
  if (g.stages == 3 && 3 * (size_t)blob_cap<T>(c) + 1024 > (size_t)optin) g.stages = 2;
  return g.stages == 3 ? spmv_config_n<T, 3>(c, g) : spmv_config_n<T, 2>(c, g);
}
template <typename T>
void launch_spmv(Context* c, const Grids& g, const void* p, void* q, double* partials, PcgScalars* sc,
                 double* node_dot = nullptr) {
  using V = typename Vec4<T>::type;
  const bool f32 = std::is_same<T, float>::value;
  if (g.sym) {
    sym_launch(c, f32 ? TG_MIXED : TG_FP64, g.sl, p, q, partials, sc, node_dot);
    return;
  }
  const long long* off = f32 ? c->d_blob_off32 : c->d_blob_off64;
  const unsigned char* blob = f32 ? c->d_blob32 : c->d_blob64;
  const int cap = blob_cap<T>(c);
#define TG_SPMV_ARGS c->ntiles, off, blob, cap, (const V*)p, (V*)q, partials, sc, c->d_status, node_dot, g.keep
  if (g.warp_release) {
    if (g.stages == 3)
      pcg_spmv_wr_kernel<T, 3><<<g.spmv, 256, g.spmv_smem, c->stream>>>(TG_SPMV_ARGS);
    else
      pcg_spmv_wr_kernel<T, 2><<<g.spmv, 256, g.spmv_smem, c->stream>>>(TG_SPMV_ARGS);
  } else {
    if (g.stages == 3)
      pcg_spmv_kernel<T, 3><<<g.spmv, 256, g.spmv_smem, c->stream>>>(TG_SPMV_ARGS);
    else
      pcg_spmv_kernel<T, 2><<<g.spmv, 256, g.spmv_smem, c->stream>>>(TG_SPMV_ARGS);
  }
#undef TG_SPMV_ARGS
}

// The vector update as a cooperative launch (its grid barrier needs every
// CTA resident; the grid is clamped to what fits at once).
template <typename T>
cudaError_t launch_update(Context* c, int grid, const T* minv, void* x, void* r, void* z, void* p, const void* q,
                          double* partials, PcgScalars* sc) {
  using V = typename Vec4<T>::type;
  int per_sm = 0;
  const cudaError_t oe = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pcg_update_kernel<T>, 256, 0);
  if (oe != cudaSuccess) return oe;
  grid = std::max(1, std::min(grid, c->num_sms * per_sm));  // every CTA resident at once
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = c->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, pcg_update_kernel<T>, c->nnd, minv, (V*)x, (V*)r, (V*)z, (V*)p, (const V*)q,
                            partials, sc, c->d_status);
}

Grids grids(const Context* c) {
  Grids g;
  g.spmv = 0;
  g.spmv_smem = 0;
  g.stages = 8;
  g.vec = std::min((c->nnd + 255) / 256, c->num_sms * 2);
  return g;
}

template <typename T>
int capture_chunk(Context* c, const T* minv) {
  Grids g = grids(c);
  {
    const int sc = spmv_config<T>(c, g);
    if (sc) return sc;
  }
  cudaGraph_t graph;
  if (!ok(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture")) return TG_ERR_CUDA;
  cudaError_t le = cudaSuccess;
  for (int k = 0; k < kChunk && le == cudaSuccess; ++k) {
    launch_spmv<T>(c, g, c->d_p, c->d_q, c->d_partials, c->d_pcg);
    le = cudaGetLastError();
    if (le == cudaSuccess)
      le = launch_update<T>(c, g.vec, minv, c->d_x, c->d_r, c->d_z, c->d_p, c->d_q, c->d_partials, c->d_pcg);
  }
  const cudaError_t ee = cudaStreamEndCapture(c->stream, &graph);
  if (!ok(c, le, "capture launch") || !ok(c, ee, "end capture")) {
    if (ee == cudaSuccess) cudaGraphDestroy(graph);
    return TG_ERR_CUDA;
  }
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
  cg_free(c);  // its captured chunk names the old vectors
  return TG_OK;
}

template <typename T>
int start_t(Context* c, const double4_32a* d_rhs, const T* minv, double rel_tol, int max_it) {
  using V = typename Vec4<T>::type;
  const Grids g = grids(c);
  pcg_scale_kernel<T><<<g.vec, 256, 0, c->stream>>>(c->nnd, d_rhs, c->d_mask, minv, c->d_partials, c->d_pcg);
  c->launches++;
  pcg_init_kernel<T><<<g.vec, 256, 0, c->stream>>>(c->nnd, d_rhs, c->d_mask, minv, (V*)c->d_x, (V*)c->d_r,
                                                  (V*)c->d_z, (V*)c->d_p, (V*)c->d_q, c->d_partials, c->d_pcg,
                                                  rel_tol, max_it);
  c->launches++;
  return ok(c, cudaGetLastError(), "pcg_init_kernel") ? TG_OK : TG_ERR_CUDA;
}

template <typename T>
int solve_t(Context* c, const double4_32a* d_rhs, double rel_tol, int max_it, int precond, int* iters,
            double* rel_res) {
  const int precision = std::is_same<T, float>::value ? TG_MIXED : TG_FP64;
  int s = ensure_vectors<T>(c, precision);
  if (s) return s;
  const T* minv_base = std::is_same<T, float>::value ? (const T*)c->d_minv32 : (const T*)c->d_minv64;
  const T* minv = minv_base + (precond == TG_PRECOND_BLOCK_JACOBI ? (long long)c->nnd * 9 : 0);
  const int key = precision * 2 + (precond == TG_PRECOND_BLOCK_JACOBI ? 1 : 0);
  s = start_t<T>(c, d_rhs, minv, rel_tol, max_it);
  if (s) return s;
  if (c->pcg_graph_key != key || !c->pcg_graph) {
    s = capture_chunk<T>(c, minv);
    if (s) return s;
    c->pcg_graph_key = key;
  }
  // The scalars after each chunk are copied into alternating pinned mirrors;
  // the host checks a chunk's flag while the next chunk already runs, so the
  // GPU never idles for the round trip.  A chunk queued after convergence
  // costs only kernels that return at once.
  const int max_chunks = max_it / kChunk + 2;
  int last = 0;
  for (int k = 0; k < max_chunks; ++k) {
    if (!ok(c, cudaGraphLaunch(c->pcg_graph, c->stream), "graph launch")) return TG_ERR_CUDA;
    c->launches += 2 * kChunk;
    last = k & 1;
    if (!ok(c, cudaMemcpyAsync(&c->h_pcg[last], c->d_pcg, sizeof(PcgScalars), cudaMemcpyDeviceToHost, c->stream),
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

int pcg_start(Context* c, int precision, const double4_32a* d_rhs, const void* minv, double rel_tol, int max_it) {
  if (precision == TG_MIXED) return start_t<float>(c, d_rhs, (const float*)minv, rel_tol, max_it);
  return start_t<double>(c, d_rhs, (const double*)minv, rel_tol, max_it);
}

int pcg_finish(Context* c, const PcgScalars& h, int* iters, double* rel_res) {
  if (iters) *iters = h.iters;
  if (rel_res) *rel_res = h.rr0 > 0 ? std::sqrt(h.rr / h.rr0) : 0.0;
  c->have_du = true;
  if (h.done == 1) return TG_OK;
  if (h.done == 2) {
    static const char* why[] = {"", "non-finite initial residual", "p.Ap <= 0 (indefinite operator)",
                                "non-finite p.Ap", "non-finite r.z or r.r",
                                "staged tile or grid barrier wait timed out"};
    c->err = std::string("PCG breakdown: ") + why[h.fail >= 1 && h.fail <= 5 ? h.fail : 0] + " at iteration " +
             std::to_string(h.iters);
    return TG_ERR_NAN;
  }
  c->err = "PCG iteration limit reached";
  return TG_ERR_NOT_CONVERGED;
}

namespace {

// rhs = R - K v on the node-block matrix (prescribed rows are zero in K and
// in R), accumulated in FP64 whatever the matrix precision
template <typename T>
__global__ void __launch_bounds__(256) lift_rhs_kernel(int nnd, const int* __restrict__ rowptr,
                                                       const int* __restrict__ row_tile,
                                                       const long long* __restrict__ blob_off,
                                                       const unsigned char* __restrict__ blob,
                                                       const double4_32a* __restrict__ v_all,
                                                       const double4_32a* __restrict__ R,
                                                       double4_32a* __restrict__ rhs_all) {
  // grid rows (blockIdx.y) are independent vectors v, rhs (nnd apart)
  const double4_32a* __restrict__ v = v_all + (long long)blockIdx.y * nnd;
  double4_32a* __restrict__ rhs = rhs_all + (long long)blockIdx.y * nnd;
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; I < nnd; I += warps) {
    const unsigned char* base = blob + blob_off[row_tile[I]];
    const int* hdr = reinterpret_cast<const int*>(base);
    const int r0 = hdr[0], nrows = hdr[1], nb = hdr[2], ps = hdr[3];
    const int* rp = hdr + 4;
    const int* cl = rp + ceil4(nrows + 1);
    const T* pl = reinterpret_cast<const T*>(cl + ceil4(nb));
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    const int e1 = rp[I - r0 + 1];
    for (int j = rp[I - r0] + lane; j < e1; j += 32) {
      const double4_32a vj = v[cl[j]];
      // v is a prescribed increment, zero away from the prescribed nodes: a
      // zero column block adds a signed zero to a sum that is never -0, so
      // skipping it (and its value reads) leaves the result bitwise the same
      if (vj.x == 0.0 && vj.y == 0.0 && vj.z == 0.0) continue;
      const T* vv = pl + j;
      a0 += (double)vv[0 * ps] * vj.x + (double)vv[1 * ps] * vj.y + (double)vv[2 * ps] * vj.z;
      a1 += (double)vv[3 * ps] * vj.x + (double)vv[4 * ps] * vj.y + (double)vv[5 * ps] * vj.z;
      a2 += (double)vv[6 * ps] * vj.x + (double)vv[7 * ps] * vj.y + (double)vv[8 * ps] * vj.z;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, o);
      a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if (lane == 0) {
      const double4_32a r = R ? R[I] : make_double4_32a(0.0, 0.0, 0.0, 0.0);
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
                                       const PcgScalars* __restrict__ sc, double* __restrict__ eq) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= neq) return;
  const int s = slot[k];
  const V v = x[s >> 2];
  const int d = s & 3;
  eq[k] = sc->unscale * (double)(d == 0 ? v.x : (d == 1 ? v.y : v.z));
}

}  // namespace

int launch_lift_rhs(Context* c, const double4_32a* d_v, double4_32a* d_rhs, bool zero_base, int nvec) {
  {
    const int sf = ensure_full_assembly(c);
    if (sf) return sf;
  }
  const double4_32a* base = zero_base ? nullptr : c->d_R;
  Grids g = grids(c);
  const dim3 grid(std::min((c->nnd + 7) / 8, c->num_sms * 8), nvec);
  if (c->tangent_precision == TG_MIXED)
    lift_rhs_kernel<float><<<grid, 256, 0, c->stream>>>(c->nnd, c->d_rowptr, c->d_row_tile, c->d_blob_off32,
                                                         c->d_blob32, d_v, base, d_rhs);
  else
    lift_rhs_kernel<double><<<grid, 256, 0, c->stream>>>(c->nnd, c->d_rowptr, c->d_row_tile, c->d_blob_off64,
                                                          c->d_blob64, d_v, base, d_rhs);
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
    gather_solution_kernel<float4><<<grid, 256, 0, c->stream>>>(c->neq, c->d_eq_slot, (const float4*)c->d_x, c->d_pcg, d_eq);
  else
    gather_solution_kernel<double4_32a><<<grid, 256, 0, c->stream>>>(c->neq, c->d_eq_slot, (const double4_32a*)c->d_x, c->d_pcg,
                                                                      d_eq);
  c->launches++;
  return ok(c, cudaGetLastError(), "gather_solution_kernel") ? TG_OK : TG_ERR_CUDA;
}

// Average device time of standalone launches of the two PCG kernels on the
// current tangent, with the scalars pinned so every launch does the same work
// (alpha = 0: x and r unchanged; the product is q = A p).
template <typename T>
int time_pcg_t(Context* c, int which, int reps, double* ms) {
  {
    const int sf = ensure_full_assembly(c);
    if (sf) return sf;
  }
  using V = typename Vec4<T>::type;
  const int precision = std::is_same<T, float>::value ? TG_MIXED : TG_FP64;
  int s = ensure_vectors<T>(c, precision);
  if (s) return s;
  const T* minv = std::is_same<T, float>::value ? (const T*)c->d_minv32 : (const T*)c->d_minv64;
  Grids g = grids(c);
  {
    const int sc = spmv_config<T>(c, g);
    if (sc) return sc;
  }
  pcg_scale_kernel<T><<<g.vec, 256, 0, c->stream>>>(c->nnd, c->d_R, c->d_mask, minv, c->d_partials, c->d_pcg);
  c->launches++;
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
      launch_spmv<T>(c, g, c->d_p, c->d_q, c->d_partials, c->d_pcg);
    else if (!ok(c, launch_update<T>(c, g.vec, minv, c->d_x, c->d_r, c->d_z, c->d_p, c->d_q, c->d_partials,
                                     c->d_pcg),
                 "pcg_update_kernel"))
      s = TG_ERR_CUDA;
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
  if (s) return s;
  return ok(c, cudaGetLastError(), "time_pcg_kernel") ? TG_OK : TG_ERR_CUDA;
}

int time_pcg_kernel(Context* c, int which, int reps, double* ms) {
  // the kernels the solve runs: the single-reduction form's own pair, or
  // the product of a segmented batch on the push storage
  if (c->nseg > 0 && which == 0 && push_active(c)) return time_seg_push(c, reps, ms);
  if (c->pcg_form == 1 && !sym_active(c) && c->nseg == 0) return time_cg_kernel(c, which, reps, ms);
  if (c->tangent_precision == TG_MIXED) return time_pcg_t<float>(c, which, reps, ms);
  if (c->tangent_precision == TG_FP64) return time_pcg_t<double>(c, which, reps, ms);
  c->err = "form the tangent first";
  return TG_ERR_ARG;
}

// ---- PCG on caller-provided scratch (used by tg_pcg_solve_noalloc) ------
namespace {

template <typename T>
int solve_scratch_t(Context* c, const double* d_rhs_eq, double* d_du_eq, unsigned char* scratch, double rel_tol,
                    int max_it, int precond, int* iters, double* rel_res) {
  using V = typename Vec4<T>::type;
  {
    const int sf = ensure_full_assembly(c);
    if (sf) return sf;
  }
  // scratch layout: scalars | partials | rhs (nodal FP64) | x r z p q
  unsigned char* cur = scratch;
  PcgScalars* sc = reinterpret_cast<PcgScalars*>(cur);
  cur += kScratchScalarBytes;
  double* partials = reinterpret_cast<double*>(cur);
  cur += kScratchPartialBytes;
  double4_32a* rhs = reinterpret_cast<double4_32a*>(cur);
  cur += sizeof(double4_32a) * (size_t)c->nnd;
  V* vec[5];
  for (int k = 0; k < 5; ++k) {
    vec[k] = reinterpret_cast<V*>(cur);
    cur += sizeof(V) * (size_t)c->nnd;
  }
  V *x = vec[0], *r = vec[1], *z = vec[2], *p = vec[3], *q = vec[4];
  // what must start at zero: the scalars (last-block counters) and the nodal
  // right-hand side (prescribed slots are never written by the scatter)
  if (!ok(c, cudaMemsetAsync(sc, 0, sizeof(PcgScalars), c->stream), "memset") ||
      !ok(c, cudaMemsetAsync(rhs, 0, sizeof(double4_32a) * (size_t)c->nnd, c->stream), "memset"))
    return TG_ERR_CUDA;
  int s = launch_scatter_eq(c, d_rhs_eq, rhs);
  if (s) return s;
  Grids g = grids(c);
  s = spmv_config<T>(c, g);
  if (s) return s;
  const T* minv_base = std::is_same<T, float>::value ? (const T*)c->d_minv32 : (const T*)c->d_minv64;
  const T* minv = minv_base + (precond == TG_PRECOND_BLOCK_JACOBI ? (long long)c->nnd * 9 : 0);
  g.warp_release = 0;  // the CTA-barrier product
  pcg_scale_kernel<T><<<g.vec, 256, 0, c->stream>>>(c->nnd, rhs, c->d_mask, minv, partials, sc);
  pcg_init_kernel<T><<<g.vec, 256, 0, c->stream>>>(c->nnd, rhs, c->d_mask, minv, x, r, z, p, q, partials, sc,
                                                  rel_tol, max_it);
  c->launches += 2;
  if (!ok(c, cudaGetLastError(), "pcg init")) return TG_ERR_CUDA;
  const int max_chunks = max_it / kChunk + 2;
  for (int ch = 0; ch < max_chunks; ++ch) {
    for (int k = 0; k < kChunk; ++k) {
      launch_spmv<T>(c, g, p, q, partials, sc);
      if (!ok(c, launch_update<T>(c, g.vec, minv, x, r, z, p, q, partials, sc), "pcg_update_kernel"))
        return TG_ERR_CUDA;
    }
    c->launches += 2 * kChunk;
    if (!ok(c, cudaGetLastError(), "pcg chunk") ||
        !ok(c, cudaMemcpyAsync(c->h_pcg, sc, sizeof(PcgScalars), cudaMemcpyDeviceToHost, c->stream), "copy") ||
        !ok(c, cudaStreamSynchronize(c->stream), "pcg sync"))
      return TG_ERR_CUDA;
    if (c->h_pcg->done) break;
  }
  const PcgScalars h = *c->h_pcg;
  if (iters) *iters = h.iters;
  if (rel_res) *rel_res = h.rr0 > 0 ? std::sqrt(h.rr / h.rr0) : 0.0;
  if (h.done == 2) {
    c->err = "PCG breakdown";
    return TG_ERR_NAN;
  }
  if (c->neq > 0) {
    gather_solution_kernel<V><<<(c->neq + 255) / 256, 256, 0, c->stream>>>(c->neq, c->d_eq_slot, x, sc, d_du_eq);
    c->launches++;
  }
  if (!ok(c, cudaGetLastError(), "gather") || !ok(c, cudaStreamSynchronize(c->stream), "sync")) return TG_ERR_CUDA;
  if (h.done == 1) return TG_OK;
  c->err = "PCG iteration limit reached";
  return TG_ERR_NOT_CONVERGED;
}

}  // namespace

size_t pcg_scratch_bytes(const Context* c) {
  const size_t v = c->tangent_precision == TG_MIXED ? sizeof(float4) : sizeof(double4_32a);
  return kScratchScalarBytes + kScratchPartialBytes + (sizeof(double4_32a) + 5 * v) * (size_t)c->nnd;
}

int pcg_solve_scratch(Context* c, const double* d_rhs_eq, double* d_du_eq, unsigned char* scratch, double rel_tol,
                      int max_it, int precond, int* iters, double* rel_res) {
  if (c->tangent_precision == TG_MIXED)
    return solve_scratch_t<float>(c, d_rhs_eq, d_du_eq, scratch, rel_tol, max_it, precond, iters, rel_res);
  return solve_scratch_t<double>(c, d_rhs_eq, d_du_eq, scratch, rel_tol, max_it, precond, iters, rel_res);
}

int pcg_vectors(Context* c, int precision) {
  return precision == TG_MIXED ? ensure_vectors<float>(c, precision) : ensure_vectors<double>(c, precision);
}

int spmv_grid_for(Context* c, long long cap32) {
  const size_t cap = (size_t)((cap32 + 127) / 128 * 128);
  const int nst = c->spmv_stages == 3 ? 3 : 2;
  int optin = 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device) != cudaSuccess) return 0;
  if ((size_t)nst * cap + 1024 > (size_t)optin) return 0;
  auto kern = c->spmv_warp_release ? (nst == 3 ? pcg_spmv_wr_kernel<float, 3> : pcg_spmv_wr_kernel<float, 2>)
                                   : (nst == 3 ? pcg_spmv_kernel<float, 3> : pcg_spmv_kernel<float, 2>);
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, kern) != cudaSuccess ||
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes) !=
          cudaSuccess)
    return 0;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, (size_t)nst * cap) != cudaSuccess) return 0;
  return c->num_sms * per_sm;
}

int spmv_plan(Context* c, int precision, SpmvPlan& P) {
  P = grids(c);
  return precision == TG_MIXED ? spmv_config<float>(c, P) : spmv_config<double>(c, P);
}

void spmv_run(Context* c, int precision, const SpmvPlan& P, const void* p, void* q, double* partials, PcgScalars* sc,
              double* node_dot) {
  if (precision == TG_MIXED)
    launch_spmv<float>(c, P, p, q, partials, sc, node_dot);
  else
    launch_spmv<double>(c, P, p, q, partials, sc, node_dot);
}

int pcg_solve(Context* c, const double4_32a* d_rhs, double rel_tol, int max_it, int precond, int* iters,
              double* rel_res) {
  // a solve that streams the full storage: its values from the last tangent
  if (!push_solve(c)) {
    const int sf = ensure_full_assembly(c);
    if (sf) return sf;
  }
  // a batch of RVEs: one Krylov solve per RVE over the shared matrix stream
  if (c->nseg > 0 && c->seg_pcg_mode) return pcg_solve_segmented(c, d_rhs, rel_tol, max_it, precond, iters, rel_res);
  const int prec = c->tangent_precision;
  if ((prec == TG_MIXED || prec == TG_FP64) && c->pcg_form == 1 && !sym_active(c))
    return pcg_solve_cg(c, prec, d_rhs, rel_tol, max_it, precond, iters, rel_res);
  if (prec == TG_MIXED) return solve_t<float>(c, d_rhs, rel_tol, max_it, precond, iters, rel_res);
  if (prec == TG_FP64) return solve_t<double>(c, d_rhs, rel_tol, max_it, precond, iters, rel_res);
  c->err = "tg_pcg_solve: no tangent formed";
  return TG_ERR_ARG;
}

}  // namespace tg
