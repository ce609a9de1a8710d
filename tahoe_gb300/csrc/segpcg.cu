// Per-RVE Krylov solves of a segmented batch, sm_103a.
//
// A batch of independent RVEs is one disconnected mesh on the device (RVE r
// owns nodes [node_off[r], node_off[r+1])).  The matrix product streams the
// whole batch at once -- that is where the bandwidth goes -- but every RVE
// runs its own (block-)Jacobi CG: its own right-hand-side scaling, its own
// alpha and beta, its own convergence test relative to its own initial
// residual, its own iteration count and breakdown status.  An RVE that has
// converged (or broken down) is frozen: its solution stays as it is, its
// nodes take no further update.  So one RVE's solve does not depend on which
// other RVEs share the batch, and a failing RVE fails alone.
//
// Recurrences: the single-reduction form of CG (Chronopoulos & Gear, J.
// Comput. Appl. Math. 25 (1989) 153-168): per iteration the product
// w = A z with each row's own z.w written per node, a per-RVE reduction of
// z.w giving alpha = gamma / (z.w - beta gamma / alpha_old) and
// beta = gamma / gamma_old, and one streaming update p = z + beta p,
// s = w + beta s (s = A p by recurrence), x += alpha p, r -= alpha s,
// z = M^-1 r with the per-RVE reduction of r.z (the next gamma) and r.r.
// Three kernels per iteration, captured in a CUDA graph in chunks.
//
// Reductions: an RVE's nodes are cut into chunks of kChunkNodes from its
// first node on; one CTA per chunk sums its nodes in a fixed order, and the
// last of the RVE's chunks to finish (an arrival counter per RVE) adds the
// chunk partials in chunk order.  Every sum therefore depends only on the
// RVE's own nodes, not on its position in the batch: an RVE solved alone
// and the same RVE inside any batch take bitwise the same iterates.
//
// The reference has no FE^2 driver (each RVE would be its own element group
// and solver, NLSolver.cpp:675-755 per RVE); this is that independence,
// kept while the batch shares one matrix stream.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "krylov_common.cuh"

namespace tg {

namespace {

constexpr int kChunkNodes = 1024;
constexpr int kSegChunk = 16;  // iterations per graph replay

// The RVE's iteration is over (converged, broken down or out of
// iterations): one fewer RVE iterating; the last one opens the gate that
// makes the batch's remaining product launches return at once.
__device__ __forceinline__ void seg_retire(SegControl* ctl, PcgScalars* gate) {
  if (atomicSub(&ctl->active, 1) == 1) gate->done = 1;
}

// Chunk totals (thread 0) into the partials; true in the RVE's last chunk to
// arrive, with the RVE totals (chunk order) on thread 0.
template <int NV>
__device__ __forceinline__ bool seg_last_chunk(const double (&bt)[NV], int chunk, int c0, int nch, double* part,
                                               unsigned int* counter, double (&tot)[NV]) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) part[(long long)chunk * NV + k] = bt[k];
    __threadfence();
    last = atomicAdd(counter, 1u) == (unsigned)(nch - 1);
  }
  __syncthreads();
  if (!last) return false;
  if (threadIdx.x == 0) {
    __threadfence();
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double a = 0.0;
      for (int i = 0; i < nch; ++i) a += ((volatile double*)part)[(long long)(c0 + i) * NV + k];
      tot[k] = a;
    }
    *counter = 0u;
  }
  return true;
}

template <typename T>
__global__ void __launch_bounds__(256) seg_scale_kernel(const int4* __restrict__ chunks,
                                                        const int* __restrict__ seg_chunk0,
                                                        const uint8_t* __restrict__ active,
                                                        const double4_32a* __restrict__ rhs,
                                                        const uint8_t* __restrict__ mask, const T* __restrict__ minv,
                                                        double* part, unsigned int* count, SegScalars* ssc) {
  const int4 ch = chunks[blockIdx.x];
  const int sg = ch.x;
  if (!active[sg]) return;  // the same for every chunk of the RVE
  Acc<double> v[1];
  for (int n = ch.y + threadIdx.x; n < ch.z; n += blockDim.x) {
    const double4_32a b = rhs[n];
    const uint8_t m = mask[n];
    const double bx = (m & 1) ? b.x : 0.0, by = (m & 2) ? b.y : 0.0, bz = (m & 4) ? b.z : 0.0;
    const T* B = minv + (long long)n * 9;
    const double zx = (double)B[0] * bx + (double)B[1] * by + (double)B[2] * bz;
    const double zy = (double)B[3] * bx + (double)B[4] * by + (double)B[5] * bz;
    const double zz = (double)B[6] * bx + (double)B[7] * by + (double)B[8] * bz;
    v[0].add(bx * zx + by * zy + bz * zz);
  }
  double bt[1], tot[1];
  block_total<double, 1>(v, bt);
  const int c0 = seg_chunk0[sg], nch = seg_chunk0[sg + 1] - c0;
  if (seg_last_chunk<1>(bt, blockIdx.x, c0, nch, part, &count[sg], tot) && threadIdx.x == 0) {
    const double sc = (tot[0] > 0.0 && isfinite(tot[0])) ? 1.0 / sqrt(tot[0]) : 1.0;
    ssc[sg].scale = sc;
    ssc[sg].unscale = 1.0 / sc;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) seg_init_kernel(
    const int4* __restrict__ chunks, const int* __restrict__ seg_chunk0, const uint8_t* __restrict__ active,
    const double4_32a* __restrict__ rhs, const uint8_t* __restrict__ mask, const T* __restrict__ minv,
    typename Vec4<T>::type* x, typename Vec4<T>::type* r, typename Vec4<T>::type* z, typename Vec4<T>::type* p,
    typename Vec4<T>::type* s, typename Vec4<T>::type* w, double* part, unsigned int* count, SegScalars* ssc,
    SegControl* ctl, PcgScalars* gate, double tol, int max_it) {
  using V = typename Vec4<T>::type;
  const int4 ch = chunks[blockIdx.x];
  const int sg = ch.x;
  const V zero = mk<V, T>(T(0), T(0), T(0));
  if (!active[sg]) {
    // not solved: zero update, iterates cleared
    for (int n = ch.y + threadIdx.x; n < ch.z; n += blockDim.x) x[n] = r[n] = z[n] = p[n] = s[n] = w[n] = zero;
    if (ch.w == 0 && threadIdx.x == 0) {
      SegScalars q = {};
      q.scale = q.unscale = 1.0;
      q.done = 1;
      ssc[sg] = q;
    }
    return;
  }
  const double scale = ssc[sg].scale;
  Acc<T> v[2];
  for (int n = ch.y + threadIdx.x; n < ch.z; n += blockDim.x) {
    const double4_32a b = rhs[n];
    const uint8_t mk_ = mask[n];
    const T rx = (mk_ & 1) ? T(b.x * scale) : T(0), ry = (mk_ & 2) ? T(b.y * scale) : T(0),
            rz = (mk_ & 4) ? T(b.z * scale) : T(0);
    T zx, zy, zz;
    apply_minv<T>(minv, n, rx, ry, rz, zx, zy, zz);
    x[n] = p[n] = s[n] = w[n] = zero;
    r[n] = mk<V, T>(rx, ry, rz);
    z[n] = mk<V, T>(zx, zy, zz);
    v[0].add_prod(rx, zx);
    v[0].add_prod(ry, zy);
    v[0].add_prod(rz, zz);
    v[1].add_prod(rx, rx);
    v[1].add_prod(ry, ry);
    v[1].add_prod(rz, rz);
  }
  double bt[2], tot[2];
  block_total<T, 2>(v, bt);
  const int c0 = seg_chunk0[sg], nch = seg_chunk0[sg + 1] - c0;
  if (seg_last_chunk<2>(bt, blockIdx.x, c0, nch, part, &count[sg], tot) && threadIdx.x == 0) {
    SegScalars& q = ssc[sg];
    q.rz = tot[0];
    q.rz_old = 0.0;
    q.rr = q.rr0 = tot[1];
    q.alpha = q.beta = 0.0;
    q.iters = 0;
    q.fail = 0;
    q.tol2 = tol * tol;
    q.max_it = max_it;
    q.done = (tot[1] == 0.0) ? 1 : (isfinite(tot[0]) && isfinite(tot[1]) ? 0 : 2);
    if (q.done == 2) q.fail = 1;
    if (q.done) seg_retire(ctl, gate);
  }
}

// alpha and beta of every iterating RVE from the rows' z.w
__global__ void __launch_bounds__(256) seg_alpha_kernel(const int4* __restrict__ chunks,
                                                        const int* __restrict__ seg_chunk0,
                                                        const double* __restrict__ node_dot, double* part,
                                                        unsigned int* count, SegScalars* ssc, SegControl* ctl,
                                                        PcgScalars* gate) {
  const int4 ch = chunks[blockIdx.x];
  const int sg = ch.x;
  if (((volatile SegScalars*)ssc)[sg].done) return;  // set only by earlier kernels: the same for every chunk
  Acc<double> v[1];
  for (int n = ch.y + threadIdx.x; n < ch.z; n += blockDim.x) v[0].add(node_dot[n]);
  double bt[1], tot[1];
  block_total<double, 1>(v, bt);
  const int c0 = seg_chunk0[sg], nch = seg_chunk0[sg + 1] - c0;
  if (seg_last_chunk<1>(bt, blockIdx.x, c0, nch, part, &count[sg], tot) && threadIdx.x == 0) {
    SegScalars& q = ssc[sg];
    const double g = q.rz;
    double beta = 0.0, den = tot[0];
    if (q.iters > 0) {
      beta = g / q.rz_old;
      den = tot[0] - beta * g / q.alpha;
    }
    if (!(den > 0.0) || !isfinite(den)) {
      q.done = 2;
      q.fail = isfinite(den) ? 2 : 3;
      seg_retire(ctl, gate);
    } else {
      q.alpha = g / den;
      q.beta = beta;
    }
  }
}

// With the push storage (PUSH) the product's w holds the upper part of A z:
// a node's w is completed from its push slots (rank planes of pstride, in
// rank order, the prescribed dofs left out), and a 128-byte plane line whose
// nodes all lie in this warp's pass and this chunk is dropped from L2 once
// read (chunks start at any node, so lines at their edges are left as they
// are: another CTA may still read them).
template <typename T, bool PUSH>
__global__ void __launch_bounds__(256) seg_update_kernel(
    const int4* __restrict__ chunks, const int* __restrict__ seg_chunk0, const T* __restrict__ minv,
    typename Vec4<T>::type* __restrict__ x, typename Vec4<T>::type* __restrict__ r,
    typename Vec4<T>::type* __restrict__ z, typename Vec4<T>::type* __restrict__ p,
    typename Vec4<T>::type* __restrict__ s, const typename Vec4<T>::type* __restrict__ w, double* part,
    unsigned int* count, SegScalars* ssc, SegControl* ctl, PcgScalars* gate,
    const typename Vec4<T>::type* __restrict__ push, const int* __restrict__ lptr, const uint8_t* __restrict__ mask,
    int pstride) {
  using V = typename Vec4<T>::type;
  const int4 ch = chunks[blockIdx.x];
  const int sg = ch.x;
  if (((volatile SegScalars*)ssc)[sg].done) return;
  const T alpha = T(ssc[sg].alpha), beta = T(ssc[sg].beta);
  const int lane = threadIdx.x & 31;
  Acc<T> v[2];
  // warps iterate together (the push lines are dropped per warp)
  for (int nb = ch.y + (int)(threadIdx.x & ~31u); nb < ch.z; nb += blockDim.x) {
    const int n = nb + lane;
    const bool live = n < ch.z;
    V wn = mk<V, T>(T(0), T(0), T(0));
    if (live) wn = w[n];
    if (PUSH) {
      const uint64_t keep = l2_policy_evict_last();
      T s0 = T(0), s1 = T(0), s2 = T(0);
      const int cnt = live ? lptr[n + 1] - lptr[n] : 0;
#pragma unroll 4
      for (int k = 0; k < cnt; ++k) {
        const V pv = ld_hint(push + ((long long)k * pstride + n), keep);
        s0 += pv.x;
        s1 += pv.y;
        s2 += pv.z;
      }
      if (live) {
        const uint8_t m = mask[n];
        wn = mk<V, T>(wn.x + ((m & 1) ? s0 : T(0)), wn.y + ((m & 2) ? s1 : T(0)), wn.z + ((m & 4) ? s2 : T(0)));
      }
      constexpr int kLine = 128 / (int)sizeof(V);  // slots per line
      // the largest count over the kLine nodes from this lane on (the
      // warp base need not be line aligned)
      int lc = 0;
#pragma unroll
      for (int j = 0; j < kLine; ++j) lc = max(lc, __shfl_sync(0xffffffffu, cnt, (lane + j) & 31));
      __syncwarp();
      const int last = min(nb + 31, ch.z - 1);  // the warp pass's last node of this chunk
      if ((n % kLine) == 0 && n >= ch.y && n + kLine - 1 <= last)
        for (int k = 0; k < lc; ++k) l2_discard(push + ((long long)k * pstride + n));
    }
    if (!live) continue;
    const V zn = z[n], pn = p[n], sn = s[n], xn = x[n], rn = r[n];
    T B[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) B[k] = minv[(long long)n * 9 + k];
    const T px = zn.x + beta * pn.x, py = zn.y + beta * pn.y, pz = zn.z + beta * pn.z;
    const T sx = wn.x + beta * sn.x, sy = wn.y + beta * sn.y, sz = wn.z + beta * sn.z;
    const T rx = rn.x - alpha * sx, ry = rn.y - alpha * sy, rz = rn.z - alpha * sz;
    const T zx = B[0] * rx + B[1] * ry + B[2] * rz;
    const T zy = B[3] * rx + B[4] * ry + B[5] * rz;
    const T zz = B[6] * rx + B[7] * ry + B[8] * rz;
    p[n] = mk<V, T>(px, py, pz);
    s[n] = mk<V, T>(sx, sy, sz);
    x[n] = mk<V, T>(xn.x + alpha * px, xn.y + alpha * py, xn.z + alpha * pz);
    r[n] = mk<V, T>(rx, ry, rz);
    z[n] = mk<V, T>(zx, zy, zz);
    v[0].add_prod(rx, zx);
    v[0].add_prod(ry, zy);
    v[0].add_prod(rz, zz);
    v[1].add_prod(rx, rx);
    v[1].add_prod(ry, ry);
    v[1].add_prod(rz, rz);
  }
  double bt[2], tot[2];
  block_total<T, 2>(v, bt);
  const int c0 = seg_chunk0[sg], nch = seg_chunk0[sg + 1] - c0;
  if (seg_last_chunk<2>(bt, blockIdx.x, c0, nch, part, &count[sg], tot) && threadIdx.x == 0) {
    SegScalars& q = ssc[sg];
    const int it = q.iters + 1;
    q.iters = it;
    q.rz_old = q.rz;
    q.rz = tot[0];
    q.rr = tot[1];
    int done = 0;
    if (!isfinite(tot[0]) || !isfinite(tot[1])) {
      q.fail = 4;
      done = 2;
    } else if (tot[1] <= q.tol2 * q.rr0) {
      done = 1;
    } else if (it >= q.max_it) {
      done = 3;
    }
    if (done) {
      q.done = done;
      seg_retire(ctl, gate);
    }
  }
}

// A push tile takes part in the next product while one of its RVEs (its
// rows' first to last) still iterates; the tiles of converged or failed RVEs
// are skipped (RVEs share no blocks, so nothing an iterating RVE reads comes
// from them).  Read by the product only: the flags hold for its whole launch.
__global__ void seg_tile_active_kernel(int ntiles, const int2* __restrict__ tile_seg,
                                       const SegScalars* __restrict__ ssc, uint8_t* __restrict__ act) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  const int2 r = tile_seg[t];
  uint8_t a = 0;
  for (int sg = r.x; sg <= r.y && !a; ++sg) a = ssc[sg].done == 0 ? 1 : 0;
  act[t] = a;
}

// the solution back to the unscaled right-hand side; an RVE that broke
// down takes no update
template <typename T>
__global__ void __launch_bounds__(256) seg_finish_kernel(const int4* __restrict__ chunks,
                                                         const SegScalars* __restrict__ ssc,
                                                         typename Vec4<T>::type* __restrict__ x, PcgScalars* sc) {
  using V = typename Vec4<T>::type;
  const int4 ch = chunks[blockIdx.x];
  const SegScalars& q = ssc[ch.x];
  const T u = q.done == 2 ? T(0) : T(q.unscale);
  for (int n = ch.y + threadIdx.x; n < ch.z; n += blockDim.x) {
    const V xn = x[n];
    x[n] = mk<V, T>(u * xn.x, u * xn.y, u * xn.z);
  }
  // the solution is unscaled in place: the update applies it as it is
  if (blockIdx.x == 0 && threadIdx.x == 0) sc->unscale = 1.0;
}

int ensure_seg(Context* c) {
  SegSolve& S = c->seg;
  if (S.built) return TG_OK;
  if ((int)c->h_seg_node.size() != c->nseg + 1) {
    c->err = "segmented solve: no RVE partition";
    return TG_ERR_ARG;
  }
  std::vector<int4> chunks;
  std::vector<int> c0(c->nseg + 1, 0);
  for (int sg = 0; sg < c->nseg; ++sg) {
    c0[sg] = (int)chunks.size();
    const int a = c->h_seg_node[sg], b = c->h_seg_node[sg + 1];
    int k = 0;
    for (int n = a; n < b; n += kChunkNodes, ++k) chunks.push_back(make_int4(sg, n, std::min(b, n + kChunkNodes), k));
    if (a == b) {
      c->err = "segmented solve: an RVE without nodes";
      return TG_ERR_ARG;
    }
  }
  c0[c->nseg] = (int)chunks.size();
  S.nchunks = (int)chunks.size();
  if (!dalloc(c, &S.d_chunk, chunks.size()) || !dalloc(c, &S.d_seg_chunk0, c0.size()) ||
      !dalloc(c, &S.d_sc, (size_t)c->nseg) || !dalloc(c, &S.d_count, (size_t)c->nseg) ||
      !dalloc(c, &S.d_part, (size_t)S.nchunks * 2) || !dalloc(c, &S.d_node_dot, (size_t)c->nnd) ||
      !dalloc(c, &S.d_active, (size_t)c->nseg) || !dalloc(c, &S.d_ctl, 1) || !dalloc(c, &S.d_gate, 1))
    return TG_ERR_OOM;
  cudaStream_t st = c->stream;
  if (!ok(c, cudaMemcpyAsync(S.d_chunk, chunks.data(), sizeof(int4) * chunks.size(), cudaMemcpyHostToDevice, st),
          "chunks") ||
      !ok(c, cudaMemcpyAsync(S.d_seg_chunk0, c0.data(), sizeof(int) * c0.size(), cudaMemcpyHostToDevice, st), "c0") ||
      !ok(c, cudaMemsetAsync(S.d_count, 0, sizeof(unsigned int) * c->nseg, st), "count") ||
      !ok(c, cudaMemsetAsync(S.d_sc, 0, sizeof(SegScalars) * c->nseg, st), "sc") ||
      !ok(c, cudaStreamSynchronize(st), "sync"))
    return TG_ERR_CUDA;
  S.built = true;
  return TG_OK;
}

// first and last RVE of every push tile's rows (per mesh and partition)
int seg_tile_ranges(Context* c) {
  SegSolve& S = c->seg;
  const PushStore& ps = c->push;
  if (S.d_tile_seg && S.tile_seg_n == ps.ntiles) return TG_OK;
  if (S.d_tile_seg) dfree(c, S.d_tile_seg);
  if (S.d_tile_act) dfree(c, S.d_tile_act);
  S.d_tile_seg = nullptr;
  S.d_tile_act = nullptr;
  const std::vector<int>& tr = ps.h_tile_row;
  const std::vector<int>& sn = c->h_seg_node;
  if ((int)tr.size() != ps.ntiles + 1 || (int)sn.size() != c->nseg + 1) {
    c->err = "segmented solve: push tiles or RVE partition missing";
    return TG_ERR_ARG;
  }
  std::vector<int2> rng(ps.ntiles);
  for (int t = 0; t < ps.ntiles; ++t) {
    // RVE of a row: the last RVE whose first node is at most the row
    auto seg_of = [&](int row) { return (int)(std::upper_bound(sn.begin(), sn.end(), row) - sn.begin()) - 1; };
    rng[t] = make_int2(seg_of(tr[t]), seg_of(tr[t + 1] - 1));
  }
  if (!dalloc(c, &S.d_tile_seg, (size_t)ps.ntiles) || !dalloc(c, &S.d_tile_act, (size_t)ps.ntiles))
    return TG_ERR_OOM;
  if (!ok(c, cudaMemcpyAsync(S.d_tile_seg, rng.data(), sizeof(int2) * ps.ntiles, cudaMemcpyHostToDevice, c->stream),
          "tile ranges") ||
      !ok(c, cudaStreamSynchronize(c->stream), "sync"))
    return TG_ERR_CUDA;
  S.tile_seg_n = ps.ntiles;
  return TG_OK;
}

template <typename T>
int capture_seg_chunk(Context* c, const T* minv, int precision) {
  using V = typename Vec4<T>::type;
  SegSolve& S = c->seg;
  const bool push = push_active(c);
  if (push) {
    const int sr = seg_tile_ranges(c);
    if (sr) return sr;
  }
  SpmvPlan plan;
  if (!push) {
    const int s = spmv_plan(c, precision, plan);
    if (s) return s;
  }
  const PushStore& ps = c->push;
  const V* pushbuf = reinterpret_cast<const V*>(precision == TG_MIXED ? ps.d_push32 : ps.d_push64);
  cudaGraph_t graph;
  if (!ok(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture")) return TG_ERR_CUDA;
  cudaError_t le = cudaSuccess;
  int ls = TG_OK;
  for (int k = 0; k < kSegChunk && le == cudaSuccess && !ls; ++k) {
    if (push) {
      seg_tile_active_kernel<<<(S.tile_seg_n + 255) / 256, 256, 0, c->stream>>>(S.tile_seg_n, S.d_tile_seg, S.d_sc,
                                                                                S.d_tile_act);
      ls = launch_seg_push(c, precision, c->d_z, c->d_q, S.d_node_dot, S.d_gate, S.d_tile_act);
    } else
      spmv_run(c, precision, plan, c->d_z, c->d_q, c->d_partials, S.d_gate, S.d_node_dot);
    seg_alpha_kernel<<<S.nchunks, 256, 0, c->stream>>>(S.d_chunk, S.d_seg_chunk0, S.d_node_dot, S.d_part, S.d_count,
                                                      S.d_sc, S.d_ctl, S.d_gate);
    if (push)
      seg_update_kernel<T, true><<<S.nchunks, 256, 0, c->stream>>>(
          S.d_chunk, S.d_seg_chunk0, minv, (V*)c->d_x, (V*)c->d_r, (V*)c->d_z, (V*)c->d_p, (V*)S.d_s,
          (const V*)c->d_q, S.d_part, S.d_count, S.d_sc, S.d_ctl, S.d_gate, pushbuf, ps.d_lptr, c->d_mask,
          ps.pstride);
    else
      seg_update_kernel<T, false><<<S.nchunks, 256, 0, c->stream>>>(
          S.d_chunk, S.d_seg_chunk0, minv, (V*)c->d_x, (V*)c->d_r, (V*)c->d_z, (V*)c->d_p, (V*)S.d_s,
          (const V*)c->d_q, S.d_part, S.d_count, S.d_sc, S.d_ctl, S.d_gate, nullptr, nullptr, nullptr, 0);
    le = cudaGetLastError();
  }
  if (ls) {
    cudaGraph_t g2;
    if (cudaStreamEndCapture(c->stream, &g2) == cudaSuccess) cudaGraphDestroy(g2);
    return ls;
  }
  const cudaError_t ee = cudaStreamEndCapture(c->stream, &graph);
  if (!ok(c, le, "capture launch") || !ok(c, ee, "end capture")) {
    if (ee == cudaSuccess) cudaGraphDestroy(graph);
    return TG_ERR_CUDA;
  }
  if (S.graph) cudaGraphExecDestroy(S.graph);
  S.graph = nullptr;
  const cudaError_t e = cudaGraphInstantiate(&S.graph, graph, 0);
  cudaGraphDestroy(graph);
  return ok(c, e, "graph instantiate") ? TG_OK : TG_ERR_CUDA;
}

template <typename T>
int solve_seg_t(Context* c, const double4_32a* d_rhs, double rel_tol, int max_it, int precond, int* iters,
                double* rel_res) {
  using V = typename Vec4<T>::type;
  const int precision = std::is_same<T, float>::value ? TG_MIXED : TG_FP64;
  SegSolve& S = c->seg;
  int s = ensure_seg(c);
  if (!s) s = pcg_vectors(c, precision);
  if (s) return s;
  if (S.s_precision != precision || !S.d_s) {
    if (S.d_s) dfree(c, S.d_s);
    V* v = nullptr;
    if (!dalloc(c, &v, (size_t)c->nnd)) return TG_ERR_OOM;
    S.d_s = v;
    S.s_precision = precision;
    if (S.graph) cudaGraphExecDestroy(S.graph);
    S.graph = nullptr;
  }
  const T* minv_base = std::is_same<T, float>::value ? (const T*)c->d_minv32 : (const T*)c->d_minv64;
  const T* minv = minv_base + (precond == TG_PRECOND_BLOCK_JACOBI ? (long long)c->nnd * 9 : 0);
  // which RVEs this solve iterates (default: all)
  std::vector<uint8_t> act(c->nseg, 1);
  if ((int)c->seg_active.size() == c->nseg) act = c->seg_active;
  int nact = 0;
  for (uint8_t a : act) nact += a ? 1 : 0;
  SegControl ctl{nact, 0};
  PcgScalars gate;
  std::memset(&gate, 0, sizeof(gate));
  gate.done = nact == 0 ? 1 : 0;
  gate.unscale = 1.0;
  cudaStream_t st = c->stream;
  if (!ok(c, cudaMemcpyAsync(S.d_active, act.data(), act.size(), cudaMemcpyHostToDevice, st), "active") ||
      !ok(c, cudaMemcpyAsync(S.d_ctl, &ctl, sizeof(ctl), cudaMemcpyHostToDevice, st), "ctl") ||
      !ok(c, cudaMemcpyAsync(S.d_gate, &gate, sizeof(gate), cudaMemcpyHostToDevice, st), "gate"))
    return TG_ERR_CUDA;
  seg_scale_kernel<T><<<S.nchunks, 256, 0, st>>>(S.d_chunk, S.d_seg_chunk0, S.d_active, d_rhs, c->d_mask, minv,
                                                 S.d_part, S.d_count, S.d_sc);
  seg_init_kernel<T><<<S.nchunks, 256, 0, st>>>(S.d_chunk, S.d_seg_chunk0, S.d_active, d_rhs, c->d_mask, minv,
                                                (V*)c->d_x, (V*)c->d_r, (V*)c->d_z, (V*)c->d_p, (V*)S.d_s,
                                                (V*)c->d_q, S.d_part, S.d_count, S.d_sc, S.d_ctl, S.d_gate, rel_tol,
                                                max_it);
  c->launches += 2;
  if (!ok(c, cudaGetLastError(), "seg init")) return TG_ERR_CUDA;
  if (push_active(c)) {
    // the push storage's values follow the last assembly (before the
    // capture: the graph replays only the iteration)
    s = push_prepare(c, precision);
    if (s) return s;
  }
  const int key = precision * 4 + (precond == TG_PRECOND_BLOCK_JACOBI ? 1 : 0) + (push_active(c) ? 2 : 0);
  if (!S.graph || S.graph_key != key || S.graph_x != c->d_x) {
    s = capture_seg_chunk<T>(c, minv, precision);
    if (s) return s;
    S.graph_key = key;
    S.graph_x = c->d_x;
  }
  // gate copies alternate between the pinned mirrors; a chunk's flag is read
  // while the next chunk runs
  const int max_chunks = max_it / kSegChunk + 2;
  int last = 0;
  for (int k = 0; k < max_chunks && nact > 0; ++k) {
    if (!ok(c, cudaGraphLaunch(S.graph, st), "graph launch")) return TG_ERR_CUDA;
    c->launches += (push_active(c) ? 4 : 3) * kSegChunk;
    last = k & 1;
    if (!ok(c, cudaMemcpyAsync(&c->h_pcg[last], S.d_gate, sizeof(PcgScalars), cudaMemcpyDeviceToHost, st), "copy") ||
        !ok(c, cudaEventRecord(c->ev_poll[last], st), "event"))
      return TG_ERR_CUDA;
    if (k > 0) {
      if (!ok(c, cudaEventSynchronize(c->ev_poll[last ^ 1]), "pcg poll")) return TG_ERR_CUDA;
      if (c->h_pcg[last ^ 1].done) break;
    }
  }
  seg_finish_kernel<T><<<S.nchunks, 256, 0, st>>>(S.d_chunk, S.d_sc, (V*)c->d_x, c->d_pcg);
  c->launches++;
  S.h_sc.resize(c->nseg);
  if (!ok(c, cudaGetLastError(), "seg finish") ||
      !ok(c, cudaMemcpyAsync(S.h_sc.data(), S.d_sc, sizeof(SegScalars) * c->nseg, cudaMemcpyDeviceToHost, st), "sc") ||
      !ok(c, cudaMemcpyAsync(&c->h_pcg[0], S.d_gate, sizeof(PcgScalars), cudaMemcpyDeviceToHost, st), "gate") ||
      !ok(c, cudaStreamSynchronize(st), "pcg sync"))
    return TG_ERR_CUDA;
  c->have_du = true;
  int worst_it = 0, broke = 0, limit = 0;
  double worst_rel = 0.0;
  c->seg_status.assign(c->nseg, TG_OK);
  for (int i = 0; i < c->nseg; ++i) {
    if (!act[i]) continue;
    const SegScalars& q = S.h_sc[i];
    worst_it = std::max(worst_it, q.iters);
    if (q.rr0 > 0.0) worst_rel = std::max(worst_rel, std::sqrt(q.rr / q.rr0));
    if (q.done == 2) {
      c->seg_status[i] = TG_ERR_NAN;
      ++broke;
    } else if (q.done != 1) {
      c->seg_status[i] = TG_ERR_NOT_CONVERGED;
      ++limit;
    }
  }
  if (iters) *iters = worst_it;
  if (rel_res) *rel_res = worst_rel;
  if (c->h_pcg[0].done == 2 && c->h_pcg[0].fail == 5) {
    c->err = "PCG breakdown: staged tile wait timed out";
    return TG_ERR_NAN;
  }
  if (broke && (!c->seg_tolerate || broke == nact)) {
    c->err = "PCG breakdown in " + std::to_string(broke) + " of " + std::to_string(nact) + " RVEs";
    return TG_ERR_NAN;
  }
  if (limit) {
    c->err = "PCG iteration limit reached in " + std::to_string(limit) + " RVEs";
    return TG_ERR_NOT_CONVERGED;
  }
  return TG_OK;
}

}  // namespace

int pcg_solve_segmented(Context* c, const double4_32a* d_rhs, double rel_tol, int max_it, int precond, int* iters,
                        double* rel_res) {
  if (c->tangent_precision == TG_MIXED) return solve_seg_t<float>(c, d_rhs, rel_tol, max_it, precond, iters, rel_res);
  if (c->tangent_precision == TG_FP64) return solve_seg_t<double>(c, d_rhs, rel_tol, max_it, precond, iters, rel_res);
  c->err = "segmented PCG: no tangent formed";
  return TG_ERR_ARG;
}

void seg_free(Context* c) {
  SegSolve& S = c->seg;
  if (S.graph) cudaGraphExecDestroy(S.graph);
  for (void* p : {(void*)S.d_chunk, (void*)S.d_seg_chunk0, (void*)S.d_sc, (void*)S.d_count, (void*)S.d_part,
                  (void*)S.d_node_dot, S.d_s, (void*)S.d_active, (void*)S.d_ctl, (void*)S.d_gate,
                  (void*)S.d_tile_seg, (void*)S.d_tile_act})
    if (p) dfree(c, p);
  S = SegSolve{};
  c->seg_active.clear();
  c->seg_status.clear();
}

}  // namespace tg
