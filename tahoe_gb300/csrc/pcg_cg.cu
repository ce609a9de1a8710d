// Single-reduction PCG on the streamed node-block matrix, sm_103a.
//
// (Block-)Jacobi CG in the single-reduction form of Chronopoulos & Gear
// (J. Comput. Appl. Math. 25 (1989) 153-168), two kernels per iteration and
// no grid-wide synchronisation inside either of them:
//
//   product  w = A u; each CTA (one per SM) writes its partial of u.w
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
constexpr int kVecCap = 1024;      // vector-kernel CTAs
constexpr int kCtaCap = 1024;      // product CTAs
// partials (8-byte slots): two buffers of the vector kernel's {r.u
// [kVecCap], r.r [kVecCap]}, then the product's CTA partials [kCtaCap]
constexpr int kCgPartials = 4 * kVecCap;

// Programmatic dependent launch: a kernel lets the next one in the stream
// launch its CTAs as its own exit (launch_dependents), and a kernel that
// consumes the previous one's results waits for that grid's completion and
// memory (wait; a no-op when launched without the dependency).  Each kernel
// of the iteration does the work that does not depend on the previous one
// first -- the product stages its first matrix tiles, the vector kernel
// loads its nodes' vectors -- so that work overlaps the previous kernel's
// last CTAs and the launch gap.  A kernel releases its dependents only after
// its own wait: released earlier, the next vector kernel could start while
// the one before the product was still writing the vectors it preloads
// (seen on meshes small enough for all three grids to be resident at once).
__device__ __forceinline__ void griddep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// The rows of one staged tile of the symmetric push storage (pushfmt.cu):
// LPR lanes per row, each taking every LPR-th upper block of the row, the
// first K of them with every load issued before any use.  A block adds
// A_IJ u_J to the row's upper sum y_I; an off-diagonal block also stores
// A_IJ^T u_I at its push slot (row J's share of the product, added by the
// vector kernel).  The row's first block is its diagonal (its first lane),
// so u.w of the whole matrix is the sum over rows of u_I.(2 y_I - A_II u_I).
//
// With node_dot (a segmented batch) the row's own u_I.(2 y_I - A_II u_I) is
// written per node instead of accumulated (the batch reduces it per RVE).
template <typename T, int LPR>
__device__ __forceinline__ void push_tile_rows(const unsigned char* base, int lane, int warp, int nwarps,
                                               const typename Vec4<T>::type* __restrict__ uv,
                                               typename Vec4<T>::type* __restrict__ wup,
                                               typename Vec4<T>::type* __restrict__ push, Acc<T>& dot,
                                               double* __restrict__ node_dot) {
  using V = typename Vec4<T>::type;
  constexpr int RPW = 32 / LPR;  // rows per warp pass
  constexpr int K = 4;
  const int sub = lane % LPR, grp = lane / LPR;
  const int* hdr = reinterpret_cast<const int*>(base);
  const int r0 = hdr[0], nrows = hdr[1], nb = hdr[2], ps = hdr[3];
  const int* rp = hdr + 4;
  const int* cl = rp + ceil4(nrows + 1);
  const int* sl = cl + ceil4(nb);
  const T* pl = reinterpret_cast<const T*>(sl + ceil4(nb));
  // the pushes stay in L2 for the vector kernel that reads them next
  const uint64_t keep = l2_policy_evict_last();
  for (int li = warp * RPW + grp; li - grp < nrows; li += nwarps * RPW) {
    const bool live = li < nrows;
    const int I = r0 + li;
    V ui = mk<V, T>(T(0), T(0), T(0));
    if (live) ui = uv[I];
    const int e0 = live ? rp[li] : 0, e1 = live ? rp[li + 1] : 0;
    T a0 = T(0), a1 = T(0), a2 = T(0), d0 = T(0), d1 = T(0), d2 = T(0);
    auto block = [&](int j, const V& uj) {
      const T* vv = pl + j;
      const T m0 = vv[0 * ps], m1 = vv[1 * ps], m2 = vv[2 * ps], m3 = vv[3 * ps], m4 = vv[4 * ps],
              m5 = vv[5 * ps], m6 = vv[6 * ps], m7 = vv[7 * ps], m8 = vv[8 * ps];
      const T b0 = m0 * uj.x + m1 * uj.y + m2 * uj.z;
      const T b1 = m3 * uj.x + m4 * uj.y + m5 * uj.z;
      const T b2 = m6 * uj.x + m7 * uj.y + m8 * uj.z;
      a0 += b0;
      a1 += b1;
      a2 += b2;
      if (j == e0) {
        d0 = b0;
        d1 = b1;
        d2 = b2;
      } else {
        st_hint(push + sl[j],
                mk<V, T>(m0 * ui.x + m3 * ui.y + m6 * ui.z, m1 * ui.x + m4 * ui.y + m7 * ui.z,
                         m2 * ui.x + m5 * ui.y + m8 * ui.z),
                keep);
      }
    };
    {
      int Jk[K];
      V pk[K];
#pragma unroll
      for (int u = 0; u < K; ++u) {
        const int j = e0 + sub + LPR * u;
        Jk[u] = j < e1 ? cl[j] : -1;
      }
#pragma unroll
      for (int u = 0; u < K; ++u)
        if (Jk[u] >= 0) pk[u] = uv[Jk[u]];
#pragma unroll
      for (int u = 0; u < K; ++u)
        if (Jk[u] >= 0) block(e0 + sub + LPR * u, pk[u]);
    }
    for (int j = e0 + sub + LPR * K; j < e1; j += LPR) block(j, uv[cl[j]]);
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, o);
      a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if (live && sub == 0) {
      wup[I] = mk<V, T>(a0, a1, a2);
      if (node_dot) {
        Acc<T> d;
        d.add_prod(ui.x, T(2) * a0 - d0);
        d.add_prod(ui.y, T(2) * a1 - d1);
        d.add_prod(ui.z, T(2) * a2 - d2);
        node_dot[I] = d.value();
      } else {
        dot.add_prod(ui.x, T(2) * a0 - d0);
        dot.add_prod(ui.y, T(2) * a1 - d1);
        dot.add_prod(ui.z, T(2) * a2 - d2);
      }
    }
  }
}

constexpr int kPushLanes = 4;  // lanes per row of the push product (upper rows hold about 14 blocks)
constexpr bool kPushDiscard = true;  // read push lines are dropped from L2 without write-back

// The product on a persistent grid of 256-thread CTAs (as many as fit, a
// few per SM): w = A u and the CTA partials of u.w, with the matrix in the
// full storage (PUSH false) or the symmetric push storage (PUSH true: w holds
// the upper part, push the lower part's slots).  CTA b streams tiles b,
// b + G, ... through a ring of NST shared-memory stages filled by bulk
// copies on mbarriers (each stage refilled as soon as every warp is done with
// it); eight warps take each tile's rows.  The CTA's u.w is reduced in a
// fixed order into its partial.
// Every wait is bounded; a timeout flags the solve broken down in both
// scalar states and drains the copies in flight.  (Measured on C2: four
// such CTAs per SM stream the matrix faster than one CTA of four groups
// sharing the SM's tiles, and faster than tiles pulled from a global
// counter; the spread of finishing times is per SM, not per tile count.)
//
// SEG: the product of a segmented batch's per-RVE solves -- sc is the
// batch's gate (its done flag ends the launch at once), each row's own z.w
// goes to node_dot, and no CTA partial is written.
template <typename T, int NST, bool PUSH, bool SEG>
__device__ __forceinline__ void cg_product(int ntiles, const long long* __restrict__ blob_off,
                                           const unsigned char* __restrict__ blob, int cap, int keep,
                                           const typename Vec4<T>::type* __restrict__ p,
                                           typename Vec4<T>::type* __restrict__ q,
                                           typename Vec4<T>::type* __restrict__ push,
                                           typename Partial<T>::type* __restrict__ cta_part,
                                           double* __restrict__ node_dot, PcgScalars* sc, int* status,
                                           const uint8_t* __restrict__ tile_act) {
  using P = typename Partial<T>::type;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bars[NST];
  __shared__ int released[NST];  // warps done with the stage, over the whole launch
  __shared__ int nissued[NST];   // copies issued into the stage
  __shared__ int abort_flag;
  __shared__ int last_k;         // position of the last tile issued
  // SEG: the CTA's tiles that hold rows of an RVE still iterating (bit k:
  // tile t0 + k G), from the batch's per-tile flags; the tiles of converged
  // RVEs are neither copied nor multiplied
  constexpr int kActWords = SEG ? 256 : 1;
  __shared__ unsigned act_bits[kActWords];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int t0 = blockIdx.x, G = gridDim.x;
  const int nk = t0 < ntiles ? (ntiles - t0 + G - 1) / G : 0;  // this CTA's tiles
  const bool skip_tiles = SEG && tile_act && nk <= kActWords * 32;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NST; ++k) {
      mbar_init(&bars[k], 1);
      released[k] = 0;
      nissued[k] = 0;
    }
    fence_mbar_init();
    abort_flag = 0;
    last_k = -1;
  }
  if (SEG) {
    for (int w = threadIdx.x; w < kActWords; w += blockDim.x) act_bits[w] = 0u;
    __syncthreads();
    if (skip_tiles)
      for (int k = threadIdx.x; k < nk; k += blockDim.x)
        if (tile_act[t0 + (long long)k * G]) atomicOr(&act_bits[k >> 5], 1u << (k & 31));
  }
  __syncthreads();
  // the first active position >= k (nk if none); every position without
  // the flags
  auto next_k = [&](int k) {
    if (!skip_tiles) return k;
    while (k < nk) {
      const unsigned w = act_bits[k >> 5] >> (k & 31);
      if (w) return k + __ffs((int)w) - 1;
      k = (k | 31) + 1;
    }
    return nk;
  };
  // tile t into stage st (one thread)
  auto issue = [&](int t, int st) {
    nissued[st] += 1;
    const long long o0 = blob_off[t], o1 = blob_off[t + 1];
    const unsigned bytes = (unsigned)(o1 - o0);
    mbar_expect_tx(&bars[st], bytes);
    if (keep < 0)
      bulk_copy(smem + (size_t)st * cap, blob + o0, bytes, &bars[st]);
    else
      bulk_copy_hint(smem + (size_t)st * cap, blob + o0, bytes, &bars[st],
                     t < keep ? l2_policy_evict_last() : l2_policy_evict_first());
  };
  // copies still in flight complete before the CTA leaves (bounded waits;
  // at most one copy per stage can be pending)
  auto drain = [&]() {
#pragma unroll
    for (int k = 0; k < NST; ++k)
      if (nissued[k] > 0) mbar_wait(&bars[k], (unsigned)((nissued[k] - 1) & 1), kWaitLimit);
  };
  // the first NST tiles (the matrix does not depend on the last vector kernel)
  if (threadIdx.x == 0) {
    int k = next_k(0);
    for (int st = 0; st < NST && k < nk; ++st) {
      issue(t0 + k * G, st);
      last_k = k;
      k = next_k(k + 1);
    }
  }
  griddep_wait();  // u and the scalars of the last vector kernel
  griddep_launch();
  if (skip_launch(sc, SEG ? 0 : 1)) {
    if (threadIdx.x == 0) drain();
    return;
  }
  // Each warp takes its rows of every staged tile without waiting for the
  // other warps: the warp that finishes a stage last refills it with the
  // CTA's tile NST positions ahead (release: each warp's reads of the stage
  // happen before its count; the last counter orders them before the bulk
  // copy through the proxy fence).  A CTA barrier per tile made every warp
  // wait for the slowest one (the largest stall of the product).
  Acc<T> v;
  int it = 0;
  for (int k = next_k(0); k < nk; k = next_k(k + 1), ++it) {
    const int t = t0 + k * G;
    const int s = it % NST;
    if (!mbar_wait(&bars[s], (unsigned)((it / NST) & 1), kWaitLimit)) atomicOr(&abort_flag, 1);
    __syncwarp();
    if (*(volatile int*)&abort_flag) break;
    if (PUSH)
      push_tile_rows<T, kPushLanes>(smem + (size_t)s * cap, lane, warp, nwarps, p, q, push, v,
                                    SEG ? node_dot : nullptr);
    else
      spmv_tile_rows<T>(smem + (size_t)s * cap, lane, warp, nwarps, p, q, v, SEG ? node_dot : nullptr);
    __syncwarp();
    if (lane == 0) {
      __threadfence_block();
      const int done = atomicAdd(&released[s], 1);
      if (done == (it / NST + 1) * nwarps - 1) {  // the last warp of this use of the stage
        __threadfence_block();
        // stages are released in tile order, so the next tile to stage is
        // the active one after the last issued
        const int kn = next_k(last_k + 1);
        if (kn < nk) {
          last_k = kn;
          fence_async_smem();  // the stage was last read through generic loads
          issue(t0 + kn * G, s);
        }
      }
    }
  }
  __syncthreads();
  if (abort_flag && threadIdx.x == 0) {
    // a staged tile never completed: record it, drain the copies still in
    // flight and flag the solve broken down
    atomicOr(status, kStatusWaitTimeout);
    drain();
    if (SEG) {
      sc->done = 2;
      sc->fail = 5;
    } else {
      sc[0].done = sc[1].done = 2;
      sc[0].fail = sc[1].fail = 5;
    }
  }
  if (SEG) return;
  Acc<T> vv[1] = {v};
  P bt[1];
  block_total_acc<T, 1>(vv, bt);
  if (threadIdx.x == 0) cta_part[blockIdx.x] = bt[0];
}

#define TG_CG_PRODUCT_PARAMS                                                                                  \
  int ntiles, const long long *__restrict__ blob_off, const unsigned char *__restrict__ blob, int cap, int keep, \
      const typename Vec4<T>::type *__restrict__ p, typename Vec4<T>::type *__restrict__ q,                  \
      typename Vec4<T>::type *__restrict__ push, typename Partial<T>::type *__restrict__ cta_part,            \
      double *__restrict__ node_dot, PcgScalars *sc, int *status, const uint8_t *__restrict__ tile_act
#define TG_CG_PRODUCT_ARGS ntiles, blob_off, blob, cap, keep, p, q, push, cta_part, node_dot, sc, status, tile_act

template <typename T, int NST>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 2) pcg_cg_spmv_kernel(TG_CG_PRODUCT_PARAMS) {
  cg_product<T, NST, false, false>(TG_CG_PRODUCT_ARGS);
}

template <typename T, int NST>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 2) pcg_cg_push_kernel(TG_CG_PRODUCT_PARAMS) {
  cg_product<T, NST, true, false>(TG_CG_PRODUCT_ARGS);
}

// the segmented batch's product on the push storage
template <typename T, int NST>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 2) pcg_seg_push_kernel(TG_CG_PRODUCT_PARAMS) {
  cg_product<T, NST, true, true>(TG_CG_PRODUCT_ARGS);
}
#undef TG_CG_PRODUCT_PARAMS
#undef TG_CG_PRODUCT_ARGS

// The preconditioner block of one node: the 3x3 (block-)Jacobi inverse, or
// with DIAG (Jacobi) its diagonal from the compact 4-vector per node.
template <typename T, bool DIAG>
struct PrecBlock {
  T b[DIAG ? 3 : 9];
  __device__ __forceinline__ void load(const T* __restrict__ minv, int n) {
    if constexpr (DIAG) {
      const typename Vec4<T>::type d = reinterpret_cast<const typename Vec4<T>::type*>(minv)[n];
      b[0] = d.x;
      b[1] = d.y;
      b[2] = d.z;
    } else {
#pragma unroll
      for (int m = 0; m < 9; ++m) b[m] = minv[(long long)n * 9 + m];
    }
  }
  __device__ __forceinline__ void apply(T rx, T ry, T rz, T& zx, T& zy, T& zz) const {
    if constexpr (DIAG) {
      zx = b[0] * rx;
      zy = b[1] * ry;
      zz = b[2] * rz;
    } else {
      zx = b[0] * rx + b[1] * ry + b[2] * rz;
      zy = b[3] * rx + b[4] * ry + b[5] * rz;
      zz = b[6] * rx + b[7] * ry + b[8] * rz;
    }
  }
};

// One CTA per SM, one node per thread per pass: 1024 (FP32, 64 registers)
// or 512 (FP64) nodes in flight per SM cover the L2 latency of the vector
// pass (its vectors stay L2-resident), and one CTA per SM keeps the partials
// every CTA sums at the start few (one per SM).
template <typename T>
struct CgShape {
  static constexpr int threads = sizeof(T) == 4 ? 1024 : 512;
};

//
// With the symmetric push storage (PUSH) the product's w holds the upper
// part of A u only: a node's w is completed here from its push slots, added
// in slot order, with the dofs of prescribed rows left out (the stored upper
// blocks keep their prescribed columns, whose transposes would reach them).
//
// DIAG: Jacobi, minv the compact diagonal (minv_diag_offset); otherwise the
// node's 3x3 block.
template <typename T, bool PUSH, bool DIAG>
__global__ void __launch_bounds__(CgShape<T>::threads, 1) pcg_cg_vector_kernel(
    int nnd, const T* __restrict__ minv, typename Vec4<T>::type* __restrict__ x,
    typename Vec4<T>::type* __restrict__ r, typename Vec4<T>::type* __restrict__ u,
    typename Vec4<T>::type* __restrict__ p, typename Vec4<T>::type* __restrict__ s,
    const typename Vec4<T>::type* __restrict__ w, const typename Partial<T>::type* __restrict__ dpart, int ndp,
    double* vpart, PcgScalars* sc, const typename Vec4<T>::type* __restrict__ push, const int* __restrict__ lptr,
    const uint8_t* __restrict__ mask, int pstride) {
  using V = typename Vec4<T>::type;
  using P = typename Partial<T>::type;
  // w of node n: the product's value, plus the pushed lower part
  // Node n's pushes are rank planes of pstride slots, read coalesced and in
  // rank order.  Read, a plane line is dead until the next product writes it:
  // once all eight nodes of a 128-byte line have their values (the warp
  // converges first), the first of them discards the line, so the L2 never
  // writes dead pushes back to DRAM.  Called by whole warps (n < nnd or not).
  auto w_of = [&](int n) {
    V wv = mk<V, T>(T(0), T(0), T(0));
    if (n < nnd) wv = w[n];
    if (PUSH) {
      const uint64_t keep = l2_policy_evict_last();
      T s0 = T(0), s1 = T(0), s2 = T(0);
      const int cnt = n < nnd ? lptr[n + 1] - lptr[n] : 0;
#pragma unroll 4
      for (int k = 0; k < cnt; ++k) {
        const V pv = ld_hint(push + ((long long)k * pstride + n), keep);
        s0 += pv.x;
        s1 += pv.y;
        s2 += pv.z;
      }
      if (n < nnd) {
        const uint8_t m = mask[n];
        wv = mk<V, T>(wv.x + ((m & 1) ? s0 : T(0)), wv.y + ((m & 2) ? s1 : T(0)), wv.z + ((m & 4) ? s2 : T(0)));
      }
      if (kPushDiscard) {
        // the line's largest rank count, over its eight nodes (one warp)
        int lc = cnt;
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) lc = max(lc, __shfl_xor_sync(0xffffffffu, lc, o));
        __syncwarp();
        constexpr int kLine = 128 / (int)sizeof(V);  // slots per line
        if ((n % kLine) == 0)
          for (int k = 0; k < lc; ++k) l2_discard(push + ((long long)k * pstride + n));
      }
    }
    return wv;
  };
  __shared__ double coef[2];  // alpha, beta
  __shared__ int go;
  // the first pass's node vectors: the product this kernel waits for writes
  // none of them, and the vector kernel before it has completed (the product
  // released this kernel only after its own wait for it)
  const int n0 = blockIdx.x * blockDim.x + threadIdx.x;
  V u0, p0, s0, x0, r0;
  PrecBlock<T, DIAG> B0;
  if (n0 < nnd) {
    u0 = u[n0];
    p0 = p[n0];
    s0 = s[n0];
    x0 = x[n0];
    r0 = r[n0];
    B0.load(minv, n0);
  }
  griddep_wait();  // w, the CTA partials and the scalars of the product
  griddep_launch();
  // one round trip for everything the scalars need: the state (read by one
  // thread -- every warp of the grid loading the same line would queue at
  // one L2 slice; scalars[0] is not written while this kernel runs, so every
  // CTA reads the same), w, the product's partials and both buffers of the
  // last vector kernel's partials (which one is the last depends on the
  // iteration)
  __shared__ PcgScalars so;  // kept in shared memory: registers stay free for the vector pass
  if (threadIdx.x == 0) so = *sc;
  V w0;
  w0 = w_of(n0);  // in flight while the scalars are formed
  const int nb = gridDim.x;  // at most one partial of each buffer per thread
  P g0{}, g1{}, q0{}, q1{};
  if ((int)threadIdx.x < nb) {
    g0 = reinterpret_cast<const P*>(vpart)[threadIdx.x];
    q0 = reinterpret_cast<const P*>(vpart)[kVecCap + threadIdx.x];
    g1 = reinterpret_cast<const P*>(vpart)[2 * kVecCap + threadIdx.x];
    q1 = reinterpret_cast<const P*>(vpart)[3 * kVecCap + threadIdx.x];
  }
  Acc<T> a[3];
  for (int b = threadIdx.x; b < ndp; b += blockDim.x) acc_merge(a[0], dpart[b]);
  __syncthreads();
  if (so.done) return;
  const int it = so.iters;  // updates done so far
  P* next = reinterpret_cast<P*>(vpart + (size_t)((it + 1) & 1) * 2 * kVecCap);
  {
    // totals of the product's u.w and the last vector kernel's r.u, r.r:
    // thread-strided sums in a fixed order, then the fixed block tree, in
    // the accumulator's arithmetic (compensated FP32 in the FP32 form)
    if (it > 0 && (int)threadIdx.x < nb) {
      acc_merge(a[1], (it & 1) ? g1 : g0);
      acc_merge(a[2], (it & 1) ? q1 : q0);
    }
    P tot[3];
    block_total_acc<T, 3>(a, tot);
    if (threadIdx.x == 0) {
      PcgScalars o = so;
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
        // alpha = gamma / (delta - beta gamma / alpha_old) with beta =
        // gamma / gamma_old, as gamma t / (delta t - gamma^2), t = gamma_old
        // alpha_old: one division on the dependent chain (FP64 division is
        // long on GB300), beta's beside it
        double num = gamma, den = delta;
        if (it > 0) {
          const double t = o.rz * o.alpha;  // o.rz, o.alpha: the last update's gamma and alpha
          beta = gamma / o.rz;
          num = gamma * t;
          den = delta * t - gamma * gamma;
        }
        if (!(den > 0.0) || !isfinite(den)) {
          done = 2;
          fail = isfinite(den) ? 2 : 3;
        } else {
          alpha = num / den;
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
  auto update = [&](int n, const V& un, const V& wn, const V& pn, const V& sn, const V& xn, const V& rn,
                    const PrecBlock<T, DIAG>& B) {
    V pv, sv;
    if (first) {  // p = u, s = w (p and s hold nothing yet)
      pv = un;
      sv = wn;
    } else {
      pv = mk<V, T>(un.x + b_ * pn.x, un.y + b_ * pn.y, un.z + b_ * pn.z);
      sv = mk<V, T>(wn.x + b_ * sn.x, wn.y + b_ * sn.y, wn.z + b_ * sn.z);
    }
    const T rx = rn.x - a_ * sv.x, ry = rn.y - a_ * sv.y, rz = rn.z - a_ * sv.z;
    T zx, zy, zz;
    B.apply(rx, ry, rz, zx, zy, zz);
    p[n] = pv;
    s[n] = sv;
    x[n] = mk<V, T>(xn.x + a_ * pv.x, xn.y + a_ * pv.y, xn.z + a_ * pv.z);
    r[n] = mk<V, T>(rx, ry, rz);
    u[n] = mk<V, T>(zx, zy, zz);
    acc[0].add_prod(rx, zx);
    acc[0].add_prod(ry, zy);
    acc[0].add_prod(rz, zz);
    acc[1].add_prod(rx, rx);
    acc[1].add_prod(ry, ry);
    acc[1].add_prod(rz, rz);
  };
  const int step = gridDim.x * blockDim.x;  // a multiple of 32: warps stay whole
  if (n0 < nnd) update(n0, u0, w0, p0, s0, x0, r0, B0);
  for (int n = n0 + step; n - (int)(threadIdx.x & 31) < nnd; n += step) {
    const V wn = w_of(n);
    if (n < nnd) {
      const V un = u[n], pn = p[n], sn = s[n], xn = x[n], rn = r[n];
      PrecBlock<T, DIAG> B;
      B.load(minv, n);
      update(n, un, wn, pn, sn, xn, rn, B);
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
template <typename T, bool PUSH, bool DIAG>
int vec_grid(Context* c, int* grid) {
  int per_sm = 0;
  if (!ok(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pcg_cg_vector_kernel<T, PUSH, DIAG>,
                                                           CgShape<T>::threads, 0),
          "occupancy"))
    return TG_ERR_CUDA;
  const int per = CgShape<T>::threads;
  // at most one CTA per thread of a CTA: each thread loads at most one of
  // the previous vector kernel's partials of each kind
  *grid = std::max(1, std::min({(c->nnd + per - 1) / per, c->num_sms * std::max(per_sm, 1), kVecCap, per}));
  return TG_OK;
}

// The matrix storage the product streams: the full-storage tiles, or the
// symmetric push storage (tg_pcg_form 3) with its push buffer and slot
// pointers; the push storage's values are brought up to the last assembly.
template <typename T>
struct CgStore {
  bool push = false;
  int ntiles = 0;
  long long cap = 0;
  const std::vector<long long>* h_off = nullptr;
  const long long* off = nullptr;
  const unsigned char* blob = nullptr;
  typename Vec4<T>::type* pushbuf = nullptr;
  const int* lptr = nullptr;
  int pstride = 0;
};

template <typename T>
int cg_store(Context* c, CgStore<T>& st) {
  const bool f32 = std::is_same<T, float>::value;
  st.push = push_active(c);
  if (!st.push) {
    const int sf = ensure_full_assembly(c);
    if (sf) return sf;
    st.ntiles = c->ntiles;
    st.cap = f32 ? c->blob_cap32 : c->blob_cap64;
    st.h_off = f32 ? &c->h_blob_off32 : &c->h_blob_off64;
    st.off = f32 ? c->d_blob_off32 : c->d_blob_off64;
    st.blob = f32 ? c->d_blob32 : c->d_blob64;
    return TG_OK;
  }
  const int s = push_prepare(c, f32 ? TG_MIXED : TG_FP64);
  if (s) return s;
  const PushStore& ps = c->push;
  st.ntiles = ps.ntiles;
  st.cap = f32 ? ps.cap32 : ps.cap64;
  st.h_off = f32 ? &ps.h_off32 : &ps.h_off64;
  st.off = f32 ? ps.d_off32 : ps.d_off64;
  st.blob = f32 ? ps.d_blob32 : ps.d_blob64;
  st.pushbuf = reinterpret_cast<typename Vec4<T>::type*>(f32 ? ps.d_push32 : ps.d_push64);
  st.lptr = ps.d_lptr;
  st.pstride = ps.pstride;
  return TG_OK;
}

// Launch shape of the product: a ring of the context's stages (2 or 3, 2 if
// 3 do not fit) over the largest tile, as many CTAs as are resident.
struct CgProduct {
  int grid = 0, nst = 2, cap = 0, keep = -1;
  size_t smem = 0;
  void* fn = nullptr;
};

template <typename T>
int product_shape(Context* c, const CgStore<T>& st, CgProduct& pr, bool seg = false) {
  pr.cap = (int)((st.cap + 127) / 128 * 128);
  int optin = 0;
  if (!ok(c, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device), "attribute"))
    return TG_ERR_CUDA;
  pr.nst = c->spmv_stages == 3 && 3 * (size_t)pr.cap + 1024 <= (size_t)optin ? 3 : 2;
  if (seg)
    pr.fn = pr.nst == 3 ? reinterpret_cast<void*>(pcg_seg_push_kernel<T, 3>)
                        : reinterpret_cast<void*>(pcg_seg_push_kernel<T, 2>);
  else if (st.push)
    pr.fn = pr.nst == 3 ? reinterpret_cast<void*>(pcg_cg_push_kernel<T, 3>)
                        : reinterpret_cast<void*>(pcg_cg_push_kernel<T, 2>);
  else
    pr.fn = pr.nst == 3 ? reinterpret_cast<void*>(pcg_cg_spmv_kernel<T, 3>)
                        : reinterpret_cast<void*>(pcg_cg_spmv_kernel<T, 2>);
  pr.smem = (size_t)pr.nst * pr.cap;
  cudaFuncAttributes fa;
  if (!ok(c, cudaFuncGetAttributes(&fa, pr.fn), "function attributes")) return TG_ERR_CUDA;
  if (pr.smem + fa.sharedSizeBytes + 1024 > (size_t)optin) {
    c->err = "single-reduction PCG: tile ring does not fit in shared memory";
    return TG_ERR_CAPACITY;
  }
  // one value for every caller: other contexts may configure and launch it
  if (!ok(c, cudaFuncSetAttribute(pr.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes),
          "smem attribute"))
    return TG_ERR_CUDA;
  int per_sm = 0;
  if (!ok(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pr.fn, 256, pr.smem), "occupancy"))
    return TG_ERR_CUDA;
  if (per_sm < 1) {
    c->err = "single-reduction PCG: product tile does not fit";
    return TG_ERR_CAPACITY;
  }
  pr.grid = std::max(1, std::min({st.ntiles, c->num_sms * per_sm, kCtaCap}));
  pr.keep = -1;
  if (c->l2_keep >= 0) {
    const std::vector<long long>& off = *st.h_off;
    int t = 0;
    while (t < st.ntiles && off[t + 1] <= c->l2_keep) ++t;
    pr.keep = t;
  }
  return TG_OK;
}

// the two kernels' arguments for one storage
template <typename T>
struct CgArgs {
  using V = typename Vec4<T>::type;
  using P = typename Partial<T>::type;
  int ntiles, cap, keep, nnd, ndp;
  const long long* off;
  const unsigned char* blob;
  const V* pu;
  V* qw;
  V* pushw;
  const V* pushr;
  P* cta_part;
  const P* dpart;
  PcgScalars* sc;
  int* status;
  const T* mv;
  V *x, *r, *u, *p, *sv;
  const V* w;
  double* vpart;
  const int* lptr;
  const uint8_t* mask;
  int pstride;
  double* node_dot = nullptr;
  const uint8_t* tile_act = nullptr;
  void* pargs[13];
  void* vargs[16];
  const void* vfn;
  CgArgs(Context* c, const CgStore<T>& st, const CgProduct& pr, const T* minv, bool diag) {
    ntiles = st.ntiles;
    cap = pr.cap;
    keep = pr.keep;
    nnd = c->nnd;
    ndp = pr.grid;
    off = st.off;
    blob = st.blob;
    pu = (const V*)c->d_z;
    qw = (V*)c->d_q;
    pushw = st.pushbuf;
    pushr = st.pushbuf;
    cta_part = reinterpret_cast<P*>(c->d_partials + kCgPartials);
    dpart = cta_part;
    sc = c->d_pcg;
    status = c->d_status;
    mv = minv;
    x = (V*)c->d_x;
    r = (V*)c->d_r;
    u = (V*)c->d_z;
    p = (V*)c->d_p;
    sv = (V*)c->d_cg_s;
    w = (const V*)c->d_q;
    vpart = c->d_partials;
    lptr = st.lptr;
    mask = c->d_mask;
    pstride = st.pstride;
    void* pa[] = {&ntiles, &off, &blob, &cap, &keep, &pu, &qw, &pushw, &cta_part, &node_dot, &sc, &status, &tile_act};
    void* va[] = {&nnd, &mv, &x, &r, &u, &p, &sv, &w, &dpart, &ndp, &vpart, &sc, &pushr, &lptr, &mask, &pstride};
    std::memcpy(pargs, pa, sizeof(pa));
    std::memcpy(vargs, va, sizeof(va));
    vfn = st.push ? (diag ? reinterpret_cast<const void*>(pcg_cg_vector_kernel<T, true, true>)
                          : reinterpret_cast<const void*>(pcg_cg_vector_kernel<T, true, false>))
                  : (diag ? reinterpret_cast<const void*>(pcg_cg_vector_kernel<T, false, true>)
                          : reinterpret_cast<const void*>(pcg_cg_vector_kernel<T, false, false>));
  }
  CgArgs(const CgArgs&) = delete;
};

// minv: the vector kernel's preconditioner (the compact diagonal with diag)
template <typename T>
int capture(Context* c, int precision, const T* minv, bool diag) {
  CgStore<T> st;
  int s = cg_store<T>(c, st);
  if (s) return s;
  CgProduct pr;
  s = product_shape<T>(c, st, pr);
  if (s) return s;
  int nv = 0;
  s = st.push ? (diag ? vec_grid<T, true, true>(c, &nv) : vec_grid<T, true, false>(c, &nv))
              : (diag ? vec_grid<T, false, true>(c, &nv) : vec_grid<T, false, false>(c, &nv));
  if (s) return s;
  CgArgs<T> A(c, st, pr, minv, diag);
  // every launch after the first of the chunk depends programmatically on
  // the one before it
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t pc = {};
  pc.gridDim = dim3(pr.grid);
  pc.blockDim = dim3(256);
  pc.dynamicSmemBytes = pr.smem;
  pc.stream = c->stream;
  cudaLaunchConfig_t vc = {};
  vc.gridDim = dim3(nv);
  vc.blockDim = dim3(CgShape<T>::threads);
  vc.dynamicSmemBytes = 0;
  vc.stream = c->stream;
  vc.attrs = at;
  vc.numAttrs = c->cg_pdl ? 1 : 0;
  cudaGraph_t graph;
  if (!ok(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture")) return TG_ERR_CUDA;
  cudaError_t le = cudaSuccess;
  for (int k = 0; k < kCgChunk && le == cudaSuccess; ++k) {
    pc.attrs = at;
    pc.numAttrs = (k > 0 && c->cg_pdl) ? 1 : 0;
    le = cudaLaunchKernelExC(&pc, pr.fn, A.pargs);
    if (le != cudaSuccess) break;
    le = cudaLaunchKernelExC(&vc, A.vfn, A.vargs);
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
  static_assert(kCgPartials + kCtaCap <= 8192, "partials buffer");
  if (c->partials_cap * 2 < kCgPartials + kCtaCap) {
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
  if (push_active(c)) {
    // the push storage's values follow the last assembly (a no-op when
    // they already do; the captured graph reads the same buffers)
    s = push_prepare(c, precision);
    if (s) return s;
  }
  const int key = precision * 4 + (precond == TG_PRECOND_BLOCK_JACOBI ? 1 : 0) + (push_active(c) ? 2 : 0);
  if (!c->cg_graph || c->cg_graph_key != key) {
    // Jacobi: the vector kernel reads the compact diagonal
    const bool diag = precond != TG_PRECOND_BLOCK_JACOBI;
    s = capture<T>(c, precision, diag ? minv_base + minv_diag_offset(c->nnd) : minv, diag);
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

// Average device time of standalone launches of one kernel of the form
// (which 0: product, 1: vector kernel) on the current tangent, each launch
// doing the same work: the solve's vectors and scalars are set up from R as
// for a solve, the product's partials come from one product launch, and the
// scalars are reset to the first iteration before every vector launch.
template <typename T>
int time_cg_t(Context* c, int precision, int which, int reps, double* ms) {
  using V = typename Vec4<T>::type;
  using P = typename Partial<T>::type;
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
  // Jacobi, as the solves the bench times (the vector kernel on the compact
  // diagonal)
  const T* minv = std::is_same<T, float>::value ? (const T*)c->d_minv32 : (const T*)c->d_minv64;
  s = pcg_start(c, precision, c->d_R, minv, 1e-30, 1 << 30);
  if (s) return s;
  const T* vminv = minv + minv_diag_offset(c->nnd);
  const bool diag = true;
  PcgScalars h;
  if (!ok(c, cudaMemcpyAsync(&h, c->d_pcg, sizeof(PcgScalars), cudaMemcpyDeviceToHost, c->stream), "scalars") ||
      !ok(c, cudaStreamSynchronize(c->stream), "sync"))
    return TG_ERR_CUDA;
  h.done = 0;
  h.iters = 0;
  CgStore<T> st;
  s = cg_store<T>(c, st);
  if (s) return s;
  CgProduct pr;
  s = product_shape<T>(c, st, pr);
  if (s) return s;
  int nv = 0;
  s = st.push ? (diag ? vec_grid<T, true, true>(c, &nv) : vec_grid<T, true, false>(c, &nv))
              : (diag ? vec_grid<T, false, true>(c, &nv) : vec_grid<T, false, false>(c, &nv));
  if (s) return s;
  CgArgs<T> A(c, st, pr, vminv, diag);
  void** pargs = A.pargs;
  void** vargs = A.vargs;
  const void* vfn = A.vfn;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  double total = 0.0;
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < reps + 1 && e == cudaSuccess; ++k) {
    // both scalar states at the first iteration (the product hands [1] to [0])
    cudaMemcpyAsync(c->d_pcg, &h, sizeof(h), cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(c->d_pcg + 1, &h, sizeof(h), cudaMemcpyHostToDevice, c->stream);
    // each vector launch follows an untimed product launch, as in the solve:
    // the product's partials, and on the push storage its pushed products,
    // are then where the vector kernel finds them in the PCG (the L2)
    if (which == 1) {
      e = cudaLaunchKernel(pr.fn, dim3(pr.grid), dim3(256), pargs, pr.smem, c->stream);
      c->launches++;
      if (k == 0 || e != cudaSuccess) continue;
    }
    cudaEventRecord(a, c->stream);
    e = which == 0 ? cudaLaunchKernel(pr.fn, dim3(pr.grid), dim3(256), pargs, pr.smem, c->stream)
                   : cudaLaunchKernel(vfn, dim3(nv), dim3(CgShape<T>::threads), vargs, 0, c->stream);
    cudaEventRecord(b, c->stream);
    c->launches++;
    cudaEventSynchronize(b);
    float t = 0.f;
    cudaEventElapsedTime(&t, a, b);
    if (which == 1 || k > 0) total += t;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = total / reps;
  if (!ok(c, e, "time_cg_kernel")) return TG_ERR_CUDA;
  return ok(c, cudaGetLastError(), "time_cg_kernel") ? TG_OK : TG_ERR_CUDA;
}

}  // namespace

int time_cg_kernel(Context* c, int which, int reps, double* ms) {
  if (c->tangent_precision == TG_MIXED) return time_cg_t<float>(c, TG_MIXED, which, reps, ms);
  if (c->tangent_precision == TG_FP64) return time_cg_t<double>(c, TG_FP64, which, reps, ms);
  c->err = "form the tangent first";
  return TG_ERR_ARG;
}

void cg_free(Context* c) {
  if (c->cg_graph) cudaGraphExecDestroy(c->cg_graph);
  c->cg_graph = nullptr;
  c->cg_graph_key = -1;
}

namespace {
template <typename T>
int seg_push_t(Context* c, const void* z, void* w, double* node_dot, PcgScalars* gate, const uint8_t* tile_act) {
  using V = typename Vec4<T>::type;
  CgStore<T> st;
  int s = cg_store<T>(c, st);
  if (s) return s;
  if (!st.push) {
    c->err = "segmented push product without the push storage";
    return TG_ERR_ARG;
  }
  CgProduct pr;
  s = product_shape<T>(c, st, pr, true);
  if (s) return s;
  int ntiles = st.ntiles, cap = pr.cap, keep = pr.keep;
  const long long* off = st.off;
  const unsigned char* blob = st.blob;
  const V* p = (const V*)z;
  V* q = (V*)w;
  V* push = st.pushbuf;
  typename Partial<T>::type* cta_part = nullptr;
  int* status = c->d_status;
  void* args[] = {&ntiles, &off, &blob, &cap, &keep, &p, &q, &push, &cta_part, &node_dot, &gate, &status, &tile_act};
  const cudaError_t e = cudaLaunchKernel(pr.fn, dim3(pr.grid), dim3(256), args, pr.smem, c->stream);
  c->launches++;
  return ok(c, e, "pcg_seg_push_kernel") ? TG_OK : TG_ERR_CUDA;
}
}  // namespace

// Average device time of standalone launches of the segmented batch's push
// product on the current tangent (a zero gate, a scratch node_dot).
int time_seg_push(Context* c, int reps, double* ms) {
  const int precision = c->tangent_precision;
  if (precision != TG_MIXED && precision != TG_FP64) {
    c->err = "form the tangent first";
    return TG_ERR_ARG;
  }
  int s = pcg_vectors(c, precision);
  if (!s) s = push_prepare(c, precision);
  if (s) return s;
  double* nd = nullptr;
  if (!dalloc(c, &nd, (size_t)c->nnd)) return TG_ERR_OOM;
  if (!ok(c, cudaMemsetAsync(c->d_pcg, 0, sizeof(PcgScalars), c->stream), "gate")) {
    dfree(c, nd);
    return TG_ERR_CUDA;
  }
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  double total = 0.0;
  for (int k = 0; k < reps + 1 && !s; ++k) {
    cudaEventRecord(a, c->stream);
    s = launch_seg_push(c, precision, c->d_z, c->d_q, nd, c->d_pcg);
    cudaEventRecord(b, c->stream);
    cudaEventSynchronize(b);
    float t = 0.f;
    cudaEventElapsedTime(&t, a, b);
    if (k > 0) total += t;  // the first launch also sets the shapes up
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  dfree(c, nd);
  *ms = total / reps;
  return s;
}

int launch_seg_push(Context* c, int precision, const void* z, void* w, double* node_dot, PcgScalars* gate,
                    const uint8_t* tile_act) {
  if (precision == TG_MIXED) return seg_push_t<float>(c, z, w, node_dot, gate, tile_act);
  return seg_push_t<double>(c, z, w, node_dot, gate, tile_act);
}

int pcg_solve_cg(Context* c, int precision, const double4_32a* d_rhs, double rel_tol, int max_it, int precond,
                 int* iters, double* rel_res) {
  if (precision == TG_MIXED) return solve_cg_t<float>(c, precision, d_rhs, rel_tol, max_it, precond, iters, rel_res);
  return solve_cg_t<double>(c, precision, d_rhs, rel_tol, max_it, precond, iters, rel_res);
}

}  // namespace tg
