// Device helpers shared by the Krylov translation units: vector types,
// compensated dot-product accumulators, fixed-order block and last-block
// reductions, the preconditioner application and the mbarrier / bulk-copy
// primitives of the streamed matrix.  Internal to the library.
#pragma once

#include "tg_internal.h"

namespace tg {
namespace {

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

// Dot-product accumulators.  GB300 issues an FP64 warp instruction at a
// small fraction of the FP32 rate, so in the FP32 form the per-element
// products are accumulated as compensated FP32 pairs (hi + lo, error-free
// two-product and two-sum, about 48 significant bits) and only the per-block
// totals are converted to FP64 for the cross-block sum.  The FP64 form
// accumulates in FP64 throughout.
template <typename T>
struct Acc;

template <>
struct Acc<float> {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float b) {  // Knuth two-sum, error into lo
    const float s = __fadd_rn(hi, b);
    const float bb = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    hi = s;
    lo = __fadd_rn(lo, e);
  }
  __device__ __forceinline__ void add_prod(float x, float y) {  // exact product p + pe
    const float p = __fmul_rn(x, y);
    const float pe = __fmaf_rn(x, y, -p);
    add(p);
    lo = __fadd_rn(lo, pe);
  }
  __device__ __forceinline__ void merge(float ohi, float olo) {
    add(ohi);
    lo = __fadd_rn(lo, olo);
  }
  __device__ __forceinline__ void shfl_merge(int o) {
    const float ohi = __shfl_xor_sync(0xffffffffu, hi, o);
    const float olo = __shfl_xor_sync(0xffffffffu, lo, o);
    merge(ohi, olo);
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

template <>
struct Acc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double b) { s += b; }
  __device__ __forceinline__ void add_prod(double x, double y) { s = fma(x, y, s); }
  __device__ __forceinline__ void merge(double o, double) { s += o; }
  __device__ __forceinline__ void shfl_merge(int o) { s += __shfl_xor_sync(0xffffffffu, s, o); }
  __device__ __forceinline__ double value() const { return s; }
};

// Block total of NV accumulators (fixed order), FP64 value on thread 0.
template <typename T, int NV>
__device__ __forceinline__ void block_total(Acc<T> (&v)[NV], double (&out)[NV]) {
  __shared__ double sh[NV][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k].shfl_merge(o);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[k][w] = v[k].value();
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double x = lane < nw ? sh[k][lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
      out[k] = x;
    }
  }
  __syncthreads();
}

// CTA partial of a reduction as kept between kernels, in one 8-byte slot: a
// compensated FP32 pair (hi, lo) in the FP32 form -- summed across CTAs with
// error-free FP32 transformations, since GB300 issues FP64 at a small
// fraction of the FP32 rate and every CTA of a kernel may repeat the sum --
// and an FP64 value in the FP64 form.
template <typename T> struct Partial;
template <> struct Partial<float> { using type = float2; };
template <> struct Partial<double> { using type = double; };

__device__ __forceinline__ float2 to_partial(const Acc<float>& a) { return make_float2(a.hi, a.lo); }
__device__ __forceinline__ double to_partial(const Acc<double>& a) { return a.s; }
__device__ __forceinline__ void acc_merge(Acc<float>& a, float2 p) { a.merge(p.x, p.y); }
__device__ __forceinline__ void acc_merge(Acc<double>& a, double p) { a.add(p); }
__device__ __forceinline__ double partial_value(float2 p) { return (double)p.x + (double)p.y; }
__device__ __forceinline__ double partial_value(double p) { return p; }

// Block total of NV accumulators kept in the accumulator's own arithmetic
// (no FP64 in the FP32 form), fixed order, on thread 0.
template <typename T, int NV>
__device__ __forceinline__ void block_total_acc(Acc<T> (&v)[NV], typename Partial<T>::type (&out)[NV]) {
  using P = typename Partial<T>::type;
  __shared__ P shp[NV][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k].shfl_merge(o);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) shp[k][w] = to_partial(v[k]);
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      Acc<T> a;
      if (lane < nw) acc_merge(a, shp[k][lane]);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) a.shfl_merge(o);
      out[k] = to_partial(a);
    }
  }
  __syncthreads();
}

// Last-block reduction of per-block partials (partials[k*gridDim + b]) in
// FP64 and a fixed order; true in the last block, totals on thread 0.
template <typename T, int NV>
__device__ __forceinline__ bool last_block_total(Acc<T> (&v)[NV], double* partials, unsigned int* counter,
                                                 double (&tot)[NV]) {
  __shared__ bool last;
  double bt[NV];
  block_total<T, NV>(v, bt);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) partials[k * gridDim.x + blockIdx.x] = bt[k];
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  Acc<double> acc[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k)
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) acc[k].add(((volatile double*)partials)[k * gridDim.x + b]);
  block_total<double, NV>(acc, tot);
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

// ---- bulk-copy (TMA) staging of the streamed matrix ----------------------
__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ready;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ready)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ready != 0;
}
// Bounded wait: gives up after `limit` polls (the caller records the timeout).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, int limit) {
  for (int i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void bulk_copy(void* dst_smem, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst_smem)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
// L2 eviction priorities of the streamed matrix.  The matrix is larger than
// the L2 and is read once per product, so most of it is streamed with
// evict_first (it never displaces the PCG vectors, which every kernel of an
// iteration reads and writes); a leading part of it may be kept with
// evict_last, so that part is served from the L2 on every later product.
__device__ __forceinline__ uint64_t l2_policy_evict_first() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ uint64_t l2_policy_evict_last() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
// global stores and loads of node vectors with an L2 cache policy
__device__ __forceinline__ void st_hint(float4* p, const float4& v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "f"(v.x), "f"(v.y),
               "f"(v.z), "f"(v.w), "l"(pol)
               : "memory");
}
__device__ __forceinline__ void st_hint(double4_32a* p, const double4_32a& v, uint64_t pol) {
  double* d = reinterpret_cast<double*>(p);
  asm volatile("st.global.L2::cache_hint.v2.f64 [%0], {%1, %2}, %3;" ::"l"(d), "d"(v.x), "d"(v.y), "l"(pol)
               : "memory");
  asm volatile("st.global.L2::cache_hint.v2.f64 [%0], {%1, %2}, %3;" ::"l"(d + 2), "d"(v.z), "d"(v.w), "l"(pol)
               : "memory");
}
__device__ __forceinline__ float4 ld_hint(const float4* p, uint64_t pol) {
  float4 v;
  asm volatile("ld.global.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ double4_32a ld_hint(const double4_32a* p, uint64_t pol) {
  double4_32a v;
  const double* d = reinterpret_cast<const double*>(p);
  asm volatile("ld.global.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;" : "=d"(v.x), "=d"(v.y) : "l"(d), "l"(pol));
  asm volatile("ld.global.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;" : "=d"(v.z), "=d"(v.w) : "l"(d + 2), "l"(pol));
  return v;
}
// drops a 128-byte L2 line without writing it back (its data is dead)
__device__ __forceinline__ void l2_discard(const void* p) {
  asm volatile("discard.global.L2 [%0], 128;" ::"l"(p) : "memory");
}

__device__ __forceinline__ void bulk_copy_hint(void* dst_smem, const void* src, unsigned bytes, uint64_t* bar,
                                               uint64_t pol) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
          smem_addr(dst_smem)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(pol)
      : "memory");
}
// One staged tile: a plain bulk copy (keep < 0), or with the tile's L2
// priority (tiles below `keep` evict_last, the rest evict_first).
__device__ __forceinline__ void stage_tile(void* dst_smem, const void* src, unsigned bytes, uint64_t* bar, int t,
                                           int keep, uint64_t pol_last, uint64_t pol_first) {
  if (keep < 0)
    bulk_copy(dst_smem, src, bytes, bar);
  else
    bulk_copy_hint(dst_smem, src, bytes, bar, t < keep ? pol_last : pol_first);
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

constexpr int kWaitLimit = 1 << 18;  // polls before a staged tile is declared lost

// The rows of one staged tile handled by this warp: 8 lanes per row, 4 rows
// per warp at a time, each lane over every 8th block; q = A p written for the
// rows, p.q accumulated into v.
template <typename T>
__device__ __forceinline__ void spmv_tile_rows(const unsigned char* base, int lane, int warp, int nwarps,
                                               const typename Vec4<T>::type* __restrict__ p,
                                               typename Vec4<T>::type* __restrict__ q, Acc<T>& v0,
                                               double* __restrict__ node_dot) {
  using V = typename Vec4<T>::type;
  const int sub = lane & 7;
  Acc<T>* v = &v0;
  const int* hdr = reinterpret_cast<const int*>(base);
  const int r0 = hdr[0], nrows = hdr[1], nb = hdr[2], ps = hdr[3];
  const int* rp = hdr + 4;
  const int* cl = rp + ceil4(nrows + 1);
  const T* pl = reinterpret_cast<const T*>(cl + ceil4(nb));
  for (int li = warp * 4 + (lane >> 3); li - (lane >> 3) < nrows; li += nwarps * 4) {
    const bool live = li < nrows;
    const int I = r0 + li;
    V pi;
    if (live && sub == 0) pi = p[I];
    T a0 = T(0), a1 = T(0), a2 = T(0);
    const int e0 = live ? rp[li] : 0;
    const int e1 = live ? rp[li + 1] : 0;
    // the first 4 blocks of this lane (32 per row, a hex8 row has at most
    // 27): all column indices, then all neighbour gathers, then the
    // arithmetic, so the L2 round trips of one lane overlap instead of
    // chaining
    {
      int Jk[4];
      V pk[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int j = e0 + sub + 8 * u;
        Jk[u] = j < e1 ? cl[j] : -1;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (Jk[u] >= 0) pk[u] = p[Jk[u]];
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (Jk[u] >= 0) {
          const T* vv = pl + e0 + sub + 8 * u;
          a0 += vv[0 * ps] * pk[u].x + vv[1 * ps] * pk[u].y + vv[2 * ps] * pk[u].z;
          a1 += vv[3 * ps] * pk[u].x + vv[4 * ps] * pk[u].y + vv[5 * ps] * pk[u].z;
          a2 += vv[6 * ps] * pk[u].x + vv[7 * ps] * pk[u].y + vv[8 * ps] * pk[u].z;
        }
    }
    for (int j = e0 + sub + 32; j < e1; j += 8) {
      const V pj = p[cl[j]];
      const T* vv = pl + j;
      a0 += vv[0 * ps] * pj.x + vv[1 * ps] * pj.y + vv[2 * ps] * pj.z;
      a1 += vv[3 * ps] * pj.x + vv[4 * ps] * pj.y + vv[5 * ps] * pj.z;
      a2 += vv[6 * ps] * pj.x + vv[7 * ps] * pj.y + vv[8 * ps] * pj.z;
    }
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, o);
      a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if (live && sub == 0) {
      q[I] = mk<V, T>(a0, a1, a2);
      v[0].add_prod(pi.x, a0);
      v[0].add_prod(pi.y, a1);
      v[0].add_prod(pi.z, a2);
      if (node_dot) {  // the row's own p.q (per-RVE reductions of a segmented batch)
        Acc<T> d;
        d.add_prod(pi.x, a0);
        d.add_prod(pi.y, a1);
        d.add_prod(pi.z, a2);
        node_dot[I] = d.value();
      }
    }
  }
}

// Whether a product launch has nothing to do (the solve is over), decided
// by one thread and the same for every thread of the CTA.  For the
// single-reduction PCG (handoff) block 0 first hands the state the last
// vector kernel wrote (scalars[1]) over to the one the next vector kernel
// reads (scalars[0]); the flag is read from scalars[1], which no kernel
// rewrites while a product runs except on a stage timeout.
__device__ __forceinline__ bool skip_launch(PcgScalars* sc, int handoff) {
  __shared__ int skip;
  if (threadIdx.x == 0) {
    if (handoff && blockIdx.x == 0) sc[0] = sc[1];
    skip = ((volatile PcgScalars*)(handoff ? sc + 1 : sc))->done != 0;
  }
  __syncthreads();
  return skip != 0;
}

// ---- grid-wide barrier of a cooperative launch ---------------------------
constexpr int kBarrierLimit = 1 << 24;  // polls before a grid barrier is declared broken

// Every CTA of a cooperative launch (all resident at once) adds one to a
// counter that only grows (reset to zero when a solve starts, so it stays far
// below 2^32) and polls it until it reaches the end of this launch's group of
// arrivals (one per CTA of the grid).  Bounded: after `limit` polls a CTA stops waiting and the
// call returns false (the caller records the failure); it never spins forever.
__device__ __forceinline__ bool grid_barrier(unsigned int* count, int limit) {
  __shared__ int met;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();  // this CTA's partial sums before its arrival
    const unsigned int nb = gridDim.x * gridDim.y * gridDim.z;
    const unsigned int old = atomicAdd(count, 1u);
    const unsigned int target = (old / nb + 1u) * nb;
    int ok = 1;
    for (int i = 0;; ++i) {
      unsigned int cur;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(count) : "memory");
      if (cur >= target) break;
      if (i >= limit) {
        ok = 0;
        break;
      }
    }
    met = ok;
  }
  __syncthreads();
  return met != 0;
}

}  // namespace
}  // namespace tg
