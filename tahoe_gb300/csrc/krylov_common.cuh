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
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

constexpr int kWaitLimit = 1 << 18;  // polls before a staged tile is declared lost

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
