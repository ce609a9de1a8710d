// Per-RVE (segmented) reductions for batched FE^2 micro-solves.
//
// A batch of independent RVEs is uploaded as one disconnected mesh; RVE r owns
// nodes [node_off[r], node_off[r+1]) and elements [elem_off[r], elem_off[r+1]).
// One CTA per RVE reduces over its range in a fixed order (no atomics):
//  * segment_norms_kernel: ||R_r||^2 of the residual restricted to the RVE;
//  * segment_stress_kernel: sum over the RVE's element nodes of fint (x) X,
//    which is the integral of the first Piola stress over the RVE (the
//    element-level identity sum_a f_a (x) X_a = int P dV), i.e. V0 times the
//    volume-averaged P; at equilibrium it equals the reaction sum
//    sum_{boundary a} f_a (x) X_a of the macro-stress definition.
#include "tg_internal.h"

namespace tg {

namespace {

template <int NV>
__device__ __forceinline__ void cta_sum(double (&v)[NV]) {
  __shared__ double sh[NV][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[k][w] = v[k];
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double x = lane < nw ? sh[k][lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
      v[k] = x;
    }
  }
  __syncthreads();
}

__global__ void __launch_bounds__(256) segment_norms_kernel(int nseg, const int* __restrict__ off,
                                                            const double4_32a* __restrict__ R, double* __restrict__ out) {
  for (int sg = blockIdx.x; sg < nseg; sg += gridDim.x) {
    double v[1] = {0.0};
    for (int n = off[sg] + threadIdx.x; n < off[sg + 1]; n += blockDim.x) {
      const double4_32a r = R[n];
      v[0] += r.x * r.x + r.y * r.y + r.z * r.z;
    }
    cta_sum<1>(v);
    if (threadIdx.x == 0) out[sg] = v[0];
  }
}

__global__ void __launch_bounds__(256) segment_stress_kernel(int nseg, const int* __restrict__ eoff,
                                                             const int* __restrict__ conn, const double* __restrict__ X,
                                                             int nnd, const double4_32a* __restrict__ fint,
                                                             double* __restrict__ out) {
  for (int sg = blockIdx.x; sg < nseg; sg += gridDim.x) {
    double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const long long k0 = (long long)eoff[sg] * 8, k1 = (long long)eoff[sg + 1] * 8;
    for (long long k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
      const int n = conn[k];
      const double4_32a f = fint[k];
      const double Xn[3] = {X[n], X[nnd + n], X[2 * nnd + n]};
#pragma unroll
      for (int J = 0; J < 3; ++J) {
        v[0 * 3 + J] += f.x * Xn[J];
        v[1 * 3 + J] += f.y * Xn[J];
        v[2 * 3 + J] += f.z * Xn[J];
      }
    }
    cta_sum<9>(v);
    if (threadIdx.x == 0)
#pragma unroll
      for (int k = 0; k < 9; ++k) out[(long long)sg * 9 + k] = v[k];
  }
}

}  // namespace

int launch_segment_norms(Context* c, int nseg, const int* d_node_off, double* d_out) {
  segment_norms_kernel<<<std::min(nseg, kNumSMs * 16), 256, 0, c->stream>>>(nseg, d_node_off, c->d_R, d_out);
  c->launches++;
  return ok(c, cudaGetLastError(), "segment_norms_kernel") ? TG_OK : TG_ERR_CUDA;
}

int launch_segment_stress(Context* c, int nseg, const int* d_elem_off, double* d_out) {
  segment_stress_kernel<<<std::min(nseg, kNumSMs * 16), 256, 0, c->stream>>>(nseg, d_elem_off, c->d_conn, c->d_X,
                                                                              c->nnd, c->d_fint, d_out);
  c->launches++;
  return ok(c, cudaGetLastError(), "segment_stress_kernel") ? TG_OK : TG_ERR_CUDA;
}

}  // namespace tg
