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

// v = (e_k (x) e_L) X on prescribed dofs, zero elsewhere: the boundary
// displacement of a unit perturbation dF = e_k (x) e_L of the macro gradient.
__global__ void macro_perturb_kernel(int nnd, const uint8_t* __restrict__ mask, const double* __restrict__ X, int k,
                                     int L, double4_32a* __restrict__ v) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnd) return;
  const int m = mask[n];
  const double xl = X[(long long)L * nnd + n];
  v[n] = make_double4_32a((k == 0 && !(m & 1)) ? xl : 0.0, (k == 1 && !(m & 2)) ? xl : 0.0,
                          (k == 2 && !(m & 4)) ? xl : 0.0, 0.0);
}

// w = v + unscale * x (x: the PCG solution on the free dofs, zero elsewhere)
template <typename V>
__global__ void macro_combine_kernel(int nnd, const double4_32a* __restrict__ v, const V* __restrict__ x,
                                     const PcgScalars* __restrict__ sc, double4_32a* __restrict__ w) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnd) return;
  const double us = sc->unscale;
  const double4_32a a = v[n];
  const V b = x[n];
  w[n] = make_double4_32a(a.x + us * (double)b.x, a.y + us * (double)b.y, a.z + us * (double)b.z, 0.0);
}

__device__ __forceinline__ int upper_slot_of(int a, int b) { return a * 8 - a * (a - 1) / 2 + (b - a); }

// Column kL of every RVE's macro tangent: sum over the RVE's element nodes of
// (K_e w_e)_a (x) X_a, from the staged element matrices (36 upper node-pair
// blocks; lower blocks by symmetry).  Written to out[seg*81 + jJ*9 + kL].
template <typename T>
__global__ void __launch_bounds__(256) segment_macro_kernel(int nseg, const int* __restrict__ eoff,
                                                            const int* __restrict__ conn, const double* __restrict__ X,
                                                            int nnd, const T* __restrict__ Ke,
                                                            const double4_32a* __restrict__ w_all, int kL0,
                                                            const double* __restrict__ vol0, double* __restrict__ out) {
  // grid rows (blockIdx.y) are the columns kL0 + y, each with its own w
  const int kL = kL0 + blockIdx.y;
  const double4_32a* __restrict__ w = w_all + (long long)blockIdx.y * nnd;
  for (int sg = blockIdx.x; sg < nseg; sg += gridDim.x) {
    double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const long long k0 = (long long)eoff[sg] * 8, k1 = (long long)eoff[sg + 1] * 8;
    for (long long k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
      const long long e = k >> 3;
      const int a = (int)(k & 7);
      const int* ce = conn + e * 8;
      const T* Kb = Ke + e * kKeStride;
      double y0 = 0.0, y1 = 0.0, y2 = 0.0;
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        const double4_32a wb = w[ce[b]];
        if (a <= b) {
          const T* B = Kb + upper_slot_of(a, b) * kKeBlock;
          y0 += (double)B[0] * wb.x + (double)B[1] * wb.y + (double)B[2] * wb.z;
          y1 += (double)B[4] * wb.x + (double)B[5] * wb.y + (double)B[6] * wb.z;
          y2 += (double)B[8] * wb.x + (double)B[9] * wb.y + (double)B[10] * wb.z;
        } else {
          const T* B = Kb + upper_slot_of(b, a) * kKeBlock;
          y0 += (double)B[0] * wb.x + (double)B[4] * wb.y + (double)B[8] * wb.z;
          y1 += (double)B[1] * wb.x + (double)B[5] * wb.y + (double)B[9] * wb.z;
          y2 += (double)B[2] * wb.x + (double)B[6] * wb.y + (double)B[10] * wb.z;
        }
      }
      const int n = ce[a];
      const double Xn[3] = {X[n], X[nnd + n], X[2 * nnd + n]};
#pragma unroll
      for (int J = 0; J < 3; ++J) {
        v[0 * 3 + J] += y0 * Xn[J];
        v[1 * 3 + J] += y1 * Xn[J];
        v[2 * 3 + J] += y2 * Xn[J];
      }
    }
    cta_sum<9>(v);
    if (threadIdx.x == 0) {
      const double s = vol0 ? 1.0 / vol0[sg] : 1.0;
#pragma unroll
      for (int jJ = 0; jJ < 9; ++jJ) out[(long long)sg * 81 + jJ * 9 + kL] = v[jJ] * s;
    }
  }
}

}  // namespace

int launch_macro_perturb(Context* c, int k, int L, double4_32a* d_v) {
  macro_perturb_kernel<<<(c->nnd + 255) / 256, 256, 0, c->stream>>>(c->nnd, c->d_mask, c->d_X, k, L, d_v);
  c->launches++;
  return ok(c, cudaGetLastError(), "macro_perturb_kernel") ? TG_OK : TG_ERR_CUDA;
}

int launch_macro_combine(Context* c, const double4_32a* d_v, double4_32a* d_w) {
  const int grid = (c->nnd + 255) / 256;
  if (c->pcg_vec_precision == TG_MIXED)
    macro_combine_kernel<float4><<<grid, 256, 0, c->stream>>>(c->nnd, d_v, (const float4*)c->d_x, c->d_pcg, d_w);
  else
    macro_combine_kernel<double4_32a><<<grid, 256, 0, c->stream>>>(c->nnd, d_v, (const double4_32a*)c->d_x, c->d_pcg,
                                                                    d_w);
  c->launches++;
  return ok(c, cudaGetLastError(), "macro_combine_kernel") ? TG_OK : TG_ERR_CUDA;
}

int launch_segment_macro(Context* c, const double4_32a* d_w, int kL, int ncols, const double* d_vol0,
                         double* d_out) {
  const dim3 grid(std::min(c->nseg, c->num_sms * 16), ncols);
  if (c->tangent_precision == TG_MIXED)
    segment_macro_kernel<float><<<grid, 256, 0, c->stream>>>(c->nseg, c->d_seg_elem, c->d_conn, c->d_X, c->nnd,
                                                             c->d_Ke32, d_w, kL, d_vol0, d_out);
  else
    segment_macro_kernel<double><<<grid, 256, 0, c->stream>>>(c->nseg, c->d_seg_elem, c->d_conn, c->d_X, c->nnd,
                                                              c->d_Ke64, d_w, kL, d_vol0, d_out);
  c->launches++;
  return ok(c, cudaGetLastError(), "segment_macro_kernel") ? TG_OK : TG_ERR_CUDA;
}

int launch_segment_norms(Context* c, int nseg, const int* d_node_off, double* d_out) {
  segment_norms_kernel<<<std::min(nseg, c->num_sms * 16), 256, 0, c->stream>>>(nseg, d_node_off, c->d_R, d_out);
  c->launches++;
  return ok(c, cudaGetLastError(), "segment_norms_kernel") ? TG_OK : TG_ERR_CUDA;
}

int launch_segment_stress(Context* c, int nseg, const int* d_elem_off, double* d_out) {
  segment_stress_kernel<<<std::min(nseg, c->num_sms * 16), 256, 0, c->stream>>>(nseg, d_elem_off, c->d_conn, c->d_X,
                                                                              c->nnd, c->d_fint, d_out);
  c->launches++;
  return ok(c, cudaGetLastError(), "segment_stress_kernel") ? TG_OK : TG_ERR_CUDA;
}

}  // namespace tg
