// Multi-right-hand-side PCG: NR independent (block-)Jacobi CG iterations on
// the same matrix that share one streamed pass over it per iteration.
//
// The nine static-condensation solves of the RVE macro tangent have the same
// operator K_ii and different right-hand sides.  Solved one after another,
// each iteration streams the whole tile-contiguous matrix from HBM for one
// product; here every staged tile is applied to NR search directions at once,
// so the matrix traffic per iteration is that of one product and the extra
// cost is the NR-fold vector traffic (mostly L2-resident gathers).  Each
// right-hand side keeps its own scaling, alpha, beta and convergence flag; a
// converged one is frozen (alpha = beta = 0) while the others continue.
//
// Vector layout: the right-hand sides are taken in groups of three; group g
// stores node n's three padded 4-vectors contiguously at (g*nnd + n)*3, so a
// gather of one neighbour for one group is one 48-byte run and a thread
// updating (node, group) reads contiguous memory.  The product runs one pass
// per group over each staged tile (the tile stays in shared memory), which
// keeps a lane's accumulators to three 3-vectors.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <type_traits>

#include "krylov_common.cuh"

namespace tg {

namespace {

constexpr int kNR = 9;
constexpr int kGS = 3;            // right-hand sides per group
constexpr int kNG = kNR / kGS;    // groups
constexpr int kPollEvery = 16;  // iterations between host polls of the flag

__host__ __device__ __forceinline__ long long vidx(int nnd, int n, int k) {
  return ((long long)(k / kGS) * nnd + n) * kGS + (k % kGS);
}

// Last-CTA reduction over a grid whose rows (blockIdx.y) are groups: CTA
// (bx, g) contributes NV values of group g; the last CTA to finish gets, on
// thread 0, tot[g*NV + j] for every group in a fixed order.
template <typename T, int NV, int NGR>
__device__ __forceinline__ bool last_block_total_groups(Acc<T> (&v)[NV], double* partials, unsigned int* counter,
                                                        double (&tot)[NGR * NV]) {
  __shared__ bool last;
  double bt[NV];
  block_total<T, NV>(v, bt);
  const int gx = gridDim.x;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) partials[((long long)blockIdx.y * NV + j) * gx + blockIdx.x] = bt[j];
    __threadfence();
    last = atomicAdd(counter, 1u) == gx * gridDim.y - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  for (int g = 0; g < NGR; ++g) {
    Acc<double> acc[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j)
      for (int b = threadIdx.x; b < gx; b += blockDim.x)
        acc[j].add(((volatile double*)partials)[((long long)g * NV + j) * gx + b]);
    double t[NV];
    block_total<double, NV>(acc, t);
    if (threadIdx.x == 0)
#pragma unroll
      for (int j = 0; j < NV; ++j) tot[g * NV + j] = t[j];
  }
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

template <int NR>
struct MScalars {
  double rz[NR], rr[NR], rr0[NR], alpha[NR], beta[NR], pq[NR], scale[NR], unscale[NR];
  double tol2;
  int active[NR];
  int done;  // 1 all converged, 2 breakdown / non-finite, 3 iteration limit
  int iters, max_it, fail;
  unsigned count_a, count_b;
  unsigned bar_count;  // arrivals at the update's grid barrier (reset per solve)
};

template <typename T, int NR>
__global__ void __launch_bounds__(256) mrhs_scale_kernel(int nnd, const double4_32a* __restrict__ rhs,
                                                         const uint8_t* __restrict__ mask, const T* __restrict__ minv,
                                                         double* partials, MScalars<NR>* sc) {
  Acc<double> v[NR];
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nnd; n += gridDim.x * blockDim.x) {
    const uint8_t m = mask[n];
    const T* B = minv + (long long)n * 9;
    double Bd[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) Bd[i] = (double)B[i];
#pragma unroll
    for (int k = 0; k < NR; ++k) {
      const double4_32a b = rhs[(long long)k * nnd + n];
      const double bx = (m & 1) ? b.x : 0.0, by = (m & 2) ? b.y : 0.0, bz = (m & 4) ? b.z : 0.0;
      const double zx = Bd[0] * bx + Bd[1] * by + Bd[2] * bz;
      const double zy = Bd[3] * bx + Bd[4] * by + Bd[5] * bz;
      const double zz = Bd[6] * bx + Bd[7] * by + Bd[8] * bz;
      v[k].add(bx * zx + by * zy + bz * zz);
    }
  }
  double tot[NR];
  if (last_block_total<double, NR>(v, partials, &sc->count_a, tot) && threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NR; ++k) {
      const double s = (tot[k] > 0.0 && isfinite(tot[k])) ? 1.0 / sqrt(tot[k]) : 1.0;
      sc->scale[k] = s;
      sc->unscale[k] = 1.0 / s;
    }
}

template <typename T, int NR>
__global__ void __launch_bounds__(256) mrhs_init_kernel(int nnd, const double4_32a* __restrict__ rhs,
                                                        const uint8_t* __restrict__ mask, const T* __restrict__ minv,
                                                        typename Vec4<T>::type* x, typename Vec4<T>::type* r,
                                                        typename Vec4<T>::type* z, typename Vec4<T>::type* p,
                                                        typename Vec4<T>::type* q, double* partials,
                                                        MScalars<NR>* sc, double tol, int max_it) {
  using V = typename Vec4<T>::type;
  const int g = blockIdx.y;
  Acc<T> v[2 * kGS];  // r.z then r.r of the group's right-hand sides
  double scale[kGS];
#pragma unroll
  for (int j = 0; j < kGS; ++j) scale[j] = sc->scale[g * kGS + j];
  const V zero = mk<V, T>(T(0), T(0), T(0));
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nnd; n += gridDim.x * blockDim.x) {
    const uint8_t m = mask[n];
#pragma unroll
    for (int j = 0; j < kGS; ++j) {
      const int k = g * kGS + j;
      const double4_32a b = rhs[(long long)k * nnd + n];
      const T rx = (m & 1) ? T(b.x * scale[j]) : T(0), ry = (m & 2) ? T(b.y * scale[j]) : T(0),
              rz = (m & 4) ? T(b.z * scale[j]) : T(0);
      T zx, zy, zz;
      apply_minv<T>(minv, n, rx, ry, rz, zx, zy, zz);
      const long long i = vidx(nnd, n, k);
      x[i] = zero;
      r[i] = mk<V, T>(rx, ry, rz);
      z[i] = mk<V, T>(zx, zy, zz);
      p[i] = mk<V, T>(zx, zy, zz);  // first direction p = z
      q[i] = zero;
      v[j].add_prod(rx, zx);
      v[j].add_prod(ry, zy);
      v[j].add_prod(rz, zz);
      v[kGS + j].add_prod(rx, rx);
      v[kGS + j].add_prod(ry, ry);
      v[kGS + j].add_prod(rz, rz);
    }
  }
  double tot[kNG * 2 * kGS];
  if (last_block_total_groups<T, 2 * kGS, kNG>(v, partials, &sc->count_b, tot) && threadIdx.x == 0) {
    int any = 0, bad = 0;
    for (int k = 0; k < NR; ++k) {
      const double rzk = tot[(k / kGS) * 2 * kGS + (k % kGS)], rrk = tot[(k / kGS) * 2 * kGS + kGS + (k % kGS)];
      sc->rz[k] = rzk;
      sc->rr[k] = rrk;
      sc->rr0[k] = rrk;
      sc->alpha[k] = 0.0;
      sc->beta[k] = 0.0;
      const bool fin = isfinite(rzk) && isfinite(rrk);
      bad |= !fin;
      sc->active[k] = (fin && rrk > 0.0) ? 1 : 0;
      any |= sc->active[k];
    }
    sc->tol2 = tol * tol;
    sc->max_it = max_it;
    sc->iters = 0;
    sc->count_a = 0u;
    sc->bar_count = 0u;
    sc->fail = bad ? 1 : 0;
    sc->done = bad ? 2 : (any ? 0 : 1);
  }
}

// q_k = A p_k for all k; the same tile ring as the single-vector product.
// Each lane takes its row's blocks two at a time with both neighbours'
// gathers in flight before the arithmetic.
template <typename T, int NST, int NR>
__global__ void __launch_bounds__(256) mrhs_spmv_kernel(int nnd, int ntiles, const long long* __restrict__ blob_off,
                                                        const unsigned char* __restrict__ blob, int cap,
                                                        const typename Vec4<T>::type* __restrict__ p,
                                                        typename Vec4<T>::type* __restrict__ q, double* partials,
                                                        MScalars<NR>* sc, int* status) {
  using V = typename Vec4<T>::type;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bars[NST];
  __shared__ int abort_flag;
  if (((volatile MScalars<NR>*)sc)->done) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NST; ++k) mbar_init(&bars[k], 1);
    fence_mbar_init();
    abort_flag = 0;
  }
  __syncthreads();
  Acc<T> v[NR];
  const int t0 = blockIdx.x, G = gridDim.x;
  auto issue = [&](int t, int stage) {
    const long long o0 = blob_off[t], o1 = blob_off[t + 1];
    const unsigned bytes = (unsigned)(o1 - o0);
    mbar_expect_tx(&bars[stage], bytes);
    bulk_copy(smem + (size_t)stage * cap, blob + o0, bytes, &bars[stage]);
  };
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NST - 1; ++k)
      if (t0 + k * G < ntiles) issue(t0 + k * G, k);
  unsigned phases = 0u;
  int stuck = -1;
  int it = 0;
  const int sub = lane & 7;
  for (int t = t0; t < ntiles; ++it, t += G) {
    const int s = it % NST;
    const int tn = t + (NST - 1) * G;
    if (threadIdx.x == 0 && tn < ntiles) {
      fence_async_smem();
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
    const unsigned char* base = smem + (size_t)s * cap;
    const int* hdr = reinterpret_cast<const int*>(base);
    const int r0 = hdr[0], nrows = hdr[1], nb = hdr[2], ps = hdr[3];
    const int* rp = hdr + 4;
    const int* cl = rp + ceil4(nrows + 1);
    const T* pl = reinterpret_cast<const T*>(cl + ceil4(nb));
#pragma unroll
    for (int g = 0; g < kNG; ++g) {
      for (int li = warp * 4 + (lane >> 3); li - (lane >> 3) < nrows; li += nwarps * 4) {
        const bool live = li < nrows;
        const int I = r0 + li;
        T a[kGS][3];
#pragma unroll
        for (int jj = 0; jj < kGS; ++jj) a[jj][0] = a[jj][1] = a[jj][2] = T(0);
        const int e0 = live ? rp[li] : 0;
        const int e1 = live ? rp[li + 1] : 0;
        for (int j = e0 + sub; j < e1; j += 16) {
          const int jb = j + 8;
          const bool two = jb < e1;
          const long long oa = vidx(nnd, cl[j], g * kGS);
          const long long ob = two ? vidx(nnd, cl[jb], g * kGS) : oa;
          V pa[kGS], pb[kGS];
#pragma unroll
          for (int jj = 0; jj < kGS; ++jj) {
            pa[jj] = p[oa + jj];
            pb[jj] = p[ob + jj];
          }
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            if (h == 1 && !two) break;
            const T* vv = pl + (h == 0 ? j : jb);
            T mv[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) mv[i] = vv[i * ps];
#pragma unroll
            for (int jj = 0; jj < kGS; ++jj) {
              const V pp = h == 0 ? pa[jj] : pb[jj];
              a[jj][0] += mv[0] * pp.x + mv[1] * pp.y + mv[2] * pp.z;
              a[jj][1] += mv[3] * pp.x + mv[4] * pp.y + mv[5] * pp.z;
              a[jj][2] += mv[6] * pp.x + mv[7] * pp.y + mv[8] * pp.z;
            }
          }
        }
#pragma unroll
        for (int jj = 0; jj < kGS; ++jj)
#pragma unroll
          for (int o = 4; o > 0; o >>= 1) {
            a[jj][0] += __shfl_xor_sync(0xffffffffu, a[jj][0], o);
            a[jj][1] += __shfl_xor_sync(0xffffffffu, a[jj][1], o);
            a[jj][2] += __shfl_xor_sync(0xffffffffu, a[jj][2], o);
          }
        if (live) {
          // lane jj of the row writes right-hand side g*3 + jj
#pragma unroll
          for (int jj = 0; jj < kGS; ++jj)
            if (jj == sub) {
              const long long i = vidx(nnd, I, g * kGS + jj);
              const V pi = p[i];
              q[i] = mk<V, T>(a[jj][0], a[jj][1], a[jj][2]);
              v[g * kGS + jj].add_prod(pi.x, a[jj][0]);
              v[g * kGS + jj].add_prod(pi.y, a[jj][1]);
              v[g * kGS + jj].add_prod(pi.z, a[jj][2]);
            }
        }
      }
    }
    __syncthreads();
  }
  if (stuck >= 0 && threadIdx.x == 0) {
    atomicOr(status, kStatusWaitTimeout);
    for (int k = 0; k < NST; ++k) {
      const unsigned parity = ((phases >> k) & 1u) ^ (k == stuck ? 1u : 0u);
      mbar_wait(&bars[k], parity, kWaitLimit);
    }
    sc->done = 2;
    sc->fail = 5;
  }
  double tot[NR];
  if (last_block_total<T, NR>(v, partials, &sc->count_a, tot) && threadIdx.x == 0) {
    if (sc->done == 2) return;
    for (int k = 0; k < NR; ++k) {
      sc->pq[k] = tot[k];
      if (!sc->active[k]) {
        sc->alpha[k] = 0.0;
      } else if (!(tot[k] > 0.0) || !isfinite(tot[k])) {
        sc->done = 2;
        sc->fail = isfinite(tot[k]) ? 2 : 3;
      } else {
        sc->alpha[k] = sc->rz[k] / tot[k];
      }
    }
  }
}

// Totals of group g's 2*kGS partial sums (r.z of its right-hand sides, then
// r.r) over the gx CTAs of its grid row: one warp, lane-strided sums and a
// fixed shuffle tree, so every CTA that forms them gets the same bits.
// Valid on lane 0.
__device__ __forceinline__ void group_totals(const double* partials, int gx, int g, double (&tot)[2 * kGS]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < 2 * kGS; ++j) {
    double s = 0.0;
    for (int b = lane; b < gx; b += 32) s += ((volatile const double*)partials)[((long long)g * 2 * kGS + j) * gx + b];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    tot[j] = s;
  }
}

// x_k += alpha_k p_k, r_k -= alpha_k q_k, z_k = M^-1 r_k; then, after a
// bounded grid barrier (cooperative launch: every CTA resident), p_k = z_k +
// beta_k p_k in place, every CTA forming its group's beta from the partials in
// the same order.  A right-hand side that is converged (or converges now) gets
// beta = 0 and, in the next product, alpha = 0: it stays frozen.
template <typename T, int NR>
__global__ void __launch_bounds__(256) mrhs_update_kernel(int nnd, const T* __restrict__ minv,
                                                          typename Vec4<T>::type* __restrict__ x,
                                                          typename Vec4<T>::type* __restrict__ r,
                                                          typename Vec4<T>::type* __restrict__ z,
                                                          typename Vec4<T>::type* __restrict__ p,
                                                          const typename Vec4<T>::type* __restrict__ q,
                                                          double* partials, MScalars<NR>* sc, int* status) {
  using V = typename Vec4<T>::type;
  __shared__ double sbeta[kGS];
  if (((volatile MScalars<NR>*)sc)->done) return;
  const int g = blockIdx.y;
  const int gx = gridDim.x;
  T alpha[kGS];
  double rz_old[kGS];
  int active[kGS];
#pragma unroll
  for (int j = 0; j < kGS; ++j) {
    alpha[j] = T(sc->alpha[g * kGS + j]);
    rz_old[j] = sc->rz[g * kGS + j];  // read before the barrier: CTA (0,0) replaces them after
    active[j] = sc->active[g * kGS + j];
  }
  const double tol2 = sc->tol2;
  Acc<T> v[2 * kGS];
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nnd; n += gx * blockDim.x) {
    const long long i0 = vidx(nnd, n, g * kGS);
#pragma unroll
    for (int j = 0; j < kGS; ++j) {
      const long long i = i0 + j;
      const V pn = p[i], qn = q[i];
      V xn = x[i], rn = r[i];
      xn.x += alpha[j] * pn.x;
      xn.y += alpha[j] * pn.y;
      xn.z += alpha[j] * pn.z;
      rn.x -= alpha[j] * qn.x;
      rn.y -= alpha[j] * qn.y;
      rn.z -= alpha[j] * qn.z;
      T zx, zy, zz;
      apply_minv<T>(minv, n, rn.x, rn.y, rn.z, zx, zy, zz);
      x[i] = xn;
      r[i] = rn;
      z[i] = mk<V, T>(zx, zy, zz);
      v[j].add_prod(rn.x, zx);
      v[j].add_prod(rn.y, zy);
      v[j].add_prod(rn.z, zz);
      v[kGS + j].add_prod(rn.x, rn.x);
      v[kGS + j].add_prod(rn.y, rn.y);
      v[kGS + j].add_prod(rn.z, rn.z);
    }
  }
  {
    double bt[2 * kGS];
    block_total<T, 2 * kGS>(v, bt);
    if (threadIdx.x == 0)
#pragma unroll
      for (int j = 0; j < 2 * kGS; ++j) partials[((long long)g * 2 * kGS + j) * gx + blockIdx.x] = bt[j];
  }
  if (!grid_barrier(&sc->bar_count, kBarrierLimit)) {
    if (threadIdx.x == 0) {
      atomicOr(status, kStatusWaitTimeout);
      sc->fail = 5;
      atomicExch(&sc->done, 2);
    }
    return;
  }
  if (threadIdx.x < 32) {
    double tot[2 * kGS];
    group_totals(partials, gx, g, tot);
    if (threadIdx.x == 0)
#pragma unroll
      for (int j = 0; j < kGS; ++j) {
        const double rzk = tot[j], rrk = tot[kGS + j];
        double beta = 0.0;
        if (active[j] && isfinite(rzk) && isfinite(rrk) && !(rrk <= tol2 * sc->rr0[g * kGS + j]))
          beta = rzk / rz_old[j];
        sbeta[j] = beta;
      }
  }
  __syncthreads();
  T beta[kGS];
#pragma unroll
  for (int j = 0; j < kGS; ++j) beta[j] = T(sbeta[j]);
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nnd; n += gx * blockDim.x) {
    const long long i0 = vidx(nnd, n, g * kGS);
#pragma unroll
    for (int j = 0; j < kGS; ++j) {
      const V zn = z[i0 + j], pn = p[i0 + j];
      p[i0 + j] = mk<V, T>(zn.x + beta[j] * pn.x, zn.y + beta[j] * pn.y, zn.z + beta[j] * pn.z);
    }
  }
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x < 32) {
    // the scalars of every right-hand side, from the same totals
    double tot[kNG][2 * kGS];
#pragma unroll
    for (int gg = 0; gg < kNG; ++gg) group_totals(partials, gx, gg, tot[gg]);
    if (threadIdx.x == 0) {
      const int it = sc->iters + 1;
      sc->iters = it;
      int any = 0, bad = 0;
      for (int k = 0; k < NR; ++k) {
        if (!sc->active[k]) {
          sc->beta[k] = 0.0;
          continue;
        }
        const double rzk = tot[k / kGS][k % kGS], rrk = tot[k / kGS][kGS + (k % kGS)];
        if (!isfinite(rzk) || !isfinite(rrk)) {
          bad = 1;
          continue;
        }
        sc->beta[k] = rzk / sc->rz[k];
        sc->rz[k] = rzk;
        sc->rr[k] = rrk;
        if (rrk <= sc->tol2 * sc->rr0[k]) {
          sc->active[k] = 0;
          sc->beta[k] = 0.0;
        }
        any |= sc->active[k];
      }
      int done = 0;
      if (bad) {
        sc->fail = 4;
        done = 2;
      } else if (!any) {
        done = 1;
      } else if (it >= sc->max_it) {
        done = 3;
      }
      if (done) atomicCAS(&sc->done, 0, done);  // a barrier failure elsewhere keeps its flag
    }
  }
}

// w_k = v_k + unscale_k * x_k, nodal (k-major output)
template <typename V, int NR>
__global__ void mrhs_combine_kernel(int nnd, const double4_32a* __restrict__ v, const V* __restrict__ x,
                                    const MScalars<NR>* __restrict__ sc, double4_32a* __restrict__ w) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnd) return;
#pragma unroll
  for (int k = 0; k < NR; ++k) {
    const double us = sc->unscale[k];
    const double4_32a a = v[(long long)k * nnd + n];
    const V b = x[vidx(nnd, n, k)];
    w[(long long)k * nnd + n] =
        make_double4_32a(a.x + us * (double)b.x, a.y + us * (double)b.y, a.z + us * (double)b.z, 0.0);
  }
}

template <typename T, int NST>
int mrhs_config(Context* c, size_t smem, int* grid) {
  int optin = 0;
  if (!ok(c, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device), "attribute"))
    return TG_ERR_CUDA;
  if (smem + 1024 > (size_t)optin) {
    c->err = "multi-vector SpMV tile ring does not fit in shared memory";
    return TG_ERR_CAPACITY;
  }
  // the attribute belongs to the function and other contexts may launch it
  // from other threads: always the device's largest dynamic size (one value
  // for every caller), not this mesh's ring
  cudaFuncAttributes fa;
  if (!ok(c, cudaFuncGetAttributes(&fa, mrhs_spmv_kernel<T, NST, kNR>), "function attributes") ||
      !ok(c, cudaFuncSetAttribute(mrhs_spmv_kernel<T, NST, kNR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  optin - (int)fa.sharedSizeBytes),
          "smem attribute"))
    return TG_ERR_CUDA;
  int per_sm = 0;
  if (!ok(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mrhs_spmv_kernel<T, NST, kNR>, 256, smem),
          "occupancy"))
    return TG_ERR_CUDA;
  if (per_sm < 1) {
    c->err = "multi-vector SpMV does not fit on an SM";
    return TG_ERR_CAPACITY;
  }
  *grid = std::max(1, std::min(c->ntiles, c->num_sms * per_sm));
  return TG_OK;
}

// Solves K X = B for kNR right-hand sides (B: kNR nodal vectors, k-major,
// active rows), then writes W = V + X (V: kNR nodal vectors) into d_w.
template <typename T>
int mrhs_solve_t(Context* c, const double4_32a* d_b, const double4_32a* d_v, double4_32a* d_w, double rel_tol,
                 int max_it, int precond, int* iters, double* worst_rel) {
  using V = typename Vec4<T>::type;
  using S = MScalars<kNR>;
  const bool f32 = std::is_same<T, float>::value;
  const T* minv_base = f32 ? (const T*)c->d_minv32 : (const T*)c->d_minv64;
  const T* minv = minv_base + (precond == TG_PRECOND_BLOCK_JACOBI ? (long long)c->nnd * 9 : 0);
  const int cap = (int)(((f32 ? c->blob_cap32 : c->blob_cap64) + 127) / 128 * 128);
  const long long* off = f32 ? c->d_blob_off32 : c->d_blob_off64;
  const unsigned char* blob = f32 ? c->d_blob32 : c->d_blob64;
  int grid = 0;
  const size_t smem = 2 * (size_t)cap;
  int s = mrhs_config<T, 2>(c, smem, &grid);
  if (s) return s;
  const int vgrid = std::min((c->nnd + 255) / 256, c->num_sms * 2);            // scale pass (1-D)
  // the update is a cooperative launch: its kNG grid rows together fit at once
  int upd_per_sm = 0;
  if (!ok(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&upd_per_sm, mrhs_update_kernel<T, kNR>, 256, 0),
          "occupancy"))
    return TG_ERR_CUDA;
  const int ugrid = std::max(1, std::min((c->nnd + 255) / 256, c->num_sms * upd_per_sm / kNG));  // per group row
  const size_t npart = (size_t)std::max({(long long)grid * kNR, (long long)vgrid * kNR, (long long)ugrid * kNR * 2});
  const size_t nv = (size_t)c->nnd * kNR;
  V *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr;
  S* sc = nullptr;
  double* part = nullptr;
  cudaStream_t st = c->stream;
  bool good = ok(c, cudaMallocAsync((void**)&part, sizeof(double) * npart, st), "alloc");
  for (V** pp : {&x, &r, &z, &p, &q}) good = good && ok(c, cudaMallocAsync((void**)pp, sizeof(V) * nv, st), "alloc");
  good = good && ok(c, cudaMallocAsync((void**)&sc, sizeof(S), st), "alloc");
  if (!good) return TG_ERR_OOM;
  good = ok(c, cudaMemsetAsync(sc, 0, sizeof(S), st), "memset");
  if (good) {
    mrhs_scale_kernel<T, kNR><<<vgrid, 256, 0, st>>>(c->nnd, d_b, c->d_mask, minv, part, sc);
    mrhs_init_kernel<T, kNR><<<dim3(ugrid, kNG), 256, 0, st>>>(c->nnd, d_b, c->d_mask, minv, x, r, z, p, q, part, sc,
                                                              rel_tol, max_it);
    c->launches += 2;
    good = ok(c, cudaGetLastError(), "mrhs init");
  }
  S h;
  std::memset(&h, 0, sizeof(h));
  for (int k = 0; good && k * kPollEvery <= max_it + 2 * kPollEvery; ++k) {
    for (int j = 0; j < kPollEvery && good; ++j) {
      mrhs_spmv_kernel<T, 2, kNR><<<grid, 256, smem, st>>>(c->nnd, c->ntiles, off, blob, cap, p, q, part, sc,
                                                           c->d_status);
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(ugrid, kNG);
      cfg.blockDim = dim3(256);
      cfg.stream = st;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeCooperative;
      at[0].val.cooperative = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      good = ok(c, cudaLaunchKernelEx(&cfg, mrhs_update_kernel<T, kNR>, c->nnd, minv, x, r, z, p, (const V*)q, part,
                                      sc, c->d_status),
                "mrhs update");
    }
    c->launches += 2 * kPollEvery;
    good = ok(c, cudaGetLastError(), "mrhs iterate") &&
           ok(c, cudaMemcpyAsync(&h, sc, sizeof(S), cudaMemcpyDeviceToHost, st), "scalars") &&
           ok(c, cudaStreamSynchronize(st), "mrhs sync");
    if (good && h.done) break;
  }
  if (good) {
    mrhs_combine_kernel<V, kNR><<<(c->nnd + 255) / 256, 256, 0, st>>>(c->nnd, d_v, x, sc, d_w);
    c->launches++;
    good = ok(c, cudaGetLastError(), "mrhs combine");
  }
  for (void* ptr : {(void*)x, (void*)r, (void*)z, (void*)p, (void*)q, (void*)sc, (void*)part})
    if (ptr) cudaFreeAsync(ptr, st);
  if (!ok(c, cudaStreamSynchronize(st), "sync") || !good) return TG_ERR_CUDA;
  if (iters) *iters = h.iters;
  double worst = 0.0;
  for (int k = 0; k < kNR; ++k)
    if (h.rr0[k] > 0) worst = std::max(worst, std::sqrt(h.rr[k] / h.rr0[k]));
  if (worst_rel) *worst_rel = worst;
  if (h.done == 2) {
    static const char* why[] = {"", "non-finite initial residual", "p.Ap <= 0 (indefinite operator)",
                                "p.Ap not finite", "non-finite update",
                                "staged tile copy or grid barrier wait timed out"};
    c->err = std::string("multi-vector PCG breakdown: ") + why[(h.fail >= 0 && h.fail <= 5) ? h.fail : 0];
    return TG_ERR_NAN;
  }
  return h.done == 1 ? TG_OK : TG_ERR_NOT_CONVERGED;
}

}  // namespace

// Macro tangent of every segment with the nine condensation solves done as
// one multi-vector PCG.  The tangent (of the requested precision) must be
// formed at the current state.
int macro_tangent_mrhs(Context* c, int precision, int precond, double rel_tol, int max_it, const double* d_vol,
                       double* d_C, int* iters) {
  {
    // the multi-vector product streams the full storage
    const int sf = ensure_full_assembly(c);
    if (sf) return sf;
  }
  const size_t nb = sizeof(double4_32a) * c->nnd * kNR;
  double4_32a *d_v = nullptr, *d_b = nullptr;
  if (!ok(c, cudaMallocAsync((void**)&d_v, nb, c->stream), "alloc") ||
      !ok(c, cudaMallocAsync((void**)&d_b, nb, c->stream), "alloc"))
    return TG_ERR_OOM;
  int s = TG_OK;
  // boundary perturbations v_kL = (e_k (x) e_L) X and right-hand sides -K v
  for (int kL = 0; kL < kNR && !s; ++kL) s = launch_macro_perturb(c, kL / 3, kL % 3, d_v + (size_t)kL * c->nnd);
  if (!s) s = launch_lift_rhs(c, d_v, d_b, true, kNR);
  double worst = 0.0;
  if (!s) {
    s = precision == TG_MIXED ? mrhs_solve_t<float>(c, d_b, d_v, d_b, rel_tol, max_it, precond, iters, &worst)
                              : mrhs_solve_t<double>(c, d_b, d_v, d_b, rel_tol, max_it, precond, iters, &worst);
    if (s == TG_ERR_NOT_CONVERGED) s = TG_OK;
  }
  // d_b now holds the total displacement perturbations w_kL
  if (!s) s = launch_segment_macro(c, d_b, 0, kNR, d_vol, d_C);
  cudaFreeAsync(d_v, c->stream);
  cudaFreeAsync(d_b, c->stream);
  return s;
}

}  // namespace tg
