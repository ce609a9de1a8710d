// Symmetric stream format of the single-vector PCG product, sm_103a.
//
// The assembled tangent is symmetric block by block (block (J,I) is the
// transpose of block (I,J), bitwise: both are sums of the same element
// blocks in the same element order), so the product streams the upper node
// blocks only -- the diagonal block and every block (I,J) with J > I -- and
// forms each lower block (I,J), J < I, as the transpose of its upper twin
// (J,I).  That twin belongs to a row J at most one matrix bandwidth behind
// row I, whose tile the persistent grid streamed moments earlier (or streams
// concurrently), so the transposed read is served from L2 and every matrix
// byte leaves DRAM once.  Per product the DRAM stream shrinks from
// nnzb*(9*s+4) bytes (full storage) to nu*(9*s+4) + nl*8 (nu upper blocks,
// nl = nnzb - nu lower entries of (column, upper block id)): 188 MB instead
// of 297 MB on the 64^3 block in FP32.  The reference stores the upper
// triangle too (MSRMatrixT with a symmetric system, MSRMatrixT.cpp:104-175)
// and applies the lower part by symmetry in MSRMatrixT::Multx
// (MSRMatrixT.cpp:385-420); this is that product, restructured for a
// bandwidth-bound GPU stream.
//
// Storage:
//   values  two arrays indexed by the global upper block id k (row-major over
//           the upper blocks): V8[k] the first eight entries of the row-major
//           3x3 block (32 B FP32 / 64 B FP64, aligned: one or two vector
//           loads) and V1[k] the ninth;
//   tiles   rows grouped so that a tile holds at most tile_blocks upper
//           blocks; tile t's structure is one 16-byte-aligned range: header
//           {first row, rows, first upper id k0, lower entries}, upper and
//           lower local row pointers, upper column indices, lower column
//           indices and the upper block id of every lower entry.
// A tile moves into shared memory with three bulk copies completing on one
// mbarrier (structure, V8[k0..k1), V1 rounded out to 16 bytes); lower blocks
// are read from global memory (L2).  The values are filled after every
// assembly by a conversion pass over the assembled full-storage tiles.
// Rows of prescribed dofs are zero in the full storage but their columns are
// kept, so a transposed upper block carries prescribed-column entries into a
// prescribed row: the product masks its output at prescribed dofs, which
// makes it equal to the full-storage product on every dof.
#include <algorithm>
#include <cstring>
#include <type_traits>

#include "krylov_common.cuh"

namespace tg {

namespace {

struct SymTileView {
  int r0, nrows, k0, nl;
  const int* urp;
  const int* lrp;
  const int* ucol;
  const int* lcol;
  const int* lk;
};

__host__ __device__ inline long long sym_struct_bytes(int nrows, int nu, int nl) {
  return 16 + 4LL * ceil4(nrows + 1) * 2 + 4LL * ceil4(nu) + 8LL * ceil4(nl);
}

__device__ __forceinline__ SymTileView sym_view(const unsigned char* base) {
  SymTileView v;
  const int* h = reinterpret_cast<const int*>(base);
  v.r0 = h[0];
  v.nrows = h[1];
  v.k0 = h[2];
  v.nl = h[3];
  v.urp = h + 4;
  v.lrp = v.urp + ceil4(v.nrows + 1);
  const int nu = v.urp[v.nrows];
  v.ucol = v.lrp + ceil4(v.nrows + 1);
  v.lcol = v.ucol + ceil4(nu);
  v.lk = v.lcol + ceil4(v.nl);
  return v;
}

template <typename T> struct V8T;
template <> struct V8T<float> {
  struct __align__(32) type { float4 a, b; };
};
template <> struct V8T<double> {
  struct __align__(32) type { double4_32a a, b; };
};

// a += A z (upper block, row-major A = [e0..e7, e8]) or a += A^T z (lower)
template <typename T, typename V8, typename V>
__device__ __forceinline__ void block_mul(const V8& m, T e8, const V& z, T& a0, T& a1, T& a2) {
  a0 += m.a.x * z.x + m.a.y * z.y + m.a.z * z.z;
  a1 += m.a.w * z.x + m.b.x * z.y + m.b.y * z.z;
  a2 += m.b.z * z.x + m.b.w * z.y + e8 * z.z;
}
template <typename T, typename V8, typename V>
__device__ __forceinline__ void block_mul_t(const V8& m, T e8, const V& z, T& a0, T& a1, T& a2) {
  a0 += m.a.x * z.x + m.a.w * z.y + m.b.z * z.z;
  a1 += m.a.y * z.x + m.b.x * z.y + m.b.w * z.z;
  a2 += m.a.z * z.x + m.b.y * z.y + e8 * z.z;
}

// The rows of one staged tile handled by this warp: 8 lanes per row, 4 rows
// per warp at a time; each lane takes every 8th upper block (from shared
// memory) and every 8th lower entry (its transposed block from global
// memory), the first two of each with every load issued before any use.
template <typename T>
__device__ __forceinline__ void sym_tile_rows(const unsigned char* sbase, const typename V8T<T>::type* sv8,
                                              const T* sv1, const typename V8T<T>::type* __restrict__ gv8,
                                              const T* __restrict__ gv1, const uint8_t* __restrict__ mask, int lane,
                                              int warp, int nwarps, const typename Vec4<T>::type* __restrict__ p,
                                              typename Vec4<T>::type* __restrict__ q, Acc<T>& dot,
                                              double* __restrict__ node_dot) {
  using V = typename Vec4<T>::type;
  using V8 = typename V8T<T>::type;
  const SymTileView tv = sym_view(sbase);
  const int sub = lane & 7;
  for (int li = warp * 4 + (lane >> 3); li - (lane >> 3) < tv.nrows; li += nwarps * 4) {
    const bool live = li < tv.nrows;
    const int I = tv.r0 + li;
    V pi;
    if (live && sub == 0) pi = p[I];
    T a0 = T(0), a1 = T(0), a2 = T(0);
    const int u0 = live ? tv.urp[li] : 0, u1 = live ? tv.urp[li + 1] : 0;
    const int l0 = live ? tv.lrp[li] : 0, l1 = live ? tv.lrp[li + 1] : 0;
    {
      int Ju[2], Jl[2], kl[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int j = u0 + sub + 8 * u, l = l0 + sub + 8 * u;
        Ju[u] = j < u1 ? tv.ucol[j] : -1;
        Jl[u] = l < l1 ? tv.lcol[l] : -1;
        kl[u] = l < l1 ? tv.lk[l] : 0;
      }
      V pu[2], pl[2];
      V8 ml[2];
      T el[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        if (Ju[u] >= 0) pu[u] = p[Ju[u]];
        if (Jl[u] >= 0) {
          pl[u] = p[Jl[u]];
          ml[u] = gv8[kl[u]];
          el[u] = gv1[kl[u]];
        }
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        if (Ju[u] >= 0) {
          const int j = u0 + sub + 8 * u;
          block_mul<T>(sv8[j], sv1[j], pu[u], a0, a1, a2);
        }
        if (Jl[u] >= 0) block_mul_t<T>(ml[u], el[u], pl[u], a0, a1, a2);
      }
    }
    for (int j = u0 + sub + 16; j < u1; j += 8) block_mul<T>(sv8[j], sv1[j], p[tv.ucol[j]], a0, a1, a2);
    for (int l = l0 + sub + 16; l < l1; l += 8) {
      const int k = tv.lk[l];
      block_mul_t<T>(gv8[k], gv1[k], p[tv.lcol[l]], a0, a1, a2);
    }
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, o);
      a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if (live && sub == 0) {
      const uint8_t m = mask[I];
      if (!(m & 1)) a0 = T(0);
      if (!(m & 2)) a1 = T(0);
      if (!(m & 4)) a2 = T(0);
      q[I] = mk<V, T>(a0, a1, a2);
      dot.add_prod(pi.x, a0);
      dot.add_prod(pi.y, a1);
      dot.add_prod(pi.z, a2);
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

// q = A p on a persistent grid; each CTA streams its tiles through a ring of
// NST shared-memory stages (structure | V8 | V1 per stage), three bulk
// copies per tile on the stage's mbarrier, issued NST-1 tiles ahead.  Every
// wait is bounded; a timeout sets an error flag, drains the copies in flight
// (bounded) and marks the solve broken down.  The last CTA forms p.q and
// alpha exactly as the full-storage product does.
template <typename T, int NST, int MINB>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? MINB : 2) pcg_spmv_sym_kernel(
    int ntiles, const long long* __restrict__ soff, const int* __restrict__ koff,
    const unsigned char* __restrict__ sblob, int cap_s, int cap_v8,
    int cap_v1, const typename V8T<T>::type* __restrict__ gv8, const T* __restrict__ gv1,
    const uint8_t* __restrict__ mask, const typename Vec4<T>::type* __restrict__ p, typename Vec4<T>::type* __restrict__ q,
    double* partials, PcgScalars* sc, int* status, double* node_dot) {
  using V8 = typename V8T<T>::type;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bars[NST];
  __shared__ int abort_flag;
  if (((volatile PcgScalars*)sc)->done) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const size_t stage_bytes = (size_t)cap_s + cap_v8 + cap_v1;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NST; ++k) mbar_init(&bars[k], 1);
    fence_mbar_init();
    abort_flag = 0;
  }
  __syncthreads();
  Acc<T> v[1];
  const int t0 = blockIdx.x, G = gridDim.x;
  constexpr int kV1Align = 16 / (int)sizeof(T);  // V1 entries per 16 bytes
  auto issue = [&](int t, int stage) {
    const long long o0 = soff[t], o1 = soff[t + 1];
    const int k0 = koff[t], nu = koff[t + 1] - k0;  // the tile's upper block ids
    unsigned char* st = smem + (size_t)stage * stage_bytes;
    const int k0r = k0 & ~(kV1Align - 1);
    const int k1r = (k0 + nu + kV1Align - 1) & ~(kV1Align - 1);
    const unsigned bs = (unsigned)(o1 - o0), b8 = (unsigned)(nu * sizeof(V8)), b1 = (unsigned)((k1r - k0r) * sizeof(T));
    mbar_expect_tx(&bars[stage], bs + b8 + b1);
    bulk_copy(st, sblob + o0, bs, &bars[stage]);
    if (b8) bulk_copy(st + cap_s, gv8 + k0, b8, &bars[stage]);
    if (b1) bulk_copy(st + cap_s + cap_v8, gv1 + k0r, b1, &bars[stage]);
  };
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NST - 1; ++k)
      if (t0 + k * G < ntiles) issue(t0 + k * G, k);
  unsigned phases = 0u;
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
    const unsigned char* st = smem + (size_t)s * stage_bytes;
    const int k0 = reinterpret_cast<const int*>(st)[2];
    const V8* sv8 = reinterpret_cast<const V8*>(st + cap_s);
    const T* sv1 = reinterpret_cast<const T*>(st + cap_s + cap_v8) + (k0 & (kV1Align - 1));
    sym_tile_rows<T>(st, sv8, sv1, gv8, gv1, mask, lane, warp, nwarps, p, q, v[0], node_dot);
    __syncthreads();  // stage s is free for the copy issued next iteration
  }
  if (stuck >= 0 && threadIdx.x == 0) {
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

// Fills V8/V1 from the assembled full-storage tiles: one warp per row, the
// row's blocks from its diagonal on (the upper blocks, in column order) read
// from the value planes and written at their upper block ids.
template <typename T>
__global__ void __launch_bounds__(256) sym_convert_kernel(int nnd, const int* __restrict__ rowptr,
                                                          const int* __restrict__ diag_pos,
                                                          const int* __restrict__ urow,
                                                          const unsigned char* __restrict__ blob,
                                                          const long long* __restrict__ blob_off,
                                                          const int* __restrict__ row_tile,
                                                          typename V8T<T>::type* __restrict__ v8, T* __restrict__ v1) {
  using V8 = typename V8T<T>::type;
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; I < nnd; I += warps) {
    const unsigned char* base = blob + blob_off[row_tile[I]];
    const int* hdr = reinterpret_cast<const int*>(base);
    const int trow0 = hdr[0], tnrows = hdr[1], tnb = hdr[2], ps = hdr[3];
    const T* planes = reinterpret_cast<const T*>(base + 16 + 4 * ceil4(tnrows + 1) + 4 * ceil4(tnb));
    const int tb0 = rowptr[trow0];
    const int jd = diag_pos[I], r1 = rowptr[I + 1], k0 = urow[I];
    for (int j = jd + lane; j < r1; j += 32) {
      const T* src = planes + (j - tb0);
      V8 m;
      m.a.x = src[0 * (long long)ps];
      m.a.y = src[1 * (long long)ps];
      m.a.z = src[2 * (long long)ps];
      m.a.w = src[3 * (long long)ps];
      m.b.x = src[4 * (long long)ps];
      m.b.y = src[5 * (long long)ps];
      m.b.z = src[6 * (long long)ps];
      m.b.w = src[7 * (long long)ps];
      const int k = k0 + (j - jd);
      v8[k] = m;
      v1[k] = src[8 * (long long)ps];
    }
  }
}

template <typename T>
int cap_bytes_v8(const SymStore& s) {
  return (int)((size_t)s.cap_blocks * sizeof(typename V8T<T>::type));
}
template <typename T>
int cap_bytes_v1(const SymStore& s) {
  return (int)(((size_t)(s.cap_blocks + 2 * (16 / sizeof(T))) * sizeof(T) + 127) / 128 * 128);
}

}  // namespace

// Host structure of the symmetric format from the node-block CSR: upper row
// pointers, the diagonal's position in every full row, the tiles and their
// structure ranges; uploaded once per mesh (and per tile size).
int sym_build(Context* c, int tile_blocks) {
  if (ensure_host_mesh(c)) return TG_ERR_CUDA;
  SymStore& s = c->sym;
  const int n = c->nnd;
  const std::vector<int>& rp = c->h_rowptr;
  const std::vector<int>& col = c->h_col;
  std::vector<int> urow(n + 1, 0), diag(n, 0), lcount(n, 0);
  for (int I = 0; I < n; ++I) {
    const int* b = col.data() + rp[I];
    const int* e = col.data() + rp[I + 1];
    const int* d = std::lower_bound(b, e, I);
    if (d == e || *d != I) {
      c->err = "symmetric product: a row without its diagonal block";
      return TG_ERR_ARG;
    }
    diag[I] = (int)(d - col.data());
    urow[I + 1] = urow[I] + (int)(e - d);
    lcount[I] = (int)(d - b);
  }
  const long long nu_tot = urow[n];
  if (nu_tot >= (1LL << 31)) {
    c->err = "symmetric product: too many upper blocks for 32-bit ids";
    return TG_ERR_CAPACITY;
  }
  // tiles: rows grouped while the tile holds at most tile_blocks upper blocks
  std::vector<int> tiles(1, 0);
  for (int r = 0; r < n; ++r)
    if (r > tiles.back() && urow[r + 1] - urow[tiles.back()] > tile_blocks) tiles.push_back(r);
  tiles.push_back(n);
  const int nt = (int)tiles.size() - 1;
  std::vector<long long> off(nt + 1, 0);
  std::vector<int> koff(nt + 1, 0);
  for (int t = 0; t <= nt; ++t) koff[t] = urow[tiles[t]];
  int cap_blocks = 0;
  long long cap_s = 0;
  for (int t = 0; t < nt; ++t) {
    const int r0 = tiles[t], r1 = tiles[t + 1];
    int nl = 0;
    for (int r = r0; r < r1; ++r) nl += lcount[r];
    const int nu = urow[r1] - urow[r0];
    const long long b = sym_struct_bytes(r1 - r0, nu, nl);
    off[t + 1] = off[t] + b;
    cap_s = std::max(cap_s, b);
    cap_blocks = std::max(cap_blocks, nu);
  }
  // structure bytes
  std::vector<unsigned char> blob((size_t)off[nt], 0);
  for (int t = 0; t < nt; ++t) {
    const int r0 = tiles[t], r1 = tiles[t + 1], nrows = r1 - r0;
    int* h = reinterpret_cast<int*>(blob.data() + off[t]);
    int nl = 0;
    for (int r = r0; r < r1; ++r) nl += lcount[r];
    const int nu = urow[r1] - urow[r0];
    h[0] = r0;
    h[1] = nrows;
    h[2] = urow[r0];
    h[3] = nl;
    int* urp = h + 4;
    int* lrp = urp + ceil4(nrows + 1);
    int* ucol = lrp + ceil4(nrows + 1);
    int* lcol = ucol + ceil4(nu);
    int* lk = lcol + ceil4(nl);
    int ku = 0, kl = 0;
    for (int r = r0; r < r1; ++r) {
      urp[r - r0] = ku;
      lrp[r - r0] = kl;
      for (int j = diag[r]; j < rp[r + 1]; ++j) ucol[ku++] = col[j];
      for (int j = rp[r]; j < diag[r]; ++j) {
        // block (r, J), J < r: the transpose of upper block (J, r) in row J
        const int J = col[j];
        const int* jb = col.data() + diag[J];
        const int* je = col.data() + rp[J + 1];
        const int* pos = std::lower_bound(jb, je, r);
        lcol[kl] = J;
        lk[kl] = urow[J] + (int)(pos - jb);
        ++kl;
      }
    }
    urp[nrows] = ku;
    lrp[nrows] = kl;
  }
  // release the previous format, allocate and upload
  sym_free(c);
  s.ntiles = nt;
  s.tile_blocks = tile_blocks;
  s.nu = nu_tot;
  s.nl = c->nnzb - nu_tot;
  s.cap_struct = (int)((cap_s + 127) / 128 * 128);
  s.cap_blocks = cap_blocks;
  s.h_off = off;
  if (!dalloc(c, &s.d_blob, blob.size()) || !dalloc(c, &s.d_off, (size_t)nt + 1) ||
      !dalloc(c, &s.d_koff, (size_t)nt + 1) || !dalloc(c, &s.d_urow, (size_t)n + 1) ||
      !dalloc(c, &s.d_diag, (size_t)n))
    return TG_ERR_OOM;
  cudaStream_t st = c->stream;
  if (!ok(c, cudaMemcpyAsync(s.d_blob, blob.data(), blob.size(), cudaMemcpyHostToDevice, st), "sym blob") ||
      !ok(c, cudaMemcpyAsync(s.d_off, off.data(), sizeof(long long) * (nt + 1), cudaMemcpyHostToDevice, st), "sym off") ||
      !ok(c, cudaMemcpyAsync(s.d_koff, koff.data(), sizeof(int) * (nt + 1), cudaMemcpyHostToDevice, st), "sym koff") ||
      !ok(c, cudaMemcpyAsync(s.d_urow, urow.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, st), "sym urow") ||
      !ok(c, cudaMemcpyAsync(s.d_diag, diag.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st), "sym diag") ||
      !ok(c, cudaStreamSynchronize(st), "sync"))
    return TG_ERR_CUDA;
  s.built = true;
  // the captured PCG chunk bakes in the product
  if (c->pcg_graph) cudaGraphExecDestroy(c->pcg_graph);
  c->pcg_graph = nullptr;
  c->pcg_graph_key = -1;
  return TG_OK;
}

bool sym_active(const Context* c) { return c->sym_mode != 0 && !c->composed && c->nnd > 0; }

// Values of the symmetric format from the last assembly (one pass over the
// full-storage tiles).
int sym_convert(Context* c, int precision) {
  SymStore& s = c->sym;
  if (!s.built || s.tile_blocks != c->sym_tile_blocks) {
    const int b = sym_build(c, c->sym_tile_blocks);
    if (b) return b;
  }
  const bool f32 = precision == TG_MIXED;
  const size_t pad = 16;  // V1 copies are rounded out to 16 bytes
  if (f32 && !s.d_v8_32 && (!dalloc(c, &s.d_v8_32, (size_t)s.nu * 8) || !dalloc(c, &s.d_v1_32, (size_t)s.nu + pad)))
    return TG_ERR_OOM;
  if (!f32 && !s.d_v8_64 && (!dalloc(c, &s.d_v8_64, (size_t)s.nu * 8) || !dalloc(c, &s.d_v1_64, (size_t)s.nu + pad)))
    return TG_ERR_OOM;
  const int grid = std::max(1, std::min((c->nnd + 7) / 8, c->num_sms * 16));
  if (f32)
    sym_convert_kernel<float><<<grid, 256, 0, c->stream>>>(
        c->nnd, c->d_rowptr, s.d_diag, s.d_urow, c->d_blob32, c->d_blob_off32, c->d_row_tile,
        reinterpret_cast<V8T<float>::type*>(s.d_v8_32), s.d_v1_32);
  else
    sym_convert_kernel<double><<<grid, 256, 0, c->stream>>>(
        c->nnd, c->d_rowptr, s.d_diag, s.d_urow, c->d_blob64, c->d_blob_off64, c->d_row_tile,
        reinterpret_cast<V8T<double>::type*>(s.d_v8_64), s.d_v1_64);
  c->launches++;
  if (!ok(c, cudaGetLastError(), "sym_convert_kernel")) return TG_ERR_CUDA;
  s.precision = precision;
  return TG_OK;
}

template <typename T, int NST, int MINB>
static int sym_config_n(Context* c, SymLaunch& L) {
  const SymStore& s = c->sym;
  L.smem = (size_t)NST * ((size_t)s.cap_struct + cap_bytes_v8<T>(s) + cap_bytes_v1<T>(s));
  int optin = 0;
  if (!ok(c, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device), "attribute"))
    return TG_ERR_CUDA;
  cudaFuncAttributes fa;
  if (!ok(c, cudaFuncGetAttributes(&fa, pcg_spmv_sym_kernel<T, NST, MINB>), "function attributes")) return TG_ERR_CUDA;
  if (L.smem + fa.sharedSizeBytes + 1024 > (size_t)optin) {
    c->err = "symmetric SpMV tile ring does not fit in shared memory (reduce the tile size)";
    return TG_ERR_CAPACITY;
  }
  // one value for every context (the attribute belongs to the function)
  if (!ok(c, cudaFuncSetAttribute(pcg_spmv_sym_kernel<T, NST, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  optin - (int)fa.sharedSizeBytes),
          "smem attribute"))
    return TG_ERR_CUDA;
  int per_sm = 0;
  if (!ok(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pcg_spmv_sym_kernel<T, NST, MINB>, 256, L.smem),
          "occupancy"))
    return TG_ERR_CUDA;
  if (per_sm < 1) {
    c->err = "symmetric SpMV tile does not fit in shared memory";
    return TG_ERR_CAPACITY;
  }
  L.grid = std::max(1, std::min(s.ntiles, c->num_sms * per_sm));
  L.stages = NST;
  L.minb = MINB;
  return TG_OK;
}

int sym_config(Context* c, int precision, SymLaunch& L) {
  if (!c->sym.built || c->sym.precision != precision) {
    c->err = "symmetric SpMV: values not converted for this precision";
    return TG_ERR_ARG;
  }
  // launch shapes: 1 two staged tiles at up to 80 registers (3 CTAs/SM), 2
  // two staged tiles at 64 (4 CTAs/SM), 3 three staged tiles at 80
  const bool f32 = precision == TG_MIXED;
  switch (c->sym_mode) {
    case 2: return f32 ? sym_config_n<float, 2, 4>(c, L) : sym_config_n<double, 2, 4>(c, L);
    case 3: return f32 ? sym_config_n<float, 3, 3>(c, L) : sym_config_n<double, 3, 3>(c, L);
    default: return f32 ? sym_config_n<float, 2, 3>(c, L) : sym_config_n<double, 2, 3>(c, L);
  }
}

template <typename T>
static void sym_launch_t(Context* c, const SymLaunch& L, const void* p, void* q, double* partials, PcgScalars* sc,
                         double* node_dot) {
  using V = typename Vec4<T>::type;
  const SymStore& s = c->sym;
  const bool f32 = std::is_same<T, float>::value;
  const typename V8T<T>::type* gv8 =
      reinterpret_cast<const typename V8T<T>::type*>(f32 ? (const void*)s.d_v8_32 : (const void*)s.d_v8_64);
  const T* gv1 = reinterpret_cast<const T*>(f32 ? (const void*)s.d_v1_32 : (const void*)s.d_v1_64);
#define TG_SYM_ARGS s.ntiles, s.d_off, s.d_koff, s.d_blob, s.cap_struct, cap_bytes_v8<T>(s), cap_bytes_v1<T>(s), gv8, \
    gv1, c->d_mask, (const V*)p, (V*)q, partials, sc, c->d_status, node_dot
  if (L.stages == 3)
    pcg_spmv_sym_kernel<T, 3, 3><<<L.grid, 256, L.smem, c->stream>>>(TG_SYM_ARGS);
  else if (L.minb == 4)
    pcg_spmv_sym_kernel<T, 2, 4><<<L.grid, 256, L.smem, c->stream>>>(TG_SYM_ARGS);
  else
    pcg_spmv_sym_kernel<T, 2, 3><<<L.grid, 256, L.smem, c->stream>>>(TG_SYM_ARGS);
#undef TG_SYM_ARGS
}

void sym_launch(Context* c, int precision, const SymLaunch& L, const void* p, void* q, double* partials,
                PcgScalars* sc, double* node_dot) {
  if (precision == TG_MIXED)
    sym_launch_t<float>(c, L, p, q, partials, sc, node_dot);
  else
    sym_launch_t<double>(c, L, p, q, partials, sc, node_dot);
}

void sym_free(Context* c) {
  SymStore& s = c->sym;
  for (void* p : {(void*)s.d_blob, (void*)s.d_off, (void*)s.d_koff, (void*)s.d_urow, (void*)s.d_diag,
                  (void*)s.d_v8_32, (void*)s.d_v1_32, (void*)s.d_v8_64, (void*)s.d_v1_64})
    if (p) dfree(c, p);
  s = SymStore{};
}

}  // namespace tg
