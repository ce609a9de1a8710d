// Symmetric push storage of the single-reduction PCG product, sm_103a.
//
// The assembled tangent is symmetric block by block on the active dofs, so
// the product needs only the upper node blocks of every row (its diagonal
// block and every block (I, J), J > I: 3.73 M of the 7.19 M blocks of the
// 64^3 block).  Instead of reading a lower block (I, J) as the transpose of
// its upper twin -- a dependent gather of 36 bytes per block -- the row that
// streams the upper block (J, I) applies its transpose to u_J and stores the
// result in a slot of row I: stores do not stall the streaming warp, and row
// I's slots are read back contiguously by the vector kernel of the same
// iteration (about 55 MB on the 64^3 block, L2-resident between the two
// kernels).  The reference stores the upper triangle of a symmetric system
// too and applies the lower part by symmetry (MSRMatrixT::Multx,
// MSRMatrixT.cpp:385-420); this is that product restructured for a
// bandwidth-bound GPU stream.
//
// Layout of tile t (16-byte aligned, one bulk copy), over rows
// [tile_row[t], tile_row[t+1]):
//   int header[4] {first row r0, rows, upper blocks nb, plane stride ps = ceil4(nb)}
//   int rp[ceil4(rows+1)]   local row pointers (rp[0] = 0)
//   int col[ceil4(nb)]      column of every upper block (the row's diagonal first)
//   int slot[ceil4(nb)]     push slot of every upper block (-1 for the diagonal)
//   T   planes[9][ps]       entry k of every block in plane k
// A block (I, J), J > I, pushes to slot k pstride + J, k the position of I
// among row J's lower columns and pstride nnd rounded up to 8: the slots are
// 128-byte aligned planes by rank, so rank k of every row is one node vector.  On a structured numbering a rank is one direction of
// the stencil, and the rows of a warp pass push to consecutive slots of the
// same plane -- whole sectors, no partially written sector left in L2 to be
// merged on its way to DRAM -- and the vector kernel reads each plane
// coalesced.
//
// Everything is built on the device from the node-block CSR (a composed
// batch mesh has no host copy of it): the diagonal of every row by binary
// search, exclusive scans for the upper and lower row pointers, k G tiles of
// equal upper block count (G the product's resident CTAs), the tile byte
// offsets on the host from the tiles' sizes, then the structure in one pass.
// Values are assembled straight into the tiles when the solve streams this
// storage (assemble_upper_kernel), or converted from the full-storage tiles
// when the tangent went to the full storage and a solve here needs it.
#include <algorithm>
#include <vector>

#include "krylov_common.cuh"

namespace tg {

namespace {

// upper blocks per tile.  C2 (64^3), Newton step with 2 stages of four CTAs
// per SM: 256 -> 36.7 ms, 320 -> 33.7, 384 -> 32.0, 448 -> 30.7, 512 -> 30.65,
// 576 -> 32.6; dealing the rows of a tile to the warps from a rotating first
// warp changed nothing
constexpr int kPushTileBlocks = 512;
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;         // items per thread of a scan block

__host__ __device__ inline long long push_tile_bytes(int nrows, int nb, int elem) {
  return 16 + 4LL * ceil4(nrows + 1) + 8LL * ceil4(nb) + 9LL * ceil4(nb) * elem;
}

// per row: position of the diagonal block in the full CSR, counts of upper
// (diagonal included) and strictly lower blocks; a row without its diagonal
// raises the flag
__global__ void push_count_kernel(int nnd, const int* __restrict__ rowptr, const int* __restrict__ col,
                                  int* __restrict__ diag, int* __restrict__ ucnt, int* __restrict__ lcnt,
                                  int* __restrict__ flag) {
  // flag[0]: a row without its diagonal; flag[1]: the largest lower count
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= nnd) return;
  const int b = rowptr[I], e = rowptr[I + 1];
  int lo = b, hi = e;  // first column >= I
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (col[mid] < I)
      lo = mid + 1;
    else
      hi = mid;
  }
  if (lo == e || col[lo] != I) atomicOr(flag, 1);
  diag[I] = lo;
  ucnt[I] = e - lo;
  lcnt[I] = lo - b;
  atomicMax(flag + 1, lo - b);
}

// Exclusive scan of n counts into out[0..n] (out[n] the total), three
// passes: block sums, one block scanning the block sums, block offsets added.
__global__ void __launch_bounds__(kScanThreads) scan_block_kernel(int n, const int* __restrict__ in,
                                                                   int* __restrict__ out, int* __restrict__ bsum) {
  __shared__ int warp_tot[kScanThreads / 32];
  const int base = (blockIdx.x * kScanThreads + threadIdx.x) * kScanItems;
  int v[kScanItems], run = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = base + k < n ? in[base + k] : 0;
    run += v[k];
  }
  // inclusive scan of the thread totals: warp shuffles, then the warp totals
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int t = lane < kScanThreads / 32 ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < kScanThreads / 32) warp_tot[lane] = t;
  }
  __syncthreads();
  int acc = incl - run + (warp > 0 ? warp_tot[warp - 1] : 0);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) out[base + k] = acc;
    acc += v[k];
  }
  if (threadIdx.x == kScanThreads - 1) bsum[blockIdx.x] = acc;
}

// one block: exclusive scan of the nb block sums in place, in chunks
__global__ void __launch_bounds__(kScanThreads) scan_sums_kernel(int nb, int* __restrict__ bsum, int* __restrict__ total) {
  __shared__ int warp_tot[kScanThreads / 32];
  __shared__ int carry;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int c0 = 0; c0 < nb; c0 += kScanThreads) {
    const int i = c0 + threadIdx.x;
    const int v = i < nb ? bsum[i] : 0;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      int t = warp_tot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      warp_tot[lane] = t;
    }
    __syncthreads();
    const int excl = carry + incl - v + (warp > 0 ? warp_tot[warp - 1] : 0);
    if (i < nb) bsum[i] = excl;
    __syncthreads();
    if (threadIdx.x == kScanThreads - 1) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void scan_add_kernel(int n, const int* __restrict__ bsum, const int* __restrict__ total,
                                int* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += bsum[i / (kScanThreads * kScanItems)];
  if (i == 0) out[n] = *total;
}

// tile j of `parts` starts at the row boundary nearest j nu / parts
__global__ void push_tile_start_kernel(int parts, int nnd, const int* __restrict__ urow, int* __restrict__ start) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j > parts) return;
  if (j == 0 || j == parts) {
    start[j] = j == 0 ? 0 : nnd;
    return;
  }
  const long long nu = urow[nnd];
  const long long target = ((long long)j * nu + parts / 2) / parts;
  int lo = 0, hi = nnd;  // first row r with urow[r] >= target
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (urow[mid] < target)
      lo = mid + 1;
    else
      hi = mid;
  }
  if (lo > 0 && target - urow[lo - 1] < urow[lo] - target) --lo;
  start[j] = lo;
}

// the upper row pointer at every tile start
__global__ void push_tile_blocks_kernel(int nt, const int* __restrict__ tile_row, const int* __restrict__ urow,
                                        int* __restrict__ ut) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t <= nt) ut[t] = urow[tile_row[t]];
}

// rows of every tile -> tile (one CTA per tile)
__global__ void push_row_tile_kernel(const int* __restrict__ tile_row, int* __restrict__ row_tile) {
  const int t = blockIdx.x;
  for (int r = tile_row[t] + threadIdx.x; r < tile_row[t + 1]; r += blockDim.x) row_tile[r] = t;
}

// The structure of both precisions' tiles: one warp per row writes its row
// pointer, the columns of its upper blocks and their push slots (the lower
// position of row I in row J by binary search); the first row of a tile
// writes the header, the last its closing row pointer.
__global__ void __launch_bounds__(256) push_structure_kernel(
    int nnd, int pstride, const int* __restrict__ rowptr, const int* __restrict__ col, const int* __restrict__ diag,
    const int* __restrict__ urow, const int* __restrict__ tile_row,
    const int* __restrict__ row_tile, const long long* __restrict__ off32, const long long* __restrict__ off64,
    unsigned char* __restrict__ blob32, unsigned char* __restrict__ blob64) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; I < nnd; I += warps) {
    const int t = row_tile[I];
    const int r0 = tile_row[t], r1 = tile_row[t + 1], nrows = r1 - r0;
    const int k0 = urow[r0], nb = urow[r1] - k0;
    for (int pr = 0; pr < 2; ++pr) {
      unsigned char* blob = pr == 0 ? blob32 : blob64;
      if (!blob) continue;
      int* h = reinterpret_cast<int*>(blob + (pr == 0 ? off32[t] : off64[t]));
      int* rp = h + 4;
      int* cl = rp + ceil4(nrows + 1);
      int* sl = cl + ceil4(nb);
      if (lane == 0) {
        if (I == r0) {
          h[0] = r0;
          h[1] = nrows;
          h[2] = nb;
          h[3] = ceil4(nb);
        }
        rp[I - r0] = urow[I] - k0;
        if (I == r1 - 1) rp[nrows] = nb;
      }
      const int jd = diag[I], je = rowptr[I + 1];
      for (int j = jd + lane; j < je; j += 32) {
        const int k = urow[I] - k0 + (j - jd);
        const int J = col[j];
        cl[k] = J;
        int slot = -1;
        if (J != I) {
          int lo = rowptr[J], hi = diag[J];  // I among row J's lower columns
          while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (col[mid] < I)
              lo = mid + 1;
            else
              hi = mid;
          }
          slot = (lo - rowptr[J]) * pstride + J;
        }
        sl[k] = slot;
      }
    }
  }
}

// Values from the assembled full-storage tiles: one warp per row copies its
// upper blocks (the full row from its diagonal on) plane by plane.
template <typename T>
__global__ void __launch_bounds__(256) push_convert_kernel(
    int nnd, const int* __restrict__ rowptr, const int* __restrict__ diag, const int* __restrict__ urow,
    const unsigned char* __restrict__ fblob, const long long* __restrict__ foff, const int* __restrict__ frow_tile,
    const int* __restrict__ tile_row, const int* __restrict__ row_tile, const long long* __restrict__ poff,
    unsigned char* __restrict__ pblob) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; I < nnd; I += warps) {
    const unsigned char* fb = fblob + foff[frow_tile[I]];
    const int* fh = reinterpret_cast<const int*>(fb);
    const int ftrow0 = fh[0], ftnrows = fh[1], ftnb = fh[2], fps = fh[3];
    const T* fpl = reinterpret_cast<const T*>(fb + 16 + 4 * ceil4(ftnrows + 1) + 4 * ceil4(ftnb));
    const int ftb0 = rowptr[ftrow0];
    const int t = row_tile[I];
    const int r0 = tile_row[t], nrows = tile_row[t + 1] - r0;
    const int k0 = urow[r0], nb = urow[tile_row[t + 1]] - k0, ps = ceil4(nb);
    T* ppl = reinterpret_cast<T*>(pblob + poff[t] + 16 + 4 * ceil4(nrows + 1) + 8 * ceil4(nb));
    const int jd = diag[I], je = rowptr[I + 1], kr = urow[I] - k0;
    for (int j = jd + lane; j < je; j += 32) {
      const T* src = fpl + (j - ftb0);
      T* dst = ppl + kr + (j - jd);
#pragma unroll
      for (int m = 0; m < 9; ++m) dst[(long long)m * ps] = src[(long long)m * fps];
    }
  }
}

int launch_scan(Context* c, int n, const int* d_in, int* d_out, int* d_tmp) {
  const int nblk = (n + kScanThreads * kScanItems - 1) / (kScanThreads * kScanItems);
  int* bsum = d_tmp;
  int* total = d_tmp + std::max(nblk, 1);
  if (nblk > 0) scan_block_kernel<<<nblk, kScanThreads, 0, c->stream>>>(n, d_in, d_out, bsum);
  scan_sums_kernel<<<1, kScanThreads, 0, c->stream>>>(nblk, bsum, total);
  scan_add_kernel<<<(n + 256) / 256, 256, 0, c->stream>>>(n, bsum, total, d_out);
  c->launches += 3;
  return ok(c, cudaGetLastError(), "scan") ? TG_OK : TG_ERR_CUDA;
}

int push_build(Context* c) {
  PushStore& ps = c->push;
  push_free(c);
  const int n = c->nnd;
  if (n <= 0 || c->nnzb <= 0) {
    c->err = "symmetric push storage: no mesh";
    return TG_ERR_ARG;
  }
  cudaStream_t st = c->stream;
  int *d_ucnt = nullptr, *d_lcnt = nullptr, *d_tmp = nullptr, *d_flag = nullptr;
  const int nblk = (n + kScanThreads * kScanItems - 1) / (kScanThreads * kScanItems);
  if (!dalloc(c, &ps.d_diag, (size_t)n) || !dalloc(c, &ps.d_urow, (size_t)n + 1) ||
      !dalloc(c, &ps.d_lptr, (size_t)n + 1) || !dalloc(c, &ps.d_row_tile, (size_t)n) ||
      !dalloc(c, &d_ucnt, (size_t)n) || !dalloc(c, &d_lcnt, (size_t)n) ||
      !dalloc(c, &d_tmp, (size_t)nblk + 2) || !dalloc(c, &d_flag, 2))
    return TG_ERR_OOM;
  auto release = [&]() {
    dfree(c, d_ucnt);
    dfree(c, d_lcnt);
    dfree(c, d_tmp);
    dfree(c, d_flag);
  };
  int s = TG_OK;
  if (!ok(c, cudaMemsetAsync(d_flag, 0, 2 * sizeof(int), st), "flag")) s = TG_ERR_CUDA;
  if (!s) {
    push_count_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, c->d_rowptr, c->d_col, ps.d_diag, d_ucnt, d_lcnt, d_flag);
    c->launches++;
    if (!ok(c, cudaGetLastError(), "push_count_kernel")) s = TG_ERR_CUDA;
  }
  if (!s) s = launch_scan(c, n, d_ucnt, ps.d_urow, d_tmp);
  if (!s) s = launch_scan(c, n, d_lcnt, ps.d_lptr, d_tmp);
  int h_flag[2] = {0, 0}, nu = 0, nl = 0;
  if (!s && (!ok(c, cudaMemcpyAsync(h_flag, d_flag, 2 * sizeof(int), cudaMemcpyDeviceToHost, st), "flag") ||
             !ok(c, cudaMemcpyAsync(&nu, ps.d_urow + n, sizeof(int), cudaMemcpyDeviceToHost, st), "nu") ||
             !ok(c, cudaMemcpyAsync(&nl, ps.d_lptr + n, sizeof(int), cudaMemcpyDeviceToHost, st), "nl") ||
             !ok(c, cudaStreamSynchronize(st), "sync")))
    s = TG_ERR_CUDA;
  release();
  if (s) return s;
  if (h_flag[0]) {
    c->err = "symmetric push storage: a row without its diagonal block";
    return TG_ERR_ARG;
  }
  ps.pstride = (n + 7) / 8 * 8;
  if ((long long)h_flag[1] * ps.pstride >= (1LL << 31)) {
    c->err = "symmetric push storage: too many push slots for 32-bit indices";
    return TG_ERR_CAPACITY;
  }
  ps.nu = nu;
  ps.nl = nl;
  ps.kmax = h_flag[1];
  // k G tiles of equal upper block count, G the product's resident CTAs
  // (four per SM in FP32; FP64 runs two, G/2, on the same tiles)
  const long long G = (long long)c->num_sms * 4;
  const long long k = std::max(1LL, (nu + G * kPushTileBlocks - 1) / (G * kPushTileBlocks));
  const int parts = (int)std::min<long long>(k * G, n);
  int* d_start = nullptr;
  if (!dalloc(c, &d_start, (size_t)parts + 1)) return TG_ERR_OOM;
  push_tile_start_kernel<<<(parts + 256) / 256, 256, 0, st>>>(parts, n, ps.d_urow, d_start);
  c->launches++;
  std::vector<int> start(parts + 1);
  if (!ok(c, cudaGetLastError(), "push_tile_start_kernel") ||
      !ok(c, cudaMemcpyAsync(start.data(), d_start, sizeof(int) * (parts + 1), cudaMemcpyDeviceToHost, st), "tiles") ||
      !ok(c, cudaStreamSynchronize(st), "sync")) {
    dfree(c, d_start);
    return TG_ERR_CUDA;
  }
  dfree(c, d_start);
  std::vector<int> tiles(1, 0);
  for (int j = 1; j <= parts; ++j)
    if (start[j] > tiles.back()) tiles.push_back(start[j]);
  if (tiles.back() != n) tiles.push_back(n);
  const int nt = (int)tiles.size() - 1;
  ps.ntiles = nt;
  ps.h_tile_row = tiles;
  if (!dalloc(c, &ps.d_tile_row, (size_t)nt + 1) || !dalloc(c, &ps.d_off32, (size_t)nt + 1) ||
      !dalloc(c, &ps.d_off64, (size_t)nt + 1))
    return TG_ERR_OOM;
  // the upper row pointer at every tile start, for the tile sizes
  std::vector<int> ut(nt + 1);
  {
    int* d_ut = nullptr;
    if (!dalloc(c, &d_ut, (size_t)nt + 1)) return TG_ERR_OOM;
    const bool good =
        ok(c, cudaMemcpyAsync(ps.d_tile_row, tiles.data(), sizeof(int) * (nt + 1), cudaMemcpyHostToDevice, st),
           "tiles");
    if (good) {
      push_tile_blocks_kernel<<<(nt + 256) / 256, 256, 0, st>>>(nt, ps.d_tile_row, ps.d_urow, d_ut);
      c->launches++;
    }
    const bool got = good && ok(c, cudaGetLastError(), "push_tile_blocks_kernel") &&
                     ok(c, cudaMemcpyAsync(ut.data(), d_ut, sizeof(int) * (nt + 1), cudaMemcpyDeviceToHost, st), "ut") &&
                     ok(c, cudaStreamSynchronize(st), "sync");
    dfree(c, d_ut);
    if (!got) return TG_ERR_CUDA;
  }
  ps.h_off32.assign(nt + 1, 0);
  ps.h_off64.assign(nt + 1, 0);
  ps.cap32 = ps.cap64 = 0;
  for (int t = 0; t < nt; ++t) {
    const int nrows = tiles[t + 1] - tiles[t], nb = ut[t + 1] - ut[t];
    const long long b32 = push_tile_bytes(nrows, nb, 4), b64 = push_tile_bytes(nrows, nb, 8);
    ps.h_off32[t + 1] = ps.h_off32[t] + b32;
    ps.h_off64[t + 1] = ps.h_off64[t] + b64;
    ps.cap32 = std::max(ps.cap32, b32);
    ps.cap64 = std::max(ps.cap64, b64);
  }
  if (!ok(c, cudaMemcpyAsync(ps.d_off32, ps.h_off32.data(), sizeof(long long) * (nt + 1), cudaMemcpyHostToDevice, st),
          "off") ||
      !ok(c, cudaMemcpyAsync(ps.d_off64, ps.h_off64.data(), sizeof(long long) * (nt + 1), cudaMemcpyHostToDevice, st),
          "off"))
    return TG_ERR_CUDA;
  push_row_tile_kernel<<<nt, 256, 0, st>>>(ps.d_tile_row, ps.d_row_tile);
  c->launches++;
  if (!ok(c, cudaGetLastError(), "push_row_tile_kernel")) return TG_ERR_CUDA;
  ps.built = true;
  return TG_OK;
}

// the tiles of one precision: allocated, zeroed, structure written
int push_blob(Context* c, int precision) {
  PushStore& ps = c->push;
  const bool f32 = precision == TG_MIXED;
  unsigned char** blob = f32 ? &ps.d_blob32 : &ps.d_blob64;
  void** push = f32 ? &ps.d_push32 : &ps.d_push64;
  if (*blob) return TG_OK;
  const long long total = (f32 ? ps.h_off32 : ps.h_off64)[ps.ntiles];
  if (!dalloc(c, blob, (size_t)total)) return TG_ERR_OOM;
  const size_t vb = f32 ? sizeof(float4) : sizeof(double4_32a);
  // rank planes; slots no block pushes to (rows with fewer lower blocks
  // than the largest count) are never read
  unsigned char* pb = nullptr;
  if (!dalloc(c, &pb, (size_t)std::max(ps.kmax, 1) * ps.pstride * vb)) return TG_ERR_OOM;
  *push = pb;
  if (!ok(c, cudaMemsetAsync(*blob, 0, (size_t)total, c->stream), "push blob")) return TG_ERR_CUDA;
  const int grid = std::max(1, std::min((c->nnd + 7) / 8, c->num_sms * 16));
  push_structure_kernel<<<grid, 256, 0, c->stream>>>(c->nnd, ps.pstride, c->d_rowptr, c->d_col, ps.d_diag, ps.d_urow,
                                                     ps.d_tile_row, ps.d_row_tile, ps.d_off32, ps.d_off64,
                                                     f32 ? *blob : nullptr, f32 ? nullptr : *blob);
  c->launches++;
  return ok(c, cudaGetLastError(), "push_structure_kernel") ? TG_OK : TG_ERR_CUDA;
}

}  // namespace

int push_structure(Context* c, int precision) {
  PushStore& ps = c->push;
  if (!ps.built) {
    const int s = push_build(c);
    if (s) return s;
  }
  return push_blob(c, precision);
}

int push_prepare(Context* c, int precision) {
  PushStore& ps = c->push;
  const bool f32 = precision == TG_MIXED;
  int s = push_structure(c, precision);
  if (s) return s;
  long long& serial = f32 ? ps.serial32 : ps.serial64;
  if (serial == c->tangent_serial) return TG_OK;
  // copied from the full storage (assembled there for another solve)
  s = ensure_full_assembly(c);
  if (s) return s;
  const int grid = std::max(1, std::min((c->nnd + 7) / 8, c->num_sms * 16));
  if (f32)
    push_convert_kernel<float><<<grid, 256, 0, c->stream>>>(c->nnd, c->d_rowptr, ps.d_diag, ps.d_urow, c->d_blob32,
                                                            c->d_blob_off32, c->d_row_tile, ps.d_tile_row,
                                                            ps.d_row_tile, ps.d_off32, ps.d_blob32);
  else
    push_convert_kernel<double><<<grid, 256, 0, c->stream>>>(c->nnd, c->d_rowptr, ps.d_diag, ps.d_urow, c->d_blob64,
                                                             c->d_blob_off64, c->d_row_tile, ps.d_tile_row,
                                                             ps.d_row_tile, ps.d_off64, ps.d_blob64);
  c->launches++;
  if (!ok(c, cudaGetLastError(), "push_convert_kernel")) return TG_ERR_CUDA;
  serial = c->tangent_serial;
  return TG_OK;
}

void push_free(Context* c) {
  PushStore& ps = c->push;
  for (void* p : {(void*)ps.d_off32, (void*)ps.d_off64, (void*)ps.d_blob32, (void*)ps.d_blob64,
                  (void*)ps.d_tile_row, (void*)ps.d_row_tile, (void*)ps.d_urow, (void*)ps.d_diag, (void*)ps.d_lptr,
                  ps.d_push32, ps.d_push64})
    if (p) dfree(c, p);
  ps = PushStore{};
}

}  // namespace tg
