// Resident mesh templates and device-side composition of batch meshes.
//
// A serving loop solves a stream of batches whose meshes are disjoint unions
// of a few distinct RVE meshes (one per side length).  Each distinct mesh is
// registered once as a template: its equation slots, node-block pattern,
// contribution map, node-element map and row tiles are built on the host one
// time and stay in device memory.  Composing a batch mesh is then a handful
// of O(batch) host bookkeeping and one memory-bound kernel that writes every
// per-mesh index array with its instance offsets, instead of rebuilding the
// pattern of the whole batch on the host and copying it over.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "tg_internal.h"

namespace tg {

struct TplDev {
  const double* X;        // SoA 3*nnd
  const int* conn;        // nel*8
  const int8_t* block;    // nel
  const uint8_t* mask;    // nnd
  const int* eq_slot;     // neq
  const int* nptr;        // nnd+1
  const int* nlist;       // nel*8
  const int* rowptr;      // nnd+1
  const int* col;         // nnzb
  const int* cptr;        // nnzb+1
  const int* contrib;     // nel*64
  const int* row_tile;    // nnd
  int nnd, nel, neq, nnzb;
  int geo_off;            // first element in the template geometry pool
};

struct MeshTemplate {
  TplDev dev{};
  std::vector<int> rowptr;      // host block-row pointers (re-tiling)
  std::vector<int> tile_row;    // local tile starts, ntiles+1
  std::vector<long long> tile_b32, tile_b64;  // bytes of every tile in the tile-contiguous storage
  int tile_blocks = 0;
  int* row_tile = nullptr;      // device, owned through dev.row_tile
  std::vector<void*> allocs;
};

struct InstDev {
  int tpl, node_off, elem_off, eq_off, nnzb_off, tile_off;
};

struct ComposeOut {
  double* X;
  int* conn;
  int8_t* block;
  uint8_t* mask;
  int* eq_slot;
  int* nptr;
  int* nlist;
  int* rowptr;
  int* col;
  int* cptr;
  int* contrib;
  int* row_tile;
  int* seg_node;
  int* seg_elem;
  int* elem_src;  // each element's element in the template geometry pool
  int nnd, nel;
  int nnzb;
};

namespace {

int set_dev(Context* c) { return ok(c, cudaSetDevice(c->device), "cudaSetDevice") ? TG_OK : TG_ERR_CUDA; }

template <typename T>
bool talloc(Context* c, MeshTemplate* t, T** p, size_t n) {
  if (n == 0) n = 1;
  cudaError_t e = cudaMallocAsync((void**)p, n * sizeof(T), c->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    c->err = std::string("cudaMallocAsync failed: ") + cudaGetErrorString(e);
    *p = nullptr;
    return false;
  }
  t->allocs.push_back((void*)*p);
  return true;
}

void release(Context* c, MeshTemplate* t) {
  for (void* p : t->allocs) cudaFreeAsync(p, c->stream);
  t->allocs.clear();
}

// Row tiles of a template (the same rule as the streamed SpMV's tiles of an
// uploaded mesh) and its row -> tile map on the device.
int tile_template(Context* c, MeshTemplate* t, int tile_blocks) {
  const int nnd = t->dev.nnd;
  std::vector<int> tiles(1, 0);
  for (int r = 0; r < nnd; ++r)
    if (r > tiles.back() && t->rowptr[r + 1] - t->rowptr[tiles.back()] > tile_blocks) tiles.push_back(r);
  tiles.push_back(nnd);
  const int nt = (int)tiles.size() - 1;
  std::vector<int> row_tile(nnd);
  t->tile_b32.assign(nt, 0);
  t->tile_b64.assign(nt, 0);
  for (int k = 0; k < nt; ++k) {
    const int nrows = tiles[k + 1] - tiles[k];
    const int nb = t->rowptr[tiles[k + 1]] - t->rowptr[tiles[k]];
    for (int r = tiles[k]; r < tiles[k + 1]; ++r) row_tile[r] = k;
    t->tile_b32[k] = blob_tile_bytes(nrows, nb, 4);
    t->tile_b64[k] = blob_tile_bytes(nrows, nb, 8);
  }
  t->tile_row = tiles;
  t->tile_blocks = tile_blocks;
  if (!t->row_tile && !talloc(c, t, &t->row_tile, (size_t)nnd)) return TG_ERR_OOM;
  t->dev.row_tile = t->row_tile;
  return ok(c, cudaMemcpyAsync(t->row_tile, row_tile.data(), sizeof(int) * nnd, cudaMemcpyHostToDevice, c->stream),
            "row_tile") &&
                 ok(c, cudaStreamSynchronize(c->stream), "sync")
             ? TG_OK
             : TG_ERR_CUDA;
}

__device__ __forceinline__ void copy_add(int* __restrict__ dst, const int* __restrict__ src, int n, int add,
                                         int start, int stride) {
  for (int k = start; k < n; k += stride) dst[k] = src[k] + add;
}

// One CTA row (blockIdx.y) per instance; the CTAs of a row stride over the
// instance's index arrays.  Every write is an offset copy of the template.
__global__ void __launch_bounds__(256) compose_kernel(const TplDev* __restrict__ tpls,
                                                      const InstDev* __restrict__ inst, int count, ComposeOut o) {
  const InstDev I = inst[blockIdx.y];
  const TplDev T = tpls[I.tpl];
  const int start = blockIdx.x * blockDim.x + threadIdx.x;
  const int stride = gridDim.x * blockDim.x;
  for (int k = start; k < T.nnd; k += stride) {
    o.X[I.node_off + k] = T.X[k];
    o.X[o.nnd + I.node_off + k] = T.X[T.nnd + k];
    o.X[2 * o.nnd + I.node_off + k] = T.X[2 * T.nnd + k];
    o.mask[I.node_off + k] = T.mask[k];
  }
  copy_add(o.row_tile + I.node_off, T.row_tile, T.nnd, I.tile_off, start, stride);
  copy_add(o.nptr + I.node_off, T.nptr, T.nnd, I.elem_off * 8, start, stride);
  copy_add(o.rowptr + I.node_off, T.rowptr, T.nnd, I.nnzb_off, start, stride);
  for (int k = start; k < T.nel; k += stride) {
    o.block[I.elem_off + k] = T.block[k];
    o.elem_src[I.elem_off + k] = T.geo_off + k;
  }
  copy_add(o.conn + I.elem_off * 8, T.conn, T.nel * 8, I.node_off, start, stride);
  copy_add(o.nlist + I.elem_off * 8, T.nlist, T.nel * 8, I.elem_off * 8, start, stride);
  copy_add(o.eq_slot + I.eq_off, T.eq_slot, T.neq, I.node_off * 4, start, stride);
  copy_add(o.col + I.nnzb_off, T.col, T.nnzb, I.node_off, start, stride);
  copy_add(o.cptr + I.nnzb_off, T.cptr, T.nnzb, I.elem_off * 64, start, stride);
  copy_add(o.contrib + I.elem_off * 64, T.contrib, T.nel * 64, I.elem_off * 64, start, stride);
  if (start == 0) {
    o.seg_node[blockIdx.y] = I.node_off;
    o.seg_elem[blockIdx.y] = I.elem_off;
    if ((int)blockIdx.y == count - 1) {
      o.nptr[o.nnd] = o.nel * 8;
      o.rowptr[o.nnd] = o.nnzb;
      o.cptr[o.nnzb] = o.nel * 64;
      o.seg_node[count] = o.nnd;
      o.seg_elem[count] = o.nel;
    }
  }
}

// u_d = sum_j (F_s - I)_dj X_j on every prescribed dof of segment s.
__global__ void affine_prescribed_kernel(int nnd, int nseg, const int* __restrict__ seg_node,
                                         const double* __restrict__ F, const double* __restrict__ X,
                                         const uint8_t* __restrict__ mask, double4_32a* __restrict__ u) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nnd) return;
  const int m = mask[n];
  if (m == 7) return;
  int lo = 0, hi = nseg;  // last segment with seg_node[s] <= n
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (seg_node[mid] <= n) lo = mid;
    else hi = mid;
  }
  const double* f = F + 9 * lo;
  const double x[3] = {X[n], X[nnd + n], X[2 * nnd + n]};
  double* p = reinterpret_cast<double*>(u + n);
  for (int d = 0; d < 3; ++d)
    if (!(m & (1 << d))) p[d] = (f[3 * d] - (d == 0)) * x[0] + (f[3 * d + 1] - (d == 1)) * x[1] + (f[3 * d + 2] - (d == 2)) * x[2];
}

}  // namespace

void free_templates(Context* c) {
  for (MeshTemplate* t : c->templates) {
    release(c, t);
    delete t;
  }
  c->templates.clear();
  for (TplGeoPool* p : {&c->tpl_geo_ff, &c->tpl_geo64}) {
    if (p->d) cudaFreeAsync(p->d, c->stream);
    *p = TplGeoPool{};
  }
  c->tpl_elems = 0;
}

// The geometry planes of every resident template in one pool (25 planes of
// 8 points per template element), rebuilt when templates were added since;
// the templates' pool offsets never change.  Without room for it the pool
// stays empty and batch meshes form their own planes.
template <typename G>
int template_geometry_pool(Context* c, TplGeoPool& pool) {
  const int nt = (int)c->templates.size();
  if (pool.d && pool.count == nt) return TG_OK;
  if (pool.d) cudaFreeAsync(pool.d, c->stream);
  pool = TplGeoPool{};
  const long long elems = c->tpl_elems;
  G* g = nullptr;
  if (elems <= 0 || cudaMallocAsync((void**)&g, sizeof(G) * (size_t)elems * 8 * kGeoPlanes, c->stream) != cudaSuccess) {
    cudaGetLastError();
    return TG_OK;
  }
  for (const MeshTemplate* t : c->templates) {
    const TplDev& d = t->dev;
    const int s = launch_geometry<G>(c, d.X, d.nnd, d.conn, d.nel, g, elems * 8, (long long)d.geo_off * 8);
    if (s) {
      cudaFreeAsync(g, c->stream);
      return s;
    }
  }
  pool.d = g;
  pool.elems = elems;
  pool.count = nt;
  return TG_OK;
}
template int template_geometry_pool<float2>(Context*, TplGeoPool&);
template int template_geometry_pool<double>(Context*, TplGeoPool&);

int launch_affine_prescribed(Context* c, const double* d_F) {
  affine_prescribed_kernel<<<(c->nnd + 255) / 256, 256, 0, c->stream>>>(c->nnd, c->nseg, c->d_seg_node, d_F, c->d_X,
                                                                         c->d_mask, c->d_u);
  c->launches++;
  return ok(c, cudaGetLastError(), "affine_prescribed_kernel") ? TG_OK : TG_ERR_CUDA;
}

// Host copies of the structure of a composed mesh (connectivity, coordinates,
// equation numbers, block pattern), read back once when a host-side routine
// needs them: pattern and tangent dumps, segment checks, re-tiling.
int ensure_host_mesh(Context* c) {
  if (!c->composed || !c->h_rowptr.empty()) return TG_OK;
  const int nnd = c->nnd;
  std::vector<uint8_t> mask(nnd);
  c->h_conn.resize((size_t)c->nel * 8);
  c->h_coords.resize((size_t)nnd * 3);
  c->h_rowptr.resize((size_t)nnd + 1);
  c->h_col.resize((size_t)c->nnzb);
  c->h_eq_slot.resize((size_t)c->neq);
  cudaStream_t s = c->stream;
  if (!ok(c, cudaMemcpyAsync(c->h_conn.data(), c->d_conn, sizeof(int) * c->h_conn.size(), cudaMemcpyDeviceToHost, s), "conn") ||
      !ok(c, cudaMemcpyAsync(c->h_coords.data(), c->d_X, sizeof(double) * c->h_coords.size(), cudaMemcpyDeviceToHost, s), "X") ||
      !ok(c, cudaMemcpyAsync(c->h_rowptr.data(), c->d_rowptr, sizeof(int) * (nnd + 1), cudaMemcpyDeviceToHost, s), "rp") ||
      !ok(c, cudaMemcpyAsync(c->h_col.data(), c->d_col, sizeof(int) * c->nnzb, cudaMemcpyDeviceToHost, s), "col") ||
      !ok(c, cudaMemcpyAsync(c->h_eq_slot.data(), c->d_eq_slot, sizeof(int) * c->neq, cudaMemcpyDeviceToHost, s), "slot") ||
      !ok(c, cudaMemcpyAsync(mask.data(), c->d_mask, nnd, cudaMemcpyDeviceToHost, s), "mask") ||
      !ok(c, cudaStreamSynchronize(s), "sync")) {
    c->h_rowptr.clear();
    return TG_ERR_CUDA;
  }
  c->h_eqnos.assign((size_t)nnd * 3, -1);
  int q = 0;
  for (int n = 0; n < nnd; ++n)
    for (int d = 0; d < 3; ++d)
      if (mask[n] & (1 << d)) c->h_eqnos[(size_t)n * 3 + d] = ++q;
  return TG_OK;
}

}  // namespace tg

using namespace tg;

extern "C" {

int tg_template_add(tg_context* c, int nnd, const double* coords, int nel, const int* conn, const int* eqnos,
                    const int* blocks, int* template_id) {
  if (!c || nnd <= 0 || nel <= 0 || !coords || !conn || !eqnos || !template_id) return TG_ERR_ARG;
  if ((long long)nel * 64 >= (1LL << 31)) {
    c->err = "too many elements for the 32-bit contribution map";
    return TG_ERR_CAPACITY;
  }
  for (long long k = 0; k < (long long)nel * 8; ++k)
    if (conn[k] < 0 || conn[k] >= nnd) {
      c->err = "connectivity out of range";
      return TG_ERR_ARG;
    }
  std::vector<int8_t> blk(nel, 0);
  if (blocks)
    for (int e = 0; e < nel; ++e) {
      if (blocks[e] < 0 || blocks[e] >= kMaxBlocks) return TG_ERR_ARG;
      blk[e] = (int8_t)blocks[e];
    }
  std::vector<uint8_t> mask;
  std::vector<int> slot;
  const int neq = equation_slots(c, nnd, eqnos, mask, slot);
  if (neq < 0) return TG_ERR_ARG;
  if (set_dev(c)) return TG_ERR_CUDA;
  MeshTemplate* t = new MeshTemplate();
  std::vector<int> col, cptr, contrib, nptr, nlist;
  build_block_pattern(nnd, nel, conn, t->rowptr, col);
  build_contrib_map(nnd, nel, conn, t->rowptr, col, cptr, contrib);
  build_node_elem(nnd, nel, conn, nptr, nlist);
  TplDev& d = t->dev;
  d.nnd = nnd;
  d.nel = nel;
  d.neq = neq;
  d.nnzb = t->rowptr[nnd];
  if ((c->tpl_elems + nel) * 8 * kGeoPlanes >= (1LL << 31)) {
    c->err = "too many template elements for the 32-bit geometry pool";
    delete t;
    return TG_ERR_CAPACITY;
  }
  d.geo_off = (int)c->tpl_elems;
  double* X;
  int *cn, *es, *np, *nl, *rp, *cl, *cp, *ct;
  int8_t* bk;
  uint8_t* mk;
  const size_t nip = (size_t)nel * 8;
  bool good = talloc(c, t, &X, (size_t)nnd * 3) && talloc(c, t, &cn, nip) && talloc(c, t, &bk, (size_t)nel) &&
              talloc(c, t, &mk, (size_t)nnd) && talloc(c, t, &es, (size_t)std::max(neq, 1)) &&
              talloc(c, t, &np, (size_t)nnd + 1) && talloc(c, t, &nl, nip) && talloc(c, t, &rp, (size_t)nnd + 1) &&
              talloc(c, t, &cl, (size_t)d.nnzb) && talloc(c, t, &cp, (size_t)d.nnzb + 1) && talloc(c, t, &ct, nip * 8);
  if (!good) {
    release(c, t);
    delete t;
    return TG_ERR_OOM;
  }
  cudaStream_t s = c->stream;
  good = ok(c, cudaMemcpyAsync(X, coords, sizeof(double) * nnd * 3, cudaMemcpyHostToDevice, s), "X") &&
         ok(c, cudaMemcpyAsync(cn, conn, sizeof(int) * nip, cudaMemcpyHostToDevice, s), "conn") &&
         ok(c, cudaMemcpyAsync(bk, blk.data(), nel, cudaMemcpyHostToDevice, s), "blocks") &&
         ok(c, cudaMemcpyAsync(mk, mask.data(), nnd, cudaMemcpyHostToDevice, s), "mask") &&
         ok(c, cudaMemcpyAsync(es, slot.data(), sizeof(int) * neq, cudaMemcpyHostToDevice, s), "slot") &&
         ok(c, cudaMemcpyAsync(np, nptr.data(), sizeof(int) * (nnd + 1), cudaMemcpyHostToDevice, s), "np") &&
         ok(c, cudaMemcpyAsync(nl, nlist.data(), sizeof(int) * nip, cudaMemcpyHostToDevice, s), "nl") &&
         ok(c, cudaMemcpyAsync(rp, t->rowptr.data(), sizeof(int) * (nnd + 1), cudaMemcpyHostToDevice, s), "rp") &&
         ok(c, cudaMemcpyAsync(cl, col.data(), sizeof(int) * d.nnzb, cudaMemcpyHostToDevice, s), "col") &&
         ok(c, cudaMemcpyAsync(cp, cptr.data(), sizeof(int) * (d.nnzb + 1), cudaMemcpyHostToDevice, s), "cp") &&
         ok(c, cudaMemcpyAsync(ct, contrib.data(), sizeof(int) * nip * 8, cudaMemcpyHostToDevice, s), "ct") &&
         ok(c, cudaStreamSynchronize(s), "template sync");
  int st = good ? TG_OK : TG_ERR_CUDA;
  d.X = X;
  d.conn = cn;
  d.block = bk;
  d.mask = mk;
  d.eq_slot = es;
  d.nptr = np;
  d.nlist = nl;
  d.rowptr = rp;
  d.col = cl;
  d.cptr = cp;
  d.contrib = ct;
  if (!st) st = tile_template(c, t, c->spmv_tile_blocks);
  if (st) {
    release(c, t);
    delete t;
    return st;
  }
  *template_id = (int)c->templates.size();
  c->templates.push_back(t);
  c->tpl_elems += nel;
  return TG_OK;
}

int tg_mesh_compose(tg_context* c, int count, const int* template_ids) {
  if (!c || count <= 0 || !template_ids) return TG_ERR_ARG;
  if (count > 65535) {
    c->err = "at most 65535 instances per composed mesh";
    return TG_ERR_CAPACITY;
  }
  const int ntpl = (int)c->templates.size();
  for (int i = 0; i < count; ++i)
    if (template_ids[i] < 0 || template_ids[i] >= ntpl) return TG_ERR_ARG;
  if (set_dev(c)) return TG_ERR_CUDA;
  // templates tiled for another tile size are re-tiled first
  for (int i = 0; i < count; ++i) {
    MeshTemplate* t = c->templates[template_ids[i]];
    if (t->tile_blocks != c->spmv_tile_blocks) {
      const int s = tile_template(c, t, c->spmv_tile_blocks);
      if (s) return s;
    }
  }
  std::vector<InstDev> inst(count);
  long long nnd = 0, nel = 0, neq = 0, nnzb = 0, ntiles = 0;
  for (int i = 0; i < count; ++i) {
    const MeshTemplate* t = c->templates[template_ids[i]];
    inst[i] = InstDev{template_ids[i], (int)nnd, (int)nel, (int)neq, (int)nnzb, (int)ntiles};
    nnd += t->dev.nnd;
    nel += t->dev.nel;
    neq += t->dev.neq;
    nnzb += t->dev.nnzb;
    ntiles += (long long)t->tile_row.size() - 1;
    if (nel * 64 >= (1LL << 31) || nnzb >= (1LL << 31) || nnd >= (1LL << 29)) {
      c->err = "composed mesh too large for 32-bit indices";
      return TG_ERR_CAPACITY;
    }
  }
  int s = alloc_mesh(c, (int)nnd, (int)nel, (int)neq, nnzb);
  if (s) return s;
  c->composed = true;
  c->h_inst_tpl.assign(template_ids, template_ids + count);
  // row tiles and storage offsets: the instances' own tiles, concatenated
  std::vector<int> tile_row;
  tile_row.reserve(ntiles + 1);
  c->h_blob_off32.assign(ntiles + 1, 0);
  c->h_blob_off64.assign(ntiles + 1, 0);
  c->blob_cap32 = c->blob_cap64 = 0;
  long long k = 0;
  for (int i = 0; i < count; ++i) {
    const MeshTemplate* t = c->templates[template_ids[i]];
    for (size_t j = 0; j + 1 < t->tile_row.size(); ++j, ++k) {
      tile_row.push_back(t->tile_row[j] + inst[i].node_off);
      c->h_blob_off32[k + 1] = c->h_blob_off32[k] + t->tile_b32[j];
      c->h_blob_off64[k + 1] = c->h_blob_off64[k] + t->tile_b64[j];
      c->blob_cap32 = std::max(c->blob_cap32, t->tile_b32[j]);
      c->blob_cap64 = std::max(c->blob_cap64, t->tile_b64[j]);
    }
  }
  tile_row.push_back((int)nnd);
  c->ntiles = (int)ntiles;
  c->h_tile_row = tile_row;
  std::vector<TplDev> tdev(ntpl);
  for (int j = 0; j < ntpl; ++j) tdev[j] = c->templates[j]->dev;
  TplDev* d_tpl = nullptr;
  InstDev* d_inst = nullptr;
  bool good = dalloc(c, &c->d_block, (size_t)nel) && dalloc(c, &c->d_tile_row, (size_t)ntiles + 1) &&
              dalloc(c, &c->d_row_tile, (size_t)nnd) && dalloc(c, &c->d_blob_off32, (size_t)ntiles + 1) &&
              dalloc(c, &c->d_blob_off64, (size_t)ntiles + 1) && dalloc(c, &c->d_seg_node, (size_t)count + 1) &&
              dalloc(c, &c->d_seg_elem, (size_t)count + 1) && dalloc(c, &c->d_seg_out, (size_t)count * 9) &&
              dalloc(c, &c->d_elem_src, (size_t)nel) &&
              dalloc(c, &d_tpl, (size_t)ntpl) && dalloc(c, &d_inst, (size_t)count);
  if (!good) return TG_ERR_OOM;
  cudaStream_t st = c->stream;
  good = ok(c, cudaMemcpyAsync(c->d_tile_row, tile_row.data(), sizeof(int) * (ntiles + 1), cudaMemcpyHostToDevice, st), "tiles") &&
         ok(c, cudaMemcpyAsync(c->d_blob_off32, c->h_blob_off32.data(), sizeof(long long) * (ntiles + 1), cudaMemcpyHostToDevice, st), "off") &&
         ok(c, cudaMemcpyAsync(c->d_blob_off64, c->h_blob_off64.data(), sizeof(long long) * (ntiles + 1), cudaMemcpyHostToDevice, st), "off") &&
         ok(c, cudaMemcpyAsync(d_tpl, tdev.data(), sizeof(TplDev) * ntpl, cudaMemcpyHostToDevice, st), "tpl") &&
         ok(c, cudaMemcpyAsync(d_inst, inst.data(), sizeof(InstDev) * count, cudaMemcpyHostToDevice, st), "inst");
  if (!good) return TG_ERR_CUDA;
  ComposeOut o{c->d_X, c->d_conn, c->d_block, c->d_mask, c->d_eq_slot, c->d_node_elem_ptr, c->d_node_elem,
               c->d_rowptr, c->d_col, c->d_contrib_ptr, c->d_contrib, c->d_row_tile, c->d_seg_node, c->d_seg_elem,
               c->d_elem_src, (int)nnd, (int)nel, (int)nnzb};
  compose_kernel<<<dim3(8, count), 256, 0, st>>>(d_tpl, d_inst, count, o);
  c->launches++;
  if (!ok(c, cudaGetLastError(), "compose_kernel")) return TG_ERR_CUDA;
  dfree(c, d_tpl);
  dfree(c, d_inst);
  c->have_blocks = true;
  c->nseg = count;
  c->h_seg_node.resize(count + 1);
  c->h_seg_elem.resize(count + 1);
  for (int i = 0; i < count; ++i) {
    c->h_seg_node[i] = inst[i].node_off;
    c->h_seg_elem[i] = inst[i].elem_off;
  }
  c->h_seg_node[count] = (int)nnd;
  c->h_seg_elem[count] = (int)nel;
  return ok(c, cudaStreamSynchronize(st), "compose sync") ? TG_OK : TG_ERR_CUDA;
}

int tg_set_affine_prescribed(tg_context* c, const double* F) {
  if (!c || !F || c->nnd <= 0 || c->nseg <= 0) return TG_ERR_ARG;
  if (set_dev(c)) return TG_ERR_CUDA;
  double* d_F = nullptr;
  if (!ok(c, cudaMallocAsync((void**)&d_F, sizeof(double) * 9 * c->nseg, c->stream), "alloc")) return TG_ERR_OOM;
  int s = ok(c, cudaMemcpyAsync(d_F, F, sizeof(double) * 9 * c->nseg, cudaMemcpyHostToDevice, c->stream), "F")
              ? launch_affine_prescribed(c, d_F)
              : TG_ERR_CUDA;
  cudaFreeAsync(d_F, c->stream);
  if (!ok(c, cudaStreamSynchronize(c->stream), "sync") && !s) s = TG_ERR_CUDA;
  return s;
}

}  // extern "C"
