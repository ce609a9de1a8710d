// C ABI of the tahoe_gb300 library: context, mesh/equation set-up, state and
// load management, and the Newton driver (NLSolver equivalent) over the
// device kernels.  Host code only; kernels live in the .cu files.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "tg_internal.h"

namespace tg {

bool ok(Context* c, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  c->err = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}

void dfree(Context* c, void* p) {
  if (!p) return;
  cudaFreeAsync(p, c->stream);
  auto it = std::find(c->allocations.begin(), c->allocations.end(), p);
  if (it != c->allocations.end()) c->allocations.erase(it);
}

namespace {

// Device buffers go back to the stream-ordered pool; pinned host buffers are
// released only with the context (freeing pinned memory can synchronise the
// device).
void free_device(Context* c) {
  // the caller's timer events outlive mesh changes (a timed region may
  // cover composing a batch mesh)
  seg_free(c);
  cg_free(c);
  c->d_u_ckpt = c->d_R_ckpt = nullptr;
  c->ckpt_valid = false;
  if (c->pcg_graph) cudaGraphExecDestroy(c->pcg_graph);
  c->pcg_graph = nullptr;
  for (void* p : c->allocations) cudaFreeAsync(p, c->stream);
  c->allocations.clear();
}

void free_all(Context* c) {
  seg_free(c);
  cg_free(c);
  if (c->ev_a) cudaEventDestroy(c->ev_a);
  if (c->ev_b) cudaEventDestroy(c->ev_b);
  c->ev_a = c->ev_b = nullptr;
  for (cudaEvent_t& e : c->ev_poll) {
    if (e) cudaEventDestroy(e);
    e = nullptr;
  }
  c->d_u_ckpt = c->d_R_ckpt = nullptr;
  c->ckpt_valid = false;
  if (c->pcg_graph) cudaGraphExecDestroy(c->pcg_graph);
  c->pcg_graph = nullptr;
  for (void* p : c->allocations) cudaFreeAsync(p, c->stream);
  c->allocations.clear();
  free_templates(c);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->h_pcg) cudaFreeHost(c->h_pcg);
  if (c->h_resid) cudaFreeHost(c->h_resid);
  if (c->h_status) cudaFreeHost(c->h_status);
  c->h_pcg = nullptr;
  c->h_resid = nullptr;
  c->h_status = nullptr;
}

int set_device(Context* c) { return ok(c, cudaSetDevice(c->device), "cudaSetDevice") ? TG_OK : TG_ERR_CUDA; }

// read back the device status word and residual norm; clears the status
int sync_status(Context* c) {
  if (!ok(c, cudaMemcpyAsync(c->h_status, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "status"))
    return TG_ERR_CUDA;
  if (!ok(c, cudaStreamSynchronize(c->stream), "sync")) return TG_ERR_CUDA;
  const int st = *c->h_status;
  if (st) {
    cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream);
    if (st & kStatusBadJacobian) {
      c->err = "non-positive Jacobian determinant";
      return TG_ERR_BAD_JACOBIAN;
    }
    c->err = "non-finite value";
    return TG_ERR_NAN;
  }
  return TG_OK;
}

bool valid_material(int kind, const double* p, int np, MatParams& m) {
  std::memset(&m, 0, sizeof(m));
  m.kind = kind;
  auto set_E_nu = [&](double E, double nu) {  // IsotropicT::Set_E_nu (IsotropicT.cpp:32-44)
    if (E < 0.0 || nu > 0.5 || nu < -1.0) return false;
    m.mu = 0.5 * E / (1.0 + nu);
    m.lambda = 2.0 * m.mu * nu / (1.0 - 2.0 * nu);
    m.kappa = m.lambda + 2.0 / 3.0 * m.mu;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) m.C[i * 6 + j] = m.lambda + (i == j ? 2.0 * m.mu : 0.0);
    for (int i = 3; i < 6; ++i) m.C[i * 6 + i] = m.mu;
    return true;
  };
  switch (kind) {
    case TG_MAT_SS_HOOKEAN:
      if (np == 36) {
        std::memcpy(m.C, p, sizeof(m.C));
        return true;
      }
      return np == 2 && set_E_nu(p[0], p[1]);
    case TG_MAT_SS_J2:
      if (np < 4 || !set_E_nu(p[0], p[1])) return false;
      m.hard_a = p[2];
      m.hard_b = p[3];
      m.elastic_its = np > 4 ? (int)p[4] : 0;
      return true;
    case TG_MAT_FS_SIMO:  // IsotropicT::Set_mu_kappa (IsotropicT.cpp:46-57)
      if (np != 2 || p[0] < 0.0 || p[1] < 0.0) return false;
      m.mu = p[0];
      m.kappa = p[1];
      return true;
    case TG_MAT_FS_STVENANT:
      return np == 2 && set_E_nu(p[0], p[1]);
    default:
      return false;
  }
}

}  // namespace

// Active-dof bits per node and the node*4+dof slot of every equation; the
// equation numbers must be 1..neq in node-major / dof-minor order (prescribed
// dofs <= 0).  Returns neq, or -1 with the context error set.
int equation_slots(Context* c, int nnd, const int* eqnos, std::vector<uint8_t>& mask, std::vector<int>& slot) {
  int neq = 0;
  mask.assign(nnd, 0);
  slot.clear();
  for (int n = 0; n < nnd; ++n)
    for (int d = 0; d < 3; ++d) {
      const int q = eqnos[n * 3 + d];
      if (q > 0) {
        if (q != neq + 1) {
          c->err = "equation numbers must be ascending node-major from 1";
          return -1;
        }
        ++neq;
        mask[n] |= (uint8_t)(1u << d);
        slot.push_back(n * 4 + d);
      }
    }
  return neq;
}

// Releases the current mesh (buffers back to the pool) and allocates every
// per-mesh device array for the given sizes, with the state zeroed: nodal
// vectors, status words, J2 history (flags unallocated), padded index tails.
int alloc_mesh(Context* c, int nnd, int nel, int neq, long long nnzb) {
  cudaStreamSynchronize(c->stream);
  free_device(c);
  c->pcg_vec_precision = -1;
  c->pcg_graph_key = -1;
  c->tangent_precision = -1;
  c->d_x = c->d_r = c->d_z = c->d_p = c->d_q = nullptr;
  c->d_cg_s = nullptr;
  c->cg_s_precision = -1;
  c->d_Ke32 = nullptr;
  c->d_Ke64 = nullptr;
  c->d_geo = nullptr;
  c->d_geo_ff = nullptr;
  c->d_elem_src = nullptr;
  c->d_xyz = nullptr;
  c->d_blob32 = c->d_blob64 = nullptr;
  c->nseg = 0;
  c->d_seg_node = c->d_seg_elem = nullptr;
  c->d_seg_out = nullptr;
  c->h_seg_node.clear();
  c->h_seg_elem.clear();
  c->d_blob_off32 = c->d_blob_off64 = nullptr;
  c->d_row_tile = nullptr;
  c->d_tile_row = nullptr;
  c->sym = SymStore{};  // its buffers went back to the pool with the mesh
  c->push = PushStore{};
  c->d_minv32 = nullptr;
  c->d_minv64 = nullptr;
  c->d_block = nullptr;
  c->have_blocks = false;
  c->have_du = false;
  c->composed = false;
  c->h_conn.clear();
  c->h_eqnos.clear();
  c->h_coords.clear();
  c->h_eq_slot.clear();
  c->h_rowptr.clear();
  c->h_col.clear();
  c->nnd = nnd;
  c->nel = nel;
  c->neq = neq;
  c->nnzb = nnzb;
  c->nnzb_pad = (nnzb + 31) / 32 * 32;
  const size_t nip = (size_t)nel * 8;
  const size_t rp_len = (size_t)(nnd + 1 + 3) / 4 * 4 + 4;
  bool good = dalloc(c, &c->d_X, (size_t)nnd * 3) && dalloc(c, &c->d_conn, nip) &&
              dalloc(c, &c->d_mask, (size_t)nnd) && dalloc(c, &c->d_eq_slot, (size_t)std::max(neq, 1)) &&
              dalloc(c, &c->d_node_elem_ptr, (size_t)nnd + 1) && dalloc(c, &c->d_node_elem, nip) &&
              dalloc(c, &c->d_rowptr, rp_len) && dalloc(c, &c->d_col, (size_t)c->nnzb_pad) &&
              dalloc(c, &c->d_contrib_ptr, (size_t)nnzb + 1) && dalloc(c, &c->d_contrib, nip * 8) &&
              dalloc(c, &c->d_u, (size_t)nnd) && dalloc(c, &c->d_fext, (size_t)nnd) && dalloc(c, &c->d_R, (size_t)nnd) &&
              dalloc(c, &c->d_fint, nip) && dalloc(c, &c->d_status, 1) && dalloc(c, &c->d_resid, 1) &&
              dalloc(c, &c->d_pcg, 2);  // [1]: next state of the single-reduction PCG
  c->partials_cap = 4096;
  good = good && dalloc(c, &c->d_partials, (size_t)c->partials_cap * 2);
  good = good && dalloc(c, &c->d_j2_flags, nip) && dalloc(c, &c->d_j2_alloc, (size_t)nel) &&
         dalloc(c, &c->d_j2_alpha, nip) && dalloc(c, &c->d_j2_dgamma, nip) && dalloc(c, &c->d_j2_norm, nip) &&
         dalloc(c, &c->d_j2_epsp, nip * 6) && dalloc(c, &c->d_j2_nhat, nip * 6);
  if (!good) return TG_ERR_OOM;
  cudaStream_t s = c->stream;
  good = ok(c, cudaMemsetAsync(c->d_rowptr, 0, sizeof(int) * rp_len, s), "rp") &&
         ok(c, cudaMemsetAsync(c->d_col, 0, sizeof(int) * c->nnzb_pad, s), "col") &&
         ok(c, cudaMemsetAsync(c->d_u, 0, sizeof(double4_32a) * nnd, s), "u") &&
         ok(c, cudaMemsetAsync(c->d_fext, 0, sizeof(double4_32a) * nnd, s), "f") &&
         ok(c, cudaMemsetAsync(c->d_R, 0, sizeof(double4_32a) * nnd, s), "R") &&
         ok(c, cudaMemsetAsync(c->d_status, 0, sizeof(int), s), "st") &&
         ok(c, cudaMemsetAsync(c->d_resid, 0, sizeof(ResidScalars), s), "rs") &&
         ok(c, cudaMemsetAsync(c->d_pcg, 0, 2 * sizeof(PcgScalars), s), "pcg") &&
         ok(c, cudaMemsetAsync(c->d_j2_flags, TG_J2_UNALLOCATED, nip, s), "fl") &&
         ok(c, cudaMemsetAsync(c->d_j2_alloc, 0, nel, s), "al") &&
         ok(c, cudaMemsetAsync(c->d_j2_alpha, 0, sizeof(double) * nip, s), "a") &&
         ok(c, cudaMemsetAsync(c->d_j2_dgamma, 0, sizeof(double) * nip, s), "dg") &&
         ok(c, cudaMemsetAsync(c->d_j2_norm, 0, sizeof(double) * nip, s), "nr") &&
         ok(c, cudaMemsetAsync(c->d_j2_epsp, 0, sizeof(double) * nip * 6, s), "ep") &&
         ok(c, cudaMemsetAsync(c->d_j2_nhat, 0, sizeof(double) * nip * 6, s), "nh");
  return good ? TG_OK : TG_ERR_CUDA;
}

}  // namespace tg

using namespace tg;


extern "C" {

int tg_create(tg_context** out, int device) {
  if (!out) return TG_ERR_ARG;
  *out = nullptr;
  tg_context* c = new tg_context();
  c->device = device;
  c->mats.nblocks = 1;
  c->mats.formulation = TG_SMALL_STRAIN;
  // keep freed device memory in the stream-ordered pool for reuse
  if (!set_device(c)) {
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
      unsigned long long keep = ~0ULL;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
  }
  if (set_device(c) ||
      !ok(c, cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device), "multiprocessor count") ||
      !ok(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream") ||
      !ok(c, cudaMallocHost((void**)&c->h_pcg, 2 * sizeof(PcgScalars)), "pinned") ||
      !ok(c, cudaEventCreateWithFlags(&c->ev_poll[0], cudaEventDisableTiming), "event") ||
      !ok(c, cudaEventCreateWithFlags(&c->ev_poll[1], cudaEventDisableTiming), "event") ||
      !ok(c, cudaMallocHost((void**)&c->h_resid, sizeof(ResidScalars)), "pinned") ||
      !ok(c, cudaMallocHost((void**)&c->h_status, sizeof(int)), "pinned")) {
    free_all(c);
    delete c;
    return TG_ERR_CUDA;
  }
  *out = c;
  return TG_OK;
}

int tg_destroy(tg_context* c) {
  if (!c) return TG_ERR_ARG;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_all(c);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return TG_OK;
}

const char* tg_last_error(const tg_context* c) { return c ? c->err.c_str() : "null context"; }
long long tg_launch_count(const tg_context* c) { return c ? c->launches : 0; }

int tg_mesh_upload(tg_context* c, int nnd, const double* coords, int nel, const int* conn, const int* eqnos) {
  if (!c || nnd <= 0 || nel <= 0 || !coords || !conn || !eqnos) return TG_ERR_ARG;
  if ((long long)nel * 64 >= (1LL << 31)) {
    c->err = "too many elements for the 32-bit contribution map";
    return TG_ERR_CAPACITY;
  }
  for (long long k = 0; k < (long long)nel * 8; ++k)
    if (conn[k] < 0 || conn[k] >= nnd) {
      c->err = "connectivity out of range";
      return TG_ERR_ARG;
    }
  std::vector<uint8_t> mask;
  std::vector<int> slot;
  const int neq = equation_slots(c, nnd, eqnos, mask, slot);
  if (neq < 0) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  std::vector<int> rowptr, col, cptr, contrib, nptr, nlist;
  build_block_pattern(nnd, nel, conn, rowptr, col);
  build_contrib_map(nnd, nel, conn, rowptr, col, cptr, contrib);
  build_node_elem(nnd, nel, conn, nptr, nlist);
  int s = alloc_mesh(c, nnd, nel, neq, rowptr[nnd]);
  if (s) return s;
  c->h_conn.assign(conn, conn + (size_t)nel * 8);
  c->h_eqnos.assign(eqnos, eqnos + (size_t)nnd * 3);
  c->h_coords.assign(coords, coords + (size_t)nnd * 3);
  c->h_eq_slot = slot;
  c->h_rowptr.swap(rowptr);
  c->h_col.swap(col);
  const size_t nip = (size_t)nel * 8;
  cudaStream_t st = c->stream;
  const bool good =
      ok(c, cudaMemcpyAsync(c->d_X, coords, sizeof(double) * nnd * 3, cudaMemcpyHostToDevice, st), "X") &&
      ok(c, cudaMemcpyAsync(c->d_conn, conn, sizeof(int) * nip, cudaMemcpyHostToDevice, st), "conn") &&
      ok(c, cudaMemcpyAsync(c->d_mask, mask.data(), nnd, cudaMemcpyHostToDevice, st), "mask") &&
      ok(c, cudaMemcpyAsync(c->d_eq_slot, slot.data(), sizeof(int) * neq, cudaMemcpyHostToDevice, st), "slot") &&
      ok(c, cudaMemcpyAsync(c->d_node_elem_ptr, nptr.data(), sizeof(int) * (nnd + 1), cudaMemcpyHostToDevice, st), "np") &&
      ok(c, cudaMemcpyAsync(c->d_node_elem, nlist.data(), sizeof(int) * nip, cudaMemcpyHostToDevice, st), "nl") &&
      ok(c, cudaMemcpyAsync(c->d_rowptr, c->h_rowptr.data(), sizeof(int) * (nnd + 1), cudaMemcpyHostToDevice, st), "rp") &&
      ok(c, cudaMemcpyAsync(c->d_col, c->h_col.data(), sizeof(int) * c->nnzb, cudaMemcpyHostToDevice, st), "col") &&
      ok(c, cudaMemcpyAsync(c->d_contrib_ptr, cptr.data(), sizeof(int) * (c->nnzb + 1), cudaMemcpyHostToDevice, st), "cp") &&
      ok(c, cudaMemcpyAsync(c->d_contrib, contrib.data(), sizeof(int) * nip * 8, cudaMemcpyHostToDevice, st), "ct") &&
      ok(c, cudaStreamSynchronize(st), "upload sync");
  if (!good) return TG_ERR_CUDA;
  return build_tiles(c, c->spmv_tile_blocks);
}

}  // extern "C"

namespace tg {
// Row tiles of the streamed SpMV and the byte offsets of every tile in the
// tile-contiguous matrix storage of each precision.  Any existing matrix
// storage is dropped (its layout changes).
//
// The persistent product grid of G CTAs takes tiles t, t + G, ...: tiles
// cut greedily (consecutive rows holding at most tile_blocks block
// nonzeros) leave some CTAs one tile more than others, and the whole
// product waits for them.  So the rows are cut into exactly k G tiles of
// equal block count (k the smallest count keeping tiles within
// tile_blocks, cut at the row boundary nearest each share), which gives
// every CTA k tiles of the same size -- unless that tiling no longer fits
// G CTAs (a larger largest tile) or the mesh has too few rows, where the
// greedy tiles stay.
namespace {
struct TileSet {
  std::vector<int> start;  // first row of each tile, then nnd
  long long cap32 = 0, cap64 = 0;
};
TileSet tile_set(const Context* c, const std::vector<int>& start) {
  TileSet ts;
  ts.start = start;
  for (size_t t = 0; t + 1 < start.size(); ++t) {
    const int nrows = start[t + 1] - start[t];
    const int nb = c->h_rowptr[start[t + 1]] - c->h_rowptr[start[t]];
    ts.cap32 = std::max(ts.cap32, blob_tile_bytes(nrows, nb, 4));
    ts.cap64 = std::max(ts.cap64, blob_tile_bytes(nrows, nb, 8));
  }
  return ts;
}
}  // namespace

int build_tiles(Context* c, int tile_blocks) {
  if (ensure_host_mesh(c)) return TG_ERR_CUDA;
  std::vector<int> greedy(1, 0);
  for (int r = 0; r < c->nnd; ++r)
    if (r > greedy.back() && c->h_rowptr[r + 1] - c->h_rowptr[greedy.back()] > tile_blocks) greedy.push_back(r);
  greedy.push_back(c->nnd);
  TileSet ts = tile_set(c, greedy);
  const long long nnzb = c->h_rowptr[c->nnd];
  const int G = spmv_grid_for(c, ts.cap32);
  if (G > 0 && nnzb > 0) {
    const long long k = (nnzb + (long long)G * tile_blocks - 1) / ((long long)G * tile_blocks);
    const long long parts = k * G;
    if (parts <= c->nnd) {
      std::vector<int> bal(1, 0);
      for (long long j = 1; j < parts; ++j) {
        const long long target = (j * nnzb + parts / 2) / parts;
        int r = (int)(std::lower_bound(c->h_rowptr.begin(), c->h_rowptr.begin() + c->nnd + 1, (int)target) -
                      c->h_rowptr.begin());
        if (r > 0 && target - c->h_rowptr[r - 1] < c->h_rowptr[r] - target) --r;
        if (r > bal.back() && r < c->nnd) bal.push_back(r);
      }
      bal.push_back(c->nnd);
      TileSet tb = tile_set(c, bal);
      if ((long long)bal.size() - 1 == parts && spmv_grid_for(c, tb.cap32) == G) ts = tb;
    }
  }
  const std::vector<int>& tiles = ts.start;
  const int nt = (int)tiles.size() - 1;
  std::vector<int> row_tile(c->nnd);
  c->h_blob_off32.assign(nt + 1, 0);
  c->h_blob_off64.assign(nt + 1, 0);
  c->blob_cap32 = ts.cap32;
  c->blob_cap64 = ts.cap64;
  for (int t = 0; t < nt; ++t) {
    const int nrows = tiles[t + 1] - tiles[t];
    const int nb = c->h_rowptr[tiles[t + 1]] - c->h_rowptr[tiles[t]];
    for (int r = tiles[t]; r < tiles[t + 1]; ++r) row_tile[r] = t;
    c->h_blob_off32[t + 1] = c->h_blob_off32[t] + blob_tile_bytes(nrows, nb, 4);
    c->h_blob_off64[t + 1] = c->h_blob_off64[t] + blob_tile_bytes(nrows, nb, 8);
  }
  for (void** p : {(void**)&c->d_tile_row, (void**)&c->d_row_tile, (void**)&c->d_blob_off32,
                   (void**)&c->d_blob_off64, (void**)&c->d_blob32, (void**)&c->d_blob64}) {
    if (*p) dfree(c, *p);
    *p = nullptr;
  }
  c->tangent_precision = -1;  // values must be assembled into the new layout
  c->ntiles = nt;
  c->h_tile_row = tiles;
  c->spmv_tile_blocks = tile_blocks;
  if (!dalloc(c, &c->d_tile_row, tiles.size()) || !dalloc(c, &c->d_row_tile, (size_t)c->nnd) ||
      !dalloc(c, &c->d_blob_off32, (size_t)nt + 1) || !dalloc(c, &c->d_blob_off64, (size_t)nt + 1))
    return TG_ERR_OOM;
  cudaStream_t st = c->stream;
  if (!ok(c, cudaMemcpyAsync(c->d_tile_row, tiles.data(), sizeof(int) * tiles.size(), cudaMemcpyHostToDevice, st), "tiles") ||
      !ok(c, cudaMemcpyAsync(c->d_row_tile, row_tile.data(), sizeof(int) * c->nnd, cudaMemcpyHostToDevice, st), "rows") ||
      !ok(c, cudaMemcpyAsync(c->d_blob_off32, c->h_blob_off32.data(), sizeof(long long) * (nt + 1), cudaMemcpyHostToDevice, st),
          "off") ||
      !ok(c, cudaMemcpyAsync(c->d_blob_off64, c->h_blob_off64.data(), sizeof(long long) * (nt + 1), cudaMemcpyHostToDevice, st),
          "off") ||
      !ok(c, cudaStreamSynchronize(st), "sync"))
    return TG_ERR_CUDA;
  drop_graphs(c);  // the captured iterations bake in the launch shape
  return TG_OK;
}

void drop_graphs(Context* c) {
  cg_free(c);
  if (c->pcg_graph) cudaGraphExecDestroy(c->pcg_graph);
  c->pcg_graph = nullptr;
  c->pcg_graph_key = -1;
  if (c->seg.graph) cudaGraphExecDestroy(c->seg.graph);
  c->seg.graph = nullptr;
  c->seg.graph_key = -1;
}

// Allocates the matrix storage of one precision and writes its structure
// (headers, local row pointers, column indices); the value planes are filled
// by the assembly.
int ensure_blob(Context* c, int precision) {
  unsigned char** blob = precision == TG_MIXED ? &c->d_blob32 : &c->d_blob64;
  if (*blob) return TG_OK;
  const std::vector<long long>& off = precision == TG_MIXED ? c->h_blob_off32 : c->h_blob_off64;
  const long long total = off[c->ntiles];
  if (!dalloc(c, blob, (size_t)total)) return TG_ERR_OOM;
  if (!ok(c, cudaMemsetAsync(*blob, 0, (size_t)total, c->stream), "blob")) return TG_ERR_CUDA;
  return launch_blob_structure(c, precision);
}
}  // namespace tg

extern "C" {

int tg_spmv_config(tg_context* c, int tile_blocks, int stages) {
  if (!c || tile_blocks < 32 || tile_blocks > 16384 || stages < 2 || stages > 3) return TG_ERR_ARG;
  c->spmv_stages = stages;
  if (c->nnd <= 0) {
    c->spmv_tile_blocks = tile_blocks;
    return TG_OK;
  }
  if (cudaSetDevice(c->device) != cudaSuccess) return TG_ERR_CUDA;
  return build_tiles(c, tile_blocks);
}

int tg_spmv_release(tg_context* c, int per_warp) {
  if (!c || (per_warp != 0 && per_warp != 1)) return TG_ERR_ARG;
  c->spmv_warp_release = per_warp;
  drop_graphs(c);  // the captured iterations bake in the kernel
  return TG_OK;
}

int tg_pcg_form(tg_context* c, int form) {
  if (!c || form < -1 || form > 3) return TG_ERR_ARG;
  c->pcg_form = form == 0 ? 0 : 1;
  const int pdl = form == 2 ? 0 : 1;
  const int push = form == 3 ? 1 : form == -1 ? -1 : 0;
  if (pdl != c->cg_pdl || push != c->cg_push) {
    c->cg_pdl = pdl;
    c->cg_push = push;
    drop_graphs(c);  // the captured chunk bakes in its launch dependencies and storage
  }
  return TG_OK;
}

int tg_pcg_form_get(const tg_context* c, int* form) {
  if (!c || !form) return TG_ERR_ARG;
  if (c->pcg_form == 0)
    *form = 0;
  else if (!c->cg_pdl)
    *form = 2;
  else
    *form = push_active(c) ? 3 : 1;
  return TG_OK;
}

int tg_spmv_l2_keep(tg_context* c, long long bytes) {
  if (!c || bytes < -1) return TG_ERR_ARG;
  c->l2_keep = bytes;
  drop_graphs(c);  // the captured iterations bake in the tiles kept
  return TG_OK;
}

int tg_spmv_symmetric(tg_context* c, int on, int tile_blocks) {
  if (!c || on < 0 || on > 3 || (tile_blocks != 0 && (tile_blocks < 32 || tile_blocks > 4096))) return TG_ERR_ARG;
  if (c->nnd > 0 && cudaSetDevice(c->device) != cudaSuccess) return TG_ERR_CUDA;
  c->sym_mode = on;
  if (tile_blocks) c->sym_tile_blocks = tile_blocks;
  drop_graphs(c);  // the captured iterations bake in the product
  // values of the current tangent in the (re-)built format, converted from
  // the full storage (assembled first when the tangent went to the push
  // storage only)
  if (sym_active(c) && c->tangent_precision >= 0) {
    const int s = ensure_full_assembly(c);
    return s ? s : sym_convert(c, c->tangent_precision);
  }
  return TG_OK;
}

int tg_segment_solver(tg_context* c, int per_rve) {
  if (!c || (per_rve != 0 && per_rve != 1)) return TG_ERR_ARG;
  c->seg_pcg_mode = per_rve;
  return TG_OK;
}

int tg_tangent_config(tg_context* c, int elems_per_block) {
  if (!c || (elems_per_block != 2 && elems_per_block != 4 && elems_per_block != 8)) return TG_ERR_ARG;
  c->tangent_epb = elems_per_block;
  return TG_OK;
}

int tg_tuning_get(const tg_context* c, int* tile_blocks, int* stages, int* tangent_elems_per_block) {
  if (!c) return TG_ERR_ARG;
  if (tile_blocks) *tile_blocks = c->spmv_tile_blocks;
  if (stages) *stages = c->spmv_stages;
  if (tangent_elems_per_block) *tangent_elems_per_block = c->tangent_epb;
  return TG_OK;
}

int tg_element_strain_displacement(tg_context* c, int option) {
  if (!c || (option != TG_STRAIN_STANDARD && option != TG_STRAIN_BBAR)) return TG_ERR_ARG;
  c->mats.bbar = option == TG_STRAIN_BBAR;
  return TG_OK;
}

int tg_element_set(tg_context* c, int formulation) {
  if (!c || (formulation != TG_SMALL_STRAIN && formulation != TG_TOTAL_LAGRANGIAN &&
             formulation != TG_UPDATED_LAGRANGIAN))
    return TG_ERR_ARG;
  c->formulation = formulation;
  c->mats.formulation = formulation;
  return TG_OK;
}

int tg_material_set(tg_context* c, int block, int kind, const double* params, int np) {
  if (!c || block < 0 || block >= kMaxBlocks || !params) return TG_ERR_ARG;
  MatParams m;
  if (!valid_material(kind, params, np, m)) {
    c->err = "invalid material parameters";
    return TG_ERR_ARG;
  }
  c->mats.m[block] = m;
  c->mats.nblocks = std::max(c->mats.nblocks, block + 1);
  c->has_j2 = false;
  for (int b = 0; b < c->mats.nblocks; ++b) c->has_j2 |= c->mats.m[b].kind == TG_MAT_SS_J2;
  return TG_OK;
}

int tg_element_blocks(tg_context* c, const int* blocks) {
  if (!c || !blocks || c->nel <= 0) return TG_ERR_ARG;
  std::vector<int8_t> b(c->nel);
  for (int e = 0; e < c->nel; ++e) {
    if (blocks[e] < 0 || blocks[e] >= kMaxBlocks) return TG_ERR_ARG;
    b[e] = (int8_t)blocks[e];
  }
  if (set_device(c)) return TG_ERR_CUDA;
  if (!c->d_block && !dalloc(c, &c->d_block, (size_t)c->nel)) return TG_ERR_OOM;
  c->have_blocks = true;
  return ok(c, cudaMemcpyAsync(c->d_block, b.data(), c->nel, cudaMemcpyHostToDevice, c->stream), "blocks") &&
                 ok(c, cudaStreamSynchronize(c->stream), "sync")
             ? TG_OK
             : TG_ERR_CUDA;
}

int tg_sizes(const tg_context* c, int* neq, long long* nnzb) {
  if (!c) return TG_ERR_ARG;
  if (neq) *neq = c->neq;
  if (nnzb) *nnzb = c->nnzb;
  return TG_OK;
}

// Scalar expansion of the block pattern over active equations.
int tg_pattern_build(tg_context* c, int upper_only, int* row_ptr, int* col_idx, long long* nnz) {
  if (!c || c->nnd <= 0) return TG_ERR_ARG;
  if (set_device(c) || ensure_host_mesh(c)) return TG_ERR_CUDA;
  expand_pattern(c->nnd, c->h_eqnos.data(), c->h_rowptr, c->h_col, upper_only != 0, row_ptr, col_idx, nnz);
  return TG_OK;
}

// The same structure from the mesh alone, on the host (no context, no GPU):
// the node-block pattern tg_mesh_upload builds, expanded the same way.
int tg_pattern_build_host(int nnd, int nel, const int* conn, const int* eqnos, int upper_only, int* row_ptr,
                          int* col_idx, long long* nnz) {
  if (nnd <= 0 || nel < 0 || !conn || !eqnos || !nnz) return TG_ERR_ARG;
  for (long long k = 0; k < (long long)nel * 8; ++k)
    if (conn[k] < 0 || conn[k] >= nnd) return TG_ERR_ARG;
  std::vector<int> rowptr, col;
  build_block_pattern(nnd, nel, conn, rowptr, col);
  expand_pattern(nnd, eqnos, rowptr, col, upper_only != 0, row_ptr, col_idx, nnz);
  return TG_OK;
}

// The caller's (x, y, z) array is copied as it is (directly by DMA when the
// caller's memory is pinned) into a device staging array and re-laid out
// into the padded nodal vector on the device.
int tg_set_displacement(tg_context* c, const double* u) {
  if (!c || !u || c->nnd <= 0) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  if (!c->d_xyz && !dalloc(c, &c->d_xyz, (size_t)c->nnd * 3)) return TG_ERR_OOM;
  if (!ok(c, cudaMemcpyAsync(c->d_xyz, u, sizeof(double) * 3 * c->nnd, cudaMemcpyHostToDevice, c->stream), "u"))
    return TG_ERR_CUDA;
  const int s = launch_xyz_to_nodal(c, c->d_xyz, c->d_u);
  if (s) return s;
  return ok(c, cudaStreamSynchronize(c->stream), "sync") ? TG_OK : TG_ERR_CUDA;
}

int tg_get_displacement(tg_context* c, double* u) {
  if (!c || !u || c->nnd <= 0) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  if (!c->d_xyz && !dalloc(c, &c->d_xyz, (size_t)c->nnd * 3)) return TG_ERR_OOM;
  const int s = launch_nodal_to_xyz(c, c->d_u, c->d_xyz);
  if (s) return s;
  return ok(c, cudaMemcpyAsync(u, c->d_xyz, sizeof(double) * 3 * c->nnd, cudaMemcpyDeviceToHost, c->stream), "u") &&
                 ok(c, cudaStreamSynchronize(c->stream), "sync")
             ? TG_OK
             : TG_ERR_CUDA;
}

int tg_set_prescribed(tg_context* c, int n, const int* idx, const double* val) {
  if (!c || n < 0 || (n > 0 && (!idx || !val))) return TG_ERR_ARG;
  if (n == 0) return TG_OK;
  for (int k = 0; k < n; ++k)
    if (idx[k] < 0 || idx[k] >= c->nnd * 3) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  int* d_idx = nullptr;
  double* d_val = nullptr;
  if (!ok(c, cudaMallocAsync((void**)&d_idx, sizeof(int) * n, c->stream), "alloc") ||
      !ok(c, cudaMallocAsync((void**)&d_val, sizeof(double) * n, c->stream), "alloc"))
    return TG_ERR_OOM;
  int s = TG_OK;
  if (!ok(c, cudaMemcpyAsync(d_idx, idx, sizeof(int) * n, cudaMemcpyHostToDevice, c->stream), "idx") ||
      !ok(c, cudaMemcpyAsync(d_val, val, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream), "val"))
    s = TG_ERR_CUDA;
  if (!s) s = launch_set_prescribed(c, n, d_idx, d_val);
  cudaFreeAsync(d_idx, c->stream);
  cudaFreeAsync(d_val, c->stream);
  if (!s && !ok(c, cudaStreamSynchronize(c->stream), "sync")) s = TG_ERR_CUDA;
  return s;
}

int tg_set_external_force(tg_context* c, const double* f) {
  if (!c || !f || c->nnd <= 0) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  std::vector<double4_32a> h(c->nnd);
  for (int n = 0; n < c->nnd; ++n) h[n] = make_double4_32a(f[n * 3], f[n * 3 + 1], f[n * 3 + 2], 0.0);
  return ok(c, cudaMemcpyAsync(c->d_fext, h.data(), sizeof(double4_32a) * c->nnd, cudaMemcpyHostToDevice, c->stream), "f") &&
                 ok(c, cudaStreamSynchronize(c->stream), "sync")
             ? TG_OK
             : TG_ERR_CUDA;
}

int tg_set_load_factor(tg_context* c, double factor) {
  if (!c) return TG_ERR_ARG;
  c->load_factor = factor;
  return TG_OK;
}

int tg_set_iteration(tg_context* c, int it) {
  if (!c) return TG_ERR_ARG;
  c->iteration = it;
  return TG_OK;
}

// HexahedronT::NodesOnFacet (HexahedronT.cpp:1913-1918) facet node lists and a
// 2x2 Gauss rule on each facet in the reference configuration.
int tg_traction_forces(int nnd, const double* X, int nel, const int* conn, int nf, const int* elem, const int* facet,
                       const double* t3, double* f) {
  static const int fn[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}};
  if (nnd <= 0 || nel <= 0 || !X || !conn || nf < 0 || (nf > 0 && (!elem || !facet || !t3)) || !f) return TG_ERR_ARG;
  const double g = 1.0 / std::sqrt(3.0);
  const double qr[4] = {-g, g, g, -g}, qs[4] = {-g, -g, g, g};
  const double nr[4] = {-1, 1, 1, -1}, ns[4] = {-1, -1, 1, 1};
  for (int k = 0; k < nf; ++k) {
    if (elem[k] < 0 || elem[k] >= nel || facet[k] < 0 || facet[k] > 5) return TG_ERR_ARG;
    int nodes[4];
    for (int i = 0; i < 4; ++i) nodes[i] = conn[elem[k] * 8 + fn[facet[k]][i]];
    for (int q = 0; q < 4; ++q) {
      double Na[4], dr[4], ds[4];
      for (int i = 0; i < 4; ++i) {
        Na[i] = 0.25 * (1 + qr[q] * nr[i]) * (1 + qs[q] * ns[i]);
        dr[i] = 0.25 * nr[i] * (1 + qs[q] * ns[i]);
        ds[i] = 0.25 * ns[i] * (1 + qr[q] * nr[i]);
      }
      double m1[3] = {0, 0, 0}, m2[3] = {0, 0, 0};
      for (int i = 0; i < 4; ++i)
        for (int d = 0; d < 3; ++d) {
          m1[d] += X[d * nnd + nodes[i]] * dr[i];
          m2[d] += X[d * nnd + nodes[i]] * ds[i];
        }
      const double n3[3] = {m1[1] * m2[2] - m1[2] * m2[1], m1[2] * m2[0] - m1[0] * m2[2], m1[0] * m2[1] - m1[1] * m2[0]};
      const double jw = std::sqrt(n3[0] * n3[0] + n3[1] * n3[1] + n3[2] * n3[2]);
      for (int i = 0; i < 4; ++i)
        for (int d = 0; d < 3; ++d) f[nodes[i] * 3 + d] += jw * t3[k * 3 + d] * Na[i];
    }
  }
  return TG_OK;
}

int tg_form_residual(tg_context* c, double* R_out, double* norm_out) {
  return tg_form_residual_precision(c, TG_FP64, R_out, norm_out);
}

int tg_form_residual_precision(tg_context* c, int precision, double* R_out, double* norm_out) {
  if (!c || c->nnd <= 0 || (precision != TG_FP64 && precision != TG_MIXED)) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  int s = launch_residual(c, precision == TG_MIXED ? kResidualDoubleFloat : kResidualFP64);
  if (s) return s;
  if (!ok(c, cudaMemcpyAsync(c->h_resid, c->d_resid, sizeof(ResidScalars), cudaMemcpyDeviceToHost, c->stream), "norm"))
    return TG_ERR_CUDA;
  double* d_eq = nullptr;
  if (R_out && c->neq > 0) {
    if (!ok(c, cudaMallocAsync((void**)&d_eq, sizeof(double) * c->neq, c->stream), "alloc")) return TG_ERR_OOM;
    s = launch_gather_eq(c, c->d_R, d_eq);
    if (!s && !ok(c, cudaMemcpyAsync(R_out, d_eq, sizeof(double) * c->neq, cudaMemcpyDeviceToHost, c->stream), "R"))
      s = TG_ERR_CUDA;
    cudaFreeAsync(d_eq, c->stream);
    if (s) return s;
  }
  s = sync_status(c);
  if (s) return s;
  const double n2 = c->h_resid->norm2;
  if (!std::isfinite(n2)) {
    c->err = "non-finite residual";
    return TG_ERR_NAN;
  }
  if (norm_out) *norm_out = std::sqrt(n2);
  return TG_OK;
}

int tg_form_tangent(tg_context* c, int precision) {
  if (!c || c->nnd <= 0 || (precision != TG_FP64 && precision != TG_MIXED)) return TG_ERR_ARG;
  if (set_device(c)) return TG_ERR_CUDA;
  return form_tangent(c, precision);
}

}  // extern "C"
