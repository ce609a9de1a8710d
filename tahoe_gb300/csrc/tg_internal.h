// Internal declarations shared by the host C++ and the CUDA translation units
// of the tahoe_gb300 library.  Nothing here is part of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tahoe_gb300.h"

namespace tg {

constexpr int kMaxBlocks = 4;      // material blocks per element group
constexpr int kSlots = 36;         // upper-triangle node-pair blocks of a hex8 element
// A staged 3x3 element block is three 4-value rows (the 4th value is zero
// padding), so a row is one 16-byte (FP32) or 32-byte (FP64) aligned vector.
constexpr int kKeBlock = 12;
constexpr int kKeStride = kSlots * kKeBlock;  // 432 values per element

// Device status bits (set by kernels with atomicOr, never by trapping).
enum : int { kStatusBadJacobian = 1, kStatusNaN = 2, kStatusWaitTimeout = 4 };
constexpr int kTileBlocks = 640;   // block nonzeros per streamed SpMV tile

struct MatParams {
  int kind;
  int elastic_its;
  double mu, kappa, lambda;
  double hard_a, hard_b;
  double C[36];  // row-major 6x6, engineering-shear Voigt
};

struct MatTable {
  int nblocks;
  int formulation;
  int bbar;  // small strain: B-bar (mean dilatation) strain-displacement
  MatParams m[kMaxBlocks];
};

// Scalars of one PCG solve, resident in device memory.
struct PcgScalars {
  double rz, rz_old, rr, rr0, pq, alpha, beta, tol2;
  double scale;    // rhs scaling applied before the solve (b.M^-1.b -> 1)
  double unscale;  // 1/scale, applied to the solution
  int done;       // 1 converged, 2 breakdown / non-finite
  int iters;
  int max_it;
  unsigned int count_a, count_b;  // last-block-done counters
  unsigned int bar_count;  // arrivals at the vector update's grid barrier (reset per solve)
  int fail;  // breakdown cause: 1 init non-finite, 2 p.q <= 0, 3 p.q non-finite, 4 update non-finite
};

// Scalars of one RVE's Krylov solve in a segmented batch (segpcg.cu).
struct SegScalars {
  double rz, rz_old, rr, rr0, alpha, beta, scale, unscale, tol2;
  int done;   // 0 iterating, 1 converged (or not solved), 2 breakdown, 3 iteration limit
  int iters;
  int fail;   // breakdown cause as PcgScalars::fail
  int max_it;
};
struct SegControl {
  int active;  // RVEs still iterating
  int pad;
};

// Scalars of the residual kernel.
struct ResidScalars {
  double norm2;
  unsigned int count;
  int pad;
};

struct MeshTemplate;  // a resident template mesh (compose.cu)
// geometry planes (25 planes of 8 points per element) of every resident
// template: the element-major offsets are the templates' pool offsets
struct TplGeoPool {
  void* d = nullptr;
  long long elems = 0;  // elements the pool holds
  int count = 0;        // templates it covers
};

// Symmetric stream format of the single-vector PCG product (symspmv.cu):
// upper node blocks only, lower blocks read as transposes of their upper
// twins.  Structure per tile in d_blob; values V8/V1 indexed by upper id.
struct SymStore {
  bool built = false;
  int ntiles = 0;
  int tile_blocks = 0;     // upper blocks per tile the structure was built for
  long long nu = 0, nl = 0;  // upper blocks, lower entries
  int cap_struct = 0;      // largest tile structure, bytes (rounded to 128)
  int cap_blocks = 0;      // largest tile, upper blocks
  int precision = -1;      // precision of the converted values
  std::vector<long long> h_off;
  unsigned char* d_blob = nullptr;
  long long* d_off = nullptr;  // ntiles+1 structure offsets
  int* d_koff = nullptr;       // ntiles+1 first upper id of each tile
  int* d_urow = nullptr;       // nnd+1 first upper id of each row
  int* d_diag = nullptr;       // nnd position of each row's diagonal block in the full CSR
  float* d_v8_32 = nullptr;    // nu*8
  float* d_v1_32 = nullptr;    // nu (+16 padding)
  double* d_v8_64 = nullptr;
  double* d_v1_64 = nullptr;
};
// Symmetric push storage of the single-reduction PCG product (pushfmt.cu,
// pcg_cg.cu): the upper node blocks of every row, its diagonal first, in
// tile-contiguous ranges {header (first row, rows, blocks, plane stride),
// local row pointers, columns, push slots, nine value planes}.  The product
// adds A_IJ u_J into row I and stores A_IJ^T u_I (J > I) at the block's push
// slot, k pstride + J with k the rank of I among row J's lower columns; the
// vector kernel adds row J's lptr[J+1] - lptr[J] slots in rank order.  Built
// on the device from the node-block CSR (composed meshes included); values
// assembled straight into it when the solve streams it, else converted from
// the full-storage tiles when a solve first needs them.
struct PushStore {
  bool built = false;
  int ntiles = 0;
  long long nu = 0, nl = 0;  // upper blocks (diagonals included), pushed blocks
  int kmax = 0;              // largest lower count of a row: rank planes of pstride push slots
  int pstride = 0;           // nnd rounded up to 8 (128-byte aligned planes)
  long long cap32 = 0, cap64 = 0;  // largest tile, bytes
  std::vector<long long> h_off32, h_off64;
  std::vector<int> h_tile_row;  // ntiles+1 first row of each tile
  long long* d_off32 = nullptr;
  long long* d_off64 = nullptr;
  unsigned char* d_blob32 = nullptr;
  unsigned char* d_blob64 = nullptr;
  int* d_tile_row = nullptr;  // ntiles+1 first row of each tile
  int* d_row_tile = nullptr;  // nnd
  int* d_urow = nullptr;      // nnd+1 first upper block of each row
  int* d_diag = nullptr;      // nnd position of each row's diagonal in the full CSR
  int* d_lptr = nullptr;      // nnd+1 first push slot of each row
  void* d_push32 = nullptr;   // kmax*pstride float4
  void* d_push64 = nullptr;   // kmax*pstride double4
  long long serial32 = -1, serial64 = -1;  // tangent serial of the converted values
};
struct SegScalars;
struct SegControl;
// Per-RVE Krylov solves of a segmented batch (segpcg.cu): node chunks of
// every RVE, per-RVE scalars and arrival counters, the captured iteration.
struct SegSolve {
  bool built = false;
  int nchunks = 0;
  int4* d_chunk = nullptr;        // {RVE, first node, end node, chunk index within the RVE}
  int* d_seg_chunk0 = nullptr;    // nseg+1 first chunk of each RVE
  SegScalars* d_sc = nullptr;     // nseg
  unsigned int* d_count = nullptr;  // nseg last-chunk counters (back to zero after each pass)
  double* d_part = nullptr;       // nchunks*2 chunk partials
  double* d_node_dot = nullptr;   // nnd: each row's z.w
  void* d_s = nullptr;            // A p by recurrence (vectors of the solve's precision)
  int s_precision = -1;
  uint8_t* d_active = nullptr;    // nseg: 1 = the solve iterates the RVE
  SegControl* d_ctl = nullptr;
  PcgScalars* d_gate = nullptr;   // done = 1 once no RVE iterates (the product returns at once)
  int2* d_tile_seg = nullptr;     // per push tile: first and last RVE of its rows
  uint8_t* d_tile_act = nullptr;  // per push tile: 1 while one of its RVEs iterates
  int tile_seg_n = 0;             // push tiles the two arrays were built for
  cudaGraphExec_t graph = nullptr;
  int graph_key = -1;
  void* graph_x = nullptr;
  std::vector<SegScalars> h_sc;
};
struct SymLaunch {
  int grid = 0;
  size_t smem = 0;
  int stages = 2;
  int minb = 3;  // CTAs per SM the register budget targets
};
// Launch plan of the single-vector PCG product (krylov.cu): the streamed
// full-storage kernel (grid, ring) or the symmetric format.
struct SpmvPlan {
  int spmv = 0, vec = 0;
  size_t spmv_smem = 0;
  int stages = 2;
  int warp_release = 0;
  int keep = -1;  // matrix tiles streamed with L2 priorities: -1 none, else tiles [0, keep) evict_last
  bool sym = false;
  SymLaunch sl;
};

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
};

struct Context {
  int device = 0;
  int num_sms = 1;  // multiprocessors of the device (grid sizing), queried at creation
  cudaStream_t stream = nullptr;
  std::string err;
  long long launches = 0;

  // mesh
  int nnd = 0, nel = 0, neq = 0;
  int formulation = TG_SMALL_STRAIN;
  MatTable mats{};
  bool have_blocks = false;
  bool has_j2 = false;
  std::vector<int> h_conn;       // nel*8
  std::vector<int> h_eqnos;      // nnd*3
  std::vector<double> h_coords;  // SoA 3*nnd
  std::vector<int> h_eq_slot;    // neq -> node*4+dof

  // device mesh
  double* d_X = nullptr;        // SoA 3*nnd
  int* d_conn = nullptr;        // nel*8
  int8_t* d_block = nullptr;    // nel (optional)
  uint8_t* d_mask = nullptr;    // nnd, active-dof bits
  int* d_eq_slot = nullptr;     // neq
  int* d_node_elem_ptr = nullptr;  // nnd+1
  int* d_node_elem = nullptr;      // nel*8: e*8+a, sorted per node

  // block CSR (3x3 node blocks)
  long long nnzb = 0;
  long long nnzb_pad = 0;       // SoA stride of the value arrays
  int* d_rowptr = nullptr;      // nnd+1, padded to a multiple of 4 plus 4 (bulk copies)
  int* d_col = nullptr;         // nnzb_pad (tail zero: bulk copies round up to 16 B)
  // row tiles of the streamed SpMV: tile t covers rows [tile_row[t], tile_row[t+1])
  int ntiles = 0;
  int* d_tile_row = nullptr;
  int spmv_tile_blocks = kTileBlocks;
  int spmv_stages = 2;
  int spmv_warp_release = 0;   // 1: per-warp stage release instead of a CTA barrier per tile
  long long l2_keep = 16ll << 20;  // matrix bytes the product keeps in L2 (<0: no L2 priorities)
  int tangent_epb = 8;         // elements per CTA of the tangent kernel (2, 4, 8)
  int sym_mode = 0;            // 1-3: the single-vector product streams the symmetric format (single meshes)
  int seg_pcg_mode = 1;        // 1: a segmented batch runs one Krylov solve per RVE (segpcg.cu)
  SegSolve seg;
  std::vector<uint8_t> seg_active;  // RVEs the next segmented solve iterates (empty: all)
  std::vector<int> seg_status;      // per-RVE status of the last segmented solve
  bool seg_tolerate = false;        // a breakdown of some RVEs is reported per RVE, not as an error
  int sym_tile_blocks = 512;   // upper blocks per tile of the symmetric format
  SymStore sym;
  PushStore push;
  // single-reduction PCG on the symmetric push storage: 1 (tg_pcg_form 3), 0
  // (forms 1, 2), -1 automatic (the default: the push storage for segmented
  // batches and for meshes of at least kPushAutoBlocks block nonzeros, whose
  // product amortises its build; the full storage below)
  int cg_push = -1;
  long long tangent_serial = 0; // assemblies so far (values of derived storages follow it)
  long long full_serial32 = -1, full_serial64 = -1;  // tangent serial of the full storage's values
  int* d_contrib_ptr = nullptr; // nnzb+1
  int* d_contrib = nullptr;     // nel*64: e*64 + a*8 + b
  std::vector<int> h_rowptr, h_col;
  // Tile-contiguous matrix storage ("blob", one per precision): tile t
  // occupies bytes [blob_off[t], blob_off[t+1]) and holds a 16-byte header
  // {first row, rows, blocks, plane stride}, the local row pointers, the
  // column indices and the nine value planes, each part 16-byte aligned, so
  // one bulk copy moves a whole tile and the product streams the matrix as
  // one sequential range.
  unsigned char* d_blob32 = nullptr;
  unsigned char* d_blob64 = nullptr;
  long long* d_blob_off32 = nullptr;  // ntiles+1
  long long* d_blob_off64 = nullptr;
  std::vector<long long> h_blob_off32, h_blob_off64;
  long long blob_cap32 = 0, blob_cap64 = 0;  // largest tile, bytes
  int* d_row_tile = nullptr;   // nnd: tile of each row
  std::vector<int> h_tile_row;
  float* d_minv32 = nullptr;    // 18*nnd: Jacobi then block-Jacobi
  double* d_minv64 = nullptr;
  double* d_geo = nullptr;      // 25 planes over nel*8 points: dN/dX (3x8), w det J (residual)
  float2* d_geo_ff = nullptr;   // the same planes as double-floats (hi, lo), for the double-float residual
  int* d_elem_src = nullptr;    // composed mesh: every element's element in the template geometry pool
  double* d_xyz = nullptr;      // nnd*3: staging of caller (x, y, z) nodal arrays
  float* d_Ke32 = nullptr;      // nel*432: 36 upper node-pair blocks, rows padded to 4
  double* d_Ke64 = nullptr;
  int tangent_precision = -1;   // precision of the last tangent
  int tangent_precond = -1;

  // nodal vectors (padded to 4 per node)
  double4_32a* d_u = nullptr;
  double4_32a* d_fext = nullptr;
  double4_32a* d_R = nullptr;
  double4_32a* d_fint = nullptr;   // nel*8
  double load_factor = 1.0;
  int iteration = 0;

  // J2 history (structure of arrays over nel*8 integration points)
  int8_t* d_j2_flags = nullptr;
  int8_t* d_j2_alloc = nullptr;  // nel
  double* d_j2_alpha = nullptr;
  double* d_j2_dgamma = nullptr;
  double* d_j2_norm = nullptr;
  double* d_j2_epsp = nullptr;   // 6*nel*8 (component-major)
  double* d_j2_nhat = nullptr;   // 6*nel*8

  // PCG work
  void* d_x = nullptr;  // float4 or double4_32a per node (solution du)
  void* d_r = nullptr;
  void* d_z = nullptr;
  void* d_p = nullptr;   // search direction (updated in place by the vector update)
  void* d_q = nullptr;
  void* d_cg_s = nullptr;  // s = A p by recurrence (single-reduction PCG), in the solve's precision
  int cg_s_precision = -1;
  int pcg_form = 1;        // 1: single-vector solves run the single-reduction PCG (pcg_cg.cu)
  int cg_pdl = 1;           // its kernels launch with programmatic dependencies
  cudaGraphExec_t cg_graph = nullptr;  // captured chunk of the single-reduction PCG
  int cg_graph_key = -1;
  int pcg_vec_precision = -1;
  PcgScalars* d_pcg = nullptr;
  double* d_partials = nullptr;  // reduction partials
  int partials_cap = 0;
  ResidScalars* d_resid = nullptr;
  int* d_status = nullptr;
  PcgScalars* h_pcg = nullptr;       // pinned mirrors [2]: chunk scalars alternate between them
  cudaEvent_t ev_poll[2] = {nullptr, nullptr};  // arrival of each mirror's copy
  ResidScalars* h_resid = nullptr;   // pinned mirror
  int* h_status = nullptr;           // pinned mirror
  double4_32a* d_du_last = nullptr;      // FP64 update (nnd)
  bool have_du = false;

  // CUDA graph of a chunk of PCG iterations
  cudaGraphExec_t pcg_graph = nullptr;
  int pcg_graph_key = -1;  // precision*2 + precond

  // RVE partition of a batch mesh (tg_set_segments)
  int nseg = 0;
  int* d_seg_node = nullptr;   // nseg+1
  int* d_seg_elem = nullptr;   // nseg+1
  double* d_seg_out = nullptr; // nseg*9 scratch for segmented results
  std::vector<int> h_seg_node, h_seg_elem;

  // step-start snapshot (tg_checkpoint / tg_rollback)
  double4_32a* d_u_ckpt = nullptr;
  double4_32a* d_R_ckpt = nullptr;
  bool ckpt_valid = false;  // cleared when the state is replaced (tg_state_load, new mesh)
  // caller timer (tg_timer_start / tg_timer_stop)
  cudaEvent_t ev_a = nullptr, ev_b = nullptr;

  // resident mesh templates (tg_template_add) and the composed mesh
  std::vector<MeshTemplate*> templates;
  // geometry planes of every resident template, one pool per arithmetic
  // (a composed mesh's elements share their template's planes: the batch
  // mesh copies the template's coordinates and connectivity verbatim)
  TplGeoPool tpl_geo_ff, tpl_geo64;
  long long tpl_elems = 0;      // elements of every template added (pool offsets, append-only)
  bool composed = false;           // mesh built by tg_mesh_compose (host copies on demand)
  std::vector<int> h_inst_tpl;     // template of every instance of the composed mesh

  std::vector<void*> allocations;
};

// ---- helpers ----
bool ok(Context* c, cudaError_t e, const char* what);
template <typename T>
bool dalloc(Context* c, T** p, size_t n) {
  if (n == 0) n = 1;
  // stream-ordered: no device-wide synchronisation, so contexts on other
  // streams keep running while this one (re)allocates
  cudaError_t e = cudaMallocAsync((void**)p, n * sizeof(T), c->stream);
  // the buffer is then valid for any stream and for synchronous copies
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    c->err = std::string("cudaMallocAsync failed: ") + cudaGetErrorString(e);
    *p = nullptr;
    return false;
  }
  c->allocations.push_back((void*)*p);
  return true;
}
void dfree(Context* c, void* p);

int equation_slots(Context* c, int nnd, const int* eqnos, std::vector<uint8_t>& mask, std::vector<int>& slot);
int alloc_mesh(Context* c, int nnd, int nel, int neq, long long nnzb);
// host copies of the mesh structure of a composed mesh, fetched on demand
int ensure_host_mesh(Context* c);
void free_templates(Context* c);
int launch_affine_prescribed(Context* c, const double* d_F);

// ---- host mesh utilities (mesh.cpp) ----
void build_block_pattern(int nnd, int nel, const int* conn, std::vector<int>& rowptr, std::vector<int>& col);
void build_contrib_map(int nnd, int nel, const int* conn, const std::vector<int>& rowptr,
                       const std::vector<int>& col, std::vector<int>& cptr, std::vector<int>& contrib);
int build_tiles(Context* c, int tile_blocks);
// CTAs of the full-storage product's persistent grid for FP32 tiles of at
// most cap32 bytes (0 if the ring does not fit) (krylov.cu)
int spmv_grid_for(Context* c, long long cap32);
void drop_graphs(Context* c);  // captured Krylov iterations (their launches bake in the product's shape)
int ensure_blob(Context* c, int precision);

// blob geometry shared by host and device code
__host__ __device__ inline int ceil4(int n) { return (n + 3) & ~3; }
// Preconditioner storage of one precision (values of T): the Jacobi inverse
// as 3x3 blocks [0, 9 nnd), the block-Jacobi inverse [9 nnd, 18 nnd), then
// from minv_diag_offset the Jacobi inverse's diagonal as one padded 4-vector
// per node (what the single-vector PCG reads with Jacobi: 16 instead of 36
// bytes per node in FP32)
__host__ __device__ inline long long minv_diag_offset(int nnd) { return (18LL * nnd + 3) / 4 * 4; }
inline size_t minv_values(int nnd) { return (size_t)minv_diag_offset(nnd) + 4 * (size_t)nnd; }
__host__ __device__ inline long long blob_tile_bytes(int nrows, int nb, int elem) {
  const long long pstride = ((long long)nb * elem + 15) / 16 * 16 / elem;
  return 16 + 4LL * ceil4(nrows + 1) + 4LL * ceil4(nb) + 9LL * pstride * elem;
}
void build_node_elem(int nnd, int nel, const int* conn, std::vector<int>& ptr, std::vector<int>& list);
void expand_pattern(int nnd, const int* eq, const std::vector<int>& rowptr, const std::vector<int>& col,
                    bool upper_only, int* row_ptr, int* col_idx, long long* nnz);

// ---- symmetric stream format (symspmv.cu) ----
bool sym_active(const Context* c);
int sym_build(Context* c, int tile_blocks);
int sym_convert(Context* c, int precision);  // values from the last assembly
int sym_config(Context* c, int precision, SymLaunch& L);
void sym_launch(Context* c, int precision, const SymLaunch& L, const void* p, void* q, double* partials,
                PcgScalars* sc, double* node_dot);
// per-RVE solves of a segmented batch (segpcg.cu)
int pcg_solve_segmented(Context* c, const double4_32a* d_rhs, double rel_tol, int max_it, int precond, int* iters,
                        double* rel_res);
void seg_free(Context* c);  // graph and bookkeeping (buffers go back with the mesh)
int pcg_vectors(Context* c, int precision);  // x r z p q of the solve's precision (krylov.cu)
// the single-vector product for other solvers (segpcg.cu): plan once per
// mesh/precision, launch on (p, q); node_dot (nnd, may be NULL) receives
// each row's p.q
int spmv_plan(Context* c, int precision, SpmvPlan& P);
void spmv_run(Context* c, int precision, const SpmvPlan& P, const void* p, void* q, double* partials, PcgScalars* sc,
              double* node_dot);
void sym_free(Context* c);

// ---- kernel launchers (elements.cu / assembly.cu / krylov.cu) ----
// Arithmetic of the element residual: FP64, or double-float on the FP32 pipe
// (about 48 significant bits; total-Lagrangian Simo groups, the others stay
// FP64).  Chosen by the caller: the mixed-precision Newton drivers use
// double-float, everything else FP64.
enum : int { kResidualFP64 = 0, kResidualDoubleFloat = 1 };
constexpr int kGeoPlanes = 25;  // per point: dN_a/dX_l (24), w det J
int launch_residual(Context* c, int arith = kResidualFP64);  // fint per element + gather + norm
// the total-Lagrangian Simo element forces in double-float (residual_ff.cu)
// src: each element's element in the planes (nullptr: the element itself);
// gstride: points per plane
int launch_residual_ff(Context* c, const float2* d_geo_ff, const int* src, long long gstride);
// the template geometry pool of one arithmetic (G float2: double-float,
// double: FP64), built for every resident template (compose.cu)
template <typename G>
int template_geometry_pool(Context* c, TplGeoPool& pool);
template <typename G>
int launch_geometry(Context* c, const double* X, int nnd, const int* conn, int nel, G* geo, long long stride,
                    long long off);
int launch_tangent(Context* c, int precision);   // Ke per element
int launch_assemble(Context* c, int precision);
int launch_blob_structure(Context* c, int precision);
// segmented (per-RVE) reductions over node / element ranges
int launch_segment_norms(Context* c, int nseg, const int* d_node_off, double* d_out);
int launch_segment_stress(Context* c, int nseg, const int* d_elem_off, double* d_out);
// macro tangent of every segment (static condensation by nine solves)
int launch_macro_perturb(Context* c, int k, int L, double4_32a* d_v);
int launch_macro_combine(Context* c, const double4_32a* d_v, double4_32a* d_w);
// columns kL .. kL+ncols-1 of the macro tangent; d_w holds ncols nodal vectors
int launch_segment_macro(Context* c, const double4_32a* d_w, int kL, int ncols, const double* d_vol0,
                         double* d_out);
// the nine condensation solves as one multi-vector PCG (mrhs.cu)
int macro_tangent_mrhs(Context* c, int precision, int precond, double rel_tol, int max_it, const double* d_vol,
                       double* d_C, int* iters);
int form_tangent(Context* c, int precision);
int launch_element_dump(Context* c, int first, int count, double* dKe, double* dfint);
int launch_close_step(Context* c, int reset);
int launch_set_prescribed(Context* c, int n, const int* d_idx, const double* d_val);
int launch_apply_update(Context* c);
int pcg_solve(Context* c, const double4_32a* d_rhs, double rel_tol, int max_it, int precond, int* iters,
              double* rel_res);
int time_pcg_kernel(Context* c, int which, int reps, double* ms);
// scale + init launches of a single-vector PCG, and the result of its final scalars (krylov.cu)
int pcg_start(Context* c, int precision, const double4_32a* d_rhs, const void* minv, double rel_tol, int max_it);
int pcg_finish(Context* c, const PcgScalars& h, int* iters, double* rel_res);
// single-reduction PCG (Chronopoulos-Gear) on full storage (pcg_cg.cu)
int pcg_solve_cg(Context* c, int precision, const double4_32a* d_rhs, double rel_tol, int max_it, int precond,
                 int* iters, double* rel_res);
void cg_free(Context* c);  // the captured iterations
// symmetric push storage: structure (once per mesh) and values of the last
// assembly in the given precision (pushfmt.cu)
int push_prepare(Context* c, int precision);
int push_structure(Context* c, int precision);  // structure and tiles of one precision, no values
// upper-only assembly into the push storage; the full storage on demand
int launch_assemble_upper(Context* c, int precision);
int ensure_full_assembly(Context* c);
// the product of a segmented batch's per-RVE solves on the push storage:
// w's upper part, the pushes, each row's own z.w (pcg_cg.cu)
int launch_seg_push(Context* c, int precision, const void* z, void* w, double* node_dot, PcgScalars* gate,
                    const uint8_t* tile_act = nullptr);
constexpr long long kPushAutoBlocks = 1000000;
// Segmented batches take the push storage at any size under the default, so
// an RVE solved alone and the same RVE in a batch run the same kernels
// (bitwise the same iterates).
inline bool push_active(const Context* c) {
  return c->cg_push > 0 || (c->cg_push < 0 && (c->nseg > 0 || c->nnzb >= kPushAutoBlocks));
}
int time_seg_push(Context* c, int reps, double* ms);  // standalone segmented push product (pcg_cg.cu)
// the next single-vector (or segmented batch) solve streams the push storage
inline bool push_solve(const Context* c) {
  if (c->nseg > 0 && c->seg_pcg_mode) return push_active(c);
  return c->pcg_form == 1 && !sym_active(c) && push_active(c);
}
void push_free(Context* c);
int time_cg_kernel(Context* c, int which, int reps, double* ms);  // 0 product, 1 vector kernel
// PCG with every work vector, partial sum and scalar in caller scratch
constexpr size_t kScratchScalarBytes = 256;
constexpr size_t kScratchPartialBytes = 32768;
size_t pcg_scratch_bytes(const Context* c);
int pcg_solve_scratch(Context* c, const double* d_rhs_eq, double* d_du_eq, unsigned char* scratch, double rel_tol,
                      int max_it, int precond, int* iters, double* rel_res);
int launch_residual_nocommit(Context* c, int arith = kResidualFP64);
// output pass (no history written): per point the Cauchy stress and the J2
// material output (alpha, von Mises, pressure) into d_ip_sig (nel*8*9), the
// extrapolated, element-averaged nodal values into d_out (nnd*9)
int launch_nodal_stress(Context* c, double* d_ip_sig, double* d_out);
// rhs = R - K v on active rows (v nodal, K the last tangent), FP64
// accumulation; with zero_base, rhs = -K v
int launch_lift_rhs(Context* c, const double4_32a* d_v, double4_32a* d_rhs, bool zero_base = false, int nvec = 1);
int launch_diff(Context* c, const double4_32a* a, const double4_32a* b, double4_32a* out);
int launch_gather_eq(Context* c, const double4_32a* d_nodal, double* d_eq);
int launch_xyz_to_nodal(Context* c, const double* d_xyz, double4_32a* d_nodal);  // 3 -> padded 4 per node
int launch_nodal_to_xyz(Context* c, const double4_32a* d_nodal, double* d_xyz);
int launch_scatter_eq(Context* c, const double* d_eq, double4_32a* d_nodal);

}  // namespace tg

// The opaque handle of the C ABI is the context itself.
struct tg_context : public tg::Context {};
