// tg_pcg_solve_noalloc: the Krylov solve for callers that cannot allocate.
//
// Some hosts of this library own every byte of device memory themselves (a
// solver embedded in a larger application with a fixed, pre-reserved device
// arena; a serving loop whose latency budget forbids allocator calls between
// requests; code running where the CUDA allocator must not be entered at
// all).  For them this entry point runs the same (block-)Jacobi PCG as
// tg_pcg_solve without any allocation: the work vectors, reduction partials
// and solver scalars live in one file-scope device array below, sized for
// meshes of up to kNoAllocMaxNodes nodes.  Every GPU that loads the library
// holds that array until the process exits.
#include <mutex>

#include "tg_internal.h"

namespace {

constexpr int kNoAllocMaxNodes = 32768;
constexpr size_t kNoAllocScratchBytes = 8u << 20;  // 8 MiB per device
static_assert(tg::kScratchScalarBytes + tg::kScratchPartialBytes + (32 + 5 * 32) * (size_t)kNoAllocMaxNodes <=
                  kNoAllocScratchBytes,
              "scratch too small for the stated node limit");

// Shared by every call on a device; it keeps the last call's contents.
static __device__ __align__(256) unsigned char g_pcg_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array for the current device.  The host-side
// name g_pcg_scratch is only a stand-in, so the address is looked up once per
// device (with that device current) and cached.  The cache assumes the
// device's primary context for the life of the process (the runtime API's
// context): after a cudaDeviceReset, or when the caller makes another driver
// context current, the cached address no longer names the array.
int scratch_address(tg::Context* c, void** out) {
  if (c->device < 0 || c->device >= kMaxDevices) {
    c->err = "device index out of range for the no-allocation scratch table";
    return TG_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[c->device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_pcg_scratch);
    if (e != cudaSuccess) {
      c->err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return TG_ERR_CUDA;
    }
    g_addr[c->device] = p;
  }
  *out = g_addr[c->device];
  return TG_OK;
}

}  // namespace

extern "C" int tg_pcg_solve_noalloc(tg_context* c, const double* d_rhs, double* d_du, double rel_tol, int max_it,
                                    int precond, int* iterations, double* rel_res) {
  if (!c || !d_rhs || !d_du || c->nnd <= 0 || max_it <= 0 || rel_tol <= 0.0) return TG_ERR_ARG;
  if (precond != TG_PRECOND_JACOBI && precond != TG_PRECOND_BLOCK_JACOBI) return TG_ERR_ARG;
  if (c->tangent_precision < 0) {
    c->err = "tg_pcg_solve_noalloc: form the tangent first";
    return TG_ERR_ARG;
  }
  if (c->nnd > kNoAllocMaxNodes || tg::pcg_scratch_bytes(c) > kNoAllocScratchBytes) {
    c->err = "tg_pcg_solve_noalloc: mesh has " + std::to_string(c->nnd) + " nodes; the fixed scratch holds at most " +
             std::to_string(kNoAllocMaxNodes) + " (use tg_pcg_solve)";
    return TG_ERR_CAPACITY;
  }
  if (!tg::ok(c, cudaSetDevice(c->device), "cudaSetDevice")) return TG_ERR_CUDA;
  void* scratch = nullptr;
  const int s = scratch_address(c, &scratch);
  if (s) return s;
  return tg::pcg_solve_scratch(c, d_rhs, d_du, static_cast<unsigned char*>(scratch), rel_tol, max_it, precond,
                               iterations, rel_res);
}
