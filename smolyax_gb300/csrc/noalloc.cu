// FP64 evaluation that allocates nothing: the basis table lives in a
// file-scope device array instead of caller-provided scratch.
//
// Who needs it: callers that cannot (or must not) allocate device memory at
// evaluation time -- foreign-language hosts (Go, Java, Rust over FFI) that do
// not own a CUDA allocator, serving processes whose device memory is fully
// reserved by a pool allocator, and code paths that must not call cudaMalloc
// because it synchronises the device.  They pass inputs and outputs only.
//
// Limits and rules (stated in the header as well):
//  * the scratch holds SMX_STATIC_SCRATCH_BYTES; a call whose basis table
//    (n_values * P doubles) does not fit is rejected with SMX_ERR_WORKSPACE;
//    evaluate larger batches in chunks of points;
//  * every GPU that loads the library keeps the array until the process exits;
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress, with that device current); make that first call
//    before any stream capture;
//  * all calls share the one array: calls that overlap on the GPU (different
//    streams, or threads) race; serialise them.  The basis kernel overwrites
//    every slot it later reads, so nothing needs clearing between calls;
//  * the address is cached per device together with the CUDA context it was
//    looked up in; after a device reset (a new primary context) the next call
//    looks it up again instead of using the old context's address.
#include <cuda.h>

#include <mutex>

#include "common.cuh"

namespace {

constexpr size_t kScratchDoubles = size_t(SMX_STATIC_SCRATCH_BYTES) / sizeof(double);

static __device__ __align__(256) double g_static_scratch[kScratchDoubles];

std::mutex g_mu;
constexpr int kMaxDevices = 256;
void* g_scratch_addr[kMaxDevices] = {};
CUcontext g_scratch_ctx[kMaxDevices] = {};

using CtxGetCurrentFn = CUresult (*)(CUcontext*);

// The driver's cuCtxGetCurrent, through the runtime's entry-point query (the
// library links only the CUDA runtime); null if unavailable.
CtxGetCurrentFn ctx_get_current() {
  static CtxGetCurrentFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return static_cast<CtxGetCurrentFn>(nullptr);
    return reinterpret_cast<CtxGetCurrentFn>(p);
  }();
  return fn;
}

CUcontext current_context() {
  CUcontext c = nullptr;
  const CtxGetCurrentFn fn = ctx_get_current();
  if (!fn || fn(&c) != CUDA_SUCCESS) return nullptr;
  return c;
}

}  // namespace

extern "C" int smx_eval_f64_noalloc(const smx_plan* pl, const double* x, int64_t P, int64_t ldx, double* y,
                                    void* stream) {
  SMX_REQUIRE(pl != nullptr, "smx_eval_f64_noalloc: null plan");
  SMX_REQUIRE(P >= 0 && pl->n_values >= 0, "smx_eval_f64_noalloc: bad sizes");
  const double need = double(pl->n_values) * double(P);
  if (need > double(kScratchDoubles)) {
    return smx::set_error(SMX_ERR_WORKSPACE,
                          "smx_eval_f64_noalloc: basis table of " + std::to_string(pl->n_values) + " x " +
                              std::to_string(P) + " doubles exceeds the static scratch of " +
                              std::to_string(SMX_STATIC_SCRATCH_BYTES) + " bytes; evaluate at most " +
                              std::to_string(pl->n_values ? kScratchDoubles / size_t(pl->n_values) : 0) +
                              " points per call");
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return smx::set_error(SMX_ERR_CUDA, "smx_eval_f64_noalloc: no current CUDA device");
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    const CUcontext ctx = current_context();
    if (!g_scratch_addr[dev] || !ctx || ctx != g_scratch_ctx[dev]) {
      void* addr = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&addr, g_static_scratch);
      if (e != cudaSuccess || addr == nullptr)
        return smx::set_error(SMX_ERR_CUDA, std::string("smx_eval_f64_noalloc: cudaGetSymbolAddress failed: ") +
                                                cudaGetErrorString(e));
      g_scratch_addr[dev] = addr;
      g_scratch_ctx[dev] = current_context();  // the lookup made the device's context current if it was not
    }
    scratch = g_scratch_addr[dev];
  }
  double* Lt = static_cast<double*>(scratch);
  int rc = smx_basis_f64(pl, x, P, ldx, Lt, nullptr, stream);
  if (rc) return rc;
  return smx_contract_f64(pl, Lt, P, y, stream);
}
