// Radix sort of (key, value) pairs for callers that cannot allocate device
// memory -- for example a host engine that owns every device allocation
// through its own pool, or a per-frame callback where cudaMalloc/cudaFree
// would synchronise the device and stall the frame.  Same sort as
// pbf_op_sort_pairs; its scratch is a file-scope device array instead of a
// caller buffer.
//
// The array holds the scratch for up to kNoAllocMaxKeys keys
// (words_for(kNoAllocMaxKeys) 32-bit words, about 9.4 MB).  Every GPU that
// loads this library keeps it until the process exits.  All calls share it
// and it keeps the last call's contents: each call first zeroes the
// histogram, tile-counter and look-back words it relies on, in stream order.
// Calls whose work overlaps on the GPU (different streams, or different host
// threads without ordering) race on the array.
#include <mutex>

#include "pbf_device.cuh"
#include "pbf_host.hpp"

namespace pbf {
namespace {

constexpr uint32_t kNoAllocMaxKeys = 1u << 20;
constexpr int kMaxDevices = 64;

// The largest plan of any key width for the most keys.
constexpr size_t kNoAllocWords = sort_words_max(kNoAllocMaxKeys);

static __device__ __align__(256) uint32_t g_sort_scratch[kNoAllocWords];

// The device address of g_sort_scratch is looked up once per CUDA context
// (the host-side name is only a stand-in for it) and cached per device
// ordinal together with the context's unique id.  A context created later on
// the same device -- after cudaDeviceReset, or after the primary context was
// released and retained again -- loads the module afresh, possibly at another
// address; its different id makes the next call look the address up again.
struct ScratchEntry {
  unsigned long long ctx_id = 0;
  void *address = nullptr;
};
std::mutex g_mutex;
ScratchEntry g_scratch[kMaxDevices];

using CtxGetCurrentFn = int (*)(void **);
using CtxGetIdFn = int (*)(void *, unsigned long long *);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;
std::once_flag g_entry_once;

// Driver entry points (no link-time dependency on the driver library).
void resolve_entry_points() {
  void *fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) ==
          cudaSuccess && q == cudaDriverEntryPointSuccess)
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(fn);
  fn = nullptr;
  if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) ==
          cudaSuccess && q == cudaDriverEntryPointSuccess)
    g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(fn);
}

// Unique id of the calling thread's current context, or 0 if none is current
// (or the driver cannot tell).
unsigned long long current_context_id() {
  std::call_once(g_entry_once, resolve_entry_points);
  if (!g_ctx_get_current || !g_ctx_get_id) return 0;
  void *ctx = nullptr;
  if (g_ctx_get_current(&ctx) != 0 || !ctx) return 0;
  unsigned long long id = 0;
  return g_ctx_get_id(ctx, &id) == 0 ? id : 0;
}

// Device address of g_sort_scratch in the current device's context.
int scratch_address(uint32_t **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) {
    set_error_message("device ordinal beyond the no-alloc sort's table");
    return PBF_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_mutex);
  ScratchEntry &entry = g_scratch[dev];
  const unsigned long long id = current_context_id();
  if (!entry.address || id == 0 || id != entry.ctx_id) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_sort_scratch);  // makes the primary context current
    if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress");
    entry.address = p;
    entry.ctx_id = current_context_id();
  }
  *out = static_cast<uint32_t *>(entry.address);
  return PBF_OK;
}

}  // namespace
}  // namespace pbf

extern "C" int pbf_op_sort_pairs_noalloc(const uint32_t *d_keys_in,
                                         const uint32_t *d_vals_in, uint32_t n,
                                         uint32_t key_bits,
                                         uint32_t *d_keys_out,
                                         uint32_t *d_vals_out,
                                         uint32_t *d_status, void *stream) {
  using namespace pbf;
  if (n == 0) return PBF_OK;
  if (!d_keys_in || !d_keys_out || !d_vals_out) return PBF_ERR_INVALID;
  if (key_bits < 1 || key_bits > 32) return PBF_ERR_INVALID;
  if (n > kNoAllocMaxKeys) {
    set_error_message("pbf_op_sort_pairs_noalloc sorts at most 1048576 keys");
    return PBF_ERR_INVALID;
  }
  const SortPlan plan = make_sort_plan(n, key_bits);
  if (plan.words > kNoAllocWords) return PBF_ERR_INVALID;
  uint32_t *scratch = nullptr;
  const int rc = scratch_address(&scratch);
  if (rc != PBF_OK) return rc;
  uint32_t *err = d_status ? d_status : scratch + plan.off_counter + 31;
  const cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = sort_clear(plan, scratch, st);
  if (e == cudaSuccess) e = sort_histogram(plan, d_keys_in, scratch, st);
  if (e == cudaSuccess) e = sort_scan(plan, scratch, st);
  if (e == cudaSuccess)
    e = sort_passes(plan, d_keys_in, d_vals_in, d_keys_out, d_vals_out, scratch,
                    err, st);
  return cuda_status(e, "pbf_op_sort_pairs_noalloc");
}
