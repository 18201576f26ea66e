// Allocation-free variant of the decoupled look-back scan entry point.
//
// Who needs it: callers that must not allocate device memory at the moment
// they scan. Latency-critical loops must stay out of the allocator, whose
// calls can synchronise the whole device; plug-ins hosted by a framework that
// owns all device memory through its own pool may not create allocations
// behind its back; and a process whose device-memory budget is already spent
// still has to scan. The regular entry points take their scratch (workspace
// header plus look-back descriptors) from a per-stream cache that grows with
// cudaMallocAsync, or from a buffer the caller passes in; this one takes it
// from a fixed array compiled into the library's device image, so it
// allocates nothing at all.
//
// Limits and rules:
//   * the scratch holds kNoAllocScratchBytes = 1 MiB, enough for 114,176
//     descriptor words: up to 1,870,659,581 elements of a 4-byte integer type
//     (16,384-element tiles, one word each), 2,104,492,029 floats (18,432-
//     element tiles), 511,508,479 elements of an 8-byte integer type (8,960-
//     element tiles, two words each) and 460,357,631 doubles (8,064-element
//     tiles, two words each); three, three, one and one elements more when
//     the input is 16-byte aligned. Larger n is rejected with PP_ERR_WORKSPACE
//     before anything is launched;
//   * every GPU that loads the library holds the 1 MiB until the process
//     exits;
//   * all calls share the one array, which keeps the last call's contents.
//     Each call therefore clears the part it uses (cudaMemsetAsync on the
//     stream, no allocation) before its kernel, all but the sticky error word.
//     Calls that overlap on the GPU (on different streams, or from different
//     threads without ordering) race on the array and give wrong results:
//     order them on one stream;
//   * the first call on each device looks up the array's device address with
//     cudaGetSymbolAddress (once per device, with that device current), so
//     that first call belongs before any stream capture on the device;
//   * a device-side timeout is recorded in the array's error word, which the
//     next call leaves alone; pp_stream_status() on the stream of the calls
//     returns it (and clears it) after the stream's own workspace errors.
#include <cstddef>
#include <cstdint>
#include <mutex>

#include <cuda_runtime.h>

#include "dispatch.cuh"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(1) << 20;

// Host code must never use this name as an address: on the host it is only a
// stand-in for the device symbol. The device address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once).
pp_status scratch_address(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return PP_ERR_NO_DEVICE;
  if (dev < 0 || dev >= kMaxDevices) return PP_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> g(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return PP_ERR_CUDA;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return PP_OK;
}

}  // namespace

namespace pp {
namespace capi {
// The scratch of the allocation-free variant on the current device, or null
// when that variant has not run on it.
void* noalloc_scratch_used_on_current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
  std::lock_guard<std::mutex> g(g_scratch_mu);
  return g_scratch_addr[dev];
}
}  // namespace capi
}  // namespace pp

extern "C" pp_status pp_decoupled_scan_device_noalloc(pp_stream stream, pp_scan_kind kind, pp_op op,
                                                      pp_dtype dtype, const void* d_in, void* d_out, uint64_t n) {
  if (kind != PP_SCAN_INCLUSIVE && kind != PP_SCAN_EXCLUSIVE) return PP_ERR_INVALID_ARG;
  if (op < PP_OP_PLUS || op > PP_OP_MAXIMUM || dtype < PP_I32 || dtype > PP_F64) return PP_ERR_INVALID_ARG;
  if (n > 0 && (!d_in || !d_out)) return PP_ERR_INVALID_ARG;
  const bool is_float = dtype == PP_F32 || dtype == PP_F64;
  if (is_float && (op == PP_OP_BIT_AND || op == PP_OP_BIT_OR || op == PP_OP_BIT_XOR)) return PP_ERR_UNSUPPORTED;
  if (n == 0) return PP_OK;

  size_t need = 0;
  pp_status st = pp_workspace_size(PP_ALGO_DECOUPLED, dtype, PP_PREC_DEFAULT, d_in, d_out, n, &need);
  if (st != PP_OK) return st;
  if (need > kNoAllocScratchBytes) return PP_ERR_WORKSPACE;

  void* scratch = nullptr;
  st = scratch_address(&scratch);
  if (st != PP_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the previous call's header and descriptors must not leak into this one;
  // its error word stays until pp_stream_status() reads it
  constexpr size_t kErr = offsetof(pp::WsHeader, error);
  unsigned char* base = static_cast<unsigned char*>(scratch);
  if (cudaMemsetAsync(base, 0, kErr, s) != cudaSuccess) return PP_ERR_CUDA;
  if (cudaMemsetAsync(base + kErr + sizeof(unsigned int), 0, need - kErr - sizeof(unsigned int), s) != cudaSuccess)
    return PP_ERR_CUDA;

  pp::capi::ScanReq r;
  r.s = s;
  r.exclusive = kind == PP_SCAN_EXCLUSIVE;
  r.op = op;
  r.in = d_in;
  r.out = d_out;
  r.n = n;
  r.algo = PP_ALGO_DECOUPLED;
  r.ws = scratch;
  r.ws_bytes = kNoAllocScratchBytes;
  pp::host::Status hs = pp::host::Status::invalid_arg;
  switch (dtype) {
    case PP_I32:
      hs = pp::capi::scan_typed<int32_t>(r);
      break;
    case PP_U32:
      hs = pp::capi::scan_typed<uint32_t>(r);
      break;
    case PP_I64:
      hs = pp::capi::scan_typed<int64_t>(r);
      break;
    case PP_U64:
      hs = pp::capi::scan_typed<uint64_t>(r);
      break;
    case PP_F32:
      hs = pp::capi::scan_typed<float>(r);
      break;
    case PP_F64:
      hs = pp::capi::scan_typed<double>(r);
      break;
  }
  return static_cast<pp_status>(static_cast<int>(hs));
}
