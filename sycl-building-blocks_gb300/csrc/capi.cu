// extern "C" entry points of libppgb300.so (declared in include/pp_gb300.h).
#include <cstdint>
#include <cstring>
#include <mutex>

#include <cuda_runtime.h>

#include "dispatch.cuh"

using pp::capi::ScanReq;
using pp::host::Status;

namespace {

pp_status to_c(Status s) { return static_cast<pp_status>(static_cast<int>(s)); }

bool valid_kind(pp_scan_kind k) { return k == PP_SCAN_INCLUSIVE || k == PP_SCAN_EXCLUSIVE; }
bool valid_op(pp_op op) { return op >= PP_OP_PLUS && op <= PP_OP_MAXIMUM; }
bool valid_dtype(pp_dtype d) { return d >= PP_I32 && d <= PP_F64; }
bool valid_algo(pp_scan_algo a) { return a >= PP_ALGO_AUTO && a <= PP_ALGO_SINGLE_GROUP; }
bool valid_prec(pp_precision p) { return p >= PP_PREC_DEFAULT && p <= PP_PREC_FP64_CARRY; }
bool is_float(pp_dtype d) { return d == PP_F32 || d == PP_F64; }
bool is_bitop(pp_op op) { return op == PP_OP_BIT_AND || op == PP_OP_BIT_OR || op == PP_OP_BIT_XOR; }

size_t dtype_size(pp_dtype d) {
  switch (d) {
    case PP_I32:
    case PP_U32:
    case PP_F32:
      return 4;
    default:
      return 8;
  }
}

// Element access needs pointers aligned to the element size.
bool aligned_to(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

// Validation that needs no GPU: enums, pointers, combinations.
pp_status check_scan_args(pp_scan_kind kind, pp_op op, pp_dtype dt, const void* in, const void* out, uint64_t n,
                          pp_scan_algo algo, pp_precision prec) {
  if (!valid_kind(kind) || !valid_op(op) || !valid_dtype(dt) || !valid_algo(algo) || !valid_prec(prec))
    return PP_ERR_INVALID_ARG;
  if (n > 0 && (!in || !out)) return PP_ERR_INVALID_ARG;
  if (n > 0 && (!aligned_to(in, dtype_size(dt)) || !aligned_to(out, dtype_size(dt)))) return PP_ERR_INVALID_ARG;
  if (is_float(dt) && is_bitop(op)) return PP_ERR_UNSUPPORTED;
  if (prec != PP_PREC_DEFAULT && (dt != PP_F32 || op != PP_OP_PLUS)) return PP_ERR_UNSUPPORTED;
  return PP_OK;
}

Status scan_dispatch(const ScanReq& r, pp_dtype dt, pp_precision prec) {
  using namespace pp::capi;
  if (prec != PP_PREC_DEFAULT) return scan_f32_precision(r, prec);
  switch (dt) {
    case PP_I32:
      return scan_typed<int32_t>(r);
    case PP_U32:
      return scan_typed<uint32_t>(r);
    case PP_I64:
      return scan_typed<int64_t>(r);
    case PP_U64:
      return scan_typed<uint64_t>(r);
    case PP_F32:
      return scan_typed<float>(r);
    case PP_F64:
      return scan_typed<double>(r);
  }
  return Status::invalid_arg;
}

Status reduce_dispatch(cudaStream_t s, pp_op op, pp_dtype dt, const void* in, uint64_t n, void* d_res, void* ws,
                       size_t ws_bytes) {
  using namespace pp::capi;
  switch (dt) {
    case PP_I32:
      return reduce_typed<int32_t>(s, op, in, n, d_res, ws, ws_bytes);
    case PP_U32:
      return reduce_typed<uint32_t>(s, op, in, n, d_res, ws, ws_bytes);
    case PP_I64:
      return reduce_typed<int64_t>(s, op, in, n, d_res, ws, ws_bytes);
    case PP_U64:
      return reduce_typed<uint64_t>(s, op, in, n, d_res, ws, ws_bytes);
    case PP_F32:
      return reduce_typed<float>(s, op, in, n, d_res, ws, ws_bytes);
    case PP_F64:
      return reduce_typed<double>(s, op, in, n, d_res, ws, ws_bytes);
  }
  return Status::invalid_arg;
}

Status dispatch_carry(pp_dtype dt, cudaStream_t s, pp_op op, void* out, const void* in, uint64_t n,
                      const void* carry_prev, void* carry_next, bool excl, bool first) {
  using namespace pp::capi;
  switch (dt) {
    case PP_I32:
      return carry_typed<int32_t>(s, op, out, in, n, carry_prev, carry_next, excl, first);
    case PP_U32:
      return carry_typed<uint32_t>(s, op, out, in, n, carry_prev, carry_next, excl, first);
    case PP_I64:
      return carry_typed<int64_t>(s, op, out, in, n, carry_prev, carry_next, excl, first);
    case PP_U64:
      return carry_typed<uint64_t>(s, op, out, in, n, carry_prev, carry_next, excl, first);
    case PP_F32:
      return carry_typed<float>(s, op, out, in, n, carry_prev, carry_next, excl, first);
    case PP_F64:
      return carry_typed<double>(s, op, out, in, n, carry_prev, carry_next, excl, first);
  }
  return Status::invalid_arg;
}

pp_status scan_entry(pp_stream stream, pp_scan_kind kind, pp_op op, pp_dtype dt, const void* in, void* out,
                     uint64_t n, pp_scan_algo algo, pp_precision prec, void* ws, size_t ws_bytes) {
  pp_status c = check_scan_args(kind, op, dt, in, out, n, algo, prec);
  if (c != PP_OK) return c;
  if (n == 0) return PP_OK;
  ScanReq r;
  r.s = static_cast<cudaStream_t>(stream);
  r.exclusive = kind == PP_SCAN_EXCLUSIVE;
  r.op = op;
  r.in = in;
  r.out = out;
  r.n = n;
  r.algo = algo;
  r.ws = ws;
  r.ws_bytes = ws_bytes;
  return to_c(scan_dispatch(r, dt, prec));
}

// Host-pointer scans stream the array through the GPU in chunks on three
// streams: copy in (chunk i+1), scan and offset (chunk i), copy out (chunk
// i-1) overlap, and the copy engines run both directions at once. Chunk i is
// scanned on its own and offset by the running total of chunks 0..i-1 (kept
// on the device, double-buffered). A ring of kSlots chunk buffers bounds the
// device memory at 2 * kSlots * kChunkBytes.
constexpr size_t kChunkBytes = size_t(64) << 20;
constexpr int kSlots = 4;
constexpr uint64_t kMaxChunks = 16384;  // per-chunk partial results of a host reduction (1 TiB of input)

struct HostPipeline {
  std::mutex mu;
  int device = -1;
  cudaStream_t h2d = nullptr, comp = nullptr, d2h = nullptr;
  cudaEvent_t in_ready[kSlots] = {}, out_ready[kSlots] = {}, slot_free[kSlots] = {};
  void* d_in[kSlots] = {};
  void* d_out[kSlots] = {};
  void* carry = nullptr;     // two 16-byte running totals
  void* result = nullptr;    // one reduction result
  void* partials = nullptr;  // kMaxChunks per-chunk reduction results
};
HostPipeline& pipeline() {
  static HostPipeline* p = new HostPipeline();
  return *p;
}

pp_status ensure_pipeline(HostPipeline& p) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return PP_ERR_NO_DEVICE;
  if (p.device == dev) return PP_OK;
  if (p.device >= 0) return PP_ERR_UNSUPPORTED;  // one device per process for the host entry points
  bool ok = cudaStreamCreateWithFlags(&p.h2d, cudaStreamNonBlocking) == cudaSuccess &&
            cudaStreamCreateWithFlags(&p.comp, cudaStreamNonBlocking) == cudaSuccess &&
            cudaStreamCreateWithFlags(&p.d2h, cudaStreamNonBlocking) == cudaSuccess;
  for (int k = 0; ok && k < kSlots; ++k) {
    ok = cudaEventCreateWithFlags(&p.in_ready[k], cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&p.out_ready[k], cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&p.slot_free[k], cudaEventDisableTiming) == cudaSuccess &&
         cudaMalloc(&p.d_in[k], kChunkBytes) == cudaSuccess && cudaMalloc(&p.d_out[k], kChunkBytes) == cudaSuccess;
  }
  ok = ok && cudaMalloc(&p.carry, 32) == cudaSuccess && cudaMalloc(&p.result, 16) == cudaSuccess &&
       cudaMalloc(&p.partials, kMaxChunks * 8) == cudaSuccess;
  if (!ok) return PP_ERR_CUDA;
  p.device = dev;
  return PP_OK;
}

pp_status host_scan_entry(pp_scan_kind kind, pp_op op, pp_dtype dt, const void* h_in, void* h_out, uint64_t n,
                          pp_scan_algo algo) {
  pp_status c = check_scan_args(kind, op, dt, h_in, h_out, n, algo, PP_PREC_DEFAULT);
  if (c != PP_OK) return c;
  if (n == 0) return PP_OK;
  const size_t esz = dtype_size(dt);
  const uint64_t chunk = kChunkBytes / esz;
  const uint64_t chunks = (n + chunk - 1) / chunk;
  HostPipeline& p = pipeline();
  std::lock_guard<std::mutex> g(p.mu);
  c = ensure_pipeline(p);
  if (c != PP_OK) return c;
  const bool excl = kind == PP_SCAN_EXCLUSIVE;
  const unsigned char* hi = static_cast<const unsigned char*>(h_in);
  unsigned char* ho = static_cast<unsigned char*>(h_out);
  unsigned char* carry = static_cast<unsigned char*>(p.carry);
  for (uint64_t i = 0; i < chunks && c == PP_OK; ++i) {
    const int k = int(i % kSlots);
    const uint64_t off = i * chunk;
    const uint64_t m = n - off < chunk ? n - off : chunk;
    const size_t bytes = m * esz;
    // the slot's previous chunk must be out before its buffers are reused
    if (i >= uint64_t(kSlots) && cudaStreamWaitEvent(p.h2d, p.slot_free[k], 0) != cudaSuccess) c = PP_ERR_CUDA;
    if (c == PP_OK && cudaMemcpyAsync(p.d_in[k], hi + off * esz, bytes, cudaMemcpyHostToDevice, p.h2d) != cudaSuccess)
      c = PP_ERR_CUDA;
    if (c == PP_OK && (cudaEventRecord(p.in_ready[k], p.h2d) != cudaSuccess ||
                       cudaStreamWaitEvent(p.comp, p.in_ready[k], 0) != cudaSuccess))
      c = PP_ERR_CUDA;
    if (c == PP_OK) c = scan_entry(p.comp, kind, op, dt, p.d_in[k], p.d_out[k], m, algo, PP_PREC_DEFAULT, nullptr, 0);
    if (c == PP_OK) {
      c = to_c(dispatch_carry(dt, p.comp, op, p.d_out[k], p.d_in[k], m, carry + ((i + 1) & 1) * 16,
                              carry + (i & 1) * 16, excl, i == 0));
    }
    if (c == PP_OK && (cudaEventRecord(p.out_ready[k], p.comp) != cudaSuccess ||
                       cudaStreamWaitEvent(p.d2h, p.out_ready[k], 0) != cudaSuccess))
      c = PP_ERR_CUDA;
    if (c == PP_OK && cudaMemcpyAsync(ho + off * esz, p.d_out[k], bytes, cudaMemcpyDeviceToHost, p.d2h) != cudaSuccess)
      c = PP_ERR_CUDA;
    if (c == PP_OK && cudaEventRecord(p.slot_free[k], p.d2h) != cudaSuccess) c = PP_ERR_CUDA;
  }
  // nothing may still read or write the caller's buffers when this returns
  const cudaError_t e1 = cudaStreamSynchronize(p.h2d);
  const cudaError_t e2 = cudaStreamSynchronize(p.comp);
  const cudaError_t e3 = cudaStreamSynchronize(p.d2h);
  if (c != PP_OK) return c;
  if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) return PP_ERR_CUDA;
  return to_c(pp::host::read_device_error(p.comp, nullptr));
}

}  // namespace

extern "C" {

pp_status pp_scan(pp_stream stream, pp_scan_kind kind, pp_op op, pp_dtype dtype, const void* d_in, void* d_out,
                  uint64_t n, pp_scan_algo algo, pp_precision precision) {
  return scan_entry(stream, kind, op, dtype, d_in, d_out, n, algo, precision, nullptr, 0);
}

pp_status pp_scan_ws(pp_stream stream, pp_scan_kind kind, pp_op op, pp_dtype dtype, const void* d_in, void* d_out,
                     uint64_t n, pp_scan_algo algo, pp_precision precision, void* d_workspace,
                     size_t workspace_bytes) {
  if (!d_workspace) return PP_ERR_INVALID_ARG;
  return scan_entry(stream, kind, op, dtype, d_in, d_out, n, algo, precision, d_workspace, workspace_bytes);
}

pp_status pp_workspace_size(pp_scan_algo algo, pp_dtype dtype, pp_precision precision, const void* d_in,
                            const void* d_out, uint64_t n, size_t* bytes) {
  if (!bytes || !valid_algo(algo) || !valid_dtype(dtype) || !valid_prec(precision)) return PP_ERR_INVALID_ARG;
  if (!aligned_to(d_in, dtype_size(dtype)) || !aligned_to(d_out, dtype_size(dtype))) return PP_ERR_INVALID_ARG;
  using namespace pp::capi;
  if (precision != PP_PREC_DEFAULT) {
    if (dtype != PP_F32) return PP_ERR_UNSUPPORTED;
    *bytes = workspace_f32_precision(algo, precision, d_in, d_out, n);
    return PP_OK;
  }
  switch (dtype) {
    case PP_I32:
      *bytes = workspace_typed<int32_t>(algo, d_in, d_out, n);
      break;
    case PP_U32:
      *bytes = workspace_typed<uint32_t>(algo, d_in, d_out, n);
      break;
    case PP_I64:
      *bytes = workspace_typed<int64_t>(algo, d_in, d_out, n);
      break;
    case PP_U64:
      *bytes = workspace_typed<uint64_t>(algo, d_in, d_out, n);
      break;
    case PP_F32:
      *bytes = workspace_typed<float>(algo, d_in, d_out, n);
      break;
    case PP_F64:
      *bytes = workspace_typed<double>(algo, d_in, d_out, n);
      break;
  }
  return PP_OK;
}

pp_status pp_decoupled_scan_device(pp_stream stream, pp_scan_kind kind, pp_op op, pp_dtype dtype,
                                   const void* d_in, void* d_out, uint64_t n) {
  return pp_scan(stream, kind, op, dtype, d_in, d_out, n, PP_ALGO_DECOUPLED, PP_PREC_DEFAULT);
}

pp_status pp_cooperative_scan_device(pp_stream stream, pp_scan_kind kind, pp_op op, pp_dtype dtype,
                                     const void* d_in, void* d_out, uint64_t n) {
  return pp_scan(stream, kind, op, dtype, d_in, d_out, n, PP_ALGO_COOPERATIVE, PP_PREC_DEFAULT);
}

pp_status pp_scan_device(pp_stream stream, pp_scan_kind kind, pp_op op, pp_dtype dtype, const void* d_in,
                         void* d_out, uint64_t n) {
  return pp_scan(stream, kind, op, dtype, d_in, d_out, n, PP_ALGO_DECOUPLED, PP_PREC_DEFAULT);
}

pp_status pp_group_scan_device(pp_stream stream, pp_scan_kind kind, pp_op op, pp_dtype dtype, const void* d_in,
                               void* d_out, uint64_t n) {
  return pp_scan(stream, kind, op, dtype, d_in, d_out, n, PP_ALGO_SINGLE_GROUP, PP_PREC_DEFAULT);
}

pp_status pp_reduce(pp_stream stream, pp_op op, pp_dtype dtype, const void* d_in, uint64_t n, void* d_result) {
  if (!valid_op(op) || !valid_dtype(dtype) || !d_result || (n > 0 && !d_in)) return PP_ERR_INVALID_ARG;
  if (!aligned_to(d_result, dtype_size(dtype)) || (n > 0 && !aligned_to(d_in, dtype_size(dtype))))
    return PP_ERR_INVALID_ARG;
  if (is_float(dtype) && is_bitop(op)) return PP_ERR_UNSUPPORTED;
  return to_c(reduce_dispatch(static_cast<cudaStream_t>(stream), op, dtype, d_in, n, d_result, nullptr, 0));
}

pp_status pp_reduce_ws(pp_stream stream, pp_op op, pp_dtype dtype, const void* d_in, uint64_t n, void* d_result,
                       void* d_workspace, size_t workspace_bytes) {
  if (!valid_op(op) || !valid_dtype(dtype) || !d_result || !d_workspace || (n > 0 && !d_in))
    return PP_ERR_INVALID_ARG;
  if (!aligned_to(d_result, dtype_size(dtype)) || (n > 0 && !aligned_to(d_in, dtype_size(dtype))))
    return PP_ERR_INVALID_ARG;
  if (is_float(dtype) && is_bitop(op)) return PP_ERR_UNSUPPORTED;
  return to_c(reduce_dispatch(static_cast<cudaStream_t>(stream), op, dtype, d_in, n, d_result, d_workspace,
                              workspace_bytes));
}

pp_status pp_reduce_device(pp_stream stream, pp_op op, pp_dtype dtype, const void* d_in, uint64_t n,
                           void* h_result) {
  if (!h_result) return PP_ERR_INVALID_ARG;
  if (!valid_op(op) || !valid_dtype(dtype) || (n > 0 && !d_in)) return PP_ERR_INVALID_ARG;
  if (n > 0 && !aligned_to(d_in, dtype_size(dtype))) return PP_ERR_INVALID_ARG;
  if (is_float(dtype) && is_bitop(op)) return PP_ERR_UNSUPPORTED;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  HostPipeline& p = pipeline();
  std::lock_guard<std::mutex> g(p.mu);
  pp_status c = ensure_pipeline(p);
  if (c != PP_OK) return c;
  Status r = reduce_dispatch(s, op, dtype, d_in, n, p.result, nullptr, 0);
  if (r != Status::ok) return to_c(r);
  if (cudaMemcpyAsync(h_result, p.result, dtype_size(dtype), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return PP_ERR_CUDA;
  return to_c(pp::host::read_device_error(s, nullptr));
}

pp_status pp_decoupled_scan_host(pp_scan_kind kind, pp_op op, pp_dtype dtype, const void* h_in, void* h_out,
                                 uint64_t n) {
  return host_scan_entry(kind, op, dtype, h_in, h_out, n, PP_ALGO_DECOUPLED);
}
pp_status pp_cooperative_scan_host(pp_scan_kind kind, pp_op op, pp_dtype dtype, const void* h_in, void* h_out,
                                   uint64_t n) {
  return host_scan_entry(kind, op, dtype, h_in, h_out, n, PP_ALGO_COOPERATIVE);
}
pp_status pp_scan_host(pp_scan_kind kind, pp_op op, pp_dtype dtype, const void* h_in, void* h_out, uint64_t n) {
  return host_scan_entry(kind, op, dtype, h_in, h_out, n, PP_ALGO_DECOUPLED);
}

pp_status pp_reduce_host(pp_op op, pp_dtype dtype, const void* h_in, uint64_t n, void* h_result) {
  if (!h_result || !valid_op(op) || !valid_dtype(dtype) || (n > 0 && !h_in)) return PP_ERR_INVALID_ARG;
  if (is_float(dtype) && is_bitop(op)) return PP_ERR_UNSUPPORTED;
  const size_t esz = dtype_size(dtype);
  const uint64_t chunk = kChunkBytes / esz;
  const uint64_t chunks = (n + chunk - 1) / chunk;
  if (chunks > kMaxChunks) return PP_ERR_UNSUPPORTED;
  HostPipeline& p = pipeline();
  std::lock_guard<std::mutex> g(p.mu);
  pp_status c = ensure_pipeline(p);
  if (c != PP_OK) return c;
  // every chunk is reduced on its own while the next one streams in; the
  // per-chunk results are reduced last
  const unsigned char* hi = static_cast<const unsigned char*>(h_in);
  unsigned char* parts = static_cast<unsigned char*>(p.partials);
  for (uint64_t i = 0; i < chunks && c == PP_OK; ++i) {
    const int k = int(i % kSlots);
    const uint64_t off = i * chunk;
    const uint64_t m = n - off < chunk ? n - off : chunk;
    if (i >= uint64_t(kSlots) && cudaStreamWaitEvent(p.h2d, p.slot_free[k], 0) != cudaSuccess) c = PP_ERR_CUDA;
    if (c == PP_OK && cudaMemcpyAsync(p.d_in[k], hi + off * esz, m * esz, cudaMemcpyHostToDevice, p.h2d) != cudaSuccess)
      c = PP_ERR_CUDA;
    if (c == PP_OK && (cudaEventRecord(p.in_ready[k], p.h2d) != cudaSuccess ||
                       cudaStreamWaitEvent(p.comp, p.in_ready[k], 0) != cudaSuccess))
      c = PP_ERR_CUDA;
    if (c == PP_OK) c = to_c(reduce_dispatch(p.comp, op, dtype, p.d_in[k], m, parts + i * esz, nullptr, 0));
    if (c == PP_OK && cudaEventRecord(p.slot_free[k], p.comp) != cudaSuccess) c = PP_ERR_CUDA;
  }
  if (c == PP_OK) c = to_c(reduce_dispatch(p.comp, op, dtype, parts, chunks, p.result, nullptr, 0));
  if (c == PP_OK && cudaMemcpyAsync(h_result, p.result, esz, cudaMemcpyDeviceToHost, p.comp) != cudaSuccess)
    c = PP_ERR_CUDA;
  const cudaError_t e1 = cudaStreamSynchronize(p.h2d);
  const cudaError_t e2 = cudaStreamSynchronize(p.comp);
  if (c != PP_OK) return c;
  if (e1 != cudaSuccess || e2 != cudaSuccess) return PP_ERR_CUDA;
  return to_c(pp::host::read_device_error(p.comp, nullptr));
}

const char* pp_status_string(pp_status status) {
  switch (status) {
    case PP_OK:
      return "ok";
    case PP_ERR_INVALID_ARG:
      return "invalid argument";
    case PP_ERR_UNSUPPORTED:
      return "unsupported operator / type / precision combination";
    case PP_ERR_GRID_TOO_LARGE:
      return "cooperative grid larger than the device can hold co-resident";
    case PP_ERR_TIMEOUT:
      return "a device-side wait timed out";
    case PP_ERR_CUDA:
      return "CUDA runtime error";
    case PP_ERR_WORKSPACE:
      return "workspace too small (or allocation needed during stream capture)";
    case PP_ERR_NO_DEVICE:
      return "no usable CUDA device";
  }
  return "unknown status";
}

pp_status pp_stream_status(pp_stream stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const pp_status st = to_c(pp::host::read_device_error(s, nullptr));
  if (st != PP_OK) return st;
  // an error of the allocation-free scan stays in its scratch until read here
  if (void* scratch = pp::capi::noalloc_scratch_used_on_current_device())
    return to_c(pp::host::read_device_error(s, scratch));
  return PP_OK;
}

pp_status pp_workspace_status(pp_stream stream, void* d_workspace) {
  if (!d_workspace) return PP_ERR_INVALID_ARG;
  return to_c(pp::host::read_device_error(static_cast<cudaStream_t>(stream), d_workspace));
}

pp_status pp_set_timeout_ns(uint64_t ns) {
  if (ns == 0) return PP_ERR_INVALID_ARG;
  pp::host::settings().timeout_ns.store(ns);
  return PP_OK;
}

pp_status pp_set_max_ctas(int ctas) {
  if (ctas < 0) return PP_ERR_INVALID_ARG;
  pp::host::settings().max_ctas.store(ctas);
  return PP_OK;
}

pp_status pp_set_cooperative_window(int tiles_per_cta) {
  if (tiles_per_cta < 0 || tiles_per_cta > 4096) return PP_ERR_INVALID_ARG;
  pp::host::settings().coop_window_tiles.store(tiles_per_cta);
  return PP_OK;
}

pp_status pp_debug_set_skip_tile(long long tile) {
  pp::host::settings().debug_skip_tile.store(tile < 0 ? -1 : tile);
  return PP_OK;
}

pp_status pp_debug_set_lookback_delay(uint32_t max_delay_ns, uint32_t seed) {
  if (max_delay_ns > 1000000u) return PP_ERR_INVALID_ARG;
  pp::host::settings().debug_seed.store(seed);
  pp::host::settings().debug_delay_ns.store(max_delay_ns);
  return PP_OK;
}

pp_status pp_debug_lookback_counters(pp_stream stream, uint64_t* counters) {
  if (!counters) return PP_ERR_INVALID_ARG;
  for (int i = 0; i < 4; ++i) counters[i] = 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  void* ws = pp::host::WorkspaceCache::instance().find(s);
  if (!ws) return to_c(pp::host::from_cuda(cudaStreamSynchronize(s)));
  unsigned long long* d = static_cast<pp::WsHeader*>(ws)->dbg;
  unsigned long long h[4] = {0, 0, 0, 0};
  cudaError_t e = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d, 0, sizeof(h), s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return PP_ERR_CUDA;
  for (int i = 0; i < 4; ++i) counters[i] = h[i];
  return PP_OK;
}

namespace {
Status seg_dispatch(const pp::capi::SegReq& r, pp_dtype dt, int which) {
  using namespace pp::capi;
  switch (dt) {
    case PP_I32:
      return which == 0 ? seg_scan_typed<int32_t>(r) : which == 1 ? seg_reduce_typed<int32_t>(r) : rows_scan_typed<int32_t>(r);
    case PP_U32:
      return which == 0 ? seg_scan_typed<uint32_t>(r) : which == 1 ? seg_reduce_typed<uint32_t>(r) : rows_scan_typed<uint32_t>(r);
    case PP_I64:
      return which == 0 ? seg_scan_typed<int64_t>(r) : which == 1 ? seg_reduce_typed<int64_t>(r) : rows_scan_typed<int64_t>(r);
    case PP_U64:
      return which == 0 ? seg_scan_typed<uint64_t>(r) : which == 1 ? seg_reduce_typed<uint64_t>(r) : rows_scan_typed<uint64_t>(r);
    case PP_F32:
      return which == 0 ? seg_scan_typed<float>(r) : which == 1 ? seg_reduce_typed<float>(r) : rows_scan_typed<float>(r);
    case PP_F64:
      return which == 0 ? seg_scan_typed<double>(r) : which == 1 ? seg_reduce_typed<double>(r) : rows_scan_typed<double>(r);
  }
  return Status::invalid_arg;
}
bool valid_seg_op(pp_op op) { return op == PP_OP_PLUS || op == PP_OP_MINIMUM || op == PP_OP_MAXIMUM; }
}  // namespace

pp_status pp_segmented_scan(pp_stream stream, pp_scan_kind kind, pp_op op, pp_dtype dtype, const void* d_in,
                            void* d_out, uint64_t n, const int64_t* d_offsets, uint64_t num_segments) {
  if (!valid_kind(kind) || !valid_op(op) || !valid_dtype(dtype)) return PP_ERR_INVALID_ARG;
  if (!valid_seg_op(op)) return PP_ERR_UNSUPPORTED;
  if (n == 0 || num_segments == 0) return PP_OK;
  if (!d_in || !d_out || !d_offsets) return PP_ERR_INVALID_ARG;
  pp::capi::SegReq r;
  r.s = static_cast<cudaStream_t>(stream);
  r.exclusive = kind == PP_SCAN_EXCLUSIVE;
  r.op = op;
  r.in = d_in;
  r.out = d_out;
  r.n = n;
  r.offsets = d_offsets;
  r.num_segments = num_segments;
  return to_c(seg_dispatch(r, dtype, 0));
}

pp_status pp_segmented_reduce(pp_stream stream, pp_op op, pp_dtype dtype, const void* d_in, uint64_t n,
                              const int64_t* d_offsets, uint64_t num_segments, void* d_out) {
  if (!valid_op(op) || !valid_dtype(dtype)) return PP_ERR_INVALID_ARG;
  if (!valid_seg_op(op)) return PP_ERR_UNSUPPORTED;
  if (num_segments == 0) return PP_OK;
  if (!d_offsets || !d_out || (n > 0 && !d_in)) return PP_ERR_INVALID_ARG;
  pp::capi::SegReq r;
  r.s = static_cast<cudaStream_t>(stream);
  r.op = op;
  r.in = d_in;
  r.out = d_out;
  r.n = n;
  r.offsets = d_offsets;
  r.num_segments = num_segments;
  return to_c(seg_dispatch(r, dtype, 1));
}

pp_status pp_rows_scan(pp_stream stream, pp_scan_kind kind, pp_op op, pp_dtype dtype, const void* d_in, void* d_out,
                       uint64_t rows, uint64_t cols, int reverse) {
  if (!valid_kind(kind) || !valid_op(op) || !valid_dtype(dtype)) return PP_ERR_INVALID_ARG;
  if (!valid_seg_op(op)) return PP_ERR_UNSUPPORTED;
  if (rows == 0 || cols == 0) return PP_OK;
  if (!d_in || !d_out) return PP_ERR_INVALID_ARG;
  pp::capi::SegReq r;
  r.s = static_cast<cudaStream_t>(stream);
  r.exclusive = kind == PP_SCAN_EXCLUSIVE;
  r.op = op;
  r.in = d_in;
  r.out = d_out;
  r.rows = rows;
  r.cols = cols;
  r.reverse = reverse != 0;
  return to_c(seg_dispatch(r, dtype, 2));
}

const char* pp_version(void) { return "ppgb300 0.1.0 (sm_103a)"; }

}  // extern "C"
