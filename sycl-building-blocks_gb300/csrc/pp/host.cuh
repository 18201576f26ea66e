// Host-side launch layer shared by the C ABI (libppgb300.so) and the
// header-only C++ API (include/parallel_primitives/*.hpp):
//   * per-(device, stream) cached workspaces, grown stream-ordered with
//     cudaMallocAsync and zero-filled once (the epoch protocol then keeps
//     them valid across calls and graph replays without another fill);
//   * occupancy-based persistent grid sizing (replaces get_max_occupancy,
//     include/cooperative_groups.hpp:150-167);
//   * the launch functions for every kernel template.
// Nothing here synchronises the stream except the explicit *_sync helpers.
#pragma once

#include <atomic>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>

#include <cuda_runtime.h>

#include "cooperative_scan.cuh"
#include "decoupled_scan.cuh"
#include "reduce.cuh"
#include "rows.cuh"
#include "scan_policy.cuh"
#include "segmented.cuh"
#include "workspace.cuh"

namespace pp {
namespace host {

enum class Status : int {
  ok = 0,
  invalid_arg = 1,
  unsupported = 2,
  grid_too_large = 3,
  timeout = 4,
  cuda = 5,
  workspace = 6,
  no_device = 7,
};

struct Settings {
  std::atomic<unsigned long long> timeout_ns{1000000000ull};  // every device wait gives up after 1 s
  std::atomic<long long> debug_skip_tile{-1};
  std::atomic<unsigned> debug_delay_ns{0};  // descriptor perturbation knob (0 = off)
  std::atomic<unsigned> debug_seed{0};
  std::atomic<int> max_ctas{0};  // 0 = occupancy x SMs
  std::atomic<int> coop_window_tiles{0};  // cooperative rounds: tiles per CTA per window (0 = ~20 MB windows)
};
inline Settings& settings() {
  static Settings s;
  return s;
}

inline Status from_cuda(cudaError_t e) { return e == cudaSuccess ? Status::ok : Status::cuda; }

struct DeviceInfo {
  int sm_count = 0;
  int smem_optin = 0;
  bool valid = false;
};

inline Status device_info(DeviceInfo& out) {
  static std::mutex mu;
  static std::map<int, DeviceInfo> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return Status::no_device;
  std::lock_guard<std::mutex> g(mu);
  DeviceInfo& d = cache[dev];
  if (!d.valid) {
    if (cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return Status::no_device;
    cudaDeviceGetAttribute(&d.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    d.valid = true;
  }
  out = d;
  return Status::ok;
}

// ---------------------------------------------------------------------------
// Workspace cache: one zero-initialised buffer per (device, stream). Calls on
// the same stream are ordered, so they may share it; calls on different
// streams never do.
class WorkspaceCache {
 public:
  // kind 0: control words + look-back descriptors (only ever holds descriptor
  // words past the header, so stale contents are always older-epoch
  // descriptors or zero); kind 1: general scratch (head bitmaps, ranks).
  Status get(cudaStream_t s, size_t need, void** out, int kind = 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return Status::no_device;
    std::lock_guard<std::mutex> g(mu_);
    Entry& e = map_[Key{dev, reinterpret_cast<uintptr_t>(s), kind}];
    if (e.bytes >= need) {
      *out = e.ptr;
      return Status::ok;
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) return Status::cuda;
    if (cs != cudaStreamCaptureStatusNone) return Status::workspace;  // size it before capturing
    size_t nb = need;
    if (nb < (size_t(1) << 20)) nb = size_t(1) << 20;
    if (nb < e.bytes * 2) nb = e.bytes * 2;
    nb = (nb + 4095) & ~size_t(4095);
    void* p = nullptr;
    if (cudaMallocAsync(&p, nb, s) != cudaSuccess) return Status::cuda;
    if (cudaMemsetAsync(p, 0, nb, s) != cudaSuccess) return Status::cuda;
    if (e.ptr) cudaFreeAsync(e.ptr, s);
    e.ptr = p;
    e.bytes = nb;
    *out = p;
    return Status::ok;
  }
  // Returns the control workspace of this stream if one exists.
  void* find(cudaStream_t s) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> g(mu_);
    auto it = map_.find(Key{dev, reinterpret_cast<uintptr_t>(s), 0});
    return it == map_.end() ? nullptr : it->second.ptr;
  }
  static WorkspaceCache& instance() {
    static WorkspaceCache* c = new WorkspaceCache();  // never destroyed: outlives CUDA teardown
    return *c;
  }

 private:
  struct Entry {
    void* ptr = nullptr;
    size_t bytes = 0;
  };
  struct Key {
    int dev;
    uintptr_t stream;
    int kind;
    bool operator<(const Key& o) const {
      if (dev != o.dev) return dev < o.dev;
      if (stream != o.stream) return stream < o.stream;
      return kind < o.kind;
    }
  };
  std::mutex mu_;
  std::map<Key, Entry> map_;
};

// A workspace either supplied by the caller (must have been zero-filled once
// before its first use, and must not be shared by calls that overlap on the
// GPU) or taken from the per-stream cache.
struct Ws {
  WsHeader* hdr = nullptr;
  void* aux = nullptr;
  uint64_t* desc = nullptr;
};

inline Status acquire_ws(cudaStream_t s, size_t need, void* user_ws, size_t user_bytes, Ws& w) {
  void* p = user_ws;
  if (p) {
    if (user_bytes < need) return Status::workspace;
    if (reinterpret_cast<uintptr_t>(p) & 255u) return Status::invalid_arg;
  } else {
    Status st = WorkspaceCache::instance().get(s, need, &p);
    if (st != Status::ok) return st;
  }
  w.hdr = static_cast<WsHeader*>(p);
  w.aux = static_cast<unsigned char*>(p) + kHeaderBytes;
  w.desc = reinterpret_cast<uint64_t*>(static_cast<unsigned char*>(p) + kDescOffset);
  return Status::ok;
}

// Copies the sticky device error word of a workspace to the host, clears it
// and returns it as a Status. Synchronises `s`.
inline Status read_device_error(cudaStream_t s, void* ws) {
  if (!ws) {
    ws = WorkspaceCache::instance().find(s);
    if (!ws) return from_cuda(cudaStreamSynchronize(s));
  }
  WsHeader* h = static_cast<WsHeader*>(ws);
  unsigned int err = 0;
  cudaError_t e = cudaMemcpyAsync(&err, &h->error, sizeof(err), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return Status::cuda;
  if (err != 0) {
    const unsigned int zero = 0;
    cudaMemcpyAsync(&h->error, &zero, sizeof(zero), cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);
    return static_cast<Status>(err);
  }
  return Status::ok;
}

template <class K>
inline Status prepare_kernel(K kernel, int threads, size_t smem, int& blocks_per_sm) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, int> cache;  // (kernel, device) -> blocks/SM
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return Status::no_device;
  std::lock_guard<std::mutex> g(mu);
  auto key = std::make_pair(reinterpret_cast<const void*>(kernel), dev);
  auto it = cache.find(key);
  if (it != cache.end()) {
    blocks_per_sm = it->second;
    return Status::ok;
  }
  if (smem > 48 * 1024) {
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess)
      return Status::cuda;
  }
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, threads, smem) != cudaSuccess) return Status::cuda;
  if (b < 1) return Status::unsupported;
  cache[key] = b;
  blocks_per_sm = b;
  return Status::ok;
}

// ---------------------------------------------------------------------------
// Decoupled look-back scan.
// Policy classes of the tuning table.
enum class TuneKind { int4, float4, wide8, float8, compensated, fp64_carry };
template <class Pol>
struct tune_kind {
  static constexpr TuneKind value = TuneKind::int4;
};
template <class T, class Op>
struct tune_kind<PlainScan<T, Op>> {
  static constexpr TuneKind value =
      std::is_same_v<T, double>
          ? TuneKind::float8
          : (sizeof(T) == 8 ? TuneKind::wide8 : (std::is_same_v<T, float> ? TuneKind::float4 : TuneKind::int4));
};
template <>
struct tune_kind<CompensatedF32> {
  static constexpr TuneKind value = TuneKind::compensated;
};
template <>
struct tune_kind<F64CarryF32> {
  static constexpr TuneKind value = TuneKind::fp64_carry;
};

// Staged-kernel configuration per policy class, from sweeps of 2^32-byte
// inputs on GB300 (all: 3 stages, one CTA per SM):
//   int4         striped 64 KB tiles, ticket one stage life ahead, one poll of
//                4 windows of 32 descriptors;
//   float4       rows of 9 chunks (72 KB), late ticket, two polls of one window;
//   wide8        rows of 7 chunks over 20 warps (70 KB), late ticket, two polls
//                of one window, a store warp;
//   float8       rows of 9 chunks over 14 warps (63 KB), late ticket, two polls,
//                a store warp: FP64 additions, not HBM, bound double scans on
//                this part, and the row chains need the fewest of them;
//   compensated  as wide8 (the arithmetic, not the stores, bounds this one:
//                with the store warp the compute warps never wait for stores);
//   fp64_carry   as float4, with a store warp.
template <class Pol>
struct DecoupledTuning {
  static constexpr TuneKind K = tune_kind<Pol>::value;
  static constexpr bool kRows = K == TuneKind::float4 || K == TuneKind::float8 || K == TuneKind::compensated ||
                                K == TuneKind::fp64_carry;
  static constexpr bool k20 = K == TuneKind::compensated || K == TuneKind::wide8;
  static constexpr int NC = k20 ? 20 : (K == TuneKind::float8 ? 14 : 16);  // compute warps
  static constexpr int CH = K == TuneKind::int4 ? 8 : (k20 ? 7 : 9);        // chunks per lane
  static constexpr int STAGES = 3;  // shared-memory ring depth
  static constexpr int LBW = K == TuneKind::int4 ? 4 : 1;  // windows of 32 descriptors per poll
  static constexpr int LAY = (kRows || K == TuneKind::wide8) ? 2 : 0;                  // striped / rows
  static constexpr int TK = K == TuneKind::int4 ? 0 : 2;                  // when tickets are drawn
  static constexpr unsigned PG = K == TuneKind::int4 ? 0u : 250u;         // second poll delay (ns)
  // stores: a store warp writes finished tiles back by bulk copy (compensated,
  // FP64 carry, 8-byte integers), else the compute warps store striped
  static constexpr int BS = (K == TuneKind::compensated || K == TuneKind::fp64_carry || K == TuneKind::wide8 ||
                             K == TuneKind::float8)
                                ? 2
                                : 0;
  static constexpr int GEN_NC = 8;
  static constexpr int GEN_IPT = 8;
};
template <class Pol>
using StagedFor = StagedCfg<Pol, DecoupledTuning<Pol>::NC, DecoupledTuning<Pol>::CH, DecoupledTuning<Pol>::STAGES,
                            DecoupledTuning<Pol>::LBW, DecoupledTuning<Pol>::LAY,
                            (DecoupledTuning<Pol>::BS == 2 ? 1 : 0)>;

// The staged (bulk-copy) kernel takes any naturally aligned pointers of an
// element type whose size divides 16 bytes; the tile grid is shifted so that
// tile starts fall on 16-byte boundaries of the input.
template <class Pol>
inline bool tma_path_ok(const void* in, const void* out) {
  using in_t = typename Pol::in_t;
  if constexpr (16 % sizeof(in_t) != 0 || sizeof(typename Pol::out_t) != sizeof(in_t)) {
    return false;
  } else {
    return ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) % sizeof(in_t)) == 0;
  }
}

// Phantom elements in front of `in` up to the previous 16-byte boundary.
template <class Pol>
inline int staged_head(const void* in) {
  return int((reinterpret_cast<uintptr_t>(in) & 15u) / sizeof(typename Pol::in_t));
}

template <class Pol>
inline uint64_t decoupled_tiles(uint64_t n, const void* in, const void* out) {
  using Tn = DecoupledTuning<Pol>;
  if constexpr (16 % sizeof(typename Pol::in_t) == 0) {
    if (tma_path_ok<Pol>(in, out)) {
      const uint64_t tile = StagedFor<Pol>::TILE;
      return (n + uint64_t(staged_head<Pol>(in)) + tile - 1) / tile;
    }
  }
  const uint64_t tile = DecoupledGenericCfg<Pol, Tn::GEN_NC, Tn::GEN_IPT>::TILE;
  return (n + tile - 1) / tile;
}

template <class Pol>
inline size_t decoupled_workspace_bytes(uint64_t n, const void* in, const void* out) {
  return workspace_bytes_for_desc_words(decoupled_tiles<Pol>(n, in, out) * desc_codec<typename Pol::carry_t>::W);
}

// Pointers must be aligned to the element type (element loads and stores).
template <class T>
inline bool type_aligned(const void* p) {
  return (reinterpret_cast<uintptr_t>(p) % alignof(T)) == 0;
}

// grid_ctas: 0 = persistent grid (occupancy x SMs); otherwise the CTA count
// (1 gives the single work-group scan of scan.hpp:125-130). Element types
// whose size does not divide 16 bytes take the register-tile kernel.
template <class Pol>
inline Status decoupled_scan(cudaStream_t s, const void* in, void* out, uint64_t n, bool exclusive,
                             void* user_ws = nullptr, size_t user_ws_bytes = 0, int grid_ctas = 0) {
  if (n == 0) return Status::ok;
  if (!in || !out) return Status::invalid_arg;
  if (!type_aligned<typename Pol::in_t>(in) || !type_aligned<typename Pol::out_t>(out)) return Status::invalid_arg;
  using Tn = DecoupledTuning<Pol>;
  DeviceInfo di;
  Status st = device_info(di);
  if (st != Status::ok) return st;
  Ws w;
  st = acquire_ws(s, decoupled_workspace_bytes<Pol>(n, in, out), user_ws, user_ws_bytes, w);
  if (st != Status::ok) return st;
  ScanArgs a{};
  a.in = in;
  a.out = out;
  a.n = n;
  a.hdr = w.hdr;
  a.desc = w.desc;
  a.timeout_ns = settings().timeout_ns.load();
  a.debug_skip_tile = settings().debug_skip_tile.load();
  a.debug_delay_ns = settings().debug_delay_ns.load();
  a.debug_seed = settings().debug_seed.load();
  a.exclusive = exclusive ? 1 : 0;
  a.head = 0;
  const int cap = grid_ctas > 0 ? grid_ctas : settings().max_ctas.load();
  if constexpr (16 % sizeof(typename Pol::in_t) == 0) {
    if (tma_path_ok<Pol>(in, out)) {
      using Cfg = StagedFor<Pol>;
      auto k = decoupled_staged_kernel<Pol, Tn::NC, Tn::CH, Tn::STAGES, Tn::LBW, Tn::LAY, Tn::TK, Tn::PG, Tn::BS>;
      int bps = 0;
      st = prepare_kernel(k, Cfg::THREADS, Cfg::SMEM, bps);
      if (st != Status::ok) return st;
      a.head = staged_head<Pol>(in);
      const uint64_t ntiles = decoupled_tiles<Pol>(n, in, out);
      uint64_t grid = uint64_t(bps) * di.sm_count;
      if (cap > 0 && uint64_t(cap) < grid) grid = cap;
      if (ntiles < grid) grid = ntiles;
      k<<<unsigned(grid), Cfg::THREADS, Cfg::SMEM, s>>>(a);
      return from_cuda(cudaGetLastError());
    }
  }
  using Cfg = DecoupledGenericCfg<Pol, Tn::GEN_NC, Tn::GEN_IPT>;
  auto k = decoupled_generic_kernel<Pol, Tn::GEN_NC, Tn::GEN_IPT>;
  int bps = 0;
  st = prepare_kernel(k, Cfg::THREADS, 0, bps);
  if (st != Status::ok) return st;
  const uint64_t ntiles = (n + Cfg::TILE - 1) / Cfg::TILE;
  uint64_t grid = uint64_t(bps) * di.sm_count;
  if (cap > 0 && uint64_t(cap) < grid) grid = cap;
  if (ntiles < grid) grid = ntiles;
  k<<<unsigned(grid), Cfg::THREADS, 0, s>>>(a);
  return from_cuda(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// Cooperative grid-barrier scan.
template <class Pol>
struct CoopTuning {
  static constexpr int NC = 8;
  static constexpr int CH = 4;
};

// Workspace of the cooperative scan: the staged kernel keeps one record per
// tile (its aggregate and segment prefixes) between the two reads of a
// window; the register-tile kernel needs the header and block slots only.
template <class Pol>
inline size_t cooperative_workspace_bytes(uint64_t n, const void* in, const void* out) {
  if constexpr (16 % sizeof(typename Pol::in_t) == 0) {
    if (tma_path_ok<Pol>(in, out)) {
      using Cfg = StagedFor<Pol>;
      const uint64_t ntiles = (n + uint64_t(staged_head<Pol>(in)) + Cfg::TILE - 1) / Cfg::TILE;
      return workspace_bytes_for_desc_words(ntiles * (Cfg::REC_BYTES / 8));
    }
  }
  return workspace_bytes_for_desc_words(0);
}

// Window of the cooperative rounds: about this many input bytes per window
// (two tiles per CTA with 64-72 KB tiles on 152 SMs). The window being
// scanned and the one being reduced stay in L2 next to the streaming output;
// on GB300 2^30-element scans ran fastest with 20 MB windows (5.8 TB/s at
// 2n bytes), 10 MB windows pay the window barrier twice as often (4.9 TB/s)
// and 30-60 MB windows lose the second read to L2 misses (5.3-4.7 TB/s).
constexpr uint64_t kCoopWindowBytes = 20ull << 20;

// grid_ctas: 0 = every block the device holds co-resident; a larger request
// than that fails with grid_too_large (the reference's perform_check,
// include/cooperative_groups.hpp:65-76). Element-aligned data of element
// sizes dividing 16 bytes take the staged kernel in cooperative rounds
// (window_tiles tiles per CTA per window, 0 = about kCoopWindowBytes per
// window; l2_keep: evict_last instead of evict_normal for a window's first
// read, which measured the same); the rest take the register-tile kernel
// (3n traffic).
template <class Pol>
inline Status cooperative_scan(cudaStream_t s, const void* in, void* out, uint64_t n, bool exclusive,
                               void* user_ws = nullptr, size_t user_ws_bytes = 0, int grid_ctas = 0,
                               int window_tiles = 0, int l2_keep = 0) {
  if (n == 0) return Status::ok;
  if (!in || !out) return Status::invalid_arg;
  if (!type_aligned<typename Pol::in_t>(in) || !type_aligned<typename Pol::out_t>(out)) return Status::invalid_arg;
  if constexpr (16 % sizeof(typename Pol::in_t) == 0) {
    if (tma_path_ok<Pol>(in, out)) {
      using Tn = DecoupledTuning<Pol>;
      using Cfg = StagedCfg<Pol, Tn::NC, Tn::CH, Tn::STAGES, Tn::LBW, Tn::LAY, (Tn::BS == 2 ? 1 : 0), 1>;
      DeviceInfo di;
      Status st = device_info(di);
      if (st != Status::ok) return st;
      auto k = decoupled_staged_kernel<Pol, Tn::NC, Tn::CH, Tn::STAGES, Tn::LBW, Tn::LAY, Tn::TK, Tn::PG, Tn::BS,
                                       NoTrace, 1>;
      int bps = 0;
      st = prepare_kernel(k, Cfg::THREADS, Cfg::SMEM, bps);
      if (st != Status::ok) return st;
      const uint64_t max_grid = uint64_t(bps) * di.sm_count;
      uint64_t grid = max_grid;
      if (grid_ctas > 0) {
        if (uint64_t(grid_ctas) > max_grid) return Status::grid_too_large;
        grid = grid_ctas;
      } else if (settings().max_ctas.load() > 0 && uint64_t(settings().max_ctas.load()) < grid) {
        grid = settings().max_ctas.load();
      }
      const int head = staged_head<Pol>(in);
      const uint64_t ntiles = (n + uint64_t(head) + Cfg::TILE - 1) / Cfg::TILE;
      if (ntiles < grid) grid = ntiles;
      if (grid > uint64_t(kMaxPartials / 4)) grid = kMaxPartials / 4;  // 4 window slots per CTA
      if (window_tiles <= 0) window_tiles = settings().coop_window_tiles.load();
      uint64_t kt = window_tiles > 0 ? uint64_t(window_tiles)
                                     : (kCoopWindowBytes + grid * Cfg::TILE_BYTES / 2) / (grid * Cfg::TILE_BYTES);
      if (kt < 1) kt = 1;
      Ws w;
      st = acquire_ws(s, cooperative_workspace_bytes<Pol>(n, in, out), user_ws, user_ws_bytes, w);
      if (st != Status::ok) return st;
      ScanArgs a{};
      a.in = in;
      a.out = out;
      a.n = n;
      a.hdr = w.hdr;
      a.desc = w.desc;
      a.timeout_ns = settings().timeout_ns.load();
      a.debug_skip_tile = settings().debug_skip_tile.load();
      a.exclusive = exclusive ? 1 : 0;
      a.head = head;
      a.coop_kt = int(kt);
      a.coop_l2 = l2_keep;
      a.coop_aggs = w.aux;
      void* params[] = {&a};
      return from_cuda(cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(k), dim3(unsigned(grid)),
                                                   dim3(Cfg::THREADS), params, Cfg::SMEM, s));
    }
  }
  using Tn = CoopTuning<Pol>;
  using Cfg = CoopCfg<Pol, Tn::NC, Tn::CH>;
  DeviceInfo di;
  Status st = device_info(di);
  if (st != Status::ok) return st;
  auto k = cooperative_scan_kernel<Pol, Tn::NC, Tn::CH>;
  int bps = 0;
  st = prepare_kernel(k, Cfg::THREADS, 0, bps);
  if (st != Status::ok) return st;
  const uint64_t max_grid = uint64_t(bps) * di.sm_count;
  uint64_t grid = max_grid;
  if (grid_ctas > 0) {
    if (uint64_t(grid_ctas) > max_grid) return Status::grid_too_large;
    grid = grid_ctas;
  } else if (settings().max_ctas.load() > 0 && uint64_t(settings().max_ctas.load()) < grid) {
    grid = settings().max_ctas.load();
  }
  const uint64_t ntiles = (n + Cfg::TILE - 1) / Cfg::TILE;
  if (ntiles < grid) grid = ntiles;
  if (grid > uint64_t(kMaxPartials)) grid = kMaxPartials;
  Ws w;
  st = acquire_ws(s, workspace_bytes_for_desc_words(0), user_ws, user_ws_bytes, w);
  if (st != Status::ok) return st;
  CoopArgs ca{};
  ca.s.in = in;
  ca.s.out = out;
  ca.s.n = n;
  ca.s.hdr = w.hdr;
  ca.s.desc = w.desc;
  ca.s.timeout_ns = settings().timeout_ns.load();
  ca.s.debug_skip_tile = -1;
  ca.s.exclusive = exclusive ? 1 : 0;
  ca.block_aggs = w.aux;
  void* params[] = {&ca};
  return from_cuda(cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(k), dim3(unsigned(grid)),
                                               dim3(Cfg::THREADS), params, 0, s));
}

// ---------------------------------------------------------------------------
// Reduction: result written to device memory (d_result, one T).
template <class T, class Op>
struct ReduceTuning {
  static constexpr int BLOCK = 512;
  static constexpr int UNROLL = 4;
};

template <class T, class Op>
inline Status reduce(cudaStream_t s, const T* in, uint64_t n, T* d_result, void* user_ws = nullptr,
                     size_t user_ws_bytes = 0) {
  if (!d_result || (n > 0 && !in)) return Status::invalid_arg;
  if (!type_aligned<T>(d_result) || (n > 0 && !type_aligned<T>(in))) return Status::invalid_arg;
  using Tn = ReduceTuning<T, Op>;
  DeviceInfo di;
  Status st = device_info(di);
  if (st != Status::ok) return st;
  auto k = reduce_kernel<T, Op, Tn::BLOCK, Tn::UNROLL>;
  int bps = 0;
  st = prepare_kernel(k, Tn::BLOCK, 0, bps);
  if (st != Status::ok) return st;
  Ws w;
  st = acquire_ws(s, workspace_bytes_for_desc_words(0), user_ws, user_ws_bytes, w);
  if (st != Status::ok) return st;
  constexpr int V = (16 % sizeof(T) == 0) ? int(16 / sizeof(T)) : 1;
  uint64_t grid = uint64_t(bps) * di.sm_count;
  const int cap = settings().max_ctas.load();
  if (cap > 0 && uint64_t(cap) < grid) grid = cap;
  // no more blocks than there are vectors to hand out
  const uint64_t work_blocks = (n / V + Tn::BLOCK - 1) / Tn::BLOCK;
  if (work_blocks < grid) grid = work_blocks;
  if (grid < 1) grid = 1;
  if (grid > uint64_t(kMaxPartials)) grid = kMaxPartials;
  ReduceArgs a{};
  a.in = in;
  a.n = n;
  a.result = d_result;
  a.hdr = w.hdr;
  a.partials = w.aux;
  k<<<unsigned(grid), Tn::BLOCK, 0, s>>>(a);
  return from_cuda(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// Batched segmented scan / reduce and row scans (segmented.cuh).
#include "seg_tuned.inc"
// Variant of the segmented kernel. CSR forward scans and reductions take the
// autotuned variant (seg_tuned.inc, written by ppautotune.py) of their payload
// type and segment-length class (mean length n / S >= kSegLongMean: "long");
// unsigned payloads take their signed counterpart's. Row scans that fall back
// to this kernel (uniform heads, either direction) take 16 warps of 8 16-byte
// chunks.
constexpr uint64_t kSegLongMean = 512;
template <int LAY_, int NC_, int CH_, int VB_, class T, int LBW_ = 4, int BS_ = 0>
struct SegVariant {
  static constexpr int LAY = LAY_, NC = NC_, CH = CH_, VB = VB_, LBW = LBW_, BS = BS_;
  static constexpr int TILE_BYTES = NC * 32 * CH * VB;
  static constexpr int ST0 = 196608 / TILE_BYTES;
  static constexpr int STAGES = LAY == 2 ? 3 : (ST0 < 2 ? 2 : (ST0 > 8 ? 8 : ST0));
};
#define PP_SEG_VARIANT(DT, LEN)                                                                              \
  SegVariant<PP_SEG_##DT##_##LEN##_LAY, PP_SEG_##DT##_##LEN##_NC, PP_SEG_##DT##_##LEN##_CH, PP_SEG_##DT##_##LEN##_VB, \
             T, PP_SEG_##DT##_##LEN##_LBW, PP_SEG_##DT##_##LEN##_BS>
template <class T, bool LONG>
using SegTunedCsr = std::conditional_t<
    std::is_floating_point_v<T>,
    std::conditional_t<sizeof(T) == 4,
                       std::conditional_t<LONG, PP_SEG_VARIANT(F32, LONG), PP_SEG_VARIANT(F32, SHORT)>,
                       std::conditional_t<LONG, PP_SEG_VARIANT(F64, LONG), PP_SEG_VARIANT(F64, SHORT)>>,
    std::conditional_t<sizeof(T) == 4,
                       std::conditional_t<LONG, PP_SEG_VARIANT(I32, LONG), PP_SEG_VARIANT(I32, SHORT)>,
                       std::conditional_t<LONG, PP_SEG_VARIANT(I64, LONG), PP_SEG_VARIANT(I64, SHORT)>>>;
#undef PP_SEG_VARIANT
template <class T>
using SegUniform = SegVariant<0, 16, 8, 16, T>;
template <class Tn, class T, class Op>
using SegCfgOf = SegCfg<SegPlainScan<T, Op>, Tn::NC, Tn::CH, Tn::STAGES, Tn::LBW, Tn::VB, Tn::LAY>;

// Control workspace: header + descriptors (room for both the segmented pass
// and the rank scan of a reduce). Scratch workspace (a separate buffer, so
// descriptor memory never holds anything but descriptor words): head bitmap,
// nonempty flags, ranks, rank -> segment map.
struct SegWsLayout {
  size_t control_bytes;
  size_t bitmap_off, bitmap_bytes, nonempty_off, rank_off, rank_out_off;
  size_t tile_base_off, tile_rec_off, tile_rec_bytes;  // reduce: per-tile base ranks and records
  size_t chunk_v_off, chunk_c_off;                     // reduce: per-chunk summaries of the records
  size_t block_count_off;                              // reduce: non-empty segments per pre-pass block
  size_t scratch_bytes;
};

// Blocks of the reduce's pre-passes over segments (segment_heads_count_kernel,
// segment_rank_kernel): at most 1,024 blocks of 256 threads, each thread a run
// of per_thread consecutive segments.
struct SegPrepassGrid {
  uint64_t blocks, per_thread;
};
inline SegPrepassGrid seg_prepass_grid(uint64_t num_segments) {
  const uint64_t threads = num_segments < 262144 ? (num_segments + 255) / 256 * 256 : 262144;
  SegPrepassGrid g;
  g.per_thread = (num_segments + threads - 1) / threads;
  if (g.per_thread < 1) g.per_thread = 1;
  const uint64_t used_threads = (num_segments + g.per_thread - 1) / g.per_thread;
  g.blocks = (used_threads + 255) / 256;
  if (g.blocks < 1) g.blocks = 1;
  return g;
}
template <class T, class Op>
inline SegWsLayout seg_ws_layout(uint64_t n, uint64_t num_segments, bool csr, bool reduce) {
  // sized for every variant a call may take
  using C0 = SegCfgOf<SegUniform<T>, T, Op>;
  using C1 = SegCfgOf<SegTunedCsr<T, true>, T, Op>;
  using C2 = SegCfgOf<SegTunedCsr<T, false>, T, Op>;
  constexpr uint64_t t01 = uint64_t(C0::TILE < C1::TILE ? C0::TILE : C1::TILE);
  constexpr uint64_t kTile = t01 < uint64_t(C2::TILE) ? t01 : uint64_t(C2::TILE);
  constexpr uint64_t m01 = uint64_t(C0::MAP_BYTES > C1::MAP_BYTES ? C0::MAP_BYTES : C1::MAP_BYTES);
  constexpr uint64_t kMap = m01 > uint64_t(C2::MAP_BYTES) ? m01 : uint64_t(C2::MAP_BYTES);
  SegWsLayout L{};
  const uint64_t ntiles = (n + kTile - 1) / kTile;
  uint64_t words = ntiles * desc_codec<typename SegPlainScan<T, Op>::carry_t>::W;
  if (reduce) {
    const uint64_t rt = (num_segments + StagedFor<PlainScan<uint32_t, plus>>::TILE - 1) /
                        StagedFor<PlainScan<uint32_t, plus>>::TILE;
    if (rt > words) words = rt;
  }
  L.control_bytes = workspace_bytes_for_desc_words(words);
  size_t off = 0;
  L.bitmap_off = off;
  L.bitmap_bytes = csr ? align_up(((n + 127) / 128) * 16 + kMap, 256) : 0;
  off += L.bitmap_bytes;
  L.nonempty_off = off;
  if (reduce) off += align_up(num_segments * 4, 256);
  L.rank_off = off;
  if (reduce) off += align_up(num_segments * 4, 256);
  L.rank_out_off = off;  // reduce: totals by rank
  if (reduce) off += align_up(num_segments * sizeof(T), 256);
  L.tile_base_off = off;  // reduce: sized for the smallest tile of any variant
  if (reduce) off += align_up(ntiles * 4, 256);
  L.tile_rec_off = off;
  L.tile_rec_bytes = reduce ? ntiles * sizeof(SegTileRec<T>) : 0;
  off += align_up(L.tile_rec_bytes, 256);
  const uint64_t nchunks = (ntiles + kSegChunk - 1) / kSegChunk;
  L.chunk_v_off = off;
  if (reduce) off += align_up(nchunks * sizeof(T), 256);
  L.chunk_c_off = off;
  if (reduce) off += align_up(nchunks * 4, 256);
  L.block_count_off = off;
  if (reduce) off += align_up(1024 * 4, 256);
  L.scratch_bytes = off;
  return L;
}

inline Status acquire_scratch(cudaStream_t s, size_t need, unsigned char** out) {
  void* p = nullptr;
  Status st = WorkspaceCache::instance().get(s, need ? need : 256, &p, 1);
  *out = static_cast<unsigned char*>(p);
  return st;
}

// What a CSR reduction adds to the main launch: per-tile base ranks before it
// (from the offsets and the rank scan of the non-empty flags), the per-tile
// records zero-filled, and the fix-up of segments that cross tiles after it.
struct SegReduceExtra {
  const int64_t* offsets = nullptr;
  const uint32_t* nonempty = nullptr;
  uint32_t* rank = nullptr;
  const uint32_t* block_count = nullptr;  // from segment_heads_count_kernel
  uint64_t prepass_blocks = 0, per_thread = 0;
  uint32_t* tile_base = nullptr;
  void* tile_rec = nullptr;
  size_t tile_rec_bytes = 0;
  void* chunk_v = nullptr;
  uint32_t* chunk_c = nullptr;
};

template <class Tn, class Pol, class Heads, bool REVERSE, bool REDUCE, bool SKIP = false>
inline Status launch_segmented_variant(cudaStream_t s, const SegArgs& a0, uint64_t num_segments = 0,
                                       const SegReduceExtra* rx = nullptr) {
  constexpr int BS = REDUCE ? 0 : Tn::BS;  // the store warp serves scans only
  using Cfg = SegCfg<Pol, Tn::NC, Tn::CH, Tn::STAGES, Tn::LBW, Tn::VB, Tn::LAY, (BS == 2 ? 1 : 0)>;
  auto k = segmented_staged_kernel<Pol, Tn::NC, Tn::CH, Tn::STAGES, Tn::LBW, Heads, REVERSE, REDUCE, Tn::VB, Tn::LAY,
                                   BS, SKIP && Tn::LAY == 2>;
  DeviceInfo di;
  Status st = device_info(di);
  if (st != Status::ok) return st;
  int bps = 0;
  st = prepare_kernel(k, Cfg::THREADS, Cfg::SMEM, bps);
  if (st != Status::ok) return st;
  const uint64_t ntiles = (a0.s.n + Cfg::TILE - 1) / Cfg::TILE;
  SegArgs a = a0;
  if constexpr (REDUCE) {
    if (!rx || rx->tile_rec_bytes < ntiles * sizeof(SegTileRec<typename Pol::in_t>)) return Status::workspace;
    a.tile_base = rx->tile_base;
    a.tile_rec = rx->tile_rec;
    // ranks of the non-empty segments and the base rank of every tile of this variant
    segment_rank_kernel<<<unsigned(rx->prepass_blocks), 256, 0, s>>>(rx->offsets, rx->nonempty, num_segments,
                                                                       a0.s.n, rx->per_thread, rx->block_count,
                                                                       uint64_t(Cfg::TILE), rx->rank, rx->tile_base);
    if (cudaGetLastError() != cudaSuccess) return Status::cuda;
    if (cudaMemsetAsync(rx->tile_rec, 0, ntiles * sizeof(SegTileRec<typename Pol::in_t>), s) != cudaSuccess)
      return Status::cuda;
  }
  uint64_t grid = uint64_t(bps) * di.sm_count;
  const int cap = settings().max_ctas.load();
  if (cap > 0 && uint64_t(cap) < grid) grid = cap;
  if (ntiles < grid) grid = ntiles;
  k<<<unsigned(grid), Cfg::THREADS, Cfg::SMEM, s>>>(a);
  if (cudaGetLastError() != cudaSuccess) return Status::cuda;
  if constexpr (REDUCE) {
    using T = typename Pol::in_t;
    using Op = decltype(Pol{}.op);
    const auto* rec = static_cast<const SegTileRec<T>*>(rx->tile_rec);
    const uint64_t nchunks = (ntiles + kSegChunk - 1) / kSegChunk;
    segment_chunk_kernel<T, Op><<<unsigned(nchunks), 256, 0, s>>>(rec, ntiles, static_cast<T*>(rx->chunk_v),
                                                                  rx->chunk_c);
    if (cudaGetLastError() != cudaSuccess) return Status::cuda;
    const unsigned fgrid = unsigned((ntiles + 7) / 8 < 4096 ? (ntiles + 7) / 8 : 4096);  // a warp per tile
    segment_fixup_kernel<T, Op><<<fgrid, 256, 0, s>>>(rec, ntiles, static_cast<const T*>(rx->chunk_v), rx->chunk_c,
                                                      rx->tile_base, static_cast<T*>(a.rank_out));
    if (cudaGetLastError() != cudaSuccess) return Status::cuda;
  }
  return Status::ok;
}

template <class Pol, class Heads, bool REVERSE, bool REDUCE>
inline Status launch_segmented(cudaStream_t s, const SegArgs& a, uint64_t num_segments = 0,
                               const SegReduceExtra* rx = nullptr) {
  using T = typename Pol::in_t;
  if constexpr (Heads::kBitmap && !REVERSE) {
    const bool long_segments = num_segments == 0 || a.s.n / num_segments >= kSegLongMean;
    // long segments: reductions take the head-free branch (measured: 5-11 %
    // faster at mean lengths of 900-5,900; scans gain nothing from it, and
    // both lose 2-8 % with it at mean lengths below 100)
    if (long_segments)
      return launch_segmented_variant<SegTunedCsr<T, true>, Pol, Heads, REVERSE, REDUCE, REDUCE>(s, a, num_segments,
                                                                                                rx);
    return launch_segmented_variant<SegTunedCsr<T, false>, Pol, Heads, REVERSE, REDUCE>(s, a, num_segments, rx);
  } else {
    static_assert(!REDUCE, "reductions take CSR segments");
    return launch_segmented_variant<SegUniform<T>, Pol, Heads, REVERSE, REDUCE>(s, a);
  }
}

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// CSR segmented scan: offsets[0] = 0, offsets[num_segments] = n, nondecreasing.
template <class T, class Op>
inline Status segmented_scan(cudaStream_t s, const T* in, T* out, uint64_t n, const int64_t* offsets,
                             uint64_t num_segments, bool exclusive, void* user_ws = nullptr,
                             size_t user_ws_bytes = 0) {
  if (n == 0 || num_segments == 0) return Status::ok;
  if (!in || !out || !offsets) return Status::invalid_arg;
  if (!aligned16(in) || !aligned16(out)) return Status::invalid_arg;
  if (reinterpret_cast<uintptr_t>(offsets) & 7u) return Status::invalid_arg;
  const SegWsLayout L = seg_ws_layout<T, Op>(n, num_segments, true, false);
  Ws w;
  Status st = acquire_ws(s, L.control_bytes, user_ws, user_ws_bytes, w);
  if (st != Status::ok) return st;
  unsigned char* base = nullptr;
  st = acquire_scratch(s, L.scratch_bytes, &base);
  if (st != Status::ok) return st;
  uint32_t* heads = reinterpret_cast<uint32_t*>(base + L.bitmap_off);
  if (cudaMemsetAsync(heads, 0, L.bitmap_bytes, s) != cudaSuccess) return Status::cuda;
  const unsigned pre_grid = unsigned((num_segments + 255) / 256 < 1024 ? (num_segments + 255) / 256 : 1024);
  segment_heads_kernel<T, Op><<<pre_grid, 256, 0, s>>>(offsets, num_segments, n, heads, nullptr, nullptr);
  if (cudaGetLastError() != cudaSuccess) return Status::cuda;
  SegArgs a{};
  a.s.in = in;
  a.s.out = out;
  a.s.n = n;
  a.s.hdr = w.hdr;
  a.s.desc = w.desc;
  a.s.timeout_ns = settings().timeout_ns.load();
  a.s.debug_skip_tile = -1;
  a.s.exclusive = exclusive ? 1 : 0;
  a.heads = heads;
  return launch_segmented<SegPlainScan<T, Op>, CsrHeads, false, false>(s, a, num_segments);
}

// CSR segmented reduce: out[s] = op-reduction of segment s (identity if empty).
template <class T, class Op>
inline Status segmented_reduce(cudaStream_t s, const T* in, uint64_t n, const int64_t* offsets,
                               uint64_t num_segments, T* out, void* user_ws = nullptr, size_t user_ws_bytes = 0) {
  if (num_segments == 0) return Status::ok;
  if (!offsets || !out || (n > 0 && !in)) return Status::invalid_arg;
  if (n > 0 && !aligned16(in)) return Status::invalid_arg;
  if (!type_aligned<T>(out) || (reinterpret_cast<uintptr_t>(offsets) & 7u)) return Status::invalid_arg;
  const SegWsLayout L = seg_ws_layout<T, Op>(n, num_segments, true, true);
  Ws w;
  Status st = acquire_ws(s, L.control_bytes, user_ws, user_ws_bytes, w);
  if (st != Status::ok) return st;
  unsigned char* base = nullptr;
  st = acquire_scratch(s, L.scratch_bytes, &base);
  if (st != Status::ok) return st;
  uint32_t* heads = reinterpret_cast<uint32_t*>(base + L.bitmap_off);
  uint32_t* nonempty = reinterpret_cast<uint32_t*>(base + L.nonempty_off);
  uint32_t* rank = reinterpret_cast<uint32_t*>(base + L.rank_off);
  T* by_rank = reinterpret_cast<T*>(base + L.rank_out_off);
  if (cudaMemsetAsync(heads, 0, L.bitmap_bytes, s) != cudaSuccess) return Status::cuda;
  const unsigned pre_grid = unsigned((num_segments + 255) / 256 < 1024 ? (num_segments + 255) / 256 : 1024);
  // heads, flags and identities in contiguous blocks, then ranks from the blocks' counts
  const SegPrepassGrid pg = seg_prepass_grid(num_segments);
  uint32_t* block_count = reinterpret_cast<uint32_t*>(base + L.block_count_off);
  segment_heads_count_kernel<T, Op><<<unsigned(pg.blocks), 256, 0, s>>>(offsets, num_segments, n, pg.per_thread,
                                                                         heads, nonempty, out, block_count);
  if (cudaGetLastError() != cudaSuccess) return Status::cuda;
  if (n == 0) return Status::ok;
  SegArgs a{};
  a.s.in = in;
  a.s.out = nullptr;
  a.s.n = n;
  a.s.hdr = w.hdr;
  a.s.desc = w.desc;
  a.s.timeout_ns = settings().timeout_ns.load();
  a.s.debug_skip_tile = -1;
  a.heads = heads;
  a.rank_out = by_rank;
  SegReduceExtra rx;
  rx.offsets = offsets;
  rx.nonempty = nonempty;
  rx.rank = rank;
  rx.block_count = block_count;
  rx.prepass_blocks = pg.blocks;
  rx.per_thread = pg.per_thread;
  rx.tile_base = reinterpret_cast<uint32_t*>(base + L.tile_base_off);
  rx.tile_rec = base + L.tile_rec_off;
  rx.tile_rec_bytes = L.tile_rec_bytes;
  rx.chunk_v = base + L.chunk_v_off;
  rx.chunk_c = reinterpret_cast<uint32_t*>(base + L.chunk_c_off);
  st = launch_segmented<SegPlainScan<T, Op>, CsrHeads, false, true>(s, a, num_segments, &rx);
  if (st != Status::ok) return st;
  segment_gather_kernel<T><<<pre_grid, 256, 0, s>>>(nonempty, rank, by_rank, num_segments, out);
  return from_cuda(cudaGetLastError());
}

// Row scans of a rows x cols row-major matrix (every row its own segment);
// reverse = suffix scans.
template <class T, class Op>
inline Status rows_scan(cudaStream_t s, const T* in, T* out, uint64_t rows, uint64_t cols, bool exclusive,
                        bool reverse, void* user_ws = nullptr, size_t user_ws_bytes = 0) {
  const uint64_t n = rows * cols;
  if (n == 0) return Status::ok;
  if (!in || !out) return Status::invalid_arg;
  if (!aligned16(in) || !aligned16(out)) return Status::invalid_arg;
  DeviceInfo di;
  Status st0 = device_info(di);
  if (st0 != Status::ok) return st0;
  // Rows that tile a 64 KB stage exactly stream through it as contiguous
  // whole-row tiles (rows_tile_kernel) while there are too few of them to give
  // every SM two rounds of 32 row warps (GB300, 4096 x 8192 floats: 5.63 vs
  // 5.48 TB/s); with more rows one warp per row is 2-3 % faster.
  using TC = RowsTileCfg<T, 16, 8, 3>;
  Ws tw;
  Status wst = Status::workspace;
  if (TC::fits(cols) && rows <= uint64_t(64) * di.sm_count)  // its bounded waits report through a workspace
    wst = acquire_ws(s, workspace_bytes_for_desc_words(0), user_ws, user_ws_bytes, tw);
  if (wst != Status::ok && wst != Status::workspace) return wst;
  // (a stream captured without a sized workspace takes the kernels below, which need none)
  if (wst == Status::ok) {
    Status st = Status::ok;
    auto k = reverse ? rows_tile_kernel<T, Op, true, TC::NC, TC::CH, TC::STAGES>
                     : rows_tile_kernel<T, Op, false, TC::NC, TC::CH, TC::STAGES>;
    int bps = 0;
    st = prepare_kernel(k, TC::THREADS, TC::SMEM, bps);
    if (st != Status::ok) return st;
    const uint64_t per_tile = uint64_t(TC::NC) / (cols / TC::SEG);
    const uint64_t ntiles = (rows + per_tile - 1) / per_tile;
    uint64_t grid = uint64_t(bps) * di.sm_count;
    const int cap = settings().max_ctas.load();
    if (cap > 0 && uint64_t(cap) < grid) grid = cap;
    if (ntiles < grid) grid = ntiles;
    k<<<unsigned(grid), TC::THREADS, TC::SMEM, s>>>(in, out, rows, cols, exclusive ? 1 : 0, tw.hdr,
                                                    settings().timeout_ns.load());
    return from_cuda(cudaGetLastError());
  }
  // One warp per row when rows are long enough to stream and there are
  // enough of them (or they are not too long); else rows are segments of the
  // decoupled look-back kernel, which spreads long rows over many SMs.
  if (cols >= 256 && (rows >= uint64_t(2 * di.sm_count) || cols <= (uint64_t(1) << 16))) {
    constexpr int U = 8;
    const bool vec = (cols * sizeof(T)) % 16 == 0;
    // one-warp blocks: the block scheduler spreads them evenly over the SMs
    // (4096 rows of 8192 floats: 3 % faster than 8-warp blocks, which leave
    // a third of the SMs with 4 blocks and the rest with 3)
    auto launch = [&](auto kernel) -> Status {
      int bps = 0;
      Status st = prepare_kernel(kernel, 32, 0, bps);
      if (st != Status::ok) return st;
      uint64_t grid = rows;
      const uint64_t cap = uint64_t(bps) * di.sm_count;
      if (grid > cap) grid = cap;
      kernel<<<unsigned(grid), 32, 0, s>>>(in, out, rows, cols, exclusive ? 1 : 0);
      return from_cuda(cudaGetLastError());
    };
    constexpr int VV = 16 / int(sizeof(T));
    if (reverse) {
      return vec ? launch(rows_warp_kernel<T, Op, true, VV, U>) : launch(rows_warp_kernel<T, Op, true, 1, U>);
    }
    return vec ? launch(rows_warp_kernel<T, Op, false, VV, U>) : launch(rows_warp_kernel<T, Op, false, 1, U>);
  }
  const SegWsLayout L = seg_ws_layout<T, Op>(n, 0, false, false);
  Ws w;
  Status st = acquire_ws(s, L.control_bytes, user_ws, user_ws_bytes, w);
  if (st != Status::ok) return st;
  SegArgs a{};
  a.s.in = in;
  a.s.out = out;
  a.s.n = n;
  a.s.hdr = w.hdr;
  a.s.desc = w.desc;
  a.s.timeout_ns = settings().timeout_ns.load();
  a.s.debug_skip_tile = -1;
  a.s.exclusive = exclusive ? 1 : 0;
  a.seg_len = cols;
  if (reverse) return launch_segmented<SegPlainScan<T, Op>, UniformHeads, true, false>(s, a);
  return launch_segmented<SegPlainScan<T, Op>, UniformHeads, false, false>(s, a);
}

}  // namespace host
}  // namespace pp
