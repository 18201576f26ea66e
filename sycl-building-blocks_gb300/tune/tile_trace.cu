// Per-tile timelines of the staged decoupled look-back scan: a tracing build of
// the library's own configuration (DecoupledTuning) for one scan policy. Every
// tile of one launch records %globaltimer at fixed points of its life (ticket
// drawn, bulk copy issued, data in, reduce pass done and aggregate published,
// look-back done, scan pass started and done, ...; the kTr* events of
// pp/decoupled_scan.cuh) into a device buffer of 16 words per tile, written to
// a file for tile_trace.py to summarise. The traced launch follows three
// untraced ones and a 256 MiB read that leaves none of the input in the L2.
//
//   tile_trace <policy> <log2 of the input bytes> <output file>
//   policy: u32 | f32 | u64 | f64 | f32_compensated | f32_fp64_carry
//           seg_i32 | seg_f32 | seg_i32_reduce | seg_f32_reduce
// The seg_* policies trace the batched segmented kernel (its long-segment
// configuration) on log-uniform segment lengths in [1, 2^16] that fill the
// input; there the ticket slot holds when the producer began to wait for a
// free stage (tickets are drawn once a stage is free).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "pp/host.cuh"

using namespace pp;
using pp::host::DecoupledTuning;
using pp::host::StagedFor;

constexpr int kSlots = 16;
constexpr long long kMaxTiles = 12000;  // tiles recorded (the first ones by ticket)
__device__ unsigned long long* g_trace;

struct RecTrace {
  static constexpr bool kOn = true;
  __device__ __forceinline__ void operator()(int ev, long long tile, unsigned long long v) const {
    unsigned long long* t = g_trace;
    if (t != nullptr && tile >= 0 && tile < kMaxTiles && ev >= 0 && ev < kSlots) {
      t[tile * kSlots + ev] = v;
      if (ev == kTrFull) t[tile * kSlots + 8] = blockIdx.x;
    }
  }
};

template <class T>
__global__ void fill(T* p, uint64_t n) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t z = (i * 0x9E3779B97F4A7C15ull) >> 40;
    if constexpr (std::is_floating_point_v<T>)
      p[i] = T(float(z & 0xFFFF) / 16384.0f - 2.0f);
    else
      p[i] = T(z & 0xFFFF);
  }
}

__global__ void flush_read(const uint4* p, uint64_t nv, unsigned* sink) {
  uint32_t a = 0;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < nv; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint4 v = p[i];
    a ^= v.x ^ v.y ^ v.z ^ v.w;
  }
  if (a == 0x12345678u) *sink = a;
}

#define CHECK(x)                                                                    \
  do {                                                                              \
    cudaError_t e_ = (x);                                                           \
    if (e_ != cudaSuccess) {                                                        \
      fprintf(stderr, "%s failed: %s\n", #x, cudaGetErrorString(e_));               \
      return 2;                                                                     \
    }                                                                               \
  } while (0)

template <class Pol>
int trace(const char* name, int log2_bytes, const char* path) {
  using T = typename Pol::in_t;
  using Tn = DecoupledTuning<Pol>;
  using Cfg = StagedFor<Pol>;
  auto k = decoupled_staged_kernel<Pol, Tn::NC, Tn::CH, Tn::STAGES, Tn::LBW, Tn::LAY, Tn::TK, Tn::PG, Tn::BS, RecTrace>;
  const uint64_t n = (uint64_t(1) << log2_bytes) / sizeof(T);
  CHECK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(Cfg::SMEM)));
  int bps = 0, sms = 0;
  CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k, Cfg::THREADS, Cfg::SMEM));
  CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0));
  const long long ntiles = (long long)((n + Cfg::TILE - 1) / Cfg::TILE);
  const unsigned grid = unsigned(std::min<long long>(ntiles, (long long)bps * sms));
  T *in = nullptr, *out = nullptr;
  CHECK(cudaMalloc(&in, n * sizeof(T)));
  CHECK(cudaMalloc(&out, n * sizeof(T)));
  fill<<<1024, 256>>>(in, n);
  const size_t wsb = workspace_bytes_for_desc_words(uint64_t(ntiles) * desc_codec<typename Pol::carry_t>::W);
  void* ws = nullptr;
  CHECK(cudaMalloc(&ws, wsb));
  CHECK(cudaMemset(ws, 0, wsb));
  uint4* fl = nullptr;
  unsigned* sink = nullptr;
  CHECK(cudaMalloc(&fl, size_t(1) << 28));
  CHECK(cudaMemset(fl, 1, size_t(1) << 28));
  CHECK(cudaMalloc(&sink, 4));
  ScanArgs a{};
  a.in = in;
  a.out = out;
  a.n = n;
  a.hdr = static_cast<WsHeader*>(ws);
  a.desc = reinterpret_cast<uint64_t*>(static_cast<char*>(ws) + kDescOffset);
  a.timeout_ns = 1000000000ull;
  a.debug_skip_tile = -1;
  for (int i = 0; i < 3; ++i) k<<<grid, Cfg::THREADS, Cfg::SMEM>>>(a);
  const long long nrec = ntiles < kMaxTiles ? ntiles : kMaxTiles;
  unsigned long long* tr = nullptr;
  CHECK(cudaMalloc(&tr, size_t(nrec) * kSlots * 8));
  CHECK(cudaMemset(tr, 0, size_t(nrec) * kSlots * 8));
  CHECK(cudaMemcpyToSymbol(g_trace, &tr, sizeof(tr)));
  flush_read<<<1024, 512>>>(fl, (uint64_t(1) << 28) / 16, sink);
  cudaEvent_t e0, e1;
  CHECK(cudaEventCreate(&e0));
  CHECK(cudaEventCreate(&e1));
  CHECK(cudaEventRecord(e0));
  k<<<grid, Cfg::THREADS, Cfg::SMEM>>>(a);
  CHECK(cudaEventRecord(e1));
  CHECK(cudaEventSynchronize(e1));
  float ms = 0.0f;
  CHECK(cudaEventElapsedTime(&ms, e0, e1));
  unsigned err = 0;
  CHECK(cudaMemcpy(&err, &a.hdr->error, 4, cudaMemcpyDeviceToHost));
  std::vector<unsigned long long> h(size_t(nrec) * kSlots);
  CHECK(cudaMemcpy(h.data(), tr, h.size() * 8, cudaMemcpyDeviceToHost));
  FILE* f = fopen(path, "wb");
  if (f == nullptr) {
    fprintf(stderr, "cannot write %s\n", path);
    return 2;
  }
  fwrite(h.data(), 8, h.size(), f);
  fclose(f);
  printf("{\"policy\":\"%s\",\"n\":%llu,\"tile\":%d,\"tiles\":%lld,\"recorded\":%lld,\"grid\":%u,\"threads\":%d,"
         "\"smem\":%zu,\"traced_ms\":%.4f,\"gbs\":%.1f,\"device_error\":%u}\n",
         name, (unsigned long long)n, Cfg::TILE, ntiles, nrec, grid, Cfg::THREADS, size_t(Cfg::SMEM), ms,
         2.0 * double(n) * sizeof(T) / (ms * 1e-3) / 1e9, err);
  cudaFree(tr);
  cudaFree(fl);
  cudaFree(sink);
  cudaFree(ws);
  cudaFree(in);
  cudaFree(out);
  return err == 0 ? 0 : 3;
}

template <class T, bool REDUCE>
int trace_seg(const char* name, int log2_bytes, const char* path) {
  using Pol = SegPlainScan<T, plus>;
  using Tn = pp::host::SegTunedCsr<T, true>;
  constexpr int BS = REDUCE ? 0 : Tn::BS;
  using Cfg = SegCfg<Pol, Tn::NC, Tn::CH, Tn::STAGES, Tn::LBW, Tn::VB, Tn::LAY, (BS == 2 ? 1 : 0)>;
  auto k = segmented_staged_kernel<Pol, Tn::NC, Tn::CH, Tn::STAGES, Tn::LBW, CsrHeads, false, REDUCE, Tn::VB, Tn::LAY,
                                   BS, REDUCE && Tn::LAY == 2, RecTrace>;
  const uint64_t n = (uint64_t(1) << log2_bytes) / sizeof(T);
  std::vector<int64_t> off{0};
  uint64_t x = 0x5EC;
  while (uint64_t(off.back()) < n) {
    x = x * 6364136223846793005ull + 1442695040888963407ull;
    const double u = double(x >> 11) * (1.0 / 9007199254740992.0);
    const int64_t len = std::max<int64_t>(1, std::min<int64_t>(int64_t(std::floor(std::exp(u * std::log(65536.0)))), 65536));
    off.push_back(std::min<int64_t>(off.back() + len, int64_t(n)));
  }
  const uint64_t S = off.size() - 1;
  CHECK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(Cfg::SMEM)));
  int bps = 0, sms = 0;
  CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k, Cfg::THREADS, Cfg::SMEM));
  CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0));
  const long long ntiles = (long long)((n + Cfg::TILE - 1) / Cfg::TILE);
  const unsigned grid = unsigned(std::min<long long>(ntiles, (long long)bps * sms));
  T *in = nullptr, *out = nullptr;
  int64_t* d_off = nullptr;
  uint32_t* heads = nullptr;
  const size_t map_bytes = ((n + 127) / 128) * 16 + 4096;
  CHECK(cudaMalloc(&in, n * sizeof(T)));
  CHECK(cudaMalloc(&out, (REDUCE ? S : n) * sizeof(T)));
  CHECK(cudaMalloc(&d_off, off.size() * sizeof(int64_t)));
  CHECK(cudaMalloc(&heads, map_bytes));
  CHECK(cudaMemcpy(d_off, off.data(), off.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
  CHECK(cudaMemset(heads, 0, map_bytes));
  fill<<<1024, 256>>>(in, n);
  segment_heads_kernel<T, plus><<<1024, 256>>>(d_off, S, n, heads, nullptr, nullptr);
  const size_t wsb = workspace_bytes_for_desc_words(uint64_t(ntiles) * desc_codec<typename Pol::carry_t>::W);
  void* ws = nullptr;
  CHECK(cudaMalloc(&ws, wsb));
  CHECK(cudaMemset(ws, 0, wsb));
  uint4* fl = nullptr;
  unsigned* sink = nullptr;
  CHECK(cudaMalloc(&fl, size_t(1) << 28));
  CHECK(cudaMemset(fl, 1, size_t(1) << 28));
  CHECK(cudaMalloc(&sink, 4));
  // reductions: the non-empty segments before each tile (every segment here
  // is non-empty, so that is the index of the first segment starting at or
  // after the tile) and the per-tile records
  uint32_t* tile_base = nullptr;
  void* tile_rec = nullptr;
  if (REDUCE) {
    std::vector<uint32_t> tb(static_cast<size_t>(ntiles));
    for (long long t = 0; t < ntiles; ++t) {
      const int64_t target = int64_t(t) * Cfg::TILE;
      size_t lo = 0, hi = S;  // first segment starting at or after the tile
      while (lo < hi) {
        const size_t mid = (lo + hi) / 2;
        if (off[mid] < target)
          lo = mid + 1;
        else
          hi = mid;
      }
      tb[size_t(t)] = uint32_t(lo);
    }
    CHECK(cudaMalloc(&tile_base, tb.size() * 4));
    CHECK(cudaMemcpy(tile_base, tb.data(), tb.size() * 4, cudaMemcpyHostToDevice));
    CHECK(cudaMalloc(&tile_rec, size_t(ntiles) * sizeof(SegTileRec<T>)));
    CHECK(cudaMemset(tile_rec, 0, size_t(ntiles) * sizeof(SegTileRec<T>)));
  }
  SegArgs a{};
  a.s.in = in;
  a.s.out = REDUCE ? nullptr : out;
  a.s.n = n;
  a.s.hdr = static_cast<WsHeader*>(ws);
  a.s.desc = reinterpret_cast<uint64_t*>(static_cast<char*>(ws) + kDescOffset);
  a.s.timeout_ns = 1000000000ull;
  a.s.debug_skip_tile = -1;
  a.heads = heads;
  a.rank_out = REDUCE ? out : nullptr;
  a.tile_base = tile_base;
  a.tile_rec = tile_rec;
  for (int i = 0; i < 3; ++i) k<<<grid, Cfg::THREADS, Cfg::SMEM>>>(a);
  const long long nrec = ntiles < kMaxTiles ? ntiles : kMaxTiles;
  unsigned long long* tr = nullptr;
  CHECK(cudaMalloc(&tr, size_t(nrec) * kSlots * 8));
  CHECK(cudaMemset(tr, 0, size_t(nrec) * kSlots * 8));
  CHECK(cudaMemcpyToSymbol(g_trace, &tr, sizeof(tr)));
  flush_read<<<1024, 512>>>(fl, (uint64_t(1) << 28) / 16, sink);
  cudaEvent_t e0, e1;
  CHECK(cudaEventCreate(&e0));
  CHECK(cudaEventCreate(&e1));
  CHECK(cudaEventRecord(e0));
  k<<<grid, Cfg::THREADS, Cfg::SMEM>>>(a);
  CHECK(cudaEventRecord(e1));
  CHECK(cudaEventSynchronize(e1));
  float ms = 0.0f;
  CHECK(cudaEventElapsedTime(&ms, e0, e1));
  unsigned err = 0;
  CHECK(cudaMemcpy(&err, &a.s.hdr->error, 4, cudaMemcpyDeviceToHost));
  std::vector<unsigned long long> h(size_t(nrec) * kSlots);
  CHECK(cudaMemcpy(h.data(), tr, h.size() * 8, cudaMemcpyDeviceToHost));
  FILE* f = fopen(path, "wb");
  if (f == nullptr) {
    fprintf(stderr, "cannot write %s\n", path);
    return 2;
  }
  fwrite(h.data(), 8, h.size(), f);
  fclose(f);
  printf("{\"policy\":\"%s\",\"n\":%llu,\"segments\":%llu,\"tile\":%d,\"tiles\":%lld,\"recorded\":%lld,"
         "\"grid\":%u,\"threads\":%d,\"smem\":%zu,\"traced_ms\":%.4f,\"gbs\":%.1f,\"device_error\":%u}\n",
         name, (unsigned long long)n, (unsigned long long)S, Cfg::TILE, ntiles, nrec, grid, Cfg::THREADS,
         size_t(Cfg::SMEM), ms, (REDUCE ? 1.0 : 2.0) * double(n) * sizeof(T) / (ms * 1e-3) / 1e9, err);
  cudaFree(tr);
  cudaFree(fl);
  cudaFree(sink);
  cudaFree(ws);
  cudaFree(heads);
  cudaFree(d_off);
  if (tile_base) cudaFree(tile_base);
  if (tile_rec) cudaFree(tile_rec);
  cudaFree(in);
  cudaFree(out);
  return err == 0 ? 0 : 3;
}

int main(int argc, char** argv) {
  if (argc != 4) {
    fprintf(stderr,
            "usage: %s <u32|f32|u64|f64|f32_compensated|f32_fp64_carry|seg_i32|seg_f32|seg_i32_reduce|seg_f32_reduce>"
            " <log2 bytes> <out file>\n",
            argv[0]);
    return 1;
  }
  const int lg = atoi(argv[2]);
  if (lg < 12 || lg > 34) {
    fprintf(stderr, "log2 bytes must be in [12, 34]\n");
    return 1;
  }
  const char* p = argv[1];
  if (!strcmp(p, "u32")) return trace<PlainScan<uint32_t, plus>>(p, lg, argv[3]);
  if (!strcmp(p, "f32")) return trace<PlainScan<float, plus>>(p, lg, argv[3]);
  if (!strcmp(p, "u64")) return trace<PlainScan<uint64_t, plus>>(p, lg, argv[3]);
  if (!strcmp(p, "f64")) return trace<PlainScan<double, plus>>(p, lg, argv[3]);
  if (!strcmp(p, "f32_compensated")) return trace<CompensatedF32>(p, lg, argv[3]);
  if (!strcmp(p, "f32_fp64_carry")) return trace<F64CarryF32>(p, lg, argv[3]);
  if (!strcmp(p, "seg_i32")) return trace_seg<int32_t, false>(p, lg, argv[3]);
  if (!strcmp(p, "seg_f32")) return trace_seg<float, false>(p, lg, argv[3]);
  if (!strcmp(p, "seg_i32_reduce")) return trace_seg<int32_t, true>(p, lg, argv[3]);
  if (!strcmp(p, "seg_f32_reduce")) return trace_seg<float, true>(p, lg, argv[3]);
  fprintf(stderr, "unknown policy %s\n", p);
  return 1;
}
