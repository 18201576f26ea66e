// Autotuner of the batched segmented scan: times every variant of the
// segmented kernel over
//   compute warps (block size 128 / 256 / 512 compute threads),
//   items per thread 4 / 8 / 16 / 32,
//   chunk vector width 4 / 8 / 16 bytes,
// on the batched workload (65,536 segments with log-uniform lengths in
// [1, 2^16], int64 offsets) for int32 U[0,1000) and float32 N(0,1) payloads,
// checks every variant's output against the default variant, and prints one
// JSON line per variant. ppautotune.py compiles and runs it and writes the
// winners to csrc/pp/seg_tuned.inc.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "pp/host.cuh"

using namespace pp;

template <class T>
struct Workload {
  uint64_t n = 0, S = 0;
  T *in = nullptr, *out = nullptr, *ref = nullptr;
  int64_t* offsets = nullptr;
  uint32_t* heads = nullptr;
  void* ctrl = nullptr;
  size_t ctrl_bytes = 0;
};

__global__ void fill_i32(int32_t* p, uint64_t n, uint64_t seed) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    p[i] = int32_t(((z >> 32) * 1000ull) >> 32);
  }
}
__global__ void fill_f32(float* p, uint64_t n, uint64_t seed) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const float u1 = (float((z >> 40) + 1)) * 0x1.0p-24f, u2 = float(z & 0xFFFFFF) * 0x1.0p-24f;
    p[i] = sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
  }
}

template <class T, int NC, int ITEMS, int VB>
void run_variant(Workload<T>& w, const char* dt, bool is_reference) {
  using Pol = SegPlainScan<T, plus>;
  constexpr int V = VB / int(sizeof(T));
  constexpr int CH = ITEMS / V;
  if constexpr (CH < 1 || ITEMS % V != 0) {
    return;
  } else {
    constexpr int TILE_BYTES = NC * 32 * ITEMS * int(sizeof(T));
    constexpr int ST0 = 196608 / TILE_BYTES;
    constexpr int STAGES = ST0 < 2 ? 2 : (ST0 > 8 ? 8 : ST0);
    using Cfg = SegCfg<Pol, NC, CH, STAGES, 4, VB>;
    auto k = segmented_staged_kernel<Pol, NC, CH, STAGES, 4, CsrHeads, false, false, VB>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(Cfg::SMEM));
    int bps = 0, sms = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k, Cfg::THREADS, Cfg::SMEM);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    const uint64_t ntiles = (w.n + Cfg::TILE - 1) / Cfg::TILE;
    const size_t need = workspace_bytes_for_desc_words(ntiles * desc_codec<typename Pol::carry_t>::W);
    if (need > w.ctrl_bytes || bps < 1) {
      printf("{\"dtype\":\"%s\",\"nc\":%d,\"items\":%d,\"vb\":%d,\"skipped\":true}\n", dt, NC, ITEMS, VB);
      return;
    }
    cudaMemset(w.ctrl, 0, w.ctrl_bytes);
    SegArgs a{};
    a.s.in = w.in;
    a.s.out = w.out;
    a.s.n = w.n;
    a.s.hdr = static_cast<WsHeader*>(w.ctrl);
    a.s.desc = reinterpret_cast<uint64_t*>(static_cast<unsigned char*>(w.ctrl) + kDescOffset);
    a.s.timeout_ns = 1000000000ull;
    a.s.debug_skip_tile = -1;
    a.heads = w.heads;
    unsigned grid = unsigned(std::min<uint64_t>(uint64_t(bps) * sms, ntiles));
    for (int i = 0; i < 3; ++i) k<<<grid, Cfg::THREADS, Cfg::SMEM>>>(a);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    std::vector<float> ms(15);
    for (float& m : ms) {
      cudaEventRecord(e0);
      k<<<grid, Cfg::THREADS, Cfg::SMEM>>>(a);
      cudaEventRecord(e1);
      cudaEventSynchronize(e1);
      cudaEventElapsedTime(&m, e0, e1);
    }
    std::sort(ms.begin(), ms.end());
    unsigned err = 0;
    cudaMemcpy(&err, &a.s.hdr->error, 4, cudaMemcpyDeviceToHost);
    bool same = true;
    if (is_reference) {
      cudaMemcpy(w.ref, w.out, w.n * sizeof(T), cudaMemcpyDeviceToDevice);
    } else {
      std::vector<T> h1(w.n), h2(w.n);
      cudaMemcpy(h1.data(), w.out, w.n * sizeof(T), cudaMemcpyDeviceToHost);
      cudaMemcpy(h2.data(), w.ref, w.n * sizeof(T), cudaMemcpyDeviceToHost);
      for (uint64_t i = 0; i < w.n && same; ++i) {
        const double d = double(h1[i]) - double(h2[i]);
        same = std::fabs(d) <= 1e-3 * (1.0 + std::fabs(double(h2[i])));
      }
    }
    const double med = ms[ms.size() / 2];
    printf("{\"dtype\":\"%s\",\"nc\":%d,\"items\":%d,\"vb\":%d,\"stages\":%d,\"tile\":%d,\"grid\":%u,\"ms\":%.5f,"
           "\"elems_per_s\":%.4e,\"gbs\":%.1f,\"err\":%u,\"matches_default\":%s}\n",
           dt, NC, ITEMS, VB, STAGES, Cfg::TILE, grid, med, double(w.n) / (med * 1e-3),
           2.0 * w.n * sizeof(T) / (med * 1e-3) / 1e9, err, same ? "true" : "false");
    fflush(stdout);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
}

template <class T, int NC>
void run_nc(Workload<T>& w, const char* dt) {
  run_variant<T, NC, 4, 4>(w, dt, false);
  run_variant<T, NC, 4, 8>(w, dt, false);
  run_variant<T, NC, 4, 16>(w, dt, false);
  run_variant<T, NC, 8, 4>(w, dt, false);
  run_variant<T, NC, 8, 8>(w, dt, false);
  run_variant<T, NC, 8, 16>(w, dt, false);
  run_variant<T, NC, 16, 4>(w, dt, false);
  run_variant<T, NC, 16, 8>(w, dt, false);
  run_variant<T, NC, 16, 16>(w, dt, false);
  run_variant<T, NC, 32, 4>(w, dt, false);
  run_variant<T, NC, 32, 8>(w, dt, false);
  run_variant<T, NC, 32, 16>(w, dt, false);
}

template <class T>
void tune(const char* dt, const std::vector<int64_t>& off) {
  Workload<T> w;
  w.S = off.size() - 1;
  w.n = uint64_t(off.back());
  cudaMalloc(&w.in, w.n * sizeof(T));
  cudaMalloc(&w.out, w.n * sizeof(T));
  cudaMalloc(&w.ref, w.n * sizeof(T));
  cudaMalloc(&w.offsets, off.size() * 8);
  cudaMemcpy(w.offsets, off.data(), off.size() * 8, cudaMemcpyHostToDevice);
  if constexpr (std::is_same_v<T, float>) fill_f32<<<1024, 256>>>(w.in, w.n, 0x5EC);
  else fill_i32<<<1024, 256>>>(w.in, w.n, 0x5EC);
  const size_t map_bytes = ((w.n + 127) / 128) * 16 + 8192;
  cudaMalloc(&w.heads, map_bytes);
  cudaMemset(w.heads, 0, map_bytes);
  segment_heads_kernel<T, plus><<<256, 256>>>(w.offsets, w.S, w.n, w.heads, nullptr, nullptr);
  w.ctrl_bytes = workspace_bytes_for_desc_words((w.n / 128 + 1) * 2);
  cudaMalloc(&w.ctrl, w.ctrl_bytes);
  run_variant<T, 16, 32, 16>(w, dt, true);  // default variant: reference output
  run_nc<T, 4>(w, dt);
  run_nc<T, 8>(w, dt);
  run_nc<T, 16>(w, dt);
  cudaFree(w.in);
  cudaFree(w.out);
  cudaFree(w.ref);
  cudaFree(w.offsets);
  cudaFree(w.heads);
  cudaFree(w.ctrl);
}

int main() {
  const int S = 65536;
  std::mt19937_64 rng(0x5EC);
  std::uniform_real_distribution<double> u(0.0, std::log(65536.0));
  std::vector<int64_t> off(S + 1, 0);
  for (int s = 0; s < S; ++s) {
    int64_t len = int64_t(std::floor(std::exp(u(rng))));
    len = std::min<int64_t>(std::max<int64_t>(len, 1), 65536);
    off[s + 1] = off[s] + len;
  }
  printf("{\"segments\":%d,\"elements\":%lld}\n", S, (long long)off.back());
  tune<int32_t>("i32", off);
  tune<float>("f32", off);
  printf("{\"last_error\":\"%s\"}\n", cudaGetErrorString(cudaGetLastError()));
  return 0;
}
