// Autotuner of the batched segmented scan: times every variant of the
// segmented kernel on two length distributions and one payload type (chosen
// at compile time with -DPP_TUNE_DT=0..3: int32, float32, int64, float64) and
// prints one JSON line per (payload, distribution, variant). Variants:
//   striped chunks (LAY 0): compute warps {4, 8, 16} (block size 128 / 256 /
//     512 compute threads), items per thread {4, 8, 16, 32}, chunk vector
//     width {8, 16} bytes;
//   lane rows (LAY 2): compute warps {12, 14, 16, 18, 20}, {5, 7, 9} 16-byte
//     chunks per lane (items per thread 20 / 28 / 36 for 4-byte payloads),
//     look-back polls of {1, 4} windows of 32 descriptors, and with one-window
//     polls also a store warp that writes finished tiles by bulk copy.
// Distributions: "long" = 65,536 segments with lengths floor(exp(U[0, ln 2^16]))
// clipped to [1, 2^16] (about 2^28 elements, the batched benchmark), "short" =
// 2^21 segments with lengths U[1, 128] (about 2^27 elements). Payloads: int32
// U[0,1000), float32 N(0,1), int64 U[0,1000), float64 N(0,1). Every variant's
// output is checked against the first (default) variant of the same case.
// ppautotune.py compiles one binary per payload (in parallel), runs them, and
// writes the variant with the best worst-case throughput per (payload size,
// distribution) to csrc/pp/seg_tuned.inc.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "pp/host.cuh"

using namespace pp;

template <class T>
struct Workload {
  const char* dist = "";
  uint64_t n = 0, S = 0;
  T *in = nullptr, *out = nullptr, *ref = nullptr;
  int64_t* offsets = nullptr;
  uint32_t* heads = nullptr;
  void* ctrl = nullptr;
  size_t ctrl_bytes = 0;
};

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

template <class T>
__global__ void fill(T* p, uint64_t n, uint64_t seed) {
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t z = mix64(seed + (i + 1) * 0x9E3779B97F4A7C15ull);
    if constexpr (std::is_floating_point_v<T>) {
      const float u1 = (float((z >> 40) + 1)) * 0x1.0p-24f, u2 = float(z & 0xFFFFFF) * 0x1.0p-24f;
      p[i] = T(sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2));
    } else {
      p[i] = T(((z >> 32) * 1000ull) >> 32);
    }
  }
}

template <class T, int LAY, int NC, int CH, int VB, int LBW = 4, int BS = 0>
void run_variant(Workload<T>& w, const char* dt, bool is_reference) {
  using Pol = SegPlainScan<T, plus>;
  constexpr int V = VB / int(sizeof(T));
  if constexpr (V < 1 || (LAY == 2 && (VB != 16 || CH % 2 == 0))) {
    return;
  } else {
    constexpr int ITEMS = CH * V;
    constexpr int TILE_BYTES = NC * 32 * ITEMS * int(sizeof(T));
    constexpr int ST0 = 196608 / TILE_BYTES;
    constexpr int STAGES = LAY == 2 ? 3 : (ST0 < 2 ? 2 : (ST0 > 8 ? 8 : ST0));
    using Cfg = SegCfg<Pol, NC, CH, STAGES, LBW, VB, LAY, (BS == 2 ? 1 : 0)>;
    if constexpr (Cfg::SMEM > 232448 || (Cfg::TILE % 128) != 0) {
      printf("{\"dtype\":\"%s\",\"dist\":\"%s\",\"lay\":%d,\"nc\":%d,\"ch\":%d,\"vb\":%d,\"skipped\":true}\n", dt,
             w.dist, LAY, NC, CH, VB);
      return;
    } else {
      auto k = segmented_staged_kernel<Pol, NC, CH, STAGES, LBW, CsrHeads, false, false, VB, LAY, BS>;
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(Cfg::SMEM));
      int bps = 0, sms = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k, Cfg::THREADS, Cfg::SMEM);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
      const uint64_t ntiles = (w.n + Cfg::TILE - 1) / Cfg::TILE;
      const size_t need = workspace_bytes_for_desc_words(ntiles * desc_codec<typename Pol::carry_t>::W);
      if (need > w.ctrl_bytes || bps < 1) {
        printf("{\"dtype\":\"%s\",\"dist\":\"%s\",\"lay\":%d,\"nc\":%d,\"ch\":%d,\"vb\":%d,\"skipped\":true}\n", dt,
               w.dist, LAY, NC, CH, VB);
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
      std::vector<float> ms(11);
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
      printf("{\"dtype\":\"%s\",\"dist\":\"%s\",\"lay\":%d,\"nc\":%d,\"ch\":%d,\"vb\":%d,\"lbw\":%d,\"items\":%d,"
             "\"bs\":%d,\"stages\":%d,\"tile\":%d,\"grid\":%u,\"ms\":%.5f,\"elems_per_s\":%.4e,\"gbs\":%.1f,"
             "\"err\":%u,\"matches_default\":%s}\n",
             dt, w.dist, LAY, NC, CH, VB, LBW, ITEMS, BS, STAGES, Cfg::TILE, grid, med, double(w.n) / (med * 1e-3),
             2.0 * w.n * sizeof(T) / (med * 1e-3) / 1e9, err, same ? "true" : "false");
      fflush(stdout);
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
    }
  }
}

// striped: items per thread {4, 8, 16, 32} at vector widths {8, 16} bytes
template <class T, int NC, int VB>
void run_striped_vb(Workload<T>& w, const char* dt) {
  constexpr int V = VB / int(sizeof(T));
  if constexpr (4 / V >= 1) run_variant<T, 0, NC, 4 / V, VB>(w, dt, false);
  run_variant<T, 0, NC, 8 / V, VB>(w, dt, false);
  run_variant<T, 0, NC, 16 / V, VB>(w, dt, false);
  run_variant<T, 0, NC, 32 / V, VB>(w, dt, false);
}
template <class T, int NC>
void run_striped(Workload<T>& w, const char* dt) {
  run_striped_vb<T, NC, 8>(w, dt);
  run_striped_vb<T, NC, 16>(w, dt);
}
template <class T, int NC>
void run_rows(Workload<T>& w, const char* dt) {
  run_variant<T, 2, NC, 5, 16, 4>(w, dt, false);
  run_variant<T, 2, NC, 7, 16, 4>(w, dt, false);
  run_variant<T, 2, NC, 9, 16, 4>(w, dt, false);
  run_variant<T, 2, NC, 5, 16, 1>(w, dt, false);
  run_variant<T, 2, NC, 7, 16, 1>(w, dt, false);
  run_variant<T, 2, NC, 9, 16, 1>(w, dt, false);
  run_variant<T, 2, NC, 5, 16, 1, 2>(w, dt, false);
  run_variant<T, 2, NC, 7, 16, 1, 2>(w, dt, false);
  run_variant<T, 2, NC, 9, 16, 1, 2>(w, dt, false);
}

template <class T>
void tune(const char* dt, const char* dist, const std::vector<int64_t>& off) {
  Workload<T> w;
  w.dist = dist;
  w.S = off.size() - 1;
  w.n = uint64_t(off.back());
  cudaMalloc(&w.in, w.n * sizeof(T));
  cudaMalloc(&w.out, w.n * sizeof(T));
  cudaMalloc(&w.ref, w.n * sizeof(T));
  cudaMalloc(&w.offsets, off.size() * 8);
  cudaMemcpy(w.offsets, off.data(), off.size() * 8, cudaMemcpyHostToDevice);
  fill<T><<<1024, 256>>>(w.in, w.n, 0x5EC);
  const size_t map_bytes = ((w.n + 127) / 128) * 16 + 16384;
  cudaMalloc(&w.heads, map_bytes);
  cudaMemset(w.heads, 0, map_bytes);
  segment_heads_kernel<T, plus><<<1024, 256>>>(w.offsets, w.S, w.n, w.heads, nullptr, nullptr);
  w.ctrl_bytes = workspace_bytes_for_desc_words((w.n / 128 + 1) * 2);
  cudaMalloc(&w.ctrl, w.ctrl_bytes);
  run_variant<T, 0, 16, 8, 16>(w, dt, true);  // default variant (16 warps, 8 16-byte chunks): reference output
  run_striped<T, 4>(w, dt);
  run_striped<T, 8>(w, dt);
  run_striped<T, 16>(w, dt);
  run_rows<T, 12>(w, dt);
  run_rows<T, 14>(w, dt);
  run_rows<T, 16>(w, dt);
  run_rows<T, 18>(w, dt);
  run_rows<T, 20>(w, dt);
  cudaFree(w.in);
  cudaFree(w.out);
  cudaFree(w.ref);
  cudaFree(w.offsets);
  cudaFree(w.heads);
  cudaFree(w.ctrl);
}

int main() {
  std::mt19937_64 rng(0x5EC);
  const int SL = 65536;
  std::uniform_real_distribution<double> u(0.0, std::log(65536.0));
  std::vector<int64_t> lng(SL + 1, 0);
  for (int s = 0; s < SL; ++s) {
    int64_t len = int64_t(std::floor(std::exp(u(rng))));
    len = std::min<int64_t>(std::max<int64_t>(len, 1), 65536);
    lng[s + 1] = lng[s] + len;
  }
  const int SS = 1 << 21;
  std::uniform_int_distribution<int64_t> us(1, 128);
  std::vector<int64_t> sht(SS + 1, 0);
  for (int s = 0; s < SS; ++s) sht[s + 1] = sht[s] + us(rng);
  printf("{\"long_segments\":%d,\"long_elements\":%lld,\"short_segments\":%d,\"short_elements\":%lld}\n", SL,
         (long long)lng.back(), SS, (long long)sht.back());
#ifndef PP_TUNE_DT
#define PP_TUNE_DT 0
#endif
#if PP_TUNE_DT == 0
  using T = int32_t;
  const char* dt = "i32";
#elif PP_TUNE_DT == 1
  using T = float;
  const char* dt = "f32";
#elif PP_TUNE_DT == 2
  using T = int64_t;
  const char* dt = "i64";
#else
  using T = double;
  const char* dt = "f64";
#endif
  tune<T>(dt, "long", lng);
  tune<T>(dt, "short", sht);
  printf("{\"last_error\":\"%s\"}\n", cudaGetErrorString(cudaGetLastError()));
  return 0;
}
