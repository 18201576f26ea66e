// C++ tests of the header-only drop-in API (include/parallel_primitives/),
// written after the reference's own tests:
//   tests/test_reduction.cpp  - uint64 iota sums, device and host arrays
//   tests/test_scan.cpp       - Basel sum and Wallis product through scan and
//                               decoupled_scan (the reference only prints
//                               them; here they are checked against FP64)
//   benchmarks/benchmark_scan.cpp - fill(1) -> out[n-1] == n
//   tests/test_intrinsics.cpp - the intrinsics known answers, evaluated on
//                               the GPU into a result buffer (no device traps)
// plus a non-commutative user operator (affine-map composition) and the
// subset grid barrier of cooperative_groups.hpp (membership by list and by
// predicate, reuse across many phases, a wait that runs out of time).
// Prints one line per check and exits non-zero on any failure.
#include <cmath>
#include <cstdio>
#include <numeric>
#include <span>
#include <vector>

#include <parallel_primitives/cooperative_groups.hpp>
#include <parallel_primitives/intrinsics.hpp>
#include <parallel_primitives/reduction.hpp>
#include <parallel_primitives/scan.hpp>
#include <parallel_primitives/scan_cooperative.hpp>
#include <parallel_primitives/scan_decoupled_lookback.hpp>

using namespace parallel_primitives;

static int failures = 0;
#define CHECK(cond, ...)                      \
  do {                                        \
    if (!(cond)) {                            \
      ++failures;                             \
      std::printf("FAIL %s:%d ", __FILE__, __LINE__); \
      std::printf(__VA_ARGS__);               \
      std::printf("\n");                      \
    }                                         \
  } while (0)

// ---- reduction (tests/test_reduction.cpp) ------------------------------------
static void test_reduction(cudaStream_t s) {
  for (size_t n = 1; n < 1000000; n *= 4) {
    std::vector<uint64_t> h(n);
    std::iota(h.begin(), h.end(), uint64_t(0));
    uint64_t* d = nullptr;
    cudaMalloc(&d, n * sizeof(uint64_t));
    cudaMemcpy(d, h.data(), n * sizeof(uint64_t), cudaMemcpyHostToDevice);
    const uint64_t want = uint64_t(n) * (n - 1) / 2;
    const uint64_t dev = reduce_device<plus<>>(s, std::span<const uint64_t>(d, n));
    const uint64_t host = reduce<plus<>>(s, std::span<const uint64_t>(h));
    CHECK(dev == want, "reduce_device n=%zu got %llu", n, (unsigned long long)dev);
    CHECK(host == want, "reduce n=%zu got %llu", n, (unsigned long long)host);
    cudaFree(d);
  }
  std::printf("reduction: done\n");
}

// ---- scans (tests/test_scan.cpp) -----------------------------------------------
static void test_basel(cudaStream_t s) {
  const size_t n = 1000000;
  std::vector<float> in(n), out(n);
  std::vector<double> exact(n);
  double acc = 0.0;
  for (size_t i = 0; i < n; ++i) {
    const double idx = double(i + 1);
    in[i] = float(1.0 / (idx * idx));
    acc += double(in[i]);
    exact[i] = acc;
  }
  for (int which = 0; which < 2; ++which) {
    if (which == 0)
      scan<scan_type::inclusive, plus<>>(s, in.data(), out.data(), n);
    else
      decoupled_scan<scan_type::inclusive, plus<>>(s, in.data(), out.data(), n);
    double worst = 0.0;
    for (size_t i = 0; i < n; ++i) worst = std::fmax(worst, std::fabs(double(out[i]) - exact[i]) / exact[i]);
    // every term is positive: relative error bounded by (tree depth) * eps
    CHECK(worst < 2e-5, "basel (%d) max rel err %g", which, worst);
    const double pi = std::sqrt(6.0 * double(out[n - 1]));
    CHECK(std::fabs(pi - M_PI) < 2e-5, "basel (%d) pi estimate %.9f", which, pi);
  }
  std::printf("basel: sqrt(6 S_n) = %.7f\n", std::sqrt(6.0 * double(out[n - 1])));
}

static void test_wallis(cudaStream_t s) {
  const size_t n = 20000000;
  std::vector<float> in(n), out(n);
  for (size_t i = 0; i < n; ++i) {
    const double idx = double(i + 1);
    in[i] = float(4.0 * idx * idx / (4.0 * idx * idx - 1.0));
  }
  double prod = 1.0;
  for (size_t i = 0; i < n; ++i) prod *= double(in[i]);
  for (int which = 0; which < 2; ++which) {
    if (which == 0)
      scan<scan_type::inclusive, multiplies<>>(s, in.data(), out.data(), n);
    else
      decoupled_scan<scan_type::inclusive, multiplies<>>(s, in.data(), out.data(), n);
    const double rel = std::fabs(double(out[n - 1]) - prod) / prod;
    // n products, each rounded once in FP32, combined in a tree of depth ~n/tile
    CHECK(rel < 1e-3, "wallis (%d) rel err %g", which, rel);
  }
  std::printf("wallis: 2 P_n = %.7f (pi = %.7f)\n", 2.0 * double(out[n - 1]), M_PI);
}

static void test_fill_one(cudaStream_t s) {
  for (size_t n : {size_t(1), size_t(1000), size_t(65537), size_t(1) << 24}) {
    uint32_t *d_in, *d_out;
    cudaMalloc(&d_in, n * 4);
    cudaMalloc(&d_out, n * 4);
    std::vector<uint32_t> ones(n, 1u);
    cudaMemcpy(d_in, ones.data(), n * 4, cudaMemcpyHostToDevice);
    uint32_t last = 0;
    decoupled_scan_device<scan_type::inclusive, plus<>>(s, d_in, d_out, n);
    cudaMemcpyAsync(&last, d_out + n - 1, 4, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    CHECK(last == n, "decoupled fill(1) n=%zu last=%u", n, last);
    cooperative_scan_device<scan_type::exclusive, plus<>>(s, d_in, d_out, n);
    cudaMemcpyAsync(&last, d_out + n - 1, 4, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    CHECK(last == n - 1, "cooperative exclusive fill(1) n=%zu last=%u", n, last);
    group_scan_device<scan_type::inclusive, plus<>>(s, d_in, d_out, n < 70000 ? n : 70000);
    cudaMemcpyAsync(&last, d_out + (n < 70000 ? n : 70000) - 1, 4, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    CHECK(last == (n < 70000 ? n : 70000), "group scan fill(1) n=%zu last=%u", n, last);
    cudaFree(d_in);
    cudaFree(d_out);
  }
  std::printf("fill(1): done\n");
}

// ---- a user-defined, associative but non-commutative operator ------------------
struct Affine {  // x -> a*x + b (mod 2^32)
  uint32_t a, b;
};
struct compose {  // apply f, then g
  __host__ __device__ Affine operator()(const Affine& f, const Affine& g) const {
    return Affine{g.a * f.a, g.a * f.b + g.b};
  }
};
template <>
struct pp::op_traits<compose, Affine> {
  __host__ __device__ static Affine identity() { return Affine{1u, 0u}; }
};

static void test_user_functor(cudaStream_t s) {
  const size_t n = 3000001;
  std::vector<Affine> h(n), got(n), want(n);
  uint32_t r = 12345u;
  for (size_t i = 0; i < n; ++i) {
    r = r * 1664525u + 1013904223u;
    h[i].a = (r >> 8) | 1u;
    r = r * 1664525u + 1013904223u;
    h[i].b = r;
  }
  Affine acc{1u, 0u};
  for (size_t i = 0; i < n; ++i) {
    acc = compose{}(acc, h[i]);
    want[i] = acc;
  }
  decoupled_scan<scan_type::inclusive, compose>(s, h.data(), got.data(), n);
  size_t bad = 0;
  for (size_t i = 0; i < n; ++i) bad += (got[i].a != want[i].a || got[i].b != want[i].b);
  CHECK(bad == 0, "affine composition scan: %zu mismatches", bad);
  cooperative_scan<scan_type::inclusive, compose>(s, h.data(), got.data(), n);
  bad = 0;
  for (size_t i = 0; i < n; ++i) bad += (got[i].a != want[i].a || got[i].b != want[i].b);
  CHECK(bad == 0, "affine composition cooperative scan: %zu mismatches", bad);
  std::printf("user functor: done\n");
}

// ---- intrinsics (tests/test_intrinsics.cpp) -------------------------------------
__global__ void intrinsics_kernel(uint32_t* res) {
  using namespace parallel_primitives::ext;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t hi = 0xDEADBEEF, lo = 0xCAFED00D;
  bool ok = true;
  ok &= funnelshift_l(lo, hi, 8) == 0xADBEEFCAu;
  ok &= funnelshift_l(lo, hi, 0) == 0xDEADBEEFu;
  ok &= funnelshift_r(lo, hi, 8) == 0xEFCAFED0u;
  ok &= funnelshift_r(lo, hi, 0) == 0xCAFED00Du;
  ok &= brev32(2u) == (1u << 30);
  ok &= brev32(0xFu) == (0xFu << 28);
  ok &= brev32(0u) == 0u;
  ok &= brev32(brev32(lo)) == lo;
  ok &= brev64(1ull) == (1ull << 63);
  ok &= brev64(0xFull) == (0xFull << 60);
  ok &= brev64(0ull) == 0ull;
  ok &= brev64(brev64(uint64_t(lo))) == uint64_t(lo);
  ok &= upsample(uint8_t('S'), uint8_t('Y'), uint8_t('C'), uint8_t('L')) == 0x5359434cu;
  const uint32_t all = predicate_to_mask([](int) { return true; });
  const uint32_t even = predicate_to_mask([](int i) { return i % 2 == 0; });
  const uint32_t odd = predicate_to_mask([](int i) { return i % 2 != 0; });
  ok &= popcount(ballot(1)) == 32u;
  ok &= broadcast_leader(lane) == 0u;
  ok &= match_all(1u, 1u);
  ok &= match_all(all, 0xDEADBEEFu);
  ok &= !match_all(all, lane);
  ok &= match_all(even, lane % 2);
  ok &= match_any(uint32_t(lane % 2 == 0)) == ((lane % 2 == 0) ? even : odd);
  prefetch(&res[0]);
  prefetch_constant(&res[0]);
  res[1 + lane] = ok ? 1u : 0u;
  // funnel shifts over every shift amount, for the host to compare
  if (lane == 0) {
    for (uint32_t sft = 0; sft < 64; ++sft) {
      res[64 + sft] = funnelshift_l(lo, hi, sft);
      res[128 + sft] = funnelshift_r(lo, hi, sft);
    }
    res[0] = 1u;
  }
}

static void test_intrinsics() {
  uint32_t* d = nullptr;
  cudaMalloc(&d, 256 * 4);
  cudaMemset(d, 0, 256 * 4);
  intrinsics_kernel<<<1, 32>>>(d);
  std::vector<uint32_t> h(256);
  cudaMemcpy(h.data(), d, 256 * 4, cudaMemcpyDeviceToHost);
  CHECK(h[0] == 1u, "intrinsics kernel did not run");
  for (int l = 0; l < 32; ++l) CHECK(h[1 + l] == 1u, "intrinsics known answers failed on lane %d", l);
  using namespace parallel_primitives::ext;
  for (uint32_t sft = 0; sft < 64; ++sft) {
    CHECK(h[64 + sft] == funnelshift_l(0xCAFED00Du, 0xDEADBEEFu, sft), "funnelshift_l host/device %u", sft);
    CHECK(h[128 + sft] == funnelshift_r(0xCAFED00Du, 0xDEADBEEFu, sft), "funnelshift_r host/device %u", sft);
  }
  // host versions of the known answers (the reference's "cpp" test)
  CHECK(funnelshift_l(0xCAFED00Du, 0xDEADBEEFu, 8) == 0xADBEEFCAu, "host funnelshift_l");
  CHECK(brev64(1ull) == (1ull << 63), "host brev64");
  std::printf("intrinsics: done\n");
  std::printf("funnelshift:");
  for (uint32_t sft = 0; sft < 64; ++sft) std::printf(" %u:%08x/%08x", sft, h[64 + sft], h[128 + sft]);
  std::printf("\n");
  cudaFree(d);
}

// ---- subset grid barrier (nd_range_barrier) ----------------------------------
// Member blocks publish their phase number, cross the barrier, and check that
// every other member has published at least that phase. Non-members leave.
__global__ void barrier_phases_kernel(nd_range_barrier* b, unsigned* stamp, unsigned* errors, unsigned* ok_out,
                                      int phases) {
  const unsigned g = blockIdx.x;
  const bool member = b->is_member();
  for (int p = 1; p <= phases; ++p) {
    if (member && threadIdx.x == 0) atomicExch(&stamp[g], unsigned(p));
    if (!b->wait()) {
      if (threadIdx.x == 0) ok_out[g] = 0u;
      return;
    }
    if (member && threadIdx.x == 0) {
      for (unsigned o = 0; o < gridDim.x; ++o) {
        const unsigned v = atomicAdd(&stamp[o], 0u);
        if (v != 0xFFFFFFFFu && v < unsigned(p)) atomicAdd(errors, 1u);
      }
    }
  }
  if (threadIdx.x == 0) ok_out[g] = 1u;
}

// Block 0 never arrives: the other members' waits run out of time.
__global__ void barrier_missing_member_kernel(nd_range_barrier* b, unsigned* ok_out) {
  if (blockIdx.x == 0) {
    if (threadIdx.x == 0) ok_out[0] = 2u;
    return;
  }
  const bool ok = b->wait();
  if (threadIdx.x == 0) ok_out[blockIdx.x] = ok ? 1u : 0u;
}

static void run_phases(cudaStream_t s, nd_range_barrier* b, unsigned grid, const std::vector<bool>& member,
                       const char* what) {
  unsigned *stamp, *errors, *ok;
  cudaMalloc(&stamp, grid * 4);
  cudaMalloc(&errors, 4);
  cudaMalloc(&ok, grid * 4);
  std::vector<unsigned> init(grid);
  for (unsigned g = 0; g < grid; ++g) init[g] = member[g] ? 0u : 0xFFFFFFFFu;  // non-members never publish
  cudaMemcpy(stamp, init.data(), grid * 4, cudaMemcpyHostToDevice);
  cudaMemset(errors, 0, 4);
  cudaMemset(ok, 0, grid * 4);
  int phases = 200;
  void* args[] = {&b, &stamp, &errors, &ok, &phases};
  const cudaError_t e = cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(barrier_phases_kernel), dim3(grid),
                                                    dim3(128), args, 0, s);
  CHECK(e == cudaSuccess, "%s: cooperative launch: %s", what, cudaGetErrorString(e));
  cudaStreamSynchronize(s);
  unsigned err = 0;
  std::vector<unsigned> okh(grid);
  cudaMemcpy(&err, errors, 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(okh.data(), ok, grid * 4, cudaMemcpyDeviceToHost);
  unsigned done = 0;
  for (unsigned g = 0; g < grid; ++g) done += okh[g];
  CHECK(err == 0, "%s: %u members ran ahead of the barrier", what, err);
  CHECK(done == grid, "%s: %u of %u blocks finished", what, done, grid);
  CHECK(!nd_range_barrier::timed_out(b, s), "%s: barrier reports a timeout", what);
  std::printf("barrier %s: %u blocks, 200 phases, ok\n", what, grid);
  cudaFree(stamp);
  cudaFree(errors);
  cudaFree(ok);
}

static void test_barrier(cudaStream_t s) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const unsigned grid = unsigned(sms);
  {  // every other block, by predicate
    nd_range_barrier* b =
        nd_range_barrier::make_barrier_if(s, dim3(grid), dim3(128), [](size_t g) { return g % 2 == 0; });
    std::vector<bool> member(grid);
    for (unsigned g = 0; g < grid; ++g) member[g] = g % 2 == 0;
    run_phases(s, b, grid, member, "even blocks (predicate)");
    nd_range_barrier::destroy(b);
  }
  {  // an explicit list, checked against the kernel's occupancy
    std::vector<size_t> list = {1, 3, 4, 9, size_t(grid - 1)};
    nd_range_barrier* b = nd_range_barrier::make_barrier_for(s, barrier_phases_kernel, dim3(grid), dim3(128), 0, list);
    std::vector<bool> member(grid, false);
    for (size_t g : list) member[g] = true;
    run_phases(s, b, grid, member, "listed blocks");
    nd_range_barrier::destroy(b);
  }
  {  // all blocks
    nd_range_barrier* b = nd_range_barrier::make_barrier(s, dim3(grid), dim3(128));
    run_phases(s, b, grid, std::vector<bool>(grid, true), "all blocks");
    nd_range_barrier::destroy(b);
  }
  {  // a member that never arrives: the waits end with an error, the kernel ends
    nd_range_barrier* b = nd_range_barrier::make_barrier(s, dim3(8), dim3(64), {}, 20000000ull);
    unsigned* ok;
    cudaMalloc(&ok, 8 * 4);
    cudaMemset(ok, 0xFF, 8 * 4);
    void* args[] = {&b, &ok};
    const cudaError_t e = cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(barrier_missing_member_kernel),
                                                      dim3(8), dim3(64), args, 0, s);
    CHECK(e == cudaSuccess, "timeout launch: %s", cudaGetErrorString(e));
    CHECK(cudaStreamSynchronize(s) == cudaSuccess, "timeout kernel did not finish cleanly");
    std::vector<unsigned> okh(8);
    cudaMemcpy(okh.data(), ok, 8 * 4, cudaMemcpyDeviceToHost);
    CHECK(okh[0] == 2u, "block 0 did not leave");
    for (int g = 1; g < 8; ++g) CHECK(okh[g] == 0u, "block %d: wait did not report the timeout (%u)", g, okh[g]);
    CHECK(nd_range_barrier::timed_out(b, s), "barrier does not report the timeout");
    std::printf("barrier timeout: waits returned false, error recorded\n");
    cudaFree(ok);
    nd_range_barrier::destroy(b);
  }
  {  // host-side checks (perform_check): out-of-range member, oversized grid
    bool threw = false;
    try {
      nd_range_barrier::make_barrier(s, dim3(4), dim3(32), {7});
    } catch (const error&) {
      threw = true;
    }
    CHECK(threw, "out-of-range member accepted");
    threw = false;
    try {
      nd_range_barrier::make_barrier(s, dim3(grid * 1000), dim3(32));
    } catch (const error& e) {
      threw = e.status == pp::host::Status::grid_too_large;
    }
    CHECK(threw, "oversized grid accepted");
    const dim3 occ = get_max_occupancy(barrier_phases_kernel, 128);
    CHECK(occ.x >= grid, "get_max_occupancy %u < SMs", occ.x);
  }
}

int main() {
  cudaStream_t s;
  cudaStreamCreate(&s);
  try {
    test_intrinsics();
    test_reduction(s);
    test_fill_one(s);
    test_basel(s);
    test_wallis(s);
    test_user_functor(s);
    test_barrier(s);
  } catch (const std::exception& e) {
    std::printf("FAIL exception: %s\n", e.what());
    ++failures;
  }
  cudaStreamDestroy(s);
  std::printf(failures ? "FAILED %d\n" : "ALL PASSED\n", failures);
  return failures ? 1 : 0;
}
