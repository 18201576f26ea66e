// The reference's own call sites, written against this library's C++ drop-in
// with `sycl::queue q` replaced by a cudaStream_t and `sycl::plus<>` by
// parallel_primitives::plus<> (everything else as the reference writes it):
//   tests/test_reduction.cpp:4-18      usm_unique_ptr<T, alloc::shared> filled
//                                      with std::iota, reduce_device<plus<>>(q,
//                                      in.get_span()); reduce<plus<>>(q,
//                                      span<T>{vector}); n = 4^k, k = 0..9
//   benchmarks/benchmark_reduce.cpp:9-47  usm_unique_ptr<T, alloc::device>
//                                      filled with 1 and reduce_device<plus<>>
//                                      (q, in.get_span()); iota in shared USM
//   benchmarks/benchmark_scan.cpp:11-51  decoupled_scan_device<inclusive,
//                                      plus<>>(q, in.get(), out.get(), size)
//                                      on device USM filled with 1, and the
//                                      cooperative scan of the Basel terms in
//                                      shared USM
//   scan_decoupled_lookback.hpp:209,219,227  the trailing template parameters
//                                      <..., bool optimised_offload> and
//                                      <..., bool, size_t offload_threshold>,
//                                      instantiated with false as the
//                                      reference itself does.
// Prints one line per check and exits non-zero on any failure.
#include <cmath>
#include <cstdio>
#include <numeric>
#include <vector>

#include <parallel_primitives/reduction.hpp>
#include <parallel_primitives/scan_cooperative.hpp>
#include <parallel_primitives/scan_decoupled_lookback.hpp>
#include <usm_smart_ptr.hpp>

using namespace parallel_primitives;

static int failures = 0;
#define CHECK(cond, ...)                              \
  do {                                                \
    if (!(cond)) {                                    \
      ++failures;                                     \
      std::printf("FAIL %s:%d ", __FILE__, __LINE__); \
      std::printf(__VA_ARGS__);                       \
      std::printf("\n");                              \
    }                                                 \
  } while (0)

// tests/test_reduction.cpp:4-10
static void reduce_device_iota(size_t size, cudaStream_t q) {
  using T = uint64_t;
  auto in = usm_unique_ptr<T, alloc::shared>(size, q);
  std::iota(in.get(), in.get() + in.size(), 0);
  T res = parallel_primitives::reduce_device<plus<>>(q, in.get_span());
  CHECK(res == (size * (size - 1)) / 2, "reduce_device iota n=%zu: %llu", size, (unsigned long long)res);
}

// tests/test_reduction.cpp:12-18
static void reduce_host_iota(size_t size, cudaStream_t q) {
  using T = uint64_t;
  auto in = std::vector<T>(size, T{});
  std::iota(in.begin(), in.end(), 0);
  T res = parallel_primitives::reduce<plus<>>(q, std::span<T>{in});
  CHECK(res == (size * (size - 1)) / 2, "reduce iota n=%zu: %llu", size, (unsigned long long)res);
}

// benchmarks/benchmark_reduce.cpp:9-27: device USM filled with 1
static void reduce_device_fill_one(size_t size, cudaStream_t q) {
  using T = uint32_t;
  auto in = usm_unique_ptr<T, alloc::device>(size, q);
  std::vector<T> ones(size, T(1));
  cudaMemcpyAsync(in.get(), ones.data(), in.size_bytes(), cudaMemcpyHostToDevice, q);
  T res = reduce_device<plus<>>(q, in.get_span());
  CHECK(res == T(size), "reduce_device fill(1) n=%zu: %u", size, res);
  // the template parameters of the reference's signature, spelled out
  res = reduce_device<plus<>, T, false, 16384>(q, in.get_span());
  CHECK(res == T(size), "reduce_device<plus<>, T, false, 16384> n=%zu: %u", size, res);
}

// benchmarks/benchmark_scan.cpp:32-51 (fill(1) -> out[n-1] == n)
static void decoupled_fill_one(size_t size, cudaStream_t q) {
  using T = uint;
  auto in = usm_unique_ptr<T, alloc::device>(size, q);
  auto out = usm_unique_ptr<T, alloc::device>(size, q);
  std::vector<T> ones(size, T(1));
  cudaMemcpyAsync(in.get(), ones.data(), in.size_bytes(), cudaMemcpyHostToDevice, q);
  decoupled_scan_device<scan_type::inclusive, plus<>>(q, in.get(), out.get(), size);
  T out_v = 0;
  cudaMemcpyAsync(&out_v, out.get() + size - 1, sizeof(T), cudaMemcpyDeviceToHost, q);
  cudaStreamSynchronize(q);
  CHECK(out_v == size, "decoupled_scan_device fill(1) n=%zu: %u", size, out_v);
  // scan_decoupled_lookback.hpp:227 instantiates the device scan with
  // optimised_offload = false
  decoupled_scan_device<scan_type::inclusive, plus<>, uint32_t, false>(q, in.get(), out.get(), size);
  cudaMemcpyAsync(&out_v, out.get() + size - 1, sizeof(T), cudaMemcpyDeviceToHost, q);
  cudaStreamSynchronize(q);
  CHECK(out_v == size, "decoupled_scan_device<..., false> fill(1) n=%zu: %u", size, out_v);
  decoupled_scan_device<scan_type::exclusive, plus<>, uint32_t, true>(q, in.get(), out.get(), size);
  cudaMemcpyAsync(&out_v, out.get() + size - 1, sizeof(T), cudaMemcpyDeviceToHost, q);
  cudaStreamSynchronize(q);
  CHECK(out_v == size - 1, "decoupled_scan_device<exclusive, ..., true> fill(1) n=%zu: %u", size, out_v);
}

// scan_decoupled_lookback.hpp:219-230: host arrays, both offload settings
static void decoupled_host(size_t size, cudaStream_t q) {
  std::vector<uint32_t> in(size), out(size), want(size);
  uint32_t r = 7u, acc = 0u;
  for (size_t i = 0; i < size; ++i) {
    r = r * 1664525u + 1013904223u;
    in[i] = r >> 16;
    acc += in[i];
    want[i] = acc;
  }
  decoupled_scan<scan_type::inclusive, plus<>, uint32_t, true, 131072>(q, in.data(), out.data(), size);
  CHECK(out == want, "decoupled_scan<..., true, 131072> n=%zu", size);
  std::fill(out.begin(), out.end(), 0u);
  decoupled_scan<scan_type::inclusive, plus<>, uint32_t, false>(q, in.data(), out.data(), size);
  CHECK(out == want, "decoupled_scan<..., false> n=%zu", size);
  std::fill(out.begin(), out.end(), 0u);
  decoupled_scan<scan_type::inclusive, plus<>>(q, in.data(), out.data(), size);
  CHECK(out == want, "decoupled_scan n=%zu", size);
}

// benchmarks/benchmark_scan.cpp:11-30: Basel terms in shared USM, cooperative
// scan, sqrt(6 S_n) -> pi
static void cooperative_basel(size_t size, cudaStream_t q) {
  using T = float;
  auto in = usm_unique_ptr<T, alloc::shared>(size, q);
  auto out = usm_unique_ptr<T, alloc::shared>(size, q);
  double exact = 0.0;
  for (size_t i = 0; i < size; ++i) {
    auto idx = (double)(i + 1);
    in.get()[i] = (T)(1. / (idx * idx));
    exact += double(in.get()[i]);
  }
  cooperative_scan_device<scan_type::inclusive, plus<>>(q, in.get(), out.get(), size);
  cudaStreamSynchronize(q);
  const double last = double(out.get()[size - 1]);
  CHECK(std::fabs(last - exact) / exact < 2e-5, "cooperative Basel n=%zu: %.9f vs %.9f", size, last, exact);
  std::printf("basel cooperative n=%zu: sqrt(6 S_n) = %.7f\n", size, std::sqrt(6.0 * last));
}

// usm_shared_ptr (usm_smart_ptr.hpp:80-105) and the host kind
static void shared_ptr_and_host_kind(cudaStream_t q) {
  using T = uint64_t;
  auto a = usm_shared_ptr<T, alloc::shared>(1000, q);
  auto b = a;  // shared ownership
  std::iota(b.get(), b.get() + b.size(), 0);
  CHECK(a.size() == 1000 && a.size_bytes() == 8000, "usm_shared_ptr size");
  CHECK(reduce_device<plus<>>(q, a.get_span()) == 999 * 1000 / 2, "usm_shared_ptr reduce");
  auto h = usm_unique_ptr<T, alloc::host>(4096, q);
  std::iota(h.get(), h.get() + h.size(), 1);
  CHECK(reduce<plus<>>(q, h.get_span()) == 4096ull * 4097 / 2, "pinned host reduce");
  auto one = usm_unique_ptr<T, alloc::device>(q);
  CHECK(one.size() == 1 && one.get() != nullptr, "single-element buffer");
  auto none = usm_unique_ptr<T, alloc::device>(0, q);
  CHECK(none.get() == nullptr && none.size() == 0, "empty buffer");
}

int main() {
  cudaStream_t q;
  cudaStreamCreate(&q);
  try {
    for (size_t i = 1; i < 1'000'000; i *= 4) {  // tests/test_reduction.cpp:21-31
      reduce_device_iota(i, q);
      reduce_host_iota(i, q);
    }
    std::printf("reduction iota n = 4^0 .. 4^9: done\n");
    for (size_t n : {size_t(1), size_t(1000), size_t(65535), size_t(65536), size_t(1) << 22}) {
      reduce_device_fill_one(n, q);
      decoupled_fill_one(n, q);
      decoupled_host(n, q);
    }
    std::printf("fill(1), host arrays: done\n");
    cooperative_basel(1'000'000, q);
    shared_ptr_and_host_kind(q);
  } catch (const std::exception& e) {
    std::printf("FAIL exception: %s\n", e.what());
    ++failures;
  }
  cudaStreamDestroy(q);
  std::printf(failures ? "FAILED %d\n" : "ALL PASSED\n", failures);
  return failures ? 1 : 0;
}
