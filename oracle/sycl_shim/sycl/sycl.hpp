// sycl.hpp - a SYCL 2020 subset that runs kernels on CPU threads.
// TEST INFRASTRUCTURE ONLY: it exists so that the reference's scan / reduce
// headers compile UNMODIFIED with g++ and run on the host cores
// (oracle/ref_entry.cpp, built by oracle/build_oracle.py into oracle/_ref).
//
// Device model (a "CPU device" that is not a GPU):
//   * is_gpu() == false, so the reference's small-input host offloads are
//     skipped and its device algorithms always run;
//   * max_compute_units = number of host threads (SHIM_CUS overrides);
//   * max_work_group_size = 1 and every kernel's work-group size is 1, so
//     group barriers are no-ops and group algorithms are sequential loops;
//   * local_mem_size = 64 KiB (SHIM_LOCAL_MEM overrides);
//   * every work-group of a launch runs on its own std::thread when the launch
//     has at most max_compute_units groups (the persistent and cooperative
//     kernels spin on each other, so they must be co-resident); larger
//     launches are spread over a pool of max_compute_units threads;
//   * USM allocations are plain host memory; queues execute synchronously.
#pragma once

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <limits>
#include <memory>
#include <mutex>
#include <numeric>
#include <optional>
#include <span>
#include <stdexcept>
#include <string>
#include <thread>
#include <type_traits>
#include <utility>
#include <vector>
#include <sys/types.h>

#ifndef __builtin_assume
#define __builtin_assume(x) ((void)0)
#endif

// The reference calls fail_to_compile<value, T, func>() unqualified in
// discarded `if constexpr` branches; a template of that shape must be
// visible for the headers to parse (it is never instantiated).
template <auto V, class... Ts>
constexpr void fail_to_compile() {}

namespace sycl {

// ---------------------------------------------------------------- basics
struct half {
  uint16_t bits;
};

template <class T>
constexpr T min(T a, T b) {
  return b < a ? b : a;
}
template <class T>
constexpr T max(T a, T b) {
  return a < b ? b : a;
}

template <class T, std::size_t E = std::dynamic_extent>
using span = std::span<T, E>;

inline uint32_t upsample(uint16_t hi, uint16_t lo) { return (uint32_t(hi) << 16) | lo; }

namespace ext::intel {
inline uint32_t ctz(uint32_t x) { return x ? uint32_t(__builtin_ctz(x)) : 32u; }
}  // namespace ext::intel

// ---------------------------------------------------------------- functors
template <class T = void>
struct plus {
  T operator()(const T& a, const T& b) const { return a + b; }
};
template <>
struct plus<void> {
  template <class T, class U>
  auto operator()(const T& a, const U& b) const {
    return a + b;
  }
};
template <class T = void>
struct multiplies {
  T operator()(const T& a, const T& b) const { return a * b; }
};
template <>
struct multiplies<void> {
  template <class T, class U>
  auto operator()(const T& a, const U& b) const {
    return a * b;
  }
};
template <class T = void>
struct bit_and {
  T operator()(const T& a, const T& b) const { return a & b; }
};
template <>
struct bit_and<void> {
  template <class T, class U>
  auto operator()(const T& a, const U& b) const {
    return a & b;
  }
};
template <class T = void>
struct bit_or {
  T operator()(const T& a, const T& b) const { return a | b; }
};
template <>
struct bit_or<void> {
  template <class T, class U>
  auto operator()(const T& a, const U& b) const {
    return a | b;
  }
};
template <class T = void>
struct bit_xor {
  T operator()(const T& a, const T& b) const { return a ^ b; }
};
template <>
struct bit_xor<void> {
  template <class T, class U>
  auto operator()(const T& a, const U& b) const {
    return a ^ b;
  }
};
template <class T = void>
struct minimum {
  T operator()(const T& a, const T& b) const { return (a < b) ? a : b; }
};
template <>
struct minimum<void> {
  template <class T, class U>
  std::common_type_t<T, U> operator()(const T& a, const U& b) const {
    return (a < b) ? a : b;
  }
};
template <class T = void>
struct maximum {
  T operator()(const T& a, const T& b) const { return (a > b) ? a : b; }
};
template <>
struct maximum<void> {
  template <class T, class U>
  std::common_type_t<T, U> operator()(const T& a, const U& b) const {
    return (a > b) ? a : b;
  }
};

// known_identity / has_known_identity (SYCL 2020 4.9.2)
template <class Op, class T>
struct known_identity {
 private:
  template <template <class> class F>
  static constexpr bool is() {
    return std::is_same_v<Op, F<void>> || std::is_same_v<Op, F<T>>;
  }

 public:
  static constexpr bool arith = std::is_arithmetic_v<T>;
  static constexpr bool known = (arith && (is<plus>() || is<multiplies>() || is<minimum>() || is<maximum>())) ||
                                (std::is_integral_v<T> && (is<bit_and>() || is<bit_or>() || is<bit_xor>()));
  static constexpr T compute() {
    if constexpr (is<plus>() || is<bit_or>() || is<bit_xor>()) {
      return T{};
    } else if constexpr (is<multiplies>()) {
      return T{1};
    } else if constexpr (is<bit_and>()) {
      return static_cast<T>(~T{});
    } else if constexpr (is<minimum>()) {
      if constexpr (std::numeric_limits<T>::has_infinity) return std::numeric_limits<T>::infinity();
      else return std::numeric_limits<T>::max();
    } else if constexpr (is<maximum>()) {
      if constexpr (std::numeric_limits<T>::has_infinity) return -std::numeric_limits<T>::infinity();
      else return std::numeric_limits<T>::lowest();
    } else {
      return T{};
    }
  }
  static constexpr T value = compute();
};
template <class Op, class T>
struct has_known_identity : std::bool_constant<known_identity<Op, T>::known> {};

// ---------------------------------------------------------------- enums
enum class memory_order { relaxed, acquire, release, acq_rel, seq_cst };
inline constexpr memory_order memory_order_relaxed = memory_order::relaxed;
inline constexpr memory_order memory_order_acquire = memory_order::acquire;
inline constexpr memory_order memory_order_release = memory_order::release;
inline constexpr memory_order memory_order_acq_rel = memory_order::acq_rel;
inline constexpr memory_order memory_order_seq_cst = memory_order::seq_cst;
enum class memory_scope { work_item, sub_group, work_group, device, system };
inline constexpr memory_scope memory_scope_work_item = memory_scope::work_item;
inline constexpr memory_scope memory_scope_sub_group = memory_scope::sub_group;
inline constexpr memory_scope memory_scope_work_group = memory_scope::work_group;
inline constexpr memory_scope memory_scope_device = memory_scope::device;
inline constexpr memory_scope memory_scope_system = memory_scope::system;

namespace access {
enum class mode { read, write, read_write, discard_write, discard_read_write, atomic };
enum class target { global_buffer, constant_buffer, local, host_buffer, device };
enum class fence_space { local_space, global_space, global_and_local };
enum class address_space {
  private_space,
  global_space,
  constant_space,
  local_space,
  generic_space,
  ext_intel_global_device_space,
  ext_intel_host_device_space
};
}  // namespace access
using access_mode = access::mode;

namespace usm {
enum class alloc { host, device, shared, unknown };
}

enum class bundle_state { input, object, executable };

inline std::memory_order to_std(memory_order o) {
  switch (o) {
    case memory_order::relaxed:
      return std::memory_order_relaxed;
    case memory_order::acquire:
      return std::memory_order_acquire;
    case memory_order::release:
      return std::memory_order_release;
    case memory_order::acq_rel:
      return std::memory_order_acq_rel;
    default:
      return std::memory_order_seq_cst;
  }
}

inline void atomic_fence(memory_order o, memory_scope) { std::atomic_thread_fence(to_std(o)); }

template <class T, memory_order DefaultOrder, memory_scope Scope,
          access::address_space Space = access::address_space::generic_space>
class atomic_ref {
 public:
  explicit atomic_ref(T& r) : ref_(r) {}
  T load(memory_order o = DefaultOrder) const { return ref_.load(to_std(o)); }
  void store(T v, memory_order o = DefaultOrder) const { ref_.store(v, to_std(o)); }
  T fetch_or(T v, memory_order o = DefaultOrder) const { return ref_.fetch_or(v, to_std(o)); }
  T fetch_and(T v, memory_order o = DefaultOrder) const { return ref_.fetch_and(v, to_std(o)); }
  T fetch_add(T v, memory_order o = DefaultOrder) const { return ref_.fetch_add(v, to_std(o)); }
  T exchange(T v, memory_order o = DefaultOrder) const { return ref_.exchange(v, to_std(o)); }

 private:
  mutable std::atomic_ref<T> ref_;
};

template <class T, access::address_space Space, int Decorated = 0>
class multi_ptr {
 public:
  multi_ptr(T* p) : p_(p) {}  // NOLINT(implicit)
  T* get() const { return p_; }
  operator T*() const { return p_; }

 private:
  T* p_;
};

// ---------------------------------------------------------------- ranges / items
template <int D = 1>
class range {
  static_assert(D == 1, "the shim supports one-dimensional ranges");

 public:
  range(std::size_t n = 0) : n_(n) {}  // NOLINT(implicit): SYCL allows range<1> from a size
  std::size_t size() const { return n_; }
  std::size_t get(int) const { return n_; }
  std::size_t operator[](int) const { return n_; }

 private:
  std::size_t n_;
};
range(std::size_t)->range<1>;

template <int D = 1>
class id {
 public:
  id(std::size_t v = 0) : v_(v) {}  // NOLINT(implicit)
  operator std::size_t() const { return v_; }

 private:
  std::size_t v_;
};

template <int D = 1>
class nd_range {
 public:
  nd_range(range<D> global, range<D> local) : global_(global), local_(local) {}
  range<D> get_global_range() const { return global_; }
  range<D> get_local_range() const { return local_; }
  range<D> get_group_range() const { return range<D>(local_.size() ? global_.size() / local_.size() : 0); }

 private:
  range<D> global_, local_;
};

template <int D = 1>
class group {
 public:
  group(std::size_t id, std::size_t count) : id_(id), count_(count) {}
  std::size_t get_group_linear_id() const { return id_; }
  range<D> get_group_range() const { return range<D>(count_); }
  range<D> get_local_range() const { return range<D>(1); }
  std::size_t get_local_linear_id() const { return 0; }

 private:
  std::size_t id_, count_;
};

class sub_group {
 public:
  range<1> get_local_range() const { return range<1>(1); }
  range<1> get_max_local_range() const { return range<1>(1); }
  range<1> get_group_range() const { return range<1>(1); }
  std::size_t get_local_linear_id() const { return 0; }
  std::size_t get_group_linear_id() const { return 0; }
  bool leader() const { return true; }
};

template <int D = 1>
class nd_item {
 public:
  nd_item(std::size_t group_id, std::size_t group_count) : g_(group_id), count_(group_count) {}
  group<D> get_group() const { return group<D>(g_, count_); }
  sub_group get_sub_group() const { return sub_group{}; }
  std::size_t get_group_linear_id() const { return g_; }
  std::size_t get_local_linear_id() const { return 0; }
  std::size_t get_global_linear_id() const { return g_; }
  range<D> get_group_range() const { return range<D>(count_); }
  range<D> get_local_range() const { return range<D>(1); }
  range<D> get_global_range() const { return range<D>(count_); }
  void barrier(access::fence_space = access::fence_space::global_and_local) const {}

 private:
  std::size_t g_, count_;
};

// ---------------------------------------------------------------- group algorithms (one work-item)
template <class G, class InPtr, class OutPtr, class Op, class T>
OutPtr joint_inclusive_scan(G, InPtr first, InPtr last, OutPtr result, Op op, T init) {
  T acc = init;
  for (; first != last; ++first, ++result) {
    acc = op(acc, *first);
    *result = acc;
  }
  return result;
}
template <class G, class InPtr, class OutPtr, class Op>
OutPtr joint_inclusive_scan(G, InPtr first, InPtr last, OutPtr result, Op op) {
  if (first == last) return result;
  auto acc = *first;
  *result = acc;
  for (++first, ++result; first != last; ++first, ++result) {
    acc = op(acc, *first);
    *result = acc;
  }
  return result;
}
template <class G, class InPtr, class OutPtr, class T, class Op>
OutPtr joint_exclusive_scan(G, InPtr first, InPtr last, OutPtr result, T init, Op op) {
  T acc = init;
  for (; first != last; ++first, ++result) {
    const T x = *first;
    *result = acc;
    acc = op(acc, x);
  }
  return result;
}
template <class G, class T, class Op>
T reduce_over_group(G, T x, Op) {
  return x;
}
template <class G, class T, class Op>
T reduce_over_group(G, T x, T init, Op op) {
  return op(init, x);
}
template <class G, class T, class Op>
T inclusive_scan_over_group(G, T x, Op) {
  return x;
}
template <class G, class T, class Op>
T exclusive_scan_over_group(G, T x, Op) {
  return known_identity<Op, T>::value;
}
template <class G, class T>
T select_from_group(G, T x, std::size_t) {
  return x;
}
template <class G, class T>
T group_broadcast(G, T x, std::size_t = 0) {
  return x;
}

// ---------------------------------------------------------------- device / queue
namespace info {
namespace device {
struct local_mem_size {
  using return_type = uint64_t;
};
struct max_compute_units {
  using return_type = uint32_t;
};
struct max_work_group_size {
  using return_type = std::size_t;
};
struct name {
  using return_type = std::string;
};
struct driver_version {
  using return_type = std::string;
};
}  // namespace device
namespace kernel_device_specific {
struct work_group_size {
  using return_type = std::size_t;
};
struct ext_codeplay_num_regs {
  using return_type = uint32_t;
};
}  // namespace kernel_device_specific
}  // namespace info

namespace shim {
inline uint32_t compute_units() {
  if (const char* e = std::getenv("SHIM_CUS")) return uint32_t(std::max(1, std::atoi(e)));
  const unsigned h = std::thread::hardware_concurrency();
  return h ? h : 1u;
}
inline uint64_t local_mem() {
  if (const char* e = std::getenv("SHIM_LOCAL_MEM")) return uint64_t(std::atoll(e));
  return 65536;
}
// local memory of the work-group the current thread is running
inline thread_local unsigned char* tl_local = nullptr;
}  // namespace shim

class device {
 public:
  bool is_gpu() const { return false; }
  bool is_cpu() const { return true; }
  bool is_host() const { return false; }
  template <class Param>
  typename Param::return_type get_info() const {
    if constexpr (std::is_same_v<Param, info::device::local_mem_size>) {
      return shim::local_mem();
    } else if constexpr (std::is_same_v<Param, info::device::max_compute_units>) {
      return shim::compute_units();
    } else if constexpr (std::is_same_v<Param, info::device::max_work_group_size>) {
      return 1;
    } else if constexpr (std::is_same_v<Param, info::device::name>) {
      return "SYCL CPU shim";
    } else {
      return "shim";
    }
  }
};

class context {};

class kernel_id {};
template <class Name>
kernel_id get_kernel_id() {
  return {};
}
class kernel {
 public:
  template <class Param>
  typename Param::return_type get_info(const device&) const {
    if constexpr (std::is_same_v<Param, info::kernel_device_specific::work_group_size>) return 1;
    else return 0;
  }
};
template <bundle_state S>
class kernel_bundle {
 public:
  kernel get_kernel(const kernel_id&) const { return {}; }
};
template <bundle_state S>
kernel_bundle<S> get_kernel_bundle(const context&) {
  return {};
}

class event {
 public:
  void wait() {}
  void wait_and_throw() {}
};

template <class T>
class buffer {
 public:
  buffer(T* host, const range<1>& r) : p_(host), n_(r.size()) {}
  T* data() const { return p_; }
  std::size_t size() const { return n_; }

 private:
  T* p_;
  std::size_t n_;
};

class handler;

// accessor: local (per work-group arena) or constant_buffer (over a host buffer)
template <class T, int D = 1, access::mode M = access::mode::read_write,
          access::target Tg = access::target::global_buffer>
class accessor;

template <class T, int D, access::mode M>
class accessor<T, D, M, access::target::local> {
 public:
  accessor(range<D> r, handler& cgh);
  T* get_pointer() const { return reinterpret_cast<T*>(shim::tl_local + offset_); }
  T& operator[](std::size_t i) const { return get_pointer()[i]; }

 private:
  std::size_t offset_ = 0;
};

template <class T, int D, access::mode M>
class accessor<T, D, M, access::target::constant_buffer> {
 public:
  accessor(buffer<T>& b, handler&) : p_(b.data()) {}
  const T& operator[](std::size_t i) const { return p_[i]; }

 private:
  T* p_;
};

template <class T, class Op>
struct reduction_desc {
  T* out;
  Op op;
};
template <class T, class Op>
reduction_desc<T, Op> reduction(buffer<T>& b, handler&, Op op) {
  return {b.data(), op};
}

template <class T, class Op>
class reducer {
 public:
  explicit reducer(Op op) : op_(op), v_(known_identity<Op, T>::value) {}
  void combine(const T& x) { v_ = op_(v_, x); }
  T value() const { return v_; }

 private:
  Op op_;
  T v_;
};

class handler {
 public:
  std::size_t alloc_local(std::size_t bytes) {
    const std::size_t off = (local_bytes_ + 63) & ~std::size_t(63);
    local_bytes_ = off + bytes;
    return off;
  }
  void depends_on(const event&) {}

  template <class Name = void, class F>
  void parallel_for(const nd_range<1>& r, F f) {
    check(r);
    run_groups(r.get_group_range().size(), [&](std::size_t g, std::size_t G, std::size_t) { f(nd_item<1>(g, G)); });
  }

  template <class Name = void, class T, class Op, class F>
  void parallel_for(const nd_range<1>& r, reduction_desc<T, Op> red, F f) {
    check(r);
    const std::size_t G = r.get_group_range().size();
    const std::size_t P = std::max<std::size_t>(1, std::min<std::size_t>(G, shim::compute_units()));
    std::vector<reducer<T, Op>> parts(P, reducer<T, Op>(red.op));
    run_groups(G, [&](std::size_t g, std::size_t Gc, std::size_t worker) { f(nd_item<1>(g, Gc), parts[worker]); });
    T acc = *red.out;
    for (auto& p : parts) acc = red.op(acc, p.value());
    *red.out = acc;
  }

  template <class Name = void, class F>
  void single_task(F f) {
    f();
  }

 private:
  static void check(const nd_range<1>& r) {
    if (r.get_local_range().size() != 1)
      throw std::runtime_error("SYCL shim: only work-groups of one work-item are supported");
  }

  // Runs groups 0..G-1. When G fits the compute units every group gets its own
  // thread (co-residency for kernels that wait on each other); otherwise a
  // pool of compute_units threads takes groups in order.
  template <class Body>
  void run_groups(std::size_t G, Body body) {
    if (G == 0) return;
    const std::size_t cus = shim::compute_units();
    const std::size_t P = std::min(G, cus);
    std::atomic<std::size_t> next{0};
    auto worker = [&](std::size_t w) {
      std::vector<unsigned char> arena(local_bytes_ + 64);
      shim::tl_local = arena.data();
      for (std::size_t g = next.fetch_add(1); g < G; g = next.fetch_add(1)) body(g, G, w);
      shim::tl_local = nullptr;
    };
    if (P == 1) {
      worker(0);
      return;
    }
    std::vector<std::thread> th;
    th.reserve(P);
    for (std::size_t w = 0; w < P; ++w) th.emplace_back(worker, w);
    for (auto& t : th) t.join();
  }

  std::size_t local_bytes_ = 0;
};

template <class T, int D, access::mode M>
accessor<T, D, M, access::target::local>::accessor(range<D> r, handler& cgh)
    : offset_(cgh.alloc_local(r.size() * sizeof(T))) {}

class queue {
 public:
  queue() = default;
  template <class Selector>
  explicit queue(const Selector&) {}
  device get_device() const { return {}; }
  context get_context() const { return {}; }
  template <class CGF>
  event submit(CGF cgf) {
    handler h;
    cgf(h);
    return {};
  }
  template <class T>
  event fill(T* p, const T& v, std::size_t count) {
    for (std::size_t i = 0; i < count; ++i) new (p + i) T(v);
    return {};
  }
  event memcpy(void* dst, const void* src, std::size_t bytes) {
    std::memmove(dst, src, bytes);
    return {};
  }
  void wait() {}
};

// ---------------------------------------------------------------- USM
inline void* shim_alloc(std::size_t bytes) {
  void* p = nullptr;
  if (posix_memalign(&p, 64, bytes ? bytes : 1) != 0) throw std::bad_alloc();
  return p;
}
template <class T>
T* malloc_device(std::size_t count, const queue&) {
  return static_cast<T*>(shim_alloc(count * sizeof(T)));
}
template <class T>
T* malloc_shared(std::size_t count, const queue&) {
  return static_cast<T*>(shim_alloc(count * sizeof(T)));
}
template <class T>
T* malloc_host(std::size_t count, const queue&) {
  return static_cast<T*>(shim_alloc(count * sizeof(T)));
}
template <class T>
T* malloc(std::size_t count, const queue&, usm::alloc) {
  return static_cast<T*>(shim_alloc(count * sizeof(T)));
}
inline void free(void* p, const queue&) { std::free(p); }

}  // namespace sycl
