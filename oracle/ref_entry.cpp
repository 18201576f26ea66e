// ref_entry.cpp - extern "C" entry points over the reference's own scan /
// reduce / intrinsics headers, compiled unmodified from the reference
// checkout (include path) against the SYCL CPU shim (oracle/sycl_shim).
// TEST INFRASTRUCTURE ONLY: it produces the reference's outputs on the CPU
// to pin the oracle and to generate the golden fixtures in tests/golden/.
//
// Built with -fwrapv so that the reference's signed-integer plus / multiplies
// wrap like the product library's (the C++ standard leaves them undefined).
#include <sycl/sycl.hpp>

#include <parallel_primitives/reduction.hpp>
#include <parallel_primitives/scan_cooperative.hpp>
#include <parallel_primitives/scan_decoupled_lookback.hpp>
#include <intrinsics.hpp>

#include <cstdint>

using parallel_primitives::scan_type;

namespace {

sycl::queue& queue() {
  static sycl::queue q;
  return q;
}

enum { kDecoupled = 0, kCooperative = 1, kRegular = 2 };

template <class T, class Op>
int run_scan(int algo, int exclusive, const void* in, void* out, uint64_t n) {
  const T* i = static_cast<const T*>(in);
  T* o = static_cast<T*>(out);
  auto& q = queue();
  if (algo == kDecoupled) {
    if (exclusive)
      parallel_primitives::decoupled_scan_device<scan_type::exclusive, Op, T>(q, i, o, n);
    else
      parallel_primitives::decoupled_scan_device<scan_type::inclusive, Op, T>(q, i, o, n);
  } else if (algo == kCooperative) {
    if (exclusive)
      parallel_primitives::cooperative_scan_device<scan_type::exclusive, Op, T>(q, i, o, n);
    else
      parallel_primitives::cooperative_scan_device<scan_type::inclusive, Op, T>(q, i, o, n);
  } else {
    return -1;
  }
  return 0;
}

template <class T, class Op>
int run_reduce(const void* in, uint64_t n, void* result) {
  T r = parallel_primitives::reduce_device<Op, T>(queue(), sycl::span<T>(const_cast<T*>(static_cast<const T*>(in)), n));
  *static_cast<T*>(result) = r;
  return 0;
}

template <class T, class F>
int with_op(int op, F&& f) {
  switch (op) {
    case 0:
      return f.template operator()<T, sycl::plus<>>();
    case 1:
      return f.template operator()<T, sycl::multiplies<>>();
    case 5:
      return f.template operator()<T, sycl::minimum<>>();
    case 6:
      return f.template operator()<T, sycl::maximum<>>();
    default:
      break;
  }
  if constexpr (std::is_integral_v<T>) {
    switch (op) {
      case 2:
        return f.template operator()<T, sycl::bit_and<>>();
      case 3:
        return f.template operator()<T, sycl::bit_or<>>();
      case 4:
        return f.template operator()<T, sycl::bit_xor<>>();
      default:
        break;
    }
  }
  return -1;
}

template <class F>
int with_type(int dtype, int op, F&& f) {
  switch (dtype) {
    case 0:
      return with_op<int32_t>(op, f);
    case 1:
      return with_op<uint32_t>(op, f);
    case 2:
      return with_op<int64_t>(op, f);
    case 3:
      return with_op<uint64_t>(op, f);
    case 4:
      return with_op<float>(op, f);
    case 5:
      return with_op<double>(op, f);
    default:
      return -1;
  }
}

}  // namespace

extern "C" {

// dtype / op numbering as pp_dtype / pp_op; algo 0 = decoupled, 1 = cooperative
int ref_scan(int algo, int dtype, int op, int exclusive, const void* in, void* out, uint64_t n) {
  return with_type(dtype, op, [&]<class T, class Op>() { return run_scan<T, Op>(algo, exclusive, in, out, n); });
}

int ref_reduce(int dtype, int op, const void* in, uint64_t n, void* result) {
  return with_type(dtype, op, [&]<class T, class Op>() { return run_reduce<T, Op>(in, n, result); });
}

int ref_decoupled_scan_u32_plus(const void* in, void* out, uint64_t n, int exclusive) {
  return run_scan<uint32_t, sycl::plus<>>(kDecoupled, exclusive, in, out, n);
}

int ref_num_groups(void) { return int(sycl::shim::compute_units()); }

uint32_t ref_funnelshift_l(uint32_t lo, uint32_t hi, uint32_t shift) { return sycl::ext::funnelshift_l(lo, hi, shift); }
uint32_t ref_funnelshift_r(uint32_t lo, uint32_t hi, uint32_t shift) { return sycl::ext::funnelshift_r(lo, hi, shift); }
uint32_t ref_brev32(uint32_t x) { return sycl::ext::brev32(x); }
uint64_t ref_brev64(uint64_t x) { return sycl::ext::brev64(x); }
uint32_t ref_upsample(uint8_t a, uint8_t b, uint8_t c, uint8_t d) { return sycl::ext::upsample<uint8_t>(a, b, c, d); }

// Byte / bit helpers (intrinsics.hpp:150-202) on unsigned words of `width`
// bytes (1, 2, 4 or 8), the word passed and returned zero-extended to 64 bits.
// op: 0 get_byte(word, a), 1 set_byte(word, byte b, a), 2 set_bit_in_word<b>(word, a),
//     3 set_bit_in_word(word, a, bool b), 4 read_bit(word, a), 5 flip_bit(word, a).
uint64_t ref_byte_bit(int op, int width, uint64_t word, uint32_t a, uint32_t b) {
  auto run = [&]<class T>(T w) -> uint64_t {
    switch (op) {
      case 0:
        return sycl::ext::get_byte<T>(w, a);
      case 1:
        return sycl::ext::set_byte<T>(w, uint8_t(b), a);
      case 2:
        return b ? sycl::ext::set_bit_in_word<true, T>(w, a) : sycl::ext::set_bit_in_word<false, T>(w, a);
      case 3:
        return sycl::ext::set_bit_in_word<T>(w, a, b != 0);
      case 4:
        return sycl::ext::read_bit<T>(w, a) ? 1u : 0u;
      case 5:
        return sycl::ext::flip_bit<T>(w, a);
      default:
        return ~uint64_t(0);
    }
  };
  switch (width) {
    case 1:
      return run(uint8_t(word));
    case 2:
      return run(uint16_t(word));
    case 4:
      return run(uint32_t(word));
    case 8:
      return run(uint64_t(word));
    default:
      return ~uint64_t(0);
  }
}
}
