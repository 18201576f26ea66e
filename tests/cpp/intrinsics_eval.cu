// Evaluates the bit and byte intrinsics of include/parallel_primitives/
// intrinsics.hpp on requests read from standard input, on the host or (one
// thread per request) on the GPU, and prints one result per line. The tests
// feed it the operands of the reference-produced fixtures in tests/golden/
// and compare the answers with the reference's.
//
// Request line: "op width word a b" (decimal), result: one decimal per line.
//   op 0 get_byte(word, a)             op 1 set_byte(word, byte b, a)
//   op 2 set_bit_in_word<b != 0>(word, a)
//   op 3 set_bit_in_word(word, a, b != 0)
//   op 4 read_bit(word, a) as 0/1      op 5 flip_bit(word, a)
//   (word of `width` bytes: 1, 2, 4 or 8)
//   op 10 funnelshift_l(lo = word & 0xffffffff, hi = word >> 32, a)
//   op 11 funnelshift_r(lo, hi, a)     op 12 brev32(word)
//   op 13 brev64(word)                 op 14 upsample of the 4 low bytes of
//                                            word, most significant first
// Usage: intrinsics_eval host|device < requests
#include <cinttypes>
#include <cstdio>
#include <cstring>
#include <vector>

#include <parallel_primitives/intrinsics.hpp>

struct Req {
  int op, width;
  uint64_t word;
  uint32_t a, b;
};

template <class T>
__host__ __device__ uint64_t byte_bit(const Req& r) {
  using namespace parallel_primitives::ext;
  const T w = static_cast<T>(r.word);
  switch (r.op) {
    case 0:
      return get_byte<T>(w, r.a);
    case 1:
      return set_byte<T>(w, uint8_t(r.b), r.a);
    case 2:
      return r.b ? set_bit_in_word<true, T>(w, r.a) : set_bit_in_word<false, T>(w, r.a);
    case 3:
      return set_bit_in_word<T>(w, r.a, r.b != 0);
    case 4:
      return read_bit<T>(w, r.a) ? 1u : 0u;
    case 5:
      return flip_bit<T>(w, r.a);
    default:
      return ~uint64_t(0);
  }
}

__host__ __device__ uint64_t eval(const Req& r) {
  using namespace parallel_primitives::ext;
  if (r.op <= 5) {
    switch (r.width) {
      case 1:
        return byte_bit<uint8_t>(r);
      case 2:
        return byte_bit<uint16_t>(r);
      case 4:
        return byte_bit<uint32_t>(r);
      case 8:
        return byte_bit<uint64_t>(r);
      default:
        return ~uint64_t(0);
    }
  }
  const uint32_t lo = uint32_t(r.word), hi = uint32_t(r.word >> 32);
  switch (r.op) {
    case 10:
      return funnelshift_l(lo, hi, r.a);
    case 11:
      return funnelshift_r(lo, hi, r.a);
    case 12:
      return brev32(lo);
    case 13:
      return brev64(r.word);
    case 14:
      return upsample(uint8_t(r.word >> 24), uint8_t(r.word >> 16), uint8_t(r.word >> 8), uint8_t(r.word));
    default:
      return ~uint64_t(0);
  }
}

__global__ void eval_kernel(const Req* req, uint64_t* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = eval(req[i]);
}

int main(int argc, char** argv) {
  const bool device = argc > 1 && std::strcmp(argv[1], "device") == 0;
  std::vector<Req> req;
  Req r;
  unsigned long long w;
  while (std::scanf("%d %d %llu %u %u", &r.op, &r.width, &w, &r.a, &r.b) == 5) {
    r.word = w;
    req.push_back(r);
  }
  const int n = int(req.size());
  std::vector<uint64_t> out(n, 0);
  if (!device) {
    for (int i = 0; i < n; ++i) out[i] = eval(req[i]);
  } else if (n > 0) {
    Req* d_req = nullptr;
    uint64_t* d_out = nullptr;
    if (cudaMalloc(&d_req, n * sizeof(Req)) != cudaSuccess || cudaMalloc(&d_out, n * sizeof(uint64_t)) != cudaSuccess) {
      std::fprintf(stderr, "cudaMalloc failed\n");
      return 2;
    }
    cudaMemcpy(d_req, req.data(), n * sizeof(Req), cudaMemcpyHostToDevice);
    eval_kernel<<<(n + 255) / 256, 256>>>(d_req, d_out, n);
    const cudaError_t e = cudaMemcpy(out.data(), d_out, n * sizeof(uint64_t), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      std::fprintf(stderr, "device evaluation failed: %s\n", cudaGetErrorString(e));
      return 2;
    }
    cudaFree(d_req);
    cudaFree(d_out);
  }
  for (int i = 0; i < n; ++i) std::printf("%" PRIu64 "\n", out[i]);
  return 0;
}
