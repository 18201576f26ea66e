// parallel_primitives/cooperative_groups.hpp - a grid barrier over any subset
// of the blocks of one launch, and the launch sizing helper.
//
// Mirrors include/cooperative_groups.hpp of the reference:
//   nd_range_barrier<dim> (:26-147): a barrier object in device-accessible
//     memory, built on the host for a launch (nd_range) and a set of
//     cooperating groups given either as a list of group ids (:34-47, :80-83)
//     or as a predicate over group ids (:49-58, :86-89); `wait(item)` returns
//     at once for groups outside the set (:115-116) and is a full barrier among
//     the groups inside it;
//   perform_check (:65-76): the launch must fit co-resident on the device,
//     or forward progress is not guaranteed;
//   get_max_occupancy (:150-167): the largest launch that fits co-resident.
//
// GB300 version. The barrier is a generation counter (count of arrived member
// blocks, generation word advanced by the last arrival with a release store,
// waited on with acquire loads) instead of the reference's two-phase 64-bit
// group mask, so it is reusable back to back and is not limited to 64 groups:
// membership is a bitmap of any length. Every wait is bounded (%globaltimer);
// a wait that runs out records a sticky error in the barrier and returns
// false in every thread of the waiting block, so kernels can leave instead of
// hanging. The co-residency check uses the kernel's real occupancy
// (cudaOccupancyMaxActiveBlocksPerMultiprocessor x SMs) when the kernel is
// given, the SM count (the reference's max_compute_units) otherwise.
// Launch kernels that use it with cudaLaunchCooperativeKernel (or keep the
// grid within get_max_occupancy).
#pragma once

#include <cstdint>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "common.hpp"
#include "pp/ptx.cuh"

namespace parallel_primitives {

class nd_range_barrier {
 public:
  // ---- host side --------------------------------------------------------------
  // All blocks of the launch cooperate when `cooperating_groups` is empty.
  static nd_range_barrier* make_barrier(cudaStream_t s, dim3 grid, dim3 block,
                                        const std::vector<size_t>& cooperating_groups = {},
                                        uint64_t timeout_ns = 1000000000ull) {
    const uint64_t groups = uint64_t(grid.x) * grid.y * grid.z;
    std::vector<uint32_t> mask(words_for(groups), 0u);
    if (cooperating_groups.empty()) {
      for (uint64_t g = 0; g < groups; ++g) mask[g >> 5] |= 1u << (g & 31);
    } else {
      for (size_t g : cooperating_groups) {
        if (g >= groups) throw error(pp::host::Status::invalid_arg, "barrier on an out-of-range group");
        mask[g >> 5] |= 1u << (g & 31);
      }
    }
    return create(s, block, groups, mask, timeout_ns, nullptr, 0);
  }

  // Groups g with predicate(g) true cooperate.
  template <class F>
  static nd_range_barrier* make_barrier_if(cudaStream_t s, dim3 grid, dim3 block, F&& predicate,
                                           uint64_t timeout_ns = 1000000000ull) {
    const uint64_t groups = uint64_t(grid.x) * grid.y * grid.z;
    std::vector<uint32_t> mask(words_for(groups), 0u);
    for (uint64_t g = 0; g < groups; ++g)
      if (predicate(size_t(g))) mask[g >> 5] |= 1u << (g & 31);
    return create(s, block, groups, mask, timeout_ns, nullptr, 0);
  }

  // As make_barrier, with the co-residency check made against the occupancy
  // of `kernel` at this block size and dynamic shared memory.
  template <class K>
  static nd_range_barrier* make_barrier_for(cudaStream_t s, K kernel, dim3 grid, dim3 block,
                                            size_t dynamic_smem = 0,
                                            const std::vector<size_t>& cooperating_groups = {},
                                            uint64_t timeout_ns = 1000000000ull) {
    const uint64_t groups = uint64_t(grid.x) * grid.y * grid.z;
    std::vector<uint32_t> mask(words_for(groups), 0u);
    if (cooperating_groups.empty()) {
      for (uint64_t g = 0; g < groups; ++g) mask[g >> 5] |= 1u << (g & 31);
    } else {
      for (size_t g : cooperating_groups) {
        if (g >= groups) throw error(pp::host::Status::invalid_arg, "barrier on an out-of-range group");
        mask[g >> 5] |= 1u << (g & 31);
      }
    }
    return create(s, block, groups, mask, timeout_ns, reinterpret_cast<const void*>(kernel), dynamic_smem);
  }

  static void destroy(nd_range_barrier* b) {
    if (b) cudaFree(b);
  }

  // Blocking: true when a wait on this barrier has run out of time.
  static bool timed_out(const nd_range_barrier* b, cudaStream_t s) {
    uint32_t e = 0;
    internal::check(pp::host::from_cuda(cudaMemcpyAsync(&e, &b->error_, sizeof(e), cudaMemcpyDeviceToHost, s)),
                    "barrier status");
    internal::check(pp::host::from_cuda(cudaStreamSynchronize(s)), "barrier status");
    return e != 0;
  }

  // ---- device side ------------------------------------------------------------
#if defined(__CUDACC__)
  __device__ __forceinline__ bool is_member() const { return member(linear_group()); }

  // Called by every thread of the block. Non-member blocks return true at
  // once; member blocks return true after every member block has arrived, or
  // false (in all threads) when the wait timed out or a member timed out
  // before.
  __device__ __forceinline__ bool wait() {
    if (!member(linear_group())) return true;
    __syncthreads();
    int ok = 1;
    if (threadIdx.x == 0 && threadIdx.y == 0 && threadIdx.z == 0) {
      const uint32_t gen = pp::ptx::ld_acquire(&gen_);
      __threadfence();
      const uint32_t arrived = atomicAdd(&count_, 1u) + 1u;
      if (arrived == members_) {
        count_ = 0u;
        __threadfence();
        pp::ptx::st_release(&gen_, gen + 1u);
      } else {
        const uint64_t t0 = pp::ptx::globaltimer_ns();
        uint32_t it = 0;
        while (pp::ptx::ld_acquire(&gen_) == gen) {
          if ((++it & 15u) == 0u) {
            if (pp::ptx::ld_relaxed(&error_) != 0u || pp::ptx::globaltimer_ns() - t0 > timeout_ns_) {
              atomicExch(&error_, 1u);
              ok = 0;
              break;
            }
          }
        }
      }
    }
    return __syncthreads_and(ok) != 0;
  }
#endif

 private:
  uint32_t count_;    // member blocks arrived in the current generation
  uint32_t gen_;      // generation, advanced by the last arrival
  uint32_t members_;  // member block count
  uint32_t error_;    // sticky: some wait ran out of time
  uint64_t timeout_ns_;
  uint64_t groups_;
  uint32_t mask_[1];  // membership bitmap, words_for(groups_) words (allocated past the object)

  static size_t words_for(uint64_t groups) { return size_t((groups + 31) / 32); }

#if defined(__CUDACC__)
  __device__ __forceinline__ static uint64_t linear_group() {
    return blockIdx.x + uint64_t(gridDim.x) * (blockIdx.y + uint64_t(gridDim.y) * blockIdx.z);
  }
  __device__ __forceinline__ bool member(uint64_t g) const {
    return g < groups_ && ((mask_[g >> 5] >> (g & 31)) & 1u) != 0u;
  }
#endif

  static nd_range_barrier* create(cudaStream_t s, dim3 block, uint64_t groups,
                                  const std::vector<uint32_t>& mask, uint64_t timeout_ns, const void* kernel,
                                  size_t dynamic_smem) {
    int dev = 0;
    internal::check(pp::host::from_cuda(cudaGetDevice(&dev)), "cudaGetDevice");
    cudaDeviceProp prop{};
    internal::check(pp::host::from_cuda(cudaGetDeviceProperties(&prop, dev)), "cudaGetDeviceProperties");
    const uint64_t threads = uint64_t(block.x) * block.y * block.z;
    if (threads == 0 || threads > uint64_t(prop.maxThreadsPerBlock))
      throw error(pp::host::Status::grid_too_large, "too many items per group: forward progress not guaranteed");
    uint64_t resident = uint64_t(prop.multiProcessorCount);
    if (kernel) {
      int per_sm = 0;
      internal::check(pp::host::from_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                          &per_sm, kernel, int(threads), dynamic_smem)),
                      "occupancy");
      resident = uint64_t(per_sm) * uint64_t(prop.multiProcessorCount);
    }
    if (groups > resident)
      throw error(pp::host::Status::grid_too_large, "too many groups on a grid barrier: forward progress not guaranteed");
    uint32_t members = 0;
    for (uint32_t w : mask) members += uint32_t(__builtin_popcount(w));
    const size_t bytes = offsetof(nd_range_barrier, mask_) + (mask.empty() ? 1 : mask.size()) * sizeof(uint32_t);
    std::vector<unsigned char> image(bytes, 0);
    nd_range_barrier h{};
    h.count_ = 0;
    h.gen_ = 0;
    h.members_ = members;
    h.error_ = 0;
    h.timeout_ns_ = timeout_ns;
    h.groups_ = groups;
    std::memcpy(image.data(), &h, offsetof(nd_range_barrier, mask_));
    if (!mask.empty()) std::memcpy(image.data() + offsetof(nd_range_barrier, mask_), mask.data(), mask.size() * 4);
    void* d = nullptr;
    internal::check(pp::host::from_cuda(cudaMalloc(&d, bytes)), "cudaMalloc");
    const cudaError_t e1 = cudaMemcpyAsync(d, image.data(), bytes, cudaMemcpyHostToDevice, s);
    const cudaError_t e2 = e1 == cudaSuccess ? cudaStreamSynchronize(s) : e1;
    if (e2 != cudaSuccess) {
      cudaFree(d);
      throw error(pp::host::Status::cuda, "barrier upload");
    }
    return static_cast<nd_range_barrier*>(d);
  }
};

// The largest 1-D launch of `kernel` with `block` threads that fits
// co-resident on the current device (get_max_occupancy, :150-167).
template <class K>
inline dim3 get_max_occupancy(K kernel, int block, size_t dynamic_smem = 0) {
  int dev = 0, sms = 0, per_sm = 0;
  internal::check(pp::host::from_cuda(cudaGetDevice(&dev)), "cudaGetDevice");
  internal::check(pp::host::from_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)), "SMs");
  internal::check(pp::host::from_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                      &per_sm, reinterpret_cast<const void*>(kernel), block, dynamic_smem)),
                  "occupancy");
  return dim3(unsigned(per_sm * sms));
}

}  // namespace parallel_primitives
