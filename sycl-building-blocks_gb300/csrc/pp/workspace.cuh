// Device workspace shared by the scan / reduce kernels, and the packed
// look-back descriptors.
//
// Layout (one contiguous, 256-byte aligned device buffer):
//   [0, 4096)                      WsHeader: ticket counter, CTA exit counter,
//                                  epoch, sticky error word, abort flag, grid
//                                  barrier words.
//   [4096, 4096 + kAuxBytes)       per-block partials (reduction, cooperative
//                                  scan block and window aggregates).
//   [4096 + kAuxBytes, ...)        look-back descriptors, desc_words() 64-bit
//                                  words per tile.
//
// Descriptor words replace the reference's unpacked partition_descriptor
// {inclusive_prefix_, aggregate_, status} (include/parallel_primitives/
// internal/partition_descriptor.h:92-141, status enum :10-14). Each 64-bit
// word is {tag:32 | payload:32} with tag = (epoch << 2) | status, status
// 1 = aggregate available, 2 = inclusive prefix available, anything else
// invalid. A value wider than 32 bits is split over 2 or 4 words that all
// carry the tag; a reader accepts a descriptor only when every word carries
// the same current-epoch tag, so a half-updated descriptor reads as invalid.
// Every word is published with one 64-bit atomic max (red.max: the tag sits in
// the high bits, so within an epoch a word can only move invalid -> aggregate
// -> prefix, whatever order two publishers' writes land in) and read with
// ld.relaxed.gpu: the payload travels with its flag, so no fence is needed on
// either side.
//
// The epoch removes the per-call descriptor fill of the reference
// (scan_decoupled_lookback.hpp:115-116): the last CTA of every launch bumps
// the epoch and re-arms the ticket and exit counters, so back-to-back calls
// and CUDA-graph replays need no memset node. When the 30-bit epoch wraps the
// last CTA clears every descriptor word ever used (high-water mark).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "ptx.cuh"
#include "warp.cuh"

namespace pp {

// Status codes shared with the C ABI (include/pp_gb300.h).
enum DeviceError : uint32_t {
  kDevOk = 0,
  kDevTimeout = 4,
};

struct WsHeader {
  unsigned long long ticket;          // next tile ticket
  unsigned long long desc_words_hwm;  // descriptor words ever used
  unsigned long long error_detail;    // e.g. the tile whose wait gave up
  unsigned int done;                  // CTAs that have exited this launch
  unsigned int epoch;                 // in [0, kEpochLimit): tags use epoch + 1
  unsigned int error;                 // first device error, sticky until read
  unsigned int abort;                 // set on a timeout; every spin exits
  unsigned int bar_count;             // grid barrier arrivals
  unsigned int bar_gen;               // grid barrier generation
  unsigned int debug_spin;            // unused padding / diagnostics
  unsigned int pad_;
  // look-back counters, kept only while the descriptor perturbation knob is
  // on (ScanArgs::debug_delay_ns != 0) and never re-armed by a launch:
  // [0] tiles whose nearest predecessor already held its inclusive prefix
  //     (reduce-then-scan), [1] tiles that folded published aggregates back to
  //     an older prefix (scan-then-reduce), [2] look-backs that folded more
  //     than 32 predecessors (two or more windows), [3] polls that met a
  //     descriptor whose words carried different tags (half written)
  unsigned long long dbg[4];
  // cooperative rounds of the staged kernel: arrivals at the window barriers,
  // window w counted in slot w % 2 (re-armed by the last CTA of a launch)
  unsigned long long coop_arrive[2];
};

constexpr size_t kHeaderBytes = 4096;
constexpr int kMaxPartials = 8192;                 // blocks with a partial slot
constexpr size_t kAuxBytes = size_t(kMaxPartials) * 16;
constexpr size_t kDescOffset = kHeaderBytes + kAuxBytes;
constexpr uint32_t kEpochLimit = (1u << 30) - 1;  // tag epoch = epoch + 1 in [1, 2^30)

enum DescStatus : uint32_t { kInvalid = 0, kAggregate = 1, kPrefix = 2 };

__host__ __device__ constexpr size_t workspace_bytes_for_desc_words(uint64_t words) {
  return kDescOffset + words * 8;
}

template <class C>
struct desc_codec {
  static constexpr int PW = (sizeof(C) + 3) / 4;  // 32-bit payload words
  static_assert(PW <= 4, "look-back carries wider than 16 bytes are not supported");
  static constexpr int W = PW == 1 ? 1 : (PW == 2 ? 2 : 4);  // 64-bit descriptor words

  __device__ __forceinline__ static void publish(uint64_t* d, const C& v, uint32_t tag) {
    words<C> p = to_words(v);
    const uint64_t hi = uint64_t(tag) << 32;
#pragma unroll
    for (int i = 0; i < W; ++i) {
      const uint32_t w = i < PW ? p.w[i < PW ? i : 0] : 0u;
      atomicMax(reinterpret_cast<unsigned long long*>(d + i), (unsigned long long)(hi | w));
    }
  }

  // publish() with `gap_ns` between the words of a multi-word descriptor, so
  // that readers can meet it half written (descriptor perturbation knob).
  __device__ __forceinline__ static void publish_spaced(uint64_t* d, const C& v, uint32_t tag, uint32_t gap_ns) {
    words<C> p = to_words(v);
    const uint64_t hi = uint64_t(tag) << 32;
#pragma unroll
    for (int i = 0; i < W; ++i) {
      if (i > 0 && gap_ns) ptx::nanosleep(gap_ns);
      const uint32_t w = i < PW ? p.w[i < PW ? i : 0] : 0u;
      atomicMax(reinterpret_cast<unsigned long long*>(d + i), (unsigned long long)(hi | w));
    }
  }

  // True when the words of a loaded descriptor carry different tags and one
  // of them is of epoch tag `etag`: a descriptor caught between the atomic
  // updates of its words (decode() rejects it).
  __device__ __forceinline__ static bool torn(const uint64_t (&w)[W], uint32_t etag) {
    if constexpr (W == 1) {
      return false;
    } else {
      const uint32_t t0 = uint32_t(w[0] >> 32);
      bool differ = false, current = (t0 >> 2) == etag;
#pragma unroll
      for (int i = 1; i < W; ++i) {
        const uint32_t ti = uint32_t(w[i] >> 32);
        differ |= ti != t0;
        current |= (ti >> 2) == etag;
      }
      return differ && current;
    }
  }

  // Issues the loads of descriptor `d` (decode() consumes them later, so
  // several polls can be in flight).
  __device__ __forceinline__ static void load_raw(const uint64_t* d, uint64_t (&w)[W]) {
    if constexpr (W == 1) {
      w[0] = ptx::ld_relaxed(d);
    } else {
#pragma unroll
      for (int i = 0; i < W; i += 2) ptx::ld_relaxed_v2(d + i, w[i], w[i + 1]);
    }
  }

  // Returns the status of descriptor `d` in epoch tag `etag` (= epoch+1) and
  // its payload in `v`; kInvalid when not (fully) written in this epoch.
  __device__ __forceinline__ static uint32_t read(const uint64_t* d, uint32_t etag, C& v) {
    uint64_t w[W];
    load_raw(d, w);
    return decode(w, etag, v);
  }

  __device__ __forceinline__ static uint32_t decode(const uint64_t (&w)[W], uint32_t etag, C& v) {
    const uint32_t tag = uint32_t(w[0] >> 32);
    bool same = true;
#pragma unroll
    for (int i = 1; i < W; ++i) same &= uint32_t(w[i] >> 32) == tag;
    const uint32_t st = tag & 3u;
    if (!same || (tag >> 2) != etag || (st != kAggregate && st != kPrefix)) return kInvalid;
    words<C> p;
#pragma unroll
    for (int i = 0; i < PW; ++i) p.w[i] = uint32_t(w[i]);
    v = from_words<C>(p);
    return st;
  }
};

__device__ __forceinline__ uint32_t make_tag(uint32_t etag, uint32_t status) {
  return (etag << 2) | status;
}

// Records the first device error and raises the abort flag.
__device__ __forceinline__ void raise_error(WsHeader* h, uint32_t code, unsigned long long detail) {
  if (atomicCAS(&h->error, 0u, code) == 0u) h->error_detail = detail;
  atomicExch(&h->abort, 1u);
}

__device__ __forceinline__ bool aborted(WsHeader* h) {
  return ptx::ld_relaxed(reinterpret_cast<const uint32_t*>(&h->abort)) != 0u;
}

// A wait looks at the abort flag (a global load) only once it has lasted this
// long: the short waits of a healthy pipeline never leave shared memory, and
// a failure elsewhere still ends every wait within microseconds.
constexpr uint64_t kAbortCheckAfterNs = 20000;

// Bounded wait on an mbarrier phase. Returns false (after raising a timeout)
// when the phase has not completed within timeout_ns or another CTA aborted.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, WsHeader* h,
                                                  uint64_t timeout_ns, unsigned long long detail) {
  if (ptx::mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = ptx::globaltimer_ns();
  for (uint32_t it = 1;; ++it) {
    if (ptx::mbar_try_wait(bar, parity)) return true;
    if ((it & 15u) == 0u) {
      const uint64_t waited = ptx::globaltimer_ns() - t0;
      if (waited > kAbortCheckAfterNs && aborted(h)) return false;
      if (waited > timeout_ns) {
        raise_error(h, kDevTimeout, detail);
        return false;
      }
    }
  }
}

// Wait for this CTA's own bulk copy into a stage before the CTA exits. The
// abort flag does not end it (the copy must land before the shared memory is
// released); the time limit does, after recording a timeout.
__device__ __forceinline__ bool mbar_wait_drain(uint64_t* bar, uint32_t parity, WsHeader* h, uint64_t timeout_ns) {
  if (ptx::mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = ptx::globaltimer_ns();
  for (uint32_t it = 1;; ++it) {
    if (ptx::mbar_try_wait(bar, parity)) return true;
    if ((it & 15u) == 0u && ptx::globaltimer_ns() - t0 > timeout_ns) {
      raise_error(h, kDevTimeout, ~0ull);
      return false;
    }
  }
}

// Called by thread 0 of every CTA after the CTA's last access to the shared
// control words, with the workspace epoch the launch read when it started.
// The last CTA to exit re-arms the workspace for the next launch on the same
// stream: ticket and exit counters to zero, abort cleared, epoch advanced
// (clearing all descriptors when the epoch wraps). The fences around the exit
// count order every CTA's counter updates (window arrivals, abort) before the
// re-arm's stores; the re-arm itself loads nothing (the epoch is the one the
// launch started with, the descriptor high-water mark grows by a reduction),
// so the last CTA waits for one atomic and two fences only.
__device__ __forceinline__ void cta_exit_rearm(WsHeader* h, uint64_t* desc, uint64_t desc_words_used,
                                               uint32_t epoch) {
  __threadfence();
  const unsigned prev = atomicAdd(&h->done, 1u);
  if (prev != gridDim.x - 1) return;
  __threadfence();
  if (desc_words_used) atomicMax(&h->desc_words_hwm, (unsigned long long)desc_words_used);
  uint32_t next = epoch + 1;
  if (next >= kEpochLimit) {
    const unsigned long long hwm = *reinterpret_cast<volatile unsigned long long*>(&h->desc_words_hwm);
    for (unsigned long long i = 0; i < hwm; ++i) desc[i] = 0ull;
    next = 0;
  }
  h->epoch = next;
  h->ticket = 0ull;
  h->abort = 0u;
  h->bar_count = 0u;
  h->coop_arrive[0] = 0ull;
  h->coop_arrive[1] = 0ull;
  h->done = 0u;
}

}  // namespace pp
