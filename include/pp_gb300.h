/*
 * pp_gb300.h - C ABI of the GB300 (sm_103a) parallel primitives library
 * (libppgb300.so).
 *
 * Drop-in boundary for the scan / reduce path of SYCL-Building-Blocks. The
 * reference is a header-only C++ template library, so it has no C ABI of its
 * own; every entry point below names the reference template it replaces
 * (file:line within the reference project). The C++ template API with the
 * reference's own names lives in include/parallel_primitives/.
 *
 * Conventions
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default
 *     stream). Device-pointer calls are stream-ordered and asynchronous; the
 *     reference blocks on every call (.wait()), the *_host wrappers and
 *     pp_reduce_device keep that blocking behaviour.
 *   - The library never throws: every call returns a pp_status. Errors found
 *     on the device (a look-back or grid-barrier wait that gave up) are kept
 *     in the stream's workspace and returned by pp_stream_status().
 *   - Integer plus / multiplies wrap modulo 2^bits (signed types too).
 *   - in == out (in-place) is supported by every scan.
 */
#ifndef PP_GB300_H
#define PP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef void* pp_stream;

typedef enum pp_status {
  PP_OK = 0,
  PP_ERR_INVALID_ARG = 1,    /* bad enum, null pointer, misaligned workspace */
  PP_ERR_UNSUPPORTED = 2,    /* op/dtype/precision combination not provided */
  PP_ERR_GRID_TOO_LARGE = 3, /* cooperative grid larger than the device holds co-resident */
  PP_ERR_TIMEOUT = 4,        /* a device-side wait gave up (see pp_set_timeout_ns) */
  PP_ERR_CUDA = 5,           /* a CUDA runtime call failed */
  PP_ERR_WORKSPACE = 6,      /* workspace too small (or would need allocation during capture) */
  PP_ERR_NO_DEVICE = 7       /* no usable CUDA device */
} pp_status;

/* scan_type (internal/common.h:27-30) */
typedef enum pp_scan_kind { PP_SCAN_INCLUSIVE = 0, PP_SCAN_EXCLUSIVE = 1 } pp_scan_kind;

/* the sycl functors the reference scans/reduces with; identities as get_init
 * (internal/common.h:41-68) */
typedef enum pp_op {
  PP_OP_PLUS = 0,
  PP_OP_MULTIPLIES = 1,
  PP_OP_BIT_AND = 2, /* integer types only */
  PP_OP_BIT_OR = 3,  /* integer types only */
  PP_OP_BIT_XOR = 4, /* integer types only */
  PP_OP_MINIMUM = 5,
  PP_OP_MAXIMUM = 6
} pp_op;

typedef enum pp_dtype { PP_I32 = 0, PP_U32 = 1, PP_I64 = 2, PP_U64 = 3, PP_F32 = 4, PP_F64 = 5 } pp_dtype;

typedef enum pp_scan_algo {
  PP_ALGO_AUTO = 0,        /* decoupled look-back */
  PP_ALGO_DECOUPLED = 1,   /* scan_decoupled_lookback.hpp */
  PP_ALGO_COOPERATIVE = 2, /* scan_cooperative.hpp */
  PP_ALGO_SINGLE_GROUP = 3 /* one CTA walks every tile (scan.hpp:125-130) */
} pp_scan_algo;

typedef enum pp_precision {
  PP_PREC_DEFAULT = 0,     /* arithmetic in the element type */
  PP_PREC_COMPENSATED = 1, /* F32 plus only: float-float (TwoSum) accumulation everywhere */
  PP_PREC_FP64_CARRY = 2   /* F32 plus only: FP32 in-tile, FP64 cross-tile carry chain */
} pp_precision;

/* ---- general entry ------------------------------------------------------ */

/* Scan n elements of d_in into d_out. Replaces decoupled_scan_device
 * (scan_decoupled_lookback.hpp:209-217), cooperative_scan_device
 * (scan_cooperative.hpp:95-99) and scan_device / group_scan_device
 * (scan.hpp:107-130) depending on `algo`. */
pp_status pp_scan(pp_stream stream, pp_scan_kind kind, pp_op op, pp_dtype dtype, const void* d_in, void* d_out,
                  uint64_t n, pp_scan_algo algo, pp_precision precision);

/* Same with a caller-owned device workspace of at least pp_workspace_size()
 * bytes, 256-byte aligned and zero-filled once before its first use. One
 * workspace must not be used by calls that overlap on the GPU. */
pp_status pp_scan_ws(pp_stream stream, pp_scan_kind kind, pp_op op, pp_dtype dtype, const void* d_in, void* d_out,
                     uint64_t n, pp_scan_algo algo, pp_precision precision, void* d_workspace,
                     size_t workspace_bytes);

/* Workspace bytes pp_scan_ws / pp_reduce_ws need for these arguments (the
 * alignment of the data pointers picks the kernel, hence the pointers). */
pp_status pp_workspace_size(pp_scan_algo algo, pp_dtype dtype, pp_precision precision, const void* d_in,
                            const void* d_out, uint64_t n, size_t* bytes);

/* ---- reference-named device-pointer entries ------------------------------ */

/* decoupled_scan_device<type, func, T> (scan_decoupled_lookback.hpp:209-217) */
pp_status pp_decoupled_scan_device(pp_stream stream, pp_scan_kind kind, pp_op op, pp_dtype dtype,
                                   const void* d_in, void* d_out, uint64_t n);
/* cooperative_scan_device<type, func, T> (scan_cooperative.hpp:95-99) */
pp_status pp_cooperative_scan_device(pp_stream stream, pp_scan_kind kind, pp_op op, pp_dtype dtype,
                                     const void* d_in, void* d_out, uint64_t n);
/* scan_device<type, func, T> (scan.hpp:107-123) */
pp_status pp_scan_device(pp_stream stream, pp_scan_kind kind, pp_op op, pp_dtype dtype, const void* d_in,
                         void* d_out, uint64_t n);
/* group_scan_device<type, func, T> (scan.hpp:125-130) */
pp_status pp_group_scan_device(pp_stream stream, pp_scan_kind kind, pp_op op, pp_dtype dtype, const void* d_in,
                               void* d_out, uint64_t n);

/* reduce_device<func, T> (reduction.hpp:113-139): blocking, the result is
 * written to HOST memory `h_result` (one element of dtype), as the reference
 * returns it by value. */
pp_status pp_reduce_device(pp_stream stream, pp_op op, pp_dtype dtype, const void* d_in, uint64_t n,
                           void* h_result);

/* Asynchronous reduction: the result (one element) goes to DEVICE memory. */
pp_status pp_reduce(pp_stream stream, pp_op op, pp_dtype dtype, const void* d_in, uint64_t n, void* d_result);
pp_status pp_reduce_ws(pp_stream stream, pp_op op, pp_dtype dtype, const void* d_in, uint64_t n, void* d_result,
                       void* d_workspace, size_t workspace_bytes);

/* ---- reference-named host-pointer wrappers (blocking) ---------------------
 * Copy host input to the device, run, copy the result back
 * (scan_decoupled_lookback.hpp:219-230, scan.hpp:133-140,
 * scan_cooperative.hpp:102-110, reduction.hpp:142-151). The reference runs
 * small inputs on the host CPU instead; these always run on the GPU. */
pp_status pp_decoupled_scan_host(pp_scan_kind kind, pp_op op, pp_dtype dtype, const void* h_in, void* h_out,
                                 uint64_t n);
pp_status pp_cooperative_scan_host(pp_scan_kind kind, pp_op op, pp_dtype dtype, const void* h_in, void* h_out,
                                   uint64_t n);
pp_status pp_scan_host(pp_scan_kind kind, pp_op op, pp_dtype dtype, const void* h_in, void* h_out, uint64_t n);
pp_status pp_reduce_host(pp_op op, pp_dtype dtype, const void* h_in, uint64_t n, void* h_result);

/* ---- batched segmented scans and reductions ---------------------------------
 * No counterpart in the reference (it scans one array per call). Segments are
 * given in CSR form: d_offsets holds num_segments + 1 int64 entries,
 * offsets[0] = 0, offsets[num_segments] = n, nondecreasing; segment s is
 * elements [offsets[s], offsets[s+1]). All segments run in one persistent
 * scan launch (after a small head-flag pre-pass), so the call is
 * CUDA-graph-capturable once the stream's workspace has been sized by an
 * earlier call with the same or larger n. Operators: plus, minimum, maximum.
 * Data pointers must be 16-byte aligned (PP_ERR_INVALID_ARG otherwise). */
pp_status pp_segmented_scan(pp_stream stream, pp_scan_kind kind, pp_op op, pp_dtype dtype, const void* d_in,
                            void* d_out, uint64_t n, const int64_t* d_offsets, uint64_t num_segments);
/* d_out[s] = reduction of segment s (the operator's identity for an empty one). */
pp_status pp_segmented_reduce(pp_stream stream, pp_op op, pp_dtype dtype, const void* d_in, uint64_t n,
                              const int64_t* d_offsets, uint64_t num_segments, void* d_out);
/* Scan every row of a rows x cols row-major matrix independently (a batched
 * cumsum along the last dimension); reverse != 0 gives suffix scans
 * (out[r][c] = in[r][c] op ... op in[r][cols-1]), the adjoint of a prefix
 * sum. */
pp_status pp_rows_scan(pp_stream stream, pp_scan_kind kind, pp_op op, pp_dtype dtype, const void* d_in, void* d_out,
                       uint64_t rows, uint64_t cols, int reverse);

/* ---- status / settings ----------------------------------------------------- */

const char* pp_status_string(pp_status status);

/* Synchronises `stream` and returns (then clears) the first device-side
 * error recorded in the stream's cached workspace, else one recorded by
 * pp_decoupled_scan_device_noalloc on the current device, or PP_OK. */
pp_status pp_stream_status(pp_stream stream);
/* Same for a caller-owned workspace. */
pp_status pp_workspace_status(pp_stream stream, void* d_workspace);

/* Upper bound of every device-side wait (look-back, grid barrier, pipeline
 * barriers). Default 1 s. */
pp_status pp_set_timeout_ns(uint64_t ns);
/* Caps the number of CTAs of persistent launches (0 = occupancy x SMs). */
pp_status pp_set_max_ctas(int ctas);
/* Window of the cooperative scan's rounds, in tiles per CTA (0 = windows of
 * about 20 MB, the fastest on GB300; at most 4096). The input streams through
 * L2 one window at a time: a window is read from HBM by its reduce pass and
 * again, from L2, by its scan pass one window later. */
pp_status pp_set_cooperative_window(int tiles_per_cta);
/* Fault injection for tests: the tile with this index never publishes its
 * look-back descriptor, so its successors' waits time out; in the
 * cooperative scan the CTA whose run holds it never arrives at that window's
 * barrier (-1 = off). */
pp_status pp_debug_set_skip_tile(long long tile);
/* Descriptor-protocol perturbation for tests (no counterpart in the
 * reference, whose look-back correctness depends on timing,
 * partition_descriptor.h:115-130, scan_decoupled_lookback.hpp:143-174):
 * while max_delay_ns > 0 (at most 1,000,000), every tile of a decoupled scan
 * delays publishing its aggregate and its inclusive prefix by a pseudo-random
 * time in [0, max_delay_ns] drawn from (seed, tile), spaces the words of a
 * multi-word descriptor by up to max_delay_ns / 4, and counts look-back
 * outcomes (pp_debug_lookback_counters). Every wait stays bounded. 0 = off. */
pp_status pp_debug_set_lookback_delay(uint32_t max_delay_ns, uint32_t seed);
/* Synchronises `stream` and returns, then clears, the look-back counters of
 * its cached workspace gathered while the perturbation was on: [0] tiles
 * whose nearest predecessor held its inclusive prefix (reduce-then-scan),
 * [1] tiles that folded published aggregates back to an older prefix
 * (scan-then-reduce), [2] look-backs over more than 32 predecessors, [3]
 * polls that met a half-written multi-word descriptor. */
pp_status pp_debug_lookback_counters(pp_stream stream, uint64_t counters[4]);

/* Library version string. */
const char* pp_version(void);

/* ---- allocation-free variant ------------------------------------------------
 * No counterpart in the reference. The same decoupled look-back scan as
 * pp_decoupled_scan_device, for callers that must not allocate device memory
 * when they scan: latency-critical loops that must stay out of the allocator
 * (whose calls can synchronise the device), plug-ins whose host framework owns
 * all device memory through its own pool, processes whose device-memory budget
 * is spent. Its scratch is a fixed 1 MiB array in the library's device image
 * instead of a cudaMalloc'd or per-stream cached workspace, so it allocates
 * nothing. Limit: n up to 1,870,659,581 elements of a 4-byte integer type,
 * 2,104,492,029 floats, 511,508,479 elements of an 8-byte integer type or
 * 460,357,631 doubles; larger n returns PP_ERR_WORKSPACE. All calls share the
 * array: calls that overlap on the GPU race, so order them on one stream.
 * The first call on each device looks up the array's address (once, with
 * that device current); make that first call before any stream capture on
 * the device. A device-side
 * timeout of a call stays in the array until pp_stream_status() on the calls'
 * stream returns it. */
pp_status pp_decoupled_scan_device_noalloc(pp_stream stream, pp_scan_kind kind, pp_op op, pp_dtype dtype,
                                           const void* d_in, void* d_out, uint64_t n);

#ifdef __cplusplus
}
#endif

#endif /* PP_GB300_H */
