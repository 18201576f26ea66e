/*
 * oracle.h - CPU oracle for the scan / reduce path. TEST INFRASTRUCTURE ONLY:
 * used by tests/, by __graft_entry__.smoke() as the checker and by bench.py's
 * CPU-baseline leg. The product library never links or calls it.
 *
 * Three layers:
 *  1. exact sequential restatements of the reference's host_scan
 *     (include/parallel_primitives/scan_decoupled_lookback.hpp:185-207, the
 *     inclusive branch) and host_reduce (include/parallel_primitives/
 *     reduction.hpp:68-76); the exclusive scan is the mathematical one (the
 *     inclusive scan shifted right with the identity in front), not the
 *     reference's host exclusive branch, which is wrong (:196-203);
 *  2. FP64 oracles for float inputs;
 *  3. multi-threaded restatements of the reference's device algorithms run
 *     on CPU threads (one thread per work-group of one work-item): the
 *     decoupled look-back scan (scan_decoupled_lookback.hpp:106-182 with
 *     partition_descriptor.h:92-141), the cooperative scan
 *     (scan_cooperative.hpp:35-91) and the unrolled reduction
 *     (reduction.hpp:78-139). These are the timed CPU baseline.
 *
 * Operator numbering equals pp_op in include/pp_gb300.h, dtype numbering
 * equals pp_dtype.
 */
#ifndef PP_ORACLE_H
#define PP_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 1. exact sequential scan / reduce. Returns 0, or -1 for an unsupported
 * (dtype, op). Floats here accumulate in their own type, in sequence order. */
int oracle_scan(int dtype, int op, int exclusive, const void* in, void* out, uint64_t n);
int oracle_reduce(int dtype, int op, const void* in, uint64_t n, void* result);

/* 2. FP64 oracles: float inputs, double (f32) or compensated-double (f64)
 * accumulation, double outputs. */
int oracle_scan_fp64(int dtype, int exclusive, const void* in, double* out, uint64_t n);
double oracle_sum_fp64(int dtype, const void* in, uint64_t n);

/* Batched segments (CSR int64 offsets, offsets[0] = 0, offsets[S] = n,
 * nondecreasing): the exact scan / reduction above, and the FP64 oracles,
 * applied to each segment on its own; an empty segment reduces to the
 * operator's identity. -1 for an unsupported (dtype, op) or bad offsets. */
int oracle_segmented_scan(int dtype, int op, int exclusive, const void* in, void* out, uint64_t n,
                          const int64_t* offsets, uint64_t num_segments, int threads);
int oracle_segmented_scan_fp64(int dtype, int exclusive, const void* in, double* out, uint64_t n,
                               const int64_t* offsets, uint64_t num_segments, int threads);
int oracle_segmented_reduce(int dtype, int op, const void* in, uint64_t n, const int64_t* offsets,
                            uint64_t num_segments, void* out, int threads);
int oracle_segmented_sum_fp64(int dtype, const void* in, uint64_t n, const int64_t* offsets, uint64_t num_segments,
                              double* out, int threads);

/* 3. reference algorithms on `threads` CPU threads (0 = all cores).
 * local_mem_bytes sets the partition length as the reference derives it from
 * the device's local memory size (scan_decoupled_lookback.hpp:108-112).
 * force_lookback = 1 skips the is_ready() shortcut, so every partition takes
 * the scan-then-reduce path. */
int oracle_ref_decoupled_scan(int dtype, int op, int exclusive, const void* in, void* out, uint64_t n, int threads,
                              uint64_t local_mem_bytes, int force_lookback);
int oracle_ref_cooperative_scan(int dtype, int op, int exclusive, const void* in, void* out, uint64_t n,
                                int threads);
int oracle_ref_reduce(int dtype, int op, const void* in, uint64_t n, void* result, int threads);

/* Seeded, counter-based input generators (splitmix64 of seed + index), so
 * every consumer of an input sees identical bytes. `threads` 0 = all cores. */
void gen_u32_uniform(uint64_t seed, uint32_t* out, uint64_t n, uint32_t lo, uint64_t hi_exclusive, int threads);
void gen_u64_uniform(uint64_t seed, uint64_t* out, uint64_t n, uint64_t lo, uint64_t hi_exclusive, int threads);
void gen_f32_normal(uint64_t seed, float* out, uint64_t n, int threads);
void gen_f32_signed_lognormal(uint64_t seed, float* out, uint64_t n, double mu, double sigma, int threads);
uint64_t splitmix64(uint64_t x);

/* FNV-1a 64 of a byte range (fixture checksums). */
uint64_t oracle_fnv1a64(const void* data, uint64_t bytes);

int oracle_num_threads(void);

#ifdef __cplusplus
}
#endif

#endif
