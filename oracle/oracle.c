/*
 * oracle.c - CPU oracle for the scan / reduce path (TEST INFRASTRUCTURE ONLY;
 * see oracle.h). Plain C11 + pthreads, no architecture-specific code, so it
 * builds and gives the same results on x86-64 and aarch64.
 *
 * Parity status: the exact integer scans and reductions are pinned against
 * the reference's own code compiled on the CPU (oracle/_ref, see
 * build_oracle.py) and against the reference's known answers
 * (tests/test_reduction.cpp:4-31, benchmarks/benchmark_scan.cpp:39-49) in
 * tests/test_oracle.py.
 */
#define _GNU_SOURCE
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

int oracle_num_threads(void) {
  long n = sysconf(_SC_NPROCESSORS_ONLN);
  return n > 0 ? (int)n : 1;
}

static int resolve_threads(int t) { return t > 0 ? t : oracle_num_threads(); }

/* ------------------------------------------------------------------------ */
/* generic parallel-for over [0, n) in contiguous ranges                      */

typedef void (*range_fn)(void* ctx, uint64_t begin, uint64_t end);
typedef struct {
  range_fn fn;
  void* ctx;
  uint64_t begin, end;
} range_job;

static void* range_thread(void* p) {
  range_job* j = (range_job*)p;
  j->fn(j->ctx, j->begin, j->end);
  return NULL;
}

static void parallel_ranges(uint64_t n, int threads, range_fn fn, void* ctx) {
  threads = resolve_threads(threads);
  if (threads > 256) threads = 256;
  if ((uint64_t)threads > n / 4096 + 1) threads = (int)(n / 4096 + 1);
  if (threads <= 1) {
    fn(ctx, 0, n);
    return;
  }
  pthread_t tid[256];
  range_job jobs[256];
  for (int t = 0; t < threads; ++t) {
    jobs[t].fn = fn;
    jobs[t].ctx = ctx;
    jobs[t].begin = n * (uint64_t)t / (uint64_t)threads;
    jobs[t].end = n * (uint64_t)(t + 1) / (uint64_t)threads;
    pthread_create(&tid[t], NULL, range_thread, &jobs[t]);
  }
  for (int t = 0; t < threads; ++t) pthread_join(tid[t], NULL);
}

/* ------------------------------------------------------------------------ */
/* generators                                                                 */

#define GOLDEN 0x9E3779B97F4A7C15ull

static inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
/* element i of the splitmix64 stream that starts at `seed` */
static inline uint64_t stream_at(uint64_t seed, uint64_t i) { return mix64(seed + (i + 1) * GOLDEN); }
uint64_t splitmix64(uint64_t x) { return mix64(x + GOLDEN); }

typedef struct {
  uint64_t seed;
  void* out;
  uint64_t lo, range;
  double mu, sigma;
} gen_ctx;

static void gen_u32_range(void* p, uint64_t b, uint64_t e) {
  gen_ctx* c = (gen_ctx*)p;
  uint32_t* o = (uint32_t*)c->out;
  for (uint64_t i = b; i < e; ++i) {
    const uint64_t x = stream_at(c->seed, i);
    o[i] = (uint32_t)(c->lo + (((x >> 32) * c->range) >> 32));
  }
}
void gen_u32_uniform(uint64_t seed, uint32_t* out, uint64_t n, uint32_t lo, uint64_t hi_exclusive, int threads) {
  gen_ctx c = {seed, out, lo, hi_exclusive - lo, 0, 0};
  parallel_ranges(n, threads, gen_u32_range, &c);
}

static void gen_u64_range(void* p, uint64_t b, uint64_t e) {
  gen_ctx* c = (gen_ctx*)p;
  uint64_t* o = (uint64_t*)c->out;
  for (uint64_t i = b; i < e; ++i) {
    const uint64_t x = stream_at(c->seed, i);
    o[i] = c->lo + (uint64_t)(((unsigned __int128)x * c->range) >> 64);
  }
}
void gen_u64_uniform(uint64_t seed, uint64_t* out, uint64_t n, uint64_t lo, uint64_t hi_exclusive, int threads) {
  gen_ctx c = {seed, out, lo, hi_exclusive - lo, 0, 0};
  parallel_ranges(n, threads, gen_u64_range, &c);
}

/* Box-Muller on element pairs (2k, 2k+1) of the stream, in double. */
static inline void normal_pair(uint64_t seed, uint64_t k, double* z0, double* z1, uint64_t* x0, uint64_t* x1) {
  *x0 = stream_at(seed, 2 * k);
  *x1 = stream_at(seed, 2 * k + 1);
  const double u1 = ((double)((*x0 >> 11) + 1)) * 0x1.0p-53; /* (0, 1] */
  const double u2 = ((double)(*x1 >> 11)) * 0x1.0p-53;       /* [0, 1) */
  const double r = sqrt(-2.0 * log(u1));
  const double a = 6.283185307179586476925286766559 * u2;
  *z0 = r * cos(a);
  *z1 = r * sin(a);
}

static void gen_normal_range(void* p, uint64_t b, uint64_t e) {
  gen_ctx* c = (gen_ctx*)p;
  float* o = (float*)c->out;
  for (uint64_t i = b; i < e; ++i) {
    double z0, z1;
    uint64_t x0, x1;
    normal_pair(c->seed, i / 2, &z0, &z1, &x0, &x1);
    o[i] = (float)((i & 1) ? z1 : z0);
  }
}
void gen_f32_normal(uint64_t seed, float* out, uint64_t n, int threads) {
  gen_ctx c = {seed, out, 0, 0, 0, 0};
  parallel_ranges(n, threads, gen_normal_range, &c);
}

static void gen_lognormal_range(void* p, uint64_t b, uint64_t e) {
  gen_ctx* c = (gen_ctx*)p;
  float* o = (float*)c->out;
  for (uint64_t i = b; i < e; ++i) {
    double z0, z1;
    uint64_t x0, x1;
    normal_pair(c->seed, i / 2, &z0, &z1, &x0, &x1);
    const double z = (i & 1) ? z1 : z0;
    const uint64_t sbit = (i & 1) ? (x1 & 1u) : (x0 & 1u);
    const double m = exp(c->mu + c->sigma * z);
    o[i] = (float)(sbit ? -m : m);
  }
}
void gen_f32_signed_lognormal(uint64_t seed, float* out, uint64_t n, double mu, double sigma, int threads) {
  gen_ctx c = {seed, out, 0, 0, mu, sigma};
  parallel_ranges(n, threads, gen_lognormal_range, &c);
}

uint64_t oracle_fnv1a64(const void* data, uint64_t bytes) {
  const unsigned char* p = (const unsigned char*)data;
  uint64_t h = 0xcbf29ce484222325ull;
  for (uint64_t i = 0; i < bytes; ++i) {
    h ^= p[i];
    h *= 0x100000001b3ull;
  }
  return h;
}

/* ------------------------------------------------------------------------ */
/* per-(type, op) code, generated                                            */

enum { ST_AGGREGATE = 0, ST_PREFIX = 1, ST_INVALID = 2 }; /* partition_descriptor.h:10-14 */

typedef struct {
  const void* in;
  void* out;
  uint64_t n;
  int exclusive;
  int groups;
  uint64_t part_len;
  int force_lookback;
  void* desc;
  int group;
  pthread_barrier_t* bar_all;
  pthread_barrier_t* bar_rest;
  void* partial;
} ref_ctx;

/* get_group_work_size / get_cumulative_work_size (internal/common.h:74-86) */
static inline uint64_t group_work(uint64_t groups, uint64_t g, uint64_t n) {
  return n / groups + (g < n % groups ? 1 : 0);
}
static inline uint64_t cumulative_work(uint64_t groups, uint64_t g, uint64_t n) {
  const uint64_t rem = n % groups;
  return g * (n / groups) + (g < rem ? g : rem);
}

#define DEFINE_TYPE_OP(T, NAME, OPN, COMBINE, IDENT)                                                           \
  static inline T NAME##_##OPN##_op(T a, T b) { return COMBINE; }                                              \
  static void NAME##_##OPN##_seqscan(const T* in, T* out, uint64_t n, int excl) {                             \
    T acc = IDENT;                                                                                             \
    if (!excl) {                                                                                               \
      for (uint64_t i = 0; i < n; ++i) {                                                                       \
        acc = NAME##_##OPN##_op(acc, in[i]);                                                                   \
        out[i] = acc;                                                                                          \
      }                                                                                                        \
    } else {                                                                                                   \
      for (uint64_t i = 0; i < n; ++i) {                                                                       \
        const T x = in[i];                                                                                     \
        out[i] = acc;                                                                                          \
        acc = NAME##_##OPN##_op(acc, x);                                                                       \
      }                                                                                                        \
    }                                                                                                          \
  }                                                                                                            \
  static T NAME##_##OPN##_seqreduce(const T* in, uint64_t n) {                                                 \
    T acc = IDENT;                                                                                             \
    for (uint64_t i = 0; i < n; ++i) acc = NAME##_##OPN##_op(acc, in[i]);                                      \
    return acc;                                                                                                \
  }                                                                                                            \
  typedef struct {                                                                                             \
    T inclusive_prefix;                                                                                        \
    T aggregate;                                                                                               \
    _Atomic int status;                                                                                        \
  } NAME##_##OPN##_desc;                                                                                       \
  static void NAME##_##OPN##_desc_init(void* d, uint64_t parts) {                                              \
    NAME##_##OPN##_desc* q = (NAME##_##OPN##_desc*)d;                                                          \
    for (uint64_t p = 0; p < parts; ++p) {                                                                     \
      q[p].inclusive_prefix = IDENT;                                                                           \
      q[p].aggregate = IDENT;                                                                                  \
      atomic_init(&q[p].status, ST_INVALID);                                                                   \
    }                                                                                                          \
  }                                                                                                            \
  /* run_look_back (partition_descriptor.h:115-130) */                                                        \
  static T NAME##_##OPN##_lookback(NAME##_##OPN##_desc* d, uint64_t p) {                                       \
    T tmp = IDENT;                                                                                             \
    for (uint64_t q = p; q > 0;) {                                                                             \
      --q;                                                                                                     \
      int st;                                                                                                  \
      while ((st = atomic_load_explicit(&d[q].status, memory_order_acquire)) == ST_INVALID) {                 \
      }                                                                                                        \
      if (st == ST_PREFIX) return NAME##_##OPN##_op(tmp, d[q].inclusive_prefix);                              \
      tmp = NAME##_##OPN##_op(tmp, d[q].aggregate);                                                            \
    }                                                                                                          \
    return tmp;                                                                                                \
  }                                                                                                            \
  /* one work-group of the decoupled kernel (scan_decoupled_lookback.hpp:137-175) */                          \
  static void* NAME##_##OPN##_decoupled_group(void* arg) {                                                     \
    ref_ctx* c = (ref_ctx*)arg;                                                                                \
    const T* in = (const T*)c->in;                                                                             \
    T* out = (T*)c->out;                                                                                       \
    NAME##_##OPN##_desc* d = (NAME##_##OPN##_desc*)c->desc;                                                    \
    const uint64_t L = c->part_len;                                                                            \
    T* local = (T*)malloc(L * sizeof(T));                                                                      \
    for (uint64_t p = (uint64_t)c->group; p * L < c->n; p += (uint64_t)c->groups) {                           \
      const T* gin = in + p * L;                                                                               \
      T* gout = out + p * L;                                                                                   \
      const uint64_t len = (c->n - p * L) < L ? (c->n - p * L) : L;                                            \
      int ready = 0;                                                                                           \
      T prefix = IDENT;                                                                                        \
      if (p == 0) {                                                                                            \
        ready = 1;                                                                                             \
      } else if (!c->force_lookback &&                                                                         \
                 atomic_load_explicit(&d[p - 1].status, memory_order_acquire) == ST_PREFIX) {                  \
        ready = 1;                                                                                             \
        prefix = d[p - 1].inclusive_prefix;                                                                    \
      }                                                                                                        \
      if (ready) {                                                                                             \
        /* load_local_and_reduce, set_prefix, scan_over_group(init = prefix) */                               \
        T agg = IDENT;                                                                                         \
        for (uint64_t i = 0; i < len; ++i) {                                                                   \
          const T x = gin[i];                                                                                  \
          local[i] = x;                                                                                        \
          agg = NAME##_##OPN##_op(agg, x);                                                                     \
        }                                                                                                      \
        d[p].inclusive_prefix = NAME##_##OPN##_op(agg, prefix);                                                \
        atomic_store_explicit(&d[p].status, ST_PREFIX, memory_order_release);                                  \
        T acc = prefix;                                                                                        \
        if (!c->exclusive) {                                                                                   \
          for (uint64_t i = 0; i < len; ++i) {                                                                 \
            acc = NAME##_##OPN##_op(acc, local[i]);                                                            \
            gout[i] = acc;                                                                                     \
          }                                                                                                    \
        } else {                                                                                               \
          for (uint64_t i = 0; i < len; ++i) {                                                                 \
            gout[i] = acc;                                                                                     \
            acc = NAME##_##OPN##_op(acc, local[i]);                                                            \
          }                                                                                                    \
        }                                                                                                      \
      } else {                                                                                                 \
        /* scan_over_group(in -> local), aggregate = local[len - 1]: for an exclusive */                      \
        /* scan this omits the last element, as in the reference (:42, :163, :168) */                         \
        NAME##_##OPN##_seqscan(gin, local, len, c->exclusive);                                                 \
        const T agg = local[len - 1];                                                                          \
        d[p].aggregate = agg;                                                                                  \
        atomic_store_explicit(&d[p].status, ST_AGGREGATE, memory_order_release);                               \
        prefix = NAME##_##OPN##_lookback(d, p);                                                                \
        d[p].inclusive_prefix = NAME##_##OPN##_op(agg, prefix);                                                \
        atomic_store_explicit(&d[p].status, ST_PREFIX, memory_order_release);                                  \
        for (uint64_t i = 0; i < len; ++i) gout[i] = NAME##_##OPN##_op(local[i], prefix);                      \
      }                                                                                                        \
    }                                                                                                          \
    free(local);                                                                                               \
    return NULL;                                                                                               \
  }                                                                                                            \
  /* one work-group of the cooperative kernel (scan_cooperative.hpp:41-87) */                                 \
  static void* NAME##_##OPN##_coop_group(void* arg) {                                                          \
    ref_ctx* c = (ref_ctx*)arg;                                                                                \
    const T* in = (const T*)c->in;                                                                             \
    T* out = (T*)c->out;                                                                                       \
    const uint64_t G = (uint64_t)c->groups, g = (uint64_t)c->group, n = c->n;                                  \
    const uint64_t off = cumulative_work(G, g, n), len = group_work(G, g, n);                                 \
    NAME##_##OPN##_seqscan(in + off, out + off, len, c->exclusive);                                            \
    if (G == 1) return NULL;                                                                                   \
    pthread_barrier_wait(c->bar_all);                                                                          \
    T prev = IDENT;                                                                                            \
    for (uint64_t k = 1; k <= g; ++k) prev = NAME##_##OPN##_op(prev, out[cumulative_work(G, k, n) - 1]);      \
    if (g != 0) pthread_barrier_wait(c->bar_rest);                                                             \
    for (uint64_t i = 0; i < len; ++i) out[off + i] = NAME##_##OPN##_op(out[off + i], prev);                   \
    return NULL;                                                                                               \
  }                                                                                                            \
  /* one thread's share of the unrolled reduction kernels (reduction.hpp:42-60) */                            \
  static void* NAME##_##OPN##_reduce_part(void* arg) {                                                         \
    ref_ctx* c = (ref_ctx*)arg;                                                                                \
    const T* in = (const T*)c->in;                                                                             \
    T acc = IDENT;                                                                                             \
    const uint64_t b = c->n * (uint64_t)c->group / (uint64_t)c->groups;                                        \
    const uint64_t e = c->n * (uint64_t)(c->group + 1) / (uint64_t)c->groups;                                  \
    for (uint64_t i = b; i < e; ++i) acc = NAME##_##OPN##_op(acc, in[i]);                                      \
    *(T*)c->partial = acc;                                                                                     \
    return NULL;                                                                                               \
  }

/* integer operators: plus / multiplies wrap in the unsigned type */
#define DEFINE_INT_TYPE(T, UT, NAME, MAXV, MINV)                                                \
  DEFINE_TYPE_OP(T, NAME, plus, (T)((UT)a + (UT)b), (T)0)                                       \
  DEFINE_TYPE_OP(T, NAME, mul, (T)((UT)a * (UT)b), (T)1)                                        \
  DEFINE_TYPE_OP(T, NAME, and, (T)(a & b), (T)(~(UT)0))                                         \
  DEFINE_TYPE_OP(T, NAME, or, (T)(a | b), (T)0)                                                 \
  DEFINE_TYPE_OP(T, NAME, xor, (T)(a ^ b), (T)0)                                                \
  DEFINE_TYPE_OP(T, NAME, min, ((a < b) ? a : b), MAXV)                                         \
  DEFINE_TYPE_OP(T, NAME, max, ((a > b) ? a : b), MINV)

#define DEFINE_FLOAT_TYPE(T, NAME)                                   \
  DEFINE_TYPE_OP(T, NAME, plus, a + b, (T)0)                         \
  DEFINE_TYPE_OP(T, NAME, mul, a * b, (T)1)                          \
  DEFINE_TYPE_OP(T, NAME, min, ((a < b) ? a : b), (T)INFINITY)       \
  DEFINE_TYPE_OP(T, NAME, max, ((a > b) ? a : b), (T)(-INFINITY))

DEFINE_INT_TYPE(int32_t, uint32_t, i32, INT32_MAX, INT32_MIN)
DEFINE_INT_TYPE(uint32_t, uint32_t, u32, UINT32_MAX, 0u)
DEFINE_INT_TYPE(int64_t, uint64_t, i64, INT64_MAX, INT64_MIN)
DEFINE_INT_TYPE(uint64_t, uint64_t, u64, UINT64_MAX, 0ull)
DEFINE_FLOAT_TYPE(float, f32)
DEFINE_FLOAT_TYPE(double, f64)

typedef void (*seqscan_fn)(const void*, void*, uint64_t, int);
typedef struct {
  size_t size;
  size_t desc_size;
  seqscan_fn seqscan;
  void (*seqreduce)(const void*, uint64_t, void*);
  void* (*decoupled_group)(void*);
  void* (*coop_group)(void*);
  void* (*reduce_part)(void*);
  void (*combine)(const void*, const void*, void*);
  void (*identity)(void*);
  void (*desc_init)(void*, uint64_t);
} type_op_entry;

#define ENTRY_FNS(T, NAME, OPN, IDENT)                                                          \
  static void NAME##_##OPN##_seqscan_v(const void* i, void* o, uint64_t n, int e) {             \
    NAME##_##OPN##_seqscan((const T*)i, (T*)o, n, e);                                           \
  }                                                                                             \
  static void NAME##_##OPN##_seqreduce_v(const void* i, uint64_t n, void* r) {                  \
    *(T*)r = NAME##_##OPN##_seqreduce((const T*)i, n);                                          \
  }                                                                                             \
  static void NAME##_##OPN##_combine_v(const void* a, const void* b, void* r) {                 \
    *(T*)r = NAME##_##OPN##_op(*(const T*)a, *(const T*)b);                                     \
  }                                                                                             \
  static void NAME##_##OPN##_identity_v(void* r) { *(T*)r = IDENT; }

#define ENTRY(T, NAME, OPN)                                                                                 \
  {sizeof(T),                   sizeof(NAME##_##OPN##_desc), NAME##_##OPN##_seqscan_v,                     \
   NAME##_##OPN##_seqreduce_v,  NAME##_##OPN##_decoupled_group, NAME##_##OPN##_coop_group,                 \
   NAME##_##OPN##_reduce_part,  NAME##_##OPN##_combine_v,        NAME##_##OPN##_identity_v,                 \
   NAME##_##OPN##_desc_init}
#define NO_ENTRY {0, 0, NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL}

#define INT_ENTRY_FNS(T, UT, NAME, MAXV, MINV)  \
  ENTRY_FNS(T, NAME, plus, (T)0)                \
  ENTRY_FNS(T, NAME, mul, (T)1)                 \
  ENTRY_FNS(T, NAME, and, (T)(~(UT)0))          \
  ENTRY_FNS(T, NAME, or, (T)0)                  \
  ENTRY_FNS(T, NAME, xor, (T)0)                 \
  ENTRY_FNS(T, NAME, min, MAXV)                 \
  ENTRY_FNS(T, NAME, max, MINV)
#define FLOAT_ENTRY_FNS(T, NAME)                \
  ENTRY_FNS(T, NAME, plus, (T)0)                \
  ENTRY_FNS(T, NAME, mul, (T)1)                 \
  ENTRY_FNS(T, NAME, min, (T)INFINITY)          \
  ENTRY_FNS(T, NAME, max, (T)(-INFINITY))

INT_ENTRY_FNS(int32_t, uint32_t, i32, INT32_MAX, INT32_MIN)
INT_ENTRY_FNS(uint32_t, uint32_t, u32, UINT32_MAX, 0u)
INT_ENTRY_FNS(int64_t, uint64_t, i64, INT64_MAX, INT64_MIN)
INT_ENTRY_FNS(uint64_t, uint64_t, u64, UINT64_MAX, 0ull)
FLOAT_ENTRY_FNS(float, f32)
FLOAT_ENTRY_FNS(double, f64)

#define INT_ROW(T, NAME) \
  {ENTRY(T, NAME, plus), ENTRY(T, NAME, mul), ENTRY(T, NAME, and), ENTRY(T, NAME, or), ENTRY(T, NAME, xor), \
   ENTRY(T, NAME, min), ENTRY(T, NAME, max)}
#define FLOAT_ROW(T, NAME) \
  {ENTRY(T, NAME, plus), ENTRY(T, NAME, mul), NO_ENTRY, NO_ENTRY, NO_ENTRY, ENTRY(T, NAME, min), ENTRY(T, NAME, max)}

/* [dtype][op], dtype order of pp_dtype: i32, u32, i64, u64, f32, f64 */
static const type_op_entry TABLE[6][7] = {INT_ROW(int32_t, i32),  INT_ROW(uint32_t, u32), INT_ROW(int64_t, i64),
                                          INT_ROW(uint64_t, u64), FLOAT_ROW(float, f32),  FLOAT_ROW(double, f64)};

static const type_op_entry* lookup(int dtype, int op) {
  if (dtype < 0 || dtype > 5 || op < 0 || op > 6) return NULL;
  const type_op_entry* e = &TABLE[dtype][op];
  return e->size ? e : NULL;
}

/* ------------------------------------------------------------------------ */
/* 1. exact sequential                                                       */

int oracle_scan(int dtype, int op, int exclusive, const void* in, void* out, uint64_t n) {
  const type_op_entry* e = lookup(dtype, op);
  if (!e) return -1;
  e->seqscan(in, out, n, exclusive);
  return 0;
}

int oracle_reduce(int dtype, int op, const void* in, uint64_t n, void* result) {
  const type_op_entry* e = lookup(dtype, op);
  if (!e) return -1;
  e->seqreduce(in, n, result);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* 2. FP64 oracles                                                           */

int oracle_scan_fp64(int dtype, int exclusive, const void* in, double* out, uint64_t n) {
  if (dtype == 4) {
    const float* x = (const float*)in;
    double acc = 0.0;
    for (uint64_t i = 0; i < n; ++i) {
      if (exclusive) {
        out[i] = acc;
        acc += (double)x[i];
      } else {
        acc += (double)x[i];
        out[i] = acc;
      }
    }
    return 0;
  }
  if (dtype == 5) { /* Neumaier-compensated double */
    const double* x = (const double*)in;
    double s = 0.0, c = 0.0;
    for (uint64_t i = 0; i < n; ++i) {
      if (exclusive) out[i] = s + c;
      const double t = s + x[i];
      if (fabs(s) >= fabs(x[i]))
        c += (s - t) + x[i];
      else
        c += (x[i] - t) + s;
      s = t;
      if (!exclusive) out[i] = s + c;
    }
    return 0;
  }
  return -1;
}

double oracle_sum_fp64(int dtype, const void* in, uint64_t n) {
  double s = 0.0, c = 0.0;
  for (uint64_t i = 0; i < n; ++i) {
    const double x = dtype == 4 ? (double)((const float*)in)[i] : ((const double*)in)[i];
    const double t = s + x;
    if (fabs(s) >= fabs(x))
      c += (s - t) + x;
    else
      c += (x - t) + s;
    s = t;
  }
  return s + c;
}

/* ------------------------------------------------------------------------ */
/* 1b/2b. batched segments: the definitions above applied to every segment   */
/* [offsets[s], offsets[s+1]) in turn (segments split over threads).          */

typedef struct {
  const type_op_entry* e;
  int dtype, exclusive, fp64;
  const unsigned char* in;
  unsigned char* out;
  const int64_t* off;
} seg_ctx;

static void seg_scan_range(void* p, uint64_t b, uint64_t e) {
  seg_ctx* c = (seg_ctx*)p;
  for (uint64_t k = b; k < e; ++k) {
    const uint64_t a = (uint64_t)c->off[k], len = (uint64_t)(c->off[k + 1] - c->off[k]);
    if (len == 0) continue;
    if (c->fp64) {
      const size_t es = c->dtype == 4 ? 4 : 8;
      oracle_scan_fp64(c->dtype, c->exclusive, c->in + a * es, (double*)c->out + a, len);
    } else {
      c->e->seqscan(c->in + a * c->e->size, c->out + a * c->e->size, len, c->exclusive);
    }
  }
}

static int offsets_ok(const int64_t* off, uint64_t n, uint64_t num_segments) {
  if (off[0] != 0 || (uint64_t)off[num_segments] != n) return 0;
  for (uint64_t k = 0; k < num_segments; ++k)
    if (off[k + 1] < off[k]) return 0;
  return 1;
}

int oracle_segmented_scan(int dtype, int op, int exclusive, const void* in, void* out, uint64_t n,
                          const int64_t* offsets, uint64_t num_segments, int threads) {
  const type_op_entry* e = lookup(dtype, op);
  if (!e || !offsets_ok(offsets, n, num_segments)) return -1;
  seg_ctx c = {e, dtype, exclusive, 0, (const unsigned char*)in, (unsigned char*)out, offsets};
  parallel_ranges(num_segments, threads, seg_scan_range, &c);
  return 0;
}

int oracle_segmented_scan_fp64(int dtype, int exclusive, const void* in, double* out, uint64_t n,
                               const int64_t* offsets, uint64_t num_segments, int threads) {
  if ((dtype != 4 && dtype != 5) || !offsets_ok(offsets, n, num_segments)) return -1;
  seg_ctx c = {NULL, dtype, exclusive, 1, (const unsigned char*)in, (unsigned char*)out, offsets};
  parallel_ranges(num_segments, threads, seg_scan_range, &c);
  return 0;
}

static void seg_reduce_range(void* p, uint64_t b, uint64_t e) {
  seg_ctx* c = (seg_ctx*)p;
  for (uint64_t k = b; k < e; ++k) {
    const uint64_t a = (uint64_t)c->off[k], len = (uint64_t)(c->off[k + 1] - c->off[k]);
    if (c->fp64)
      ((double*)c->out)[k] = oracle_sum_fp64(c->dtype, c->in + a * (c->dtype == 4 ? 4 : 8), len);
    else /* an empty segment reduces to the identity */
      c->e->seqreduce(c->in + a * c->e->size, len, c->out + k * c->e->size);
  }
}

int oracle_segmented_reduce(int dtype, int op, const void* in, uint64_t n, const int64_t* offsets,
                            uint64_t num_segments, void* out, int threads) {
  const type_op_entry* e = lookup(dtype, op);
  if (!e || !offsets_ok(offsets, n, num_segments)) return -1;
  seg_ctx c = {e, dtype, 0, 0, (const unsigned char*)in, (unsigned char*)out, offsets};
  parallel_ranges(num_segments, threads, seg_reduce_range, &c);
  return 0;
}

int oracle_segmented_sum_fp64(int dtype, const void* in, uint64_t n, const int64_t* offsets, uint64_t num_segments,
                              double* out, int threads) {
  if ((dtype != 4 && dtype != 5) || !offsets_ok(offsets, n, num_segments)) return -1;
  seg_ctx c = {NULL, dtype, 0, 1, (const unsigned char*)in, (unsigned char*)out, offsets};
  parallel_ranges(num_segments, threads, seg_reduce_range, &c);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* 3. reference algorithms on CPU threads                                    */

int oracle_ref_decoupled_scan(int dtype, int op, int exclusive, const void* in, void* out, uint64_t n, int threads,
                              uint64_t local_mem_bytes, int force_lookback) {
  const type_op_entry* e = lookup(dtype, op);
  if (!e) return -1;
  if (n == 0) return 0;
  const int G = resolve_threads(threads);
  /* partition length: local memory in elements minus the group size (1),
   * rounded down to a multiple of the group size (:108-112) */
  if (local_mem_bytes == 0) local_mem_bytes = 65536;
  const uint64_t L = local_mem_bytes / e->size - 1;
  if (L == 0) return -1;
  const uint64_t parts = (n + L - 1) / L;
  unsigned char* desc = (unsigned char*)malloc(parts * e->desc_size);
  if (!desc) return -1;
  /* fill: every descriptor invalid (:115-116) */
  e->desc_init(desc, parts);
  pthread_t* tid = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)G);
  ref_ctx* ctx = (ref_ctx*)malloc(sizeof(ref_ctx) * (size_t)G);
  for (int g = 0; g < G; ++g) {
    ref_ctx c = {in, out, n, exclusive, G, L, force_lookback, desc, g, NULL, NULL, NULL};
    ctx[g] = c;
    pthread_create(&tid[g], NULL, e->decoupled_group, &ctx[g]);
  }
  for (int g = 0; g < G; ++g) pthread_join(tid[g], NULL);
  free(ctx);
  free(tid);
  free(desc);
  return 0;
}

int oracle_ref_cooperative_scan(int dtype, int op, int exclusive, const void* in, void* out, uint64_t n,
                                int threads) {
  const type_op_entry* e = lookup(dtype, op);
  if (!e) return -1;
  if (n == 0) return 0;
  int G = resolve_threads(threads);
  if (G > 64) G = 64; /* nd_range_barrier's 64-group mask (cooperative_groups.hpp:66-68) */
  pthread_barrier_t bar_all, bar_rest;
  pthread_barrier_init(&bar_all, NULL, (unsigned)G);
  if (G > 1) pthread_barrier_init(&bar_rest, NULL, (unsigned)(G - 1));
  pthread_t* tid = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)G);
  ref_ctx* ctx = (ref_ctx*)malloc(sizeof(ref_ctx) * (size_t)G);
  for (int g = 0; g < G; ++g) {
    ref_ctx c = {in, out, n, exclusive, G, 0, 0, NULL, g, &bar_all, &bar_rest, NULL};
    ctx[g] = c;
    pthread_create(&tid[g], NULL, e->coop_group, &ctx[g]);
  }
  for (int g = 0; g < G; ++g) pthread_join(tid[g], NULL);
  pthread_barrier_destroy(&bar_all);
  if (G > 1) pthread_barrier_destroy(&bar_rest);
  free(ctx);
  free(tid);
  return 0;
}

/* reduce_device (reduction.hpp:113-139) with a work-group size of one: the
 * input is cut into INT32_MAX chunks; in each chunk the 64-wide level covers
 * the first floor(len/64)*64 elements, then the remainder recurses through the
 * 4-wide and 1-wide levels. Work-items are spread over the threads; each
 * thread combines its items into a partial, and the partials are combined in
 * thread order (the role of sycl::reduction). */
int oracle_ref_reduce(int dtype, int op, const void* in, uint64_t n, void* result, int threads) {
  const type_op_entry* e = lookup(dtype, op);
  if (!e) return -1;
  const int T = resolve_threads(threads);
  unsigned char acc[16], tmp[16];
  e->identity(acc);
  const unsigned char* base = (const unsigned char*)in;
  const uint64_t chunk_max = (uint64_t)INT32_MAX;
  unsigned char* partials = (unsigned char*)malloc((size_t)T * 16);
  pthread_t* tid = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)T);
  ref_ctx* ctx = (ref_ctx*)malloc(sizeof(ref_ctx) * (size_t)T);
  for (uint64_t done = 0; done < n;) {
    const uint64_t len = (n - done) < chunk_max ? (n - done) : chunk_max;
    const unsigned char* p = base + done * e->size;
    uint64_t processed = 0;
    const int levels[3] = {64, 4, 1};
    for (int l = 0; l < 3 && processed < len; ++l) {
      const uint64_t N = (uint64_t)levels[l];
      const uint64_t items = (len - processed) / N;
      if (items == 0) continue;
      const uint64_t cover = items * N;
      const int t_used = (uint64_t)T < items ? T : (int)items;
      for (int t = 0; t < t_used; ++t) {
        /* thread t takes a contiguous run of whole work-items */
        const uint64_t ib = items * (uint64_t)t / (uint64_t)t_used, ie = items * (uint64_t)(t + 1) / (uint64_t)t_used;
        ref_ctx c = {p + (processed + ib * N) * e->size, NULL, (ie - ib) * N, 0, 1, 0, 0, NULL, 0, NULL, NULL,
                     partials + (size_t)t * 16};
        ctx[t] = c;
        pthread_create(&tid[t], NULL, e->reduce_part, &ctx[t]);
      }
      for (int t = 0; t < t_used; ++t) pthread_join(tid[t], NULL);
      for (int t = 0; t < t_used; ++t) {
        e->combine(acc, partials + (size_t)t * 16, tmp);
        memcpy(acc, tmp, e->size);
      }
      processed += cover;
    }
    done += len;
  }
  free(ctx);
  free(tid);
  free(partials);
  memcpy(result, acc, e->size);
  return 0;
}
