/*
 * ej.h - C ABI of the eating_one_gb300 relational join engine (one GB300, sm_103a).
 *
 * The reference (yabuta/eating_one) has no library: each join is a standalone
 * executable whose host `join()` driver allocates device memory, launches
 * kernels loaded by name from cubins and frees everything again.  This header
 * is the boundary that replaces those drivers: plain C, plain pointers and
 * sizes, no C++ or torch types.
 *
 * Data layout (bit-identical to the reference structs):
 *   ej_tuple  == TUPLE  {int key; int val;}          joins/hashJoin_gpu/main_street/tuple.h:43-46
 *   ej_result == RESULT {int rkey, rval, lkey, lval;} joins/hashJoin_gpu/main_street/tuple.h:48-53
 * The join attribute is .val; .key is carried through as a row id.
 * R is the right/build relation (the reference's `rt`, argv[2]) and S is the
 * left/probe relation (`lt`, argv[1]); every result row holds the R tuple in
 * (rkey, rval) and the S tuple in (lkey, lval), as join_gpu.cu:104-107 writes.
 *
 * Memory: every relation and output pointer is a DEVICE pointer owned by the
 * caller, except where a function name ends in _host.  Scratch comes from the
 * handle's arena; nothing the caller passes is freed or replaced (the
 * reference's presum() frees its input, scan_main.cpp:106-108).
 *
 * Output capacity: each join writes min(count, out_cap) rows.  When the join
 * has more than out_cap results it returns EJ_ERR_CAPACITY and still stores
 * the full count in *out_count, so the caller can size a buffer and call again
 * (the count pass of the reference's count -> scan -> join sequence,
 * hj.cc:997-1069, is exposed separately as the *_count functions).
 *
 * Threading: one handle per host thread; a handle is not thread-safe.  All
 * device work is issued on the handle's stream (ej_set_stream).  Functions
 * that return a count to the host synchronise that stream before returning.
 * Errors are status codes; the library never exits, prints or traps.  Device
 * waits are bounded and report EJ_ERR_TIMEOUT through a device status word.
 */
#ifndef EJ_H
#define EJ_H

#include <stddef.h>
#include <stdint.h>
#include "ej_gen.h"

#ifdef __cplusplus
extern "C" {
#endif

#define EJ_ABI_VERSION 1
#define EJ_NULL_KEY INT32_MIN /* NULL sentinel of the left outer join */

typedef struct ej_tuple { int32_t key; int32_t val; } ej_tuple;
typedef struct ej_result { int32_t rkey; int32_t rval; int32_t lkey; int32_t lval; } ej_result;
/* one row of the 3-way star join: the two binary result rows of one fact row */
typedef struct ej_star_result { ej_result d1; ej_result d2; } ej_star_result;

/* points and result rows of the distance joins, laid out as the reference's:
 * the 2-D GPU join's TUPLE and JOIN_TUPLE (joins/blockJoin_gpu/complex_block/
 * dire_join/tuple.h:20-30, 24 and 48 bytes) and the 3-D CPU join's
 * (joins/CPU_JOIN/3d_cpu/nestLoopJoin.cc:23-33, 32 and 56 bytes) */
typedef struct ej_point2 { int32_t id; double val[2]; } ej_point2;
typedef struct ej_point3 { int32_t id; double val[3]; } ej_point3;
typedef struct ej_point_result2 { int32_t lid; double lval[2]; int32_t rid; double rval[2]; } ej_point_result2;
typedef struct ej_point_result3 { double lval[3]; double rval[3]; int32_t lid; int32_t rid; } ej_point_result3;

typedef enum ej_status {
  EJ_OK = 0,
  EJ_ERR_INVALID = 1,   /* bad argument (null pointer, size out of range) */
  EJ_ERR_CAPACITY = 2,  /* more results than out_cap; *out_count holds the total */
  EJ_ERR_CUDA = 3,      /* a CUDA runtime call failed; see ej_last_error */
  EJ_ERR_NOMEM = 4,     /* device or host allocation failed */
  EJ_ERR_TIMEOUT = 5,   /* a bounded device wait gave up */
  EJ_ERR_TOO_LARGE = 6, /* input beyond a documented size limit */
  EJ_ERR_NO_DEVICE = 7, /* no CUDA device or not an sm_103 device */
  EJ_ERR_BUSY = 8,      /* serving queue full or admission refused */
  EJ_ERR_INTERNAL = 9,  /* device-side consistency check failed */
  EJ_ERR_IO = 10        /* a table file could not be opened, read or written */
} ej_status;

typedef struct ej_handle ej_handle;
typedef struct ej_index ej_index;
typedef void* ej_stream; /* a cudaStream_t; NULL = the legacy default stream */

/* join algorithms of ej_join (mirrors the reference executables) */
typedef enum ej_algo {
  EJ_ALGO_HASH = 0,        /* radix-partitioned hash join   (joins/hashJoin_gpu/main_street) */
  EJ_ALGO_SINGLE_HASH = 1, /* build-side-only hash join     (joins/single-hashjoin/main_street) */
  EJ_ALGO_BNL = 2,         /* block nested-loop join        (joins/blockJoin_gpu/main_street) */
  EJ_ALGO_HASH_INDEX = 3,  /* hash-index inner join         (joins/innerJoin_gpu/main_street) */
  EJ_ALGO_SORT_INDEX = 4,  /* sort-index inner join         (joins/innerJoin_gpu/sort_index/main_street) */
  EJ_ALGO_LEFT_OUTER = 5   /* left outer join, NULL = INT32_MIN (joins/outerJoin_gpu, see ej_left_outer_join) */
} ej_algo;

/* ---- handle ------------------------------------------------------------- */

/* Create a handle on `device` (replaces cuInit/cuCtxCreate/cuModuleLoad,
 * joins/hashJoin_gpu/main_street/hj.cc:213-289). */
ej_status ej_create(int device, ej_handle** out);
ej_status ej_destroy(ej_handle* h);
ej_status ej_set_stream(ej_handle* h, ej_stream stream);
const char* ej_status_name(ej_status s);
/* last error text of this handle ("" when none) */
const char* ej_last_error(const ej_handle* h);
/* bytes of device scratch the handle holds (arena high-water mark) */
uint64_t ej_scratch_bytes(const ej_handle* h);
/* release the handle's cached scratch (the next call re-allocates) and the
 * memory of the device's index pool that no live index holds */
ej_status ej_trim(ej_handle* h);
/* Phase timers, like the reference's (hj.cc:1194-1237) but measured on the
 * device with CUDA events when timing is enabled.  Phases of one join, in
 * milliseconds: [0] build (R table / index), [1] partition (S radix pass),
 * [2] count + scan, [3] write.  Joins run while timing is on record into a
 * ring of EJ_PHASE_RING event sets; ej_phase_totals synchronises, sums every
 * set recorded since the previous call and clears the ring. */
#define EJ_PHASES 4
#define EJ_PHASE_RING 512
ej_status ej_set_timing(ej_handle* h, int enable);
ej_status ej_last_phase_ms(ej_handle* h, float ms[EJ_PHASES]);
ej_status ej_phase_totals(ej_handle* h, double ms[EJ_PHASES], uint32_t* joins);
/* number of CUDA kernels this handle has launched (all entry points) */
uint64_t ej_kernel_launches(const ej_handle* h);

/* Tuning knobs (the reference's compile-time #defines, e.g. PARTITION/RADIX/
 * PART_STANDARD in joins/hashJoin_gpu/main_street/tuple.h:1-16, become runtime
 * options). */
typedef enum ej_option {
  EJ_OPT_PROBE_PARTITION_BITS = 0, /* radix bits of the one S partition pass, 0..8 (0 = probe
                                      in place); -1 (default) lets the planner choose */
  EJ_OPT_BUCKET_BITS_DELTA = 1,    /* hash-table buckets = 2^(ceil(log2|R|) - 2 + delta),
                                      delta in -3..3; when neither this option nor the tuning
                                      table sets it: 0 for single tables, 1 for the tables of
                                      a batch */
  EJ_OPT_WAIT_LIMIT_NS = 2,        /* bound of every device-side wait of this handle's kernels
                                      (look-back scans, the nested loop's copy waits), in ns,
                                      0..10^10; -1 restores the default of 10^9 (1 s).  A wait
                                      that runs out makes the call return EJ_ERR_TIMEOUT (its
                                      results are then not valid); the handle stays usable.
                                      0 gives up at the first poll that finds a wait unmet, which
                                      lets tests drive the timeout path without a hung kernel */
  EJ_OPT_COUNT_REUSE = 3,          /* 1 (default): ej_hash_join_count keeps its table, partitioned
                                      S and run descriptors for an ej_hash_join that follows on the
                                      same relations; 0: the count keeps nothing (and writes no
                                      run descriptors) */
  EJ_OPT_BUILD = 4,                /* radix passes of a hash table's build: EJ_BUILD_* (0: planner) */
  EJ_OPT_TABLE = 5,                /* how probes find a hash table's runs: EJ_TABLE_FORMAT_* (0: planner) */
  EJ_OPT_PROBE_WARPS = 6           /* block shape of the probe kernels: 4 or 8 warps of 32
                                      threads per block (0: planner, 8) */
} ej_option;

/* Values of EJ_OPT_BUILD and ej_tune_entry.build.  The planner takes MSD for
 * hash tables of 2^20 rows and more, else LSD; sorted indexes sort by LSD
 * passes (their key is the value, whose top bits need not spread, so MSD does
 * not apply to them; EJ_BUILD_ONESWEEP applies to both kinds). */
enum {
  EJ_BUILD_PLANNER = 0,
  EJ_BUILD_LSD = 1,      /* four stable 8-bit passes from the least significant digit,
                            each a histogram, a scan and a scatter launch */
  EJ_BUILD_MSD = 2,      /* two unordered 8-bit passes from the most significant digit,
                            then a shared-memory sort of every 16-bit bucket (hash tables) */
  EJ_BUILD_ONESWEEP = 3  /* four stable 8-bit LSD passes, one scatter launch each, after one
                            histogram pass for all four digits (tiles learn their offsets
                            by decoupled look-back) */
};
/* Values of EJ_OPT_TABLE and ej_tune_entry.table.  The planner gives tables
 * of 2^22 rows and more a key directory when their runs average two rows or
 * more (tables of 2^20 rows and more when probed by 16 rows per table row or
 * more), the others bucket bounds. */
enum {
  EJ_TABLE_FORMAT_PLANNER = 0,
  EJ_TABLE_FORMAT_BUCKETS = 1,  /* bucket bounds: one 8-byte load, then a scan of the bucket */
  EJ_TABLE_FORMAT_DIRECTORY = 2 /* key directory: one entry per distinct key, found by linear probing */
};
ej_status ej_set_option(ej_handle* h, ej_option opt, int64_t value);

/* A tuning table (written by the autotuner, eating_one_gb300/autotune.py):
 * for joins whose build side has at least 2^log2_rows rows (the entry with the
 * largest such log2_rows applies), the S partition bits (-1: planner), the
 * bucket-bits delta (the table's load factor), the build's radix passes
 * (EJ_BUILD_*), the table format (EJ_TABLE_FORMAT_*) and the probe block shape
 * (warps per block); 0 in the last three leaves the choice to the planner.
 * Options set with ej_set_option take precedence.  n = 0 clears the table.
 * The reference's counterpart is its commented per-size #define sets
 * (joins/hashJoin_gpu/main_street/tuple.h:19-36,
 * joins/innerJoin_gpu/main_street/tuple.h:9-34). */
typedef struct ej_tune_entry {
  uint32_t log2_rows;
  int32_t partition_bits;
  int32_t bucket_delta;
  int32_t build;        /* EJ_BUILD_* */
  int32_t table;        /* EJ_TABLE_FORMAT_* */
  int32_t probe_warps;  /* 0, 4 or 8 */
  int32_t reserved[2];  /* 0 */
} ej_tune_entry;
ej_status ej_set_tuning(ej_handle* h, const ej_tune_entry* entries, uint32_t n);

/* ---- equi-joins on device relations ------------------------------------- */

/* Radix-partitioned hash join (replaces join() of joins/hashJoin_gpu/main_street/hj.cc:171-1269:
 * lcount_partitioning/rcount_partitioning + presum + lpartitioning/rpartitioning,
 * partitioning.cu:15-271, countPartition :273-293, count/join join_gpu.cu:9-113). */
ej_status ej_hash_join(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S, uint64_t nS,
                       ej_result* out, uint64_t out_cap, uint64_t* out_count);
/* Count pass only (join_gpu.cu:9-66 + presum + getValue, hj.cc:997-1048).
 * The reference sizes its output this way and then joins (hj.cc:997-1115);
 * to make that sequence one build, the count keeps its R table, its
 * partitioned copy of S and every probe's run descriptor in the handle, and
 * an ej_hash_join (or ej_hash_join_async) that follows it on the same handle
 * with the same R, nR, S and nS only writes the rows from them.  R and S must
 * not change in between.  Any other call that uses the handle's scratch drops
 * what the count kept (the join then runs whole); a write cut short by
 * out_cap keeps it for the retry.  EJ_OPT_COUNT_REUSE = 0 turns this off. */
ej_status ej_hash_join_count(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S,
                             uint64_t nS, uint64_t* out_count);
/* Asynchronous form: no host synchronisation; the total count is written to
 * the device word *d_count and rows beyond out_cap are dropped (the device
 * status word records EJ_ERR_CAPACITY; read it with ej_sync_status). */
ej_status ej_hash_join_async(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S,
                             uint64_t nS, ej_result* out, uint64_t out_cap, uint64_t* d_count);
/* synchronise the handle's stream and return (then clear) the device status */
ej_status ej_sync_status(ej_handle* h);

/* Build-side-only hash join: hash table on R, S probed in input order without
 * partitioning (replaces joins/single-hashjoin/main_street/singlehash.cc,
 * partitioning.cu:16-175, join_gpu.cu:10-44). */
ej_status ej_single_hash_join(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S,
                              uint64_t nS, ej_result* out, uint64_t out_cap, uint64_t* out_count);

/* Block nested-loop equi-join over all |R|x|S| pairs (replaces
 * joins/blockJoin_gpu/main_street/nestLoopJoin.cc:180-519 and the eval/count/join
 * kernels of join_gpu.cu:12-120).  Result rows use ej_result, not the
 * reference's 20-byte JOIN_TUPLE (tuple.h:29-35). */
ej_status ej_bnl_join(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S, uint64_t nS,
                      ej_result* out, uint64_t out_cap, uint64_t* out_count);
ej_status ej_bnl_join_count(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S,
                            uint64_t nS, uint64_t* out_count);

/* Distance nested-loop join over all |R|x|S| point pairs: S point l (left)
 * and R point r (right) match when sum_i (r.val[i] - l.val[i])^2 < radius^2,
 * evaluated in IEEE double in the reference's order (eval of
 * joins/blockJoin_gpu/complex_block/dire_join/join_gpu.cu:12-26 with its
 * count/join kernels :30-130, and of joins/CPU_JOIN/3d_cpu/nestLoopJoin.cc:73-101;
 * radius = DISTANCE = 1 there).  dims is 2 (R, S are ej_point2, out is
 * ej_point_result2) or 3 (ej_point3, ej_point_result3); arrays are device
 * memory, 8-byte aligned.  Rows come in no particular order. */
ej_status ej_distance_join(ej_handle* h, uint32_t dims, const void* R, uint64_t nR, const void* S, uint64_t nS,
                           double radius, void* out, uint64_t out_cap, uint64_t* out_count);
ej_status ej_distance_join_count(ej_handle* h, uint32_t dims, const void* R, uint64_t nR, const void* S,
                                 uint64_t nS, double radius, uint64_t* out_count);

/* ---- index joins ---------------------------------------------------------- */

/* Index on R's join attribute, built on the device and kept resident until
 * ej_index_free.  The reference builds both indexes on the CPU and uploads them:
 * hash index joins/innerJoin_gpu/main_street/inner-idx-bnlj.cc:148-181 (createIndex),
 * sort index joins/innerJoin_gpu/sort_index/main_street/inner-idx-bnlj.cc:175-217
 * (qsort + createIndex).  R must stay valid while the index is used.  An
 * index's storage comes from a stream-ordered memory pool of its device that
 * keeps freed index memory for the next index (ej_trim gives it back). */
ej_status ej_hash_index_build(ej_handle* h, const ej_tuple* R, uint64_t nR, ej_index** out);
ej_status ej_sort_index_build(ej_handle* h, const ej_tuple* R, uint64_t nR, ej_index** out);
ej_status ej_index_free(ej_handle* h, ej_index* idx);
/* Probe an index with S: inner join (hash index: count.cu:16-48, join_gpu.cu:8-86;
 * sort index: search/count/join, sort_index/main_street/join_gpu.cu:10-113). */
ej_status ej_index_join(ej_handle* h, const ej_index* idx, const ej_tuple* S, uint64_t nS,
                        ej_result* out, uint64_t out_cap, uint64_t* out_count);
ej_status ej_index_join_count(ej_handle* h, const ej_index* idx, const ej_tuple* S, uint64_t nS,
                              uint64_t* out_count);
/* Merge join of a sort index with S in value order: S's rows, 128 at a time,
 * take the window of the index between the first row at or above their first
 * value and the first row above their last, and find their runs inside it -
 * the two sorted sequences merged piece by piece along S, instead of one
 * search over the whole index per S row (sort_index/main_street/
 * join_gpu.cu:10-113).  s_sorted != 0: S is already ordered by val (signed);
 * 0: the call first sorts a copy of S in the handle's scratch (four LSD
 * passes).  Rows come in no particular order; the index must be a sort
 * index (EJ_ERR_INVALID otherwise). */
ej_status ej_index_merge_join(ej_handle* h, const ej_index* idx, const ej_tuple* S, uint64_t nS, int s_sorted,
                              ej_result* out, uint64_t out_cap, uint64_t* out_count);
/* Build + probe in one call, timed like the reference (index build then join). */
ej_status ej_hash_index_join(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S,
                             uint64_t nS, ej_result* out, uint64_t out_cap, uint64_t* out_count);
ej_status ej_sort_index_join(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S,
                             uint64_t nS, ej_result* out, uint64_t out_cap, uint64_t* out_count);

/* Left outer join preserving S: the inner join plus one row
 * (EJ_NULL_KEY, EJ_NULL_KEY, s.key, s.val) per S row without a match.  The
 * reference's joins/outerJoin_gpu/gpu/outer-idx-bnlj.cc:83-168 is named an outer
 * join but emits no unmatched rows; this entry point gives the outer semantics. */
ej_status ej_left_outer_join(ej_handle* h, const ej_tuple* R, uint64_t nR, const ej_tuple* S,
                             uint64_t nS, ej_result* out, uint64_t out_cap, uint64_t* out_count);
ej_status ej_index_left_outer_join(ej_handle* h, const ej_index* idx, const ej_tuple* S, uint64_t nS,
                                   ej_result* out, uint64_t out_cap, uint64_t* out_count);

/* 3-way star join: fact rows (F1[i], F2[i]) share row i; F1[i].val joins D1.val
 * and F2[i].val joins D2.val; every combination of matches is one row.
 * The reference has no multi-way join (joins/multi_joins is multi-threaded
 * CPU code); this entry point composes two index probes. */
ej_status ej_star_join3(ej_handle* h, const ej_tuple* F1, const ej_tuple* F2, uint64_t nF,
                        const ej_tuple* D1, uint64_t nD1, const ej_tuple* D2, uint64_t nD2,
                        ej_star_result* out, uint64_t out_cap, uint64_t* out_count);

/* Generic dispatcher mirroring `./Exe <left> <right>` of the reference drivers. */
ej_status ej_join(ej_handle* h, ej_algo algo, const ej_tuple* R, uint64_t nR, const ej_tuple* S,
                  uint64_t nS, ej_result* out, uint64_t out_cap, uint64_t* out_count);

/* ---- batched joins --------------------------------------------------------- */

/* One hash join of a batch: device relations, device output of out_cap rows. */
typedef struct ej_join_desc {
  const ej_tuple* R;
  uint64_t nR;
  const ej_tuple* S;
  uint64_t nS;
  ej_result* out;
  uint64_t out_cap;
} ej_join_desc;

/* Many hash joins as one pipeline: a fixed sequence of launches builds every
 * join's table (segmented radix passes) and probes every join (one work queue
 * of (join, tile) tasks), instead of one pipeline per join.  The reference runs
 * one join per process (joins/hashJoin_gpu/main_street/hj.cc:171-1269).  Each
 * join's rows are bitwise those of ej_single_hash_join on the same inputs.
 * counts[i] (host) receives join i's total; EJ_ERR_CAPACITY when any join has
 * more results than its out_cap (its rows past out_cap are dropped). */
ej_status ej_batch_hash_join(ej_handle* h, const ej_join_desc* joins, uint32_t njoins, uint64_t* counts);
/* Asynchronous form: counts go to the device array d_counts[njoins]; no host
 * synchronisation (the join descriptors are copied before the call returns). */
ej_status ej_batch_hash_join_async(ej_handle* h, const ej_join_desc* joins, uint32_t njoins, uint64_t* d_counts);

/* ---- serving: continuous batching of join requests -------------------------- */

/* A request server on one device.  Requests (device relations and a device
 * output of out_cap rows, owned by the client until the request completes)
 * queue on submission; whenever one of the server's lanes is free, its
 * scheduler thread takes the queued requests in arrival order, up to
 * max_batch_joins and up to the lane's device-scratch budget (the request's
 * footprint: its R copies and table plus the probe work queue), and launches
 * them as one batch (EJ_SERVE_BATCHED, ej_batch_hash_join_async) or each as
 * its own pipeline (EJ_SERVE_PER_JOIN, ej_hash_join_async).  Lanes run on
 * their own streams, so batches overlap on the device; each lane keeps its
 * scratch arena across batches.  The reference has no server (one join per
 * process). */
typedef enum ej_serve_mode { EJ_SERVE_BATCHED = 0, EJ_SERVE_PER_JOIN = 1 } ej_serve_mode;

typedef struct ej_server_config {
  int device;
  int mode;                 /* ej_serve_mode */
  uint32_t lanes;           /* batches in flight at once (0: 2) */
  uint32_t max_batch_joins; /* joins per batch (0: 1024); 1 in EJ_SERVE_PER_JOIN */
  uint64_t lane_bytes;      /* device scratch budget per lane (0: 16 GiB); a single
                               larger request still runs, alone */
  uint32_t max_queued;      /* requests waiting for a lane at once (0: no limit); a
                               submit past it is refused with EJ_ERR_BUSY */
  uint32_t flags;           /* EJ_SERVE_CHECKSUM, or 0 */
} ej_server_config;

/* ej_server_config.flags: after each batch, the lane computes on the device
 * the order-independent checksum (ej_checksum's) of every request's rows and
 * reports it in its completion, so that a client can verify each result
 * without reading its rows back */
#define EJ_SERVE_CHECKSUM 1u

typedef struct ej_completion {
  uint64_t tag;          /* the submit tag */
  uint64_t count;        /* the join's result count (rows past out_cap dropped) */
  int32_t status;        /* EJ_OK, EJ_ERR_CAPACITY or the batch's error */
  uint32_t batch_joins;  /* joins in the batch that carried the request */
  uint64_t arrival_ns;   /* ej_now_ns() clock: arrival, launch, completion */
  uint64_t launch_ns;
  uint64_t done_ns;
  uint64_t checksum;     /* EJ_SERVE_CHECKSUM: ej_checksum of the request's rows (else 0) */
} ej_completion;

typedef struct ej_server ej_server;

ej_status ej_server_create(const ej_server_config* cfg, ej_server** out);
/* Queue one request (thread-safe).  arrival_ns = 0 stamps the current time.
 * EJ_ERR_BUSY: refused (max_queued requests already wait, or the server is
 * shutting down); the request was not queued and never completes. */
ej_status ej_server_submit(ej_server* s, const ej_join_desc* join, uint64_t tag, uint64_t arrival_ns);
/* Take up to max completions; waits up to wait_us microseconds for the first. */
ej_status ej_server_poll(ej_server* s, ej_completion* out, uint32_t max, uint32_t* n, uint32_t wait_us);
/* Wait until every submitted request has completed (its completion can still be polled). */
ej_status ej_server_drain(ej_server* s);
ej_status ej_server_destroy(ej_server* s);
/* monotonic clock of the server, nanoseconds */
uint64_t ej_now_ns(void);

/* ---- host-buffer entry points --------------------------------------------- */

/* Same as ej_join, but R, S and out are HOST buffers (pinned memory is fastest):
 * the call uploads the relations, joins on the device and downloads the rows,
 * like the reference drivers' cuMemcpyHtoD/DtoH around the kernels
 * (hj.cc:345-354, :1124).  Device buffers come from the handle's arena. */
ej_status ej_join_host(ej_handle* h, ej_algo algo, const ej_tuple* R, uint64_t nR,
                       const ej_tuple* S, uint64_t nS, ej_result* out, uint64_t out_cap,
                       uint64_t* out_count);

/* Out-of-core form of ej_join_host for the hash join (EJ_ALGO_HASH) and the
 * block nested loop (EJ_ALGO_BNL): relations and result of any size.  R goes
 * to the device in blocks of at most r_block_rows (the hash join builds each
 * block's table once); S streams through in chunks of at most s_chunk_rows,
 * double-buffered, so the upload of one chunk and the download of the
 * previous chunk's rows overlap the join of the current one.  Pinned host
 * buffers are used in place (a pinned out receives rows straight from the
 * write pass); pageable ones are staged.  Rows come in (R block, S chunk)
 * order; past out_cap they are counted only (EJ_ERR_CAPACITY, *out_count =
 * the full count).  Replaces the whole-relation transfers around the
 * reference kernels (joins/hashJoin_gpu/main_street/hj.cc:345-354, :1124) and
 * the device-sized tiling of joins/blockJoin_gpu/main_street/nestLoopJoin.cc:326-519. */
typedef struct ej_chunk_config {
  uint64_t r_block_rows; /* 0: sized from the free device memory */
  uint64_t s_chunk_rows; /* 0: 2^25 rows */
} ej_chunk_config;
ej_status ej_join_host_chunked(ej_handle* h, ej_algo algo, const ej_tuple* R, uint64_t nR,
                               const ej_tuple* S, uint64_t nS, ej_result* out, uint64_t out_cap,
                               uint64_t* out_count, const ej_chunk_config* cfg);

/* ---- prefix scan ----------------------------------------------------------- */

/* Exclusive prefix sum of n uint32 counts into n+1 uint64 offsets (out[n] =
 * total), single pass with decoupled look-back.  Replaces presum()
 * (joins/hashJoin_gpu/main_street/scan_main.cpp:38-111), which scans uint32
 * in place, pads to 2048/2^20 multiples and frees its input. */
ej_status ej_exclusive_scan_u32(ej_handle* h, const uint32_t* in, uint64_t n, uint64_t* out);

/* The same scan for callers that cannot allocate device memory: code whose
 * host framework already owns all of the GPU's memory through its own pool,
 * code that must not call cudaMalloc/cudaFree because they synchronise the
 * whole device, and code that cannot keep an ej_handle (creating one
 * allocates).  No counterpart in the reference.  It allocates nothing: its
 * look-back scratch is a static device array sized for at most
 * EJ_NOALLOC_SCAN_MAX_N inputs (about 512 KB, held on every device that loads
 * the library until the process exits); larger n returns EJ_ERR_TOO_LARGE.
 * in and out (n + 1 uint64 offsets, out[n] = total) are device pointers owned
 * by the caller; the scan runs on `stream` on the current device, and every
 * call synchronises `stream` before it returns (it reads the scan's status
 * word back to the host).  The first call on a device looks up the
 * scratch address for that device; make that first call before any stream
 * capture.  All calls share the one scratch array, so calls that overlap on
 * the GPU (other streams or host threads) race and must be serialised by the
 * caller. */
#define EJ_NOALLOC_SCAN_MAX_N (1ull << 28)
ej_status ej_exclusive_scan_u32_noalloc(const uint32_t* in, uint64_t n, uint64_t* out, ej_stream stream);

/* ---- failure injection for tests ------------------------------------------- */

/* The next `count` device or pinned-host allocations the library makes (any
 * handle, index, server or host-buffer path, any thread) fail as if the memory
 * were exhausted, so that a caller's handling of EJ_ERR_NOMEM can be tested
 * without exhausting a shared GPU's memory.  0 clears it.  The reference has
 * no counterpart (its drivers exit(1) on any failed cuMemAlloc,
 * joins/hashJoin_gpu/main_street/hj.cc:467-475). */
void ej_inject_alloc_failures(uint32_t count);

/* ---- inputs and checks --------------------------------------------------- */

/* Fill a device relation from a generator spec (see ej_gen.h).  For Zipf specs
 * with s > 0, spec->cdf may be NULL: the library builds the CDF itself. */
ej_status ej_generate(ej_handle* h, const ej_gen_spec* spec, ej_tuple* out);
/* Order-independent checksum of rows (sum of a 64-bit mix per row; the same
 * function as the oracle's), for comparing result multisets without sorting. */
ej_status ej_checksum(ej_handle* h, const void* rows, uint64_t nrows, uint32_t words_per_row,
                      uint64_t* out_sum);

/* ---- on-disk relations ----------------------------------------------------
 * The reference's two table formats (little-endian):
 *   EJ_TABLE_FILE_COUNTED  int32 n, then n tuples: written by
 *                          joins/hashJoin_gpu/main_street/TableBuild.cpp:113-140,
 *                          read by joins/hashJoin_gpu/disk_hash/hj.cc:212-266;
 *   EJ_TABLE_FILE_RAW      tuples only, n = file size / 8: joins/join_ori/R and S,
 *                          read by joins/join_ori/hj.cc:68-78.
 * The reference reads these with fread/read inside each executable; these entry
 * points replace those loops.  A missing, truncated or malformed file returns
 * EJ_ERR_IO; more rows than cap return EJ_ERR_CAPACITY with *n set. */
typedef enum { EJ_TABLE_FILE_COUNTED = 0, EJ_TABLE_FILE_RAW = 1 } ej_table_file_format;
/* Rows of a table file (host only, no handle). */
ej_status ej_table_file_rows(const char* path, ej_table_file_format fmt, uint64_t* n);
/* Read a table file into host memory (host only, no handle). */
ej_status ej_table_file_read(const char* path, ej_table_file_format fmt, ej_tuple* dst, uint64_t cap, uint64_t* n);
/* Load a table file into device memory: the file streams through two pinned
 * 32 MiB buffers, each read overlapping the copy of the previous chunk on the
 * handle's stream; returns when dst holds the rows. */
ej_status ej_table_load(ej_handle* h, const char* path, ej_table_file_format fmt, ej_tuple* dst, uint64_t cap,
                        uint64_t* n);
/* Write n rows (device or host memory) as a table file; from device memory
 * each chunk's copy overlaps the write of the previous one. */
ej_status ej_table_save(ej_handle* h, const char* path, ej_table_file_format fmt, const ej_tuple* src, uint64_t n);

#ifdef __cplusplus
}
#endif

#endif /* EJ_H */
