/*
 * ej_oracle.c - CPU restatement of the reference's join algorithms.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle for the CUDA join
 * engine: the tests, the smoke check and the CPU-baseline leg of the bench call
 * it as a checker.  The engine never links it, and nothing in the engine falls
 * back to it.
 *
 * Each join below follows one reference program loop for loop, but takes the
 * relations as arguments and materialises every result row (the reference
 * programs generate their own time-seeded inputs and only print a count).
 * Paths are relative to the reference project root.
 *
 * Conventions shared with the reference and the engine:
 *   TUPLE  {int key; int val;}   - .val is the join attribute, .key a row id
 *                                  (joins/hashJoin_gpu/main_street/tuple.h:43-46)
 *   RESULT {rkey, rval, lkey, lval} - r* from the right/build relation R,
 *                                  l* from the left/probe relation S
 *                                  (joins/hashJoin_gpu/main_street/join_gpu.cu:104-107)
 *
 * Deliberate differences from the reference sources, none of which changes
 * the result multiset of a correct join:
 *   - hash_cpu's match loop reads hrt[llocation[i]+j] / hlt[rlocation[i]+k]
 *     (swapped indices, joins/CPU_JOIN/hash_cpu/hj.cc:220-223); the
 *     restatement takes r-fields from R and l-fields from S as the GPU join does.
 *   - bucket indices use the unsigned value (uint32)val % buckets; the
 *     reference's signed `val % N` would index out of bounds for negative keys.
 *   - sortIndex_cpu's upward duplicate walk reads Bucket[bidx+1] even when
 *     bidx+1 == right (joins/CPU_JOIN/sortIndex_cpu/inner-idx-bnlj.cc:226-227);
 *     the restatement checks the bound first.
 *   - counts and offsets are 64-bit (the reference uses int/uint).
 *   - the multithreaded hash join counts each partition's matches, then
 *     writes them at the partition's offset (rows in partition order); the
 *     reference appends every row to one array under one mutex
 *     (joins/multi_joins/hash/thread-hash-bnlj.cc:334-349), which only
 *     serialises it and makes the row order depend on thread timing.  Its lpartitioning
 *     clamps the probe side's chunk end to the build side's size (:190-200);
 *     the restatement clamps to the probe side's.
 *   - the left outer join and the 3-way star join have no reference
 *     implementation (joins/outerJoin_gpu computes an inner join); their
 *     semantics here are defined by this file: outer = inner join plus
 *     (INT32_MIN, INT32_MIN, s.key, s.val) for every unmatched S row;
 *     star = both dimension probes of each fact row, cross product of matches.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "ej_gen.h"

typedef struct { int32_t key, val; } ejo_tuple;
typedef struct { int32_t rkey, rval, lkey, lval; } ejo_result;
typedef struct { ejo_result d1, d2; } ejo_star_result;
typedef struct { int32_t adr, val; } ejo_bucket; /* BUCKET, CPU field order (hash_cpu/tuple.h:28-32) */

#define EJO_NULL INT32_MIN

static inline void emit(ejo_result* out, uint64_t cap, uint64_t n, const ejo_tuple* r, const ejo_tuple* s) {
  if (n < cap) {
    out[n].rkey = r->key;
    out[n].rval = r->val;
    out[n].lkey = s->key;
    out[n].lval = s->val;
  }
}

/* ---------------------------------------------------------------------------
 * Partitioned hash join: joins/CPU_JOIN/hash_cpu/hj.cc
 *   createPart (hj.cc:116-183): histogram of val % NB_BKTENT, exclusive prefix
 *   (rlocation/llocation), scatter into hrt/hlt, for R then for S;
 *   match loop (hj.cc:216-228): per bucket, every S row against every R row.
 * nb_bktent = NB_BKTENT (2^20 in hash_cpu/tuple.h:1).
 * Returns the number of matches; writes min(matches, cap) rows.
 * ------------------------------------------------------------------------- */
static int partition_side(const ejo_tuple* in, uint64_t n, uint32_t nb, ejo_tuple* out,
                          uint64_t* loc, uint64_t* cnt) {
  memset(cnt, 0, sizeof(uint64_t) * nb);
  for (uint64_t i = 0; i < n; i++) cnt[(uint32_t)in[i].val % nb]++;
  loc[0] = 0;
  for (uint32_t i = 1; i < nb; i++) loc[i] = loc[i - 1] + cnt[i - 1];
  memset(cnt, 0, sizeof(uint64_t) * nb);
  for (uint64_t i = 0; i < n; i++) {
    uint32_t idx = (uint32_t)in[i].val % nb;
    out[loc[idx] + cnt[idx]] = in[i];
    cnt[idx]++;
  }
  return 0;
}

uint64_t ejo_hash_join(const ejo_tuple* R, uint64_t nR, const ejo_tuple* S, uint64_t nS,
                       ejo_result* out, uint64_t cap, uint32_t nb_bktent) {
  if (nb_bktent == 0) nb_bktent = 1u << 20;
  ejo_tuple* hrt = (ejo_tuple*)malloc(sizeof(ejo_tuple) * (nR ? nR : 1));
  ejo_tuple* hlt = (ejo_tuple*)malloc(sizeof(ejo_tuple) * (nS ? nS : 1));
  uint64_t* rloc = (uint64_t*)malloc(sizeof(uint64_t) * nb_bktent);
  uint64_t* rcnt = (uint64_t*)malloc(sizeof(uint64_t) * nb_bktent);
  uint64_t* lloc = (uint64_t*)malloc(sizeof(uint64_t) * nb_bktent);
  uint64_t* lcnt = (uint64_t*)malloc(sizeof(uint64_t) * nb_bktent);
  uint64_t n = 0;
  if (!hrt || !hlt || !rloc || !rcnt || !lloc || !lcnt) { n = UINT64_MAX; goto done; }
  partition_side(R, nR, nb_bktent, hrt, rloc, rcnt);
  partition_side(S, nS, nb_bktent, hlt, lloc, lcnt);
  for (uint32_t i = 0; i < nb_bktent; i++) {
    for (uint64_t j = 0; j < lcnt[i]; j++) {
      const ejo_tuple* s = &hlt[lloc[i] + j];
      for (uint64_t k = 0; k < rcnt[i]; k++) {
        const ejo_tuple* r = &hrt[rloc[i] + k];
        if (s->val == r->val) { emit(out, cap, n, r, s); n++; }
      }
    }
  }
done:
  free(hrt); free(hlt); free(rloc); free(rcnt); free(lloc); free(lcnt);
  return n;
}

/* ---------------------------------------------------------------------------
 * Multithreaded partitioned hash join: joins/multi_joins/hash/thread-hash-bnlj.cc
 *   l/rcount_partitioning (:146-179, :219-252): thread t counts val % PARTITION
 *   over its contiguous chunk into L[p * THREAD_NUM + t]; createThreads
 *   (:393-396, :440-443): exclusive prefix of those counts; l/rpartitioning
 *   (:181-217, :254-290): thread t scatters its chunk at the running offsets;
 *   RTGetter + executor (:292-362): threads take partitions one at a time from
 *   a shared counter and nested-loop each partition's S rows against its R
 *   rows.  partitions = PARTITION (2^17), threads = THREAD_NUM (8 there).
 * Returns the number of matches; writes min(matches, cap) rows in partition
 * order (out NULL or cap 0: counts only).
 * ------------------------------------------------------------------------- */
typedef struct {
  const ejo_tuple* in;
  uint64_t n, lo, hi;   /* this thread's chunk of in */
  uint32_t np, t, nt;
  uint64_t* cnt;        /* [np * nt], partition-major */
  ejo_tuple* out;
} mt_part_arg;

/* Each thread counts into its own array and copies it into the shared
 * partition-major layout afterwards.  The reference increments the shared
 * LL[hash * THREAD_NUM + threadIdx] in place (thread-hash-bnlj.cc:174-176),
 * so neighbouring threads write neighbouring words of one cache line on every
 * row; the counts are the same either way, the private arrays only remove
 * that false sharing (it kept 16 threads near the speed of one). */
static void* mt_count(void* a_) {
  mt_part_arg* a = (mt_part_arg*)a_;
  uint64_t* mine = (uint64_t*)calloc(a->np, sizeof(uint64_t));
  if (!mine) { a->out = NULL; return NULL; }
  for (uint64_t i = a->lo; i < a->hi; i++) mine[(uint32_t)a->in[i].val % a->np]++;
  for (uint32_t p = 0; p < a->np; p++) a->cnt[(uint64_t)p * a->nt + a->t] = mine[p];
  free(mine);
  return NULL;
}

/* the scatter's running offsets, likewise thread-private (the reference's
 * LLS[hash * THREAD_NUM + threadIdx]++, :211-213) */
static void* mt_scatter(void* a_) {
  mt_part_arg* a = (mt_part_arg*)a_;
  uint64_t* pos = (uint64_t*)malloc(sizeof(uint64_t) * a->np);
  if (!pos) { a->out = NULL; return NULL; }
  for (uint32_t p = 0; p < a->np; p++) pos[p] = a->cnt[(uint64_t)p * a->nt + a->t];
  for (uint64_t i = a->lo; i < a->hi; i++) a->out[pos[(uint32_t)a->in[i].val % a->np]++] = a->in[i];
  free(pos);
  return NULL;
}

/* partition one side with nt threads; start[p] = first row of partition p */
static int mt_partition(const ejo_tuple* in, uint64_t n, uint32_t np, uint32_t nt, ejo_tuple* out,
                        uint64_t* start) {
  uint64_t* cnt = (uint64_t*)calloc((size_t)np * nt, sizeof(uint64_t));
  mt_part_arg* args = (mt_part_arg*)calloc(nt, sizeof(mt_part_arg));
  pthread_t* th = (pthread_t*)calloc(nt, sizeof(pthread_t));
  if (!cnt || !args || !th) { free(cnt); free(args); free(th); return -1; }
  const uint64_t chunk = (n + nt - 1) / nt;
  for (uint32_t t = 0; t < nt; t++) {
    args[t].in = in; args[t].n = n; args[t].np = np; args[t].t = t; args[t].nt = nt;
    args[t].cnt = cnt; args[t].out = out;
    args[t].lo = (uint64_t)t * chunk < n ? (uint64_t)t * chunk : n;
    args[t].hi = args[t].lo + chunk < n ? args[t].lo + chunk : n;
  }
  int failed = 0;
  for (uint32_t t = 0; t < nt; t++) pthread_create(&th[t], NULL, mt_count, &args[t]);
  for (uint32_t t = 0; t < nt; t++) pthread_join(th[t], NULL);
  for (uint32_t t = 0; t < nt; t++) failed |= args[t].out == NULL;
  if (failed) { free(cnt); free(args); free(th); return -1; }
  uint64_t run = 0;
  for (uint64_t k = 0; k < (uint64_t)np * nt; k++) {
    const uint64_t c = cnt[k];
    cnt[k] = run;
    run += c;
  }
  for (uint32_t p = 0; p < np; p++) start[p] = cnt[(uint64_t)p * nt];
  start[np] = n;
  for (uint32_t t = 0; t < nt; t++) pthread_create(&th[t], NULL, mt_scatter, &args[t]);
  for (uint32_t t = 0; t < nt; t++) pthread_join(th[t], NULL);
  for (uint32_t t = 0; t < nt; t++) failed |= args[t].out == NULL;
  free(cnt); free(args); free(th);
  return failed ? -1 : 0;
}

typedef struct {
  const ejo_tuple *pr, *ps;
  const uint64_t *rstart, *sstart;
  uint32_t np;
  uint32_t* next;        /* shared partition counter */
  uint64_t* pcount;      /* matches of each partition (first pass) */
  const uint64_t* poff;  /* output offset of each partition (second pass) */
  ejo_result* out;
  uint64_t cap;
} mt_join_arg;

/* threads take partitions from the shared counter; first pass: count each
 * partition's matches, second pass (poff set): write them at its offset */
static void* mt_join(void* a_) {
  mt_join_arg* a = (mt_join_arg*)a_;
  for (;;) {
    const uint32_t p = __atomic_fetch_add(a->next, 1u, __ATOMIC_RELAXED);
    if (p >= a->np) break;
    uint64_t n = a->poff ? a->poff[p] : 0;
    for (uint64_t i = a->sstart[p]; i < a->sstart[p + 1]; i++) {
      const ejo_tuple* s = &a->ps[i];
      for (uint64_t j = a->rstart[p]; j < a->rstart[p + 1]; j++) {
        const ejo_tuple* r = &a->pr[j];
        if (s->val != r->val) continue;
        if (a->poff) emit(a->out, a->cap, n, r, s);
        n++;
      }
    }
    if (!a->poff) a->pcount[p] = n;
  }
  return NULL;
}

static void mt_run(mt_join_arg* args, pthread_t* th, uint32_t nthreads) {
  uint32_t next = 0;
  for (uint32_t t = 0; t < nthreads; t++) {
    args[t].next = &next;
    pthread_create(&th[t], NULL, mt_join, &args[t]);
  }
  for (uint32_t t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
}

uint64_t ejo_hash_join_mt(const ejo_tuple* R, uint64_t nR, const ejo_tuple* S, uint64_t nS,
                          ejo_result* out, uint64_t cap, uint32_t partitions, uint32_t nthreads) {
  if (partitions == 0) partitions = 1u << 17;
  if (nthreads == 0) nthreads = 8;
  ejo_tuple* pr = (ejo_tuple*)malloc(sizeof(ejo_tuple) * (nR ? nR : 1));
  ejo_tuple* ps = (ejo_tuple*)malloc(sizeof(ejo_tuple) * (nS ? nS : 1));
  uint64_t* rstart = (uint64_t*)malloc(sizeof(uint64_t) * ((uint64_t)partitions + 1));
  uint64_t* sstart = (uint64_t*)malloc(sizeof(uint64_t) * ((uint64_t)partitions + 1));
  uint64_t* pcount = (uint64_t*)malloc(sizeof(uint64_t) * partitions);
  uint64_t* poff = (uint64_t*)malloc(sizeof(uint64_t) * partitions);
  mt_join_arg* args = (mt_join_arg*)calloc(nthreads, sizeof(mt_join_arg));
  pthread_t* th = (pthread_t*)calloc(nthreads, sizeof(pthread_t));
  uint64_t total = UINT64_MAX;
  if (!pr || !ps || !rstart || !sstart || !pcount || !poff || !args || !th) goto done;
  if (mt_partition(R, nR, partitions, nthreads, pr, rstart) || mt_partition(S, nS, partitions, nthreads, ps, sstart))
    goto done;
  for (uint32_t t = 0; t < nthreads; t++) {
    args[t].pr = pr; args[t].ps = ps; args[t].rstart = rstart; args[t].sstart = sstart;
    args[t].np = partitions; args[t].pcount = pcount; args[t].out = out; args[t].cap = cap;
  }
  mt_run(args, th, nthreads);
  total = 0;
  for (uint32_t p = 0; p < partitions; p++) {
    poff[p] = total;
    total += pcount[p];
  }
  if (out && cap) {
    for (uint32_t t = 0; t < nthreads; t++) args[t].poff = poff;
    mt_run(args, th, nthreads);
  }
done:
  free(pr); free(ps); free(rstart); free(sstart); free(pcount); free(poff); free(args); free(th);
  return total;
}

/* ---------------------------------------------------------------------------
 * Hash-index inner join: joins/CPU_JOIN/inner_cpu/inner-idx-bnlj.cc
 *   index (:142-166): idxcount[val % NB_BUCKET]++, Buck_array = exclusive
 *   prefix (-1 for empty buckets), Bucket[] = {val, adr=row} grouped by bucket;
 *   probe (:174-185): per S row, scan its bucket comparing val.
 * nb_bucket = NB_BUCKET (2^27 in inner_cpu/tuple.h:1).
 * ------------------------------------------------------------------------- */
typedef struct {
  uint32_t nb;
  int64_t* buck_array; /* start of bucket, -1 when empty */
  uint64_t* idxcount;
  ejo_bucket* bucket;
} ejo_hash_index;

static int hash_index_build(const ejo_tuple* R, uint64_t nR, uint32_t nb, ejo_hash_index* ix) {
  ix->nb = nb;
  ix->buck_array = (int64_t*)malloc(sizeof(int64_t) * nb);
  ix->idxcount = (uint64_t*)calloc(nb, sizeof(uint64_t));
  ix->bucket = (ejo_bucket*)malloc(sizeof(ejo_bucket) * (nR ? nR : 1));
  if (!ix->buck_array || !ix->idxcount || !ix->bucket) return -1;
  for (uint64_t i = 0; i < nR; i++) ix->idxcount[(uint32_t)R[i].val % nb]++;
  uint64_t count = 0;
  for (uint32_t i = 0; i < nb; i++) {
    ix->buck_array[i] = ix->idxcount[i] == 0 ? -1 : (int64_t)count;
    count += ix->idxcount[i];
  }
  memset(ix->idxcount, 0, sizeof(uint64_t) * nb);
  for (uint64_t i = 0; i < nR; i++) {
    uint32_t idx = (uint32_t)R[i].val % nb;
    ejo_bucket* b = &ix->bucket[ix->buck_array[idx] + ix->idxcount[idx]];
    b->val = R[i].val;
    b->adr = (int32_t)i;
    ix->idxcount[idx]++;
  }
  return 0;
}

static void hash_index_free(ejo_hash_index* ix) {
  free(ix->buck_array); free(ix->idxcount); free(ix->bucket);
}

/* matches of one probe row; emits from position n, returns the new n */
static uint64_t hash_index_probe_row(const ejo_hash_index* ix, const ejo_tuple* R, const ejo_tuple* s,
                                     ejo_result* out, uint64_t cap, uint64_t n) {
  uint32_t hash = (uint32_t)s->val % ix->nb;
  uint64_t cnt = ix->idxcount[hash];
  for (uint64_t i = 0; i < cnt; i++) {
    const ejo_bucket* b = &ix->bucket[ix->buck_array[hash] + i];
    if (b->val == s->val) { emit(out, cap, n, &R[b->adr], s); n++; }
  }
  return n;
}

uint64_t ejo_hash_index_join(const ejo_tuple* R, uint64_t nR, const ejo_tuple* S, uint64_t nS,
                             ejo_result* out, uint64_t cap, uint32_t nb_bucket) {
  if (nb_bucket == 0) nb_bucket = 1u << 27;
  ejo_hash_index ix;
  uint64_t n = 0;
  if (hash_index_build(R, nR, nb_bucket, &ix) != 0) { hash_index_free(&ix); return UINT64_MAX; }
  for (uint64_t j = 0; j < nS; j++) n = hash_index_probe_row(&ix, R, &S[j], out, cap, n);
  hash_index_free(&ix);
  return n;
}

/* ---------------------------------------------------------------------------
 * Sort-index inner join: joins/CPU_JOIN/sortIndex_cpu/inner-idx-bnlj.cc
 *   createIndex (:129-146): Bucket[i] = {val, adr=i}, recursive quicksort on
 *   val (:106-127, middle pivot, Hoare-style crossing scans);
 *   search (:163-174): binary search that stops on the first equal element;
 *   probe (:212-237): walk equal values downward from the hit, then upward.
 * ------------------------------------------------------------------------- */
static void sort_index_qsort(ejo_bucket* b, int64_t p, int64_t q) {
  /* explicit stack instead of recursion; same partition step as the reference */
  int64_t stack[2 * 64 * 2];
  int top = 0;
  stack[top++] = p; stack[top++] = q;
  while (top > 0) {
    q = stack[--top]; p = stack[--top];
    for (;;) {
      int64_t i = p, j = q;
      int32_t pivot = b[(p + q) / 2].val;
      for (;;) {
        while (b[i].val < pivot) i++;
        while (pivot < b[j].val) j--;
        if (i >= j) break;
        ejo_bucket t = b[i]; b[i] = b[j]; b[j] = t;
        i++; j--;
      }
      /* sub-ranges [p, i-1] and [j+1, q]; recurse on the smaller one first */
      int64_t lp = p, lq = i - 1, rp = j + 1, rq = q;
      int has_l = p < i - 1, has_r = j + 1 < q;
      if (has_l && has_r) {
        if (lq - lp < rq - rp) { stack[top++] = rp; stack[top++] = rq; p = lp; q = lq; }
        else { stack[top++] = lp; stack[top++] = lq; p = rp; q = rq; }
        continue;
      }
      if (has_l) { p = lp; q = lq; continue; }
      if (has_r) { p = rp; q = rq; continue; }
      break;
    }
  }
}

static int64_t sort_index_search(const ejo_bucket* b, int32_t num, uint64_t right) {
  int64_t m, l = 0, r = (int64_t)right - 1;
  do {
    m = (l + r) / 2;
    if (num < b[m].val) r = m - 1; else l = m + 1;
  } while (l <= r && num != b[m].val);
  return m;
}

uint64_t ejo_sort_index_join(const ejo_tuple* R, uint64_t nR, const ejo_tuple* S, uint64_t nS,
                             ejo_result* out, uint64_t cap) {
  if (nR == 0) return 0;
  ejo_bucket* b = (ejo_bucket*)malloc(sizeof(ejo_bucket) * nR);
  if (!b) return UINT64_MAX;
  for (uint64_t i = 0; i < nR; i++) { b[i].val = R[i].val; b[i].adr = (int32_t)i; }
  sort_index_qsort(b, 0, (int64_t)nR - 1);
  uint64_t n = 0;
  for (uint64_t j = 0; j < nS; j++) {
    const ejo_tuple* s = &S[j];
    int64_t bidx = sort_index_search(b, s->val, nR);
    int64_t x = bidx;
    while (b[x].val == s->val) {
      emit(out, cap, n, &R[b[x].adr], s); n++;
      if (x == 0) break;
      x--;
    }
    x = bidx + 1;
    while (x < (int64_t)nR && b[x].val == s->val) {
      emit(out, cap, n, &R[b[x].adr], s); n++;
      x++;
    }
  }
  free(b);
  return n;
}

/* ---------------------------------------------------------------------------
 * Block nested-loop join: joins/CPU_JOIN/block_cpu/nestLoopJoin.cc:61-77
 *   every left (S) row against every right (R) row, equality on val.
 * ------------------------------------------------------------------------- */
uint64_t ejo_bnl_join(const ejo_tuple* R, uint64_t nR, const ejo_tuple* S, uint64_t nS,
                      ejo_result* out, uint64_t cap) {
  uint64_t n = 0;
  for (uint64_t i = 0; i < nS; i++)
    for (uint64_t j = 0; j < nR; j++)
      if (S[i].val == R[j].val) { emit(out, cap, n, &R[j], &S[i]); n++; }
  return n;
}

/* ---------------------------------------------------------------------------
 * Left outer join (semantics defined here; see header): hash-index probe as in
 * inner_cpu, plus one (INT32_MIN, INT32_MIN, s.key, s.val) row per unmatched S row.
 * ------------------------------------------------------------------------- */
uint64_t ejo_left_outer_join(const ejo_tuple* R, uint64_t nR, const ejo_tuple* S, uint64_t nS,
                             ejo_result* out, uint64_t cap, uint32_t nb_bucket) {
  if (nb_bucket == 0) nb_bucket = 1u << 27;
  ejo_hash_index ix;
  uint64_t n = 0;
  if (hash_index_build(R, nR, nb_bucket, &ix) != 0) { hash_index_free(&ix); return UINT64_MAX; }
  ejo_tuple null_r = {EJO_NULL, EJO_NULL};
  for (uint64_t j = 0; j < nS; j++) {
    uint64_t before = n;
    n = hash_index_probe_row(&ix, R, &S[j], out, cap, n);
    if (n == before) { emit(out, cap, n, &null_r, &S[j]); n++; }
  }
  hash_index_free(&ix);
  return n;
}

/* ---------------------------------------------------------------------------
 * 3-way star join (semantics defined here; see header): fact rows F1[i], F2[i]
 * (same row id, two foreign-key columns) joined with D1 on F1.val and with D2
 * on F2.val; every pair of matches is one output row {d1-part, d2-part}.
 * ------------------------------------------------------------------------- */
uint64_t ejo_star_join3(const ejo_tuple* F1, const ejo_tuple* F2, uint64_t nF,
                        const ejo_tuple* D1, uint64_t nD1, const ejo_tuple* D2, uint64_t nD2,
                        ejo_star_result* out, uint64_t cap, uint32_t nb_bucket) {
  if (nb_bucket == 0) nb_bucket = 1u << 20;
  ejo_hash_index i1, i2;
  uint64_t n = 0;
  int ok = hash_index_build(D1, nD1, nb_bucket, &i1) == 0;
  ok = (hash_index_build(D2, nD2, nb_bucket, &i2) == 0) && ok;
  if (!ok) { hash_index_free(&i1); hash_index_free(&i2); return UINT64_MAX; }
  for (uint64_t f = 0; f < nF; f++) {
    uint32_t h1 = (uint32_t)F1[f].val % nb_bucket, h2 = (uint32_t)F2[f].val % nb_bucket;
    for (uint64_t a = 0; a < i1.idxcount[h1]; a++) {
      const ejo_bucket* b1 = &i1.bucket[i1.buck_array[h1] + a];
      if (b1->val != F1[f].val) continue;
      for (uint64_t c = 0; c < i2.idxcount[h2]; c++) {
        const ejo_bucket* b2 = &i2.bucket[i2.buck_array[h2] + c];
        if (b2->val != F2[f].val) continue;
        if (n < cap) {
          const ejo_tuple* d1 = &D1[b1->adr];
          const ejo_tuple* d2 = &D2[b2->adr];
          out[n].d1.rkey = d1->key; out[n].d1.rval = d1->val;
          out[n].d1.lkey = F1[f].key; out[n].d1.lval = F1[f].val;
          out[n].d2.rkey = d2->key; out[n].d2.rval = d2->val;
          out[n].d2.lkey = F2[f].key; out[n].d2.lval = F2[f].val;
        }
        n++;
      }
    }
  }
  hash_index_free(&i1); hash_index_free(&i2);
  return n;
}

/* ---------------------------------------------------------------------------
 * Count-only hash join (no materialisation): the count pass of hash_cpu for
 * sizes whose result does not fit in host memory.
 * ------------------------------------------------------------------------- */
uint64_t ejo_hash_join_count(const ejo_tuple* R, uint64_t nR, const ejo_tuple* S, uint64_t nS,
                             uint32_t nb_bucket) {
  if (nb_bucket == 0) nb_bucket = 1u << 20;
  ejo_hash_index ix;
  uint64_t n = 0;
  if (hash_index_build(R, nR, nb_bucket, &ix) != 0) { hash_index_free(&ix); return UINT64_MAX; }
  for (uint64_t j = 0; j < nS; j++) {
    uint32_t hash = (uint32_t)S[j].val % nb_bucket;
    for (uint64_t i = 0; i < ix.idxcount[hash]; i++)
      n += ix.bucket[ix.buck_array[hash] + i].val == S[j].val;
  }
  hash_index_free(&ix);
  return n;
}

/* ---------------------------------------------------------------------------
 * Distance nested-loop join: joins/CPU_JOIN/3d_cpu/nestLoopJoin.cc:73-101
 * (VAL_NUM 3) and joins/blockJoin_gpu/complex_block/2d_cpu/nestLoopJoin.cc:73-101
 * (VAL_NUM 2): every left (S) point against every right (R) point, left-major;
 * eval computes t = r.val[i] - l.val[i], temp += t * t in double and matches
 * on temp < radius * radius (DISTANCE = 1 there).  This file is compiled with
 * -ffp-contract=off, so every operation rounds on its own as in the reference.
 * Rows: dims 2 {lid; lval[2]; rid; rval[2]} (blockJoin_gpu/complex_block/
 * dire_join/tuple.h:25-30), dims 3 {lval[3]; rval[3]; lid; rid}
 * (3d_cpu/nestLoopJoin.cc:28-33); padding bytes are zero.
 * nthreads > 1 splits S into contiguous ranges, counts each, then writes each
 * at its offset: the rows come out in the single-threaded order.
 * ------------------------------------------------------------------------- */
typedef struct { int32_t lid; double lval[2]; int32_t rid; double rval[2]; } ejo_point_result2;
typedef struct { double lval[3]; double rval[3]; int32_t lid, rid; } ejo_point_result3;

static size_t dist_point_bytes(uint32_t dims) { return 8 + 8 * (size_t)dims; }
static int32_t dist_id(const char* p) { int32_t id; memcpy(&id, p, 4); return id; }
static const double* dist_val(const char* p) { return (const double*)(p + 8); }

static int dist_eval(const double* r, const double* l, uint32_t dims, double r2) {
  double temp = 0, t;
  for (uint32_t i = 0; i < dims; i++) {
    t = r[i] - l[i];
    temp += t * t;
  }
  return temp < r2;
}

static void dist_emit(void* out, uint64_t n, uint32_t dims, const char* l, const char* r) {
  const double* lv = dist_val(l);
  const double* rv = dist_val(r);
  if (dims == 2) {
    ejo_point_result2 row;
    memset(&row, 0, sizeof row);
    row.lid = dist_id(l);
    row.rid = dist_id(r);
    for (int i = 0; i < 2; i++) { row.lval[i] = lv[i]; row.rval[i] = rv[i]; }
    memcpy((char*)out + n * sizeof row, &row, sizeof row);
  } else {
    ejo_point_result3 row;
    memset(&row, 0, sizeof row);
    row.lid = dist_id(l);
    row.rid = dist_id(r);
    for (int i = 0; i < 3; i++) { row.lval[i] = lv[i]; row.rval[i] = rv[i]; }
    memcpy((char*)out + n * sizeof row, &row, sizeof row);
  }
}

typedef struct {
  uint32_t dims;
  const char *R, *S;
  uint64_t nR, s0, s1;
  double r2;
  void* out;     /* NULL: count only */
  uint64_t base; /* first row of this range */
  uint64_t cap;
  uint64_t n;
} dist_arg;

static void* dist_range(void* a_) {
  dist_arg* a = (dist_arg*)a_;
  const size_t pb = dist_point_bytes(a->dims);
  uint64_t n = 0;
  for (uint64_t i = a->s0; i < a->s1; i++) {
    const char* l = a->S + i * pb;
    for (uint64_t j = 0; j < a->nR; j++) {
      const char* r = a->R + j * pb;
      if (dist_eval(dist_val(r), dist_val(l), a->dims, a->r2)) {
        if (a->out && a->base + n < a->cap) dist_emit(a->out, a->base + n, a->dims, l, r);
        n++;
      }
    }
  }
  a->n = n;
  return NULL;
}

uint64_t ejo_distance_join(uint32_t dims, const void* R, uint64_t nR, const void* S, uint64_t nS, double radius,
                           void* out, uint64_t cap, uint32_t nthreads) {
  if (dims != 2 && dims != 3) return UINT64_MAX;
  if (nthreads == 0) nthreads = 1;
  if ((uint64_t)nthreads > nS) nthreads = nS ? (uint32_t)nS : 1;
  dist_arg* args = (dist_arg*)calloc(nthreads, sizeof(dist_arg));
  pthread_t* th = (pthread_t*)calloc(nthreads, sizeof(pthread_t));
  if (!args || !th) { free(args); free(th); return UINT64_MAX; }
  const double r2 = radius * radius;
  for (uint32_t t = 0; t < nthreads; t++) {
    dist_arg* a = &args[t];
    a->dims = dims;
    a->R = (const char*)R;
    a->S = (const char*)S;
    a->nR = nR;
    a->s0 = nS * t / nthreads;
    a->s1 = nS * (t + 1) / nthreads;
    a->r2 = r2;
  }
  /* pass 1: counts; pass 2 (rows wanted): each range at its offset */
  for (int pass = 0; pass < (out ? 2 : 1); pass++) {
    uint64_t base = 0;
    for (uint32_t t = 0; t < nthreads; t++) {
      args[t].out = pass ? out : NULL;
      args[t].cap = cap;
      args[t].base = base;
      base += args[t].n;
    }
    if (nthreads == 1) {
      dist_range(&args[0]);
    } else {
      for (uint32_t t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, dist_range, &args[t]);
      for (uint32_t t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    }
  }
  uint64_t n = 0;
  for (uint32_t t = 0; t < nthreads; t++) n += args[t].n;
  free(args);
  free(th);
  return n;
}

/* ---------------------------------------------------------------------------
 * Inputs and result canonicalisation
 * ------------------------------------------------------------------------- */
void ejo_generate(const ej_gen_spec* sp, ejo_tuple* out) {
  for (uint64_t i = 0; i < sp->n; i++) {
    out[i].key = (int32_t)((uint32_t)sp->key_base + (uint32_t)i);
    out[i].val = ej_gen_val(sp, i);
  }
}

void ejo_zipf_cdf(double s, uint32_t n, double* cdf) {
  double total = 0.0;
  for (uint32_t k = 0; k < n; k++) { total += pow((double)(k + 1u), -s); cdf[k] = total; }
  for (uint32_t k = 0; k < n; k++) cdf[k] = cdf[k] / total;
  if (n) cdf[n - 1] = 1.0;
}

static int cmp_result(const void* a, const void* b) {
  const int32_t* x = (const int32_t*)a;
  const int32_t* y = (const int32_t*)b;
  for (int i = 0; i < 4; i++) {
    if (x[i] < y[i]) return -1;
    if (x[i] > y[i]) return 1;
  }
  return 0;
}

/* canonical order: lexicographic on (rkey, rval, lkey, lval) as signed int32 */
void ejo_canon_sort(ejo_result* r, uint64_t n) { qsort(r, n, sizeof(ejo_result), cmp_result); }

static int cmp_result8(const void* a, const void* b) {
  const int32_t* x = (const int32_t*)a;
  const int32_t* y = (const int32_t*)b;
  for (int i = 0; i < 8; i++) {
    if (x[i] < y[i]) return -1;
    if (x[i] > y[i]) return 1;
  }
  return 0;
}

void ejo_canon_sort_star(ejo_star_result* r, uint64_t n) {
  qsort(r, n, sizeof(ejo_star_result), cmp_result8);
}

/* order-independent checksum of 16-byte rows: sum over rows of a 64-bit mix */
uint64_t ejo_checksum(const int32_t* words, uint64_t nrows, uint32_t words_per_row) {
  uint64_t sum = 0;
  for (uint64_t i = 0; i < nrows; i++) {
    uint64_t h = 0x243F6A8885A308D3ull;
    for (uint32_t w = 0; w < words_per_row; w++)
      h = ej_splitmix64(h ^ (uint64_t)(uint32_t)words[i * words_per_row + w]);
    sum += h;
  }
  return sum;
}

/* ---------------------------------------------------------------------------
 * Digests of results too large to materialise (full-size configurations):
 * the count and the order-independent checksum of a join's rows, computed
 * row by row as the joins above find them but fed to the checksum instead of
 * an output array.  The inner and left outer joins follow
 * joins/multi_joins/hash (ejo_hash_join_mt: partition both sides by
 * val % partitions, threads take partitions from a shared counter and
 * nested-loop each partition's S rows against its R rows); every S row
 * without a match adds its NULL-extended row when `outer` is set, as
 * ejo_left_outer_join emits it.  The star join probes the same hash indexes
 * as ejo_star_join3 (joins/CPU_JOIN/inner_cpu/inner-idx-bnlj.cc:142-185),
 * fact rows split over the threads.  The multiset of rows, and so the digest,
 * is that of the single-threaded joins.
 * ------------------------------------------------------------------------- */
static inline uint64_t row_mix4(int32_t a, int32_t b, int32_t c, int32_t d) {
  uint64_t h = 0x243F6A8885A308D3ull;
  h = ej_splitmix64(h ^ (uint64_t)(uint32_t)a);
  h = ej_splitmix64(h ^ (uint64_t)(uint32_t)b);
  h = ej_splitmix64(h ^ (uint64_t)(uint32_t)c);
  return ej_splitmix64(h ^ (uint64_t)(uint32_t)d);
}

typedef struct {
  const ejo_tuple *pr, *ps;
  const uint64_t *rstart, *sstart;
  uint32_t np;
  int outer;
  uint32_t* next;
  uint64_t count, sum;
} digest_arg;

static void* digest_join(void* a_) {
  digest_arg* a = (digest_arg*)a_;
  uint64_t count = 0, sum = 0;
  for (;;) {
    const uint32_t p = __atomic_fetch_add(a->next, 1u, __ATOMIC_RELAXED);
    if (p >= a->np) break;
    const ejo_tuple* r0 = a->pr + a->rstart[p];
    const uint64_t nr = a->rstart[p + 1] - a->rstart[p];
    for (uint64_t i = a->sstart[p]; i < a->sstart[p + 1]; i++) {
      const ejo_tuple s = a->ps[i];
      uint64_t m = 0;
      for (uint64_t j = 0; j < nr; j++) {
        if (r0[j].val != s.val) continue;
        sum += row_mix4(r0[j].key, r0[j].val, s.key, s.val);
        m++;
      }
      if (a->outer && m == 0) {
        sum += row_mix4(EJO_NULL, EJO_NULL, s.key, s.val);
        m = 1;
      }
      count += m;
    }
  }
  a->count = count;
  a->sum = sum;
  return NULL;
}

int ejo_join_digest_mt(const ejo_tuple* R, uint64_t nR, const ejo_tuple* S, uint64_t nS, int outer,
                       uint32_t partitions, uint32_t nthreads, uint64_t* count, uint64_t* checksum) {
  if (partitions == 0) partitions = 1u << 20;
  if (nthreads == 0) nthreads = 8;
  int rc = -1;
  ejo_tuple* pr = (ejo_tuple*)malloc(sizeof(ejo_tuple) * (nR ? nR : 1));
  ejo_tuple* ps = (ejo_tuple*)malloc(sizeof(ejo_tuple) * (nS ? nS : 1));
  uint64_t* rstart = (uint64_t*)malloc(sizeof(uint64_t) * ((uint64_t)partitions + 1));
  uint64_t* sstart = (uint64_t*)malloc(sizeof(uint64_t) * ((uint64_t)partitions + 1));
  digest_arg* args = (digest_arg*)calloc(nthreads, sizeof(digest_arg));
  pthread_t* th = (pthread_t*)calloc(nthreads, sizeof(pthread_t));
  uint32_t next = 0;
  if (!pr || !ps || !rstart || !sstart || !args || !th) goto done;
  if (mt_partition(R, nR, partitions, nthreads, pr, rstart) || mt_partition(S, nS, partitions, nthreads, ps, sstart))
    goto done;
  for (uint32_t t = 0; t < nthreads; t++) {
    args[t].pr = pr; args[t].ps = ps; args[t].rstart = rstart; args[t].sstart = sstart;
    args[t].np = partitions; args[t].outer = outer; args[t].next = &next;
    pthread_create(&th[t], NULL, digest_join, &args[t]);
  }
  *count = 0;
  *checksum = 0;
  for (uint32_t t = 0; t < nthreads; t++) {
    pthread_join(th[t], NULL);
    *count += args[t].count;
    *checksum += args[t].sum;
  }
  rc = 0;
done:
  free(pr); free(ps); free(rstart); free(sstart); free(args); free(th);
  return rc;
}

typedef struct {
  const ejo_tuple *F1, *F2, *D1, *D2;
  uint64_t f0, f1;
  const ejo_hash_index *i1, *i2;
  uint64_t count, sum;
} star_digest_arg;

static void* star_digest(void* a_) {
  star_digest_arg* a = (star_digest_arg*)a_;
  const ejo_hash_index *i1 = a->i1, *i2 = a->i2;
  uint64_t count = 0, sum = 0;
  for (uint64_t f = a->f0; f < a->f1; f++) {
    const ejo_tuple x = a->F1[f], y = a->F2[f];
    const uint32_t h1 = (uint32_t)x.val % i1->nb, h2 = (uint32_t)y.val % i2->nb;
    for (uint64_t u = 0; u < i1->idxcount[h1]; u++) {
      const ejo_bucket* b1 = &i1->bucket[i1->buck_array[h1] + u];
      if (b1->val != x.val) continue;
      for (uint64_t v = 0; v < i2->idxcount[h2]; v++) {
        const ejo_bucket* b2 = &i2->bucket[i2->buck_array[h2] + v];
        if (b2->val != y.val) continue;
        const ejo_tuple d1 = a->D1[b1->adr], d2 = a->D2[b2->adr];
        const int32_t w[8] = {d1.key, d1.val, x.key, x.val, d2.key, d2.val, y.key, y.val};
        uint64_t h = 0x243F6A8885A308D3ull;
        for (int k = 0; k < 8; k++) h = ej_splitmix64(h ^ (uint64_t)(uint32_t)w[k]);
        sum += h;
        count++;
      }
    }
  }
  a->count = count;
  a->sum = sum;
  return NULL;
}

int ejo_star_digest_mt(const ejo_tuple* F1, const ejo_tuple* F2, uint64_t nF, const ejo_tuple* D1, uint64_t nD1,
                       const ejo_tuple* D2, uint64_t nD2, uint32_t nb_bucket, uint32_t nthreads, uint64_t* count,
                       uint64_t* checksum) {
  if (nb_bucket == 0) nb_bucket = 1u << 20;
  if (nthreads == 0) nthreads = 8;
  ejo_hash_index i1, i2;
  int ok = hash_index_build(D1, nD1, nb_bucket, &i1) == 0;
  ok = (hash_index_build(D2, nD2, nb_bucket, &i2) == 0) && ok;
  star_digest_arg* args = (star_digest_arg*)calloc(nthreads, sizeof(star_digest_arg));
  pthread_t* th = (pthread_t*)calloc(nthreads, sizeof(pthread_t));
  int rc = -1;
  if (ok && args && th) {
    for (uint32_t t = 0; t < nthreads; t++) {
      star_digest_arg* a = &args[t];
      a->F1 = F1; a->F2 = F2; a->D1 = D1; a->D2 = D2; a->i1 = &i1; a->i2 = &i2;
      a->f0 = nF * t / nthreads;
      a->f1 = nF * (t + 1) / nthreads;
      pthread_create(&th[t], NULL, star_digest, a);
    }
    *count = 0;
    *checksum = 0;
    for (uint32_t t = 0; t < nthreads; t++) {
      pthread_join(th[t], NULL);
      *count += args[t].count;
      *checksum += args[t].sum;
    }
    rc = 0;
  }
  hash_index_free(&i1);
  hash_index_free(&i2);
  free(args);
  free(th);
  return rc;
}

/* ejo_generate over row ranges in parallel (the rows are a pure function of
 * the spec and the index, so the result is the same) */
typedef struct {
  const ej_gen_spec* sp;
  ejo_tuple* out;
  uint64_t lo, hi;
} gen_arg;

static void* gen_range(void* a_) {
  gen_arg* a = (gen_arg*)a_;
  for (uint64_t i = a->lo; i < a->hi; i++) {
    a->out[i].key = (int32_t)((uint32_t)a->sp->key_base + (uint32_t)i);
    a->out[i].val = ej_gen_val(a->sp, i);
  }
  return NULL;
}

void ejo_generate_mt(const ej_gen_spec* sp, ejo_tuple* out, uint32_t nthreads) {
  if (nthreads == 0) nthreads = 1;
  gen_arg* args = (gen_arg*)calloc(nthreads, sizeof(gen_arg));
  pthread_t* th = (pthread_t*)calloc(nthreads, sizeof(pthread_t));
  if (!args || !th) {
    free(args);
    free(th);
    ejo_generate(sp, out);
    return;
  }
  for (uint32_t t = 0; t < nthreads; t++) {
    args[t].sp = sp;
    args[t].out = out;
    args[t].lo = sp->n * t / nthreads;
    args[t].hi = sp->n * (t + 1) / nthreads;
    pthread_create(&th[t], NULL, gen_range, &args[t]);
  }
  for (uint32_t t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  free(args);
  free(th);
}
