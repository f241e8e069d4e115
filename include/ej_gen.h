/*
 * ej_gen.h - seeded, counter-based input generators for the join workloads.
 *
 * Every generated value is a pure function of (spec, row index), written with
 * integer arithmetic only (the Zipf sampler compares doubles from a CDF table
 * that the host builds once), so the same header gives bit-identical relations
 * on the host (oracle, CPU baseline) and on the device (bench inputs).
 *
 * The reference generates its inputs with time-seeded rand() and a rejection
 * sampler over [0, SELECTIVITY) (joins/hashJoin_gpu/main_street/hj.cc:62-160,
 * joins/CPU_JOIN/hash_cpu/hj.cc:54-104), which cannot be reproduced or sized to
 * the benchmark distributions; these generators replace it.  Layout follows the
 * reference: the join attribute is TUPLE.val, TUPLE.key is a row id.
 *
 * Building blocks (published algorithms, restated):
 *   splitmix64          - Steele, Lea, Flood, "Fast splittable pseudorandom
 *                         number generators", OOPSLA 2014.
 *   bounded             - Lemire, "Fast random integer generation in an
 *                         interval", 2019 (multiply-shift, no division).
 *   feistel + cycle walk- Black & Rogaway, "Ciphers with arbitrary finite
 *                         domains", 2002 (bijection on [0, n)).
 *   zipf                - inverse-CDF sampling over a host-built table.
 */
#ifndef EJ_GEN_H
#define EJ_GEN_H

#include <stdint.h>

#if defined(__CUDACC__)
#define EJ_HD __host__ __device__ __forceinline__
#else
#define EJ_HD static inline
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* generator kinds */
enum {
  EJ_GEN_PERM = 0,    /* distinct keys: val = permute(kseed, domain, shuffle(i) / dup) */
  EJ_GEN_UNIFORM = 1, /* val = val_base + uniform in [0, domain) */
  EJ_GEN_ZIPF = 2     /* with prob absent_permille/1000: absent_base + uniform[0,domain);
                         else permute(kseed, domain, rank), rank ~ Zipf(s) over [0,domain)
                         (s == 0: uniform rank) */
};

typedef struct ej_gen_spec {
  uint32_t kind;            /* EJ_GEN_* */
  uint32_t domain;          /* key domain size (ranks / distinct keys) */
  uint64_t seed;            /* per-relation row stream seed */
  uint64_t kseed;           /* key permutation seed, shared by the relations of one join */
  uint64_t n;               /* rows */
  uint32_t dup;             /* EJ_GEN_PERM: copies of each distinct key (>= 1) */
  uint32_t absent_permille; /* EJ_GEN_ZIPF: share of rows drawn from the absent range */
  int32_t val_base;         /* EJ_GEN_UNIFORM: added to the value */
  int32_t absent_base;      /* EJ_GEN_ZIPF: first key of the absent range */
  int32_t key_base;         /* TUPLE.key = key_base + row index */
  uint32_t reserved;
  double zipf_s;            /* EJ_GEN_ZIPF exponent; 0 = uniform ranks */
  const double* cdf;        /* EJ_GEN_ZIPF with s > 0: cdf[domain], cdf[domain-1] == 1.0;
                               host pointer for host generation, device pointer on device */
} ej_gen_spec;

EJ_HD uint64_t ej_splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* independent streams of one seed: value i of stream s */
EJ_HD uint64_t ej_rand(uint64_t seed, uint64_t stream, uint64_t i) {
  return ej_splitmix64(ej_splitmix64(seed ^ ej_splitmix64(stream + 0x5851F42D4C957F2Dull)) + i);
}

/* uniform integer in [0, n) from 32 random bits (multiply-shift) */
EJ_HD uint32_t ej_bounded(uint64_t r, uint32_t n) {
  return (uint32_t)(((r >> 32) * (uint64_t)n) >> 32);
}

/* uniform double in [0, 1) with 53 random bits */
EJ_HD double ej_unit(uint64_t r) { return (double)(r >> 11) * (1.0 / 9007199254740992.0); }

/* smallest h with 2h >= bits(n-1) (so a balanced Feistel network covers [0, n)) */
EJ_HD uint32_t ej_feistel_half_bits(uint32_t n) {
  uint32_t b = 0;
  uint32_t m = n - 1u;
  while (m) { b++; m >>= 1; }
  return (b + 1u) / 2u;
}

/* 4-round balanced Feistel network: a bijection on [0, 2^(2*half)) */
EJ_HD uint32_t ej_feistel(uint64_t kseed, uint32_t half, uint32_t x) {
  uint32_t mask = (half >= 32u) ? 0xFFFFFFFFu : ((1u << half) - 1u);
  uint32_t l = (x >> half) & mask;
  uint32_t r = x & mask;
  for (uint32_t round = 0; round < 4u; round++) {
    uint32_t f = (uint32_t)ej_splitmix64(kseed + 0x632BE59BD9B4E019ull * (round + 1u) + r) & mask;
    uint32_t t = r;
    r = l ^ f;
    l = t;
  }
  return (l << half) | r;
}

/* bijection on [0, n) by cycle walking the Feistel network (n >= 1, x < n) */
EJ_HD uint32_t ej_permute(uint64_t kseed, uint32_t n, uint32_t x) {
  if (n <= 1u) return 0u;
  uint32_t half = ej_feistel_half_bits(n);
  uint32_t y = ej_feistel(kseed, half, x);
  while (y >= n) y = ej_feistel(kseed, half, y);
  return y;
}

/* first rank k with u < cdf[k] (cdf ascending, cdf[n-1] == 1.0) */
EJ_HD uint32_t ej_zipf_rank(const double* cdf, uint32_t n, double u) {
  uint32_t lo = 0, hi = n - 1u;
  while (lo < hi) {
    uint32_t mid = lo + ((hi - lo) >> 1);
    if (u < cdf[mid]) hi = mid; else lo = mid + 1u;
  }
  return lo;
}

/* join attribute of row i */
EJ_HD int32_t ej_gen_val(const ej_gen_spec* sp, uint64_t i) {
  if (sp->kind == EJ_GEN_PERM) {
    uint32_t dup = sp->dup ? sp->dup : 1u;
    uint32_t pos = (uint32_t)i;
    if (dup > 1u) pos = ej_permute(sp->seed, (uint32_t)sp->n, pos);
    return (int32_t)ej_permute(sp->kseed, sp->domain, pos / dup);
  }
  if (sp->kind == EJ_GEN_UNIFORM) {
    return (int32_t)((uint32_t)sp->val_base + ej_bounded(ej_rand(sp->seed, 0, i), sp->domain));
  }
  /* EJ_GEN_ZIPF */
  uint64_t r0 = ej_rand(sp->seed, 1, i);
  if (ej_bounded(r0, 1000u) < sp->absent_permille) {
    return (int32_t)((uint32_t)sp->absent_base + ej_bounded(ej_rand(sp->seed, 2, i), sp->domain));
  }
  uint64_t r1 = ej_rand(sp->seed, 3, i);
  uint32_t rank;
  if (sp->zipf_s == 0.0 || sp->cdf == 0) rank = ej_bounded(r1, sp->domain);
  else rank = ej_zipf_rank(sp->cdf, sp->domain, ej_unit(r1));
  return (int32_t)ej_permute(sp->kseed, sp->domain, rank);
}

#ifdef __cplusplus
}
#endif

#endif /* EJ_GEN_H */
