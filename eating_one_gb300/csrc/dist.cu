// dist.cu - distance (non-equi) nested-loop join over all |R| x |S| point pairs.
//
// Reference: the 2-D GPU join joins/blockJoin_gpu/complex_block/dire_join
// (eval, count and join kernels, join_gpu.cu:12-130; VAL_NUM 2, tuple.h:18-30)
// and the CPU joins joins/CPU_JOIN/3d_cpu/nestLoopJoin.cc (eval :73-84, loop
// :86-101; VAL_NUM 3) and joins/blockJoin_gpu/complex_block/2d_cpu.  A left
// point l (from S) and a right point r (from R) match when, in IEEE double with
// every operation rounded on its own,
//   temp = 0; for each dimension i: t = r.val[i] - l.val[i]; temp += t * t;
//   temp < radius * radius                   (radius = DISTANCE = 1 there).
//
// Screen.  Every point p carries x = p.val[0] rounded to nearest float
// (+-inf beyond float range, NaN for NaN).  A CTA compares its R points with
// one tile of S points at a time and rejects a pair when
//   |round(x_s - x_r)| > W,   W = (|radius| + 2^-24 (M_S + M_R) + 2^-148)(1 + 2^-23),
// everything rounded up, with M_S and M_R the largest |x| of the S tile and
// of the CTA's R points.  Rounding a double to float moves it by at most
// 2^-24 |x| + 2^-149 and the float subtraction by a factor 1 + 2^-24, so a
// rejected pair has |r.val[0] - l.val[0]| >= |radius| in exact arithmetic;
// its rounded difference and square are then at least |radius| and radius^2
// (rounding is monotone), the other dimensions' squares only add, and the
// pair cannot match.  A NaN difference is rejected too: its double difference
// is NaN (or inf - inf) and never matches.  Points beyond float range make
// M infinite and W infinite (their x is clamped to +-FLT_MAX in the loop), a
// NaN radius makes W NaN and rejects everything, as radius^2 = NaN matches
// nothing.  Pairs that pass get the exact predicate (__dsub_rn, __dmul_rn,
// __dadd_rn in the reference's order: no fused multiply-add), so the matches
// are the reference's, bit for bit.
//
// Layout: each CTA holds x of 16384 R points in registers (64 per thread,
// packed in pairs; 160 registers, one CTA per SM, which the pure arithmetic
// loop needs no more than); the x of S stream through shared memory in
// 4096-point tiles.  Per S point a
// thread takes the smallest (x_s - x_r)^2 over its 16 R points with packed
// two-lane subtractions and products and three-input minima (three
// instructions per two pairs) and compares it with W^2 once; only then are
// the slots tested one by one.  Matches take an output slot from an atomic cursor (the row order is
// not deterministic, the row multiset is); count-only mode sums per-thread
// counters.
#include <float.h>
#include <math.h>

#include <algorithm>
#include <type_traits>

#include "ej_device.cuh"
#include "ej_entry.h"

namespace {

constexpr int DJ_THREADS = 256;
constexpr int DJ_RK = 64;                      // R points per thread
constexpr int DJ_RCHUNK = DJ_THREADS * DJ_RK;  // R points per CTA
constexpr int DJ_STILE = 4096;                 // S screen values per shared-memory tile (16 KB)

template <int D>
struct Point {
  int32_t id;
  double val[D];
};
static_assert(sizeof(Point<2>) == sizeof(ej_point2) && sizeof(Point<3>) == sizeof(ej_point3), "point layouts");

// dimension 0 of every point rounded to nearest float
template <int D>
__global__ void dist_screen_kernel(const Point<D>* __restrict__ P, uint64_t n, float* __restrict__ x) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    x[i] = __double2float_rn(P[i].val[0]);
}

// the loop's operand: +-inf clamped to +-FLT_MAX (their tiles have W = inf), NaN kept
__device__ __forceinline__ float dist_clamp(float x) {
  return fabsf(x) == INFINITY ? copysignf(FLT_MAX, x) : x;
}

// the screening bound W of the header comment, rounded up
__device__ __forceinline__ float dist_bound(float rad_up, float m_s, float m_r) {
  const float err = __fmul_ru(0x1p-24f, __fadd_ru(m_s, m_r));
  return __fmul_ru(__fadd_ru(__fadd_ru(rad_up, err), 0x1p-148f), 1.0f + 0x1p-23f);
}

// two float differences in one instruction (Blackwell packed f32x2):
// (x - lo(r), x - hi(r)) for x2 = (x, x), each rounded to nearest like __fsub_rn
__device__ __forceinline__ unsigned long long dist_sub2(unsigned long long x2, unsigned long long r) {
  unsigned long long d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(x2), "l"(r));
  return d;
}

// minimum of three floats in one instruction; NaN operands are ignored
__device__ __forceinline__ float dist_min3(float a, float b, float c) {
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

__device__ __forceinline__ unsigned long long dist_pack(float lo, float hi) {
  return (unsigned long long)__float_as_uint(hi) << 32 | __float_as_uint(lo);
}

// block-wide maximum (NaN inputs ignored); every thread gets it
__device__ __forceinline__ float dist_block_max(float v, float* red) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  float m = red[0];
#pragma unroll
  for (int w = 1; w < DJ_THREADS / 32; w++) m = fmaxf(m, red[w]);
  __syncthreads();
  return m;
}

// the reference's predicate, operation by operation
template <int D>
__device__ __forceinline__ bool dist_match(const Point<D>& r, const Point<D>& l, double r2) {
  double temp = 0.0;
#pragma unroll
  for (int i = 0; i < D; i++) {
    const double t = __dsub_rn(r.val[i], l.val[i]);
    temp = __dadd_rn(temp, __dmul_rn(t, t));
  }
  return temp < r2;
}

// result rows as the reference lays them out, written as whole 8-byte words
// (padding zero): dims 2 {lid, lval[2], rid, rval[2]}, dims 3 {lval[3], rval[3], lid, rid}
__device__ __forceinline__ void dist_store(ej_point_result2* out, uint64_t pos, const Point<2>& l,
                                           const Point<2>& r) {
  unsigned long long* w = reinterpret_cast<unsigned long long*>(out + pos);
  w[0] = (uint32_t)l.id;
  w[1] = __double_as_longlong(l.val[0]);
  w[2] = __double_as_longlong(l.val[1]);
  w[3] = (uint32_t)r.id;
  w[4] = __double_as_longlong(r.val[0]);
  w[5] = __double_as_longlong(r.val[1]);
}
__device__ __forceinline__ void dist_store(ej_point_result3* out, uint64_t pos, const Point<3>& l,
                                           const Point<3>& r) {
  unsigned long long* w = reinterpret_cast<unsigned long long*>(out + pos);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    w[i] = __double_as_longlong(l.val[i]);
    w[3 + i] = __double_as_longlong(r.val[i]);
  }
  w[6] = (unsigned long long)(uint32_t)l.id | (unsigned long long)(uint32_t)r.id << 32;
}

template <int D>
struct RowOf;
template <>
struct RowOf<2> {
  using type = ej_point_result2;
};
template <>
struct RowOf<3> {
  using type = ej_point_result3;
};

template <int D, bool COUNT_ONLY>
__global__ void __launch_bounds__(DJ_THREADS)
dist_kernel(const Point<D>* __restrict__ R, const float* __restrict__ rx_all, uint64_t nR,
            const Point<D>* __restrict__ S, const float* __restrict__ sx_all, uint64_t nS, uint64_t s_per_cta,
            float rad_up, double r2, typename RowOf<D>::type* __restrict__ out, uint64_t cap,
            unsigned long long* cursor) {
  __shared__ float tile[DJ_STILE];
  __shared__ float red[DJ_THREADS / 32];
  __shared__ unsigned long long warp_tmp[DJ_THREADS / 32 + 1];
  const uint64_t rbase = (uint64_t)blockIdx.x * DJ_RCHUNK;
  // the thread's R screen values in pairs, for the packed subtraction
  unsigned long long rx2[DJ_RK / 2];
  using Mask = typename std::conditional<(DJ_RK > 32), unsigned long long, uint32_t>::type;
  Mask valid = 0;
  float m = 0.0f;
#pragma unroll
  for (int k = 0; k < DJ_RK; k += 2) {
    float x[2];
#pragma unroll
    for (int e = 0; e < 2; e++) {
      const uint64_t ri = rbase + (uint64_t)(k + e) * DJ_THREADS + threadIdx.x;
      x[e] = __int_as_float(0x7fc00000);  // slots past nR: NaN, never a candidate
      if (ri < nR) {
        x[e] = __ldg(rx_all + ri);
        valid |= (Mask)1 << (k + e);
      }
      m = fmaxf(m, fabsf(x[e]));
    }
    rx2[k / 2] = dist_pack(dist_clamp(x[0]), dist_clamp(x[1]));
  }
  const float m_r = dist_block_max(m, red);
  const uint64_t s_begin = (uint64_t)blockIdx.y * s_per_cta;
  const uint64_t s_end = min(nS, s_begin + s_per_cta);
  unsigned long long local = 0;
  for (uint64_t t0 = s_begin; t0 < s_end; t0 += DJ_STILE) {
    const uint32_t n = (uint32_t)min((uint64_t)DJ_STILE, s_end - t0);
    __syncthreads();  // the previous tile is no longer read
    float ms = 0.0f;
    for (uint32_t k = threadIdx.x; k < n; k += DJ_THREADS) {
      const float x = __ldcs(sx_all + t0 + k);
      ms = fmaxf(ms, fabsf(x));
      tile[k] = dist_clamp(x);
    }
    const float W = dist_bound(rad_up, dist_block_max(ms, red), m_r);  // its barriers publish the tile
    if (!valid) continue;
    for (uint32_t k = 0; k < n; k++) {
      const float xs = tile[k];
      // the smallest |xs - x_r| over the thread's R points (NaN differences
      // ignored): two differences per instruction, two minima per instruction
      const unsigned long long xs2 = dist_pack(xs, xs);
      float dmin = INFINITY;
#pragma unroll
      for (int j = 0; j < DJ_RK / 2; j++) {
        const unsigned long long d = dist_sub2(xs2, rx2[j]);
        dmin = dist_min3(dmin, fabsf(__uint_as_float((uint32_t)d)), fabsf(__uint_as_float((uint32_t)(d >> 32))));
      }
      if (!(dmin <= W)) continue;
      // the rare path: candidate slots as a bit mask (static indices keep rx2 in registers)
      Mask mask = 0;
#pragma unroll
      for (int j = 0; j < DJ_RK / 2; j++) {
        const unsigned long long d = dist_sub2(xs2, rx2[j]);
        mask |= (Mask)(fabsf(__uint_as_float((uint32_t)d)) <= W) << (2 * j);
        mask |= (Mask)(fabsf(__uint_as_float((uint32_t)(d >> 32))) <= W) << (2 * j + 1);
      }
      mask &= valid;
      const Point<D> l = S[t0 + k];
      for (; mask; mask &= mask - 1) {
        const int j = DJ_RK > 32 ? __ffsll((long long)mask) - 1 : __ffs((int)mask) - 1;
        const Point<D> r = R[rbase + (uint64_t)j * DJ_THREADS + threadIdx.x];
        if (!dist_match<D>(r, l, r2)) continue;
        if (COUNT_ONLY) {
          local++;
          continue;
        }
        const unsigned long long pos = atomicAdd(cursor, 1ull);
        if (pos < cap) dist_store(out, pos, l, r);
      }
    }
  }
  if (COUNT_ONLY) {
    unsigned long long total;
    ej_block_exclusive_sum<DJ_THREADS, unsigned long long>(local, warp_tmp, &total);
    if (threadIdx.x == 0 && total) atomicAdd(cursor, total);
  }
}

// |radius| rounded up to float (infinite beyond float range, NaN for NaN)
float dist_radius_up(double radius) {
  const double a = fabs(radius);
  if (a != a) return NAN;
  if (a > (double)FLT_MAX) return INFINITY;
  float f = (float)a;
  if ((double)f < a) f = nextafterf(f, INFINITY);
  return f;
}

template <int D>
ej_status dist_run(ej_handle* h, const void* Rv, uint64_t nR, const void* Sv, uint64_t nS, double radius, void* outv,
                   uint64_t cap, bool count_only) {
  const Point<D>* R = static_cast<const Point<D>*>(Rv);
  const Point<D>* S = static_cast<const Point<D>*>(Sv);
  EJ_CUDA(h, cudaMemsetAsync(h->d_words, 0, sizeof(unsigned long long), h->stream));
  if (nR == 0 || nS == 0) return EJ_OK;
  const uint64_t rchunks = (nR + DJ_RCHUNK - 1) / DJ_RCHUNK;
  if (rchunks > 0x7FFFFFFFull) return ej_fail(h, EJ_ERR_TOO_LARGE, "R too large for the nested loop");
  ej_plan_bytes p;
  const size_t roff = p.add(nR * sizeof(float)), soff = p.add(nS * sizeof(float));
  EJ_TRY(ej_arena_reserve(h, p.bytes));
  float* rx = reinterpret_cast<float*>(ej_arena_at(h, roff));
  float* sx = reinterpret_cast<float*>(ej_arena_at(h, soff));
  ej_phase_begin(h);
  const unsigned blocks = (unsigned)std::min<uint64_t>((std::max(nR, nS) + 255) / 256, (uint64_t)h->num_sms * 8);
  dist_screen_kernel<D><<<blocks, 256, 0, h->stream>>>(R, nR, rx);
  EJ_TRY(ej_check_launch(h, "dist_screen_kernel"));
  dist_screen_kernel<D><<<blocks, 256, 0, h->stream>>>(S, nS, sx);
  EJ_TRY(ej_check_launch(h, "dist_screen_kernel"));
  // the screen values are the build phase; the nested loop is recorded as the write phase
  for (int k = 1; k < EJ_PHASES; k++) ej_phase_mark(h, k);
  // about four CTAs per SM; each CTA's S range a whole number of tiles
  const uint64_t want = (uint64_t)h->num_sms * 4;
  const uint64_t stiles = (nS + DJ_STILE - 1) / DJ_STILE;
  uint64_t splits = (want + rchunks - 1) / rchunks;
  splits = std::max<uint64_t>(1, std::min<uint64_t>(std::min<uint64_t>(splits, stiles), 65535));
  const uint64_t s_per_cta = ((stiles + splits - 1) / splits) * DJ_STILE;
  splits = (nS + s_per_cta - 1) / s_per_cta;
  const dim3 grid((unsigned)rchunks, (unsigned)splits);
  const float rad_up = dist_radius_up(radius);
  const double r2 = radius * radius;
  using Row = typename RowOf<D>::type;
  if (count_only)
    dist_kernel<D, true><<<grid, DJ_THREADS, 0, h->stream>>>(R, rx, nR, S, sx, nS, s_per_cta, rad_up, r2, nullptr,
                                                             0, h->d_words);
  else
    dist_kernel<D, false><<<grid, DJ_THREADS, 0, h->stream>>>(R, rx, nR, S, sx, nS, s_per_cta, rad_up, r2,
                                                              static_cast<Row*>(outv), cap, h->d_words);
  EJ_TRY(ej_check_launch(h, "dist_kernel"));
  ej_phase_mark(h, EJ_PHASES);
  return EJ_OK;
}

ej_status dist_entry(ej_handle* h, uint32_t dims, const void* R, uint64_t nR, const void* S, uint64_t nS,
                     double radius, void* out, uint64_t cap, uint64_t* out_count, bool count_only) {
  EJ_TRY(ej_begin(h));
  if (dims != 2 && dims != 3) return ej_fail(h, EJ_ERR_INVALID, "dims must be 2 or 3 (got %u)", dims);
  if (!out_count) return ej_fail(h, EJ_ERR_INVALID, "out_count is NULL");
  if ((nR && !R) || (nS && !S)) return ej_fail(h, EJ_ERR_INVALID, "point array is NULL");
  if (!count_only && cap && !out)
    return ej_fail(h, EJ_ERR_INVALID, "out is NULL with capacity %llu", (unsigned long long)cap);
  if (((uintptr_t)R | (uintptr_t)S | (uintptr_t)out) % 8)
    return ej_fail(h, EJ_ERR_INVALID, "point and row arrays must be 8-byte aligned");
  EJ_TRY(dims == 2 ? dist_run<2>(h, R, nR, S, nS, radius, out, cap, count_only)
                   : dist_run<3>(h, R, nR, S, nS, radius, out, cap, count_only));
  uint64_t count = 0;
  EJ_TRY(ej_finish(h, &count));
  *out_count = count;
  return count_only ? EJ_OK : ej_capacity_result(h, count, cap);
}

}  // namespace

extern "C" ej_status ej_distance_join(ej_handle* h, uint32_t dims, const void* R, uint64_t nR, const void* S,
                                      uint64_t nS, double radius, void* out, uint64_t out_cap, uint64_t* out_count) {
  return dist_entry(h, dims, R, nR, S, nS, radius, out, out_cap, out_count, false);
}

extern "C" ej_status ej_distance_join_count(ej_handle* h, uint32_t dims, const void* R, uint64_t nR, const void* S,
                                            uint64_t nS, double radius, uint64_t* out_count) {
  return dist_entry(h, dims, R, nR, S, nS, radius, nullptr, 0, out_count, true);
}
