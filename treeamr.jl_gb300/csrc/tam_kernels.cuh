// Ghost-fill kernel templates for sm_103a, shared by the units that
// instantiate them: tam_kernels.cu (the plain launch, the solo groups, the
// self-tests) and tam_fused_*.cu (the fused launches, one element type and
// dimension a unit, compiled in parallel).
//
// One transfer item is one (target point, variable) of one transfer, and
// computes what the reference's transfer_kernel! computes
// (src/ghosts.jl:372-402):
//
//   dest[tidx, v, tblock] = scaled(acc, factors, v, fcol)
//   acc = +0 + src[base, v, sblock]                         a unit copy
//   acc = +0; for m_D .. for m_1: acc += ((w_1*w_2)*..*w_D) * src[base+m]
//
// in exactly that order, with no contraction into fused multiply-adds
// (src/ghosts.jl:58-118, 120-128, 363-370): the _rn intrinsics below are
// never contracted, whatever -fmad says.  So every result is bit-identical
// to a correctly rounded evaluation of the reference's expression.
//
// Two launch forms:
//   - plain: one launch per TransferGroup, one thread per item, as the
//     reference's device path (src/ghosts.jl:420-521);
//   - fused: one launch per stage over every group of the stage.  A warp
//     takes one Tile (a run of box points of one transfer) and every
//     variable of them; tiles are ordered by target block so the ghosts of
//     one block are written close together in time and their partial
//     sectors merge in L2 before they reach HBM.
#ifndef TAM_KERNELS_CUH
#define TAM_KERNELS_CUH

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <type_traits>

#include "tam_internal.h"

namespace tam {
namespace {

template <typename T>
struct Arith;
template <>
struct Arith<double> {
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
};
template <>
struct Arith<float> {
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
};

// The tensor-product stencil sum of one item.  `src` points at element
// (base_1, base_2, base_3) of the source block's variable; `w_d` at the
// target row's weight column.  P > 0: every dimension has order P (D of
// them); P == 0: orders from `o`.
template <typename T, int D, int P>
__device__ __forceinline__ T stencil_sum(const T *__restrict__ src, int64_t s2, int64_t s3,
                                         const T *__restrict__ w1, const T *__restrict__ w2,
                                         const T *__restrict__ w3, const int o[3]) {
  using A = Arith<T>;
  const int o1 = P > 0 ? P : o[0];
  const int o2 = D >= 2 ? (P > 0 ? P : o[1]) : 1;
  const int o3 = D >= 3 ? (P > 0 ? P : o[2]) : 1;
  T acc = T(0);
#pragma unroll
  for (int m3 = 0; m3 < o3; ++m3) {
    const T wt3 = D >= 3 ? __ldg(w3 + m3) : T(1);
#pragma unroll
    for (int m2 = 0; m2 < o2; ++m2) {
      const T wt2 = D >= 2 ? __ldg(w2 + m2) : T(1);
#pragma unroll
      for (int m1 = 0; m1 < o1; ++m1) {
        const T wt1 = __ldg(w1 + m1);
        T wp = wt1;
        if (D >= 2) wp = A::mul(wp, wt2);
        if (D >= 3) wp = A::mul(wp, wt3);
        acc = A::add(acc, A::mul(wp, src[m3 * s3 + m2 * s2 + m1]));
      }
    }
  }
  return acc;
}

template <typename T>
__device__ __forceinline__ T scaled(T acc, const T *__restrict__ factors, int v, int nvars,
                                    int fcol) {
  if (fcol == 0) return acc;
  using A = Arith<T>;
  return A::add(A::mul(acc, __ldg(factors + v + (int64_t)nvars * (fcol - 1))), T(0));
}

// The item at box point (i1, i2, i3) of transfer (tblock, sblock), every
// variable in [v0, v1).
template <typename T>
struct Args {
  const DevGroup *__restrict__ groups;
  const int32_t *__restrict__ tb;
  const int32_t *__restrict__ sb;
  const int32_t *__restrict__ srcstart;
  const T *__restrict__ weights;
  const int32_t *__restrict__ cls;
  const T *__restrict__ wtab;
  int int_mul;
  const Member *__restrict__ members;
  const int32_t *__restrict__ csingle;
  const int32_t *__restrict__ perm;
  int one_tap;
  int copy_points;
  const uint2 *__restrict__ wshort;
  int pair_vars;
  int copy_ctas;
  int soft_add;
};

template <typename T>
__host__ __device__ inline Args<T> typed(const SchedArgs &a) {
  return Args<T>{a.groups,  a.tb,      a.sb,   a.srcstart, (const T *)a.weights,
                 a.cls,     (const T *)a.wtab, a.int_mul, a.members, a.csingle,
                 a.perm,    a.one_tap, a.copy_points, (const uint2 *)a.wshort, a.pair_vars,
                 a.copy_ctas, a.soft_add};
}

struct Geom {
  int64_t toff;      // element offset of the target point, variable 0
  int64_t soff;      // element offset of the source window's first point, variable 0
  int64_t vstride;   // elements between variables of the target
  int64_t s2, s3;    // strides of dimensions 2 and 3 of the source
  int64_t svstride;  // elements between variables of the source (a staged window's own)
};

template <int D>
__device__ __forceinline__ Geom geometry(const DevGroup &g, int i1, int i2, int i3,
                                         int64_t tblock, int64_t sblock,
                                         const int32_t *__restrict__ srcstart, int nvars, int S1,
                                         int S2, int S3) {
  Geom o;
  o.s2 = S1;
  o.s3 = (int64_t)S1 * S2;
  o.vstride = o.s3 * S3;
  const int64_t bstride = o.vstride * nvars;
  const int b1 = __ldg(srcstart + g.ss[0] + i1) - 1;
  const int b2 = D >= 2 ? __ldg(srcstart + g.ss[1] + i2) - 1 : 0;
  const int b3 = D >= 3 ? __ldg(srcstart + g.ss[2] + i3) - 1 : 0;
  o.toff = tblock * bstride + (int64_t)(g.tf[0] + i1) +
           (D >= 2 ? (int64_t)(g.tf[1] + i2) * o.s2 : 0) +
           (D >= 3 ? (int64_t)(g.tf[2] + i3) * o.s3 : 0);
  o.soff = sblock * bstride + b1 + (int64_t)b2 * o.s2 + (int64_t)b3 * o.s3;
  o.svstride = o.vstride;
  return o;
}

// The geometry of an affine unit copy: its source rows from the group's
// first row and step, no srcstart load.
template <int D>
__device__ __forceinline__ Geom copy_geometry(const DevGroup &g, int i1, int i2, int i3,
                                              int64_t tblock, int64_t sblock, int nvars, int S1,
                                              int S2, int S3) {
  Geom o;
  o.s2 = S1;
  o.s3 = (int64_t)S1 * S2;
  o.vstride = o.s3 * S3;
  const int64_t bstride = o.vstride * nvars;
  const int b1 = g.cs0[0] + g.cstep[0] * i1;
  const int b2 = D >= 2 ? g.cs0[1] + g.cstep[1] * i2 : 0;
  const int b3 = D >= 3 ? g.cs0[2] + g.cstep[2] * i3 : 0;
  o.toff = tblock * bstride + (int64_t)(g.tf[0] + i1) +
           (D >= 2 ? (int64_t)(g.tf[1] + i2) * o.s2 : 0) +
           (D >= 3 ? (int64_t)(g.tf[2] + i3) * o.s3 : 0);
  o.soff = sblock * bstride + b1 + (int64_t)b2 * o.s2 + (int64_t)b3 * o.s3;
  o.svstride = o.vstride;
  return o;
}

// +0 + x without the floating-point pipe: x itself, except that -0 becomes
// +0 (IEEE round-to-nearest gives +0 for +0 + -0).  A NaN stays a NaN (its
// payload kept rather than made canonical; NaNs compare as one pattern).
// Used for the F64 copies, which would otherwise queue on the GB300's narrow
// FP64 pipe.
// The halves are taken by an opaque move: a test of the bit pattern for +-0
// is the same predicate as x == 0.0, which the compiler may otherwise turn
// into a floating-point compare on the FP64 pipe.
__device__ __forceinline__ double plus_zero(double x) {
  uint32_t lo, hi;
  asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "d"(x));
  const uint32_t zero = ((hi << 1) | lo) == 0u;  // +0 or -0
  double r;
  asm("mov.b64 %0, {%1, %2};" : "=d"(r) : "r"(lo), "r"(hi & ~(zero << 31)));
  return r;
}
__device__ __forceinline__ float plus_zero(float x) { return __fadd_rn(0.0f, x); }

// RN(w * u) on the integer pipe, for a weight w whose significand has at
// most 24 significant bits: wm is that significand as an integer in
// [2^23, 2^24), we its unbiased exponent and wsign its sign bit (bit 31).
// The exact product of the 53-bit and 24-bit significands (at most 77 bits)
// is formed from two 32x32 multiplies, rounded to nearest-even at bit
// 23 or 24, and packed; a zero, subnormal, infinite or NaN u, and a result
// outside the normal range, take the hardware multiply instead.  Bit-identical
// to __dmul_rn(w, u) on every input (checked by tam_selftest).
__device__ __forceinline__ double mul_short(double w, uint32_t wm, int we, uint32_t wsign,
                                            double u) {
  const uint32_t uhi = (uint32_t)__double2hiint(u);
  const uint32_t ulo = (uint32_t)__double2loint(u);
  const int eu = (int)((uhi >> 20) & 0x7FF);
  const uint32_t mh = (uhi & 0xFFFFFu) | 0x100000u;
  const uint64_t t0 = (uint64_t)ulo * wm;                    // < 2^56
  const uint64_t t1 = (uint64_t)mh * wm;                     // < 2^45
  const uint32_t p0 = (uint32_t)t0;
  const uint64_t mid = (t0 >> 32) + (uint32_t)t1;
  const uint32_t p1 = (uint32_t)mid;
  const uint32_t p2 = (uint32_t)(t1 >> 32) + (uint32_t)(mid >> 32);  // < 2^13
  const uint32_t top = p2 >> 12;                             // the product has 77 bits
  const uint32_t s = 23u + top;
  const uint32_t lo = __funnelshift_r(p0, p1, s);
  const uint32_t hi = __funnelshift_r(p1, p2, s);            // < 2^21
  const uint32_t guard = (p0 >> (s - 1u)) & 1u;
  const uint32_t sticky = (p0 & ((1u << (s - 1u)) - 1u)) != 0u;
  const uint32_t inc = guard & (sticky | (lo & 1u));
  uint64_t m = (((uint64_t)hi << 32) | lo) + inc;
  int E = eu + we + (int)top;
  if (m >> 53) {  // rounded up to 2^53
    m >>= 1;
    E += 1;
  }
  if ((unsigned)(eu - 1) >= 2046u || (unsigned)(E - 1) >= 2046u) return __dmul_rn(w, u);
  const uint32_t rhi = ((uhi & 0x80000000u) ^ wsign) | ((uint32_t)E << 20) |
                       ((uint32_t)(m >> 32) & 0xFFFFFu);
  return __hiloint2double((int)rhi, (int)(uint32_t)m);
}

// The same multiply without the branch: `bad` is set where the fast path
// does not apply, and the caller recomputes those points on the FP64 pipe.
__device__ __forceinline__ double mul_short_flag(uint32_t wm, int we, uint32_t wsign, double u,
                                                 bool &bad) {
  const uint32_t uhi = (uint32_t)__double2hiint(u);
  const uint32_t ulo = (uint32_t)__double2loint(u);
  const int eu = (int)((uhi >> 20) & 0x7FF);
  const uint32_t mh = (uhi & 0xFFFFFu) | 0x100000u;
  const uint64_t t0 = (uint64_t)ulo * wm;
  const uint64_t t1 = (uint64_t)mh * wm;
  const uint32_t p0 = (uint32_t)t0;
  const uint64_t mid = (t0 >> 32) + (uint32_t)t1;
  const uint32_t p1 = (uint32_t)mid;
  const uint32_t p2 = (uint32_t)(t1 >> 32) + (uint32_t)(mid >> 32);
  const uint32_t top = p2 >> 12;
  const uint32_t s = 23u + top;
  const uint32_t lo = __funnelshift_r(p0, p1, s);
  const uint32_t hi = __funnelshift_r(p1, p2, s);
  const uint32_t guard = (p0 >> (s - 1u)) & 1u;
  const uint32_t sticky = (p0 & ((1u << (s - 1u)) - 1u)) != 0u;
  const uint32_t inc = guard & (sticky | (lo & 1u));
  const uint64_t m0 = (((uint64_t)hi << 32) | lo) + inc;
  const uint32_t carry = (uint32_t)(m0 >> 53);
  const uint64_t m = m0 >> carry;
  const int E = eu + we + (int)top + (int)carry;
  bad |= ((unsigned)(eu - 1) >= 2046u) | ((unsigned)(E - 1) >= 2046u);
  const uint32_t rhi = ((uhi & 0x80000000u) ^ wsign) | ((uint32_t)E << 20) |
                       ((uint32_t)(m >> 32) & 0xFFFFFu);
  return __hiloint2double((int)rhi, (int)(uint32_t)m);
}

// RN(w * u) on the integer pipe for any weight: the 106-bit product of the
// two 53-bit significands from four 32 x 32 multiplies (the high words have
// 21 bits), its top 53 bits rounded to nearest-even on the next bit and the
// rest.  `bad` is set where w or u is zero, subnormal, infinite or NaN, or
// the result leaves the normal range; the caller sums the point again on
// the FP64 pipe.  Bit-identical to __dmul_rn(w, u) wherever `bad` stays
// clear (checked by tam_selftest).
__device__ __forceinline__ double mul_full(double w, double u, bool &bad) {
  constexpr uint64_t kFrac = 0x000FFFFFFFFFFFFFull;
  const uint64_t bw = (uint64_t)__double_as_longlong(w);
  const uint64_t bu = (uint64_t)__double_as_longlong(u);
  const int ew = (int)((bw >> 52) & 0x7FF), eu = (int)((bu >> 52) & 0x7FF);
  const uint64_t mw = (bw & kFrac) | (1ull << 52), mu = (bu & kFrac) | (1ull << 52);
  const uint32_t wl = (uint32_t)mw, wh = (uint32_t)(mw >> 32);
  const uint32_t ul = (uint32_t)mu, uh = (uint32_t)(mu >> 32);
  const uint64_t ll = (uint64_t)wl * ul;
  const uint64_t mid = (uint64_t)wh * ul + (uint64_t)wl * uh;  // < 2^54
  const uint64_t lo = ll + (mid << 32);
  const uint64_t hi = (uint64_t)wh * uh + (mid >> 32) + (lo < ll);  // the product: hi 2^64 + lo
  const int t = (int)(hi >> 41);  // 1: the product has 106 bits, 0: 105
  const int sh = 52 + t;
  uint64_t m = (hi << (64 - sh)) | (lo >> sh);
  const uint64_t guard = (lo >> (sh - 1)) & 1u;
  const uint64_t sticky = (lo & ((1ull << (sh - 1)) - 1)) != 0;
  m += guard & (sticky | (m & 1u));
  int E = ew + eu - 1023 + t;
  if (m >> 53) {  // rounded up to the next power of two
    m >>= 1;
    E += 1;
  }
  bad |= ((unsigned)(ew - 1) >= 2046u) | ((unsigned)(eu - 1) >= 2046u) |
         ((unsigned)(E - 1) >= 2046u);
  return __longlong_as_double((long long)(((bw ^ bu) & 0x8000000000000000ull) |
                                          ((uint64_t)(E & 0x7FF) << 52) | (m & kFrac)));
}

// RN(a + b) on the integer pipe: the textbook IEEE adder.  The operands in
// order of magnitude, the smaller one's significand shifted to the larger's
// exponent with three extra bits (guard, round and sticky), added or
// subtracted, normalised (a carry one place right, a cancellation any number
// left) and rounded to nearest-even on the extra bits; three extra bits
// round every sum and difference correctly.  For the running sum `a` of a
// stencil and a product `b` of the integer-pipe multiply (normal, nonzero,
// finite).  A zero `a` gives b exactly; `bad` is set where `a` is
// subnormal, infinite or NaN or the result is not a normal number (the
// caller sums the point again on the FP64 pipe).  Bit-identical to
// __dadd_rn(a, b) wherever `bad` stays clear (checked by tam_selftest).
__device__ __forceinline__ double add_soft(double a, double b, bool &bad) {
  constexpr uint64_t kMag = 0x7FFFFFFFFFFFFFFFull, kFrac = 0x000FFFFFFFFFFFFFull;
  const uint64_t ua = (uint64_t)__double_as_longlong(a);
  const uint64_t ub = (uint64_t)__double_as_longlong(b);
  const bool swap = (ub & kMag) > (ua & kMag);
  const uint64_t x = swap ? ub : ua, y = swap ? ua : ub;  // |x| >= |y|
  const int ex = (int)((x >> 52) & 0x7FF), ey = (int)((y >> 52) & 0x7FF);
  if ((y & kMag) == 0) return __longlong_as_double((long long)x);  // a zero: b itself
  bad |= (ex == 0x7FF) | (ey == 0);
  const uint64_t mx = ((x & kFrac) | (1ull << 52)) << 3;  // bits 55 .. 3, 3 extra
  const uint64_t my = ((y & kFrac) | (1ull << 52)) << 3;
  const int d = ex - ey;
  uint64_t yd;
  if (d == 0)
    yd = my;
  else if (d < 56)
    yd = (my >> d) | (uint64_t)((my << (64 - d)) != 0);  // sticky
  else
    yd = 1;  // below every kept bit: sticky only
  int e = ex;
  uint64_t s;
  if (((ua ^ ub) >> 63) == 0) {
    s = mx + yd;
    if (s >> 56) {  // a carry: one place right, the lost bit kept sticky
      s = (s >> 1) | (s & 1);
      e += 1;
    }
  } else {
    s = mx - yd;
    if (s == 0) return 0.0;  // exact cancellation: +0 in round-to-nearest
    const int sh = __clzll((long long)s) - 8;  // bring the top bit to bit 55
    s <<= sh;
    e -= sh;
  }
  uint64_t m = s >> 3;
  const uint32_t low = (uint32_t)s & 7u;
  m += (low > 4u) | ((low == 4u) & (uint32_t)m & 1u);
  if (m >> 53) {  // rounded up to the next power of two
    m >>= 1;
    e += 1;
  }
  bad |= (e <= 0) | (e >= 0x7FF);
  return __longlong_as_double(
      (long long)((x & 0x8000000000000000ull) | ((uint64_t)(e & 0x7FF) << 52) | (m & kFrac)));
}

// The parts of a weight mul_short takes.
struct ShortW {
  double w;
  uint32_t wm, wsign;
  int we;
};

// The same parts from the table of them built at upload (short_weights):
// {significand, sign | (exponent + 8192)}.
__device__ __forceinline__ ShortW unpack_short(uint2 q) {
  ShortW r;
  r.w = 0.0;
  r.wm = q.x;
  r.wsign = q.y & 0x80000000u;
  r.we = (int)(q.y & 0x7FFFFFFFu) - 8192;
  return r;
}
__device__ __forceinline__ ShortW short_weight(double w) {
  const uint32_t whi = (uint32_t)__double2hiint(w);
  const uint32_t wlo = (uint32_t)__double2loint(w);
  ShortW r;
  r.w = w;
  r.wm = (((whi & 0xFFFFFu) | 0x100000u) << 3) | (wlo >> 29);
  // a zero weight gets an exponent no datum can bring into range, so the
  // multiply flags it and the point is recomputed on the FP64 pipe
  const int ew = (int)((whi >> 20) & 0x7FF);
  r.we = ew == 0 ? -4096 : ew - 1023;
  r.wsign = whi & 0x80000000u;
  return r;
}

// Within one stage no point is both read and written (targets are ghosts or
// secondaries, sources points the stage does not write), so the kernels read
// `work` through `src` and write it through `dst`, both restrict-qualified:
// the loads of several points and variables can be in flight together.

// Unit copies of every variable of NP points: +0 + x (src/ghosts.jl:127-128),
// all loads of a chunk issued before its stores; fac[p] is point p's factor
// column (FACTOR only), x * f + 0 (src/ghosts.jl:369-370).
template <typename T, int NP, int VC, bool FACTOR>
__device__ __forceinline__ void copy_point_vars(const T *const (&fac)[NP], const Geom (&o)[NP],
                                            const bool (&on)[NP], const T *__restrict__ src,
                                            T *__restrict__ dst, int vbegin, int vend) {
  for (int v0 = vbegin; v0 < vend; v0 += VC) {
    T x[NP][VC];
#pragma unroll
    for (int p = 0; p < NP; ++p)
#pragma unroll
      for (int j = 0; j < VC; ++j)
        if (on[p] && v0 + j < vend) x[p][j] = src[o[p].soff + (v0 + j) * o[p].vstride];
#pragma unroll
    for (int p = 0; p < NP; ++p)
#pragma unroll
      for (int j = 0; j < VC; ++j)
        if (on[p] && v0 + j < vend)
          dst[o[p].toff + (v0 + j) * o[p].vstride] =
              FACTOR ? Arith<T>::add(Arith<T>::mul(plus_zero(x[p][j]), __ldg(fac[p] + v0 + j)),
                                     T(0))
                     : plus_zero(x[p][j]);
  }
}

// The taps of dimension d a point takes: every row [0, P), or in the CPU
// form of the sum (src/ghosts.jl:28-56) only the row of the column's single
// nonzero weight.
__device__ __forceinline__ void tap_rows(const int32_t *__restrict__ single, int P, int &lo,
                                         int &hi) {
  const int k = __ldg(single);
  lo = k >= 0 ? k : 0;
  hi = k >= 0 ? k + 1 : P;
}

// A uniform order-P stencil through the group's product table: per tap one
// multiply and one add per variable, the weight product loaded once for
// VC variables at a time.  SKIP: the one-tap rows of `tap_rows`, which
// leave out only terms 0 * u, so the remaining products are summed in the
// same order (m_1 fastest) as the full nest.
template <typename T, int D, int P, int VC, bool SKIP, bool SOFT = false>
__device__ __forceinline__ void table_point(const DevGroup &g, int i1, int i2, int i3,
                                            const Geom &o, const Args<T> &a,
                                            const T *__restrict__ work, T *__restrict__ dst,
                                            const T *__restrict__ factors, int nvars,
                                            int vbegin, int vend) {
  using A = Arith<T>;
  constexpr int P2 = D >= 2 ? P : 1;
  constexpr int P3 = D >= 3 ? P : 1;
  constexpr int PD = P * P2 * P3;
  const int c1 = __ldg(a.cls + g.cls[0] + i1);
  const int c2 = D >= 2 ? __ldg(a.cls + g.cls[1] + i2) : 0;
  const int c3 = D >= 3 ? __ldg(a.cls + g.cls[2] + i3) : 0;
  const T *__restrict__ W = a.wtab + g.wtab + (int64_t)((c3 * g.C[1] + c2) * g.C[0] + c1) * PD;
  int lo1 = 0, hi1 = P, lo2 = 0, hi2 = P2, lo3 = 0, hi3 = P3;
  if (SKIP) {
    tap_rows(a.csingle + g.csingle[0] + i1, P, lo1, hi1);
    if (D >= 2) tap_rows(a.csingle + g.csingle[1] + i2, P, lo2, hi2);
    if (D >= 3) tap_rows(a.csingle + g.csingle[2] + i3, P, lo3, hi3);
  }
  if constexpr (sizeof(T) == 8) {
    if (g.shortw && a.int_mul) {
      // F64 with short weight products: the multiplies on the integer pipe,
      // only the adds on the FP64 pipe.
      for (int v0 = vbegin; v0 < vend; v0 += VC) {
        double acc[VC];
        const double *src = work + (o.soff + v0 * o.svstride);
        bool bad = false;
        const uint2 *__restrict__ WS =
            a.wshort + g.wtab + (int64_t)((c3 * g.C[1] + c2) * g.C[0] + c1) * PD;
        // FIRST: the sum's first term, 0 + p, is p itself (the fast path's
        // p is a nonzero finite number; anything else is flagged and summed
        // again below), so the sum costs one FP64 add a tap less
        // SOFT (TAM_OPT_SOFT_ADD): the last tap of every whole row adds on
        // the integer pipe (add_soft), beside the FP64 pipe's adds
        auto tap = [&](int m1, int m2, int m3, auto first, auto soft) {
          const ShortW sw = unpack_short(__ldg(WS + (m3 * P2 + m2) * P + m1));
          const int64_t off = m3 * o.s3 + m2 * o.s2 + m1;
#pragma unroll
          for (int j = 0; j < VC; ++j)
            if (v0 + j < vend) {
              const double p = mul_short_flag(sw.wm, sw.we, sw.wsign, src[off + j * o.svstride], bad);
              acc[j] = decltype(first)::value  ? p
                       : decltype(soft)::value ? add_soft(acc[j], p, bad)
                                               : __dadd_rn(acc[j], p);
            }
        };
        using Yes = std::true_type;
        using No = std::false_type;
        using Last = std::integral_constant<bool, SOFT>;
        auto row = [&](int m2, int m3, bool head) {
          if (SKIP && hi1 - lo1 == 1) {
            if (head)
              tap(lo1, m2, m3, Yes{}, No{});
            else
              tap(lo1, m2, m3, No{}, No{});
          } else {
            if (head)
              tap(0, m2, m3, Yes{}, No{});
            else
              tap(0, m2, m3, No{}, No{});
#pragma unroll
            for (int m1 = 1; m1 < P - 1; ++m1) tap(m1, m2, m3, No{}, No{});
            tap(P - 1, m2, m3, No{}, Last{});
          }
        };
        row(lo2, lo3, true);
#pragma unroll 1
        for (int m3 = lo3; m3 < hi3; ++m3) {
#pragma unroll 1
          for (int m2 = m3 == lo3 ? lo2 + 1 : lo2; m2 < hi2; ++m2) row(m2, m3, false);
        }
        if (bad) {  // a zero, subnormal or special datum, or an out-of-range product
#pragma unroll
          for (int j = 0; j < VC; ++j) acc[j] = 0.0;
#pragma unroll 1
          for (int m3 = lo3; m3 < hi3; ++m3)
#pragma unroll 1
            for (int m2 = lo2; m2 < hi2; ++m2)
#pragma unroll 1
              for (int m1 = lo1; m1 < hi1; ++m1) {
                const double w = __ldg(W + (m3 * P2 + m2) * P + m1);
                const int64_t off = m3 * o.s3 + m2 * o.s2 + m1;
#pragma unroll
                for (int j = 0; j < VC; ++j)
                  if (v0 + j < vend)
                    acc[j] = __dadd_rn(acc[j], __dmul_rn(w, src[off + j * o.svstride]));
              }
        }
#pragma unroll
        for (int j = 0; j < VC; ++j)
          if (v0 + j < vend)
            dst[o.toff + (v0 + j) * o.vstride] =
                scaled(acc[j], factors, v0 + j, nvars, g.factorcol);
      }
      return;
    }
    if (!g.shortw && a.int_mul) {
      // F64 with weight products of up to 53 significant bits (order 6): the
      // multiplies exact on the integer pipe all the same (mul_full), only
      // the adds on the FP64 pipe
      for (int v0 = vbegin; v0 < vend; v0 += VC) {
        double acc[VC];
        const double *src = work + (o.soff + v0 * o.svstride);
        bool bad = false;
        auto tap = [&](int m1, int m2, int m3, auto first) {
          const double w = __ldg(W + (m3 * P2 + m2) * P + m1);
          const int64_t off = m3 * o.s3 + m2 * o.s2 + m1;
#pragma unroll
          for (int j = 0; j < VC; ++j)
            if (v0 + j < vend) {
              const double p = mul_full(w, src[off + j * o.svstride], bad);
              acc[j] = decltype(first)::value ? p : __dadd_rn(acc[j], p);
            }
        };
        using Yes = std::true_type;
        using No = std::false_type;
        auto row = [&](int m2, int m3, bool head) {
          if (SKIP && hi1 - lo1 == 1) {
            if (head)
              tap(lo1, m2, m3, Yes{});
            else
              tap(lo1, m2, m3, No{});
          } else {
            if (head)
              tap(0, m2, m3, Yes{});
            else
              tap(0, m2, m3, No{});
#pragma unroll
            for (int m1 = 1; m1 < P; ++m1) tap(m1, m2, m3, No{});
          }
        };
        row(lo2, lo3, true);
#pragma unroll 1
        for (int m3 = lo3; m3 < hi3; ++m3) {
#pragma unroll 1
          for (int m2 = m3 == lo3 ? lo2 + 1 : lo2; m2 < hi2; ++m2) row(m2, m3, false);
        }
        if (bad) {  // a zero, subnormal or special datum or weight, or an out-of-range product
#pragma unroll
          for (int j = 0; j < VC; ++j) acc[j] = 0.0;
#pragma unroll 1
          for (int m3 = lo3; m3 < hi3; ++m3)
#pragma unroll 1
            for (int m2 = lo2; m2 < hi2; ++m2)
#pragma unroll 1
              for (int m1 = lo1; m1 < hi1; ++m1) {
                const double w = __ldg(W + (m3 * P2 + m2) * P + m1);
                const int64_t off = m3 * o.s3 + m2 * o.s2 + m1;
#pragma unroll
                for (int j = 0; j < VC; ++j)
                  if (v0 + j < vend)
                    acc[j] = __dadd_rn(acc[j], __dmul_rn(w, src[off + j * o.svstride]));
              }
        }
#pragma unroll
        for (int j = 0; j < VC; ++j)
          if (v0 + j < vend)
            dst[o.toff + (v0 + j) * o.vstride] =
                scaled(acc[j], factors, v0 + j, nvars, g.factorcol);
      }
      return;
    }
  }
  for (int v0 = vbegin; v0 < vend; v0 += VC) {
    T acc[VC];
#pragma unroll
    for (int j = 0; j < VC; ++j) acc[j] = T(0);
    const T *src = work + (o.soff + v0 * o.svstride);
    auto tap = [&](int m1, int m2, int m3) {
      const T w = __ldg(W + (m3 * P2 + m2) * P + m1);
      const int64_t off = m3 * o.s3 + m2 * o.s2 + m1;
#pragma unroll
      for (int j = 0; j < VC; ++j)
        if (v0 + j < vend) acc[j] = A::add(acc[j], A::mul(w, src[off + j * o.svstride]));
    };
    // Float64 rows one at a time (a whole unrolled nest holds more
    // registers than the stencil kernels' budget and spills)
#pragma unroll(SKIP || sizeof(T) == 8 ? 1 : P3)
    for (int m3 = lo3; m3 < hi3; ++m3) {
#pragma unroll(SKIP || sizeof(T) == 8 ? 1 : P2)
      for (int m2 = lo2; m2 < hi2; ++m2) {
        if (SKIP && hi1 - lo1 == 1) {
          tap(lo1, m2, m3);
        } else {
#pragma unroll
          for (int m1 = 0; m1 < P; ++m1) tap(m1, m2, m3);
        }
      }
    }
#pragma unroll
    for (int j = 0; j < VC; ++j)
      if (v0 + j < vend)
        dst[o.toff + (v0 + j) * o.vstride] = scaled(acc[j], factors, v0 + j, nvars, g.factorcol);
  }
}

// Mixed orders: the reference's nest with the product formed per tap; a
// dimension that takes one tap (SKIP) is the order-1 nest at that row.
template <typename T, int D>
__device__ __forceinline__ void generic_point(const DevGroup &g, int i1, int i2, int i3,
                                              const Geom &o, const Args<T> &a,
                                              const T *__restrict__ work, T *__restrict__ dst,
                                              const T *__restrict__ factors, int nvars,
                                              bool skip, int vbegin, int vend) {
  const T *w1 = a.weights + g.w[0] + (int64_t)g.order[0] * i1;
  const T *w2 = a.weights + g.w[1] + (int64_t)g.order[1] * i2;
  const T *w3 = a.weights + g.w[2] + (int64_t)g.order[2] * i3;
  int ord[3] = {g.order[0], g.order[1], g.order[2]};
  int64_t soff = o.soff;
  if (skip) {
    const int idx[3] = {i1, i2, i3};
    const T *w[3] = {w1, w2, w3};
    const int64_t stride[3] = {1, o.s2, o.s3};
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const int k = __ldg(a.csingle + g.csingle[d] + idx[d]);
      if (k >= 0) {
        w[d] += k;
        ord[d] = 1;
        soff += k * stride[d];
      }
    }
    w1 = w[0];
    w2 = w[1];
    w3 = w[2];
  }
  for (int v = vbegin; v < vend; ++v) {
    T acc = stencil_sum<T, D, 0>(work + (soff + v * o.svstride), o.s2, o.s3, w1, w2, w3, ord);
    dst[o.toff + v * o.vstride] = scaled(acc, factors, v, nvars, g.factorcol);
  }
}

template <typename T, int D, int P, int VC, bool SOFT = false>
__device__ __forceinline__ void table_dispatch(const DevGroup &g, int i1, int i2, int i3,
                                               const Geom &o, const Args<T> &a,
                                               const T *__restrict__ work, T *__restrict__ dst,
                                               const T *__restrict__ factors, int nvars,
                                               bool skip, int vbegin, int vend) {
  if (skip)
    table_point<T, D, P, VC, true, SOFT>(g, i1, i2, i3, o, a, work, dst, factors, nvars, vbegin,
                                         vend);
  else
    table_point<T, D, P, VC, false, SOFT>(g, i1, i2, i3, o, a, work, dst, factors, nvars, vbegin,
                                    vend);
}

// Variables [vbegin, vend) of one box point of one stencil transfer, by the
// group's class; `src` with `o` locates the source window (the array
// itself, or a window staged in shared memory).  PC = 4: the caller's
// groups are all of uniform order 4, and only that path is compiled (SOFT:
// with the integer-pipe add for a tap a row).
template <typename T, int D, int PC = 0, bool SOFT = false>
__device__ __forceinline__ void stencil_dispatch(const DevGroup &g, int i1, int i2, int i3,
                                                 const Geom &o, const Args<T> &a,
                                                 const T *__restrict__ src, T *__restrict__ dst,
                                                 const T *__restrict__ factors, int nvars,
                                                 int vbegin, int vend) {
  const bool skip = a.one_tap && g.perm >= 0;
  // Float64 one variable at a time: the FP64 pipe binds, and the fewer
  // registers a lane holds the more warps hide the loads' latency.  Float32
  // four at a time, or two where no more are left (a two-variable set would
  // otherwise issue half its taps' instructions predicated off).
  constexpr int VC = sizeof(T) == 8 ? 1 : 4;
  const bool two = sizeof(T) == 4 && vend - vbegin <= 2;
  if constexpr (PC == 4) {
    if ((sizeof(T) == 8 && a.pair_vars) || two)
      table_dispatch<T, D, 4, 2, SOFT>(g, i1, i2, i3, o, a, src, dst, factors, nvars, skip,
                                       vbegin, vend);
    else
      table_dispatch<T, D, 4, VC, SOFT>(g, i1, i2, i3, o, a, src, dst, factors, nvars, skip,
                                        vbegin, vend);
    return;
  }
  switch (g.pclass) {
    case 2:
      table_dispatch<T, D, 2, VC>(g, i1, i2, i3, o, a, src, dst, factors, nvars, skip, vbegin,
                                  vend);
      break;
    case 3:
      table_dispatch<T, D, 3, VC>(g, i1, i2, i3, o, a, src, dst, factors, nvars, skip, vbegin,
                                  vend);
      break;
    case 4:
      // Float64 order 4: one variable a lane, or (TAM_OPT_PAIR_VARS) two, whose
      // sums share each tap's weight and run as two independent chains
      if ((sizeof(T) == 8 && a.pair_vars) || two)
        table_dispatch<T, D, 4, 2>(g, i1, i2, i3, o, a, src, dst, factors, nvars, skip, vbegin,
                                   vend);
      else
        table_dispatch<T, D, 4, VC>(g, i1, i2, i3, o, a, src, dst, factors, nvars, skip, vbegin,
                                    vend);
      break;
    case 6:
      table_dispatch<T, D, 6, sizeof(T) == 8 ? 1 : 2>(g, i1, i2, i3, o, a, src, dst, factors,
                                                      nvars, skip, vbegin, vend);
      break;
    default:
      generic_point<T, D>(g, i1, i2, i3, o, a, src, dst, factors, nvars, skip, vbegin, vend);
      break;
  }
}

// Every variable of one box point of one stencil transfer, read in place.
template <typename T, int D, int PC = 0, bool SOFT = false>
__device__ __forceinline__ void stencil_point(const DevGroup &g, int i1, int i2, int i3,
                                              int64_t tblock, int64_t sblock, const Args<T> &a,
                                              const T *__restrict__ src, T *__restrict__ dst,
                                              const T *__restrict__ factors, int nvars, int S1,
                                              int S2, int S3) {
  const Geom o = geometry<D>(g, i1, i2, i3, tblock, sblock, a.srcstart, nvars, S1, S2, S3);
  stencil_dispatch<T, D, PC, SOFT>(g, i1, i2, i3, o, a, src, dst, factors, nvars, 0, nvars);
}

// ---- plain: one launch per group, one thread per (point, variable) ---------
template <typename T, int D>
__global__ void __launch_bounds__(256) plain_group_kernel(const DevGroup *__restrict__ gp,
                                                          Args<T> a, T *work,
                                                          const T *__restrict__ factors,
                                                          int nvars, int S1, int S2, int S3) {
  const DevGroup g = *gp;
  const int64_t box = (int64_t)g.n[0] * g.n[1] * g.n[2];
  const int64_t items = box * nvars * g.ntransfers;
  for (int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; it < items;
       it += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = it;
    const int i1 = (int)(r % g.n[0]);
    r /= g.n[0];
    const int i2 = (int)(r % g.n[1]);
    r /= g.n[1];
    const int i3 = (int)(r % g.n[2]);
    r /= g.n[2];
    const int v = (int)(r % nvars);
    const int64_t t = r / nvars + g.first;
    const int64_t tblock = __ldg(a.tb + t) - 1;
    const int64_t sblock = __ldg(a.sb + t) - 1;
    // one variable: the point as a one-variable field at variable v's offset
    const int64_t vs = (int64_t)S1 * S2 * S3;
    Geom o = geometry<D>(g, i1, i2, i3, tblock, sblock, a.srcstart, nvars, S1, S2, S3);
    o.toff += v * vs;
    o.soff += v * vs;
    if (g.pclass == 0) {
      using A = Arith<T>;
      T x = A::add(T(0), work[o.soff]);
      work[o.toff] = scaled(x, factors, v, nvars, g.factorcol);
    } else {
      const T *w1 = a.weights + g.w[0] + (int64_t)g.order[0] * i1;
      const T *w2 = a.weights + g.w[1] + (int64_t)g.order[1] * i2;
      const T *w3 = a.weights + g.w[2] + (int64_t)g.order[2] * i3;
      T acc;
      switch (g.pclass) {
        case 2: acc = stencil_sum<T, D, 2>(work + o.soff, o.s2, o.s3, w1, w2, w3, g.order); break;
        case 4: acc = stencil_sum<T, D, 4>(work + o.soff, o.s2, o.s3, w1, w2, w3, g.order); break;
        default: acc = stencil_sum<T, D, 0>(work + o.soff, o.s2, o.s3, w1, w2, w3, g.order); break;
      }
      work[o.toff] = scaled(acc, factors, v, nvars, g.factorcol);
    }
  }
}

// ---- fused: one launch per stage, one warp per tile ---------------------------
__device__ __forceinline__ void box_point(const DevGroup &g, int item, int &i1, int &i2,
                                          int &i3) {
  const int n1 = g.n[0], n12 = g.n[0] * g.n[1];
  const uint32_t m1 = g.mag1, m12 = g.mag12;
  i3 = m12 ? (int)__umulhi((uint32_t)item, m12) : item / n12;
  const int rem = item - i3 * n12;
  i2 = m1 ? (int)__umulhi((uint32_t)rem, m1) : rem / n1;
  i1 = rem - i2 * n1;
}

// The layout a tile works in: the kernel's own for one schedule, or its
// member's (base offsets and stored extents) in a batch of forests.
template <typename T, bool BATCH>
struct TileLayout {
  const T *src;
  T *dst;
  const T *factors;
  int S1, S2, S3;
  __device__ __forceinline__ TileLayout(const DevGroup &g, const Args<T> &a,
                                        const T *__restrict__ s, T *__restrict__ d,
                                        const T *__restrict__ f, int s1, int s2, int s3)
      : src(s), dst(d), factors(f), S1(s1), S2(s2), S3(s3) {
    if (BATCH) {
      const Member &m = a.members[g.member];
      src += m.work_off;
      dst += m.work_off;
      factors += m.fac_off;
      S1 = m.S[0];
      S2 = m.S[1];
      S3 = m.S[2];
    }
  }
};

// A warp's packed tile: lane l holds segment l; every lane then finds, for
// each of its points, the segment holding it.  All shuffles run with the full
// warp: the rounds loop to the tile's size, uniform across lanes.
struct SegPoint {
  int group, transfer, item;
  bool on;
};

__device__ __forceinline__ void load_segments(const Tile *__restrict__ tiles, const PTile &pt,
                                              int lane, Tile &seg, int &pref) {
  seg = Tile{0, 0, 0, 0};
  if (lane < pt.nseg) seg = tiles[pt.seg0 + lane];
  int incl = seg.nitems;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  pref = incl - seg.nitems;
}

// The segment of point k = b + lane (the warp's 32 consecutive points from b;
// kc is k clamped to the tile's last point).  Lane s (1 <= s < nseg) holds
// the first point pref of segment s, and the prefixes increase: one ballot
// counts the segments that start at or before b, another those that start
// within the window (b, b + 31], and only the latter are searched, so a tile
// of long segments takes no shuffle here and one of short ones at most 31.
// (The search stays a loop: straight-line forms of it let the compiler
// schedule the point's loads so early that the kernel needs half again the
// registers.)
__device__ __forceinline__ int find_segment(int pref, int nseg, int lane, int b, int kc) {
  const bool starts = lane >= 1 && lane < nseg;
  const int before = __popc(__ballot_sync(0xffffffffu, starts && pref <= b));
  const int inwin = __popc(__ballot_sync(0xffffffffu, starts && pref > b && pref <= b + 31));
  int mine = before;
  for (int s = before + 1; s <= before + inwin; ++s)
    if (kc >= __shfl_sync(0xffffffffu, pref, s)) mine = s;
  return mine;
}

__device__ __forceinline__ SegPoint find_point(const Tile &seg, int pref, int nseg, int lane,
                                               int b, int kc) {
  const int mine = find_segment(pref, nseg, lane, b, kc);
  SegPoint p;
  p.group = __shfl_sync(0xffffffffu, seg.group, mine);
  p.transfer = __shfl_sync(0xffffffffu, seg.transfer, mine);
  p.item = __shfl_sync(0xffffffffu, seg.item0, mine) + kc - __shfl_sync(0xffffffffu, pref, mine);
  p.on = true;
  return p;
}

// A segment of a batch's copy tile as its points need it, formed once per
// segment (by the lane that holds it) and kept in shared memory for the
// warp: the group's, the transfer's and the member's geometry folded into two
// base offsets and per-row strides, so that a point costs its segment's
// lookup, four shared loads and a few integer multiply-adds.  (A batch's
// blocks are small and its tiles hold many short segments; one schedule's
// tiles of long boxes do better forming each point's geometry from its
// group's loads, which broadcast across the warp.)
struct CopySeg {
  int64_t toff;        // target element of box point 0, variable 0
  int64_t soff;        // source element of box point 0, variable 0; -1: a copy
                       //   whose source rows are a table (no affine form)
  int32_t s2, s3;      // target strides of dimensions 2 and 3
  int32_t c1, c2, c3;  // source strides of a target row step in each dimension
  int32_t vstride;     // elements between variables
  int32_t n1, n12;     // box rows: the point decomposition
  uint32_t mag1, mag12;
  int32_t itemoff;     // box point of the tile's point k: k + itemoff
  int32_t fac;         // factor column's first element (FACTOR), from `factors`
};
static_assert(sizeof(CopySeg) == 64, "four 16-byte shared loads a point");

template <typename T, int D, bool BATCH, bool FACTOR>
__device__ __forceinline__ CopySeg copy_seg(const Tile &seg, int pref, const Args<T> &a,
                                            const T *src, T *dst, const T *factors, int nvars,
                                            int S1, int S2, int S3) {
  const DevGroup &g = a.groups[seg.group];
  const TileLayout<T, BATCH> L(g, a, src, dst, factors, S1, S2, S3);
  const int64_t s2 = L.S1, s3 = (int64_t)L.S1 * L.S2, vs = s3 * L.S3, bs = vs * nvars;
  const int64_t tblock = __ldg(a.tb + seg.transfer) - 1;
  const int64_t sblock = __ldg(a.sb + seg.transfer) - 1;
  CopySeg c;
  c.toff = tblock * bs + g.tf[0] + (D >= 2 ? g.tf[1] * s2 : 0) + (D >= 3 ? g.tf[2] * s3 : 0) +
           (L.dst - dst);
  c.soff = g.affine ? sblock * bs + g.cs0[0] + (D >= 2 ? g.cs0[1] * s2 : 0) +
                          (D >= 3 ? g.cs0[2] * s3 : 0) + (L.src - src)
                    : -1;
  c.s2 = (int32_t)s2;
  c.s3 = (int32_t)s3;
  c.c1 = g.cstep[0];
  c.c2 = D >= 2 ? g.cstep[1] * (int32_t)s2 : 0;
  c.c3 = D >= 3 ? g.cstep[2] * (int32_t)s3 : 0;
  c.vstride = (int32_t)vs;
  c.n1 = g.n[0];
  c.n12 = g.n[0] * g.n[1];
  c.mag1 = g.mag1;
  c.mag12 = g.mag12;
  c.itemoff = seg.item0 - pref;
  c.fac = FACTOR ? (int32_t)((L.factors - factors) + (int64_t)nvars * (g.factorcol - 1)) : 0;
  return c;
}

// Loads a lane of the copy kernel keeps in flight: NP points, kCopyVars / NP
// variables of each at a time.
constexpr int kCopyVars = 8;

// The unit-copy tiles of a stage: a light kernel, the loads of NP points a
// lane in flight together (NP, TAM_OPT_COPY_POINTS: with few variables a
// point, as in a batch of two-variable forests, more points a lane keep more
// loads in flight).
// Copies without a factor column run the FACTOR = false form, which holds
// no floating-point operation at all: with the factor's multiply in the
// same code the compiler issues it predicated, and on GB300's narrow FP64
// pipe that competes with the stencils alongside.
template <typename T, int D, bool BATCH, bool FACTOR, int NP>
__global__ void __launch_bounds__(512) fused_copy_kernel(const Tile *__restrict__ tiles,
                                                         const PTile *__restrict__ ptiles,
                                                         int64_t nptiles, Args<T> a,
                                                         const T *__restrict__ src,
                                                         T *__restrict__ dst,
                                                         const T *__restrict__ factors,
                                                         int nvars, int S1, int S2, int S3) {
  extern __shared__ __align__(16) unsigned char copy_smem[];
  const int lane = threadIdx.x & 31;
  CopySeg *segs = reinterpret_cast<CopySeg *>(copy_smem) + (threadIdx.x >> 5) * 32;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < nptiles;
       w += warps) {
    const PTile pt = ptiles[w];
    Tile seg;
    int pref;
    load_segments(tiles, pt, lane, seg, pref);
    if constexpr (!BATCH) {
      // one schedule's tiles (long boxes, few segments a tile): each point
      // forms its geometry from its group's loads, which broadcast
      for (int base = 0; base < pt.nitems; base += 32 * NP) {
        Geom o[NP];
        bool on[NP];
        const T *fac[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          const int k = base + 32 * p + lane;
          SegPoint q = find_point(seg, pref, pt.nseg, lane, base + 32 * p,
                                  k < pt.nitems ? k : pt.nitems - 1);
          on[p] = k < pt.nitems;
          const DevGroup &g = a.groups[q.group];
          const int64_t tblock = __ldg(a.tb + q.transfer) - 1;
          const int64_t sblock = __ldg(a.sb + q.transfer) - 1;
          int i1, i2, i3;
          box_point(g, q.item, i1, i2, i3);
          o[p] = g.affine ? copy_geometry<D>(g, i1, i2, i3, tblock, sblock, nvars, S1, S2, S3)
                          : geometry<D>(g, i1, i2, i3, tblock, sblock, a.srcstart, nvars, S1,
                                        S2, S3);
          fac[p] = FACTOR ? factors + (int64_t)nvars * (g.factorcol - 1) : nullptr;
        }
        copy_point_vars<T, NP, kCopyVars / NP, FACTOR>(fac, o, on, src, dst, 0, nvars);
      }
    } else {
      // A batch's tiles (small blocks, many short segments a tile): each
      // segment formed once, by its lane, into shared memory.
      bool general = false;
      if (lane < pt.nseg) {
        const CopySeg c = copy_seg<T, D, BATCH, FACTOR>(seg, pref, a, src, dst, factors, nvars,
                                                        S1, S2, S3);
        segs[lane] = c;
        general = c.soff < 0;
      }
      // a tile with a table-sourced segment takes the general form for it
      general = __any_sync(0xffffffffu, general);
      __syncwarp();
      // NP points a lane: their loads in flight together
      for (int base = 0; base < pt.nitems; base += 32 * NP) {
        Geom o[NP];
        bool on[NP];
        const T *fac[NP];
  #pragma unroll
        for (int p = 0; p < NP; ++p) {
          const int k = base + 32 * p + lane;
          const int kc = k < pt.nitems ? k : pt.nitems - 1;
          const int mine = find_segment(pref, pt.nseg, lane, base + 32 * p, kc);
          on[p] = k < pt.nitems;
          const CopySeg c = segs[mine];
          const int item = kc + c.itemoff;
          const int i3 = c.mag12 ? (int)__umulhi((uint32_t)item, c.mag12) : item / c.n12;
          const int rem = item - i3 * c.n12;
          const int i2 = c.mag1 ? (int)__umulhi((uint32_t)rem, c.mag1) : rem / c.n1;
          const int i1 = rem - i2 * c.n1;
          o[p].vstride = c.vstride;
          o[p].toff = c.toff + (i1 + i2 * c.s2 + i3 * c.s3);
          o[p].soff = c.soff + (i1 * c.c1 + i2 * c.c2 + i3 * c.c3);
          fac[p] = FACTOR ? factors + c.fac : nullptr;
          if (general) {  // warp-uniform: the shuffles take every lane
            const int gi = __shfl_sync(0xffffffffu, seg.group, mine);
            const int tr = __shfl_sync(0xffffffffu, seg.transfer, mine);
            if (c.soff < 0) {
              const DevGroup &g = a.groups[gi];
              const TileLayout<T, BATCH> L(g, a, src, dst, factors, S1, S2, S3);
              const int64_t tblock = __ldg(a.tb + tr) - 1;
              const int64_t sblock = __ldg(a.sb + tr) - 1;
              o[p] = geometry<D>(g, i1, i2, i3, tblock, sblock, a.srcstart, nvars, L.S1, L.S2,
                                 L.S3);
              o[p].soff += L.src - src;
              o[p].toff += L.dst - dst;
            }
          }
        }
        copy_point_vars<T, NP, kCopyVars / NP, FACTOR>(fac, o, on, src, dst, 0, nvars);
      }
      __syncwarp();  // every lane is done with the segments before the next tile's
    }
  }
}

// The stencil tiles of a stage: one point a lane, every variable.  PC = 4:
// tiles of uniform order-4 groups only (a stage's tiles grouped by path hold
// them in one run), the only path compiled, so that the registers it keeps
// are its own; SOFT, Float64 order 4 with TAM_OPT_SOFT_ADD.
template <typename T, int D, bool BATCH, int PC, bool SOFT = false>
__global__ void __maxnreg__(64) fused_stage_kernel(const Tile *__restrict__ tiles,
                                                          const PTile *__restrict__ ptiles,
                                                          int64_t nptiles, Args<T> a,
                                                          const T *__restrict__ src,
                                                          T *__restrict__ dst,
                                                          const T *__restrict__ factors,
                                                          int nvars, int S1, int S2, int S3) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < nptiles;
       w += warps) {
    const PTile pt = ptiles[w];
    Tile seg;
    int pref;
    load_segments(tiles, pt, lane, seg, pref);
    for (int base = 0; base < pt.nitems; base += 32) {
      const int k = base + lane;
      SegPoint q = find_point(seg, pref, pt.nseg, lane, base, k < pt.nitems ? k : pt.nitems - 1);
      if (k >= pt.nitems) continue;
      const DevGroup &g = a.groups[q.group];
      const TileLayout<T, BATCH> L(g, a, src, dst, factors, S1, S2, S3);
      const int64_t tblock = __ldg(a.tb + q.transfer) - 1;
      const int64_t sblock = __ldg(a.sb + q.transfer) - 1;
      const int item = g.perm >= 0 ? __ldg(a.perm + g.perm + q.item) : q.item;
      int i1, i2, i3;
      box_point(g, item, i1, i2, i3);
      stencil_point<T, D, PC, SOFT>(g, i1, i2, i3, tblock, sblock, a, L.src, L.dst, L.factors,
                                    nvars,
                              L.S1,
                          L.S2, L.S3);
    }
  }
}

// The stencil transfers of large boxes, each from its source window staged in
// shared memory: a CTA per transfer loads the window (rows of the source
// block, a warp a row, a few variables at a time) and then every thread
// takes box points in tile order (the group's points by path), summing its
// taps from shared memory in the reference's order (src/ghosts.jl:75-118),
// so the result is the same bits as the in-place kernel's.  The window is
// what every point's columns read (tam::DevGroup::wlo, wn); in a
// prolongation each window point serves about P^D / 2^D box points.
template <typename T, int D, bool BATCH>
__global__ void __launch_bounds__(256, 4) staged_stencil_kernel(const Tile *__restrict__ items,
                                                                int64_t nitems, Args<T> a,
                                                                const T *__restrict__ src,
                                                                T *__restrict__ dst,
                                                                const T *__restrict__ factors,
                                                                int nvars, int S1, int S2,
                                                                int S3, int kElems) {
  extern __shared__ __align__(16) unsigned char staged_smem[];
  T *sm = reinterpret_cast<T *>(staged_smem);
  for (int64_t it = blockIdx.x; it < nitems; it += gridDim.x) {
    const Tile item = items[it];
    const DevGroup &g = a.groups[item.group];
    const TileLayout<T, BATCH> L(g, a, src, dst, factors, S1, S2, S3);
    const int64_t tblock = __ldg(a.tb + item.transfer) - 1;
    const int64_t sblock = __ldg(a.sb + item.transfer) - 1;
    const int wn1 = g.wn[0], wn2 = g.wn[1], wn3 = g.wn[2];
    const int wvol = wn1 * wn2 * wn3;
    const int vchunk = max(1, min(nvars, kElems / wvol));
    const int64_t s2 = L.S1, s3 = (int64_t)L.S1 * L.S2, vol = s3 * L.S3;
    const T *__restrict__ wsrc =
        L.src + sblock * nvars * vol + g.wlo[0] + g.wlo[1] * s2 + g.wlo[2] * s3;
    const int box = g.n[0] * g.n[1] * g.n[2];
    for (int v0 = 0; v0 < nvars; v0 += vchunk) {
      const int vc = min(vchunk, nvars - v0);
      __syncthreads();  // every thread is done with the previous window
      // the window's points in order, four loads a thread in flight
      const int nload = vc * wvol;
      for (int e0 = threadIdx.x; e0 < nload; e0 += 4 * blockDim.x) {
        T val[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int e = e0 + u * blockDim.x;
          if (e < nload) {
            const int x = e % wn1, r = e / wn1;
            const int y = r % wn2, rest = r / wn2;
            const int z = rest % wn3, v = rest / wn3;
            val[u] = wsrc[(int64_t)(v0 + v) * vol + z * s3 + y * s2 + x];
          }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int e = e0 + u * blockDim.x;
          if (e < nload) sm[e] = val[u];
        }
      }
      __syncthreads();
      for (int k = threadIdx.x; k < box; k += blockDim.x) {
        const int pt = g.perm >= 0 ? __ldg(a.perm + g.perm + k) : k;
        int i1, i2, i3;
        box_point(g, pt, i1, i2, i3);
        Geom o;
        o.s2 = wn1;
        o.s3 = (int64_t)wn1 * wn2;
        o.svstride = wvol;
        o.vstride = vol;
        const int b1 = __ldg(a.srcstart + g.ss[0] + i1) - 1 - g.wlo[0];
        const int b2 = D >= 2 ? __ldg(a.srcstart + g.ss[1] + i2) - 1 - g.wlo[1] : 0;
        const int b3 = D >= 3 ? __ldg(a.srcstart + g.ss[2] + i3) - 1 - g.wlo[2] : 0;
        // the window holds variables v0 .. v0 + vc - 1 from its start
        o.soff = b1 + (int64_t)b2 * o.s2 + (int64_t)b3 * o.s3 - (int64_t)v0 * wvol;
        o.toff = tblock * nvars * vol + (g.tf[0] + i1) + (int64_t)(g.tf[1] + i2) * s2 +
                 (int64_t)(g.tf[2] + i3) * s3;
        stencil_dispatch<T, D>(g, i1, i2, i3, o, a, sm, L.dst, L.factors, nvars, v0, v0 + vc);
      }
    }
  }
}

template <typename T>
cudaError_t plain_dispatch(int D, const DevGroup &g, const DevGroup *d_g, const Args<T> &a,
                           T *work, const T *factors, int nvars, const int S[3],
                           cudaStream_t stream) {
  const int64_t items = (int64_t)g.n[0] * g.n[1] * g.n[2] * nvars * g.ntransfers;
  if (items == 0) return cudaSuccess;
  const int threads = 256;
  int64_t blocks = (items + threads - 1) / threads;
  if (blocks > (int64_t)1 << 30) blocks = (int64_t)1 << 30;
  switch (D) {
    case 1:
      plain_group_kernel<T, 1><<<(unsigned)blocks, threads, 0, stream>>>(d_g, a, work, factors,
                                                                          nvars, S[0], S[1], S[2]);
      break;
    case 2:
      plain_group_kernel<T, 2><<<(unsigned)blocks, threads, 0, stream>>>(d_g, a, work, factors,
                                                                          nvars, S[0], S[1], S[2]);
      break;
    default:
      plain_group_kernel<T, 3><<<(unsigned)blocks, threads, 0, stream>>>(d_g, a, work, factors,
                                                                          nvars, S[0], S[1], S[2]);
      break;
  }
  return cudaGetLastError();
}

template <typename T, int D, bool BATCH, bool FACTOR>
cudaError_t launch_copies(const Tile *tiles, const PTile *ptiles, int64_t n, const Args<T> &a,
                          const T *src, T *work, const T *factors, int nvars, const int S[3],
                          int threads, cudaStream_t stream, int64_t cap) {
  if (n <= 0) return cudaSuccess;
  const int wpb = threads / 32;
  int64_t blocks = std::min<int64_t>((n + wpb - 1) / wpb, (int64_t)1 << 30);
  if (cap > 0) blocks = std::min(blocks, cap);
  // a batch's segments in shared memory: 2 KiB a warp, 32 KiB at most
  const size_t smem = BATCH ? (size_t)wpb * 32 * sizeof(CopySeg) : 0;
  if (a.copy_points >= 4)
    fused_copy_kernel<T, D, BATCH, FACTOR, 4><<<(unsigned)blocks, threads, smem, stream>>>(
        tiles, ptiles, n, a, src, work, factors, nvars, S[0], S[1], S[2]);
  else if (a.copy_points == 2)
    fused_copy_kernel<T, D, BATCH, FACTOR, 2><<<(unsigned)blocks, threads, smem, stream>>>(
        tiles, ptiles, n, a, src, work, factors, nvars, S[0], S[1], S[2]);
  else
    fused_copy_kernel<T, D, BATCH, FACTOR, 1><<<(unsigned)blocks, threads, smem, stream>>>(
        tiles, ptiles, n, a, src, work, factors, nvars, S[0], S[1], S[2]);
  return cudaSuccess;
}

template <typename T, int D>
cudaError_t launch_both(const Tile *tiles, const PTile *ptiles, const Stage &stg,
                        const Args<T> &a, const T *src, T *work, const T *factors, int nvars,
                        const int S[3], int threads, cudaStream_t stream, SideStream *side,
                        const Tile *staged) {
  const int64_t npcopy0 = stg.npcopy0, npcopy = stg.npcopy, nptiles = stg.nptiles;
  const int64_t np4_0 = stg.np4_0, np4 = stg.np4;
  const int64_t nstaged = stg.nstaged, staged_window_elems = stg.staged_window;
  const int wpb = threads / 32;
  const bool batch = a.members != nullptr;
  const int64_t nst = nptiles - npcopy;
  // both present: the stencils on the side stream, alongside the copies
  const bool fork = side && side->ok() && npcopy > 0 && (nst > 0 || nstaged > 0);
  cudaStream_t sst = stream;
  if (fork) {
    cudaError_t e = cudaEventRecord(side->fork, stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(side->stream, side->fork, 0);
    if (e != cudaSuccess) return e;
    sst = side->stream;
  }
  // TAM_OPT_COPY_SHARE: the copies' CTAs resident first, a few a
  // multiprocessor, and the stencils' around them
  const bool copies_first = fork && a.copy_ctas > 0;
  const int64_t cap = copies_first ? a.copy_ctas : 0;
  auto copies = [&]() {
    if (batch) {
      launch_copies<T, D, true, false>(tiles, ptiles, npcopy0, a, src, work, factors, nvars, S,
                                       threads, stream, cap);
      launch_copies<T, D, true, true>(tiles, ptiles + npcopy0, npcopy - npcopy0, a, src, work,
                                      factors, nvars, S, threads, stream, cap);
    } else {
      launch_copies<T, D, false, false>(tiles, ptiles, npcopy0, a, src, work, factors, nvars, S,
                                        threads, stream, cap);
      launch_copies<T, D, false, true>(tiles, ptiles + npcopy0, npcopy - npcopy0, a, src, work,
                                       factors, nvars, S, threads, stream, cap);
    }
  };
  if (copies_first) copies();
  // the stencil tiles: the order-4 run (tiles grouped by path) in the
  // kernel compiled for that order alone, the others in the general one
  auto stencils = [&](int64_t p0, int64_t n, bool four) {
    if (n <= 0) return;
    const int64_t blocks = std::min<int64_t>((n + wpb - 1) / wpb, (int64_t)1 << 30);
    const PTile *pt = ptiles + p0;
    if constexpr (sizeof(T) == 8) {  // the integer-pipe add: Float64 only
      if (four && a.soft_add && a.int_mul) {
        if (batch)
          fused_stage_kernel<T, D, true, 4, true><<<(unsigned)blocks, threads, 0, sst>>>(
              tiles, pt, n, a, src, work, factors, nvars, S[0], S[1], S[2]);
        else
          fused_stage_kernel<T, D, false, 4, true><<<(unsigned)blocks, threads, 0, sst>>>(
              tiles, pt, n, a, src, work, factors, nvars, S[0], S[1], S[2]);
        return;
      }
    }
    if (batch && four)
      fused_stage_kernel<T, D, true, 4><<<(unsigned)blocks, threads, 0, sst>>>(
          tiles, pt, n, a, src, work, factors, nvars, S[0], S[1], S[2]);
    else if (batch)
      fused_stage_kernel<T, D, true, 0><<<(unsigned)blocks, threads, 0, sst>>>(
          tiles, pt, n, a, src, work, factors, nvars, S[0], S[1], S[2]);
    else if (four)
      fused_stage_kernel<T, D, false, 4><<<(unsigned)blocks, threads, 0, sst>>>(
          tiles, pt, n, a, src, work, factors, nvars, S[0], S[1], S[2]);
    else
      fused_stage_kernel<T, D, false, 0><<<(unsigned)blocks, threads, 0, sst>>>(
          tiles, pt, n, a, src, work, factors, nvars, S[0], S[1], S[2]);
  };
  if (nst > 0) {
    const int64_t f0 = std::min(std::max(np4_0, npcopy), nptiles);
    const int64_t f1 = std::min(f0 + np4, nptiles);
    stencils(npcopy, f0 - npcopy, false);
    stencils(f0, f1 - f0, true);
    stencils(f1, nptiles - f1, false);
  }
  if (nstaged > 0) {
    // the shared memory a CTA holds: the stage's largest window for one
    // variable (the staged items' nitems field carries it, in elements),
    // as many variables at a time as fit twice that
    const int64_t blocks = std::min<int64_t>(nstaged, (int64_t)1 << 30);
    const int elems = (int)std::min<int64_t>(2 * staged_window_elems, kStagedBytes / sizeof(T));
    const size_t bytes = (size_t)elems * sizeof(T);
    if (batch)
      staged_stencil_kernel<T, D, true><<<(unsigned)blocks, 256, bytes, sst>>>(
          staged, nstaged, a, src, work, factors, nvars, S[0], S[1], S[2], elems);
    else
      staged_stencil_kernel<T, D, false><<<(unsigned)blocks, 256, bytes, sst>>>(
          staged, nstaged, a, src, work, factors, nvars, S[0], S[1], S[2], elems);
  }
  if (!copies_first) copies();
  if (fork) {
    cudaError_t e = cudaEventRecord(side->join, side->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, side->join, 0);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

// A stage: its unit copies and its stencils, two launches with no
// dependency between them (their targets are disjoint, and no transfer reads
// another's targets: a stage-P copy reads only the point it writes).
template <typename T>
cudaError_t fused_dispatch(int D, const Tile *tiles, const PTile *ptiles, const Stage &st,
                           const Args<T> &a, const T *src, T *work, const T *factors, int nvars,
                           const int S[3], int threads, cudaStream_t stream, SideStream *side,
                           const Tile *staged) {
  if (st.nptiles == 0 && st.nstaged == 0) return cudaSuccess;
  switch (D) {
    case 1:
      return launch_both<T, 1>(tiles, ptiles, st, a, src, work, factors, nvars, S, threads,
                               stream, side, staged);
    case 2:
      return launch_both<T, 2>(tiles, ptiles, st, a, src, work, factors, nvars, S, threads,
                               stream, side, staged);
    default:
      return launch_both<T, 3>(tiles, ptiles, st, a, src, work, factors, nvars, S, threads,
                               stream, side, staged);
  }
}

}  // namespace

// The fused launches of one stage: launch_fused_stage with `ptiles` and
// `staged` already at the stage's first entries and `src` set, for one
// element type and dimension each, so that the build compiles them in
// parallel: Float32 in tam_fused_f32.cu (every dimension), Float64 one
// dimension a unit (tam_fused_f64_d1.cu, _d2, _d3).
cudaError_t fused_stage_f32(int D, const Tile *tiles, const PTile *ptiles, const Stage &st,
                            const SchedArgs &a, void *work, const void *factors, int nvars,
                            const int S[3], int threads, cudaStream_t stream, SideStream *side,
                            const void *src, const Tile *staged);
cudaError_t fused_stage_f64_d1(const Tile *tiles, const PTile *ptiles, const Stage &st,
                               const SchedArgs &a, void *work, const void *factors, int nvars,
                               const int S[3], int threads, cudaStream_t stream,
                               SideStream *side, const void *src, const Tile *staged);
cudaError_t fused_stage_f64_d2(const Tile *tiles, const PTile *ptiles, const Stage &st,
                               const SchedArgs &a, void *work, const void *factors, int nvars,
                               const int S[3], int threads, cudaStream_t stream,
                               SideStream *side, const void *src, const Tile *staged);
cudaError_t fused_stage_f64_d3(const Tile *tiles, const PTile *ptiles, const Stage &st,
                               const SchedArgs &a, void *work, const void *factors, int nvars,
                               const int S[3], int threads, cudaStream_t stream,
                               SideStream *side, const void *src, const Tile *staged);

}  // namespace tam

#endif  // TAM_KERNELS_CUH
