// Ghost-fill kernels for sm_103a.
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
#include <cuda_runtime.h>
#include <stdint.h>

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

// Everything one item needs from its group and transfer.
struct ItemGeom {
  int64_t tbase;  // element offset of (tidx, v = 0) in work
  int64_t sbase;  // element offset of (base, v = 0) in work
  int wcol[3];    // target row per dimension (weight column)
};

// The body shared by both launch forms: the item at box point (i1, i2, i3)
// of transfer (tblock, sblock), every variable in [v0, v1).
template <typename T, int D, int P>
__device__ __forceinline__ void do_point(const DevGroup &g, int i1, int i2, int i3,
                                         int64_t tblock, int64_t sblock,
                                         const int32_t *__restrict__ srcstart,
                                         const T *__restrict__ weights, T *work,
                                         const T *__restrict__ factors, int nvars, int v0, int v1,
                                         int S1, int S2, int S3) {
  using A = Arith<T>;
  const int64_t s2 = S1, s3 = (int64_t)S1 * S2;
  const int64_t vstride = s3 * S3;
  const int64_t bstride = vstride * nvars;
  const int b1 = __ldg(srcstart + g.ss[0] + i1) - 1;
  const int b2 = D >= 2 ? __ldg(srcstart + g.ss[1] + i2) - 1 : 0;
  const int b3 = D >= 3 ? __ldg(srcstart + g.ss[2] + i3) - 1 : 0;
  const int64_t toff = tblock * bstride + (int64_t)(g.tf[0] + i1) +
                       (D >= 2 ? (int64_t)(g.tf[1] + i2) * s2 : 0) +
                       (D >= 3 ? (int64_t)(g.tf[2] + i3) * s3 : 0);
  const int64_t soff = sblock * bstride + b1 + (int64_t)b2 * s2 + (int64_t)b3 * s3;
  if (P == 1) {  // a unit copy: +0 + x (src/ghosts.jl:127-128)
    for (int v = v0; v < v1; ++v) {
      T x = A::add(T(0), work[soff + v * vstride]);
      work[toff + v * vstride] = scaled(x, factors, v, nvars, g.factorcol);
    }
    return;
  }
  const T *w1 = weights + g.w[0] + (int64_t)g.order[0] * i1;
  const T *w2 = weights + g.w[1] + (int64_t)g.order[1] * i2;
  const T *w3 = weights + g.w[2] + (int64_t)g.order[2] * i3;
  for (int v = v0; v < v1; ++v) {
    T acc = stencil_sum<T, D, (P > 1 ? P : 0)>(work + soff + v * vstride, s2, s3, w1, w2, w3,
                                                g.order);
    work[toff + v * vstride] = scaled(acc, factors, v, nvars, g.factorcol);
  }
}

template <typename T, int D>
__device__ __forceinline__ void dispatch_point(const DevGroup &g, int i1, int i2, int i3,
                                               int64_t tblock, int64_t sblock,
                                               const int32_t *__restrict__ srcstart,
                                               const T *__restrict__ weights, T *work,
                                               const T *__restrict__ factors, int nvars, int v0,
                                               int v1, int S1, int S2, int S3) {
  switch (g.pclass) {
    case 0:
      do_point<T, D, 1>(g, i1, i2, i3, tblock, sblock, srcstart, weights, work, factors, nvars,
                        v0, v1, S1, S2, S3);
      break;
    case 2:
      do_point<T, D, 2>(g, i1, i2, i3, tblock, sblock, srcstart, weights, work, factors, nvars,
                        v0, v1, S1, S2, S3);
      break;
    case 3:
      do_point<T, D, 3>(g, i1, i2, i3, tblock, sblock, srcstart, weights, work, factors, nvars,
                        v0, v1, S1, S2, S3);
      break;
    case 4:
      do_point<T, D, 4>(g, i1, i2, i3, tblock, sblock, srcstart, weights, work, factors, nvars,
                        v0, v1, S1, S2, S3);
      break;
    case 6:
      do_point<T, D, 6>(g, i1, i2, i3, tblock, sblock, srcstart, weights, work, factors, nvars,
                        v0, v1, S1, S2, S3);
      break;
    default:
      do_point<T, D, 0>(g, i1, i2, i3, tblock, sblock, srcstart, weights, work, factors, nvars,
                        v0, v1, S1, S2, S3);
      break;
  }
}

// ---- plain: one launch per group, one thread per (point, variable) ---------
template <typename T, int D>
__global__ void __launch_bounds__(256) plain_group_kernel(
    const DevGroup *__restrict__ gp, const int32_t *__restrict__ tb,
    const int32_t *__restrict__ sb, const int32_t *__restrict__ srcstart,
    const T *__restrict__ weights, T *work, const T *__restrict__ factors, int nvars, int S1,
    int S2, int S3) {
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
    const int64_t tblock = __ldg(tb + t) - 1;
    const int64_t sblock = __ldg(sb + t) - 1;
    dispatch_point<T, D>(g, i1, i2, i3, tblock, sblock, srcstart, weights, work, factors, nvars,
                         v, v + 1, S1, S2, S3);
  }
}

// ---- fused: one launch per stage, one warp per tile ---------------------------
template <typename T, int D>
__global__ void __launch_bounds__(256) fused_stage_kernel(
    const Tile *__restrict__ tiles, int64_t ntiles, const DevGroup *__restrict__ groups,
    const int32_t *__restrict__ tb, const int32_t *__restrict__ sb,
    const int32_t *__restrict__ srcstart, const T *__restrict__ weights, T *work,
    const T *__restrict__ factors, int nvars, int S1, int S2, int S3) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < ntiles;
       w += warps) {
    const Tile tile = tiles[w];
    const DevGroup &g = groups[tile.group];
    const int64_t tblock = __ldg(tb + tile.transfer) - 1;
    const int64_t sblock = __ldg(sb + tile.transfer) - 1;
    const int n1 = g.n[0], n12 = g.n[0] * g.n[1];
    for (int k = lane; k < tile.nitems; k += 32) {
      const int item = tile.item0 + k;
      const int i3 = item / n12;
      const int rem = item - i3 * n12;
      const int i2 = rem / n1;
      const int i1 = rem - i2 * n1;
      dispatch_point<T, D>(g, i1, i2, i3, tblock, sblock, srcstart, weights, work, factors, nvars,
                           0, nvars, S1, S2, S3);
    }
  }
}

template <typename T>
cudaError_t plain_dispatch(int D, const DevGroup &g, const DevGroup *d_g, const int32_t *tb,
                           const int32_t *sb, const int32_t *srcstart, const T *weights, T *work,
                           const T *factors, int nvars, const int S[3], cudaStream_t stream) {
  const int64_t items = (int64_t)g.n[0] * g.n[1] * g.n[2] * nvars * g.ntransfers;
  if (items == 0) return cudaSuccess;
  const int threads = 256;
  int64_t blocks = (items + threads - 1) / threads;
  if (blocks > (int64_t)1 << 30) blocks = (int64_t)1 << 30;
  switch (D) {
    case 1:
      plain_group_kernel<T, 1><<<(unsigned)blocks, threads, 0, stream>>>(
          d_g, tb, sb, srcstart, weights, work, factors, nvars, S[0], S[1], S[2]);
      break;
    case 2:
      plain_group_kernel<T, 2><<<(unsigned)blocks, threads, 0, stream>>>(
          d_g, tb, sb, srcstart, weights, work, factors, nvars, S[0], S[1], S[2]);
      break;
    default:
      plain_group_kernel<T, 3><<<(unsigned)blocks, threads, 0, stream>>>(
          d_g, tb, sb, srcstart, weights, work, factors, nvars, S[0], S[1], S[2]);
      break;
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t fused_dispatch(int D, const Tile *tiles, int64_t ntiles, const DevGroup *groups,
                           const int32_t *tb, const int32_t *sb, const int32_t *srcstart,
                           const T *weights, T *work, const T *factors, int nvars, const int S[3],
                           int threads, cudaStream_t stream) {
  if (ntiles == 0) return cudaSuccess;
  const int wpb = threads / 32;
  int64_t blocks = (ntiles + wpb - 1) / wpb;
  if (blocks > (int64_t)1 << 30) blocks = (int64_t)1 << 30;
  switch (D) {
    case 1:
      fused_stage_kernel<T, 1><<<(unsigned)blocks, threads, 0, stream>>>(
          tiles, ntiles, groups, tb, sb, srcstart, weights, work, factors, nvars, S[0], S[1], S[2]);
      break;
    case 2:
      fused_stage_kernel<T, 2><<<(unsigned)blocks, threads, 0, stream>>>(
          tiles, ntiles, groups, tb, sb, srcstart, weights, work, factors, nvars, S[0], S[1], S[2]);
      break;
    default:
      fused_stage_kernel<T, 3><<<(unsigned)blocks, threads, 0, stream>>>(
          tiles, ntiles, groups, tb, sb, srcstart, weights, work, factors, nvars, S[0], S[1], S[2]);
      break;
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_plain_group(int dtype, int D, const DevGroup &g, const DevGroup *d_g,
                               const int32_t *tb, const int32_t *sb, const int32_t *srcstart,
                               const void *weights, void *work, const void *factors, int nvars,
                               const int S[3], cudaStream_t stream) {
  if (dtype == TAM_F64)
    return plain_dispatch<double>(D, g, d_g, tb, sb, srcstart, (const double *)weights,
                                  (double *)work, (const double *)factors, nvars, S, stream);
  return plain_dispatch<float>(D, g, d_g, tb, sb, srcstart, (const float *)weights, (float *)work,
                               (const float *)factors, nvars, S, stream);
}

cudaError_t launch_fused_stage(int dtype, int D, const Tile *tiles, int64_t ntiles,
                               const DevGroup *groups, const int32_t *tb, const int32_t *sb,
                               const int32_t *srcstart, const void *weights, void *work,
                               const void *factors, int nvars, const int S[3], int threads,
                               cudaStream_t stream) {
  if (dtype == TAM_F64)
    return fused_dispatch<double>(D, tiles, ntiles, groups, tb, sb, srcstart,
                                  (const double *)weights, (double *)work, (const double *)factors,
                                  nvars, S, threads, stream);
  return fused_dispatch<float>(D, tiles, ntiles, groups, tb, sb, srcstart, (const float *)weights,
                               (float *)work, (const float *)factors, nvars, S, threads, stream);
}

}  // namespace tam
