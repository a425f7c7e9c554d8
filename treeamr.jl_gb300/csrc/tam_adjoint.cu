// The adjoint (transpose) of the ghost fill, in gather form.
//
// No reference counterpart: TreeAMR.jl has no adjoint (its only "adjoint" is
// an element restriction, src/operators.jl:72-75).  The fill is linear, and
// stage s of it (src/ghosts.jl:1099-1160) is
//
//   x <- (I - E_s) x + E_s A_s x,
//
// E_s the projection onto the stage's target points and A_s reading only
// points that are not the stage's targets (ghosts are written from owned
// points, or a coarser block's ghosts written by an earlier stage).  Its
// transpose is
//
//   y <- (I - E_s) y + A_s^T E_s y,
//
// applied stage by stage in reverse.  A_s^T is formed in gather form, with
// no atomics and a fixed order of summation, so the adjoint is deterministic:
//
//   pass 1  one CTA per transfer takes the transfer's target box of
//           f * y[target] into shared memory and applies the transposed
//           one-dimensional stencils one dimension at a time (CSR: source
//           row -> (target row, weight)), leaving the box of its source
//           footprint in a scratch box of its own.  The forward fill must
//           sum the P^D taps of a point in the reference's order; its
//           transpose has no reference rounding to follow, so the tensor
//           product is applied as D passes of P taps each (3P multiply-adds
//           a point instead of P^3 on the narrow FP64 pipe).  A copy that
//           translates or mirrors (AdjGroup::direct) has no pass 1: its
//           footprint is its target box read back through the same map;
//   pass 2  one CTA per source block adds the boxes of the transfers reading
//           it (a direct copy's read from its target box in place), in
//           waves of transfers whose footprints do not meet, a barrier
//           between waves, so that every point takes its adds in transfer
//           order;
//   zero    the stage's target points are set to zero.
//
// The transpose differs from the exact transpose of the rounded forward
// weights ((w_1*w_2)*w_3) by the rounding of the products, a few units in
// the last place of each weight: the dot-product identity holds to the
// sums' rounding.  A single weight (a unit vector y) comes out as
// ((w_1*w_2)*w_3) exactly.
//
// The scratch is Sum over a stage's transfers of footprint x nvars elements
// (tam_adjoint_scratch_bytes); the library owns one, or the caller passes
// its own (tam_fill_adjoint_scratch).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "tam_internal.h"

namespace tam {
namespace {

template <typename T>
struct AArith;
template <>
struct AArith<double> {
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double fma(double a, double b, double c) {
    return __fma_rn(a, b, c);
  }
};
template <>
struct AArith<float> {
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float fma(float a, float b, float c) {
    return __fmaf_rn(a, b, c);
  }
};

template <typename T>
struct AdjArgs {
  const DevGroup *__restrict__ groups;
  const AdjGroup *__restrict__ ag;
  const int32_t *__restrict__ tb;
  const T *__restrict__ weights;
  const int32_t *__restrict__ off;
  const int2 *__restrict__ ent;
  const int64_t *__restrict__ scr;
  const Member *__restrict__ members;  // a batch's, or null
  const int32_t *__restrict__ rotvars; // turned groups' variable table, or null
  int32_t *err;                        // error word, or null
};

// Where a transfer's field data and factors are: the kernel's own layout for
// one schedule, or its member's in a batch of forests.
template <typename T, bool BATCH>
struct AdjLayout {
  T *y;
  const T *factors;
  int64_t s2, s3, vs, bs;
  __device__ __forceinline__ AdjLayout(const AdjArgs<T> &a, int member, T *y0, const T *f0,
                                       int nvars, int S1, int S2, int S3)
      : y(y0), factors(f0) {
    if (BATCH) {
      const Member &m = a.members[member];
      y += m.work_off;
      factors += m.fac_off;
      S1 = m.S[0];
      S2 = m.S[1];
      S3 = m.S[2];
    }
    s2 = S1;
    s3 = (int64_t)S1 * S2;
    vs = s3 * S3;
    bs = vs * nvars;
  }
};

// Pass 1: one CTA per transfer and variable, the box passes in shared memory.  Entries of
// dimension d's transposed stencil are (i, w): target row i, weight index w
// into the weight pool; a dimension beyond D has one entry of weight one.
// Per variable: A = f * y over the target box (n1 x n2 x n3, row 1 fastest),
// B = T1 A (fn1 x n2 x n3), C = T2 B (fn1 x fn2 x n3) in A's place, box = T3 C.
template <typename T, int D, bool BATCH>
__global__ void __launch_bounds__(256) adjoint_box_kernel(
    const int2 *__restrict__ xfers, int64_t nxfers, AdjArgs<T> a, T *y, T *scratch,
    const T *__restrict__ factors, int nvars, int S1, int S2, int S3, int box_elems,
    int csr_ents) {
  using A = AArith<T>;
  extern __shared__ __align__(16) unsigned char adj_smem[];
  T *SA = (T *)adj_smem;
  // after the boxes, the transfer's transposed stencils: each entry's weight
  // and target row, and each footprint row's first entry, three dimensions
  // one after another
  T *SW = SA + box_elems;
  int *SE = (int *)(SW + csr_ents);
  int *SO = SE + csr_ents;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int64_t q = blockIdx.x; q < nxfers; q += gridDim.x) {
    const int2 tg = xfers[q];  // (transfer, group)
    const DevGroup &g = a.groups[tg.y];
    const AdjGroup &h = a.ag[tg.y];
    const AdjLayout<T, BATCH> L(a, g.member, y, factors, nvars, S1, S2, S3);
    const int n1 = g.n[0], n2 = g.n[1], n3 = g.n[2];
    const int f1 = h.fn[0], f2 = h.fn[1], f3 = h.fn[2];
    const int nA = n1 * n2 * n3, nB = f1 * n2 * n3, nC = f1 * f2 * n3, nO = f1 * f2 * f3;
    // C takes A's place (A is done with once B is formed), B after the larger
    T *SC = SA;
    T *SB = SA + (nA > nC ? nA : nC);
    const int64_t tblock = __ldg(a.tb + tg.x) - 1;
    T *out = scratch + __ldg(a.scr + tg.x) * nvars;
    // a direct copy (AdjGroup::direct) has no pass-1 work and no scratch:
    // the host leaves it out of the list
    if (h.direct) continue;
    // the transposed stencils into shared memory, weights looked up once:
    // the passes then read no global memory but the target box
    const int fn[3] = {f1, f2, f3};
    int rbase[3], ebase[3];
    {
      int r = 0, e = 0;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        rbase[d] = r;
        ebase[d] = e;
        r += fn[d] + 1;
        e += __ldg(a.off + h.off[d] + fn[d]) - __ldg(a.off + h.off[d]);
      }
    }
    __syncthreads();  // the previous transfer's passes are done with the tables
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int32_t *od = a.off + h.off[d];
      const int e0 = __ldg(od);
      for (int k = tid; k <= fn[d]; k += nt) SO[rbase[d] + k] = __ldg(od + k) - e0 + ebase[d];
      const int ne = __ldg(od + fn[d]) - e0;
      for (int k = tid; k < ne; k += nt) {
        const int2 q = __ldg(a.ent + e0 + k);
        SE[ebase[d] + k] = q.x;
        SW[ebase[d] + k] = __ldg(a.weights + q.y);
      }
    }
    const int *o1 = SO + rbase[0], *o2 = SO + rbase[1], *o3 = SO + rbase[2];
    // a variable a CTA row (blockIdx.y): the variables' passes are independent
    for (int v = blockIdx.y; v < nvars; v += gridDim.y) {
      const T *yv = L.y + tblock * L.bs + v * L.vs;
      const T f =
          g.factorcol ? __ldg(L.factors + v + (int64_t)nvars * (g.factorcol - 1)) : T(1);
      for (int k = tid; k < nA; k += nt) {
        const int i3 = k / (n1 * n2), r = k - i3 * (n1 * n2), i2 = r / n1, i1 = r - i2 * n1;
        T x = yv[(g.tf[0] + i1) + (int64_t)(g.tf[1] + i2) * L.s2 + (int64_t)(g.tf[2] + i3) * L.s3];
        // a factor of -1, 0 or 1 is exact here and commutes with the sums
        if (g.factorcol) x = A::mul(x, f);
        SA[k] = x;
      }
      __syncthreads();
      for (int k = tid; k < nB; k += nt) {  // B[(i3 n2 + i2) f1 + j1]
        const int row = k / f1, j1 = k - row * f1;
        const T *src = SA + row * n1;
        T acc = T(0);
        for (int e = o1[j1], e1 = o1[j1 + 1]; e < e1; ++e) acc = A::fma(SW[e], src[SE[e]], acc);
        SB[k] = acc;
      }
      __syncthreads();
      for (int k = tid; k < nC; k += nt) {  // C[(i3 f2 + j2) f1 + j1]
        const int i3 = k / (f1 * f2), r = k - i3 * (f1 * f2), j2 = r / f1, j1 = r - j2 * f1;
        const T *src = SB + i3 * n2 * f1 + j1;
        T acc = T(0);
        for (int e = o2[j2], e1 = o2[j2 + 1]; e < e1; ++e)
          acc = A::fma(SW[e], src[SE[e] * f1], acc);
        SC[k] = acc;
      }
      __syncthreads();
      T *ov = out + (int64_t)v * h.fsize;
      for (int k = tid; k < nO; k += nt) {  // box[(j3 f2 + j2) f1 + j1]
        const int j3 = k / (f1 * f2), r = k - j3 * (f1 * f2);
        const T *src = SC + r;
        T acc = T(0);
        for (int e = o3[j3], e1 = o3[j3 + 1]; e < e1; ++e)
          acc = A::fma(SW[e], src[SE[e] * f1 * f2], acc);
        ov[k] = acc;
      }
      __syncthreads();
    }
  }
}

// Pass 2: one CTA per source block and variable (blockIdx.y; the variables'
// adds are independent), its transfers' boxes added in waves (AdjReduce), so
// every point takes its adds in transfer order.  A block read by a turned
// transfer, which moves a variable onto another, is one CTA's for every
// variable.  An odd turn adds onto the block of the alternate array `yalt` (a
// RotationPair's partner: the same block and variable strides, the plane's
// extents swapped, which the turn's strides carry; or y itself), so every
// add into either array's block is this CTA's, in transfer order.
template <typename T, int D, bool BATCH>
__global__ void __launch_bounds__(256) adjoint_reduce_kernel(
    const AdjReduce *__restrict__ red, int64_t nred, const int2 *__restrict__ list,
    const uint8_t *__restrict__ wend, AdjArgs<T> a, T *y, T *yalt, const T *scratch,
    const T *__restrict__ factors, int nvars, int S1, int S2, int S3) {
  using A = AArith<T>;
  for (int64_t b = blockIdx.x; b < nred; b += gridDim.x) {
    const AdjReduce r = red[b];
    if (r.turned && blockIdx.y != 0) continue;
    const int vlo = r.turned ? 0 : (int)blockIdx.y, vn = r.turned ? nvars : 1;
    // the transfers reading one block all belong to its forest
    const int member = a.groups[list[r.first].y].member;
    const AdjLayout<T, BATCH> L(a, member, y, factors, nvars, S1, S2, S3);
    const AdjLayout<T, BATCH> La(a, member, yalt, nullptr, nvars, S1, S2, S3);
    for (int q = 0; q < r.count; ++q) {
      const int2 tg = list[r.first + q];  // (transfer, group)
      const AdjGroup &h = a.ag[tg.y];
      T *yb = ((h.col & 1) ? La.y : L.y) + (int64_t)r.sblock * L.bs;
      const int64_t n = h.fsize * vn;
      const int f0 = h.fn[0], f01 = h.fn[0] * h.fn[1];
      if (h.direct) {
        // the target box in place: footprint point j reads target row
        // j or n - 1 - j (a mirror) in each dimension, +0 + f * y
        const DevGroup &g = a.groups[tg.y];
        const T *yt = L.y + (int64_t)(__ldg(a.tb + tg.x) - 1) * L.bs;
        const T *fc = g.factorcol ? L.factors + (int64_t)nvars * (g.factorcol - 1) : nullptr;
        for (int64_t p = threadIdx.x; p < n; p += blockDim.x) {
          const int vq = (int)(p / h.fsize);
          const int pt = (int)(p - (int64_t)vq * h.fsize);
          const int v = vlo + vq;
          const int j3 = pt / f01;
          const int rr = pt - j3 * f01;
          const int j2 = rr / f0;
          const int j1 = rr - j2 * f0;
          const int i1 = g.cstep[0] < 0 ? g.n[0] - 1 - j1 : j1;
          const int i2 = g.cstep[1] < 0 ? g.n[1] - 1 - j2 : j2;
          const int i3 = g.cstep[2] < 0 ? g.n[2] - 1 - j3 : j3;
          T x = yt[v * L.vs + (g.tf[0] + i1) + (int64_t)(g.tf[1] + i2) * L.s2 +
                   (int64_t)(g.tf[2] + i3) * L.s3];
          if (fc) x = A::mul(x, __ldg(fc + v));
          x = A::add(x, T(0));
          T *dst = yb + v * L.vs + (h.flo[0] + j1) + (int64_t)(h.flo[1] + j2) * L.s2 +
                   (int64_t)(h.flo[2] + j3) * L.s3;
          *dst = A::add(*dst, x);
        }
      } else {
        const T *src = scratch + __ldg(a.scr + tg.x) * nvars + (int64_t)vlo * h.fsize;
        for (int64_t p = threadIdx.x; p < n; p += blockDim.x) {
          const int vq = (int)(p / h.fsize);
          const int pt = (int)(p - (int64_t)vq * h.fsize);
          const int v = vlo + vq;
          const int j3 = pt / f01;
          const int rr = pt - j3 * f01;
          const int j2 = rr / f0;
          const int j1 = rr - j2 * f0;
          T *dst;
          if (h.col) {  // a turned group: through the axis map and the variable table
            const int sv = __ldg(a.rotvars + v + (int64_t)nvars * h.col) - 1;
            if (sv < 0 || sv >= nvars) {  // a table naming no variable: skip, and say so
              if (a.err) atomicExch(a.err, (int32_t)TAM_EINVAL);
              continue;
            }
            dst = yb + sv * L.vs + h.tc0 + h.tvs[0] * (h.flo[0] + j1) +
                  h.tvs[1] * (h.flo[1] + j2) + h.tvs[2] * (h.flo[2] + j3);
          } else {
            dst = yb + v * L.vs + (h.flo[0] + j1) + (int64_t)(h.flo[1] + j2) * L.s2 +
                  (int64_t)(h.flo[2] + j3) * L.s3;
          }
          *dst = A::add(*dst, src[p]);
        }
      }
      // the next wave may add onto points this one did
      if (wend[r.first + q]) __syncthreads();
    }
  }
}

// Zero the targets of a stage: the forward tiles of the stage.
template <typename T, int D, bool BATCH>
__global__ void __launch_bounds__(256) adjoint_zero_kernel(const Tile *__restrict__ tiles,
                                                           int64_t ntiles, AdjArgs<T> a, T *y,
                                                           int nvars, int S1, int S2, int S3) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < ntiles;
       w += warps) {
    const Tile tile = tiles[w];
    const DevGroup &g = a.groups[tile.group];
    const AdjLayout<T, BATCH> L(a, g.member, y, nullptr, nvars, S1, S2, S3);
    const int64_t tblock = __ldg(a.tb + tile.transfer) - 1;
    const int n1 = g.n[0], n12 = g.n[0] * g.n[1];
    for (int k = lane; k < tile.nitems; k += 32) {
      const int item = tile.item0 + k;
      const int i3 = item / n12;
      const int rem = item - i3 * n12;
      const int i2 = rem / n1;
      const int i1 = rem - i2 * n1;
      const int64_t o = tblock * L.bs + (g.tf[0] + i1) + (int64_t)(g.tf[1] + i2) * L.s2 +
                        (int64_t)(g.tf[2] + i3) * L.s3;
      for (int v = 0; v < nvars; ++v) L.y[o + v * L.vs] = T(0);
    }
  }
}

// Zero the targets of a stage's turned groups (they have no forward tiles):
// group turns[blockIdx.y], every transfer, point and variable; in a batch of
// forests at its member's place in the arena.
template <typename T>
__global__ void __launch_bounds__(256)
    adjoint_zero_solo_kernel(const SoloGroup *__restrict__ turns, const DevGroup *groups,
                               const Member *__restrict__ members,
                               const int32_t *__restrict__ tb, T *y, int nvars, int S1, int S2,
                               int S3) {
  const DevGroup &g = groups[turns[blockIdx.y].group];
  if (members) {
    const Member &m = members[g.member];
    y += m.work_off;
    S1 = m.S[0];
    S2 = m.S[1];
    S3 = m.S[2];
  }
  const int64_t box = (int64_t)g.n[0] * g.n[1] * g.n[2];
  const int64_t items = box * nvars * g.ntransfers;
  const int64_t vol = (int64_t)S1 * S2 * S3;
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
    y[(tblock * nvars + v) * vol + ((int64_t)(g.tf[2] + i3) * S2 + (g.tf[1] + i2)) * S1 +
      g.tf[0] + i1] = T(0);
  }
}

template <typename T, int D, bool BATCH>
cudaError_t run_typed(const AdjPlan &p, const AdjRun &r, T *y, int nvars, const T *factors,
                      int32_t first, int32_t last, T *scratch, cudaStream_t stream) {
  const AdjArgs<T> a{r.groups, p.groups,           r.tb,  (const T *)r.weights,
                     p.off,    (const int2 *)p.ent, p.scr, r.members,
                     r.rotvars, r.err};
  const int S1 = r.S[0], S2 = r.S[1], S3 = r.S[2];
  const int threads = 256, wpb = threads / 32;
  // stages in reverse order
  for (int k = (int)p.stages.size() - 1; k >= 0; --k) {
    const AdjStage &st = p.stages[k];
    if (st.tag < first || st.tag > last) continue;
    const Stage &fw = (*r.fwd_stages)[k];
    for (const AdjPass1 &pc : st.p1) {
      if (pc.count == 0) continue;
      const size_t smem = (size_t)pc.smem_elems * sizeof(T) +
                          (size_t)pc.csr_ents * (sizeof(T) + sizeof(int)) +
                          (size_t)pc.csr_rows * sizeof(int);
      if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(adjoint_box_kernel<T, D, BATCH>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
      }
      const int64_t blocks = std::min<int64_t>(pc.count, (int64_t)1 << 30);
      if (nvars > 65535) return cudaErrorInvalidValue;  // a CTA row per variable
      adjoint_box_kernel<T, D, BATCH><<<dim3((unsigned)blocks, (unsigned)nvars), 128, smem,
                                       stream>>>(
          (const int2 *)p.xfers + pc.first, pc.count, a, y, scratch, factors, nvars, S1, S2,
          S3, (int)pc.smem_elems, (int)pc.csr_ents);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
    if (st.nred > 0) {
      if (nvars > 65535) return cudaErrorInvalidValue;  // a CTA row per variable
      const int64_t blocks = std::min<int64_t>(st.nred, (int64_t)1 << 30);
      adjoint_reduce_kernel<T, D, BATCH><<<dim3((unsigned)blocks, (unsigned)nvars), threads, 0,
                                           stream>>>(
          p.red + st.red0, st.nred, (const int2 *)p.list, p.wend, a, y,
          r.alt ? (T *)r.alt : y, scratch, factors, nvars, S1, S2, S3);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
    if (fw.ntiles > 0) {
      const int64_t blocks = std::min<int64_t>((fw.ntiles + wpb - 1) / wpb, (int64_t)1 << 30);
      adjoint_zero_kernel<T, D, BATCH><<<(unsigned)blocks, threads, 0, stream>>>(
          r.fwd_tiles + fw.tile0, fw.ntiles, a, y, nvars, S1, S2, S3);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
    if (fw.nsolo > 0 && r.turns) {
      adjoint_zero_solo_kernel<T><<<dim3(64, (unsigned)fw.nsolo), threads, 0, stream>>>(
          r.turns + fw.solo0, r.groups, r.members, r.tb, y, nvars, S1, S2, S3);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
  }
  return cudaSuccess;
}

template <typename T, bool BATCH>
cudaError_t run_dim(const AdjPlan &p, const AdjRun &r, void *y, int nvars, const void *factors,
                    int32_t first, int32_t last, void *scratch, cudaStream_t stream) {
  switch (r.D) {
    case 1:
      return run_typed<T, 1, BATCH>(p, r, (T *)y, nvars, (const T *)factors, first, last,
                                    (T *)scratch, stream);
    case 2:
      return run_typed<T, 2, BATCH>(p, r, (T *)y, nvars, (const T *)factors, first, last,
                                    (T *)scratch, stream);
    default:
      return run_typed<T, 3, BATCH>(p, r, (T *)y, nvars, (const T *)factors, first, last,
                                    (T *)scratch, stream);
  }
}

template <typename T>
cudaError_t up(T **dst, const std::vector<T> &v) {
  *dst = nullptr;
  size_t n = std::max<size_t>(v.size(), 1);
  cudaError_t e = cudaMalloc((void **)dst, n * sizeof(T));
  if (e != cudaSuccess) return e;
  if (!v.empty()) return cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  return cudaSuccess;
}

// The plan of one schedule on the host.
struct AdjHost {
  std::vector<AdjGroup> ag;
  std::vector<int32_t> off;
  std::vector<int2> ent;
  std::vector<int64_t> scr;      // per transfer
  std::vector<int2> xfers;       // per stage, by target block
  std::vector<AdjReduce> red;
  std::vector<int2> list;
  std::vector<uint8_t> wend;     // per list entry: 1 ends a wave
  std::vector<AdjStage> stages;  // one per forward stage
  int64_t maxpts = 0;
};

size_t smem_limit() {
  int dev = 0, optin = 48 * 1024;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return (size_t)optin;
}

// The transposed stencils, the pass-1 transfer lists and the pass-2 lists of
// one schedule.
int adjoint_build(const tam_sched *s, AdjHost &o, std::string &err) {
  const int D = s->D;
  o.ag.assign(s->groups.size(), AdjGroup{});
  for (size_t gi = 0; gi < s->groups.size(); ++gi) {
    const tam_group &h = s->host_groups[gi];
    const DevGroup &g = s->groups[gi];
    AdjGroup &a = o.ag[gi];
    a.fsize = 1;
    for (int d = 0; d < 3; ++d) {
      if (d >= D) {
        a.flo[d] = 0;
        a.fn[d] = 1;
        a.off[d] = (int64_t)o.off.size();
        o.off.push_back((int32_t)o.ent.size());
        o.ent.push_back(make_int2(0, (int32_t)g.w[d]));  // the weight pool's pad one
        o.off.push_back((int32_t)o.ent.size());
        continue;
      }
      const tam_stencil &st = h.stencil[d];
      int lo = INT32_MAX, hi = INT32_MIN;
      for (int i = 0; i < st.ntarget; ++i) {
        const int b = s->h_srcstart[st.srcstart + i] - 1;
        lo = std::min(lo, b);
        hi = std::max(hi, b + st.order - 1);
      }
      a.flo[d] = lo;
      a.fn[d] = hi - lo + 1;
      a.off[d] = (int64_t)o.off.size();
      for (int r = lo; r <= hi; ++r) {
        o.off.push_back((int32_t)o.ent.size());
        for (int i = 0; i < st.ntarget; ++i) {
          const int b = s->h_srcstart[st.srcstart + i] - 1;
          const int m = r - b;
          if (m < 0 || m >= st.order) continue;
          const int64_t w = g.w[d] + (int64_t)st.order * i + m;
          if (w > INT32_MAX) {
            err = "a weight pool too large for the adjoint's entries";
            return TAM_EUNSUPPORTED;
          }
          o.ent.push_back(make_int2(i, (int32_t)w));
        }
      }
      o.off.push_back((int32_t)o.ent.size());
      a.fsize *= a.fn[d];
    }
    if (o.ent.size() > (size_t)INT32_MAX) {
      err = "the adjoint's transposed stencils exceed 2^31 entries";
      return TAM_EUNSUPPORTED;
    }
    a.direct = g.pclass == 0 && g.affine && !g.turned && (g.n[0] == 1 || g.cstep[0] != 0) &&
               (g.n[1] == 1 || g.cstep[1] != 0) && (g.n[2] == 1 || g.cstep[2] != 0);
  }
  // turned groups: their footprints land on the real source through the
  // strides the forward launch reads it by
  for (const SoloGroup &t : s->h_solos) {
    AdjGroup &a = o.ag[t.group];
    a.col = t.col;
    for (int d = 0; d < 3; ++d) a.tvs[d] = t.vs[d];
    a.tc0 = t.c0;
  }
  o.scr.assign(s->ntransfers, 0);
  for (const Stage &fw : s->stages) {
    AdjStage st;
    st.tag = fw.tag;
    st.red0 = (int64_t)o.red.size();
    struct E {
      int32_t tblock, sblock, group, transfer;
    };
    std::vector<E> es;
    for (int32_t gi : fw.groups) {
      const DevGroup &g = s->groups[gi];
      for (int64_t t = 0; t < g.ntransfers; ++t)
        es.push_back({s->h_tb[g.first + t], s->h_sb[g.first + t], gi, (int32_t)(g.first + t)});
    }
    // scratch in transfer order
    std::vector<E> byt = es;
    std::sort(byt.begin(), byt.end(), [](const E &x, const E &y) { return x.transfer < y.transfer; });
    int64_t pts = 0;
    for (const E &e : byt) {  // a direct copy needs none
      o.scr[e.transfer] = pts;
      if (!o.ag[e.group].direct) pts += o.ag[e.group].fsize;
    }
    st.scratch_points = pts;
    o.maxpts = std::max(o.maxpts, pts);
    // pass-1 transfers by size class, then by target block; each class's
    // shared memory is that of its largest box
    std::vector<int64_t> gsm(s->groups.size(), 0), gents(s->groups.size(), 0),
        grows(s->groups.size(), 0);
    std::vector<int> gcls(s->groups.size(), 0);
    for (int32_t gi : fw.groups) {
      const DevGroup &g = s->groups[gi];
      const AdjGroup &a = o.ag[gi];
      if (a.direct) continue;  // no pass 1
      // the larger of the target box and the second pass (which takes its
      // place), and the first pass
      gsm[gi] = std::max((int64_t)g.n[0] * g.n[1] * g.n[2], (int64_t)a.fn[0] * a.fn[1] * g.n[2]) +
                (int64_t)a.fn[0] * g.n[1] * g.n[2];
      for (int d = 0; d < 3; ++d) {
        gents[gi] += o.off[a.off[d] + a.fn[d]] - o.off[a.off[d]];
        grows[gi] += a.fn[d] + 1;
      }
      const int64_t bytes = 8 * gsm[gi] + 12 * gents[gi] + 4 * grows[gi];
      while (gcls[gi] < kAdjClasses - 1 && bytes > kAdjClassBytes[gcls[gi]]) ++gcls[gi];
    }
    std::stable_sort(es.begin(), es.end(), [&](const E &x, const E &y) {
      if (gcls[x.group] != gcls[y.group]) return gcls[x.group] < gcls[y.group];
      return x.tblock != y.tblock ? x.tblock < y.tblock : x.group < y.group;
    });
    for (int c = 0; c < kAdjClasses; ++c) {
      AdjPass1 &pc = st.p1[c];
      pc.first = (int64_t)o.xfers.size();
      for (const E &e : es) {  // (a direct copy has no pass-1 work)
        if (o.ag[e.group].direct || gcls[e.group] != c) continue;
        o.xfers.push_back(make_int2(e.transfer, e.group));
        pc.smem_elems = std::max(pc.smem_elems, gsm[e.group]);
        pc.csr_ents = std::max(pc.csr_ents, gents[e.group]);
        pc.csr_rows = std::max(pc.csr_rows, grows[e.group]);
      }
      pc.count = (int64_t)o.xfers.size() - pc.first;
    }
    // pass-2 lists by source block, transfers in transfer order (a block's
    // list holds the odd turns that read the alternate array's block too)
    std::sort(byt.begin(), byt.end(), [](const E &x, const E &y) {
      return x.sblock != y.sblock ? x.sblock < y.sblock : x.transfer < y.transfer;
    });
    for (size_t i = 0; i < byt.size();) {
      size_t j = i;
      while (j < byt.size() && byt[j].sblock == byt[i].sblock) ++j;
      bool turned = false;
      for (size_t k = i; k < j; ++k) turned = turned || o.ag[byt[k].group].col != 0;
      o.red.push_back({byt[i].sblock - 1, (int32_t)(j - i), (int64_t)o.list.size(),
                       turned ? 1 : 0, 0});
      // waves: a transfer goes one past the last wave of an earlier one whose
      // footprint it meets (a turned one meets every other: its footprint
      // lands through the turn, and an odd turn on the partner's array)
      std::vector<int> wave(j - i, 0);
      auto meets = [&](const E &p, const E &q) {
        const AdjGroup &x = o.ag[p.group], &y = o.ag[q.group];
        if (x.col || y.col) return true;
        for (int d = 0; d < 3; ++d)
          if (x.flo[d] + x.fn[d] <= y.flo[d] || y.flo[d] + y.fn[d] <= x.flo[d]) return false;
        return true;
      };
      for (size_t k = i; k < j; ++k)
        for (size_t l = i; l < k; ++l)
          if (wave[l - i] >= wave[k - i] && meets(byt[l], byt[k])) wave[k - i] = wave[l - i] + 1;
      std::vector<size_t> ord(j - i);
      for (size_t k = 0; k < ord.size(); ++k) ord[k] = k;
      std::stable_sort(ord.begin(), ord.end(),
                       [&](size_t x, size_t y) { return wave[x] < wave[y]; });
      for (size_t k = 0; k < ord.size(); ++k) {
        const E &e = byt[i + ord[k]];
        o.list.push_back(make_int2(e.transfer, e.group));
        o.wend.push_back(k + 1 == ord.size() || wave[ord[k + 1]] != wave[ord[k]] ? 1 : 0);
      }
      i = j;
    }
    st.nred = (int64_t)o.red.size() - st.red0;
    o.stages.push_back(st);
  }
  return TAM_OK;
}

int upload_plan(AdjPlan &p, const AdjHost &o, int dtype, std::string &err) {
  const size_t esz = dtype == TAM_F64 ? 8 : 4, limit = smem_limit();
  for (const AdjStage &st : o.stages)
    for (const AdjPass1 &pc : st.p1)
      if ((size_t)pc.smem_elems * esz + (size_t)pc.csr_ents * (esz + 4) +
              (size_t)pc.csr_rows * 4 >
          limit) {
        err = "a transfer box too large for the adjoint's shared memory";
        return TAM_EUNSUPPORTED;
      }
  cudaError_t e;
  if ((e = up(&p.groups, o.ag)) != cudaSuccess || (e = up(&p.off, o.off)) != cudaSuccess ||
      (e = up((int2 **)&p.ent, o.ent)) != cudaSuccess || (e = up(&p.scr, o.scr)) != cudaSuccess ||
      (e = up((int2 **)&p.xfers, o.xfers)) != cudaSuccess || (e = up(&p.red, o.red)) != cudaSuccess ||
      (e = up((int2 **)&p.list, o.list)) != cudaSuccess ||
      (e = up(&p.wend, o.wend)) != cudaSuccess) {
    adjoint_plan_free(p);
    err = std::string("adjoint upload: ") + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? TAM_ENOMEM : TAM_ECUDA;
  }
  p.stages = o.stages;
  p.scratch_points = o.maxpts;
  p.ready = true;
  return TAM_OK;
}

}  // namespace

void adjoint_plan_free(AdjPlan &p) {
  cudaFree(p.groups);
  cudaFree(p.off);
  cudaFree(p.ent);
  cudaFree(p.scr);
  cudaFree(p.xfers);
  cudaFree(p.red);
  cudaFree(p.list);
  cudaFree(p.wend);
  p = AdjPlan{};
}

int adjoint_prepare(tam_sched *s, std::string &err) {
  if (s->adj.ready) return TAM_OK;
  AdjHost o;
  int rc = adjoint_build(s, o, err);
  if (rc != TAM_OK) return rc;
  return upload_plan(s->adj, o, s->dtype, err);
}

// Concatenate the members' plans: indices into groups, transfers, weights,
// CSR rows and entries and the reduction lists move by each member's bases;
// per stage tag the members' transfers follow one another, and so do their
// scratch boxes.
int adjoint_prepare_batch(AdjPlan &plan, const std::vector<tam_sched *> &members,
                          const std::vector<int64_t> &group_base,
                          const std::vector<int64_t> &transfer_base,
                          const std::vector<int64_t> &weight_base,
                          const std::vector<Stage> &stages, std::string &err) {
  if (plan.ready) return TAM_OK;
  const int dtype = members.empty() ? TAM_F64 : members[0]->dtype;
  std::vector<AdjHost> hs(members.size());
  AdjHost o;
  std::vector<int64_t> list_base(members.size());
  for (size_t m = 0; m < members.size(); ++m) {
    int rc = adjoint_build(members[m], hs[m], err);
    if (rc != TAM_OK) return rc;
    const AdjHost &h = hs[m];
    const int64_t off0 = (int64_t)o.off.size(), ent0 = (int64_t)o.ent.size();
    for (AdjGroup a : h.ag) {
      for (int d = 0; d < 3; ++d) a.off[d] += off0;
      o.ag.push_back(a);
    }
    for (int32_t v : h.off) o.off.push_back((int32_t)(v + ent0));
    for (int2 e : h.ent) {
      const int64_t w = e.y + weight_base[m];
      if (w > INT32_MAX) {
        err = "the batch's weight pool is too large for the adjoint's entries";
        return TAM_EUNSUPPORTED;
      }
      o.ent.push_back(make_int2(e.x, (int32_t)w));
    }
    if (o.ent.size() > (size_t)INT32_MAX || o.off.size() > (size_t)INT32_MAX) {
      err = "the batch's transposed stencils exceed 2^31 entries";
      return TAM_EUNSUPPORTED;
    }
  }
  int64_t ntransfers = 0;
  for (size_t m = 0; m < members.size(); ++m)
    ntransfers = std::max<int64_t>(ntransfers, transfer_base[m] + members[m]->ntransfers);
  o.scr.assign(ntransfers, 0);
  for (const Stage &fw : stages) {
    AdjStage st;
    st.tag = fw.tag;
    st.red0 = (int64_t)o.red.size();
    // each member's stage of this tag, and where its scratch starts
    std::vector<const AdjStage *> mst(members.size(), nullptr);
    std::vector<int64_t> base(members.size() + 1, 0);
    for (size_t m = 0; m < members.size(); ++m) {
      const tam_sched *s = members[m];
      size_t k = 0;
      while (k < s->stages.size() && s->stages[k].tag != fw.tag) ++k;
      if (k < s->stages.size()) mst[m] = &hs[m].stages[k];
      base[m + 1] = base[m] + (mst[m] ? mst[m]->scratch_points : 0);
    }
    // pass 1: the members' transfers class by class
    for (int c = 0; c < kAdjClasses; ++c) {
      AdjPass1 &pc = st.p1[c];
      pc.first = (int64_t)o.xfers.size();
      for (size_t m = 0; m < members.size(); ++m) {
        if (!mst[m]) continue;
        const AdjHost &h = hs[m];
        const AdjPass1 &mc = mst[m]->p1[c];
        const int32_t G0 = (int32_t)group_base[m], T0 = (int32_t)transfer_base[m];
        for (int64_t i = mc.first; i < mc.first + mc.count; ++i) {
          const int2 x = h.xfers[i];
          o.xfers.push_back(make_int2(x.x + T0, x.y + G0));
          o.scr[x.x + T0] = base[m] + h.scr[x.x];
        }
        pc.smem_elems = std::max(pc.smem_elems, mc.smem_elems);
        pc.csr_ents = std::max(pc.csr_ents, mc.csr_ents);
        pc.csr_rows = std::max(pc.csr_rows, mc.csr_rows);
      }
      pc.count = (int64_t)o.xfers.size() - pc.first;
    }
    // pass 2: the members' source blocks
    for (size_t m = 0; m < members.size(); ++m) {
      if (!mst[m]) continue;
      const AdjHost &h = hs[m];
      const AdjStage &ms = *mst[m];
      const int32_t G0 = (int32_t)group_base[m], T0 = (int32_t)transfer_base[m];
      for (int64_t i = ms.red0; i < ms.red0 + ms.nred; ++i) {
        AdjReduce r = h.red[i];
        const int64_t first = (int64_t)o.list.size();
        for (int32_t q = 0; q < r.count; ++q) {
          const int2 x = h.list[r.first + q];
          o.list.push_back(make_int2(x.x + T0, x.y + G0));
          o.wend.push_back(h.wend[r.first + q]);
        }
        r.first = first;
        o.red.push_back(r);
      }
    }
    st.nred = (int64_t)o.red.size() - st.red0;
    st.scratch_points = base[members.size()];
    o.maxpts = std::max(o.maxpts, st.scratch_points);
    o.stages.push_back(st);
  }
  return upload_plan(plan, o, dtype, err);
}

void adjoint_free(tam_sched *s) {
  adjoint_plan_free(s->adj);
  cudaFree(s->adj_scratch);
  s->adj_scratch = nullptr;
  s->adj_scratch_bytes = 0;
}

cudaError_t adjoint_run_plan(const AdjPlan &plan, const AdjRun &r, void *y, int nvars,
                             const void *factors, int32_t first, int32_t last, void *scratch,
                             cudaStream_t stream) {
  const bool batch = r.members != nullptr;
  if (r.dtype == TAM_F64)
    return batch ? run_dim<double, true>(plan, r, y, nvars, factors, first, last, scratch, stream)
                 : run_dim<double, false>(plan, r, y, nvars, factors, first, last, scratch, stream);
  return batch ? run_dim<float, true>(plan, r, y, nvars, factors, first, last, scratch, stream)
               : run_dim<float, false>(plan, r, y, nvars, factors, first, last, scratch, stream);
}

cudaError_t adjoint_run(tam_sched *s, void *y, void *alt, int nvars, const void *factors,
                        const int32_t *rotvars, int32_t first, int32_t last, void *scratch,
                        cudaStream_t stream) {
  AdjRun r{s->dtype, s->D, s->d_groups, s->d_tb, s->d_weights, nullptr, s->d_tiles,
           &s->stages, {s->S[0], s->S[1], s->S[2]}, s->d_solos, rotvars, s->d_err,
           alt ? alt : y};
  // stages from the last down to 0 transposed, then stage P (diagonal) forward
  const bool p = first <= TAM_STAGE_SELFIMAGE && TAM_STAGE_SELFIMAGE <= last;
  cudaError_t e = adjoint_run_plan(s->adj, r, y, nvars, factors,
                                   p ? TAM_STAGE_SELFIMAGE + 1 : first, last, scratch, stream);
  if (e != cudaSuccess || !p) return e;
  return fill_one_stage(s, y, nvars, factors, TAM_STAGE_SELFIMAGE, stream);
}

}  // namespace tam

// ---- the adjoint without allocation -----------------------------------------
//
// Scratch for tam_fill_adjoint_static: one fixed array per GPU that loads the
// library, held until the process exits.  In host code the name is only a
// host-side handle, never a device address, so each device's address is
// looked up once with that device current and kept below.
static __device__ __align__(256) unsigned char g_adjoint_static_scratch[TAM_STATIC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_static_mutex;
void *g_static_ptr[kMaxDevices] = {};

}  // namespace

extern "C" int tam_fill_adjoint_static(tam_sched *s, void *y, int32_t nvars, int64_t nblocks,
                                       const void *factors, int32_t first_stage,
                                       int32_t last_stage, void *stream) {
  if (!s) return tam::record_error(nullptr, TAM_EINVAL, "tam_fill_adjoint_static: NULL schedule");
  tam_ctx *ctx = s->ctx;
  if (!y || nvars < 1) {
    ctx->err = "tam_fill_adjoint_static: NULL vector or no variables";
    return TAM_EINVAL;
  }
  if (nblocks != s->nblocks) {
    ctx->err = "tam_fill_adjoint_static: the block count differs from the schedule's";
    return TAM_ELAYOUT;
  }
  if (s->needs_factors && !factors) {
    ctx->err = "tam_fill_adjoint_static: this schedule mirrors ghosts and needs the factor table";
    return TAM_EINVAL;
  }
  if (!s->adj.ready) {
    ctx->err = "tam_fill_adjoint_static: the schedule's transposed stencils are not built; "
               "call tam_adjoint_scratch_bytes once first (it allocates)";
    return TAM_EINVAL;
  }
  if (s->needs_rotvars) {
    ctx->err = "tam_fill_adjoint_static: this schedule turns transfers across a seam; "
               "use tam_fill_adjoint_ex with the variable table";
    return TAM_EINVAL;
  }
  const size_t need = (size_t)s->adj.scratch_points * nvars * (s->dtype == TAM_F64 ? 8 : 4);
  if (need > TAM_STATIC_SCRATCH_BYTES) {
    ctx->err = "tam_fill_adjoint_static: this schedule's adjoint needs " + std::to_string(need) +
               " bytes of scratch for " + std::to_string(nvars) +
               " variables, more than the built-in " +
               std::to_string((size_t)TAM_STATIC_SCRATCH_BYTES) +
               "; use tam_fill_adjoint or tam_fill_adjoint_scratch";
    return TAM_EUNSUPPORTED;
  }
  if (ctx->device < 0 || ctx->device >= kMaxDevices) {
    ctx->err = "tam_fill_adjoint_static: device index beyond the library's table";
    return TAM_EUNSUPPORTED;
  }
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess) {
    ctx->err = "tam_fill_adjoint_static: cudaGetDevice failed";
    return TAM_ECUDA;
  }
  if (prev != ctx->device && cudaSetDevice(ctx->device) != cudaSuccess) {
    ctx->err = "tam_fill_adjoint_static: cannot make the schedule's device current";
    return TAM_ECUDA;
  }
  void *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_static_mutex);
    if (!g_static_ptr[ctx->device]) {
      // once per device, with that device current
      cudaError_t e = cudaGetSymbolAddress(&g_static_ptr[ctx->device], g_adjoint_static_scratch);
      if (e != cudaSuccess) {
        g_static_ptr[ctx->device] = nullptr;
        if (prev != ctx->device) cudaSetDevice(prev);
        ctx->err = std::string("tam_fill_adjoint_static: cudaGetSymbolAddress: ") +
                   cudaGetErrorString(e);
        return TAM_ECUDA;
      }
    }
    scratch = g_static_ptr[ctx->device];
  }
  cudaError_t e = tam::adjoint_run(s, y, nullptr, nvars, factors, nullptr, first_stage,
                                   last_stage, scratch, (cudaStream_t)stream);
  if (prev != ctx->device) cudaSetDevice(prev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    ctx->err = std::string("tam_fill_adjoint_static: ") + cudaGetErrorString(e);
    return TAM_ECUDA;
  }
  return TAM_OK;
}
