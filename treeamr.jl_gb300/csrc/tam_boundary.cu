// The cell-wise boundary hook on the device: CellBoundary
// (src/ghosts.jl:1166-1318), with its per-cell function one of a set of
// built-in forms instead of a callback.
//
// A callback written in the caller's language cannot cross a C ABI into a
// compiled kernel, so the functions of position the reference's users write
// most -- a constant state, a polynomial manufactured solution -- are
// built in, each evaluated in a fixed order of single roundings (no fused
// multiply-add) so that a host evaluation in the same order gives the same
// bits.  Every ghost of every region beyond an outer face gets g(x, v) with
// x its position formed exactly as nodeposition forms it
// (src/storage.jl:1008-1017): fma(T(m), s, lo), m = B + I - 1 and s = h along
// a vertex-like dimension, m = 2(B + I - 1) + 1 and s = h/2 along a
// cell-like one.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "tam_internal.h"
#include "treeamr_cuda.h"

namespace {

template <typename T>
struct BArith;
template <>
struct BArith<double> {
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double fma(double a, double b, double c) {
    return __fma_rn(a, b, c);
  }
};
template <>
struct BArith<float> {
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float fma(float a, float b, float c) {
    return __fmaf_rn(a, b, c);
  }
};

// The built-in function at x for variable v.
template <typename T>
__device__ __forceinline__ T eval_fn(const tam_boundary_fn &fn, const T *__restrict__ coef, int v,
                                     const T (&x)[3]) {
  using A = BArith<T>;
  if (fn.kind == TAM_BC_CONSTANT) return coef[v];
  // sum over monomials in table order: ((c * x1^a) * x2^b) * x3^c, each
  // power by repeated multiplication left to right, from +0
  const T *cv = coef + (int64_t)v * fn.nterms;
  T val = T(0);
  for (int q = 0; q < fn.nterms; ++q) {
    T term = cv[q];
#pragma unroll
    for (int d = 0; d < 3; ++d)
      for (int e = 0; e < fn.exps[q][d]; ++e) term = A::mul(term, x[d]);
    val = A::add(val, term);
  }
  return val;
}

// One CTA per region, a thread per (point, variable).
template <typename T>
__global__ void __launch_bounds__(256) boundary_kernel(const tam_boundary_region *__restrict__ regions,
                                                       int32_t nregions, tam_boundary_fn fn,
                                                       const T *__restrict__ coef, T *work,
                                                       int32_t nvars, int S1, int S2, int S3) {
  using A = BArith<T>;
  const int64_t s2 = S1, s3 = (int64_t)S1 * S2, vs = s3 * S3, bs = vs * nvars;
  for (int r = blockIdx.x; r < nregions; r += gridDim.x) {
    const tam_boundary_region R = regions[r];
    const int n1 = R.n[0], n12 = R.n[0] * R.n[1];
    const int total = n12 * R.n[2] * nvars;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      const int v = t / (n12 * R.n[2]);
      const int p = t - v * n12 * R.n[2];
      const int i3 = p / n12, rem = p - i3 * n12, i2 = rem / n1, i1 = rem - i2 * n1;
      const int idx[3] = {R.first[0] + i1, R.first[1] + i2, R.first[2] + i3};  // 1-based
      T x[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const int64_t k = (int64_t)R.base[d] + idx[d] - 1 - R.ghosts[d];
        const bool vertex = R.stagger[d] == 1;
        const T m = vertex ? (T)k : (T)(2 * k + 1);
        const T s = vertex ? (T)R.h : (T)R.h * T(0.5);
        x[d] = A::fma(m, s, (T)R.lo[d]);
      }
      T val = eval_fn(fn, coef, v, x);
      if (fn.relative) {
        // the nearest evolved point: the clamped index along components
        // that leave the domain, the ghost's own along the others
        int r[3];
        T xr[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          r[d] = R.clamps[d] != 0 ? R.clamps[d] : idx[d];
          const int64_t k = (int64_t)R.base[d] + r[d] - 1 - R.ghosts[d];
          const bool vertex = R.stagger[d] == 1;
          const T m = vertex ? (T)k : (T)(2 * k + 1);
          const T s = vertex ? (T)R.h : (T)R.h * T(0.5);
          xr[d] = A::fma(m, s, (T)R.lo[d]);
        }
        const T ur = work[(int64_t)R.block * bs + v * vs + (r[0] - 1) + (int64_t)(r[1] - 1) * s2 +
                          (int64_t)(r[2] - 1) * s3];
        val = A::add(val, A::add(ur, -eval_fn(fn, coef, v, xr)));
      }
      work[(int64_t)R.block * bs + v * vs + (idx[0] - 1) + (int64_t)(idx[1] - 1) * s2 +
           (int64_t)(idx[2] - 1) * s3] = val;
    }
  }
}

}  // namespace

extern "C" int tam_boundary_apply(int32_t dtype, const tam_boundary_region *regions,
                                  int32_t nregions, tam_boundary_fn fn, const void *coef,
                                  void *work, int32_t nvars, const int32_t stored[3],
                                  void *stream) {
  if (nregions < 0 || nvars < 1 || !stored) return TAM_EINVAL;
  if (nregions == 0) return TAM_OK;
  if (!regions || !coef || !work) return TAM_EINVAL;
  if (fn.kind != TAM_BC_CONSTANT && fn.kind != TAM_BC_POLYNOMIAL) return TAM_EINVAL;
  if (fn.kind == TAM_BC_POLYNOMIAL && (fn.nterms < 0 || fn.nterms > TAM_BC_MAX_TERMS))
    return TAM_EINVAL;
  const int blocks = std::min<int32_t>(nregions, 1 << 30);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == TAM_F64)
    boundary_kernel<double><<<blocks, 256, 0, s>>>(regions, nregions, fn, (const double *)coef,
                                                   (double *)work, nvars, stored[0], stored[1],
                                                   stored[2]);
  else if (dtype == TAM_F32)
    boundary_kernel<float><<<blocks, 256, 0, s>>>(regions, nregions, fn, (const float *)coef,
                                                  (float *)work, nvars, stored[0], stored[1],
                                                  stored[2]);
  else
    return TAM_EINVAL;
  return cudaGetLastError() == cudaSuccess ? TAM_OK : TAM_ECUDA;
}
