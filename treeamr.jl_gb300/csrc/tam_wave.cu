// The right-hand side of the second-order wave equation over a batch of
// forests, and its transpose.
//
// The reference's wave test (test/wave.jl:49-110) advances u_t = v,
// v_t = lap(u) with the 7-point Laplacian on each block's owned points after
// a ghost fill.  This is that right-hand side for every block of every forest
// of a batch in one launch, and the transpose of it for the backward pass of a
// differentiated solve; both are gathers, so neither needs atomics.
//
// A block of the table is its field data's offset (variable u; v follows at
// one variable's stride), its stored extents S, ghost width G, owned cells N
// per dimension (cell-centred) and 1/h^2.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "tam_internal.h"
#include "treeamr_cuda.h"

namespace {

template <typename T>
__device__ __forceinline__ T ldg_t(const T *p) {
  return __ldg(p);
}

// out[u] = v and out[v] = lap(u) at every owned point; ghosts of `out` are
// not written.  One thread per (block, owned point).
template <typename T>
__global__ void __launch_bounds__(256) wave_rhs_kernel(const tam_wave_block *__restrict__ blocks,
                                                       int32_t nblocks, const T *__restrict__ in,
                                                       T *__restrict__ out) {
  const int b = blockIdx.x;
  if (b >= nblocks) return;
  const tam_wave_block B = blocks[b];
  const int N = B.N, G = B.G;
  const int own = N * N * N;
  const int64_t s2 = B.S[0], s3 = (int64_t)B.S[0] * B.S[1], vs = s3 * B.S[2];
  const T ih2 = (T)B.inv_h2;
  for (int p = blockIdx.y * blockDim.x + threadIdx.x; p < own; p += gridDim.y * blockDim.x) {
    const int k = p / (N * N), r = p - k * N * N, j = r / N, i = r - j * N;
    const int64_t c = B.off + (G + i) + (G + j) * s2 + (G + k) * s3;
    const T u = ldg_t(in + c);
    const T sum = ((ldg_t(in + c - 1) + ldg_t(in + c + 1)) + (ldg_t(in + c - s2) + ldg_t(in + c + s2))) +
                  (ldg_t(in + c - s3) + ldg_t(in + c + s3));
    out[c] = ldg_t(in + c + vs);                 // d/dt u = v
    out[c + vs] = (sum - T(6) * u) * ih2;        // d/dt v = lap(u)
  }
}

// The transpose: every stored point j of a block gathers
//   a[u][j] = (1/h^2) * sum over its face neighbours i that are owned of o[v][i]
//             - 6/h^2 * o[v][j]            (j owned)
//   a[v][j] = o[u][j]                      (j owned; 0 at a ghost)
template <typename T>
__global__ void __launch_bounds__(256) wave_rhs_adjoint_kernel(
    const tam_wave_block *__restrict__ blocks, int32_t nblocks, const T *__restrict__ o,
    T *__restrict__ a) {
  const int b = blockIdx.x;
  if (b >= nblocks) return;
  const tam_wave_block B = blocks[b];
  const int N = B.N, G = B.G;
  const int S1 = B.S[0], S2 = B.S[1], S3 = B.S[2];
  const int total = S1 * S2 * S3;
  const int64_t s2 = S1, s3 = (int64_t)S1 * S2, vs = s3 * S3;
  const T ih2 = (T)B.inv_h2;
  for (int p = blockIdx.y * blockDim.x + threadIdx.x; p < total; p += gridDim.y * blockDim.x) {
    const int k = p / (S1 * S2), r = p - k * S1 * S2, j = r / S1, i = r - j * S1;
    auto owned = [&](int x, int y, int z) {
      return x >= G && x < G + N && y >= G && y < G + N && z >= G && z < G + N;
    };
    const int64_t c = B.off + p;
    T acc = T(0);
    if (owned(i - 1, j, k)) acc += ldg_t(o + vs + c - 1);
    if (owned(i + 1, j, k)) acc += ldg_t(o + vs + c + 1);
    if (owned(i, j - 1, k)) acc += ldg_t(o + vs + c - s2);
    if (owned(i, j + 1, k)) acc += ldg_t(o + vs + c + s2);
    if (owned(i, j, k - 1)) acc += ldg_t(o + vs + c - s3);
    if (owned(i, j, k + 1)) acc += ldg_t(o + vs + c + s3);
    const bool me = owned(i, j, k);
    a[c] = acc * ih2 - (me ? T(6) * ih2 * ldg_t(o + vs + c) : T(0));
    a[c + vs] = me ? ldg_t(o + c) : T(0);
  }
}

// One stage of classical RK4 around the right-hand side, at every stored
// point of every block: k = R(x) (zero at a ghost, as the plain right-hand
// side leaves a zeroed k there), then
//   t_out = y + ct * k            (when t_out is given)
//   acc_out = (acc_in or y) + ca * k
// so a step's stage states and its weighted sum are formed without storing
// k.  x's ghosts must be filled.  acc_out may be acc_in; neither aliases x.
template <typename T>
__global__ void __launch_bounds__(256) wave_rk4_stage_kernel(
    const tam_wave_block *__restrict__ blocks, int32_t nblocks, const T *__restrict__ x,
    const T *y, T *t_out, const T *acc_in, T *acc_out, T ct, T ca) {
  const int b = blockIdx.x;
  if (b >= nblocks) return;
  const tam_wave_block B = blocks[b];
  const int N = B.N, G = B.G;
  const int S1 = B.S[0], S2 = B.S[1], S3 = B.S[2];
  const int total = S1 * S2 * S3;
  const int64_t s2 = S1, s3 = (int64_t)S1 * S2, vs = s3 * S3;
  const T ih2 = (T)B.inv_h2;
  for (int p = blockIdx.y * blockDim.x + threadIdx.x; p < total; p += gridDim.y * blockDim.x) {
    const int k = p / (S1 * S2), r = p - k * S1 * S2, j = r / S1, i = r - j * S1;
    const bool own = i >= G && i < G + N && j >= G && j < G + N && k >= G && k < G + N;
    const int64_t c = B.off + p;
    T ku = T(0), kv = T(0);
    if (own) {
      const T u = ldg_t(x + c);
      const T sum = ((ldg_t(x + c - 1) + ldg_t(x + c + 1)) + (ldg_t(x + c - s2) + ldg_t(x + c + s2))) +
                    (ldg_t(x + c - s3) + ldg_t(x + c + s3));
      ku = ldg_t(x + c + vs);
      kv = (sum - T(6) * u) * ih2;
    }
    const T yu = y[c], yv = y[c + vs];
    if (t_out) {
      t_out[c] = yu + ct * ku;
      t_out[c + vs] = yv + ct * kv;
    }
    const T au = acc_in ? acc_in[c] : yu, av = acc_in ? acc_in[c + vs] : yv;
    acc_out[c] = au + ca * ku;
    acc_out[c + vs] = av + ca * kv;
  }
}

// The transpose of one RK4 stage's right-hand side with its cotangent
// formed on the fly: out = R^T kb, kb = c1 * g + c2 * xprev (xprev may be
// NULL), and, when ybar is given, ybar += xprev at every stored point (the
// previous stage's contribution, added in stage order).  out may alias
// neither g nor xprev.
template <typename T>
__global__ void __launch_bounds__(256) wave_rk4_adjoint_stage_kernel(
    const tam_wave_block *__restrict__ blocks, int32_t nblocks, const T *__restrict__ g, T c1,
    const T *__restrict__ xprev, T c2, T *__restrict__ out, T *ybar) {
  const int b = blockIdx.x;
  if (b >= nblocks) return;
  const tam_wave_block B = blocks[b];
  const int N = B.N, G = B.G;
  const int S1 = B.S[0], S2 = B.S[1], S3 = B.S[2];
  const int total = S1 * S2 * S3;
  const int64_t s2 = S1, s3 = (int64_t)S1 * S2, vs = s3 * S3;
  const T ih2 = (T)B.inv_h2;
  auto kb = [&](int64_t q) {
    return xprev ? c1 * ldg_t(g + q) + c2 * ldg_t(xprev + q) : c1 * ldg_t(g + q);
  };
  for (int p = blockIdx.y * blockDim.x + threadIdx.x; p < total; p += gridDim.y * blockDim.x) {
    const int k = p / (S1 * S2), r = p - k * S1 * S2, j = r / S1, i = r - j * S1;
    auto owned = [&](int x, int y, int z) {
      return x >= G && x < G + N && y >= G && y < G + N && z >= G && z < G + N;
    };
    const int64_t c = B.off + p;
    T acc = T(0);
    if (owned(i - 1, j, k)) acc += kb(vs + c - 1);
    if (owned(i + 1, j, k)) acc += kb(vs + c + 1);
    if (owned(i, j - 1, k)) acc += kb(vs + c - s2);
    if (owned(i, j + 1, k)) acc += kb(vs + c + s2);
    if (owned(i, j, k - 1)) acc += kb(vs + c - s3);
    if (owned(i, j, k + 1)) acc += kb(vs + c + s3);
    const bool me = owned(i, j, k);
    out[c] = acc * ih2 - (me ? T(6) * ih2 * kb(vs + c) : T(0));
    out[c + vs] = me ? kb(c) : T(0);
    if (ybar && xprev) {
      ybar[c] += ldg_t(xprev + c);
      ybar[c + vs] += ldg_t(xprev + c + vs);
    }
  }
}

}  // namespace

extern "C" int tam_wave_rk4_adjoint_stage(int32_t dtype, const tam_wave_block *blocks,
                                          int32_t nblocks, int32_t max_points_per_block,
                                          const void *g, double c1, const void *xprev,
                                          double c2, void *out, void *ybar, void *stream) {
  if (!blocks || !g || !out || nblocks < 0 || max_points_per_block < 0) return TAM_EINVAL;
  if (out == g || out == xprev || (ybar && (ybar == out || ybar == xprev))) return TAM_EINVAL;
  if (nblocks == 0) return TAM_OK;
  const int threads = 256;
  const int chunks = std::max(1, std::min(64, (max_points_per_block + threads - 1) / threads));
  const dim3 grid(nblocks, chunks);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == TAM_F64)
    wave_rk4_adjoint_stage_kernel<double><<<grid, threads, 0, s>>>(
        blocks, nblocks, (const double *)g, c1, (const double *)xprev, c2, (double *)out,
        (double *)ybar);
  else if (dtype == TAM_F32)
    wave_rk4_adjoint_stage_kernel<float><<<grid, threads, 0, s>>>(
        blocks, nblocks, (const float *)g, (float)c1, (const float *)xprev, (float)c2,
        (float *)out, (float *)ybar);
  else
    return TAM_EINVAL;
  return cudaGetLastError() == cudaSuccess ? TAM_OK : TAM_ECUDA;
}

extern "C" int tam_wave_rk4_stage(int32_t dtype, const tam_wave_block *blocks, int32_t nblocks,
                                  int32_t max_points_per_block, const void *x, const void *y,
                                  void *t_out, const void *acc_in, void *acc_out, double ct,
                                  double ca, void *stream) {
  if (!blocks || !x || !y || !acc_out || nblocks < 0 || max_points_per_block < 0)
    return TAM_EINVAL;
  if (x == acc_out || x == t_out) return TAM_EINVAL;
  if (nblocks == 0) return TAM_OK;
  const int threads = 256;
  const int chunks = std::max(1, std::min(64, (max_points_per_block + threads - 1) / threads));
  const dim3 grid(nblocks, chunks);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == TAM_F64)
    wave_rk4_stage_kernel<double><<<grid, threads, 0, s>>>(
        blocks, nblocks, (const double *)x, (const double *)y, (double *)t_out,
        (const double *)acc_in, (double *)acc_out, ct, ca);
  else if (dtype == TAM_F32)
    wave_rk4_stage_kernel<float><<<grid, threads, 0, s>>>(
        blocks, nblocks, (const float *)x, (const float *)y, (float *)t_out,
        (const float *)acc_in, (float *)acc_out, (float)ct, (float)ca);
  else
    return TAM_EINVAL;
  return cudaGetLastError() == cudaSuccess ? TAM_OK : TAM_ECUDA;
}

extern "C" int tam_wave_rhs(int32_t dtype, const tam_wave_block *blocks, int32_t nblocks,
                            int32_t max_points_per_block, const void *in, void *out,
                            int32_t adjoint, void *stream) {
  if (!blocks || !in || !out || nblocks < 0 || max_points_per_block < 0) return TAM_EINVAL;
  if (nblocks == 0) return TAM_OK;
  const int threads = 256;
  const int chunks = std::max(1, std::min(64, (max_points_per_block + threads - 1) / threads));
  const dim3 grid(nblocks, chunks);
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == TAM_F64) {
    if (adjoint)
      wave_rhs_adjoint_kernel<double><<<grid, threads, 0, s>>>(blocks, nblocks, (const double *)in,
                                                                (double *)out);
    else
      wave_rhs_kernel<double><<<grid, threads, 0, s>>>(blocks, nblocks, (const double *)in,
                                                       (double *)out);
  } else if (dtype == TAM_F32) {
    if (adjoint)
      wave_rhs_adjoint_kernel<float><<<grid, threads, 0, s>>>(blocks, nblocks, (const float *)in,
                                                               (float *)out);
    else
      wave_rhs_kernel<float><<<grid, threads, 0, s>>>(blocks, nblocks, (const float *)in,
                                                      (float *)out);
  } else {
    return TAM_EINVAL;
  }
  return cudaGetLastError() == cudaSuccess ? TAM_OK : TAM_ECUDA;
}
