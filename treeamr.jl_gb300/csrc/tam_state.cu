// The copies between a state vector and the working array: scatter! and
// gather! (src/state.jl:101-160).
//
// The state vector holds every block's own points only, in the working
// array's index order minus the ghosts: shape (O_1, O_2, O_3, nvars, nblocks)
// with O_d = N + c_d, against (S_1, S_2, S_3, nvars, nblocks) for the
// working array, own point i_d at stored index G_d + i_d (0-based).  Both
// are column-major, so a row of O_1 state entries is a contiguous run of the
// working array too.  A CTA takes whole rows (blockDim / O_1 of them at a
// time, a thread per entry), so the state side is read or written in one
// linear sweep and the working side in runs of O_1; a row's position is two
// divisions per thread, none per entry.  Bits are moved, not arithmetic:
// NaN payloads and -0 survive.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "tam_internal.h"
#include "treeamr_cuda.h"

namespace {

// single roundings, so that no multiply-add is fused
__device__ __forceinline__ double __fmul_rn_t(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float __fmul_rn_t(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add_t(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_t(float a, float b) { return __fadd_rn(a, b); }

template <typename T, bool TO_WORK>
__global__ void __launch_bounds__(256) state_copy_kernel(T *__restrict__ work,
                                                         T *__restrict__ state, int64_t nrows,
                                                         int O1, int O2, int O3, int S1, int S2,
                                                         int S3, int G1, int G2, int G3) {
  const int rpi = blockDim.x / O1;  // rows a CTA takes at a time
  const int lr = threadIdx.x / O1, e = threadIdx.x - lr * O1;
  if (lr >= rpi) return;
  for (int64_t r0 = (int64_t)blockIdx.x * rpi; r0 < nrows; r0 += (int64_t)gridDim.x * rpi) {
    const int64_t r = r0 + lr;
    if (r >= nrows) continue;
    const int64_t q = r / O2;
    const int i2 = (int)(r - q * O2);
    const int64_t vb = q / O3;
    const int i3 = (int)(q - vb * O3);
    const int64_t w = ((vb * S3 + i3 + G3) * S2 + i2 + G2) * (int64_t)S1 + G1 + e;
    const int64_t s = r * O1 + e;
    if (TO_WORK)
      work[w] = state[s];
    else
      state[s] = work[w];
  }
}

// The own boxes of one working array into another's (both in the working
// layout): the rows of state_copy_kernel, read and written at the same
// working-array offsets.  The upload of tam_fill_host_own, which reads a
// page-locked host array through its device mapping: a small grid (it
// shares the GPU with the fills of the states in flight beside it) with
// kUnroll independent reads in flight per thread to cover the host link's
// latency.
constexpr int kUnroll = 8;

template <typename T>
__global__ void __launch_bounds__(256) own_box_kernel(T *__restrict__ dst,
                                                      const T *__restrict__ src, int64_t nrows,
                                                      int O1, int O2, int O3, int S1, int S2,
                                                      int S3, int G1, int G2, int G3) {
  const int rpi = blockDim.x / O1;
  const int lr = threadIdx.x / O1, e = threadIdx.x - lr * O1;
  if (lr >= rpi) return;
  const int64_t step = (int64_t)gridDim.x * rpi;
  for (int64_t r0 = (int64_t)blockIdx.x * rpi + lr; r0 < nrows; r0 += step * kUnroll) {
    int64_t w[kUnroll];
    T x[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      const int64_t r = r0 + u * step;
      w[u] = -1;
      if (r < nrows) {
        const int64_t q = r / O2;
        const int i2 = (int)(r - q * O2);
        const int64_t vb = q / O3;
        const int i3 = (int)(q - vb * O3);
        w[u] = ((vb * S3 + i3 + G3) * S2 + i2 + G2) * (int64_t)S1 + G1 + e;
        x[u] = src[w[u]];
      }
    }
#pragma unroll
    for (int u = 0; u < kUnroll; ++u)
      if (w[u] >= 0) dst[w[u]] = x[u];
  }
}

template <typename T>
cudaError_t launch(bool to_work, T *work, T *state, int64_t nrows, const int O[3],
                   const int S[3], const int G[3], cudaStream_t stream) {
  const int threads = O[0] <= 256 ? 256 : 1024;
  const int rpi = threads / O[0];
  int dev = 0, nsm = 152;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int64_t want = (nrows + rpi - 1) / rpi;
  const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)nsm * 32));
  if (to_work)
    state_copy_kernel<T, true><<<(unsigned)blocks, threads, 0, stream>>>(
        work, state, nrows, O[0], O[1], O[2], S[0], S[1], S[2], G[0], G[1], G[2]);
  else
    state_copy_kernel<T, false><<<(unsigned)blocks, threads, 0, stream>>>(
        work, state, nrows, O[0], O[1], O[2], S[0], S[1], S[2], G[0], G[1], G[2]);
  return cudaGetLastError();
}

}  // namespace

namespace tam {

int own_box_copy(const tam_state_layout *L, void *dst, const void *src, void *stream) {
  if (!L || !dst || !src) return TAM_EINVAL;
  if (L->ndim < 1 || L->ndim > 3 || L->nvars < 1 || L->nblocks < 0) return TAM_EINVAL;
  int O[3] = {1, 1, 1}, S[3] = {1, 1, 1}, G[3] = {0, 0, 0};
  for (int d = 0; d < L->ndim; ++d) {
    O[d] = L->own[d];
    S[d] = L->stored[d];
    G[d] = L->ghosts[d];
    if (O[d] < 1 || G[d] < 0 || G[d] + O[d] > S[d]) return TAM_ELAYOUT;
  }
  if (O[0] > 1024) return TAM_EUNSUPPORTED;
  const int64_t nrows = (int64_t)O[1] * O[2] * L->nvars * L->nblocks;
  if (nrows == 0) return TAM_OK;
  const int threads = O[0] <= 256 ? 256 : 1024;
  const int rpi = threads / O[0];
  int dev = 0, nsm = 152;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  // half the SMs, one CTA each: the rest stay with the fills in flight
  const int64_t blocks =
      std::max<int64_t>(1, std::min<int64_t>((nrows + rpi - 1) / rpi, std::max(1, nsm / 2)));
  cudaStream_t st = (cudaStream_t)stream;
  if (L->dtype == TAM_F64)
    own_box_kernel<double><<<(unsigned)blocks, threads, 0, st>>>(
        (double *)dst, (const double *)src, nrows, O[0], O[1], O[2], S[0], S[1], S[2], G[0],
        G[1], G[2]);
  else if (L->dtype == TAM_F32)
    own_box_kernel<float><<<(unsigned)blocks, threads, 0, st>>>(
        (float *)dst, (const float *)src, nrows, O[0], O[1], O[2], S[0], S[1], S[2], G[0],
        G[1], G[2]);
  else
    return TAM_EINVAL;
  return cudaGetLastError() == cudaSuccess ? TAM_OK : TAM_ECUDA;
}

}  // namespace tam

namespace {

int state_copy(bool to_work, const tam_state_layout *L, void *work, void *state,
               void *stream) {
  if (!L || !work || !state) return TAM_EINVAL;
  if (L->ndim < 1 || L->ndim > 3 || L->nvars < 1 || L->nblocks < 0) return TAM_EINVAL;
  int O[3] = {1, 1, 1}, S[3] = {1, 1, 1}, G[3] = {0, 0, 0};
  for (int d = 0; d < L->ndim; ++d) {
    O[d] = L->own[d];
    S[d] = L->stored[d];
    G[d] = L->ghosts[d];
    if (O[d] < 1 || G[d] < 0 || G[d] + O[d] > S[d]) return TAM_ELAYOUT;
  }
  if (O[0] > 1024) return TAM_EUNSUPPORTED;
  const int64_t nrows = (int64_t)O[1] * O[2] * L->nvars * L->nblocks;
  if (nrows == 0) return TAM_OK;
  cudaError_t e;
  if (L->dtype == TAM_F64)
    e = launch<double>(to_work, (double *)work, (double *)state, nrows, O, S, G,
                       (cudaStream_t)stream);
  else if (L->dtype == TAM_F32)
    e = launch<float>(to_work, (float *)work, (float *)state, nrows, O, S, G,
                      (cudaStream_t)stream);
  else
    return TAM_EINVAL;
  return e == cudaSuccess ? TAM_OK : TAM_ECUDA;
}

}  // namespace

extern "C" int tam_scatter(const tam_state_layout *layout, const void *state, void *work,
                           void *stream) {
  return state_copy(true, layout, work, const_cast<void *>(state), stream);
}

extern "C" int tam_gather(const tam_state_layout *layout, const void *work, void *state,
                          void *stream) {
  return state_copy(false, layout, const_cast<void *>(work), state, stream);
}

// ---- a seam's axis (stage P's axis part) ----------------------------------------
//
// Each axis point is its own image under the turn, so its variables become
// the mean of their images under the orbit's powers of the set's map
// (axis_project!, mean_gather_kernel! in its paired form, src/ghosts.jl:
// 599-660, 736-770): t_r = f(v, r) * u[rotvars(v, r)] (t_0 = u[v]), summed in
// pairs a half turn apart, ((t_0 + t_2) + (t_1 + t_3)) / 4, or (t_0 + t_2) / 2
// under a half turn.  Every mean is gathered into `buf` before any is
// written, since a point's variables read one another.
namespace {

template <typename T>
__global__ void __launch_bounds__(256)
    axis_gather_kernel(const int64_t *__restrict__ points, int64_t n, int members,
                       const T *__restrict__ work, int nvars, int64_t vol,
                       const T *__restrict__ factors, int ncol, const int32_t *__restrict__ rotvars,
                       T *__restrict__ buf) {
  for (int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; it < n * nvars;
       it += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = it / nvars;
    const int v = (int)(it - i * nvars);
    const int64_t off = points[i];
    bool bad = false;
    auto term = [&](int r) -> T {
      if (r == 0) return work[off + v * vol];
      const int sv = rotvars[v + (int64_t)nvars * r] - 1;
      if (sv < 0 || sv >= nvars) {
        bad = true;
        return T(0);
      }
      return __fmul_rn_t(factors[v + (int64_t)nvars * ((int64_t)ncol * r)], work[off + sv * vol]);
    };
    T acc = add_t(term(0), term(2));
    if (members == 4) acc = add_t(acc, add_t(term(1), term(3)));
    buf[it] = bad ? T(NAN) : acc / T(members);
  }
}

template <typename T>
__global__ void __launch_bounds__(256) axis_write_kernel(const int64_t *__restrict__ points,
                                                         int64_t n, T *__restrict__ work,
                                                         int nvars, int64_t vol,
                                                         const T *__restrict__ buf) {
  for (int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; it < n * nvars;
       it += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = it / nvars;
    const int v = (int)(it - i * nvars);
    work[points[i] + v * vol] = buf[it];
  }
}

}  // namespace

extern "C" int tam_axis_project(int32_t dtype, const int64_t *points, int64_t npoints,
                                int32_t members, void *work, int32_t nvars,
                                int64_t block_points, const void *factors, int32_t ncol,
                                const int32_t *rotvars, void *buffer, void *stream) {
  if (npoints == 0) return TAM_OK;
  if (!points || !work || !factors || !rotvars || !buffer || nvars < 1 || npoints < 0 ||
      (members != 2 && members != 4) || block_points < 1 || ncol < 1)
    return TAM_EINVAL;
  const int64_t n = npoints * nvars;
  const int threads = 256;
  const int64_t blocks = std::min<int64_t>((n + threads - 1) / threads, 4096);
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == TAM_F64) {
    axis_gather_kernel<double><<<(unsigned)blocks, threads, 0, st>>>(
        points, npoints, members, (const double *)work, nvars, block_points,
        (const double *)factors, ncol, rotvars, (double *)buffer);
    axis_write_kernel<double><<<(unsigned)blocks, threads, 0, st>>>(
        points, npoints, (double *)work, nvars, block_points, (const double *)buffer);
  } else if (dtype == TAM_F32) {
    axis_gather_kernel<float><<<(unsigned)blocks, threads, 0, st>>>(
        points, npoints, members, (const float *)work, nvars, block_points,
        (const float *)factors, ncol, rotvars, (float *)buffer);
    axis_write_kernel<float><<<(unsigned)blocks, threads, 0, st>>>(
        points, npoints, (float *)work, nvars, block_points, (const float *)buffer);
  } else {
    return TAM_EINVAL;
  }
  return cudaGetLastError() == cudaSuccess ? TAM_OK : TAM_ECUDA;
}
