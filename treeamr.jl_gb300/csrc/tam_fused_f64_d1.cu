// The fused launches of a 1-D Float64 stage: the copy, stencil and staged
// kernels' double instantiations for D = 1, in a unit of their own so that the
// build compiles them in parallel.
#include "tam_kernels.cuh"

namespace tam {

cudaError_t fused_stage_f64_d1(const Tile *tiles, const PTile *ptiles, const Stage &st,
                               const SchedArgs &a, void *work, const void *factors, int nvars,
                               const int S[3], int threads, cudaStream_t stream,
                               SideStream *side, const void *src, const Tile *staged) {
  if (st.nptiles == 0 && st.nstaged == 0) return cudaSuccess;
  return launch_both<double, 1>(tiles, ptiles, st, typed<double>(a), (const double *)src,
                                 (double *)work, (const double *)factors, nvars, S, threads,
                                 stream, side, staged);
}

}  // namespace tam
