// The fused launches of a Float32 stage: the copy, stencil and staged kernels'
// float instantiations, in a unit of their own so that the build compiles the
// element types in parallel.
#include "tam_kernels.cuh"

namespace tam {

cudaError_t fused_stage_f32(int D, const Tile *tiles, const PTile *ptiles, const Stage &st,
                            const SchedArgs &a, void *work, const void *factors, int nvars,
                            const int S[3], int threads, cudaStream_t stream, SideStream *side,
                            const void *src, const Tile *staged) {
  return fused_dispatch<float>(D, tiles, ptiles, st, typed<float>(a), (const float *)src,
                               (float *)work, (const float *)factors, nvars, S, threads, stream,
                               side, staged);
}

}  // namespace tam
