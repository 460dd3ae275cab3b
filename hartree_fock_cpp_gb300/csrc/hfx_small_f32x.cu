// hfx_small_f32x.cu -- float-only small-class kernels for the larger classes
// whose thread-per-quartet form fits the register file in FP32 (in FP64
// these classes run on the warp kernel).  Split from hfx_small_f32.cu so the
// two translation units compile in parallel.
#include "hfx_class.cuh"

namespace hfx {

cudaError_t small_spec_f32x(int pcb, int pck, int nk, int ntasks, KernelSpec* s)
{
    switch (pcb * 16 + pck) {
    case 2 * 16 + 2: return small_spec<float, 1, 1, 1, 1>(nk, ntasks, s);   // (pp|pp)
    case 3 * 16 + 2: return small_spec<float, 2, 0, 1, 1>(nk, ntasks, s);   // (ds|pp)
    case 4 * 16 + 1: return small_spec<float, 2, 1, 1, 0>(nk, ntasks, s);   // (dp|ps)
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace hfx
