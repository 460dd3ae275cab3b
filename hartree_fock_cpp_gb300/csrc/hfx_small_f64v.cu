// hfx_small_f64v.cu -- double class kernels for larger classes, their ket component pairs
// split over several threads per task (small_ncb, at most 36 accumulators
// per thread).  One translation unit per few classes, so that they compile in
// parallel.
#include "hfx_class.cuh"

namespace hfx {


cudaError_t small_spec_f64v(int pcb, int pck, int nk, int ntasks, KernelSpec* s)
{
    switch (pcb * 16 + pck) {
    case 5 * 16 + 2: return small_spec<double, 2, 2, 1, 1>(nk, ntasks, s);   // (dd|pp), 9 cd blocks
    case 5 * 16 + 3: return small_spec<double, 2, 2, 2, 0>(nk, ntasks, s);   // (dd|ds), 6 cd blocks
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace hfx
