// hfx_small_f32w.cu -- float-only class kernel (dd|ds) (see hfx_small_f32y.cu).
#include "hfx_class.cuh"

namespace hfx {

cudaError_t small_spec_f32w(int pcb, int pck, int nk, int ntasks, KernelSpec* s)
{
    switch (pcb * 16 + pck) {
    case 5 * 16 + 3: return small_spec<float, 2, 2, 2, 0>(nk, ntasks, s);   // (dd|ds)
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace hfx
