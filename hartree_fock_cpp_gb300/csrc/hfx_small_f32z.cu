// hfx_small_f32z.cu -- float-only class kernel (dd|pp) (see hfx_small_f32y.cu).
#include "hfx_class.cuh"

namespace hfx {

cudaError_t small_spec_f32w(int pcb, int pck, int nk, int ntasks, KernelSpec* s);   // hfx_small_f32w.cu

cudaError_t small_spec_f32z(int pcb, int pck, int nk, int ntasks, KernelSpec* s)
{
    switch (pcb * 16 + pck) {
    case 5 * 16 + 2: return small_spec<float, 2, 2, 1, 1>(nk, ntasks, s);   // (dd|pp)
    default: return small_spec_f32w(pcb, pck, nk, ntasks, s);
    }
}

}  // namespace hfx
