// hfx_small_f32y.cu -- float-only class kernels (dp|dp), (dd|ss) and (dd|ps),
// their ket component pairs split over several threads per task; the d-d
// classes are spread over hfx_small_f32y/z/w.cu so that the class kernels
// compile in parallel.
#include "hfx_class.cuh"

namespace hfx {

cudaError_t small_spec_f32z(int pcb, int pck, int nk, int ntasks, KernelSpec* s);   // hfx_small_f32z.cu

cudaError_t small_spec_f32y(int pcb, int pck, int nk, int ntasks, KernelSpec* s)
{
    switch (pcb * 16 + pck) {
    case 4 * 16 + 4: return small_spec<float, 2, 1, 2, 1>(nk, ntasks, s);   // (dp|dp)
    case 5 * 16 + 0: return small_spec<float, 2, 2, 0, 0>(nk, ntasks, s);   // (dd|ss)
    case 5 * 16 + 1: return small_spec<float, 2, 2, 1, 0>(nk, ntasks, s);   // (dd|ps)
    default: return small_spec_f32z(pcb, pck, nk, ntasks, s);
    }
}

}  // namespace hfx
