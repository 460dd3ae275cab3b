// hfx_small_f64z.cu -- double class kernels for larger classes, their ket component pairs
// split over several threads per task (small_ncb, at most 36 accumulators
// per thread).  One translation unit per few classes, so that they compile in
// parallel.
#include "hfx_class.cuh"

namespace hfx {

cudaError_t small_spec_f64w(int pcb, int pck, int nk, int ntasks, KernelSpec* s);   // hfx_small_f64w.cu

cudaError_t small_spec_f64z(int pcb, int pck, int nk, int ntasks, KernelSpec* s)
{
    switch (pcb * 16 + pck) {
    case 5 * 16 + 0: return small_spec<double, 2, 2, 0, 0>(nk, ntasks, s);   // (dd|ss)
    case 5 * 16 + 1: return small_spec<double, 2, 2, 1, 0>(nk, ntasks, s);   // (dd|ps), 3 cd blocks
    default: return small_spec_f64w(pcb, pck, nk, ntasks, s);
    }
}

}  // namespace hfx
