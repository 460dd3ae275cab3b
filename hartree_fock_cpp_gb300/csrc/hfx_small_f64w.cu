// hfx_small_f64w.cu -- double class kernels for larger classes, their ket component pairs
// split over several threads per task (small_ncb, at most 36 accumulators
// per thread).  One translation unit per few classes, so that they compile in
// parallel.
#include "hfx_class.cuh"

namespace hfx {

cudaError_t small_spec_f64v(int pcb, int pck, int nk, int ntasks, KernelSpec* s);   // hfx_small_f64v.cu

cudaError_t small_spec_f64w(int pcb, int pck, int nk, int ntasks, KernelSpec* s)
{
    switch (pcb * 16 + pck) {
    case 4 * 16 + 4: return small_spec<double, 2, 1, 2, 1>(nk, ntasks, s);   // (dp|dp), 9 cd blocks
    default: return small_spec_f64v(pcb, pck, nk, ntasks, s);
    }
}

}  // namespace hfx
