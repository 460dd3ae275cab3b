// hfx_small_f64y.cu -- double class kernels for larger classes, their ket component pairs
// split over several threads per task (small_ncb, at most 36 accumulators
// per thread).  One translation unit per few classes, so that they compile in
// parallel.
#include "hfx_class.cuh"

namespace hfx {

cudaError_t small_spec_f64z(int pcb, int pck, int nk, int ntasks, KernelSpec* s);   // hfx_small_f64z.cu

cudaError_t small_spec_f64y(int pcb, int pck, int nk, int ntasks, KernelSpec* s)
{
    switch (pcb * 16 + pck) {
    case 4 * 16 + 2: return small_spec<double, 2, 1, 1, 1>(nk, ntasks, s);   // (dp|pp), 5 cd blocks
    case 4 * 16 + 3: return small_spec<double, 2, 1, 2, 0>(nk, ntasks, s);   // (dp|ds), 3 cd blocks
    default: return small_spec_f64z(pcb, pck, nk, ntasks, s);
    }
}

}  // namespace hfx
