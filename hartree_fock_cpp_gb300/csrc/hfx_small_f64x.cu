// hfx_small_f64x.cu -- double class kernels for the classes whose
// thread-per-quartet form needs its ket component pairs split over two or
// three threads per task to fit the register file (small_ncb, at most 36
// accumulators per thread).  Split from hfx_small_f64.cu so the translation
// units compile in parallel.
#include "hfx_class.cuh"

namespace hfx {

cudaError_t small_spec_f64y(int pcb, int pck, int nk, int ntasks, KernelSpec* s);   // hfx_small_f64y.cu

cudaError_t small_spec_f64x(int pcb, int pck, int nk, int ntasks, KernelSpec* s)
{
    switch (pcb * 16 + pck) {
    case 2 * 16 + 2: return small_spec<double, 1, 1, 1, 1>(nk, ntasks, s);   // (pp|pp), 3 cd blocks
    case 3 * 16 + 2: return small_spec<double, 2, 0, 1, 1>(nk, ntasks, s);   // (ds|pp), 2 cd blocks
    case 4 * 16 + 1: return small_spec<double, 2, 1, 1, 0>(nk, ntasks, s);   // (dp|ps), 2 cd blocks
    default: return small_spec_f64y(pcb, pck, nk, ntasks, s);
    }
}

}  // namespace hfx
