// hfx_small_f32x.cu -- float class kernels for the larger classes whose
// thread-per-quartet form fits the register file once their ket component
// pairs are split over a few threads per task (the double forms are in
// hfx_small_f64x..v.cu).  Split from hfx_small_f32.cu (and the d-d classes
// into hfx_small_f32y/z/w.cu) so the translation units compile in parallel.
#include "hfx_class.cuh"

namespace hfx {

cudaError_t small_spec_f32y(int pcb, int pck, int nk, int ntasks, KernelSpec* s);   // hfx_small_f32y.cu

cudaError_t small_spec_f32x(int pcb, int pck, int nk, int ntasks, KernelSpec* s)
{
    switch (pcb * 16 + pck) {
    case 2 * 16 + 2: return small_spec<float, 1, 1, 1, 1>(nk, ntasks, s);   // (pp|pp)
    case 3 * 16 + 2: return small_spec<float, 2, 0, 1, 1>(nk, ntasks, s);   // (ds|pp)
    case 4 * 16 + 1: return small_spec<float, 2, 1, 1, 0>(nk, ntasks, s);   // (dp|ps)
    case 4 * 16 + 2: return small_spec<float, 2, 1, 1, 1>(nk, ntasks, s);   // (dp|pp)
    case 4 * 16 + 3: return small_spec<float, 2, 1, 2, 0>(nk, ntasks, s);   // (dp|ds)
    default: return small_spec_f32y(pcb, pck, nk, ntasks, s);
    }
}

}  // namespace hfx
