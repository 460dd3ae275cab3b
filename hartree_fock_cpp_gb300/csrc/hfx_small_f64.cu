// hfx_small_f64.cu -- double instantiations of the small-class kernels (hfx_class.cuh).
#include "hfx_class.cuh"

namespace hfx {

cudaError_t small_spec_f64x(int pcb, int pck, int nk, int ntasks, KernelSpec* s);   // hfx_small_f64x.cu

// Pair class index pc = l0*(l0+1)/2 + l1; bra pc >= ket pc.  Returns
// cudaErrorInvalidValue for a class that has no small-class kernel.
cudaError_t small_spec_f64(int pcb, int pck, int nk, int ntasks, KernelSpec* s)
{
    switch (pcb * 16 + pck) {
    case 0 * 16 + 0: return small_spec<double, 0, 0, 0, 0>(nk, ntasks, s);   // (ss|ss)
    case 1 * 16 + 0: return small_spec<double, 1, 0, 0, 0>(nk, ntasks, s);   // (ps|ss)
    case 1 * 16 + 1: return small_spec<double, 1, 0, 1, 0>(nk, ntasks, s);   // (ps|ps)
    case 2 * 16 + 0: return small_spec<double, 1, 1, 0, 0>(nk, ntasks, s);   // (pp|ss)
    case 2 * 16 + 1: return small_spec<double, 1, 1, 1, 0>(nk, ntasks, s);   // (pp|ps)
    case 3 * 16 + 0: return small_spec<double, 2, 0, 0, 0>(nk, ntasks, s);   // (ds|ss)
    case 3 * 16 + 1: return small_spec<double, 2, 0, 1, 0>(nk, ntasks, s);   // (ds|ps)
    case 3 * 16 + 3: return small_spec<double, 2, 0, 2, 0>(nk, ntasks, s);   // (ds|ds)
    case 4 * 16 + 0: return small_spec<double, 2, 1, 0, 0>(nk, ntasks, s);   // (dp|ss)
    default: return small_spec_f64x(pcb, pck, nk, ntasks, s);
    }
}

}  // namespace hfx
