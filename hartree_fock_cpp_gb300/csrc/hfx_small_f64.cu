// hfx_small_f64.cu -- double instantiations of the small-class kernels (hfx_class.cuh).
#include "hfx_class.cuh"

namespace hfx {

// Pair class index pc = l0*(l0+1)/2 + l1; bra pc >= ket pc.  Returns
// cudaErrorInvalidValue for a class that has no small-class kernel.
cudaError_t launch_small_f64(int pcb, int pck, const void* args, int nk, cudaStream_t st)
{
    const SmallArgs<double>& a = *(const SmallArgs<double>*)args;
    switch (pcb * 16 + pck) {
    case 0 * 16 + 0: return launch_small<double, 0, 0, 0, 0>(a, nk, st);   // (ss|ss)
    case 1 * 16 + 0: return launch_small<double, 1, 0, 0, 0>(a, nk, st);   // (ps|ss)
    case 1 * 16 + 1: return launch_small<double, 1, 0, 1, 0>(a, nk, st);   // (ps|ps)
    case 2 * 16 + 0: return launch_small<double, 1, 1, 0, 0>(a, nk, st);   // (pp|ss)
    case 2 * 16 + 1: return launch_small<double, 1, 1, 1, 0>(a, nk, st);   // (pp|ps)
    case 3 * 16 + 0: return launch_small<double, 2, 0, 0, 0>(a, nk, st);   // (ds|ss)
    case 3 * 16 + 1: return launch_small<double, 2, 0, 1, 0>(a, nk, st);   // (ds|ps)
    case 3 * 16 + 3: return launch_small<double, 2, 0, 2, 0>(a, nk, st);   // (ds|ds)
    case 4 * 16 + 0: return launch_small<double, 2, 1, 0, 0>(a, nk, st);   // (dp|ss)
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace hfx
