// hfx_noalloc.cu -- RHF Fock build on an existing job that allocates no
// device memory at call time.
//
// Why: hfx_fock_rhf_device allocates its J/K accumulators with cudaMalloc on
// first use.  Some callers cannot allow that: a host application whose own
// allocator owns the device memory (for example a PyTorch process running
// near its memory cap), or an SCF loop that must not stall other work in
// flight, since cudaMalloc can synchronise the device.  This entry point
// keeps every scratch buffer of the build (the J and K accumulators and the
// work-queue counters) in one file-scope __device__ array, so its only
// device writes besides the caller's output are into that array and, for a
// mixed-precision job, into the float density copies the job allocated when
// it was created.
//
// Limits: K <= kNoAllocMaxK basis functions and at most kNoAllocMaxGroups
// kernel launch groups per build; larger jobs are rejected with
// HFX_ERR_UNSUPPORTED.  The array (2 * 512 * 512 doubles + 64 ints, about
// 4 MB) is reserved on a device when the first job is created there (module
// loading is lazy by default; job creation resolves the array's address) and
// stays reserved until the process exits.  All calls share it: two builds that overlap on the GPU (two
// host threads, or two jobs on different streams) race on it and produce
// garbage, so callers serialise them.  Each call clears the parts that must
// start at zero.
#include <cuda_runtime.h>

#include <mutex>

#include "hfx_engine.hpp"

namespace hfx {

constexpr int kNoAllocMaxK = 512;
constexpr int kNoAllocMaxGroups = 64;

struct NoAllocScratch {
    double jacc[kNoAllocMaxK * kNoAllocMaxK];
    double kacc[kNoAllocMaxK * kNoAllocMaxK];
    int counters[kNoAllocMaxGroups];
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Device address of the scratch array, resolved once per device (the host
// symbol is only a stand-in and must never be handed to a kernel).
static NoAllocScratch* scratch_address(int device)
{
    static std::mutex mu;
    static NoAllocScratch* addr[64] = {};
    if (device < 0 || device >= 64) throw Error(HFX_ERR_INVALID, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[device]) {
        void* p = nullptr;
        cuda_check(cudaSetDevice(device), "cudaSetDevice");
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            throw Error(HFX_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch) failed: ") + cudaGetErrorString(e));
        }
        addr[device] = static_cast<NoAllocScratch*>(p);
    }
    return addr[device];
}

// Job creation resolves the address on the job's device, so that the first
// allocation-free build makes no CUDA call that could allocate: with lazy
// module loading (the CUDA default), resolving the symbol loads the module
// that holds the array, which reserves its memory.
void noalloc_prepare(int device) { scratch_address(device); }

void fock_rhf_noalloc(Job& job, int device, const double* dP, double* dG)
{
    if (job.K() > kNoAllocMaxK)
        throw Error(HFX_ERR_UNSUPPORTED, "hfx_fock_rhf_device_noalloc: K = " + std::to_string(job.K()) +
                                             " exceeds the static scratch limit of " + std::to_string(kNoAllocMaxK) +
                                             " basis functions; use hfx_fock_rhf_device");
    if (job.num_launch_groups() > kNoAllocMaxGroups)
        throw Error(HFX_ERR_UNSUPPORTED, "hfx_fock_rhf_device_noalloc: too many launch groups for the static scratch");
    NoAllocScratch* s = scratch_address(device);
    job.fock_rhf_device_scratch(dP, dG, s->jacc, s->kacc, s->counters);
}

}  // namespace hfx
