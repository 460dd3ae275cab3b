// hfx_engine.hpp -- the device-resident job: pair data, Schwarz tables,
// screened shell-quartet work lists, and the Fock-build entry points.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "hfx_device.cuh"
#include "hfx_internal.hpp"

namespace hfx {

// device launch helpers (hfx_kernels.cu)
size_t generic_smem_bytes(int maxacc, int maxw, int maxr);
cudaError_t launch_generic(int mode, int nk, const LaunchArgs& a, int maxacc, int maxw, int maxr, int grid,
                           cudaStream_t st);
cudaError_t launch_finish_rhf(const double* Jacc, const double* Kacc, double* G, int K, cudaStream_t st);
cudaError_t launch_finish_uhf(const double* Jacc, const double* Ka, const double* Kb, double* J, double* Kao,
                              double* Kbo, int K, cudaStream_t st);
cudaError_t launch_add(const double* A, const double* B, double* C, int n, cudaStream_t st);

void cuda_check(cudaError_t e, const char* what);

// Owning device buffer.
template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { reset(); }
    void reset()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count)
    {
        if (count == n && p) return;
        reset();
        if (count == 0) return;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            cudaGetLastError();
            throw Error(HFX_ERR_OOM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
        }
        n = count;
    }
    void upload(const std::vector<T>& v, cudaStream_t st)
    {
        alloc(v.size());
        if (!v.empty()) cuda_check(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st), "upload");
    }
};

struct HostPair {
    int s0, s1;       // shells (s0 has the higher L)
    int l0, l1;
    int npp;
    long long e_off;
    int pp0;
    bool same;
};

// Host image of the per-job pair data (built on the CPU, then uploaded).
struct PairData {
    std::vector<HostPair> hpairs;
    std::vector<DPair> dpairs;
    std::vector<PairGeo> geo;
    std::vector<double> epool;
};
PairData build_pair_data(const Basis& b);

class Job {
public:
    Job(Basis b, const hfx_options& opt);
    ~Job();

    int K() const { return basis_.K; }
    const Basis& basis() const { return basis_; }

    void schwarz_host(std::vector<double>& Qbf) const;
    // device-pointer Fock builds (synchronous)
    void fock_rhf_device(const double* dP, double* dG);
    void fock_uhf_device(const double* dPa, const double* dPb, double* dJ, double* dKa, double* dKb);
    void fock_rhf(const double* P, double* G);
    void fock_uhf(const double* Pa, const double* Pb, double* J, double* Ka, double* Kb);
    void eri_unique(double thr, double* out);

    hfx_build_stats stats{};
    cudaStream_t stream() const { return stream_; }

private:
    void build_pairs();
    void compute_schwarz();
    void build_tasks(double thr, std::vector<Task>& tasks, int& maxacc, int& maxw, int& maxr, double* flops = nullptr,
                     double* prims = nullptr) const;
    void run_tasks(int mode, int nk, const std::vector<Task>* host_tasks, const DevBuf<Task>& tasks, int ntasks,
                   int maxacc, int maxw, int maxr, LaunchArgs a);
    LaunchArgs base_args() const;
    void record_stats(int launches);

    Basis basis_;
    hfx_options opt_;
    int device_ = 0;
    int nsm_ = 1;
    cudaStream_t stream_ = nullptr;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr, evk0_ = nullptr, evk1_ = nullptr;

    std::vector<HostPair> hpairs_;
    std::vector<double> qsh_;     // per pair
    std::vector<double> qbf_;     // per BF pair
    DevBuf<DPair> d_pairs_;
    DevBuf<PairGeo> d_ppgeo_;
    DevBuf<double> d_epool_;
    DevBuf<double> d_boys_;
    DevBuf<double> d_qbf_;
    DevBuf<unsigned long long> d_qsh_;
    DevBuf<Task> d_tasks_;
    int ntasks_ = 0;
    int maxacc_ = 0, maxw_ = 0, maxr_ = 0;
    DevBuf<int> d_counter_;
    DevBuf<double> d_D_, d_D2_, d_Dj_, d_J_, d_K_, d_K2_, d_out1_, d_out2_, d_out3_;
    double prim_quartets_ = 0.0, flops_ = 0.0;
};

}  // namespace hfx
