// hfx_dscf.hpp -- SCF iterations with the O(K^3) algebra on the device.
#pragma once

#include <cublas_v2.h>
#include <cusolverDn.h>

#include <atomic>
#include <memory>

#include "hfx_engine.hpp"
#include "hfx_scf.hpp"
#include "hfx_sp2.hpp"

namespace hfx {

// Host-side control of a running SCF, checked between iterations (never
// inside a kernel): cancellation flag, absolute deadline (steady clock,
// seconds; 0 = none), and a test hook that fails the SCF at a given iteration.
struct ScfControl {
    std::atomic<bool>* cancel = nullptr;
    double deadline = 0.0;
    int fault_at_iteration = 0;
};

class DeviceScf {
public:
    // nspin = 1 (RHF) or 2 (UHF)
    DeviceScf(FockSource& job, const ScfSetup& setup, int nspin);
    ~DeviceScf();
    DeviceScf(const DeviceScf&) = delete;
    DeviceScf& operator=(const DeviceScf&) = delete;

    // Runs the SCF (semantics of hfx_scf.cpp) from the given initial
    // densities (null = zero); na/nb used for UHF.  delta_thr: density-weighted
    // screening of the FP64 builds of density changes (mixed precision).
    ScfOutput run(const Basis& b, const ScfSetup& setup, const hfx_scf_options& opt, int na, int nb, const double* P0a,
                  const double* P0b, double delta_thr, const ScfControl* ctl = nullptr);

private:
    void gemm(bool ta, const double* A, bool tb, const double* B, double* C, double alpha = 1.0, int kdim = 0);
    void dot(const double* a, const double* b, int n, int slot);
    void fetch(double* host, int count);
    void axpby(double a, const double* A, double b, const double* B, double* C);
    void build(int mode, double dthr);
    void error_and_energy();
    // new densities Pn_ of the (DIIS) Fock matrices; proj_[s] says which
    // spins took the SP2 projector (status in scalar slot 2 + s)
    void diagonalise(const double* const* Fs, const int* nocc, double occ_factor, bool use_proj);
    // syevd of the orthogonalised Fock matrix Fq_[s]: MO energies e_, coefficients C_, and
    // (density) the density Pn_
    void eigensolve(int s, int nocc, double occ_factor, bool density);
    // Pn_[s] from the SP2 projector of Fq_[s] within max_steps (status in slot 2 + s)
    void project(int s, int nocc, double occ_factor, int max_steps);

    FockSource& job_;
    int K_, nspin_;
    cudaStream_t st_ = nullptr;
    cublasHandle_t blas_ = nullptr;
    cusolverDnHandle_t solver_ = nullptr;
    DevBuf<double> H_, S_, X_, T1_, T2_, Fp_, W_, work_, scal_, G_, dG_, Kr_;
    DevBuf<double> P_[2], Pn_[2], F_[2], E_[2], C_[2], Gr_[2], Pr_[2], dP_[2], e_[2], Kx_[2], dK_[2], Fq_[2], D_;
    std::unique_ptr<Sp2Projector> sp2_;
    bool proj_[2] = {false, false};
    int proj_steps_[2] = {0, 0};  // steps the last projection took (0: unknown)
    int proj_cap_[2] = {0, 0};    // step cap of the projection in flight
    DevBuf<int> info_;
    int lwork_ = 0;
    double fock_ms_ = 0.0;
};

}  // namespace hfx
