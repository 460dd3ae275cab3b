// hfx_dscf.cu -- the SCF iteration on the device.
//
// Same control flow as the host drivers (hfx_scf.cpp, i.e. the reference's
// rhf_diis scf.hpp:205-419 and uhf_diis scf.hpp:423-682): damping for the
// first start_diis-1 iterations, Pulay DIIS over the last max_history
// (F, FPS-SPF) pairs with the augmented B matrix solved by complete-pivoting
// LU, symmetric orthogonalisation, convergence on RMSD(P) and ||FPS-SPF||
// followed by the final check.  The O(K^3) algebra runs on the job's stream:
// FP64 GEMMs (cuBLAS), the density step (the SP2 projector of hfx_sp2.cu, or
// the symmetric eigensolver cuSOLVER syevd), and small element-wise kernels;
// only the DIIS system ((n+1) x (n+1), n <= 8) and a handful of scalars per
// iteration travel to the host.  The reference diagonalises the Fock matrix
// every iteration; only the density enters the next iteration, and the
// projector gives the same density to rounding.  The MO energies and
// coefficients of the last iteration come from one syevd after the loop.
//
// Layout: every matrix is K x K.  The symmetric ones (S, X, H, F, P, G) are
// the same in row- and column-major order; the others (C, FPS-SPF) are kept
// column-major as cuBLAS/cuSOLVER produce them and transposed only when the
// coefficients are returned.  The commutator sign flip of that convention
// does not change the DIIS inner products or norms.
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <cstdio>
#include <mutex>
#include <map>

#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <string>
#include <vector>

#include "hfx_dscf.hpp"
#include "hfx_engine.hpp"

namespace hfx {

static void cublas_check(cublasStatus_t s, const char* what)
{
    if (s != CUBLAS_STATUS_SUCCESS) throw Error(HFX_ERR_CUDA, std::string("cuBLAS ") + what + " failed");
}
static void cusolver_check(cusolverStatus_t s, const char* what)
{
    if (s != CUSOLVER_STATUS_SUCCESS) throw Error(HFX_ERR_CUDA, std::string("cuSOLVER ") + what + " failed");
}

// C = a A + b B
__global__ void k_axpby(int n, double a, const double* A, double b, const double* B, double* C)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) C[e] = a * A[e] + b * B[e];
}
// E = T - T^T (column-major K x K)
__global__ void k_antisym(int K, const double* T, double* E)
{
    int n = K * K;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        int i = e % K, j = e / K;
        E[e] = T[e] - T[j + i * K];
    }
}
struct Coef8 {
    double c[8];
    const double* m[8];
    int n;
};
// C = sum_i c_i M_i
__global__ void k_lincomb(int n, Coef8 cf, double* C)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int i = 0; i < cf.n; ++i) s += cf.c[i] * cf.m[i][e];
        C[e] = s;
    }
}

static int grid_for(int n) { return std::min(1024, std::max(1, (n + 255) / 256)); }

// cuBLAS / cuSOLVER handles, kept per device for reuse: creating them costs
// tens of milliseconds, which every SCF of the request server and of a
// scan's chained points would otherwise pay.  A handle pair serves one
// DeviceScf at a time.
namespace {
struct HandlePair {
    cublasHandle_t blas = nullptr;
    cusolverDnHandle_t solver = nullptr;
};
std::mutex g_handle_mu;
std::map<int, std::vector<HandlePair>> g_handles;

HandlePair acquire_handles()
{
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    {
        std::lock_guard<std::mutex> lk(g_handle_mu);
        auto& v = g_handles[dev];
        if (!v.empty()) {
            HandlePair h = v.back();
            v.pop_back();
            return h;
        }
    }
    HandlePair h;
    cublas_check(cublasCreate(&h.blas), "create");
    if (cusolverDnCreate(&h.solver) != CUSOLVER_STATUS_SUCCESS) {
        cublasDestroy(h.blas);
        throw Error(HFX_ERR_CUDA, "cusolverDnCreate failed");
    }
    return h;
}

void release_handles(HandlePair h)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return;
    std::lock_guard<std::mutex> lk(g_handle_mu);
    g_handles[dev].push_back(h);
}
}  // namespace

DeviceScf::DeviceScf(FockSource& job, const ScfSetup& setup, int nspin) : job_(job), K_(job.K()), nspin_(nspin)
{
    st_ = job.stream();
    HandlePair h = acquire_handles();
    blas_ = h.blas;
    solver_ = h.solver;
    cublas_check(cublasSetStream(blas_, st_), "stream");
    cusolver_check(cusolverDnSetStream(solver_, st_), "stream");
    const size_t n = (size_t)K_ * K_;
    H_.upload(setup.H, st_);
    S_.upload(setup.S, st_);
    X_.upload(setup.X, st_);
    T1_.alloc(n);
    T2_.alloc(n);
    Fp_.alloc(n);
    W_.alloc(K_);
    info_.alloc(1);
    scal_.alloc(64);
    for (int s = 0; s < nspin_; ++s) {
        P_[s].alloc(n);
        Pn_[s].alloc(n);
        F_[s].alloc(n);
        E_[s].alloc(n);
        C_[s].alloc(n);
        Gr_[s].alloc(n);
        Pr_[s].alloc(n);
        dP_[s].alloc(n);
        e_[s].alloc(K_);
        Fq_[s].alloc(n);
    }
    G_.alloc(n);
    Kx_[0].alloc(n);
    Kx_[1].alloc(n);
    dG_.alloc(n);
    dK_[0].alloc(n);
    dK_[1].alloc(n);
    int lwork = 0;
    cusolver_check(cusolverDnDsyevd_bufferSize(solver_, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, K_, Fp_.p, K_,
                                               W_.p, &lwork),
                   "syevd buffer");
    work_.alloc(std::max(1, lwork));
    lwork_ = lwork;
}

DeviceScf::~DeviceScf()
{
    if (st_) cudaStreamSynchronize(st_);
    if (blas_ && solver_) release_handles(HandlePair{blas_, solver_});
}

void DeviceScf::gemm(bool ta, const double* A, bool tb, const double* B, double* C, double alpha, int kdim)
{
    const double beta = 0.0;
    cublas_check(cublasSetPointerMode(blas_, CUBLAS_POINTER_MODE_HOST), "pointer mode");
    int k = kdim > 0 ? kdim : K_;
    cublas_check(cublasDgemm(blas_, ta ? CUBLAS_OP_T : CUBLAS_OP_N, tb ? CUBLAS_OP_T : CUBLAS_OP_N, K_, K_, k, &alpha,
                             A, K_, B, K_, &beta, C, K_),
                 "dgemm");
}

// dot products of device vectors into the device scalar slot `slot`
void DeviceScf::dot(const double* a, const double* b, int n, int slot)
{
    cublas_check(cublasSetPointerMode(blas_, CUBLAS_POINTER_MODE_DEVICE), "pointer mode");
    cublas_check(cublasDdot(blas_, n, a, 1, b, 1, scal_.p + slot), "ddot");
    cublas_check(cublasSetPointerMode(blas_, CUBLAS_POINTER_MODE_HOST), "pointer mode");
}

void DeviceScf::fetch(double* host, int count)
{
    cuda_check(cudaMemcpyAsync(host, scal_.p, sizeof(double) * count, cudaMemcpyDeviceToHost, st_), "D2H scalars");
    cuda_check(cudaStreamSynchronize(st_), "scf sync");
}

void DeviceScf::axpby(double a, const double* A, double b, const double* B, double* C)
{
    int n = K_ * K_;
    k_axpby<<<grid_for(n), 256, 0, st_>>>(n, a, A, b, B, C);
    cuda_check(cudaGetLastError(), "axpby");
}

// Fock matrices of the current densities into F_[s]; mode as BuildMode.
void DeviceScf::build(int mode, double dthr)
{
    const bool mixed = mode == 0 && job_.mixed();
    const double dt = mode == 2 ? dthr : 0.0;
    double* src[2] = {P_[0].p, nspin_ == 2 ? P_[1].p : nullptr};
    if (mode == 2) {
        for (int s = 0; s < nspin_; ++s) axpby(1.0, P_[s].p, -1.0, Pr_[s].p, dP_[s].p);
        src[0] = dP_[0].p;
        if (nspin_ == 2) src[1] = dP_[1].p;
    }
    if (nspin_ == 1) {
        double* out = mode == 2 ? dG_.p : G_.p;
        job_.fock_rhf_device_ex(src[0], out, mixed, dt);
        fock_ms_ += job_.last_build_ms();
        if (mode == 2) axpby(1.0, Gr_[0].p, 1.0, dG_.p, G_.p);
        if (mode >= 1) {  // reference for the next incremental build
            cuda_check(cudaMemcpyAsync(Gr_[0].p, G_.p, sizeof(double) * K_ * K_, cudaMemcpyDeviceToDevice, st_), "copy");
            cuda_check(cudaMemcpyAsync(Pr_[0].p, P_[0].p, sizeof(double) * K_ * K_, cudaMemcpyDeviceToDevice, st_), "copy");
        }
        axpby(1.0, H_.p, 1.0, G_.p, F_[0].p);
    } else {
        double* J = mode == 2 ? dG_.p : G_.p;
        double* Ka = mode == 2 ? dK_[0].p : Kx_[0].p;
        double* Kb = mode == 2 ? dK_[1].p : Kx_[1].p;
        job_.fock_uhf_device_ex(src[0], src[1], J, Ka, Kb, mixed, dt);
        fock_ms_ += job_.last_build_ms();
        if (mode == 2) {
            // reference J in Gr_[0], K_a in Gr_[1]; K_b kept in Kr_
            axpby(1.0, Gr_[0].p, 1.0, dG_.p, G_.p);
            axpby(1.0, Gr_[1].p, 1.0, dK_[0].p, Kx_[0].p);
            axpby(1.0, Kr_.p, 1.0, dK_[1].p, Kx_[1].p);
        }
        if (mode >= 1) {
            if (!Kr_.p) Kr_.alloc((size_t)K_ * K_);
            size_t bytes = sizeof(double) * K_ * K_;
            cuda_check(cudaMemcpyAsync(Gr_[0].p, G_.p, bytes, cudaMemcpyDeviceToDevice, st_), "copy");
            cuda_check(cudaMemcpyAsync(Gr_[1].p, Kx_[0].p, bytes, cudaMemcpyDeviceToDevice, st_), "copy");
            cuda_check(cudaMemcpyAsync(Kr_.p, Kx_[1].p, bytes, cudaMemcpyDeviceToDevice, st_), "copy");
            for (int s = 0; s < 2; ++s)
                cuda_check(cudaMemcpyAsync(Pr_[s].p, P_[s].p, bytes, cudaMemcpyDeviceToDevice, st_), "copy");
        }
        // F_s = H + J - K_s
        for (int s = 0; s < 2; ++s) {
            axpby(1.0, H_.p, 1.0, G_.p, F_[s].p);
            axpby(1.0, F_[s].p, -1.0, Kx_[s].p, F_[s].p);
        }
    }
}

// E_[s] = F P S - S P F for every spin; energy terms and norms into scal_
// slots: [0] = sum_s 1/2 P.(H+F), [1] = sum_s ||E_s||^2
void DeviceScf::error_and_energy()
{
    const int n = K_ * K_;
    for (int s = 0; s < nspin_; ++s) {
        gemm(false, F_[s].p, false, P_[s].p, T1_.p);
        gemm(false, T1_.p, false, S_.p, T2_.p);
        k_antisym<<<grid_for(n), 256, 0, st_>>>(K_, T2_.p, E_[s].p);
        cuda_check(cudaGetLastError(), "antisym");
        axpby(1.0, H_.p, 1.0, F_[s].p, T1_.p);
        dot(P_[s].p, T1_.p, n, 10 + s);
        dot(E_[s].p, E_[s].p, n, 12 + s);
    }
}

// New densities Pn_ of the (DIIS) Fock matrices: P = f X D X^T with D the
// projector onto the nocc lowest eigenvectors of F' = X^T F X.  D comes from
// the SP2 projector (no host synchronisation) when use_proj, else from
// cuSOLVER syevd, which also gives the MO energies e_ and coefficients C_
// (column-major); F' stays in Fq_[s] for a later syevd.
void DeviceScf::diagonalise(const double* const* Fs, const int* nocc, double occ_factor, bool use_proj)
{
    for (int s = 0; s < nspin_; ++s) {
        gemm(false, Fs[s], false, X_.p, T1_.p);        // F X
        gemm(true, X_.p, false, T1_.p, Fq_[s].p);      // X^T F X
        proj_[s] = use_proj && nocc[s] > 0 && nocc[s] < K_;
        if (proj_[s]) {
            // the step count changes little between SCF iterations
            project(s, nocc[s], occ_factor, proj_steps_[s] > 0 ? proj_steps_[s] + 5 : Sp2Projector::kMaxSteps);
        } else {
            eigensolve(s, nocc[s], occ_factor, true);
        }
    }
}

void DeviceScf::project(int s, int nocc, double occ_factor, int max_steps)
{
    if (!sp2_) {
        sp2_.reset(new Sp2Projector(K_));
        D_.alloc((size_t)K_ * K_);
    }
    proj_cap_[s] = max_steps;
    sp2_->run(Fq_[s].p, nocc, D_.p, scal_.p + 2 + s, st_, max_steps);
    gemm(false, X_.p, false, D_.p, T1_.p);                  // X D
    gemm(false, T1_.p, true, T1_.p, Pn_[s].p, occ_factor);  // f (X D)(X D)^T = f X D X^T
}

void DeviceScf::eigensolve(int s, int nocc, double occ_factor, bool density)
{
    cuda_check(cudaMemcpyAsync(Fp_.p, Fq_[s].p, sizeof(double) * K_ * K_, cudaMemcpyDeviceToDevice, st_), "copy");
    cusolver_check(cusolverDnDsyevd(solver_, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, K_, Fp_.p, K_,
                                    e_[s].p, work_.p, lwork_, info_.p),
                   "syevd");
    gemm(false, X_.p, false, Fp_.p, C_[s].p);      // C = X C'
    if (!density) return;
    // P = f C_occ C_occ^T
    if (nocc > 0) {
        gemm(false, C_[s].p, true, C_[s].p, Pn_[s].p, occ_factor, nocc);
    } else {
        cuda_check(cudaMemsetAsync(Pn_[s].p, 0, sizeof(double) * K_ * K_, st_), "memset");
    }
}

ScfOutput DeviceScf::run(const Basis& b, const ScfSetup& setup, const hfx_scf_options& opt_in, int na, int nb,
                         const double* P0a, const double* P0b, double delta_thr, const ScfControl* ctl)
{
    auto t0 = std::chrono::steady_clock::now();
    hfx_scf_options opt = opt_in;
    if (opt.max_iterations <= 0) opt.max_iterations = 10000;
    if (opt.epsilon <= 0) opt.epsilon = 1e-6;
    if (opt.damping <= 0) opt.damping = 0.3;
    if (opt.start_diis <= 0) opt.start_diis = 4;
    if (opt.max_history <= 0) opt.max_history = 8;
    const int K = K_;
    const int n = K * K;
    const size_t bytes = sizeof(double) * n;
    ScfOutput out;
    out.K = K;
    out.E_nuc = setup.E_nuc;
    int n_e = -opt.charge;
    for (int z : b.atom_Z) n_e += z;
    out.n_electrons = n_e;
    int nocc[2];
    double occf;
    if (nspin_ == 1) {
        nocc[0] = n_e / 2;
        occf = 2.0;
    } else {
        if (n_e != na + nb) throw Error(HFX_ERR_INVALID, "inconsistency in electron number");
        nocc[0] = na;
        nocc[1] = nb;
        occf = 1.0;
    }
    for (int s = 0; s < nspin_; ++s) {
        const double* p0 = s == 0 ? P0a : P0b;
        if (p0)
            cuda_check(cudaMemcpyAsync(P_[s].p, p0, bytes, cudaMemcpyHostToDevice, st_), "H2D P0");
        else
            cuda_check(cudaMemsetAsync(P_[s].p, 0, bytes, st_), "memset P");
    }
    // DIIS ring (device matrices) and its inner-product matrix (host)
    const int maxh = opt.max_history;
    std::vector<DevBuf<double>> hF((size_t)maxh * nspin_), hE((size_t)maxh * nspin_);
    for (auto& m : hF) m.alloc(n);
    for (auto& m : hE) m.alloc(n);
    std::deque<int> ring;  // slot ids, oldest first
    std::vector<double> Bm((size_t)maxh * maxh, 0.0);
    const bool mixed = opt.precision == HFX_PREC_MIXED;
    int phase = mixed ? 0 : 2;
    bool have_ref = false;
    MixedPhaseSwitch to_fp64(opt.epsilon);
    const bool use_proj = opt.eigensolver == HFX_EIG_AUTO && K <= Sp2Projector::kScfMaxN;
    proj_[0] = proj_[1] = false;
    proj_steps_[0] = proj_steps_[1] = 0;
    auto do_build = [&]() {
        ++out.fock_builds;
        if (!mixed) {
            build(0, 0.0);
            ++out.fp64_builds;
        } else if (phase == 0) {
            build(0, 0.0);
            ++out.mixed_builds;
        } else if (phase == 1 || !have_ref || opt.fp64_final_cycles < 0) {
            build(1, 0.0);
            ++out.fp64_builds;
            if (opt.fp64_final_cycles >= 0) {
                have_ref = true;
                phase = 2;
            }
        } else {
            build(2, delta_thr);
            ++out.delta_builds;
        }
    };
    double sc[32];
    double E_prev = 0.0;
    int n_it = 0;
    std::vector<double> Pswap;
    for (int it = 0; it < opt.max_iterations; ++it) {
        ++n_it;
        if (ctl) {
            if (ctl->cancel && ctl->cancel->load()) throw Error(HFX_ERR_CANCELLED, "job cancelled");
            if (ctl->deadline > 0.0 &&
                std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count() >
                    ctl->deadline)
                throw Error(HFX_ERR_TIMEOUT, "job exceeded its time limit");
            if (ctl->fault_at_iteration == n_it) throw Error(HFX_ERR_NUMERIC, "injected fault at an SCF iteration");
        }
        do_build();
        error_and_energy();
        // history slot
        // slots in use are always a permutation of 0..size-1: reuse the oldest when full
        int slot;
        if ((int)ring.size() == maxh) {
            slot = ring.front();
            ring.pop_front();
        } else {
            slot = (int)ring.size();
        }
        for (int s = 0; s < nspin_; ++s) {
            cuda_check(cudaMemcpyAsync(hF[slot * nspin_ + s].p, F_[s].p, bytes, cudaMemcpyDeviceToDevice, st_), "copy");
            cuda_check(cudaMemcpyAsync(hE[slot * nspin_ + s].p, E_[s].p, bytes, cudaMemcpyDeviceToDevice, st_), "copy");
        }
        ring.push_back(slot);
        // new row of B: <E_slot, E_r> summed over spins
        for (size_t q = 0; q < ring.size(); ++q)
            for (int s = 0; s < nspin_; ++s) dot(hE[slot * nspin_ + s].p, hE[ring[q] * nspin_ + s].p, n, 16 + 2 * (int)q + s);
        fetch(sc, 32);
        const double E_cur = 0.5 * (sc[10] + (nspin_ == 2 ? sc[11] : 0.0));
        const double en = std::sqrt(sc[12] + (nspin_ == 2 ? sc[13] : 0.0));
        for (size_t q = 0; q < ring.size(); ++q) {
            double v = sc[16 + 2 * q] + (nspin_ == 2 ? sc[16 + 2 * q + 1] : 0.0);
            Bm[(size_t)slot * maxh + ring[q]] = Bm[(size_t)ring[q] * maxh + slot] = v;
        }
        if (!std::isfinite(E_cur)) throw Error(HFX_ERR_NUMERIC, "non-finite energy");
        const double* Fuse[2] = {F_[0].p, nspin_ == 2 ? F_[1].p : nullptr};
        if (n_it >= opt.start_diis) {
            const int hn = (int)ring.size();
            std::vector<double> A((size_t)(hn + 1) * (hn + 1), 0.0), rhs(hn + 1, 0.0), x(hn + 1);
            for (int i = 0; i < hn; ++i)
                for (int j = 0; j < hn; ++j) A[(size_t)i * (hn + 1) + j] = Bm[(size_t)ring[i] * maxh + ring[j]];
            for (int i = 0; i < hn; ++i) {
                A[(size_t)i * (hn + 1) + hn] = -1.0;
                A[(size_t)hn * (hn + 1) + i] = 1.0;
            }
            rhs[hn] = 1.0;
            solve_full_piv(hn + 1, A.data(), rhs.data(), x.data());
            for (int s = 0; s < nspin_; ++s) {
                Coef8 cf{};
                cf.n = hn;
                for (int i = 0; i < hn; ++i) {
                    cf.c[i] = x[i];
                    cf.m[i] = hF[ring[i] * nspin_ + s].p;
                }
                k_lincomb<<<grid_for(n), 256, 0, st_>>>(n, cf, T2_.p);
                cuda_check(cudaGetLastError(), "lincomb");
                // T2_ is reused by error_and_energy; keep the DIIS Fock in E_ (its history copy is saved)
                cuda_check(cudaMemcpyAsync(E_[s].p, T2_.p, bytes, cudaMemcpyDeviceToDevice, st_), "copy");
                Fuse[s] = E_[s].p;
            }
        }
        diagonalise(Fuse, nocc, occf, use_proj);
        // RMSD(P_new - P) per spin
        for (int s = 0; s < nspin_; ++s) {
            axpby(1.0, Pn_[s].p, -1.0, P_[s].p, T1_.p);
            dot(T1_.p, T1_.p, n, s);
        }
        fetch(sc, 4);
        // a projection that did not converge within the step cap is repeated
        // with the full cap; one that did not converge at all (no gap at the
        // Fermi level) is replaced by an eigensolve
        double status[2] = {-1.0, -1.0};
        bool counted[2] = {false, false};
        for (;;) {
            bool refetch = false;
            for (int s = 0; s < nspin_; ++s) {
                if (!proj_[s] || counted[s]) continue;
                status[s] = sc[2 + s];
                if (sc[2 + s] > 0.0) {
                    ++out.projections;
                    proj_steps_[s] = (int)sc[2 + s];
                    counted[s] = true;
                    continue;
                }
                if (proj_cap_[s] < Sp2Projector::kMaxSteps) {
                    project(s, nocc[s], occf, Sp2Projector::kMaxSteps);
                } else {
                    ++out.projection_fallbacks;
                    proj_[s] = false;
                    proj_steps_[s] = 0;
                    eigensolve(s, nocc[s], occf, true);
                }
                axpby(1.0, Pn_[s].p, -1.0, P_[s].p, T1_.p);
                dot(T1_.p, T1_.p, n, s);
                refetch = true;
            }
            if (!refetch) break;
            fetch(sc, 4);
        }
        double rm = 0.0;
        for (int s = 0; s < nspin_; ++s) rm = std::max(rm, std::sqrt(sc[s] / n));
        const bool dE_ok = opt.energy_threshold <= 0 || (n_it > 1 && std::fabs(E_cur - E_prev) < opt.energy_threshold);
        E_prev = E_cur;
        out.last_rmsd = rm;
        if (opt.verbose)
            std::fprintf(stderr,
                         "scf iteration %3d  phase %d  E %.12f  rmsd(P) %.3e  ||FPS-SPF|| %.3e  projector steps %d %d "
                         "(status %g %g)\n",
                         n_it, phase, E_cur + out.E_nuc, rm, en, proj_steps_[0], proj_steps_[1], status[0], status[1]);
        if (phase == 0 && to_fp64.update(rm, en)) phase = 1;
        bool done = false;
        if (rm < opt.epsilon && en < opt.epsilon && dE_ok && phase != 0) {
            // final check at the new densities
            for (int s = 0; s < nspin_; ++s) std::swap(P_[s].p, Pn_[s].p);
            do_build();
            error_and_energy();
            fetch(sc, 14);
            double fe = std::sqrt(sc[12] + (nspin_ == 2 ? sc[13] : 0.0));
            if (fe < opt.epsilon) {
                out.converged = true;
                out.E_ele = 0.5 * (sc[10] + (nspin_ == 2 ? sc[11] : 0.0));
                out.E_tot = out.E_nuc + out.E_ele;
                done = true;
            } else {
                for (int s = 0; s < nspin_; ++s) std::swap(P_[s].p, Pn_[s].p);
            }
        }
        if (done) break;
        for (int s = 0; s < nspin_; ++s) {
            if (n_it >= opt.start_diis)
                std::swap(P_[s].p, Pn_[s].p);
            else
                axpby(opt.damping, Pn_[s].p, 1.0 - opt.damping, P_[s].p, P_[s].p);
        }
        if (it == opt.max_iterations - 1) {
            if (phase == 0) phase = 1;
            do_build();
            error_and_energy();
            fetch(sc, 14);
            out.E_ele = 0.5 * (sc[10] + (nspin_ == 2 ? sc[11] : 0.0));
            out.E_tot = out.E_nuc + out.E_ele;
        }
    }
    out.iterations = n_it;
    // MO energies and coefficients of the last density step where it was a projection
    for (int s = 0; s < nspin_; ++s)
        if (proj_[s]) eigensolve(s, nocc[s], occf, false);
    // results to the host: densities, MO energies, coefficients (row-major)
    out.P.resize(n);
    cuda_check(cudaMemcpyAsync(out.P.data(), P_[0].p, bytes, cudaMemcpyDeviceToHost, st_), "D2H P");
    out.e.resize(K);
    cuda_check(cudaMemcpyAsync(out.e.data(), e_[0].p, sizeof(double) * K, cudaMemcpyDeviceToHost, st_), "D2H e");
    std::vector<double> Ccm(n);
    cuda_check(cudaMemcpyAsync(Ccm.data(), C_[0].p, bytes, cudaMemcpyDeviceToHost, st_), "D2H C");
    if (nspin_ == 2) {
        out.P2.resize(n);
        out.e2.resize(K);
        cuda_check(cudaMemcpyAsync(out.P2.data(), P_[1].p, bytes, cudaMemcpyDeviceToHost, st_), "D2H P");
        cuda_check(cudaMemcpyAsync(out.e2.data(), e_[1].p, sizeof(double) * K, cudaMemcpyDeviceToHost, st_), "D2H e");
    }
    cuda_check(cudaStreamSynchronize(st_), "scf results");
    out.C.resize(n);
    for (int i = 0; i < K; ++i)
        for (int j = 0; j < K; ++j) out.C[(size_t)i * K + j] = Ccm[(size_t)j * K + i];
    if (!std::isfinite(out.E_tot)) throw Error(HFX_ERR_NUMERIC, "non-finite SCF energy");
    out.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    out.fock_ms = fock_ms_;
    return out;
}

}  // namespace hfx
