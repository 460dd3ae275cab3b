// hfx_sp2.hpp -- density projector of the orthogonalised Fock matrix by
// second-order spectral projection (SP2), in place of a full eigensolve in the
// SCF iterations.
#pragma once

#include <cuda_runtime.h>

#include "hfx_engine.hpp"

namespace hfx {

// Projector D onto the span of the nocc lowest eigenvectors of a symmetric
// n x n matrix F (the orthogonalised Fock matrix X^T F X), by the
// trace-correcting SP2 recursion (A. M. N. Niklasson, Phys. Rev. B 66,
// 155115 (2002)): X_0 = (e_max I - F) / (e_max - e_min) from Gershgorin
// bounds, then X <- X^2 or X <- 2X - X^2, whichever brings tr(X^2) closer to
// nocc, until X is idempotent.  For a HOMO-LUMO gap g and spectral width W it
// takes about 2 log2(W / g) + 8 steps, each one symmetric n x n product; the
// result equals C_occ C_occ^T of an exact eigensolve to rounding (~1e-14).
//
// Everything stays on the device (no host synchronisation): a fixed number of
// launches of the step kernel (at most kMaxSteps), each of which returns at
// once after convergence, then a finishing kernel that copies the projector
// and writes a status word.
class Sp2Projector {
public:
    static constexpr int kMaxN = 1024;       // shared-memory panels of the step kernel
    static constexpr int kMaxSteps = 100;
    // Largest n for which it beats cuSOLVER syevd plus the density GEMM on a
    // GB300 (0.77 vs 5.2 ms at n = 120, 6.5 vs 13.1 ms at 454, 16 vs 19 ms at
    // 600, 35 vs 26 ms at 800; about 44 steps each).
    static constexpr int kScfMaxN = 640;

    explicit Sp2Projector(int n);
    // D <- projector (n x n); *status (device double) <- number of steps when
    // converged with tr(D) = nocc within max_steps (<= kMaxSteps), else 0 (no
    // gap, or too few steps: the caller falls back to an eigensolve).  F is not
    // modified.  Requires 0 < nocc < n.  Steps after convergence cost one
    // launch each; callers that iterate pass the last count plus a margin.
    void run(const double* F, int nocc, double* D, double* status, cudaStream_t st, int max_steps = kMaxSteps);

private:
    int n_, nt_;
    size_t smem_;
    DevBuf<double> X_[2], X2_[2], bounds_, traces_;
    DevBuf<int> state_;
};

}  // namespace hfx
