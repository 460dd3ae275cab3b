// hfx_sp2.cu -- occupied-space projector by trace-correcting SP2 (see
// hfx_sp2.hpp).
//
// One step computes X_j from X_{j-1} and X_{j-1}^2 (X_j = X^2 or 2X - X^2)
// and then X_j^2, as an 8 x 8 output tile per block over the upper triangle
// (the mirror tile is written from the same values, so every X_j and X_j^2 is
// exactly symmetric).  A block stages the two 8-row panels of X_j it needs in
// shared memory, forming them on the fly from the previous step's matrices.
// The recursion's control -- which branch, when to stop -- depends only on
// tr(X_{j-1}) and tr(X_{j-1}^2), summed in a fixed order from per-tile
// partial traces by every block alike, so all blocks agree without a grid
// barrier and the result is deterministic.  Matrices alternate between two
// buffers by step parity.
#include <algorithm>
#include <cmath>

#include "hfx_sp2.hpp"

namespace hfx {
namespace {

constexpr int kTile = 8;
constexpr int kThreads = 256;       // 64 outputs x 4 slices of the inner dimension
// Stop two steps after sum_i lambda_i (1 - lambda_i) = tr(X) - tr(X^2) falls
// below this: each of the two steps squares the larger of the occupied and
// virtual deviations, leaving them at rounding level.  The traces' own
// rounding is ~1e-13 for n <= 1024.
constexpr double kIdemTol = 1e-10;
constexpr double kTraceTol = 1e-6;  // tr(D) = nocc: otherwise no gap (fractional occupation)

// Gershgorin bounds of sym(F) = (F + F^T) / 2, one warp per row:
// bounds[0] = min_i (f_ii - r_i), bounds[1] = max_i (f_ii + r_i).
__global__ void __launch_bounds__(1024) k_sp2_bounds(int n, const double* __restrict__ F, double* __restrict__ bounds)
{
    __shared__ double lo_w[32], hi_w[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double lo = INFINITY, hi = -INFINITY;
    for (int i = warp; i < n; i += nw) {
        double r = 0.0;
        for (int c = lane; c < n; c += 32)
            if (c != i) r += fabs(0.5 * (F[(size_t)i * n + c] + F[(size_t)c * n + i]));
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
        const double d = F[(size_t)i * n + i];
        lo = fmin(lo, d - r);
        hi = fmax(hi, d + r);
    }
    if (lane == 0) {
        lo_w[warp] = lo;
        hi_w[warp] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < nw; ++w) {
            lo = fmin(lo, lo_w[w]);
            hi = fmax(hi, hi_w[w]);
        }
        bounds[0] = lo;
        bounds[1] = hi;
    }
}

struct Sp2Decision {
    int branch;  // 0: X_0 from F; 1: X <- X^2; 2: X <- 2X - X^2
    int kstar;   // first step with tr(X) - tr(X^2) < kIdemTol (-1: none yet)
    int answer;  // step whose X is the projector (-1: not yet)
};

// Fixed-order sums of the first m entries of v over one warp (lane 0's
// reduction order, broadcast), so that every block obtains the same bits.
__device__ __forceinline__ double warp_sum_fixed(const double* v, int m)
{
    const int lane = threadIdx.x & 31;
    double s = 0.0;
    for (int t = lane; t < m; t += 32) s += v[t];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    return __shfl_sync(0xffffffffu, s, 0);
}

// The recursion's control before step j, from the state and traces that step
// j-1 left.  Called by one whole warp; the same result in every block.
__device__ Sp2Decision sp2_decide(int j, int nt, int nocc, const double* traces, const int* state)
{
    Sp2Decision d{0, -1, -1};
    if (j == 0) return d;
    d.kstar = state[2 * (j - 1)];
    d.answer = state[2 * (j - 1) + 1];
    if (d.answer >= 0) return d;  // step j-1 did nothing, its traces are not written
    const double* px = traces + (size_t)(j - 1) * 2 * nt;
    const double sx = warp_sum_fixed(px, nt);
    const double sx2 = warp_sum_fixed(px + nt, nt);
    if (d.kstar < 0 && sx - sx2 < kIdemTol) d.kstar = j - 1;
    if (d.kstar >= 0 && j - 1 >= d.kstar + 2) d.answer = j - 1;
    d.branch = fabs(sx2 - nocc) < fabs(2.0 * sx - sx2 - nocc) ? 1 : 2;
    return d;
}

// element (r, c) of X_j
__device__ __forceinline__ double sp2_form(int branch, int n, int r, int c, const double* F, double emax,
                                           double inv_w, const double* Xp, const double* X2p)
{
    const size_t e = (size_t)r * n + c;
    if (branch == 0) {
        const double f = 0.5 * (F[e] + F[(size_t)c * n + r]);
        return ((r == c ? emax : 0.0) - f) * inv_w;
    }
    if (branch == 1) return X2p[e];
    return 2.0 * Xp[e] - X2p[e];
}

__global__ void __launch_bounds__(kThreads) k_sp2_step(int n, int nt, int nocc, int j, const double* __restrict__ F,
                                                        const double* __restrict__ bounds, const double* Xp,
                                                        const double* X2p, double* Xo, double* X2o,
                                                        double* __restrict__ traces, int* __restrict__ state)
{
    extern __shared__ double sm[];
    const int ld = n + 1;  // odd row stride: the 8 rows of a panel fall in distinct banks
    double* A = sm;
    double* B = sm + kTile * ld;
    double* red = B + kTile * ld;
    __shared__ int s_branch, s_kstar, s_answer;
    if (threadIdx.x < 32) {
        const Sp2Decision d = sp2_decide(j, nt, nocc, traces, state);
        if (threadIdx.x == 0) {
            s_branch = d.branch;
            s_kstar = d.kstar;
            s_answer = d.answer;
        }
    }
    __syncthreads();
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        state[2 * j] = s_kstar;
        state[2 * j + 1] = s_answer;
    }
    if (s_answer >= 0) return;
    const int branch = s_branch;
    // tile (I, J), I <= J, in row-major order of the upper triangle
    int b = blockIdx.x, I = 0;
    while (b >= nt - I) {
        b -= nt - I;
        ++I;
    }
    const int J = I + b;
    const double emax = bounds[1];
    const double inv_w = 1.0 / (bounds[1] - bounds[0]);
    for (int e = threadIdx.x; e < kTile * n; e += kThreads) {
        const int r = e / n, c = e - r * n;
        const int ra = I * kTile + r, rb = J * kTile + r;
        A[r * ld + c] = ra < n ? sp2_form(branch, n, ra, c, F, emax, inv_w, Xp, X2p) : 0.0;
        B[r * ld + c] = rb < n ? sp2_form(branch, n, rb, c, F, emax, inv_w, Xp, X2p) : 0.0;
    }
    __syncthreads();
    const int o = threadIdx.x & 63, ks = threadIdx.x >> 6;
    const int a = o >> 3, bb = o & 7;
    const double* Ar = A + a * ld;
    const double* Br = B + bb * ld;  // X_j is symmetric: row panel J is column panel J
    double acc = 0.0;
    for (int k = ks; k < n; k += 4) acc = fma(Ar[k], Br[k], acc);
    red[threadIdx.x] = acc;
    __syncthreads();
    if (threadIdx.x < 64) {
        const double v = (red[o] + red[o + 64]) + (red[o + 128] + red[o + 192]);
        const int row = I * kTile + a, col = J * kTile + bb;
        if (row < n && col < n) {
            const double x = A[a * ld + col];
            X2o[(size_t)row * n + col] = v;
            Xo[(size_t)row * n + col] = x;
            if (I != J) {
                X2o[(size_t)col * n + row] = v;
                Xo[(size_t)col * n + row] = x;
            }
        }
        red[o] = v;  // each thread reads and writes only its own o entries
    }
    if (I == J) {  // block-uniform
        __syncthreads();
        if (threadIdx.x == 0) {
            double tx = 0.0, tx2 = 0.0;
            for (int q = 0; q < kTile && I * kTile + q < n; ++q) {
                tx += A[q * ld + I * kTile + q];
                tx2 += red[q * kTile + q];
            }
            traces[(size_t)j * 2 * nt + I] = tx;
            traces[(size_t)j * 2 * nt + nt + I] = tx2;
        }
    }
}

__global__ void __launch_bounds__(256) k_sp2_finish(int n, int nt, int nocc, int steps, const double* __restrict__ traces,
                                                     const int* __restrict__ state, const double* X0,
                                                     const double* X1, double* __restrict__ D, double* status)
{
    __shared__ int s_answer;
    if (threadIdx.x < 32) {
        const Sp2Decision d = sp2_decide(steps, nt, nocc, traces, state);
        int ans = d.answer;
        if (ans >= 0) {
            const double tr = warp_sum_fixed(traces + (size_t)ans * 2 * nt, nt);
            if (!(fabs(tr - nocc) < kTraceTol)) ans = -1;
        }
        if (threadIdx.x == 0) s_answer = ans;
    }
    __syncthreads();
    const int ans = s_answer;
    if (blockIdx.x == 0 && threadIdx.x == 0) *status = ans >= 0 ? (double)(ans + 1) : 0.0;
    if (ans < 0) return;
    const double* X = (ans & 1) ? X1 : X0;
    const size_t total = (size_t)n * n;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
        D[e] = X[e];
}

}  // namespace

Sp2Projector::Sp2Projector(int n) : n_(n), nt_((n + kTile - 1) / kTile)
{
    if (n < 1 || n > kMaxN) throw Error(HFX_ERR_INVALID, "SP2 projector: matrix dimension out of range");
    const size_t nn = (size_t)n * n;
    for (int p = 0; p < 2; ++p) {
        X_[p].alloc(nn);
        X2_[p].alloc(nn);
    }
    bounds_.alloc(2);
    traces_.alloc((size_t)kMaxSteps * 2 * nt_);
    state_.alloc((size_t)kMaxSteps * 2);
    smem_ = sizeof(double) * ((size_t)2 * kTile * (n + 1) + kThreads);
    // The limit is a property of the kernel, shared by every projector in the
    // process: always raise it to what the largest n needs, never to this n's
    // figure, which would lower it under a concurrent projector of larger n.
    const size_t smem_max = sizeof(double) * ((size_t)2 * kTile * (kMaxN + 1) + kThreads);
    cuda_check(cudaFuncSetAttribute(k_sp2_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max),
               "SP2 shared memory");
}

void Sp2Projector::run(const double* F, int nocc, double* D, double* status, cudaStream_t st, int max_steps)
{
    if (nocc <= 0 || nocc >= n_) throw Error(HFX_ERR_INVALID, "SP2 projector: occupation out of range");
    const int steps = std::max(1, std::min(max_steps, kMaxSteps));
    k_sp2_bounds<<<1, 1024, 0, st>>>(n_, F, bounds_.p);
    const int blocks = nt_ * (nt_ + 1) / 2;
    for (int j = 0; j < steps; ++j) {
        const int cur = j & 1, prev = cur ^ 1;
        k_sp2_step<<<blocks, kThreads, smem_, st>>>(n_, nt_, nocc, j, F, bounds_.p, X_[prev].p, X2_[prev].p,
                                                     X_[cur].p, X2_[cur].p, traces_.p, state_.p);
    }
    const int grid = (int)std::min<size_t>(1024, ((size_t)n_ * n_ + 255) / 256);
    k_sp2_finish<<<grid, 256, 0, st>>>(n_, nt_, nocc, steps, traces_.p, state_.p, X_[0].p, X_[1].p, D, status);
    cuda_check(cudaGetLastError(), "SP2 projector");
}

}  // namespace hfx
