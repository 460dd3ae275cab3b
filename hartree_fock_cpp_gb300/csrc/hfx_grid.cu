// hfx_grid.cu -- electron density and orbitals on grids of points.
//
// The reference evaluates rho(r) = sum_{mu,nu} P_{mu nu} phi_mu(r) phi_nu(r)
// and psi_i(r) = sum_mu C_{mu i} phi_mu(r) point by point (cube.hpp:9-135 on
// the host; evaluation.cuh:59-123 on the GPU, one thread per point, two basis
// function evaluations -- each a loop of exponentials -- per (mu, nu) pair).
// Here a CTA owns a tile of kTile points:
//   1. its 4 thread groups evaluate every shell once per point (one
//      exponential per primitive, shared by the shell's Cartesian
//      components) into a shared-memory tile Phi[mu][point];
//   2. density: each group takes every 4th row mu and forms
//      Phi_mu (P_mu,mu Phi_mu + 2 sum_{nu > mu} P_mu,nu Phi_nu) -- P's row is
//      uniform across the warp (broadcast loads), Phi reads are consecutive;
//      orbital: sum_mu C_mu,i Phi_mu;
//   3. the groups' partial sums are added in shared memory.
// Grid coordinates follow the reference's box_points / linspace
// (cube.hpp:137-168, visual.hpp:42-51): x_i = start + i * step with
// step = (stop - start) / (res - 1), rounded the same way (no fused
// multiply-add), index (i * res + j) * res + k (indexing.hpp:10-12).
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "hfx_engine.hpp"

namespace hfx {

namespace {

constexpr int kTile = 32;      // points per CTA
constexpr int kGroups = 4;     // thread groups per CTA
constexpr int kGridThreads = kTile * kGroups;

struct GridShell {
    double x, y, z;
    int L, bf0, nprim, prim0;   // exponents [prim0, prim0 + nprim); weights at woff
    int woff, pad;
};

struct GridArgs {
    const GridShell* sh;
    int nsh;
    const double* exps;
    const double* w;            // per shell: w[c * nprim + i] = coefficient x cart_norm
    int K;
    const double* M;            // density P (K x K) or coefficients C (K x K)
    int column;                 // orbital mode: column of C; density mode: -1
    // points: either explicit (xyz) or the res^3 box (start, step)
    const double* xyz;          // 3 n coordinates of this launch's points (null: box points)
    long long first, n;         // point range of this launch
    int res;
    double sx, sy, sz, hx, hy, hz;
    double* out;                // n values
};

__device__ __forceinline__ double ipow(double b, int e)
{
    double r = 1.0;
    for (int i = 0; i < e; ++i) r *= b;
    return r;
}

__global__ void __launch_bounds__(kGridThreads) k_grid_eval(GridArgs a)
{
    extern __shared__ __align__(16) double phi[];   // [K][kTile], then partial sums [kGroups][kTile]
    double* part = phi + (size_t)a.K * kTile;
    const int p = threadIdx.x % kTile, g = threadIdx.x / kTile;
    const long long idx = a.first + (long long)blockIdx.x * kTile + p;
    const bool live = idx < a.first + a.n;
    double rx = 0.0, ry = 0.0, rz = 0.0;
    if (live) {
        if (a.xyz) {
            const long long li = idx - a.first;
            rx = a.xyz[3 * li];
            ry = a.xyz[3 * li + 1];
            rz = a.xyz[3 * li + 2];
        } else {
            const long long r2 = (long long)a.res * a.res;
            const int i = (int)(idx / r2), j = (int)((idx / a.res) % a.res), k = (int)(idx % a.res);
            rx = __dadd_rn(a.sx, __dmul_rn((double)i, a.hx));
            ry = __dadd_rn(a.sy, __dmul_rn((double)j, a.hy));
            rz = __dadd_rn(a.sz, __dmul_rn((double)k, a.hz));
        }
    }
    // 1. basis functions at the tile's points
    for (int s = g; s < a.nsh; s += kGroups) {
        const GridShell S = a.sh[s];
        const double dx = rx - S.x, dy = ry - S.y, dz = rz - S.z;
        const double d2 = dx * dx + dy * dy + dz * dz;
        double e[32];
        const int np = min(S.nprim, 32);
        for (int i = 0; i < np; ++i) e[i] = exp(-a.exps[S.prim0 + i] * d2);
        int c = 0;
        for (int lx = 0; lx <= S.L; ++lx)
            for (int ly = 0; ly <= S.L - lx; ++ly, ++c) {
                const int lz = S.L - lx - ly;
                double v = 0.0;
                const double* wc = a.w + S.woff + c * S.nprim;
                for (int i = 0; i < np; ++i) v += wc[i] * e[i];
                phi[(size_t)(S.bf0 + c) * kTile + p] = live ? ipow(dx, lx) * ipow(dy, ly) * ipow(dz, lz) * v : 0.0;
            }
    }
    __syncthreads();
    // 2. contraction with P (density) or a column of C (orbital)
    double acc = 0.0;
    if (a.column < 0) {
        for (int mu = g; mu < a.K; mu += kGroups) {
            const double pm = phi[(size_t)mu * kTile + p];
            const double* Prow = a.M + (size_t)mu * a.K;
            double t = 0.0;
            for (int nu = mu + 1; nu < a.K; ++nu) t += __ldg(Prow + nu) * phi[(size_t)nu * kTile + p];
            acc += pm * (__ldg(Prow + mu) * pm + 2.0 * t);
        }
    } else {
        for (int mu = g; mu < a.K; mu += kGroups)
            acc += __ldg(a.M + (size_t)mu * a.K + a.column) * phi[(size_t)mu * kTile + p];
    }
    part[g * kTile + p] = acc;
    __syncthreads();
    if (g == 0 && live) {
        double s = 0.0;
        for (int q = 0; q < kGroups; ++q) s += part[q * kTile + p];
        a.out[idx - a.first] = s;
    }
}

cudaError_t allow_grid_smem()
{
    static std::mutex mu;
    static bool done = false;
    std::lock_guard<std::mutex> lk(mu);
    if (done) return cudaSuccess;
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa{};
    cudaError_t e = cudaFuncGetAttributes(&fa, k_grid_eval);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_grid_eval, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
    if (e == cudaSuccess) done = true;
    return e;
}

size_t grid_smem_limit()
{
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return (size_t)optin - 1024;
}

}  // namespace

// Values at n points: rho (column < 0, M = P) or psi_column (M = C).  Points
// are xyz (3n, host) or, when xyz is null, the res^3 box starting at start[]
// with spacing step[].  out: n host doubles.
void grid_eval(const Basis& b, int device, const double* M, int column, const double* xyz, long long n, int res,
               const double* start, const double* step, double* out)
{
    cuda_check(cudaSetDevice(device), "cudaSetDevice");
    const int K = b.K;
    const size_t smem = sizeof(double) * ((size_t)K * kTile + kGroups * kTile);
    if (smem > grid_smem_limit()) throw Error(HFX_ERR_UNSUPPORTED, "grid evaluation: K too large for one tile");
    std::vector<GridShell> sh;
    std::vector<double> exps, w;
    for (const Shell& s : b.shells) {
        if (s.nprim() > 32) throw Error(HFX_ERR_UNSUPPORTED, "grid evaluation: more than 32 primitives in a shell");
        sh.push_back(GridShell{s.x, s.y, s.z, s.L, s.bf0, s.nprim(), (int)exps.size(), (int)w.size(), 0});
        exps.insert(exps.end(), s.exps.begin(), s.exps.end());
        w.insert(w.end(), s.w.begin(), s.w.end());
    }
    cuda_check(allow_grid_smem(), "grid kernel attribute");
    cudaStream_t st;
    cuda_check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    try {
        DevBuf<GridShell> d_sh;
        DevBuf<double> d_exps, d_w, d_M, d_xyz, d_out;
        d_sh.upload(sh, st);
        d_exps.upload(exps, st);
        d_w.upload(w, st);
        d_M.alloc((size_t)K * K);
        cuda_check(cudaMemcpyAsync(d_M.p, M, sizeof(double) * K * K, cudaMemcpyHostToDevice, st), "upload matrix");
        const long long chunk = std::min<long long>(n, 8LL << 20);   // 64 MB of values per launch
        d_out.alloc((size_t)std::max<long long>(1, chunk));
        if (xyz) d_xyz.alloc((size_t)3 * std::max<long long>(1, chunk));
        for (long long f = 0; f < n; f += chunk) {
            const long long m = std::min(chunk, n - f);
            GridArgs a{};
            a.sh = d_sh.p;
            a.nsh = (int)sh.size();
            a.exps = d_exps.p;
            a.w = d_w.p;
            a.K = K;
            a.M = d_M.p;
            a.column = column;
            if (xyz) {
                cuda_check(cudaMemcpyAsync(d_xyz.p, xyz + 3 * f, sizeof(double) * 3 * m, cudaMemcpyHostToDevice, st),
                           "upload points");
                a.xyz = d_xyz.p;
            }
            a.first = f;
            a.n = m;
            a.res = res;
            if (!xyz) {
                a.sx = start[0];
                a.sy = start[1];
                a.sz = start[2];
                a.hx = step[0];
                a.hy = step[1];
                a.hz = step[2];
            }
            a.out = d_out.p;
            const unsigned grid = (unsigned)((m + kTile - 1) / kTile);
            k_grid_eval<<<grid, kGridThreads, smem, st>>>(a);
            cuda_check(cudaGetLastError(), "grid kernel");
            cuda_check(cudaMemcpyAsync(out + f, d_out.p, sizeof(double) * m, cudaMemcpyDeviceToHost, st), "download");
            cuda_check(cudaStreamSynchronize(st), "grid evaluation");
        }
    } catch (...) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
        throw;
    }
    cudaStreamDestroy(st);
}

}  // namespace hfx
