// hfx_onee_gpu.cu -- one-electron matrices S, T, V on the device.
//
// The reference's overlap_matrix / kinetic_matrix / attraction_matrix
// (integrals.hpp:10-536) evaluate every basis-function pair on the host; the
// host restatement here (hfx_onee.cpp) does it per shell pair.  For the
// setup of served jobs (K up to ~600, ~70 nuclei) the nuclear attraction
// dominates: per primitive pair and nucleus, one Boys evaluation, one R
// recursion and a Hermite contraction per component pair.  This kernel
// spreads that over the GPU:
//   * one CTA per shell pair (A >= B in shell order), 64 threads;
//   * work item = (primitive pair, chunk of 8 nuclei); a thread builds the
//     1-D Hermite coefficients E^{ij}_t of its primitive pair (j up to
//     l_B + 2 for the kinetic term), adds S and T (first chunk only) and V
//     for its nuclei into shared-memory accumulators;
//   * the CTA writes the pair's block and its transpose.
// Same formulas as the host path:
//   S = E^x_0 E^y_0 E^z_0 (pi/p)^{3/2}
//   T^x_ij = b(2j+1) S_ij - 2 b^2 S_i,j+2 - j(j-1)/2 S_i,j-2  (integrals.hpp:122-177)
//   V = -sum_C Z_C 2 pi / p sum_tuv E_t E_u E_v R_tuv(p, P - C)
// with the Boys table of the Fock-build kernels (T_k = k/16, 7-term Taylor,
// downward recursion; asymptotic form beyond T = 36).
#include <cuda_runtime.h>

#include <cmath>
#include <map>
#include <mutex>
#include <vector>

#include "hfx_device.cuh"
#include "hfx_engine.hpp"

namespace hfx {


namespace {

constexpr int kOneeThreads = 64;
constexpr int kNucChunk = 8;
constexpr int kMaxLa = 3, kMaxJm = 5, kMaxNt = kMaxLa + kMaxJm + 1;   // E arrays per direction
constexpr int kMaxHerm = 84;                                          // Hermite triples up to L = 6

struct OneeShell {
    double x, y, z;
    int L, bf0, nprim, prim0;   // primitives [prim0, prim0 + nprim) of exps; weights at w + woff
    int woff, pad;
};

struct Nucleus {
    double x, y, z, Z;
};

struct OneeArgs {
    const OneeShell* sh;
    const double* exps;
    const double* w;        // per shell: w[c * nprim + i] = coefficient x cart_norm of component c
    const int2* pairs;      // (A, B), A >= B
    const Nucleus* nuc;
    int natom;
    const double* boys;     // [kBoysN][kBoysM], last column exp(-T_k)
    int K;
    double* S;
    double* T;
    double* V;
};

__device__ __forceinline__ int ncomp(int l) { return (l + 1) * (l + 2) / 2; }

// component c of a shell with angular momentum L (angmom_partition order, basis.hpp:52-64)
__device__ __forceinline__ void comp(int L, int c, int& lx, int& ly, int& lz)
{
    int k = 0;
    for (int x = 0; x <= L; ++x)
        for (int y = 0; y <= L - x; ++y) {
            if (k == c) {
                lx = x;
                ly = y;
                lz = L - x - y;
                return;
            }
            ++k;
        }
    lx = ly = lz = 0;
}

// E^{ij}_t, i <= la, j <= jm, into E[(i * (kMaxJm + 1) + j) * kMaxNt + t]
__device__ void hermite_1d_dev(int la, int jm, double a, double b, double A, double B, double* E)
{
    const double p = a + b, mu = a * b / p, AB = A - B;
    const double XPA = -(b / p) * AB, XPB = (a / p) * AB, o2p = 0.5 / p;
    auto at = [&](int i, int j, int t) -> double& { return E[(i * (kMaxJm + 1) + j) * kMaxNt + t]; };
    for (int i = 0; i <= la; ++i)
        for (int j = 0; j <= jm; ++j)
            for (int t = 0; t < kMaxNt; ++t) at(i, j, t) = 0.0;
    at(0, 0, 0) = exp(-mu * AB * AB);
    for (int i = 1; i <= la; ++i)
        for (int t = 0; t <= i; ++t) {
            double v = XPA * at(i - 1, 0, t);
            if (t > 0) v += o2p * at(i - 1, 0, t - 1);
            if (t + 1 <= i - 1) v += (t + 1) * at(i - 1, 0, t + 1);
            at(i, 0, t) = v;
        }
    for (int i = 0; i <= la; ++i)
        for (int j = 1; j <= jm; ++j)
            for (int t = 0; t <= i + j; ++t) {
                double v = (t <= i + j - 1) ? XPB * at(i, j - 1, t) : 0.0;
                if (t > 0) v += o2p * at(i, j - 1, t - 1);
                if (t + 1 <= i + j - 1) v += (t + 1) * at(i, j - 1, t + 1);
                at(i, j, t) = v;
            }
}

// F_0..F_L(T), L <= 6: table + Taylor for F_L and exp(-T), downward recursion;
// beyond the table the asymptotic F_0 and upward recursion.
__device__ void boys_rt(int L, double Tv, const double* __restrict__ tab, double* F)
{
    if (Tv < (double)kBoysTMax) {
        const int k = (int)(Tv * kBoysInvStep + 0.5);
        const double nd = (double)k / kBoysInvStep - Tv;
        const double* f = tab + k * kBoysM + L;
        double r = __ldg(f + 6) * (1.0 / 720.0);
        r = fma(r, nd, __ldg(f + 5) * (1.0 / 120.0));
        r = fma(r, nd, __ldg(f + 4) * (1.0 / 24.0));
        r = fma(r, nd, __ldg(f + 3) * (1.0 / 6.0));
        r = fma(r, nd, __ldg(f + 2) * 0.5);
        r = fma(r, nd, __ldg(f + 1));
        F[L] = fma(r, nd, __ldg(f));
        double x = 1.0 / 5040.0;
        x = fma(x, nd, 1.0 / 720.0);
        x = fma(x, nd, 1.0 / 120.0);
        x = fma(x, nd, 1.0 / 24.0);
        x = fma(x, nd, 1.0 / 6.0);
        x = fma(x, nd, 0.5);
        x = fma(x, nd, 1.0);
        x = fma(x, nd, 1.0);
        const double e = __ldg(tab + k * kBoysM + (kBoysM - 1)) * x;
        for (int m = L - 1; m >= 0; --m) F[m] = (2.0 * Tv * F[m + 1] + e) / (2 * m + 1);
    } else {
        const double e = exp(-Tv);
        F[0] = 0.88622692545275801365 * rsqrt(Tv);
        for (int m = 0; m < L; ++m) F[m + 1] = ((2 * m + 1) * F[m] - e) / (2.0 * Tv);
    }
}

// R^{(0)}_{tuv}(p, (X,Y,Z)) for t+u+v <= L into R[herm_index(t,u,v)]
__device__ void hermite_R_rt(int L, double p, double X, double Y, double Z, const double* F, double* R)
{
    double buf[kMaxHerm];
    double* nxt = R;
    double* cur = buf;
    double pw = 1.0;
    for (int m = 0; m < L; ++m) pw *= -2.0 * p;
    nxt[0] = pw * F[L];
    for (int m = L - 1; m >= 0; --m) {
        pw /= -2.0 * p;
        cur[0] = pw * F[m];
        const int top = L - m;
        for (int s = 1; s <= top; ++s)
            for (int t = 0; t <= s; ++t)
                for (int u = 0; u <= s - t; ++u) {
                    const int v = s - t - u;
                    double val;
                    if (t > 0) {
                        val = X * nxt[herm_index(t - 1, u, v)];
                        if (t > 1) val += (t - 1) * nxt[herm_index(t - 2, u, v)];
                    } else if (u > 0) {
                        val = Y * nxt[herm_index(t, u - 1, v)];
                        if (u > 1) val += (u - 1) * nxt[herm_index(t, u - 2, v)];
                    } else {
                        val = Z * nxt[herm_index(t, u, v - 1)];
                        if (v > 1) val += (v - 1) * nxt[herm_index(t, u, v - 2)];
                    }
                    cur[herm_index(t, u, v)] = val;
                }
        double* tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
    if (nxt != R)
        for (int h = 0; h < kMaxHerm; ++h) R[h] = nxt[h];
}

__global__ void __launch_bounds__(kOneeThreads) k_one_electron(OneeArgs a)
{
    __shared__ double acc[3][100];   // S, T, V per component pair (<= 10 x 10)
    const int2 pr = a.pairs[blockIdx.x];
    const OneeShell A = a.sh[pr.x];
    const OneeShell B = a.sh[pr.y];
    const int na = ncomp(A.L), nb = ncomp(B.L), nab = na * nb;
    for (int e = threadIdx.x; e < 3 * 100; e += blockDim.x) (&acc[0][0])[e] = 0.0;
    __syncthreads();

    const int nch = max(1, (a.natom + kNucChunk - 1) / kNucChunk);
    const int npp = A.nprim * B.nprim;
    const int jm = B.L + 2;
    const int L = A.L + B.L;
    double Ex[(kMaxLa + 1) * (kMaxJm + 1) * kMaxNt], Ey[(kMaxLa + 1) * (kMaxJm + 1) * kMaxNt],
        Ez[(kMaxLa + 1) * (kMaxJm + 1) * kMaxNt];
    auto E = [](const double* T, int i, int j, int t) { return T[(i * (kMaxJm + 1) + j) * kMaxNt + t]; };
    for (int it = threadIdx.x; it < npp * nch; it += blockDim.x) {
        const int ij = it / nch, ch = it - ij * nch;
        const int i = ij / B.nprim, j = ij - i * B.nprim;
        const double al = a.exps[A.prim0 + i], be = a.exps[B.prim0 + j], p = al + be;
        hermite_1d_dev(A.L, jm, al, be, A.x, B.x, Ex);
        hermite_1d_dev(A.L, jm, al, be, A.y, B.y, Ey);
        hermite_1d_dev(A.L, jm, al, be, A.z, B.z, Ez);
        const double Px = (al * A.x + be * B.x) / p, Py = (al * A.y + be * B.y) / p, Pz = (al * A.z + be * B.z) / p;
        if (ch == 0) {
            const double sq = sqrt(3.14159265358979323846 / p);
            for (int ab = 0; ab < nab; ++ab) {
                const int ca = ab / nb, cb = ab - ca * nb;
                int ax, ay, az, bx, by, bz;
                comp(A.L, ca, ax, ay, az);
                comp(B.L, cb, bx, by, bz);
                const double w = a.w[A.woff + ca * A.nprim + i] * a.w[B.woff + cb * B.nprim + j];
                const double Sx = E(Ex, ax, bx, 0) * sq, Sy = E(Ey, ay, by, 0) * sq, Sz = E(Ez, az, bz, 0) * sq;
                auto kin = [&](const double* T, int ii, int jj) {
                    double t = be * (2 * jj + 1) * E(T, ii, jj, 0) - 2.0 * be * be * E(T, ii, jj + 2, 0);
                    if (jj >= 2) t -= 0.5 * jj * (jj - 1) * E(T, ii, jj - 2, 0);
                    return t * sq;
                };
                const double Tx = kin(Ex, ax, bx), Ty = kin(Ey, ay, by), Tz = kin(Ez, az, bz);
                atomicAdd(&acc[0][ab], w * Sx * Sy * Sz);
                atomicAdd(&acc[1][ab], w * (Tx * Sy * Sz + Sx * Ty * Sz + Sx * Sy * Tz));
            }
        }
        double vacc[100];
        for (int ab = 0; ab < nab; ++ab) vacc[ab] = 0.0;
        const int c1 = min(a.natom, (ch + 1) * kNucChunk);
        for (int c = ch * kNucChunk; c < c1; ++c) {
            const Nucleus C = a.nuc[c];
            const double X = Px - C.x, Y = Py - C.y, Z = Pz - C.z;
            double F[7], R[kMaxHerm];
            boys_rt(L, p * (X * X + Y * Y + Z * Z), a.boys, F);
            hermite_R_rt(L, p, X, Y, Z, F, R);
            const double pref = -C.Z * 2.0 * 3.14159265358979323846 / p;
            for (int ab = 0; ab < nab; ++ab) {
                const int ca = ab / nb, cb = ab - ca * nb;
                int ax, ay, az, bx, by, bz;
                comp(A.L, ca, ax, ay, az);
                comp(B.L, cb, bx, by, bz);
                double v = 0.0;
                for (int t = 0; t <= ax + bx; ++t) {
                    const double et = E(Ex, ax, bx, t);
                    for (int u = 0; u <= ay + by; ++u) {
                        const double eu = et * E(Ey, ay, by, u);
                        for (int s = 0; s <= az + bz; ++s) v += eu * E(Ez, az, bz, s) * R[herm_index(t, u, s)];
                    }
                }
                vacc[ab] += pref * v;
            }
        }
        for (int ab = 0; ab < nab; ++ab) {
            const int ca = ab / nb, cb = ab - ca * nb;
            const double w = a.w[A.woff + ca * A.nprim + i] * a.w[B.woff + cb * B.nprim + j];
            atomicAdd(&acc[2][ab], w * vacc[ab]);
        }
    }
    __syncthreads();
    for (int ab = threadIdx.x; ab < nab; ab += blockDim.x) {
        const int ca = ab / nb, cb = ab - ca * nb;
        const long long r = A.bf0 + ca, c = B.bf0 + cb;
        a.S[r * a.K + c] = acc[0][ab];
        a.S[c * a.K + r] = acc[0][ab];
        a.T[r * a.K + c] = acc[1][ab];
        a.T[c * a.K + r] = acc[1][ab];
        a.V[r * a.K + c] = acc[2][ab];
        a.V[c * a.K + r] = acc[2][ab];
    }
}

// Boys table of the device (same values as a job's), built once per device.
const double* boys_table(int device)
{
    static std::mutex mu;
    static std::map<int, double*> tabs;
    std::lock_guard<std::mutex> lk(mu);
    auto it = tabs.find(device);
    if (it != tabs.end()) return it->second;
    const std::vector<double>& tab = boys_table_host();
    double* d = nullptr;
    cuda_check(cudaMalloc(&d, tab.size() * sizeof(double)), "boys table");
    cuda_check(cudaMemcpy(d, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice), "boys table");
    tabs[device] = d;   // kept for the process lifetime
    return d;
}

}  // namespace

void one_electron_gpu(const Basis& b, std::vector<double>& S, std::vector<double>& T, std::vector<double>& V)
{
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    const double* boys = boys_table(dev);
    const int K = b.K;
    const int ns = (int)b.shells.size();
    if (ns == 0) {
        S.assign(0, 0.0);
        T.assign(0, 0.0);
        V.assign(0, 0.0);
        return;
    }
    std::vector<OneeShell> sh(ns);
    std::vector<double> exps, w;
    for (int s = 0; s < ns; ++s) {
        const Shell& x = b.shells[s];
        if (x.L > kMaxLa) throw Error(HFX_ERR_UNSUPPORTED, "one-electron kernel: L > 3");
        sh[s] = OneeShell{x.x, x.y, x.z, x.L, x.bf0, x.nprim(), (int)exps.size(), (int)w.size(), 0};
        exps.insert(exps.end(), x.exps.begin(), x.exps.end());
        w.insert(w.end(), x.w.begin(), x.w.end());
    }
    std::vector<int2> pairs;
    pairs.reserve((size_t)ns * (ns + 1) / 2);
    for (int A = 0; A < ns; ++A)
        for (int B = 0; B <= A; ++B) pairs.push_back(make_int2(A, B));
    const int natom = (int)b.atom_Z.size();
    std::vector<Nucleus> nuc(std::max(1, natom));
    for (int c = 0; c < natom; ++c)
        nuc[c] = Nucleus{b.atom_xyz[3 * c], b.atom_xyz[3 * c + 1], b.atom_xyz[3 * c + 2], (double)b.atom_Z[c]};

    cudaStream_t st;
    cuda_check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    try {
        DevBuf<OneeShell> d_sh;
        DevBuf<double> d_exps, d_w, d_out;
        DevBuf<int2> d_pairs;
        DevBuf<Nucleus> d_nuc;
        d_sh.upload(sh, st);
        d_exps.upload(exps, st);
        d_w.upload(w, st);
        d_pairs.upload(pairs, st);
        d_nuc.upload(nuc, st);
        const size_t n = (size_t)K * K;
        d_out.alloc(3 * n);
        OneeArgs a{d_sh.p, d_exps.p, d_w.p, d_pairs.p, d_nuc.p, natom, boys, K, d_out.p, d_out.p + n,
                   d_out.p + 2 * n};
        k_one_electron<<<(unsigned)pairs.size(), kOneeThreads, 0, st>>>(a);
        cuda_check(cudaGetLastError(), "one-electron kernel");
        S.resize(n);
        T.resize(n);
        V.resize(n);
        cuda_check(cudaMemcpyAsync(S.data(), d_out.p, n * sizeof(double), cudaMemcpyDeviceToHost, st), "download S");
        cuda_check(cudaMemcpyAsync(T.data(), d_out.p + n, n * sizeof(double), cudaMemcpyDeviceToHost, st), "T");
        cuda_check(cudaMemcpyAsync(V.data(), d_out.p + 2 * n, n * sizeof(double), cudaMemcpyDeviceToHost, st), "V");
        cuda_check(cudaStreamSynchronize(st), "one-electron");
    } catch (...) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
        throw;
    }
    cudaStreamDestroy(st);
}

}  // namespace hfx
