// hfx_kernels.cu -- shell-quartet McMurchie-Davidson ERI kernels with
// direct J/K digestion (sm_103a).
//
// Reference behaviour replaced: the reference evaluates one basis-function
// quartet per CUDA block (cuda/include/kernels.cuh:84-168), recomputing the
// Hermite E coefficients six times and the whole R recursion per (t,u,v) for
// every primitive quartet (recursion.cuh:145-240), stores the full unique-ERI
// tensor and contracts it with the density on the host every iteration
// (linalg.hpp:100-129).  Here one CTA evaluates a whole *shell* quartet:
//   stage 1  Boys F_m(T) (table + Taylor) and the R_{tuv} recursion, once per
//            primitive quartet, level-parallel across a warp;
//   stage 2  ket transform  W[tuv][cd] = sum_tnp (-1)^|tnp| R[tuv+tnp] E_cd[tnp]
//   stage 3  bra transform  acc[ab][cd] += sum_tuv E_ab[tuv] W[tuv][cd]
// and the finished Cartesian block is digested into J and K (8-fold
// permutational symmetry, BF-level Schwarz mask as integrals.hpp:771), so the
// ERI tensor is never stored.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <set>

#include "hfx_device.cuh"

namespace hfx {

__device__ __forceinline__ double boys_tab(int m, double T, const double* __restrict__ tab)
{
    if (T < (double)kBoysTMax) {
        int k = __double2int_rn(T * kBoysInvStep);
        double d = T - k * (1.0 / kBoysInvStep);
        const double* f = tab + k * kBoysM + m;
        double nd = -d;
        // Taylor series in -d with coefficients F_{m+j}(T_k) / j!, j = 0..6
        double r = __ldg(f + 6) * (1.0 / 720.0);
        r = fma(r, nd, __ldg(f + 5) * (1.0 / 120.0));
        r = fma(r, nd, __ldg(f + 4) * (1.0 / 24.0));
        r = fma(r, nd, __ldg(f + 3) * (1.0 / 6.0));
        r = fma(r, nd, __ldg(f + 2) * 0.5);
        r = fma(r, nd, __ldg(f + 1));
        r = fma(r, nd, __ldg(f + 0));
        return r;
    }
    // large T: F_0 = sqrt(pi/T)/2 (erf(sqrt T) = 1 to double precision),
    // stable upward recursion F_{j+1} = ((2j+1) F_j - e^{-T}) / (2T).
    double F = 0.5 * sqrt(3.141592653589793 / T);
    double e = exp(-T);
    double inv2T = 0.5 / T;
    for (int j = 0; j < m; ++j) F = ((2 * j + 1) * F - e) * inv2T;
    return F;
}

// Inverse of herm_index: packed Hermite index -> (t,u,v,s) packed in an int.
__device__ inline int herm_comp(int e)
{
    int s = 0;
    while (dnherm(s) <= e) ++s;
    int o = e - (s == 0 ? 0 : dnherm(s - 1));
    int t = 0;
    while (true) {
        int width = s - t + 1;  // number of u values for this t
        if (o < width) break;
        o -= width;
        ++t;
    }
    int u = o, v = s - t - u;
    return t | (u << 8) | (v << 16) | (s << 24);
}

// Stage 1 on one warp: R^{(0)}_{tuv} (scaled by the ERI prefactor) for all
// t+u+v <= L into the returned buffer (one of bufA / bufB).
__device__ double* hermite_R_warp(double p, double Px, double Py, double Pz, double q, double Qx, double Qy,
                                  double Qz, int L, double* bufA, double* bufB, double* seeds,
                                  const short* idx3, const int* comp, const double* __restrict__ boys)
{
    const int lane = threadIdx.x & 31;
    double X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;
    double pq = p + q;
    double rho = p * q / pq;
    double T = rho * (X * X + Y * Y + Z * Z);
    // 2 pi^{5/2} / (p q sqrt(p+q))  (integrals.hpp:698)
    double pref = 34.98683665524972 / (p * q * sqrt(pq));
    if (lane <= L) {
        double F = boys_tab(lane, T, boys);
        double m2r = -2.0 * rho, pw = 1.0;
        for (int j = 0; j < lane; ++j) pw *= m2r;
        seeds[lane] = pref * pw * F;
    }
    __syncwarp();
    double* prev = bufA;
    double* cur = bufB;
    if (lane == 0) prev[0] = seeds[L];
    __syncwarp();
    for (int n = L - 1; n >= 0; --n) {
        int top = L - n;
        int cnt = dnherm(top);
        for (int e = lane; e < cnt; e += 32) {
            double val;
            if (e == 0) {
                val = seeds[n];
            } else {
                int c = comp[e];
                int t = c & 255, u = (c >> 8) & 255, v = (c >> 16) & 255;
                if (t > 0) {
                    val = X * prev[idx3[((t - 1) * 13 + u) * 13 + v]];
                    if (t > 1) val += (t - 1) * prev[idx3[((t - 2) * 13 + u) * 13 + v]];
                } else if (u > 0) {
                    val = Y * prev[idx3[(t * 13 + u - 1) * 13 + v]];
                    if (u > 1) val += (u - 1) * prev[idx3[(t * 13 + u - 2) * 13 + v]];
                } else {
                    val = Z * prev[idx3[(t * 13 + u) * 13 + v - 1]];
                    if (v > 1) val += (v - 1) * prev[idx3[(t * 13 + u) * 13 + v - 2]];
                }
            }
            cur[e] = val;
        }
        __syncwarp();
        double* tmp = prev;
        prev = cur;
        cur = tmp;
    }
    return prev;
}

__device__ __forceinline__ long long pair_idx(int a, int b)
{
    int hi = a > b ? a : b, lo = a > b ? b : a;
    return (long long)hi * (hi + 1) / 2 + lo;
}

// Unique-ERI kernel (the ERI_GPU replacement): one CTA (128 threads) per
// shell quartet, quartets taken from a global work queue, dense E matrices,
// every canonical BF-level integral written to its packed eri_index slot
// (zero stays where the BF-level Schwarz test fails).  The Fock builds and the
// Schwarz pass run on the class kernels instead.
__global__ void __launch_bounds__(128) k_quartet_eri(LaunchArgs a, int maxacc, int maxw, int maxr)
{
    extern __shared__ __align__(16) unsigned char smem[];
    short* idx3 = reinterpret_cast<short*>(smem);            // 13^3 shorts
    int* comp = reinterpret_cast<int*>(smem + 4400);         // 455 ints
    double* dbuf = reinterpret_cast<double*>(smem + 6240);
    double* acc = dbuf;
    double* W = acc + maxacc;
    double* Ra = W + maxw;
    double* Rb = Ra + maxr;
    double* seeds = Rb + maxr;                               // 16
    __shared__ int s_task;

    for (int e = threadIdx.x; e < 13 * 13 * 13; e += blockDim.x) {
        int t = e / 169, u = (e / 13) % 13, v = e % 13;
        idx3[e] = (t + u + v <= 12) ? (short)herm_index(t, u, v) : (short)-1;
    }
    for (int e = threadIdx.x; e < 455; e += blockDim.x) comp[e] = herm_comp(e);
    __syncthreads();

    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const double* __restrict__ epool = a.epool;

    while (true) {
        if (tid == 0) s_task = atomicAdd(a.counter, 1);
        __syncthreads();
        const int tk = s_task;
        __syncthreads();
        if (tk >= a.ntasks) break;
        const Task task = a.tasks[tk];
        const DPair bra = a.pairs[task.bra];
        const DPair ket = a.pairs[task.ket];
        const int L1 = bra.l0 + bra.l1, L2 = ket.l0 + ket.l1, L = L1 + L2;
        const int n1 = dncart(bra.l1), n3 = dncart(ket.l1);
        const int nab = dncart(bra.l0) * n1, ncd = dncart(ket.l0) * n3;
        const int H1 = dnherm(L1), H2 = dnherm(L2);
        const int nout = nab * ncd;
        for (int e = tid; e < nout; e += blockDim.x) acc[e] = 0.0;

        for (int ij = 0; ij < bra.npp; ++ij) {
            const PairGeo g1 = a.pp_geo[bra.pp0 + ij];
            const double* Eij = epool + bra.e_off + (long long)ij * nab * H1;
            for (int kl = 0; kl < ket.npp; ++kl) {
                const PairGeo g2 = a.pp_geo[ket.pp0 + kl];
                const double* Ekl = epool + ket.e_off + (long long)kl * ncd * H2;
                if (warp == 0)
                    hermite_R_warp(g1.p, g1.x, g1.y, g1.z, g2.p, g2.x, g2.y, g2.z, L, Ra, Rb, seeds, idx3, comp,
                                   a.boys);
                __syncthreads();
                const double* R = (L % 2 == 0) ? Ra : Rb;
                // stage 2: ket transform
                for (int e = tid; e < H1 * ncd; e += blockDim.x) {
                    int tuv = e / ncd, cd = e - tuv * ncd;
                    int c1 = comp[tuv];
                    int t = c1 & 255, u = (c1 >> 8) & 255, v = (c1 >> 16) & 255;
                    const double* Ec = Ekl + cd * H2;
                    double s = 0.0;
                    for (int tn = 0; tn < H2; ++tn) {
                        int c2 = comp[tn];
                        int tt = t + (c2 & 255), uu = u + ((c2 >> 8) & 255), vv = v + ((c2 >> 16) & 255);
                        double r = R[idx3[(tt * 13 + uu) * 13 + vv]];
                        double ev = __ldg(Ec + tn);
                        s = ((c2 >> 24) & 1) ? fma(-r, ev, s) : fma(r, ev, s);
                    }
                    W[e] = s;
                }
                __syncthreads();
                // stage 3: bra transform into the Cartesian block
                for (int e = tid; e < nout; e += blockDim.x) {
                    int ab = e / ncd, cd = e - ab * ncd;
                    const double* Ea = Eij + ab * H1;
                    double s = 0.0;
                    for (int tuv = 0; tuv < H1; ++tuv) s = fma(__ldg(Ea + tuv), W[tuv * ncd + cd], s);
                    acc[e] += s;
                }
                __syncthreads();
            }
        }

        // digestion
        for (int e = tid; e < nout; e += blockDim.x) {
            int ab = e / ncd, cd = e - ab * ncd;
            int ia = ab / n1, ib = ab - ia * n1, ic = cd / n3, id = cd - ic * n3;
            int i = bra.bf0 + ia, j = bra.bf1 + ib, k = ket.bf0 + ic, l = ket.bf1 + id;
            if (bra.same && ia < ib) continue;
            if (ket.same && ic < id) continue;
            long long pij = pair_idx(i, j), pkl = pair_idx(k, l);
            if (task.bra == task.ket && pij < pkl) continue;
            if (a.thr >= 0.0 && a.Qbf[pij] * a.Qbf[pkl] < a.thr) continue;
            long long hi = pij > pkl ? pij : pkl, lo = pij > pkl ? pkl : pij;
            a.eri[hi * (hi + 1) / 2 + lo] = acc[e];
        }
        __syncthreads();
    }
}

// G = (Jacc + Jacc^T)/4 - 1/2 (Kacc + Kacc^T)/8   (RHF, linalg.hpp:100-129),
// per molecule block of the packed buffers (blockIdx.y = molecule); blocks of
// molecules switched off for this build (active[f] == 0) are left untouched
__global__ void k_finish_rhf(const double* Jacc, const double* Kacc, double* G, const int* fk, const long long* fmoff,
                             const unsigned char* active)
{
    if (active && !active[blockIdx.y]) return;
    const int K = fk[blockIdx.y];
    const long long o = fmoff[blockIdx.y];
    const int n = K * K;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        int i = e / K, j = e - i * K;
        double J = 0.25 * (Jacc[o + e] + Jacc[o + j * K + i]);
        double X = 0.125 * (Kacc[o + e] + Kacc[o + j * K + i]);
        G[o + e] = J - 0.5 * X;
    }
}

// J = (Jacc + Jacc^T)/4, K = (Kacc + Kacc^T)/8  (UHF, linalg.hpp:215-296)
__global__ void k_finish_uhf(const double* Jacc, const double* Ka, const double* Kb, double* J, double* Kao,
                             double* Kbo, const int* fk, const long long* fmoff, const unsigned char* active)
{
    if (active && !active[blockIdx.y]) return;
    const int K = fk[blockIdx.y];
    const long long o = fmoff[blockIdx.y];
    const int n = K * K;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        int i = e / K, j = e - i * K;
        J[o + e] = 0.25 * (Jacc[o + e] + Jacc[o + j * K + i]);
        Kao[o + e] = 0.125 * (Ka[o + e] + Ka[o + j * K + i]);
        Kbo[o + e] = 0.125 * (Kb[o + e] + Kb[o + j * K + i]);
    }
}

// float copy of a packed density (the FP32 kernels' digestion products)
__global__ void k_to_float(const double* A, float* B, long long n)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        B[e] = (float)A[e];
}

__global__ void k_add(const double* A, const double* B, double* C, long long n)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        C[e] = A[e] + B[e];
}

// Dsh[p] = max over the (A, B) block of max(|D1|, |D2|), for every shell pair
// p (D2 may be null); the density-weighted screening of incremental builds.
__global__ void k_density_blocks(const DPair* pairs, int npairs, const double* D1, const double* D2, double* Dsh)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs) return;
    const DPair pr = pairs[p];
    const int n0 = dncart(pr.l0), n1 = dncart(pr.l1);
    double m = 0.0;
    for (int a = 0; a < n0; ++a)
        for (int b = 0; b < n1; ++b) {
            long long e = pr.moff + (long long)(pr.bf0 + a) * pr.kdim + pr.bf1 + b;
            m = fmax(m, fabs(D1[e]));
            if (D2) m = fmax(m, fabs(D2[e]));
        }
    Dsh[p] = m;
}

KernelSpec density_blocks_spec(int npairs)
{
    KernelSpec s;
    s.func = (const void*)k_density_blocks;
    s.grid = dim3((unsigned)((npairs + 127) / 128));
    s.block = dim3(128);
    return s;
}

// Host-side launch helpers (called from hfx_engine.cpp).
size_t generic_smem_bytes(int maxacc, int maxw, int maxr)
{
    return 6240 + sizeof(double) * (size_t)(maxacc + maxw + 2 * maxr + 16);
}

// Raise a kernel's dynamic shared-memory limit to the device maximum once
// per process: launches from concurrent jobs then never race on the attribute.
template <typename K>
static cudaError_t allow_max_smem_generic(K kern)
{
    static std::mutex mu;
    static std::set<const void*> done;
    std::lock_guard<std::mutex> lk(mu);
    if (done.count((const void*)kern)) return cudaSuccess;
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa{};
    cudaError_t err = cudaFuncGetAttributes(&fa, kern);
    if (err != cudaSuccess) return err;
    err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
    if (err == cudaSuccess) done.insert((const void*)kern);
    return err;
}

cudaError_t launch_eri(const LaunchArgs& a, int maxacc, int maxw, int maxr, int grid, cudaStream_t st)
{
    size_t sm = generic_smem_bytes(maxacc, maxw, maxr);
    cudaError_t e = allow_max_smem_generic(k_quartet_eri);
    if (e != cudaSuccess) return e;
    k_quartet_eri<<<grid, 128, sm, st>>>(a, maxacc, maxw, maxr);
    return cudaGetLastError();
}

// Grid-stride elementwise kernels: 256 threads, at most 1024 CTAs per grid row.
static KernelSpec elementwise_spec(const void* func, long long n, int rows)
{
    KernelSpec s;
    s.func = func;
    long long grid = (n + 255) / 256;
    s.grid = dim3((unsigned)std::max(1LL, std::min(grid, 1024LL)), (unsigned)std::max(1, rows));
    s.block = dim3(256);
    return s;
}

KernelSpec finish_rhf_spec(int Kmax, int nfrag)
{
    return elementwise_spec((const void*)k_finish_rhf, (long long)Kmax * Kmax, nfrag);
}
KernelSpec finish_uhf_spec(int Kmax, int nfrag)
{
    return elementwise_spec((const void*)k_finish_uhf, (long long)Kmax * Kmax, nfrag);
}
// Shift the pair indices of a task list copied into a combined list (the
// multi-job Fock session, hfx_session.cpp).
__global__ void k_rebase_tasks(Task* t, long long n, int delta)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        t[i].bra += delta;
        t[i].ket += delta;
    }
}

KernelSpec rebase_tasks_spec(long long n) { return elementwise_spec((const void*)k_rebase_tasks, n, 1); }
KernelSpec add_spec(long long n) { return elementwise_spec((const void*)k_add, n, 1); }
KernelSpec to_float_spec(long long n) { return elementwise_spec((const void*)k_to_float, n, 1); }

}  // namespace hfx
