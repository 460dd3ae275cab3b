// hfx_warp.cu -- warp-per-shell-quartet McMurchie-Davidson kernel with direct
// J/K digestion, for any angular-momentum class (runtime L), FP64 or FP32.
//
// Each warp takes shell quartets from a global work queue and works on its own
// slice of shared memory; there are no CTA-wide barriers.  Per bra primitive
// pair ij the warp accumulates the ket-transformed Hermite integrals
//   W[tuv][cd] = sum_kl sum_{tnp in nz(cd)} (-1)^{|tnp|} c^{kl}_{cd,tnp} R^{ij,kl}[tuv+tnp]
// over all ket primitive pairs, then applies the bra transform once:
//   acc[ab][cd] += sum_{tuv in nz(ab)} c^{ij}_{ab,tuv} W[tuv][cd]
// so the bra work is amortised over the ket contraction (the reference
// re-does the full Hermite sum per primitive quartet and per basis-function
// quartet, integrals.hpp:675-698).  Only structurally non-zero
// Hermite->Cartesian coefficients are stored and used.
//
// R_{tuv} (stage 1) is computed either one primitive quartet per lane
// (lane-parallel, for batches of ket primitives) or level-parallel across the
// warp for single primitive quartets; both use the in-place downward
// recursion over m of integrals.hpp:541-618, driven by a neighbour table.
#include <cuda_runtime.h>

#include <mutex>
#include <set>

#include "hfx_device.cuh"

namespace hfx {


__host__ __device__ constexpr int w_nh(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }
__host__ __device__ constexpr int w_nc(int l) { return (l + 1) * (l + 2) / 2; }

template <typename T>
__device__ __forceinline__ T w_fma(T a, T b, T c)
{
    return fma(a, b, c);
}

// F_L(T) by Taylor from the table, e^{-T}; or asymptotic values beyond it.
template <typename T>
__device__ __forceinline__ void boys_top(T Tv, int L, const T* __restrict__ tab, T& FL, T& e, bool& table)
{
    if constexpr (sizeof(T) == 4) {
        // FP32 table: one 8-float row per (L, k), Taylor terms pre-scaled
        if (Tv < (T)kBoysTMax) {
            table = true;
            int k;
            const T nd = boys_grid_offset(Tv, k);
            const float4* row = reinterpret_cast<const float4*>(tab + ((size_t)L * kBoysN + k) * kBoys32Row);
            const float4 c0 = __ldg(row), c1 = __ldg(row + 1);
            T r = c1.x;
            r = w_fma(r, nd, c0.w);
            r = w_fma(r, nd, c0.z);
            r = w_fma(r, nd, c0.y);
            FL = w_fma(r, nd, c0.x);
            T x = (T)(1.0 / 24.0);
            x = w_fma(x, nd, (T)(1.0 / 6.0));
            x = w_fma(x, nd, (T)0.5);
            x = w_fma(x, nd, (T)1);
            x = w_fma(x, nd, (T)1);
            e = c1.y * x;
        } else {
            table = false;
            FL = (T)0;
            e = (T)0;
        }
    } else if (Tv < (T)kBoysTMax) {
        // FP64 table: one 8-double row per (L, k), Taylor terms pre-scaled
        table = true;
        int k = (int)(Tv * (T)kBoysInvStep + (T)0.5);
        T nd = (T)k * ((T)1 / (T)kBoysInvStep) - Tv;
        const double2* row = reinterpret_cast<const double2*>(tab + ((size_t)L * kBoysN + k) * kBoys64Row);
        const double2 c0 = __ldg(row), c1 = __ldg(row + 1), c2 = __ldg(row + 2), c3 = __ldg(row + 3);
        T r = c3.x;
        r = w_fma(r, nd, c2.y);
        r = w_fma(r, nd, c2.x);
        r = w_fma(r, nd, c1.y);
        r = w_fma(r, nd, c1.x);
        r = w_fma(r, nd, c0.y);
        FL = w_fma(r, nd, c0.x);
        // exp(-T) = exp(-T_k) exp(nd), |nd| <= 1/32
        T x = (T)(1.0 / 5040.0);
        x = w_fma(x, nd, (T)(1.0 / 720.0));
        x = w_fma(x, nd, (T)(1.0 / 120.0));
        x = w_fma(x, nd, (T)(1.0 / 24.0));
        x = w_fma(x, nd, (T)(1.0 / 6.0));
        x = w_fma(x, nd, (T)0.5);
        x = w_fma(x, nd, (T)1);
        x = w_fma(x, nd, (T)1);
        e = c3.y * x;
    } else {
        table = false;
        FL = (T)0;
        e = L >= 5 ? (T)exp(-(double)Tv) : (T)0;
    }
}

// 1/(2m+1), m = 0..15, for the downward Boys recursion
__constant__ double c_inv_odd64[16] = {1.0,       1.0 / 3,  1.0 / 5,  1.0 / 7,  1.0 / 9,  1.0 / 11,
                                       1.0 / 13,  1.0 / 15, 1.0 / 17, 1.0 / 19, 1.0 / 21, 1.0 / 23,
                                       1.0 / 25,  1.0 / 27, 1.0 / 29, 1.0 / 31};
__constant__ float c_inv_odd32[16] = {1.0f,       1.0f / 3,  1.0f / 5,  1.0f / 7,  1.0f / 9,  1.0f / 11,
                                      1.0f / 13,  1.0f / 15, 1.0f / 17, 1.0f / 19, 1.0f / 21, 1.0f / 23,
                                      1.0f / 25,  1.0f / 27, 1.0f / 29, 1.0f / 31};
template <typename T>
__device__ __forceinline__ T inv_odd(int m);
template <>
__device__ __forceinline__ double inv_odd<double>(int m)
{
    return c_inv_odd64[m];
}
template <>
__device__ __forceinline__ float inv_odd<float>(int m)
{
    return c_inv_odd32[m];
}

// Seeds s_m = pref (-2 rho)^m F_m(T), m = 0..L, written to S[m * sstride];
// inv_rho = 1/rho avoids a division.
template <typename T>
__device__ __forceinline__ void boys_seeds(T Tv, T rho, T inv_rho, T pref, int L, const T* __restrict__ tab, T* S,
                                           int sstride)
{
    T FL, e;
    bool table;
    boys_top<T>(Tv, L, tab, FL, e, table);
    T m2r = (T)-2 * rho;
    if (table) {
        // downward F_m = (2T F_{m+1} + e) / (2m+1); the power of (-2 rho) built upward
        T F = FL;
        T pw = pref;
        for (int m = 0; m < L; ++m) pw *= m2r;
        S[L * sstride] = pw * F;
        T t2 = Tv + Tv;
        T rm2r = (T)-0.5 * inv_rho;
        for (int m = L - 1; m >= 0; --m) {
            F = w_fma(t2, F, e) * inv_odd<T>(m);
            pw *= rm2r;
            S[m * sstride] = pw * F;
        }
    } else {
        T rs = rsqrt(Tv);
        T F = (T)0.88622692545275801365 * rs;
        T inv2T = (T)0.5 * rs * rs;
        T pw = pref;
        S[0] = pw * F;
        T odd = (T)1;
        for (int m = 0; m < L; ++m) {
            F = (odd * F - e) * inv2T;
            odd += (T)2;
            pw *= m2r;
            S[(m + 1) * sstride] = pw * F;
        }
    }
}

// In-place recursion for the table R[e * rs] (e in packed Hermite order).
// nb[e] = dir | i1 << 2 | i2 << 11 | c2 << 20  (dir 0/1/2 = x/y/z).
template <typename T>
__device__ __forceinline__ void recur_lane(T X, T Y, T Z, int L, const T* S, int sstride, T* R, int rs,
                                           const int* nb, const T* cf)
{
    R[0] = S[L * sstride];
    for (int n = L - 1; n >= 0; --n) {
        int top = w_nh(L - n);
        for (int e = top - 1; e >= 1; --e) {
            int w = nb[e];
            int dir = w & 3, i1 = (w >> 2) & 511, i2 = (w >> 11) & 511, c2 = (w >> 20) & 15;
            T xd = dir == 0 ? X : (dir == 1 ? Y : Z);
            T val = xd * R[i1 * rs];
            if (c2) val = w_fma(cf[e], R[i2 * rs], val);
            R[e * rs] = val;
        }
        R[0] = S[n * sstride];
    }
}

__device__ __forceinline__ long long wpidx(int a, int b)
{
    int hi = a > b ? a : b, lo = a > b ? b : a;
    return (long long)hi * (hi + 1) / 2 + lo;
}

// ket primitive pairs per round of the level-parallel (non-lane) mode (8 measured
// slower on benzene/cc-pVDZ, 35.3 against 34.6 ms per FP64 build)
constexpr int kWarpKetRound = 4;

template <typename T, int NK>
__global__ void __launch_bounds__(256) k_warp_quartet(WarpArgs<T> a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    short* idx3 = reinterpret_cast<short*>(smem);                 // 2197 shorts (4394 B)
    int* nbt = reinterpret_cast<int*>(smem + 4400);               // 455 ints (1820 B) -> 6220
    int* clin = reinterpret_cast<int*>(smem + 6240);              // 455 ints -> 8060
    T* cft = reinterpret_cast<T*>(smem + 8064);                   // 455 T (recursion coefficients) -> 11704
    T* wbase = reinterpret_cast<T*>(smem + kWarpSmemHeader);
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    T* sl = wbase + (size_t)warp * a.slice;

    for (int e = threadIdx.x; e < 2197; e += blockDim.x) {
        int t = e / 169, u = (e / 13) % 13, v = e % 13;
        int s = t + u + v;
        idx3[e] = (short)(s <= 12 ? s * (s + 1) * (s + 2) / 6 + t * (s + 1) - t * (t - 1) / 2 + u : -1);
    }
    for (int e = threadIdx.x; e < 455; e += blockDim.x) {
        int s = 0;
        while (w_nh(s) <= e) ++s;
        int o = e - (s == 0 ? 0 : w_nh(s - 1));
        int t = 0;
        while (o >= s - t + 1) {
            o -= s - t + 1;
            ++t;
        }
        int u = o, v = s - t - u;
        clin[e] = t * 169 + u * 13 + v;
        int w = 0;
        if (s > 0) {
            auto h = [](int tt, int uu, int vv) {
                int ss = tt + uu + vv;
                return ss * (ss + 1) * (ss + 2) / 6 + tt * (ss + 1) - tt * (tt - 1) / 2 + uu;
            };
            int dir, i1, i2 = 0, c2 = 0;
            if (t > 0) {
                dir = 0;
                i1 = h(t - 1, u, v);
                if (t > 1) { i2 = h(t - 2, u, v); c2 = t - 1; }
            } else if (u > 0) {
                dir = 1;
                i1 = h(t, u - 1, v);
                if (u > 1) { i2 = h(t, u - 2, v); c2 = u - 1; }
            } else {
                dir = 2;
                i1 = h(t, u, v - 1);
                if (v > 1) { i2 = h(t, u, v - 2); c2 = v - 1; }
            }
            w = dir | (i1 << 2) | (i2 << 11) | (c2 << 20);
        }
        nbt[e] = w;
        cft[e] = (T)((w >> 20) & 15);
    }
    __syncthreads();

    const T* __restrict__ rec = a.rec;
    while (true) {
        int tk = 0;
        if (lane == 0) tk = atomicAdd(a.counter, 1);
        tk = __shfl_sync(0xffffffffu, tk, 0);
        if (tk >= a.ntasks) break;
        const Task task = a.tasks[tk];
        const DPair bra = a.pairs[task.bra];
        const DPair ket = a.pairs[task.ket];
        if (molecule_inactive(bra, a.active)) continue;
        if (density_negligible(bra, ket, a.Dsh, a.dthr)) continue;
        const PairClassTab cb = a.pct[bra.pc];
        const PairClassTab ck = a.pct[ket.pc];
        const int L1 = bra.l0 + bra.l1, L2 = ket.l0 + ket.l1, L = L1 + L2;
        const int n1 = w_nc(bra.l1), n3 = w_nc(ket.l1);
        const int nab = cb.nab, ncd = ck.nab;
        const int H1 = w_nh(L1), HL = w_nh(L);
        const int nout = nab * ncd, nw = H1 * ncd;
        const int* abs_b = a.ab_start + cb.ab_off;
        const int* abs_k = a.ab_start + ck.ab_off;
        const short* kh_b = a.k_herm + cb.k_off;
        const short* kl_k = a.k_lin + ck.k_off;
        // slice layout: acc[nout] W[nw] then the R area
        T* acc = sl;
        T* W = acc + nout;
        T* Ra = W + nw;
        const int kl_begin = task.k0, kl_end = task.k1, nkl = kl_end - kl_begin;
        const bool lane_mode = a.lane_min_npp > 0 && L <= 6 && nkl >= a.lane_min_npp;
        T* Sd = Ra + (lane_mode ? HL * 32 : (2 + kWarpKetRound) * HL);   // seeds: (L+1) x 32 (lane mode) or L+1
        for (int e = lane; e < nout; e += 32) acc[e] = (T)0;

        const int ij_end = task.i1;
        for (int ij = task.i0; ij < ij_end; ++ij) {
            const T* rb = rec + bra.rec_off + (long long)ij * cb.stride;
            const T p = __ldg(rb), Px = __ldg(rb + 1), Py = __ldg(rb + 2), Pz = __ldg(rb + 3), rp = __ldg(rb + 4);
            for (int e = lane; e < nw; e += 32) W[e] = (T)0;
            __syncwarp();
            if (lane_mode) {
                for (int kl0 = kl_begin; kl0 < kl_end; kl0 += 32) {
                    const int nb = min(32, kl_end - kl0);
                    if (lane < nb) {
                        const T* rk = rec + ket.rec_off + (long long)(kl0 + lane) * ck.stride;
                        const T q = __ldg(rk), Qx = __ldg(rk + 1), Qy = __ldg(rk + 2), Qz = __ldg(rk + 3),
                                rq = __ldg(rk + 4);
                        const T X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;
                        const T rs = rsqrt(p + q);
                        const T rho = p * q * (rs * rs);
                        const T Tv = rho * (X * X + Y * Y + Z * Z);
                        const T pref = (T)34.98683665524972 * rp * rq * rs;
                        boys_seeds<T>(Tv, rho, (p + q) * rp * rq, pref, L, a.boys, Sd + lane, 32);
                        recur_lane<T>(X, Y, Z, L, Sd + lane, 32, Ra + lane, 32, nbt, cft);
                    }
                    __syncwarp();
                    // stage 2: W[tuv][cd] += sum_k (+-) sum_b c_bk R_b[tuv + tnp_k]; the
                    // coefficient's Hermite offset and sign are read once per k and
                    // reused for the nb ket primitive pairs of this round
                    for (int e = lane; e < nw; e += 32) {
                        const int tuv = e / ncd, cd = e - tuv * ncd;
                        const int lt = clin[tuv];
                        const int k0 = __ldg(abs_k + cd), k1 = __ldg(abs_k + cd + 1);
                        const T* ck0 = rec + ket.rec_off + (long long)kl0 * ck.stride + 5;
                        T s = (T)0;
                        for (int k = k0; k < k1; ++k) {
                            const int w = __ldg(kl_k + k);
                            const T* Rk = Ra + idx3[lt + (w & 16383)] * 32;
                            const T* ckk = ck0 + k;
                            T t = (T)0;
                            for (int b = 0; b < nb; ++b) t = w_fma(__ldg(ckk + (long long)b * ck.stride), Rk[b], t);
                            s = (w & 16384) ? s - t : s + t;
                        }
                        W[e] += s;
                    }
                    __syncwarp();
                }
            } else {
                // kNB ket primitive pairs per round: each one's R by the
                // level-parallel recursion (ping-pong in Ra, last level into its
                // slot of Rb), then one ket transform over the round that reads
                // each coefficient's Hermite offset and sign once
                T* Rb = Ra + 2 * HL;
                for (int kl0 = kl_begin; kl0 < kl_end; kl0 += kWarpKetRound) {
                    const int nb = min(kWarpKetRound, kl_end - kl0);
                    for (int b = 0; b < nb; ++b) {
                        const T* rk = rec + ket.rec_off + (long long)(kl0 + b) * ck.stride;
                        const T q = __ldg(rk), Qx = __ldg(rk + 1), Qy = __ldg(rk + 2), Qz = __ldg(rk + 3),
                                rq = __ldg(rk + 4);
                        const T X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;
                        const T rs = rsqrt(p + q);
                        const T rho = p * q * (rs * rs);
                        const T Tv = rho * (X * X + Y * Y + Z * Z);
                        const T pref = (T)34.98683665524972 * rp * rq * rs;
                        // seeds: lane 0 (downward recursion is sequential in m)
                        if (lane == 0) boys_seeds<T>(Tv, rho, (p + q) * rp * rq, pref, L, a.boys, Sd, 1);
                        __syncwarp();
                        T* slot = Rb + b * HL;
                        T* prev = Ra;
                        T* cur = Ra + HL;
                        if (lane == 0) {
                            if (L == 0)
                                slot[0] = Sd[0];
                            else
                                prev[0] = Sd[L];
                        }
                        __syncwarp();
                        for (int n = L - 1; n >= 0; --n) {
                            const int cnt = w_nh(L - n);
                            T* dst = n == 0 ? slot : cur;
                            for (int e = lane; e < cnt; e += 32) {
                                T val;
                                if (e == 0) {
                                    val = Sd[n];
                                } else {
                                    const int w = nbt[e];
                                    const int dir = w & 3, i1 = (w >> 2) & 511, i2 = (w >> 11) & 511,
                                              c2 = (w >> 20) & 15;
                                    const T xd = dir == 0 ? X : (dir == 1 ? Y : Z);
                                    val = xd * prev[i1];
                                    if (c2) val = w_fma(cft[e], prev[i2], val);
                                }
                                dst[e] = val;
                            }
                            __syncwarp();
                            T* tmp = prev;
                            prev = cur;
                            cur = tmp;
                        }
                    }
                    const T* ck0 = rec + ket.rec_off + (long long)kl0 * ck.stride + 5;
                    for (int e = lane; e < nw; e += 32) {
                        const int tuv = e / ncd, cd = e - tuv * ncd;
                        const int lt = clin[tuv];
                        const int k0 = __ldg(abs_k + cd), k1 = __ldg(abs_k + cd + 1);
                        T s = (T)0;
                        for (int k = k0; k < k1; ++k) {
                            const int w = __ldg(kl_k + k);
                            const int ri = idx3[lt + (w & 16383)];
                            const T* ckk = ck0 + k;
                            T t = (T)0;
                            for (int b = 0; b < nb; ++b)
                                t = w_fma(__ldg(ckk + (long long)b * ck.stride), Rb[b * HL + ri], t);
                            s = (w & 16384) ? s - t : s + t;
                        }
                        W[e] += s;
                    }
                    __syncwarp();
                }
            }
            // stage 3: bra transform, once per bra primitive pair
            const T* cbp = rb + 5;
            for (int e = lane; e < nout; e += 32) {
                const int ab = e / ncd, cd = e - ab * ncd;
                const int k0 = __ldg(abs_b + ab), k1 = __ldg(abs_b + ab + 1);
                T s = (T)0;
                for (int k = k0; k < k1; ++k) s = w_fma(__ldg(cbp + k), W[__ldg(kh_b + k) * ncd + cd], s);
                acc[e] += s;
            }
            __syncwarp();
        }

        // Schwarz pass: diagonal (ab|ab) of the diagonal shell quartet (AB|AB)
        if constexpr (NK == 0) {
            for (int e = lane; e < nout; e += 32) {
                const int ab = e / ncd, cd = e - ab * ncd;
                if (ab != cd) continue;
                const int ia = ab / n1, ib = ab - ia * n1;
                if (bra.same && ia < ib) continue;
                const double v = (double)acc[e];
                const double qv = sqrt(v > 0.0 ? v : 0.0);
                a.Qout_bf[bra.qoff + wpidx(bra.bf0 + ia, bra.bf1 + ib)] = qv;
                atomicMax(a.Qout_sh + task.bra, (unsigned long long)__double_as_longlong(qv));
            }
            __syncwarp();
            continue;
        }

        // digestion (FP64), into the bra pair's molecule's matrices
        const int K = bra.kdim;
        const double* __restrict__ Qbf = a.Qbf + bra.qoff;
        const double* __restrict__ Dj = a.Dj + bra.moff;
        const double* __restrict__ Dk = a.Dk + bra.moff;
        const double* __restrict__ Dk2 = a.Dk2 + (NK == 2 ? bra.moff : 0);
        double* J = a.J + bra.moff;
        double* Kx = a.Kx + bra.moff;
        double* Kx2 = a.Kx2 + (NK == 2 ? bra.moff : 0);
        if constexpr (sizeof(T) == 8 && !kBlockDigestFP64) {
            for (int e = lane; e < nout; e += 32) {
                const int ab = e / ncd, cd = e - ab * ncd;
                const int ia = ab / n1, ib = ab - ia * n1, ic = cd / n3, id = cd - ic * n3;
                const int i = bra.bf0 + ia, j = bra.bf1 + ib, k = ket.bf0 + ic, l = ket.bf1 + id;
                if (bra.same && ia < ib) continue;
                if (ket.same && ic < id) continue;
                const long long pij = wpidx(i, j), pkl = wpidx(k, l);
                if (task.bra == task.ket && pij < pkl) continue;
                if (a.thr >= 0.0 && __ldg(Qbf + pij) * __ldg(Qbf + pkl) < a.thr) continue;
                double v = (double)acc[e] * ((i == j ? 1.0 : 2.0) * (k == l ? 1.0 : 2.0) * (pij == pkl ? 1.0 : 2.0));
                atomicAdd(J + (long long)i * K + j, __ldg(Dj + (long long)k * K + l) * v);
                atomicAdd(J + (long long)k * K + l, __ldg(Dj + (long long)i * K + j) * v);
                atomicAdd(Kx + (long long)i * K + k, __ldg(Dk + (long long)j * K + l) * v);
                atomicAdd(Kx + (long long)j * K + l, __ldg(Dk + (long long)i * K + k) * v);
                atomicAdd(Kx + (long long)i * K + l, __ldg(Dk + (long long)j * K + k) * v);
                atomicAdd(Kx + (long long)j * K + k, __ldg(Dk + (long long)i * K + l) * v);
                if (NK == 2) {
                    atomicAdd(Kx2 + (long long)i * K + k, __ldg(Dk2 + (long long)j * K + l) * v);
                    atomicAdd(Kx2 + (long long)j * K + l, __ldg(Dk2 + (long long)i * K + k) * v);
                    atomicAdd(Kx2 + (long long)i * K + l, __ldg(Dk2 + (long long)j * K + k) * v);
                    atomicAdd(Kx2 + (long long)j * K + k, __ldg(Dk2 + (long long)i * K + l) * v);
                }
            }
        } else {
            // Block digestion: weights in place (0 for non-canonical and
            // BF-screened elements), then one lane per J / K element the
            // quartet touches sums its contributions (FP32 quartets: float
            // products with the float density copies) and adds the sum to the
            // FP64 accumulator: nab + ncd + na nc + na nd + nb nc + nb nd
            // atomics per quartet instead of 6 per integral.
            const T* __restrict__ QbT = schwarz_of<T>(a) + bra.qoff;
            const bool screen = a.thr >= 0.0;
            const T thrT = (T)a.thr;
            for (int e = lane; e < nout; e += 32) {
                const int ab = e / ncd, cd = e - ab * ncd;
                const int ia = ab / n1, ib = ab - ia * n1, ic = cd / n3, id = cd - ic * n3;
                const int i = bra.bf0 + ia, j = bra.bf1 + ib, k = ket.bf0 + ic, l = ket.bf1 + id;
                const long long pij = wpidx(i, j), pkl = wpidx(k, l);
                const bool skip = (bra.same && ia < ib) || (ket.same && ic < id) ||
                                  (task.bra == task.ket && pij < pkl) ||
                                  (screen && __ldg(QbT + pij) * __ldg(QbT + pkl) < thrT);
                const T f = (i == j ? (T)1 : (T)2) * (k == l ? (T)1 : (T)2) * (pij == pkl ? (T)1 : (T)2);
                acc[e] = skip ? (T)0 : acc[e] * f;
            }
            __syncwarp();
            const int n0 = w_nc(bra.l0), n2 = w_nc(ket.l0);
            const int i0 = bra.bf0, j0 = bra.bf1, k0 = ket.bf0, l0 = ket.bf1;
            const T* __restrict__ Dj32 = density_of<T>(a.Dj, a.Dj32) + bra.moff;
            auto d32 = [&](const T* D, int r, int c) { return __ldg(D + (long long)r * K + c); };
            auto put = [&](double* M, int r, int c, T v) {
                if (v != (T)0) add_to_fp64<T>(M + (long long)r * K + c, v);
            };
            for (int ab = lane; ab < nab; ab += 32) {
                T sj = 0;
                for (int cd = 0; cd < ncd; ++cd) sj += d32(Dj32, k0 + cd / n3, l0 + cd % n3) * acc[ab * ncd + cd];
                put(J, i0 + ab / n1, j0 + ab % n1, sj);
            }
            for (int cd = lane; cd < ncd; cd += 32) {
                T sj = 0;
                for (int ab = 0; ab < nab; ++ab) sj += d32(Dj32, i0 + ab / n1, j0 + ab % n1) * acc[ab * ncd + cd];
                put(J, k0 + cd / n3, l0 + cd % n3, sj);
            }
            for (int sp = 0; sp < NK; ++sp) {
                const T* __restrict__ Dk32 =
                    (sp == 0 ? density_of<T>(a.Dk, a.Dk32) : density_of<T>(a.Dk2, a.Dk232)) + bra.moff;
                double* KK = sp == 0 ? Kx : Kx2;
                // K_ik += D_jl v over (b, d)
                for (int q = lane; q < n0 * n2; q += 32) {
                    const int ia = q / n2, ic = q - ia * n2;
                    T s = 0;
                    for (int ib = 0; ib < n1; ++ib)
                        for (int id = 0; id < n3; ++id)
                            s += d32(Dk32, j0 + ib, l0 + id) * acc[(ia * n1 + ib) * ncd + ic * n3 + id];
                    put(KK, i0 + ia, k0 + ic, s);
                }
                // K_jl += D_ik v over (a, c)
                for (int q = lane; q < n1 * n3; q += 32) {
                    const int ib = q / n3, id = q - ib * n3;
                    T s = 0;
                    for (int ia = 0; ia < n0; ++ia)
                        for (int ic = 0; ic < n2; ++ic)
                            s += d32(Dk32, i0 + ia, k0 + ic) * acc[(ia * n1 + ib) * ncd + ic * n3 + id];
                    put(KK, j0 + ib, l0 + id, s);
                }
                // K_il += D_jk v over (b, c)
                for (int q = lane; q < n0 * n3; q += 32) {
                    const int ia = q / n3, id = q - ia * n3;
                    T s = 0;
                    for (int ib = 0; ib < n1; ++ib)
                        for (int ic = 0; ic < n2; ++ic)
                            s += d32(Dk32, j0 + ib, k0 + ic) * acc[(ia * n1 + ib) * ncd + ic * n3 + id];
                    put(KK, i0 + ia, l0 + id, s);
                }
                // K_jk += D_il v over (a, d)
                for (int q = lane; q < n1 * n2; q += 32) {
                    const int ib = q / n2, ic = q - ib * n2;
                    T s = 0;
                    for (int ia = 0; ia < n0; ++ia)
                        for (int id = 0; id < n3; ++id)
                            s += d32(Dk32, i0 + ia, l0 + id) * acc[(ia * n1 + ib) * ncd + ic * n3 + id];
                    put(KK, j0 + ib, k0 + ic, s);
                }
            }
        }
        __syncwarp();
    }
}

// slice size (T elements) a task needs
int warp_slice_elems(int l0b, int l1b, int l0k, int l1k, int npp_ket, int lane_min_npp)
{
    int L1 = l0b + l1b, L2 = l0k + l1k, L = L1 + L2;
    int nab = w_nc(l0b) * w_nc(l1b), ncd = w_nc(l0k) * w_nc(l1k);
    int HL = w_nh(L);
    bool lane_mode = lane_min_npp > 0 && L <= 6 && npp_ket >= lane_min_npp;
    int r = lane_mode ? HL * 32 + (L + 1) * 32 : (2 + kWarpKetRound) * HL + (L + 1);
    return nab * ncd + w_nh(L1) * ncd + r;
}

// Raise a kernel's dynamic shared-memory limit to the device maximum once
// per process: launches from concurrent jobs then never race on the attribute.
template <typename K>
static cudaError_t allow_max_smem(K kern)
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

template <typename T>
static cudaError_t warp_spec_t(int nk, int grid, int warps_per_cta, int slice, KernelSpec* s)
{
    auto pick = [&](auto kern) -> cudaError_t {
        s->func = (const void*)kern;
        return allow_max_smem(kern);
    };
    cudaError_t e = nk == 2 ? pick(k_warp_quartet<T, 2>) : nk == 0 ? pick(k_warp_quartet<T, 0>) : pick(k_warp_quartet<T, 1>);
    s->grid = dim3((unsigned)grid);
    s->block = dim3((unsigned)(32 * warps_per_cta));
    s->smem = kWarpSmemHeader + sizeof(T) * (size_t)slice * warps_per_cta;
    return e;
}

// Launch configuration of k_warp_quartet<T, nk> (T = float when fp32); also
// raises the kernel's shared-memory limit the first time it is asked for.
cudaError_t warp_spec(bool fp32, int nk, int grid, int warps_per_cta, int slice, KernelSpec* s)
{
    return fp32 ? warp_spec_t<float>(nk, grid, warps_per_cta, slice, s)
                : warp_spec_t<double>(nk, grid, warps_per_cta, slice, s);
}

cudaError_t launch_warp(bool fp32, const void* args, int nk, int grid, int warps_per_cta, cudaStream_t st)
{
    const int slice = fp32 ? ((const WarpArgs<float>*)args)->slice : ((const WarpArgs<double>*)args)->slice;
    KernelSpec s;
    cudaError_t e = warp_spec(fp32, nk, grid, warps_per_cta, slice, &s);
    if (e != cudaSuccess) return e;
    void* prm[] = {const_cast<void*>(args)};
    return cudaLaunchKernel(s.func, s.grid, s.block, prm, s.smem, st);
}

}  // namespace hfx
