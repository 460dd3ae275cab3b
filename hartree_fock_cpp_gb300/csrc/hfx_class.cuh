// hfx_class.cuh -- thread-per-shell-quartet kernels for the small
// angular-momentum classes (at most 36 Cartesian integrals per shell quartet
// and total L <= 4: (ss|ss) (ps|ss) (ps|ps) (pp|ss) (pp|ps) (ds|ss) (ds|ps)
// (ds|ds) (dp|ss)), instantiated for T = double and T = float.
//
// These classes carry most of the primitive quartets of contracted basis sets
// (cc-pVDZ carbon s shells have 9 primitives, so one (ss|ss) shell quartet is
// up to 6561 primitive quartets).  One thread owns one shell quartet and loops
// over all of its primitive quartets with every index, loop bound and
// sparsity pattern fixed at compile time: the Boys seeds, the R_{tuv} table,
// the ket-transformed W and the Cartesian accumulators stay in registers; no
// shared memory, no barriers.  The quartet list of a class is sorted by
// primitive count, so a warp's 32 lanes run loops of equal length.
//
// Per primitive quartet (the reference's primitive_repulsion,
// integrals.hpp:624-699, evaluated once per shell quartet here):
//   s_m = 2 pi^{5/2} / (p q sqrt(p+q)) (-2 rho)^m F_m(T)
//   R   in-place downward recursion over m (integrals.hpp:541-618)
//   W_cd[tuv] = sum_{tnp in nz(cd)} (-1)^{|tnp|} c^{kl}_{cd,tnp} R[tuv+tnp]
//   acc[ab][cd] += sum_{tuv in nz(ab)} c^{ij}_{ab,tuv} W_cd[tuv]
// with the coefficient records of hfx_device.cuh.
#pragma once

#include <cuda_runtime.h>

#include "hfx_device.cuh"

namespace hfx {

__host__ __device__ constexpr int c_nc(int l) { return (l + 1) * (l + 2) / 2; }
__host__ __device__ constexpr int c_nh(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }

__host__ __device__ constexpr int comp_x(int L, int c)
{
    int n = 0;
    for (int a = 0; a <= L; ++a)
        for (int b = 0; b <= L - a; ++b) {
            if (n == c) return a;
            ++n;
        }
    return 0;
}
__host__ __device__ constexpr int comp_y(int L, int c)
{
    int n = 0;
    for (int a = 0; a <= L; ++a)
        for (int b = 0; b <= L - a; ++b) {
            if (n == c) return b;
            ++n;
        }
    return 0;
}
__host__ __device__ constexpr int comp_z(int L, int c) { return L - comp_x(L, c) - comp_y(L, c); }

__host__ __device__ constexpr int hidx(int t, int u, int v)
{
    return (t + u + v) * (t + u + v + 1) * (t + u + v + 2) / 6 + t * (t + u + v + 1) - t * (t - 1) / 2 + u;
}

// (t, u, v) of packed Hermite index h (inverse of hidx): s-major, then t, then u.
__host__ __device__ constexpr int herm_s(int h)
{
    int s = 0;
    while ((s + 1) * (s + 2) * (s + 3) / 6 <= h) ++s;
    return s;
}
__host__ __device__ constexpr int herm_t(int h)
{
    int s = herm_s(h), o = h - s * (s + 1) * (s + 2) / 6, t = 0;
    while (o >= s - t + 1) {
        o -= s - t + 1;
        ++t;
    }
    return t;
}
__host__ __device__ constexpr int herm_u(int h)
{
    int s = herm_s(h), t = herm_t(h);
    return h - s * (s + 1) * (s + 2) / 6 - (t * (s + 1) - t * (t - 1) / 2);
}
__host__ __device__ constexpr int herm_v(int h) { return herm_s(h) - herm_t(h) - herm_u(h); }
__host__ __device__ constexpr bool herm_inverse_ok()
{
    for (int h = 0; h < 455; ++h)
        if (hidx(herm_t(h), herm_u(h), herm_v(h)) != h || herm_u(h) < 0 || herm_v(h) < 0) return false;
    return true;
}
static_assert(herm_inverse_ok(), "packed Hermite index inverse");

// Compile-time loops: cfor<B, E>(f) calls f(CInt<B>{}) ... f(CInt<E-1>{}), so
// that every index inside f is a constant expression.  The class kernels
// index their register arrays (R, the ket sums, the accumulators) only
// through such constants; a loop the compiler declined to unroll would turn
// them into local-memory arrays.
template <int V>
struct CInt {
    static constexpr int value = V;
};
template <int B, int E, typename F>
__device__ __forceinline__ void cfor(F&& f)
{
    if constexpr (B < E) {
        f(CInt<B>{});
        cfor<B + 1, E>(f);
    }
}

// number of non-zero coefficients of component pair ab of a (la, lb) pair
__host__ __device__ constexpr int n_coef_ab(int la, int lb, int ab)
{
    int nb = c_nc(lb);
    int a = ab / nb, b = ab % nb;
    return (comp_x(la, a) + comp_x(lb, b) + 1) * (comp_y(la, a) + comp_y(lb, b) + 1) *
           (comp_z(la, a) + comp_z(lb, b) + 1);
}
__host__ __device__ constexpr int coef_off(int la, int lb, int ab)
{
    int o = 0;
    for (int x = 0; x < ab; ++x) o += n_coef_ab(la, lb, x);
    return o;
}
__host__ __device__ constexpr int n_coef(int la, int lb) { return coef_off(la, lb, c_nc(la) * c_nc(lb)); }
// record length: header + coefficients, padded to a multiple of 4 elements
// (records start 16-byte aligned in FP32 and 32-byte aligned in FP64)
__host__ __device__ constexpr int rec_stride(int la, int lb) { return (5 + n_coef(la, lb) + 3) & ~3; }


// F_0..F_L: table + Taylor for F_L and exp(-T), downward recursion; beyond
// the table the asymptotic F_0 and upward recursion.
template <typename T, int L>
__device__ __forceinline__ void boys_all(T Tv, const T* __restrict__ tab, T (&F)[L + 1])
{
    if constexpr (sizeof(T) == 4) {
        // FP32: both forms, then a select per order (no divergence inside a
        // warp whose lanes straddle T = 36): the table row of (L, k) as two
        // 16-byte loads, Taylor + downward recursion; and the asymptotic
        // F_0 = sqrt(pi/T)/2 with upward recursion (exp(-T) < 3e-16 there)
        const bool in_table = Tv < (T)kBoysTMax;
        int k;
        const T nd = boys_grid_offset(in_table ? Tv : (T)0, k);
        const float4* row = reinterpret_cast<const float4*>(tab + ((size_t)L * kBoysN + k) * kBoys32Row);
        const float4 c0 = __ldg(row), c1 = __ldg(row + 1);
        T Ft[L + 1];
        T r = c1.x;                       // F_{L+4}/24
        r = fma(r, nd, c0.w);             // F_{L+3}/6
        r = fma(r, nd, c0.z);             // F_{L+2}/2
        r = fma(r, nd, c0.y);             // F_{L+1}
        Ft[L] = fma(r, nd, c0.x);
        if constexpr (L > 0) {
            T x = (T)(1.0 / 24.0);
            x = fma(x, nd, (T)(1.0 / 6.0));
            x = fma(x, nd, (T)0.5);
            x = fma(x, nd, (T)1);
            x = fma(x, nd, (T)1);
            const T e = c1.y * x;
            const T t2 = Tv + Tv;
#pragma unroll
            for (int m = L - 1; m >= 0; --m) Ft[m] = fma(t2, Ft[m + 1], e) * ((T)1 / (T)(2 * m + 1));
        }
        const T rs = rsqrt(fmax(Tv, (T)1e-30));
        T Fa = (T)0.88622692545275801365 * rs;
        const T inv2T = (T)0.5 * rs * rs;
#pragma unroll
        for (int m = 0; m <= L; ++m) {
            F[m] = in_table ? Ft[m] : Fa;
            Fa = (T)(2 * m + 1) * Fa * inv2T;
        }
    } else {
        if (Tv < (T)kBoysTMax) {
            // the (L, k) row: F_{L+j}(T_k) / j!, j = 0..6, then exp(-T_k)
            const int k = (int)(Tv * (T)kBoysInvStep + (T)0.5);
            const T nd = (T)k * ((T)1 / (T)kBoysInvStep) - Tv;
            const double2* row = reinterpret_cast<const double2*>(tab + ((size_t)L * kBoysN + k) * kBoys64Row);
            const double2 c0 = __ldg(row), c1 = __ldg(row + 1), c2 = __ldg(row + 2), c3 = __ldg(row + 3);
            T r = c3.x;
            r = fma(r, nd, c2.y);
            r = fma(r, nd, c2.x);
            r = fma(r, nd, c1.y);
            r = fma(r, nd, c1.x);
            r = fma(r, nd, c0.y);
            F[L] = fma(r, nd, c0.x);
            if constexpr (L > 0) {
                T x = (T)(1.0 / 5040.0);
                x = fma(x, nd, (T)(1.0 / 720.0));
                x = fma(x, nd, (T)(1.0 / 120.0));
                x = fma(x, nd, (T)(1.0 / 24.0));
                x = fma(x, nd, (T)(1.0 / 6.0));
                x = fma(x, nd, (T)0.5);
                x = fma(x, nd, (T)1);
                x = fma(x, nd, (T)1);
                const T e = c3.y * x;
                const T t2 = Tv + Tv;
    #pragma unroll
                for (int m = L - 1; m >= 0; --m) F[m] = fma(t2, F[m + 1], e) * ((T)1 / (T)(2 * m + 1));
            }
        } else {
            const T rs = rsqrt(Tv);
            F[0] = (T)0.88622692545275801365 * rs;
            if constexpr (L > 0) {
                const T inv2T = (T)0.5 * rs * rs;
    #pragma unroll
                for (int m = 0; m < L; ++m) F[m + 1] = (T)(2 * m + 1) * F[m] * inv2T;
            }
        }
    }
}

template <typename T, int L>
__device__ __forceinline__ void hermite_R(T X, T Y, T Z, const T (&s)[L + 1], T (&R)[c_nh(L)])
{
    R[0] = s[L];
    cfor<0, L>([&](auto ic) {
        constexpr int n = L - 1 - decltype(ic)::value;
        // levels L-n down to 1, each from the two levels below it (still
        // holding the values of order n+1)
        cfor<0, L - n>([&](auto jc) {
            constexpr int sl = L - n - decltype(jc)::value;
            cfor<0, sl + 1>([&](auto tc) {
                constexpr int t = decltype(tc)::value;
                cfor<0, sl - t + 1>([&](auto uc) {
                    constexpr int u = decltype(uc)::value, v = sl - t - u;
                    T val;
                    if constexpr (t > 0) {
                        val = X * R[hidx(t - 1, u, v)];
                        if constexpr (t > 1) val = fma((T)(t - 1), R[hidx(t - 2, u, v)], val);
                    } else if constexpr (u > 0) {
                        val = Y * R[hidx(t, u - 1, v)];
                        if constexpr (u > 1) val = fma((T)(u - 1), R[hidx(t, u - 2, v)], val);
                    } else {
                        val = Z * R[hidx(t, u, v - 1)];
                        if constexpr (v > 1) val = fma((T)(v - 1), R[hidx(t, u, v - 2)], val);
                    }
                    R[hidx(t, u, v)] = val;
                });
            });
        });
        R[0] = s[n];
    });
}

// (p, Px, Py, Pz) of a primitive-pair record: one 16-byte load in FP32
// (records are 16-byte aligned), four loads in FP64
template <typename T>
__device__ __forceinline__ void load_header(const T* r, T& p, T& x, T& y, T& z)
{
    if constexpr (sizeof(T) == 4) {
        const float4 h = __ldg(reinterpret_cast<const float4*>(r));
        p = h.x;
        x = h.y;
        y = h.z;
        z = h.w;
    } else {
        p = __ldg(r);
        x = __ldg(r + 1);
        y = __ldg(r + 2);
        z = __ldg(r + 3);
    }
}

__device__ __forceinline__ long long spidx(int a, int b)
{
    int hi = a > b ? a : b, lo = a > b ? b : a;
    return (long long)hi * (hi + 1) / 2 + lo;
}

// Register bytes per thread for the ket sum Wt of the amortised bra
// transform (below this the class sums over the ket primitive pairs before
// the bra transform).
constexpr int kAmortizeBytes = 256;

// One task's ket component pairs cd in [C0, C1): primitive integrals, their
// contraction into acc[ab][cd - C0], and the digestion of that block.
template <typename T, int LA, int LB, int LC, int LD, int NK, int C0, int C1>
__device__ __forceinline__ void small_quartet(const SmallArgs<T>& a, const Task& tk, const DPair& bra,
                                              const DPair& ket)
{
    constexpr int L1 = LA + LB, L2 = LC + LD, L = L1 + L2;
    constexpr int NB = c_nc(LB), ND = c_nc(LD);
    constexpr int NAB = c_nc(LA) * NB, NCD = C1 - C0;
    constexpr int H1 = c_nh(L1), HL = c_nh(L);
    constexpr int SB = rec_stride(LA, LB), SK = rec_stride(LC, LD);
    // amortised bra transform when the ket sum fits in registers beside acc
    constexpr bool AMB = NCD * H1 * (int)sizeof(T) <= kAmortizeBytes;

    T acc[NAB][NCD];
#pragma unroll
    for (int x = 0; x < NAB; ++x)
#pragma unroll
        for (int y = 0; y < NCD; ++y) acc[x][y] = (T)0;

    const T* __restrict__ recb = a.rec + bra.rec_off;
    const T* __restrict__ reck = a.rec + ket.rec_off;
    const int ij1 = tk.i1, kl0 = tk.k0, kl1 = tk.k1;
    for (int ij = tk.i0; ij < ij1; ++ij) {
        const T* rb = recb + ij * SB;
        T p, Px, Py, Pz;
        load_header(rb, p, Px, Py, Pz);
        const T rp = __ldg(rb + 4);
        const T* cb = rb + 5;
        // kAmortizeBra: the ket-transformed integrals of every ket component
        // pair are summed over the task's ket primitive pairs first
        // (Wt[cd][tuv], in registers), and the bra transform is applied once
        // per bra primitive pair -- each bra coefficient is loaded once and
        // used for every cd.  Otherwise (classes whose Wt would not fit the
        // register file) the bra transform runs per primitive quartet.
        T Wt[AMB ? NCD : 1][AMB ? H1 : 1];
        if constexpr (AMB) {
#pragma unroll
            for (int cd = 0; cd < NCD; ++cd)
#pragma unroll
                for (int h = 0; h < H1; ++h) Wt[cd][h] = (T)0;
        }
        // the low-L classes are bound by the latency of the record and Boys-table
        // loads: two ket primitive pairs in flight per thread
#pragma unroll(L <= 2 ? 2 : 1)
        for (int kl = kl0; kl < kl1; ++kl) {
            const T* rk = reck + kl * SK;
            T q, Qx, Qy, Qz;
            load_header(rk, q, Qx, Qy, Qz);
            const T rq = __ldg(rk + 4);
            const T* ck = rk + 5;
            const T X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;
            // 1/sqrt(p+q) is the only root; 1/p, 1/q come with the records
            const T rs = rsqrt(p + q);
            const T rho = p * q * (rs * rs);
            const T Tv = rho * (X * X + Y * Y + Z * Z);
            const T pref = (T)34.98683665524972 * rp * rq * rs;   // 2 pi^{5/2} / (p q sqrt(p+q))
            T F[L + 1];
            boys_all<T, L>(Tv, a.boys, F);
            T sd[L + 1];
            {
                const T m2r = (T)-2 * rho;
                T pw = pref;
#pragma unroll
                for (int m = 0; m <= L; ++m) {
                    sd[m] = pw * F[m];
                    pw *= m2r;
                }
            }
            T R[HL];
            hermite_R<T, L>(X, Y, Z, sd, R);
            cfor<0, NCD>([&](auto cdc) {
                constexpr int cd = decltype(cdc)::value;       // local index in the block
                constexpr int c = (C0 + cd) / ND, d = (C0 + cd) % ND;
                constexpr int nx = comp_x(LC, c) + comp_x(LD, d), ny = comp_y(LC, c) + comp_y(LD, d),
                              nz = comp_z(LC, c) + comp_z(LD, d);
                constexpr int k0 = coef_off(LC, LD, C0 + cd);
                T W[AMB ? 1 : H1];
                if constexpr (!AMB) {
#pragma unroll
                    for (int h = 0; h < H1; ++h) W[h] = (T)0;
                }
                // W_cd[tuv] (+)= sum_{tnp in nz(cd)} (-1)^{|tnp|} c_{cd,tnp} R[tuv + tnp]
                cfor<0, nx + 1>([&](auto tnc) {
                    constexpr int tn = decltype(tnc)::value;
                    cfor<0, ny + 1>([&](auto nuc) {
                        constexpr int nu = decltype(nuc)::value;
                        cfor<0, nz + 1>([&](auto phc) {
                            constexpr int ph = decltype(phc)::value;
                            constexpr int k = k0 + (tn * (ny + 1) + nu) * (nz + 1) + ph;
                            T e = __ldg(ck + k);
                            if constexpr ((tn + nu + ph) & 1) e = -e;
                            cfor<0, H1>([&](auto hc) {
                                constexpr int h = decltype(hc)::value;
                                constexpr int t = herm_t(h), u = herm_u(h), v = herm_v(h);
                                constexpr int r = hidx(t + tn, u + nu, v + ph);
                                if constexpr (AMB)
                                    Wt[cd][h] = fma(e, R[r], Wt[cd][h]);
                                else
                                    W[h] = fma(e, R[r], W[h]);
                            });
                        });
                    });
                });
                if constexpr (!AMB) {
                    cfor<0, NAB>([&](auto abc) {
                        constexpr int ab = decltype(abc)::value;
                        constexpr int aa = ab / NB, bb = ab % NB;
                        constexpr int mx = comp_x(LA, aa) + comp_x(LB, bb), my = comp_y(LA, aa) + comp_y(LB, bb),
                                      mz = comp_z(LA, aa) + comp_z(LB, bb);
                        constexpr int kb0 = coef_off(LA, LB, ab);
                        T sacc = acc[ab][cd];
                        cfor<0, (mx + 1) * (my + 1) * (mz + 1)>([&](auto jc) {
                            constexpr int j = decltype(jc)::value;
                            constexpr int t = j / ((my + 1) * (mz + 1)), u = (j / (mz + 1)) % (my + 1), v = j % (mz + 1);
                            sacc = fma(__ldg(cb + kb0 + j), W[hidx(t, u, v)], sacc);
                        });
                        acc[ab][cd] = sacc;
                    });
                }
            });
        }
        if constexpr (AMB) {
            // bra transform of the ket sum, once per bra primitive pair
            cfor<0, NAB>([&](auto abc) {
                constexpr int ab = decltype(abc)::value;
                constexpr int aa = ab / NB, bb = ab % NB;
                constexpr int mx = comp_x(LA, aa) + comp_x(LB, bb), my = comp_y(LA, aa) + comp_y(LB, bb),
                              mz = comp_z(LA, aa) + comp_z(LB, bb);
                constexpr int kb0 = coef_off(LA, LB, ab);
                cfor<0, (mx + 1) * (my + 1) * (mz + 1)>([&](auto jc) {
                    constexpr int j = decltype(jc)::value;
                    constexpr int t = j / ((my + 1) * (mz + 1)), u = (j / (mz + 1)) % (my + 1), v = j % (mz + 1);
                    const T cv = __ldg(cb + kb0 + j);
                    cfor<0, NCD>([&](auto cdc) {
                        constexpr int cd = decltype(cdc)::value;
                        acc[ab][cd] = fma(cv, Wt[cd][hidx(t, u, v)], acc[ab][cd]);
                    });
                });
            });
        }
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
    const bool same_pair = (tk.bra == tk.ket);
    if constexpr (sizeof(T) == 8 && !kBlockDigestFP64) {
#pragma unroll
        for (int ab = 0; ab < NAB; ++ab) {
            const int ia = ab / NB, ib = ab % NB;
            const int i = bra.bf0 + ia, j = bra.bf1 + ib;
            const long long pij = spidx(i, j);
            const double qb = __ldg(Qbf + pij);
            if (bra.same && ia < ib) continue;
#pragma unroll
            for (int cd = 0; cd < NCD; ++cd) {
                const int ic = (C0 + cd) / ND, id = (C0 + cd) % ND;
                const int k = ket.bf0 + ic, l = ket.bf1 + id;
                if (ket.same && ic < id) continue;
                const long long pkl = spidx(k, l);
                if (same_pair && pij < pkl) continue;
                if (a.thr >= 0.0 && qb * __ldg(Qbf + pkl) < a.thr) continue;
                const double v =
                    (double)acc[ab][cd] * ((i == j ? 1.0 : 2.0) * (k == l ? 1.0 : 2.0) * (pij == pkl ? 1.0 : 2.0));
                atomicAdd(J + (long long)i * K + j, __ldg(Dj + (long long)k * K + l) * v);
                atomicAdd(J + (long long)k * K + l, __ldg(Dj + (long long)i * K + j) * v);
                atomicAdd(Kx + (long long)i * K + k, __ldg(Dk + (long long)j * K + l) * v);
                atomicAdd(Kx + (long long)j * K + l, __ldg(Dk + (long long)i * K + k) * v);
                atomicAdd(Kx + (long long)i * K + l, __ldg(Dk + (long long)j * K + k) * v);
                atomicAdd(Kx + (long long)j * K + k, __ldg(Dk + (long long)i * K + l) * v);
                if constexpr (NK == 2) {
                    atomicAdd(Kx2 + (long long)i * K + k, __ldg(Dk2 + (long long)j * K + l) * v);
                    atomicAdd(Kx2 + (long long)j * K + l, __ldg(Dk2 + (long long)i * K + k) * v);
                    atomicAdd(Kx2 + (long long)i * K + l, __ldg(Dk2 + (long long)j * K + k) * v);
                    atomicAdd(Kx2 + (long long)j * K + k, __ldg(Dk2 + (long long)i * K + l) * v);
                }
            }
        }
    } else {
        // Block digestion: the degeneracy weight is applied in place (0 for
        // the non-canonical and BF-screened elements); then every J / K
        // element the quartet touches is summed over the quartet in registers
        // (FP32 quartets: float products with the float density copies) and
        // added to the FP64 accumulators once -- nab + ncd + na nc + na nd +
        // nb nc + nb nd atomics per quartet instead of 6 per integral.
        constexpr int NA = c_nc(LA), NC = c_nc(LC);
        const T* __restrict__ QbT = schwarz_of<T>(a) + bra.qoff;
        const bool screen = a.thr >= 0.0;
        const T thrT = (T)a.thr;
#pragma unroll
        for (int ab = 0; ab < NAB; ++ab) {
            const int ia = ab / NB, ib = ab % NB;
            const int i = bra.bf0 + ia, j = bra.bf1 + ib;
            const long long pij = spidx(i, j);
            const T qb = __ldg(QbT + pij);
#pragma unroll
            for (int cd = 0; cd < NCD; ++cd) {
                const int ic = (C0 + cd) / ND, id = (C0 + cd) % ND;
                const int k = ket.bf0 + ic, l = ket.bf1 + id;
                const long long pkl = spidx(k, l);
                const bool skip = (bra.same && ia < ib) || (ket.same && ic < id) || (same_pair && pij < pkl) ||
                                  (screen && qb * __ldg(QbT + pkl) < thrT);
                const T f = (i == j ? (T)1 : (T)2) * (k == l ? (T)1 : (T)2) * (pij == pkl ? (T)1 : (T)2);
                acc[ab][cd] = skip ? (T)0 : acc[ab][cd] * f;
            }
        }
        const T* __restrict__ Dj32 = density_of<T>(a.Dj, a.Dj32) + bra.moff;
        const int i0 = bra.bf0, j0 = bra.bf1, k0 = ket.bf0, l0 = ket.bf1;
        auto d32 = [&](const T* D, int r, int c) { return __ldg(D + (long long)r * K + c); };
        auto put = [&](double* M, int r, int c, T v) {
            if (v != (T)0) add_to_fp64<T>(M + (long long)r * K + c, v);
        };
#pragma unroll
        for (int ab = 0; ab < NAB; ++ab) {
            T sj = 0;
#pragma unroll
            for (int cd = 0; cd < NCD; ++cd) sj += d32(Dj32, k0 + (C0 + cd) / ND, l0 + (C0 + cd) % ND) * acc[ab][cd];
            put(J, i0 + ab / NB, j0 + ab % NB, sj);
        }
#pragma unroll
        for (int cd = 0; cd < NCD; ++cd) {
            T sj = 0;
#pragma unroll
            for (int ab = 0; ab < NAB; ++ab) sj += d32(Dj32, i0 + ab / NB, j0 + ab % NB) * acc[ab][cd];
            put(J, k0 + (C0 + cd) / ND, l0 + (C0 + cd) % ND, sj);
        }
#pragma unroll
        for (int sp = 0; sp < NK; ++sp) {
            const T* __restrict__ Dk32 =
                (sp == 0 ? density_of<T>(a.Dk, a.Dk32) : density_of<T>(a.Dk2, a.Dk232)) + bra.moff;
            double* KK = sp == 0 ? Kx : Kx2;
            // K_ik += D_jl v, K_jl += D_ik v, K_il += D_jk v, K_jk += D_il v
#pragma unroll
            for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                for (int ic = 0; ic < NC; ++ic) {
                    T s = 0;
#pragma unroll
                    for (int ib = 0; ib < NB; ++ib)
#pragma unroll
                        for (int id = 0; id < ND; ++id)
                            if (ic * ND + id >= C0 && ic * ND + id < C1) s += d32(Dk32, j0 + ib, l0 + id) * acc[ia * NB + ib][ic * ND + id - C0];
                    put(KK, i0 + ia, k0 + ic, s);
                }
#pragma unroll
            for (int ib = 0; ib < NB; ++ib)
#pragma unroll
                for (int id = 0; id < ND; ++id) {
                    T s = 0;
#pragma unroll
                    for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                        for (int ic = 0; ic < NC; ++ic)
                            if (ic * ND + id >= C0 && ic * ND + id < C1) s += d32(Dk32, i0 + ia, k0 + ic) * acc[ia * NB + ib][ic * ND + id - C0];
                    put(KK, j0 + ib, l0 + id, s);
                }
#pragma unroll
            for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                for (int id = 0; id < ND; ++id) {
                    T s = 0;
#pragma unroll
                    for (int ib = 0; ib < NB; ++ib)
#pragma unroll
                        for (int ic = 0; ic < NC; ++ic)
                            if (ic * ND + id >= C0 && ic * ND + id < C1) s += d32(Dk32, j0 + ib, k0 + ic) * acc[ia * NB + ib][ic * ND + id - C0];
                    put(KK, i0 + ia, l0 + id, s);
                }
#pragma unroll
            for (int ib = 0; ib < NB; ++ib)
#pragma unroll
                for (int ic = 0; ic < NC; ++ic) {
                    T s = 0;
#pragma unroll
                    for (int ia = 0; ia < NA; ++ia)
#pragma unroll
                        for (int id = 0; id < ND; ++id)
                            if (ic * ND + id >= C0 && ic * ND + id < C1) s += d32(Dk32, i0 + ia, l0 + id) * acc[ia * NB + ib][ic * ND + id - C0];
                    put(KK, j0 + ib, k0 + ic, s);
                }
        }
    }
}

// Ket component-pair blocks of a class kernel: classes whose accumulators
// would not fit the register file split their ket component pairs over
// small_ncb(...) threads per task (each computes R, its block's ket sums,
// its block's integrals and their digestion; J and K are linear in the
// integrals), at most 36 (FP64) / 40 (FP32) accumulators per thread.
template <typename T, int LA, int LB, int LC, int LD>
__host__ __device__ constexpr int small_ncb()
{
    constexpr int ncd = c_nc(LC) * c_nc(LD);
    constexpr int nab = c_nc(LA) * c_nc(LB);
    constexpr int budget = sizeof(T) == 8 ? 36 : 40;   // accumulators per thread
    int nb = 1;
    while (nb < ncd && nab * ((ncd + nb - 1) / nb) > budget) ++nb;
    return nb;
}

template <typename T, int LA, int LB, int LC, int LD, int NK>
__global__ void __launch_bounds__(128) k_small(SmallArgs<T> a)
{
    constexpr int NCD = c_nc(LC) * c_nc(LD);
    constexpr int NCB = small_ncb<T, LA, LB, LC, LD>();
    const int task = blockIdx.x * blockDim.x + threadIdx.x;
    if (task >= a.ntasks) return;
    const Task tk = a.tasks[task];
    const DPair bra = a.pairs[tk.bra];
    const DPair ket = a.pairs[tk.ket];
    if (molecule_inactive(bra, a.active)) return;
    if (density_negligible(bra, ket, a.Dsh, a.dthr)) return;
    if constexpr (NCB == 1) {
        small_quartet<T, LA, LB, LC, LD, NK, 0, NCD>(a, tk, bra, ket);
    } else {
        cfor<0, NCB>([&](auto bc) {
            constexpr int b = decltype(bc)::value;
            if (blockIdx.y == b) small_quartet<T, LA, LB, LC, LD, NK, b * NCD / NCB, (b + 1) * NCD / NCB>(a, tk, bra, ket);
        });
    }
}

// One thread per task, 128 threads per CTA; the kernel takes SmallArgs<T> by value.
template <typename T, int LA, int LB, int LC, int LD>
cudaError_t small_spec(int nk, int ntasks, KernelSpec* s)
{
    s->func = nk == 2 ? (const void*)k_small<T, LA, LB, LC, LD, 2> : (const void*)k_small<T, LA, LB, LC, LD, 1>;
    s->block = dim3(128);
    s->grid = dim3((unsigned)((ntasks + 127) / 128), (unsigned)small_ncb<T, LA, LB, LC, LD>());
    s->smem = 0;
    return cudaSuccess;
}

}  // namespace hfx
