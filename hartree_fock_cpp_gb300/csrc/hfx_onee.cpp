// hfx_onee.cpp -- host one-electron integrals (S, T, V) and the host Boys
// function.  These are the SCF driver's setup matrices (the reference's
// overlap_matrix / kinetic_matrix / attraction_matrix, integrals.hpp:10-536),
// evaluated per shell pair with McMurchie-Davidson Hermite expansions:
//   S = E^x_0 E^y_0 E^z_0 (pi/p)^{3/2}
//   T : the reference's per-axis kinetic form (integrals.hpp:122-177)
//       T^x_ij = b(2j+1) S_ij - 2 b^2 S_i,j+2 - j(j-1)/2 S_i,j-2
//   V = -sum_C Z_C 2 pi / p sum_tuv E_t E_u E_v R_tuv(p, P - C)
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>

#include "hfx_internal.hpp"

namespace hfx {

double boys_host(int m, double T)
{
    // F_m(T) = exp(-T) sum_k (2T)^k / ((2m+1)(2m+3)...(2m+2k+1)), all terms
    // positive; beyond T = 50 the asymptotic form with upward recursion.
    if (T <= 50.0) {
        long double term = 1.0L / (2.0L * m + 1.0L), sum = term;
        for (int k = 1; k < 600; ++k) {
            term *= 2.0L * T / (2.0L * m + 2.0L * k + 1.0L);
            sum += term;
            if (term < 1e-21L * sum) break;
        }
        return (double)(std::exp(-(long double)T) * sum);
    }
    double F = 0.5 * std::sqrt(M_PI / T);
    double e = std::exp(-T);
    for (int k = 0; k < m; ++k) F = ((2.0 * k + 1.0) * F - e) / (2.0 * T);
    return F;
}

// F_0..F_L(T) for the host integrals: table of accurate values at T_k = k/16
// (built once from boys_host), 7-term Taylor for F_L, downward recursion;
// asymptotic form with upward recursion beyond T = 36.
static void boys_fast(int L, double T, double* F)
{
    constexpr int NM = 26, NT = 36 * 16 + 1;
    static const std::vector<double> tab = [] {
        std::vector<double> t((size_t)NT * (NM + 1));
        for (int k = 0; k < NT; ++k) {
            for (int m = 0; m < NM; ++m) t[(size_t)k * (NM + 1) + m] = boys_host(m, k / 16.0);
            t[(size_t)k * (NM + 1) + NM] = std::exp(-k / 16.0);
        }
        return t;
    }();
    if (T < 36.0 && L + 6 < NM) {
        int k = (int)(T * 16.0 + 0.5);
        double nd = k / 16.0 - T;
        const double* f = tab.data() + (size_t)k * (NM + 1);
        static const double inv_fact[7] = {1.0, 1.0, 0.5, 1.0 / 6, 1.0 / 24, 1.0 / 120, 1.0 / 720};
        double r = 0.0;
        for (int j = 6; j >= 0; --j) r = r * nd + f[L + j] * inv_fact[j];
        F[L] = r;
        double x = 1.0 / 5040.0;
        for (int j = 6; j >= 0; --j) x = x * nd + inv_fact[j];
        double e = f[NM] * x;
        for (int m = L - 1; m >= 0; --m) F[m] = (2.0 * T * F[m + 1] + e) / (2.0 * m + 1.0);
        return;
    }
    if (T >= 36.0) {
        double e = std::exp(-T);
        F[0] = 0.5 * std::sqrt(M_PI / T);
        for (int m = 0; m < L; ++m) F[m + 1] = ((2.0 * m + 1.0) * F[m] - e) / (2.0 * T);
        return;
    }
    for (int m = 0; m <= L; ++m) F[m] = boys_host(m, T);
}

// 1-D Hermite expansion coefficients E^{ij}_t for i <= imax, j <= jmax,
// stored E[(i*(jmax+1)+j)*(imax+jmax+1)+t]; same recursion as
// integrals.hpp:269-322 (without its L <= 4 cap).
void hermite_1d(int imax, int jmax, double a, double b, double A, double B, std::vector<double>& E)
{
    int nt = imax + jmax + 1;
    E.assign((size_t)(imax + 1) * (jmax + 1) * nt, 0.0);
    auto at = [&](int i, int j, int t) -> double& { return E[((size_t)i * (jmax + 1) + j) * nt + t]; };
    double p = a + b, mu = a * b / p, AB = A - B;
    double XPA = -(b / p) * AB, XPB = (a / p) * AB, o2p = 1.0 / (2.0 * p);
    at(0, 0, 0) = std::exp(-mu * AB * AB);
    for (int i = 1; i <= imax; ++i)
        for (int t = 0; t <= i; ++t) {
            double v = XPA * at(i - 1, 0, t);
            if (t > 0) v += o2p * at(i - 1, 0, t - 1);
            if (t + 1 <= i - 1) v += (t + 1) * at(i - 1, 0, t + 1);
            at(i, 0, t) = v;
        }
    for (int i = 0; i <= imax; ++i)
        for (int j = 1; j <= jmax; ++j)
            for (int t = 0; t <= i + j; ++t) {
                double v = (t <= i + j - 1) ? XPB * at(i, j - 1, t) : 0.0;
                if (t > 0) v += o2p * at(i, j - 1, t - 1);
                if (t + 1 <= i + j - 1) v += (t + 1) * at(i, j - 1, t + 1);
                at(i, j, t) = v;
            }
}

// All R_{tuv}(p, PC) with t+u+v <= L into R[(t*(L+1)+u)*(L+1)+v].
static void hermite_R(int L, double p, double X, double Y, double Z, std::vector<double>& R)
{
    int n = L + 1;
    std::vector<double> cur((size_t)n * n * n, 0.0), nxt((size_t)n * n * n, 0.0);
    double T = p * (X * X + Y * Y + Z * Z);
    std::vector<double> F(L + 1);
    boys_fast(L, T, F.data());
    auto id = [n](int t, int u, int v) { return ((size_t)t * n + u) * n + v; };
    // level m = L holds only R^{(L)}_{000}
    double pw = std::pow(-2.0 * p, L);
    nxt[0] = pw * F[L];
    for (int m = L - 1; m >= 0; --m) {
        std::fill(cur.begin(), cur.end(), 0.0);
        cur[0] = std::pow(-2.0 * p, m) * F[m];
        int top = L - m;
        for (int s = 1; s <= top; ++s)
            for (int t = 0; t <= s; ++t)
                for (int u = 0; u <= s - t; ++u) {
                    int v = s - t - u;
                    double val;
                    if (t > 0) {
                        val = X * nxt[id(t - 1, u, v)];
                        if (t > 1) val += (t - 1) * nxt[id(t - 2, u, v)];
                    } else if (u > 0) {
                        val = Y * nxt[id(t, u - 1, v)];
                        if (u > 1) val += (u - 1) * nxt[id(t, u - 2, v)];
                    } else {
                        val = Z * nxt[id(t, u, v - 1)];
                        if (v > 1) val += (v - 1) * nxt[id(t, u, v - 2)];
                    }
                    cur[id(t, u, v)] = val;
                }
        std::swap(cur, nxt);
    }
    R = nxt;
}

void one_electron(const Basis& b, std::vector<double>& S, std::vector<double>& T, std::vector<double>& V)
{
    int K = b.K;
    S.assign((size_t)K * K, 0.0);
    T.assign((size_t)K * K, 0.0);
    V.assign((size_t)K * K, 0.0);
    int natom = (int)b.atom_Z.size();
    const int ns = (int)b.shells.size();
    std::vector<std::pair<int, int>> pairs;
    for (int sa = 0; sa < ns; ++sa)
        for (int sb = 0; sb <= sa; ++sb) pairs.push_back({sa, sb});
    std::atomic<size_t> next{0};
    auto worker = [&]() {
    std::vector<double> Ex, Ey, Ez, R;
    for (size_t pi = next++; pi < pairs.size(); pi = next++) {
        {
            const int sa = pairs[pi].first, sb = pairs[pi].second;
            const Shell& A = b.shells[sa];
            const Shell& B = b.shells[sb];
            int na = ncart(A.L), nb = ncart(B.L);
            int jm = B.L + 2;  // kinetic needs j+2
            int nt = A.L + jm + 1;
            std::vector<double> s(na * nb, 0.0), t(na * nb, 0.0), v(na * nb, 0.0);
            for (int i = 0; i < A.nprim(); ++i)
                for (int j = 0; j < B.nprim(); ++j) {
                    double a = A.exps[i], be = B.exps[j], p = a + be;
                    hermite_1d(A.L, jm, a, be, A.x, B.x, Ex);
                    hermite_1d(A.L, jm, a, be, A.y, B.y, Ey);
                    hermite_1d(A.L, jm, a, be, A.z, B.z, Ez);
                    auto e = [&](const std::vector<double>& E, int ii, int jj, int tt) {
                        if (jj < 0) return 0.0;
                        return E[((size_t)ii * (jm + 1) + jj) * nt + tt];
                    };
                    double sq = std::sqrt(M_PI / p);
                    double Px = (a * A.x + be * B.x) / p, Py = (a * A.y + be * B.y) / p, Pz = (a * A.z + be * B.z) / p;
                    // nuclear attraction Hermite integrals for each atom
                    int L = A.L + B.L;
                    std::vector<std::vector<double>> Rat(natom);
                    for (int c = 0; c < natom; ++c)
                        hermite_R(L, p, Px - b.atom_xyz[3 * c], Py - b.atom_xyz[3 * c + 1], Pz - b.atom_xyz[3 * c + 2],
                                  Rat[c]);
                    for (int ca = 0; ca < na; ++ca) {
                        int ax, ay, az;
                        component(A.L, ca, ax, ay, az);
                        for (int cb = 0; cb < nb; ++cb) {
                            int bx, by, bz;
                            component(B.L, cb, bx, by, bz);
                            double w = A.w[(size_t)ca * A.nprim() + i] * B.w[(size_t)cb * B.nprim() + j];
                            double Sx = e(Ex, ax, bx, 0) * sq, Sy = e(Ey, ay, by, 0) * sq, Sz = e(Ez, az, bz, 0) * sq;
                            s[ca * nb + cb] += w * Sx * Sy * Sz;
                            auto kin = [&](const std::vector<double>& E, int ii, int jj) {
                                double t1 = be * (2 * jj + 1) * e(E, ii, jj, 0) * sq;
                                double t2 = -2 * be * be * e(E, ii, jj + 2, 0) * sq;
                                double t3 = jj >= 2 ? -0.5 * jj * (jj - 1) * e(E, ii, jj - 2, 0) * sq : 0.0;
                                return t1 + t2 + t3;
                            };
                            double Tx = kin(Ex, ax, bx), Ty = kin(Ey, ay, by), Tz = kin(Ez, az, bz);
                            t[ca * nb + cb] += w * (Tx * Sy * Sz + Sx * Ty * Sz + Sx * Sy * Tz);
                            double vv = 0.0;
                            int n1 = L + 1;
                            for (int c = 0; c < natom; ++c) {
                                double acc = 0.0;
                                for (int tt = 0; tt <= ax + bx; ++tt)
                                    for (int uu = 0; uu <= ay + by; ++uu)
                                        for (int ww = 0; ww <= az + bz; ++ww)
                                            acc += e(Ex, ax, bx, tt) * e(Ey, ay, by, uu) * e(Ez, az, bz, ww) *
                                                   Rat[c][((size_t)tt * n1 + uu) * n1 + ww];
                                vv += -b.atom_Z[c] * acc;
                            }
                            v[ca * nb + cb] += w * (2.0 * M_PI / p) * vv;
                        }
                    }
                }
            for (int ca = 0; ca < na; ++ca)
                for (int cb = 0; cb < nb; ++cb) {
                    int I = A.bf0 + ca, J = B.bf0 + cb;
                    S[(size_t)I * K + J] = S[(size_t)J * K + I] = s[ca * nb + cb];
                    T[(size_t)I * K + J] = T[(size_t)J * K + I] = t[ca * nb + cb];
                    V[(size_t)I * K + J] = V[(size_t)J * K + I] = v[ca * nb + cb];
                }
        }
    }
    };
    // each shell pair writes its own blocks of S, T, V
    const int nthreads = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (int t = 1; t < nthreads && (size_t)t < pairs.size(); ++t) th.emplace_back(worker);
    worker();
    for (auto& x : th) x.join();
}

}  // namespace hfx
