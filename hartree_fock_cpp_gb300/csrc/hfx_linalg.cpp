// hfx_linalg.cpp -- the dense host linear algebra the SCF driver needs, in
// place of the reference's Eigen calls (linalg.hpp:132-170 eigensolves,
// linalg.hpp:430-447 fullPivLu):
//   * sym_eig: Householder reduction to tridiagonal form followed by the
//     implicit symmetric QR iteration with Wilkinson shifts (Golub & Van
//     Loan, "Matrix Computations", Alg. 8.3.1 and 8.3.3), eigenvectors
//     accumulated; eigenvalues returned ascending like Eigen's
//     SelfAdjointEigenSolver.
//   * solve_full_piv: Gaussian elimination with complete pivoting.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "hfx_internal.hpp"

namespace hfx {

void matmul(int n, const double* A, const double* B, double* C)
{
    std::vector<double> tmp((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < n; ++k) {
            double a = A[(size_t)i * n + k];
            if (a == 0.0) continue;
            const double* b = B + (size_t)k * n;
            double* c = tmp.data() + (size_t)i * n;
            for (int j = 0; j < n; ++j) c[j] += a * b[j];
        }
    std::copy(tmp.begin(), tmp.end(), C);
}

void matmul_tn(int n, const double* A, const double* B, double* C)
{
    std::vector<double> tmp((size_t)n * n, 0.0);
    for (int k = 0; k < n; ++k)
        for (int i = 0; i < n; ++i) {
            double a = A[(size_t)k * n + i];
            if (a == 0.0) continue;
            const double* b = B + (size_t)k * n;
            double* c = tmp.data() + (size_t)i * n;
            for (int j = 0; j < n; ++j) c[j] += a * b[j];
        }
    std::copy(tmp.begin(), tmp.end(), C);
}

// Householder tridiagonalisation: A (row-major, symmetric, overwritten) ->
// Q^T A Q = tridiag(d, e); Q returned in Qm (row-major).
static void tridiagonalize(int n, std::vector<double>& A, std::vector<double>& d, std::vector<double>& e,
                           std::vector<double>& Qm)
{
    auto a = [&](int i, int j) -> double& { return A[(size_t)i * n + j]; };
    Qm.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) Qm[(size_t)i * n + i] = 1.0;
    std::vector<double> v(n), p(n), w(n);
    for (int k = 0; k + 2 < n; ++k) {
        // x = A[k+1:n, k]
        double alpha = 0.0;
        for (int i = k + 1; i < n; ++i) alpha += a(i, k) * a(i, k);
        alpha = std::sqrt(alpha);
        if (alpha == 0.0) continue;
        double x0 = a(k + 1, k);
        double sgn = x0 >= 0 ? 1.0 : -1.0;
        // v = x + sgn*alpha*e1
        std::fill(v.begin(), v.end(), 0.0);
        for (int i = k + 1; i < n; ++i) v[i] = a(i, k);
        v[k + 1] += sgn * alpha;
        double vnorm2 = 0.0;
        for (int i = k + 1; i < n; ++i) vnorm2 += v[i] * v[i];
        if (vnorm2 == 0.0) continue;
        double beta = 2.0 / vnorm2;
        // p = beta * A v  (over trailing block rows/cols k..n-1; column k handled too)
        for (int i = k; i < n; ++i) {
            double s = 0.0;
            for (int j = k + 1; j < n; ++j) s += a(i, j) * v[j];
            p[i] = beta * s;
        }
        // K = beta/2 * v^T p ; w = p - K v
        double vp = 0.0;
        for (int i = k + 1; i < n; ++i) vp += v[i] * p[i];
        double Kc = 0.5 * beta * vp;
        for (int i = k; i < n; ++i) w[i] = p[i] - Kc * v[i];
        // A = A - v w^T - w v^T on rows/cols >= k (v[k] = 0)
        for (int i = k; i < n; ++i)
            for (int j = k; j < n; ++j) a(i, j) -= v[i] * w[j] + w[i] * v[j];
        // Q = Q H, H = I - beta v v^T
        for (int i = 0; i < n; ++i) {
            double s = 0.0;
            for (int j = k + 1; j < n; ++j) s += Qm[(size_t)i * n + j] * v[j];
            s *= beta;
            for (int j = k + 1; j < n; ++j) Qm[(size_t)i * n + j] -= s * v[j];
        }
    }
    d.assign(n, 0.0);
    e.assign(n, 0.0);
    for (int i = 0; i < n; ++i) d[i] = a(i, i);
    for (int i = 0; i + 1 < n; ++i) e[i] = a(i + 1, i);
}

void sym_eig(int n, const double* Ain, double* wout, double* Vout)
{
    std::vector<double> A(Ain, Ain + (size_t)n * n);
    // symmetrise defensively
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j) {
            double s = 0.5 * (A[(size_t)i * n + j] + A[(size_t)j * n + i]);
            A[(size_t)i * n + j] = A[(size_t)j * n + i] = s;
        }
    std::vector<double> d, e, Q;
    tridiagonalize(n, A, d, e, Q);
    // implicit symmetric QR with Wilkinson shift on (d, e[0..n-2])
    int hi = n - 1;
    int iter = 0;
    const double eps = 2.220446049250313e-16;
    while (hi > 0 && iter < 100 * n) {
        // deflate negligible off-diagonals
        for (int i = 0; i < hi; ++i)
            if (std::fabs(e[i]) <= eps * (std::fabs(d[i]) + std::fabs(d[i + 1]))) e[i] = 0.0;
        while (hi > 0 && e[hi - 1] == 0.0) --hi;
        if (hi == 0) break;
        int lo = hi - 1;
        while (lo > 0 && e[lo - 1] != 0.0) --lo;
        // Wilkinson shift from the trailing 2x2 of the block [lo, hi]
        double dd = 0.5 * (d[hi - 1] - d[hi]);
        double ee = e[hi - 1];
        double den = dd + (dd >= 0 ? 1.0 : -1.0) * std::hypot(dd, ee);
        double mu = d[hi] - (den != 0.0 ? ee * ee / den : 0.0);
        double x = d[lo] - mu, z = e[lo];
        for (int k = lo; k < hi; ++k) {
            double r = std::hypot(x, z);
            double c = r == 0.0 ? 1.0 : x / r, s = r == 0.0 ? 0.0 : -z / r;
            // apply G(k,k+1,c,s)^T T G to the tridiagonal
            if (k > lo) e[k - 1] = c * e[k - 1] - s * z;
            double d0 = d[k], d1 = d[k + 1], e0 = e[k];
            d[k] = c * c * d0 - 2 * c * s * e0 + s * s * d1;
            d[k + 1] = s * s * d0 + 2 * c * s * e0 + c * c * d1;
            e[k] = c * s * (d0 - d1) + (c * c - s * s) * e0;
            if (k + 1 < hi) {
                z = -s * e[k + 1];
                e[k + 1] = c * e[k + 1];
                x = e[k];
            }
            // accumulate Q = Q G
            for (int i = 0; i < n; ++i) {
                double q0 = Q[(size_t)i * n + k], q1 = Q[(size_t)i * n + k + 1];
                Q[(size_t)i * n + k] = c * q0 - s * q1;
                Q[(size_t)i * n + k + 1] = s * q0 + c * q1;
            }
        }
        ++iter;
    }
    // sort ascending
    std::vector<int> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return d[a] < d[b]; });
    for (int j = 0; j < n; ++j) {
        wout[j] = d[idx[j]];
        for (int i = 0; i < n; ++i) Vout[(size_t)i * n + j] = Q[(size_t)i * n + idx[j]];
    }
}

void solve_full_piv(int n, const double* Ain, const double* b, double* x)
{
    std::vector<double> A(Ain, Ain + (size_t)n * n), r(b, b + n);
    std::vector<int> colp(n);
    std::iota(colp.begin(), colp.end(), 0);
    int rank = n;
    double maxpiv = 0.0;
    const double thr = 2.220446049250313e-16 * n;  // Eigen FullPivLU default threshold
    for (int k = 0; k < n; ++k) {
        int pi = k, pj = k;
        double best = -1.0;
        for (int i = k; i < n; ++i)
            for (int j = k; j < n; ++j)
                if (std::fabs(A[(size_t)i * n + j]) > best) {
                    best = std::fabs(A[(size_t)i * n + j]);
                    pi = i;
                    pj = j;
                }
        if (k == 0) maxpiv = best;
        if (best <= 0.0 || best <= thr * maxpiv) {
            rank = k;
            break;
        }
        if (pi != k) {
            for (int j = 0; j < n; ++j) std::swap(A[(size_t)pi * n + j], A[(size_t)k * n + j]);
            std::swap(r[pi], r[k]);
        }
        if (pj != k) {
            for (int i = 0; i < n; ++i) std::swap(A[(size_t)i * n + pj], A[(size_t)i * n + k]);
            std::swap(colp[pj], colp[k]);
        }
        double piv = A[(size_t)k * n + k];
        for (int i = k + 1; i < n; ++i) {
            double f = A[(size_t)i * n + k] / piv;
            if (f == 0.0) continue;
            for (int j = k; j < n; ++j) A[(size_t)i * n + j] -= f * A[(size_t)k * n + j];
            r[i] -= f * r[k];
        }
    }
    // back substitution on the leading rank x rank block; free variables = 0
    std::vector<double> y(n, 0.0);
    for (int i = rank - 1; i >= 0; --i) {
        double s = r[i];
        for (int j = i + 1; j < rank; ++j) s -= A[(size_t)i * n + j] * y[j];
        y[i] = s / A[(size_t)i * n + i];
    }
    for (int j = 0; j < n; ++j) x[colp[j]] = y[j];
}

}  // namespace hfx
