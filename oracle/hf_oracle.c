/*
 * hf_oracle.c -- CPU restatement of the reference's integral and Fock-build
 * algorithms (KLYYCYNN/hartree_fock_cpp).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: tests/, the smoke check
 * and bench.py's CPU-baseline leg load it as the checker (or, for the
 * baseline, as the timed CPU implementation).  Nothing in the engine
 * (hartree_fock_cpp_gb300/) links, loads or calls it.
 *
 * It follows the reference line by line, including its inefficiencies, so
 * that its outputs and its cost both stand for the reference's CPU path:
 *   boys                -> include/integrals.hpp:223-266  (series for T<1e-4,
 *                          else erf + UPWARD recursion)
 *   hermite_E_array     -> include/integrals.hpp:269-322
 *   packed_r_index_cpu  -> include/integrals.hpp:343-358
 *   coulomb_R           -> include/integrals.hpp:541-618  (full recursion per
 *                          requested (t,u,v))
 *   coulomb_R_attraction-> include/integrals.hpp:362-439
 *   primitive_repulsion -> include/integrals.hpp:624-699
 *   basis_repulsion     -> include/integrals.hpp:701-729
 *   schwarz_bounds      -> include/integrals.hpp:732-752
 *   repulsion_tensor    -> include/integrals.hpp:754-787
 *   overlap/kinetic/attraction matrices -> include/integrals.hpp:10-536
 *   pair_index/eri_index/quartet_to_pairs/pair_to_indices
 *                       -> include/indexing.hpp:33-85
 *   repulsion_matrix    -> include/linalg.hpp:100-129
 *   coulomb_matrix      -> include/linalg.hpp:215-257
 *   exchange_matrix     -> include/linalg.hpp:260-296
 *
 * One deliberate addition: a switchable accurate Boys function
 * (orc_set_stable_boys(1)), so that per-ERI parity can be split into "the
 * reference's algorithm" and "the reference's algorithm with an accurate
 * F_m(T)" -- the reference's upward recursion loses digits for moderate T and
 * large m.
 *
 * Basis functions are passed flat, one record per basis function in the
 * reference's order (atoms -> CSV shells -> angmom_partition components):
 * centre, (lx,ly,lz), and a primitive range into alpha/coeff/norm arrays.
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stddef.h>
#include <pthread.h>

typedef struct {
    int K;                 /* number of basis functions */
    const double *cx, *cy, *cz;   /* centres, K each */
    const int *lmn;        /* 3*K: lx, ly, lz */
    const int *prim_off;   /* K+1 offsets into the primitive arrays */
    const double *alpha, *coeff, *norm;
} orc_basis;

static int g_stable_boys = 0;

void orc_set_stable_boys(int on) { g_stable_boys = on; }

/* integrals.hpp:223-266 */
static double boys_reference(int m, double T)
{
    if (T < 1e-4) {
        double term = 1.0, sum = 0.0;
        for (int k = 0; k < 50; ++k) {
            double add = term / (2.0 * m + 2.0 * k + 1.0);
            sum += add;
            double s = fabs(sum) > 1.0 ? fabs(sum) : 1.0;
            if (fabs(add) < 1e-16 * s) break;
            term *= -T / (double)(k + 1);
        }
        return sum;
    }
    const double PI = 3.141592653589793238462643383279502884;
    double sqrtT = sqrt(T);
    double F = 0.5 * sqrt(PI / T) * erf(sqrtT);
    double expT = exp(-T);
    for (int k = 0; k < m; ++k) F = ((2.0 * k + 1.0) * F - expT) / (2.0 * T);
    return F;
}

/* Accurate F_m(T): the all-positive series
 *   F_m(T) = exp(-T) * sum_k (2T)^k / ((2m+1)(2m+3)...(2m+2k+1))
 * for T <= 50, the asymptotic form with upward recursion beyond (where the
 * recursion is stable and erf(sqrt T) = 1 to double precision). */
static double boys_stable(int m, double T)
{
    if (T <= 50.0) {
        double term = 1.0 / (2.0 * m + 1.0), sum = term;
        for (int k = 1; k < 400; ++k) {
            term *= 2.0 * T / (2.0 * m + 2.0 * k + 1.0);
            sum += term;
            if (term < 1e-18 * sum) break;
        }
        return exp(-T) * sum;
    }
    const double PI = 3.141592653589793238462643383279502884;
    double F = 0.5 * sqrt(PI / T);
    double expT = exp(-T);
    for (int k = 0; k < m; ++k) F = ((2.0 * k + 1.0) * F - expT) / (2.0 * T);
    return F;
}

double orc_boys(int m, double T)
{
    return g_stable_boys ? boys_stable(m, T) : boys_reference(m, T);
}

double orc_boys_reference(int m, double T) { return boys_reference(m, T); }
double orc_boys_stable(int m, double T) { return boys_stable(m, T); }

/* integrals.hpp:269-322 ; writes E^{ij}_t for t = 0..i+j into out */
#define MAX_L_CPU 4
#define MAX_E_CPU (2 * MAX_L_CPU + 1)
static int hermite_E_array(int i, int j, double alpha, double beta, double A, double B, double *out)
{
    if (i > MAX_L_CPU || j > MAX_L_CPU || i + j >= MAX_E_CPU) return -1;
    double E[MAX_L_CPU + 1][MAX_L_CPU + 1][MAX_E_CPU];
    memset(E, 0, sizeof(E));
    double p = alpha + beta;
    double q = alpha * beta / p;
    double AB = A - B;
    E[0][0][0] = exp(-q * AB * AB);
    for (int ia = 1; ia <= i; ++ia)
        for (int tt = 0; tt <= ia; ++tt) {
            double t1 = (tt > 0) ? E[ia - 1][0][tt - 1] / (2.0 * p) : 0.0;
            double t2 = -(beta / p) * AB * E[ia - 1][0][tt];
            double t3 = (tt + 1 < MAX_E_CPU) ? (tt + 1) * E[ia - 1][0][tt + 1] : 0.0;
            E[ia][0][tt] = t1 + t2 + t3;
        }
    for (int ia = 0; ia <= i; ++ia)
        for (int jb = 1; jb <= j; ++jb)
            for (int tt = 0; tt <= ia + jb; ++tt) {
                double t1 = (tt > 0) ? E[ia][jb - 1][tt - 1] / (2.0 * p) : 0.0;
                double t2 = +(alpha / p) * AB * E[ia][jb - 1][tt];
                double t3 = (tt + 1 < MAX_E_CPU) ? (tt + 1) * E[ia][jb - 1][tt + 1] : 0.0;
                E[ia][jb][tt] = t1 + t2 + t3;
            }
    for (int tt = 0; tt <= i + j; ++tt) out[tt] = E[i][j][tt];
    return 0;
}

/* integrals.hpp:325-358 */
#define MAX_R_ORDER 12
#define N_R ((MAX_R_ORDER + 1) * (MAX_R_ORDER + 2) * (MAX_R_ORDER + 3) / 6)

static int packed_r_index_cpu(int a, int b, int c)
{
    int s = a + b + c;
    int offset_s = s * (s + 1) * (s + 2) / 6;
    int offset_a = 0;
    for (int aa = 0; aa < a; ++aa) offset_a += (s - aa + 1);
    return offset_s + offset_a + b;
}

/* Shared body of coulomb_R (integrals.hpp:541-618) and coulomb_R_attraction
 * (integrals.hpp:362-439): the whole R^{(m)} recursion for one (t,u,v). */
static double coulomb_R_body(int tx, int ty, int tz, int n, double rho, double X, double Y, double Z)
{
    int max_order = tx + ty + tz + n;
    if (max_order > MAX_R_ORDER || tx < 0 || ty < 0 || tz < 0) return 0.0;
    double T = rho * (X * X + Y * Y + Z * Z);
    double *Rnext = (double *)calloc(N_R, sizeof(double));
    double *Rcurr = (double *)calloc(N_R, sizeof(double));
    Rnext[0] = pow(-2.0 * rho, max_order) * orc_boys(max_order, T);
    for (int m = max_order - 1; m >= n; --m) {
        memset(Rcurr, 0, N_R * sizeof(double));
        Rcurr[0] = pow(-2.0 * rho, m) * orc_boys(m, T);
        for (int s = 1; s <= tx + ty + tz; ++s)
            for (int a = 0; a <= s; ++a)
                for (int b = 0; b <= s - a; ++b) {
                    int c = s - a - b;
                    if (a > tx || b > ty || c > tz) continue;
                    double val = 0.0;
                    if (a > 0) {
                        val = X * Rnext[packed_r_index_cpu(a - 1, b, c)];
                        if (a >= 2) val += (a - 1) * Rnext[packed_r_index_cpu(a - 2, b, c)];
                    } else if (b > 0) {
                        val = Y * Rnext[packed_r_index_cpu(a, b - 1, c)];
                        if (b >= 2) val += (b - 1) * Rnext[packed_r_index_cpu(a, b - 2, c)];
                    } else if (c > 0) {
                        val = Z * Rnext[packed_r_index_cpu(a, b, c - 1)];
                        if (c >= 2) val += (c - 1) * Rnext[packed_r_index_cpu(a, b, c - 2)];
                    }
                    Rcurr[packed_r_index_cpu(a, b, c)] = val;
                }
        double *tmp = Rnext; Rnext = Rcurr; Rcurr = tmp;
    }
    double out = Rnext[packed_r_index_cpu(tx, ty, tz)];
    free(Rnext);
    free(Rcurr);
    return out;
}

/* integrals.hpp:624-699 */
static double primitive_repulsion(const orc_basis *bs, int f1, int f2, int f3, int f4,
                                  int i1, int i2, int i3, int i4)
{
    double Ax = bs->cx[f1], Ay = bs->cy[f1], Az = bs->cz[f1];
    double Bx = bs->cx[f2], By = bs->cy[f2], Bz = bs->cz[f2];
    double Cx = bs->cx[f3], Cy = bs->cy[f3], Cz = bs->cz[f3];
    double Dx = bs->cx[f4], Dy = bs->cy[f4], Dz = bs->cz[f4];
    double alpha = bs->alpha[i1], beta = bs->alpha[i2], gamma = bs->alpha[i3], delta = bs->alpha[i4];
    double p = alpha + beta, q = gamma + delta;
    double Px = (alpha * Ax + beta * Bx) / p, Py = (alpha * Ay + beta * By) / p, Pz = (alpha * Az + beta * Bz) / p;
    double Qx = (gamma * Cx + delta * Dx) / q, Qy = (gamma * Cy + delta * Dy) / q, Qz = (gamma * Cz + delta * Dz) / q;
    const int *l1 = bs->lmn + 3 * f1, *l2 = bs->lmn + 3 * f2, *l3 = bs->lmn + 3 * f3, *l4 = bs->lmn + 3 * f4;
    int t = l1[0] + l2[0], u = l1[1] + l2[1], v = l1[2] + l2[2];
    int tau = l3[0] + l4[0], nu = l3[1] + l4[1], phi = l3[2] + l4[2];
    double E1[MAX_E_CPU], E2[MAX_E_CPU], E3[MAX_E_CPU], E4[MAX_E_CPU], E5[MAX_E_CPU], E6[MAX_E_CPU];
    hermite_E_array(l1[0], l2[0], alpha, beta, Ax, Bx, E1);
    hermite_E_array(l1[1], l2[1], alpha, beta, Ay, By, E2);
    hermite_E_array(l1[2], l2[2], alpha, beta, Az, Bz, E3);
    hermite_E_array(l3[0], l4[0], gamma, delta, Cx, Dx, E4);
    hermite_E_array(l3[1], l4[1], gamma, delta, Cy, Dy, E5);
    hermite_E_array(l3[2], l4[2], gamma, delta, Cz, Dz, E6);
    double rho = p * q / (p + q);
    double X = Px - Qx, Y = Py - Qy, Z = Pz - Qz;
    double eri = 0.0;
    for (int ti = 0; ti <= t; ++ti)
        for (int ui = 0; ui <= u; ++ui)
            for (int vi = 0; vi <= v; ++vi)
                for (int taui = 0; taui <= tau; ++taui)
                    for (int nui = 0; nui <= nu; ++nui)
                        for (int phii = 0; phii <= phi; ++phii) {
                            double sign = ((taui + nui + phii) % 2 == 0) ? 1.0 : -1.0;
                            eri += sign * E1[ti] * E2[ui] * E3[vi] * E4[taui] * E5[nui] * E6[phii] *
                                   coulomb_R_body(ti + taui, ui + nui, vi + phii, 0, rho, X, Y, Z);
                        }
    return 2 * pow(M_PI, 2.5) * pow(p + q, -0.5) * eri / (p * q);
}

/* integrals.hpp:701-729 */
double orc_basis_repulsion(const orc_basis *bs, int f1, int f2, int f3, int f4)
{
    double eri = 0.0;
    for (int i = bs->prim_off[f1]; i < bs->prim_off[f1 + 1]; ++i)
        for (int j = bs->prim_off[f2]; j < bs->prim_off[f2 + 1]; ++j)
            for (int k = bs->prim_off[f3]; k < bs->prim_off[f3 + 1]; ++k)
                for (int l = bs->prim_off[f4]; l < bs->prim_off[f4 + 1]; ++l)
                    eri += bs->coeff[i] * bs->coeff[j] * bs->coeff[k] * bs->coeff[l] *
                           bs->norm[i] * bs->norm[j] * bs->norm[k] * bs->norm[l] *
                           primitive_repulsion(bs, f1, f2, f3, f4, i, j, k, l);
    return eri;
}

/* indexing.hpp:33-85 */
size_t orc_pair_index(int a, int b)
{
    if (a < b) { int t = a; a = b; b = t; }
    return (size_t)a * (a + 1) / 2 + b;
}

size_t orc_eri_index(int i, int j, int k, int l)
{
    size_t IJ = orc_pair_index(i, j), KL = orc_pair_index(k, l);
    if (IJ < KL) { size_t t = IJ; IJ = KL; KL = t; }
    return IJ * (IJ + 1) / 2 + KL;
}

static void quartet_to_pairs(size_t qid, int *p1, int *p2)
{
    int pid1 = (int)((sqrt(8.0 * (double)qid + 1.0) - 1.0) * 0.5);
    size_t tri = (size_t)pid1 * (pid1 + 1) / 2;
    if (tri > qid) { --pid1; tri = (size_t)pid1 * (pid1 + 1) / 2; }
    while ((size_t)(pid1 + 1) * (pid1 + 2) / 2 <= qid) { ++pid1; tri = (size_t)pid1 * (pid1 + 1) / 2; }
    *p1 = pid1;
    *p2 = (int)(qid - tri);
}

static void pair_to_indices(int pid, int *a, int *b)
{
    int x = (int)((sqrt(8.0 * pid + 1.0) - 1.0) / 2.0);
    *a = x;
    *b = pid - x * (x + 1) / 2;
}

/* integrals.hpp:732-752 */
void orc_schwarz_bounds(const orc_basis *bs, double *bounds)
{
    int n_pairs = bs->K * (bs->K + 1) / 2;
    for (int i = 0; i < n_pairs; ++i) {
        int a, b;
        pair_to_indices(i, &a, &b);
        double v = orc_basis_repulsion(bs, a, b, a, b);
        bounds[i] = sqrt(v > 0.0 ? v : 0.0);
    }
}

/* integrals.hpp:754-787, restricted to quartet ids [q_begin, q_end) so that a
 * caller can split the loop over threads or processes.  `bounds` is the
 * schwarz_bounds() array; out has n_quartets entries (only the range is
 * written). */
void orc_repulsion_tensor_range(const orc_basis *bs, const double *bounds, double threshold,
                                double *out, size_t q_begin, size_t q_end)
{
    for (size_t i = q_begin; i < q_end; ++i) {
        int p1, p2, a, b, c, d;
        quartet_to_pairs(i, &p1, &p2);
        pair_to_indices(p1, &a, &b);
        pair_to_indices(p2, &c, &d);
        if (bounds[p1] * bounds[p2] < threshold) { out[i] = 0.0; continue; }
        out[i] = orc_basis_repulsion(bs, a, b, c, d);
    }
}

void orc_repulsion_tensor(const orc_basis *bs, double threshold, double *out)
{
    size_t n_pairs = (size_t)bs->K * (bs->K + 1) / 2;
    size_t nq = n_pairs * (n_pairs + 1) / 2;
    double *bounds = (double *)malloc(n_pairs * sizeof(double));
    orc_schwarz_bounds(bs, bounds);
    orc_repulsion_tensor_range(bs, bounds, threshold, out, 0, nq);
    free(bounds);
}

/* Evaluate an explicit list of unique quartets (i,j,k,l); used to time and
 * check a seeded sample of a workload whose full tensor is too large. */
void orc_eri_list(const orc_basis *bs, const double *bounds, double threshold,
                  const int *ijkl, size_t n, double *out)
{
    for (size_t q = 0; q < n; ++q) {
        int i = ijkl[4 * q], j = ijkl[4 * q + 1], k = ijkl[4 * q + 2], l = ijkl[4 * q + 3];
        if (bounds && bounds[orc_pair_index(i, j)] * bounds[orc_pair_index(k, l)] < threshold) {
            out[q] = 0.0;
            continue;
        }
        out[q] = orc_basis_repulsion(bs, i, j, k, l);
    }
}

typedef struct {
    const orc_basis *bs;
    const double *bounds;
    double thr;
    const int *ijkl;
    size_t n;
    double *out;
} list_job;

static void *list_worker(void *arg)
{
    list_job *j = (list_job *)arg;
    orc_eri_list(j->bs, j->bounds, j->thr, j->ijkl, j->n, j->out);
    return NULL;
}

/* Same as orc_eri_list, split into contiguous chunks over nthreads POSIX
 * threads (the reference itself is single-threaded; this only spreads its
 * per-quartet loop over the host's cores). */
void orc_eri_list_mt(const orc_basis *bs, const double *bounds, double threshold,
                     const int *ijkl, size_t n, double *out, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    list_job *jobs = (list_job *)malloc(sizeof(list_job) * nthreads);
    size_t chunk = (n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; ++t) {
        size_t b = (size_t)t * chunk, e = b + chunk;
        if (b > n) b = n;
        if (e > n) e = n;
        jobs[t].bs = bs; jobs[t].bounds = bounds; jobs[t].thr = threshold;
        jobs[t].ijkl = ijkl + 4 * b; jobs[t].n = e - b; jobs[t].out = out + b;
        pthread_create(&th[t], NULL, list_worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    free(th);
    free(jobs);
}

/* ---------------- one-electron integrals (integrals.hpp:10-536) -------- */

/* integrals.hpp:13-54 */
static double overlap_1d(double alpha, double beta, int l, int m, double A, double B)
{
    if (l < 0 || m < 0) return 0.0;
    double p = alpha + beta;
    double mu = alpha * beta / p;
    double P = (alpha * A + beta * B) / p;
    if (l == 0 && m == 0) return sqrt(M_PI / p) * exp(-mu * (A - B) * (A - B));
    if (l > 0)
        return (P - A) * overlap_1d(alpha, beta, l - 1, m, A, B) +
               ((l - 1) / (2.0 * p)) * overlap_1d(alpha, beta, l - 2, m, A, B) +
               (m / (2.0 * p)) * overlap_1d(alpha, beta, l - 1, m - 1, A, B);
    return (P - B) * overlap_1d(alpha, beta, l, m - 1, A, B) +
           (l / (2.0 * p)) * overlap_1d(alpha, beta, l - 1, m - 1, A, B) +
           ((m - 1) / (2.0 * p)) * overlap_1d(alpha, beta, l, m - 2, A, B);
}

/* integrals.hpp:122-142 */
static double kinetic_1d(double alpha, double beta, int l, int m, double A, double B)
{
    double t1 = beta * (2 * m + 1) * overlap_1d(alpha, beta, l, m, A, B);
    double t2 = -2 * beta * beta * overlap_1d(alpha, beta, l, m + 2, A, B);
    double t3 = -0.5 * m * (m - 1) * overlap_1d(alpha, beta, l, m - 2, A, B);
    return t1 + t2 + t3;
}

/* integrals.hpp:56-118 (overlap) and 144-218 (kinetic), full K x K, row-major */
void orc_overlap_kinetic(const orc_basis *bs, double *S, double *T)
{
    int K = bs->K;
    for (int a = 0; a < K; ++a)
        for (int b = 0; b <= a; ++b) {
            const int *la = bs->lmn + 3 * a, *lb = bs->lmn + 3 * b;
            double s = 0.0, t = 0.0;
            double A[3] = {bs->cx[a], bs->cy[a], bs->cz[a]}, B[3] = {bs->cx[b], bs->cy[b], bs->cz[b]};
            for (int i = bs->prim_off[a]; i < bs->prim_off[a + 1]; ++i)
                for (int j = bs->prim_off[b]; j < bs->prim_off[b + 1]; ++j) {
                    double al = bs->alpha[i], be = bs->alpha[j];
                    double nrm = bs->norm[i] * bs->norm[j];
                    double Sx = overlap_1d(al, be, la[0], lb[0], A[0], B[0]);
                    double Sy = overlap_1d(al, be, la[1], lb[1], A[1], B[1]);
                    double Sz = overlap_1d(al, be, la[2], lb[2], A[2], B[2]);
                    s += bs->coeff[i] * bs->coeff[j] * nrm * Sx * Sy * Sz;
                    double t1 = kinetic_1d(al, be, la[0], lb[0], A[0], B[0]) * Sy * Sz;
                    double t2 = kinetic_1d(al, be, la[1], lb[1], A[1], B[1]) * Sx * Sz;
                    double t3 = kinetic_1d(al, be, la[2], lb[2], A[2], B[2]) * Sy * Sx;
                    t += bs->coeff[i] * bs->coeff[j] * nrm * (t1 + t2 + t3);
                }
            S[a * K + b] = S[b * K + a] = s;
            T[a * K + b] = T[b * K + a] = t;
        }
}

/* integrals.hpp:443-536 ; atoms: natom charges Z and positions xyz */
void orc_attraction(const orc_basis *bs, int natom, const int *Z, const double *xyz, double *V)
{
    int K = bs->K;
    for (int a = 0; a < K; ++a)
        for (int b = 0; b <= a; ++b) {
            const int *la = bs->lmn + 3 * a, *lb = bs->lmn + 3 * b;
            double A[3] = {bs->cx[a], bs->cy[a], bs->cz[a]}, B[3] = {bs->cx[b], bs->cy[b], bs->cz[b]};
            double v = 0.0;
            for (int i = bs->prim_off[a]; i < bs->prim_off[a + 1]; ++i)
                for (int j = bs->prim_off[b]; j < bs->prim_off[b + 1]; ++j)
                    for (int n = 0; n < natom; ++n) {
                        double al = bs->alpha[i], be = bs->alpha[j];
                        double p = al + be;
                        double P[3];
                        for (int x = 0; x < 3; ++x) P[x] = (al * A[x] + be * B[x]) / p;
                        double E1[MAX_E_CPU], E2[MAX_E_CPU], E3[MAX_E_CPU];
                        hermite_E_array(la[0], lb[0], al, be, A[0], B[0], E1);
                        hermite_E_array(la[1], lb[1], al, be, A[1], B[1], E2);
                        hermite_E_array(la[2], lb[2], al, be, A[2], B[2], E3);
                        double X = P[0] - xyz[3 * n], Y = P[1] - xyz[3 * n + 1], Zc = P[2] - xyz[3 * n + 2];
                        double val = 0.0;
                        for (int t = 0; t <= la[0] + lb[0]; ++t)
                            for (int u = 0; u <= la[1] + lb[1]; ++u)
                                for (int w = 0; w <= la[2] + lb[2]; ++w)
                                    val += E1[t] * E2[u] * E3[w] * coulomb_R_body(t, u, w, 0, p, X, Y, Zc);
                        double prim = -(2 * M_PI / p) * bs->norm[i] * bs->norm[j] * Z[n] * val;
                        v += bs->coeff[i] * bs->coeff[j] * prim;
                    }
            V[a * K + b] = V[b * K + a] = v;
        }
}

/* ---------------- Fock contractions (linalg.hpp) ------------------------ */

/* linalg.hpp:100-129 : G_ij = sum_kl P_kl [(ij|kl) - 1/2 (ik|jl)] */
void orc_repulsion_matrix(int K, const double *P, const double *eri, double *G)
{
    for (int i = 0; i < K; ++i)
        for (int j = 0; j < K; ++j) {
            double g = 0.0;
            for (int k = 0; k < K; ++k)
                for (int l = 0; l < K; ++l) {
                    double J = P[k * K + l] * eri[orc_eri_index(i, j, k, l)];
                    double Kx = P[k * K + l] * eri[orc_eri_index(i, k, j, l)];
                    g += J - 0.5 * Kx;
                }
            G[i * K + j] = g;
        }
}

/* linalg.hpp:215-257 */
void orc_coulomb_matrix(int K, const double *P1, const double *P2, const double *eri, double *J)
{
    for (int i = 0; i < K; ++i)
        for (int j = 0; j < K; ++j) {
            double s = 0.0;
            for (int k = 0; k < K; ++k)
                for (int l = 0; l < K; ++l)
                    s += (P1[k * K + l] + P2[k * K + l]) * eri[orc_eri_index(i, j, k, l)];
            J[i * K + j] = s;
        }
}

/* linalg.hpp:260-296 */
void orc_exchange_matrix(int K, const double *P, const double *eri, double *Kx)
{
    for (int i = 0; i < K; ++i)
        for (int j = 0; j < K; ++j) {
            double s = 0.0;
            for (int k = 0; k < K; ++k)
                for (int l = 0; l < K; ++l) s += P[k * K + l] * eri[orc_eri_index(i, k, j, l)];
            Kx[i * K + j] = s;
        }
}

/* ---------------- threaded drivers (fixture generation) -----------------
 * The reference is single-threaded; these only spread its loops over host
 * threads.  Every output element is computed by exactly the code above, in
 * the same order, so the results are bit-identical to the serial functions. */

typedef struct {
    const orc_basis *bs;
    const double *bounds;
    double thr;
    double *out;
    size_t nq;
    size_t *next;          /* shared block counter */
    int K;
    const double *P1, *P2, *eri;
    int kind;              /* 0 tensor, 1 repulsion, 2 coulomb, 3 exchange, 4 schwarz */
    size_t block;          /* items per claimed task */
} mt_job;

static void *mt_worker(void *arg)
{
    mt_job *j = (mt_job *)arg;
    for (;;) {
        size_t b = __atomic_fetch_add(j->next, j->block, __ATOMIC_RELAXED);
        if (b >= j->nq) break;
        size_t e = b + j->block < j->nq ? b + j->block : j->nq;
        if (j->kind == 0) {
            orc_repulsion_tensor_range(j->bs, j->bounds, j->thr, j->out, b, e);
        } else if (j->kind == 4) {
            for (size_t p = b; p < e; ++p) {
                int a, c;
                pair_to_indices((int)p, &a, &c);
                double v = orc_basis_repulsion(j->bs, a, c, a, c);
                j->out[p] = sqrt(v > 0.0 ? v : 0.0);
            }
        } else {
            int K = j->K;
            for (size_t r = b; r < e; ++r) {           /* r = i*K + j, one output element */
                int i = (int)(r / K), jj = (int)(r % K);
                double s = 0.0;
                for (int k = 0; k < K; ++k)
                    for (int l = 0; l < K; ++l) {
                        if (j->kind == 1) {
                            double Jv = j->P1[k * K + l] * j->eri[orc_eri_index(i, jj, k, l)];
                            double Kv = j->P1[k * K + l] * j->eri[orc_eri_index(i, k, jj, l)];
                            s += Jv - 0.5 * Kv;
                        } else if (j->kind == 2) {
                            s += (j->P1[k * K + l] + j->P2[k * K + l]) * j->eri[orc_eri_index(i, jj, k, l)];
                        } else {
                            s += j->P1[k * K + l] * j->eri[orc_eri_index(i, k, jj, l)];
                        }
                    }
                j->out[r] = s;
            }
        }
    }
    return NULL;
}

static void mt_run(mt_job *proto, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    size_t next = 0;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    mt_job *jobs = (mt_job *)malloc(sizeof(mt_job) * nthreads);
    for (int t = 0; t < nthreads; ++t) {
        jobs[t] = *proto;
        jobs[t].next = &next;
        pthread_create(&th[t], NULL, mt_worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    free(th);
    free(jobs);
}

/* schwarz_bounds + repulsion_tensor (integrals.hpp:732-787) over nthreads */
void orc_repulsion_tensor_mt(const orc_basis *bs, double threshold, double *out, int nthreads)
{
    size_t n_pairs = (size_t)bs->K * (bs->K + 1) / 2;
    double *bounds = (double *)malloc(n_pairs * sizeof(double));
    mt_job j;
    memset(&j, 0, sizeof j);
    j.bs = bs; j.out = bounds; j.nq = n_pairs; j.kind = 4; j.block = 8;
    mt_run(&j, nthreads);
    memset(&j, 0, sizeof j);
    j.bs = bs; j.bounds = bounds; j.thr = threshold; j.out = out; j.nq = n_pairs * (n_pairs + 1) / 2; j.kind = 0; j.block = 1024;
    mt_run(&j, nthreads);
    free(bounds);
}

/* linalg.hpp:100-129 / 215-257 / 260-296 over nthreads (one output element per task) */
void orc_contract_mt(int kind, int K, const double *P1, const double *P2, const double *eri, double *out,
                     int nthreads)
{
    mt_job j;
    memset(&j, 0, sizeof j);
    j.K = K; j.P1 = P1; j.P2 = P2; j.eri = eri; j.out = out; j.nq = (size_t)K * K; j.kind = kind; j.block = 4;
    mt_run(&j, nthreads);
}
