// hfx_scf.cpp -- RHF / UHF DIIS drivers with the reference's semantics
// (include/scf.hpp:205-419 rhf_diis, :423-682 uhf_diis): zero (or given)
// initial density, damping for the first start_diis-1 iterations, Pulay DIIS
// over the last max_history Fock / FPS-SPF error pairs from iteration
// start_diis, symmetric orthogonalisation X = S^{-1/2}, convergence when
// RMSD(P) < eps and ||FPS-SPF|| < eps followed by the same final check.
// The only change of substance: the two-electron matrix comes from the
// direct GPU Fock build instead of a stored ERI tensor.
#include <chrono>
#include <cmath>
#include <deque>
#include <functional>
#include <vector>

#include "hfx_engine.hpp"
#include "hfx_scf.hpp"

namespace hfx {

static double rmsd(const std::vector<double>& a, const std::vector<double>& b)
{
    double s = 0.0;
    for (size_t i = 0; i < a.size(); ++i) s += (a[i] - b[i]) * (a[i] - b[i]);
    return std::sqrt(s / a.size());
}

static double norm2(const std::vector<double>& a)
{
    double s = 0.0;
    for (double x : a) s += x * x;
    return std::sqrt(s);
}

// F P S - S P F (linalg.hpp:355-379)
static std::vector<double> error_matrix(int K, const std::vector<double>& P, const std::vector<double>& F,
                                        const std::vector<double>& S)
{
    std::vector<double> FP(K * K), FPS(K * K), SP(K * K), SPF(K * K);
    matmul(K, F.data(), P.data(), FP.data());
    matmul(K, FP.data(), S.data(), FPS.data());
    matmul(K, S.data(), P.data(), SP.data());
    matmul(K, SP.data(), F.data(), SPF.data());
    for (int i = 0; i < K * K; ++i) FPS[i] -= SPF[i];
    return FPS;
}

// scf.hpp:28-39
static double energy(const std::vector<double>& P, const std::vector<double>& F, const std::vector<double>& H)
{
    double E = 0.0;
    for (size_t i = 0; i < P.size(); ++i) E += P[i] * (H[i] + F[i]);
    return 0.5 * E;
}

// linalg.hpp:405-510: augmented Pulay matrix, fullPivLu solve, combination
static std::vector<double> fock_diis(const std::deque<std::vector<double>>& fh,
                                     const std::deque<std::vector<double>>& eh)
{
    int n = (int)eh.size();
    std::vector<double> B((n + 1) * (n + 1), 0.0), rhs(n + 1, 0.0), x(n + 1);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            double s = 0.0;
            for (size_t k = 0; k < eh[i].size(); ++k) s += eh[i][k] * eh[j][k];
            B[i * (n + 1) + j] = s;
        }
    for (int i = 0; i < n; ++i) {
        B[i * (n + 1) + n] = -1.0;
        B[n * (n + 1) + i] = 1.0;
    }
    rhs[n] = 1.0;
    solve_full_piv(n + 1, B.data(), rhs.data(), x.data());
    std::vector<double> F(fh[0].size(), 0.0);
    for (int i = 0; i < n; ++i)
        for (size_t k = 0; k < F.size(); ++k) F[k] += x[i] * fh[i][k];
    return F;
}

// X = S^{-1/2} (linalg.hpp:132-147)
static std::vector<double> xmatrix(int K, const std::vector<double>& S)
{
    std::vector<double> w(K), U(K * K), X(K * K, 0.0), rs(K);
    sym_eig(K, S.data(), w.data(), U.data());
    for (int k = 0; k < K; ++k) rs[k] = 1.0 / std::sqrt(w[k]);
    for (int i = 0; i < K; ++i)
        for (int j = 0; j < K; ++j) {
            double s = 0.0;
            for (int k = 0; k < K; ++k) s += U[i * K + k] * rs[k] * U[j * K + k];
            X[i * K + j] = s;
        }
    return X;
}

// EigProblem (linalg.hpp:150-170): C = X C', eigenvalues ascending
static void eig_problem(int K, const std::vector<double>& F, const std::vector<double>& X, std::vector<double>& C,
                        std::vector<double>& e)
{
    std::vector<double> FX(K * K), Fp(K * K), Cp(K * K);
    matmul(K, F.data(), X.data(), FX.data());
    matmul_tn(K, X.data(), FX.data(), Fp.data());
    e.resize(K);
    sym_eig(K, Fp.data(), e.data(), Cp.data());
    C.resize(K * K);
    matmul(K, X.data(), Cp.data(), C.data());
}

static std::vector<double> density(int K, const std::vector<double>& C, int nocc, double f)
{
    std::vector<double> P(K * K, 0.0);
    for (int i = 0; i < K; ++i)
        for (int j = 0; j < K; ++j) {
            double s = 0.0;
            for (int k = 0; k < nocc; ++k) s += C[i * K + k] * C[j * K + k];
            P[i * K + j] = f * s;
        }
    return P;
}

static void push_hist(std::deque<std::vector<double>>& h, const std::vector<double>& m, int maxh)
{
    if ((int)h.size() == maxh) h.pop_front();
    h.push_back(m);
}

static void fill_defaults(hfx_scf_options& o)
{
    if (o.max_iterations <= 0) o.max_iterations = 10000;
    if (o.epsilon <= 0) o.epsilon = 1e-6;
    if (o.damping <= 0) o.damping = 0.3;
    if (o.screening_threshold == 0) o.screening_threshold = 1e-8;
    if (o.start_diis <= 0) o.start_diis = 4;
    if (o.max_history <= 0) o.max_history = 8;
}

static bool finite_all(const std::vector<double>& v)
{
    for (double x : v)
        if (!std::isfinite(x)) return false;
    return true;
}

ScfSetup scf_setup(const Basis& b, bool gpu)
{
    ScfSetup s;
    int K = b.K;
    s.K = K;
    std::vector<double> T, V;
    if (gpu)
        one_electron_gpu(b, s.S, T, V);
    else
        one_electron(b, s.S, T, V);
    s.H.resize((size_t)K * K);
    for (int i = 0; i < K * K; ++i) s.H[i] = T[i] + V[i];
    s.E_nuc = nuclear_repulsion(b);
    s.X = xmatrix(K, s.S);
    return s;
}

ScfOutput rhf_diis(const Basis& b, const hfx_scf_options& opt, const double* P0, const GBuilder& g)
{
    return rhf_diis(b, scf_setup(b), opt, P0, g);
}

ScfOutput uhf_diis(const Basis& b, const hfx_scf_options& opt, int na, int nb, const double* Pa0, const double* Pb0,
                   const JKBuilder& jk)
{
    return uhf_diis(b, scf_setup(b), opt, na, nb, Pa0, Pb0, jk);
}

ScfOutput rhf_diis(const Basis& b, const ScfSetup& setup, const hfx_scf_options& opt_in, const double* P0,
                   const GBuilder& gbuild)
{
    auto t0 = std::chrono::steady_clock::now();
    hfx_scf_options opt = opt_in;
    fill_defaults(opt);
    int K = b.K;
    int n_e = -opt.charge;
    for (int z : b.atom_Z) n_e += z;
    const std::vector<double>& S = setup.S;
    const std::vector<double>& H = setup.H;
    const std::vector<double>& X = setup.X;
    double E_nuc = setup.E_nuc;
    std::vector<double> P(K * K, 0.0);
    if (P0) P.assign(P0, P0 + K * K);
    std::deque<std::vector<double>> fh, eh;
    ScfOutput out;
    out.K = K;
    out.n_electrons = n_e;
    out.E_nuc = E_nuc;
    std::vector<double> G(K * K), C, e;
    // Mixed precision: FP32/FP64 builds until the density settles, then one
    // full FP64 build and FP64 builds of the density change from there on
    // (G_n = G_{n-1} + G[P_n - P_{n-1}]), so the converged energy carries FP64
    // accuracy while most builds run mostly in FP32.
    const bool mixed = opt.precision == HFX_PREC_MIXED;
    int phase = mixed ? 0 : 2;          // 0 mixed, 1 next build full FP64, 2 plain / incremental FP64
    bool have_ref = false;
    std::vector<double> G_ref, P_ref, dP(K * K), dG(K * K);
    auto build = [&](const std::vector<double>& Pm, std::vector<double>& Gm) {
        ++out.fock_builds;
        if (!mixed) {
            gbuild(Pm.data(), Gm.data(), BUILD_DEFAULT);
            ++out.fp64_builds;
            return;
        }
        if (phase == 0) {
            gbuild(Pm.data(), Gm.data(), BUILD_DEFAULT);
            ++out.mixed_builds;
            return;
        }
        if (phase == 1 || !have_ref || opt.fp64_final_cycles < 0) {
            gbuild(Pm.data(), Gm.data(), BUILD_FP64);
            ++out.fp64_builds;
            if (opt.fp64_final_cycles >= 0) {
                G_ref = Gm;
                P_ref = Pm;
                have_ref = true;
                phase = 2;
            }
            return;
        }
        for (int i = 0; i < K * K; ++i) dP[i] = Pm[i] - P_ref[i];
        gbuild(dP.data(), dG.data(), BUILD_FP64_DELTA);
        ++out.delta_builds;
        for (int i = 0; i < K * K; ++i) Gm[i] = G_ref[i] + dG[i];
        G_ref = Gm;
        P_ref = Pm;
    };
    MixedPhaseSwitch to_fp64(opt.epsilon);
    int n_it = 0;
    for (int it = 0; it < opt.max_iterations; ++it) {
        ++n_it;
        build(P, G);
        std::vector<double> F(K * K);
        for (int i = 0; i < K * K; ++i) F[i] = H[i] + G[i];
        if (!finite_all(F)) throw Error(HFX_ERR_NUMERIC, "non-finite Fock matrix");
        std::vector<double> err = error_matrix(K, P, F, S);
        push_hist(fh, F, opt.max_history);
        push_hist(eh, err, opt.max_history);
        double E_cur = energy(P, F, H);
        if (n_it >= opt.start_diis) F = fock_diis(fh, eh);
        eig_problem(K, F, X, C, e);
        std::vector<double> Pn = density(K, C, n_e / 2, 2.0);
        double Pd = rmsd(Pn, P);
        double en = norm2(err);
        bool dE_ok = opt.energy_threshold <= 0 || (n_it > 1 && std::fabs(E_cur - out.E_prev) < opt.energy_threshold);
        out.E_prev = E_cur;
        out.last_rmsd = Pd;
        if (phase == 0 && to_fp64.update(Pd, en)) phase = 1;
        if (Pd < opt.epsilon && en < opt.epsilon && dE_ok && phase != 0) {
            // rhf_final_check (scf.hpp:107-137)
            build(Pn, G);
            std::vector<double> Ff(K * K);
            for (int i = 0; i < K * K; ++i) Ff[i] = H[i] + G[i];
            double fe = norm2(error_matrix(K, Pn, Ff, S));
            if (fe < opt.epsilon) {
                out.converged = true;
                P = Pn;
                out.E_ele = energy(Pn, Ff, H);
                out.E_tot = E_nuc + out.E_ele;
                break;
            }
        }
        if (n_it >= opt.start_diis) {
            P = Pn;
        } else {
            for (int i = 0; i < K * K; ++i) P[i] = opt.damping * Pn[i] + (1 - opt.damping) * P[i];
        }
        if (it == opt.max_iterations - 1) {
            if (phase == 0) phase = 1;
            build(P, G);
            std::vector<double> Ff(K * K);
            for (int i = 0; i < K * K; ++i) Ff[i] = H[i] + G[i];
            out.E_ele = energy(P, Ff, H);
            out.E_tot = E_nuc + out.E_ele;
        }
    }
    out.iterations = n_it;
    out.P = P;
    out.C = C;
    out.e = e;
    if (!std::isfinite(out.E_tot)) throw Error(HFX_ERR_NUMERIC, "non-finite SCF energy");
    out.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return out;
}

ScfOutput uhf_diis(const Basis& b, const ScfSetup& setup, const hfx_scf_options& opt_in, int na, int nb,
                   const double* Pa0, const double* Pb0, const JKBuilder& jk)
{
    auto t0 = std::chrono::steady_clock::now();
    hfx_scf_options opt = opt_in;
    fill_defaults(opt);
    int K = b.K;
    int n_e = -opt.charge;
    for (int z : b.atom_Z) n_e += z;
    if (n_e != na + nb) throw Error(HFX_ERR_INVALID, "inconsistency in electron number");
    const std::vector<double>& S = setup.S;
    const std::vector<double>& H = setup.H;
    const std::vector<double>& X = setup.X;
    double E_nuc = setup.E_nuc;
    std::vector<double> Pa(K * K, 0.0), Pb(K * K, 0.0);
    if (Pa0) Pa.assign(Pa0, Pa0 + K * K);
    if (Pb0) Pb.assign(Pb0, Pb0 + K * K);
    std::deque<std::vector<double>> fh, eh;
    ScfOutput out;
    out.K = K;
    out.n_electrons = n_e;
    out.E_nuc = E_nuc;
    std::vector<double> J(K * K), Ka(K * K), Kb(K * K), Ca, Cb, Ea, Eb;
    const bool mixed = opt.precision == HFX_PREC_MIXED;
    int phase = mixed ? 0 : 2;
    bool have_ref = false;
    std::vector<double> Jr, Kar, Kbr, Par, Pbr, dPa(K * K), dPb(K * K), dJ(K * K), dKa(K * K), dKb(K * K);
    auto build = [&](const std::vector<double>& A, const std::vector<double>& B) {
        ++out.fock_builds;
        if (!mixed) {
            jk(A.data(), B.data(), J.data(), Ka.data(), Kb.data(), BUILD_DEFAULT);
            ++out.fp64_builds;
            return;
        }
        if (phase == 0) {
            jk(A.data(), B.data(), J.data(), Ka.data(), Kb.data(), BUILD_DEFAULT);
            ++out.mixed_builds;
            return;
        }
        if (phase == 1 || !have_ref || opt.fp64_final_cycles < 0) {
            jk(A.data(), B.data(), J.data(), Ka.data(), Kb.data(), BUILD_FP64);
            ++out.fp64_builds;
            if (opt.fp64_final_cycles >= 0) {
                Jr = J;
                Kar = Ka;
                Kbr = Kb;
                Par = A;
                Pbr = B;
                have_ref = true;
                phase = 2;
            }
            return;
        }
        for (int i = 0; i < K * K; ++i) {
            dPa[i] = A[i] - Par[i];
            dPb[i] = B[i] - Pbr[i];
        }
        jk(dPa.data(), dPb.data(), dJ.data(), dKa.data(), dKb.data(), BUILD_FP64_DELTA);
        ++out.delta_builds;
        for (int i = 0; i < K * K; ++i) {
            J[i] = Jr[i] + dJ[i];
            Ka[i] = Kar[i] + dKa[i];
            Kb[i] = Kbr[i] + dKb[i];
        }
        Jr = J;
        Kar = Ka;
        Kbr = Kb;
        Par = A;
        Pbr = B;
    };
    MixedPhaseSwitch to_fp64(opt.epsilon);
    int n_it = 0;
    for (int it = 0; it < opt.max_iterations; ++it) {
        ++n_it;
        build(Pa, Pb);
        std::vector<double> Fa(K * K), Fb(K * K);
        for (int i = 0; i < K * K; ++i) {
            Fa[i] = H[i] + J[i] - Ka[i];
            Fb[i] = H[i] + J[i] - Kb[i];
        }
        if (!finite_all(Fa) || !finite_all(Fb)) throw Error(HFX_ERR_NUMERIC, "non-finite Fock matrix");
        std::vector<double> Ra = error_matrix(K, Pa, Fa, S), Rb = error_matrix(K, Pb, Fb, S);
        std::vector<double> tf = Fa, ev = Ra;
        tf.insert(tf.end(), Fb.begin(), Fb.end());
        ev.insert(ev.end(), Rb.begin(), Rb.end());
        push_hist(fh, tf, opt.max_history);
        push_hist(eh, ev, opt.max_history);
        double E_cur = energy(Pa, Fa, H) + energy(Pb, Fb, H);
        if (n_it >= opt.start_diis) {
            std::vector<double> Fd = fock_diis(fh, eh);
            Fa.assign(Fd.begin(), Fd.begin() + K * K);
            Fb.assign(Fd.begin() + K * K, Fd.end());
        }
        eig_problem(K, Fa, X, Ca, Ea);
        eig_problem(K, Fb, X, Cb, Eb);
        std::vector<double> Pan = density(K, Ca, na, 1.0), Pbn = density(K, Cb, nb, 1.0);
        double da = rmsd(Pa, Pan), db = rmsd(Pb, Pbn), en = norm2(ev);
        bool dE_ok = opt.energy_threshold <= 0 || (n_it > 1 && std::fabs(E_cur - out.E_prev) < opt.energy_threshold);
        out.E_prev = E_cur;
        out.last_rmsd = std::max(da, db);
        if (phase == 0 && to_fp64.update(std::max(da, db), en)) phase = 1;
        if (da < opt.epsilon && db < opt.epsilon && en < opt.epsilon && dE_ok && phase != 0) {
            // uhf_final_check (scf.hpp:140-185)
            build(Pan, Pbn);
            std::vector<double> Faf(K * K), Fbf(K * K);
            for (int i = 0; i < K * K; ++i) {
                Faf[i] = H[i] + J[i] - Ka[i];
                Fbf[i] = H[i] + J[i] - Kb[i];
            }
            double ea = norm2(error_matrix(K, Pan, Faf, S)), eb = norm2(error_matrix(K, Pbn, Fbf, S));
            if (std::sqrt(ea * ea + eb * eb) < opt.epsilon) {
                out.converged = true;
                out.E_ele = energy(Pan, Faf, H) + energy(Pbn, Fbf, H);
                out.E_tot = E_nuc + out.E_ele;
                Pa = Pan;
                Pb = Pbn;
                break;
            }
        }
        if (n_it >= opt.start_diis) {
            Pa = Pan;
            Pb = Pbn;
        } else {
            for (int i = 0; i < K * K; ++i) {
                Pa[i] = opt.damping * Pan[i] + (1 - opt.damping) * Pa[i];
                Pb[i] = opt.damping * Pbn[i] + (1 - opt.damping) * Pb[i];
            }
        }
        if (it == opt.max_iterations - 1) {
            if (phase == 0) phase = 1;
            build(Pa, Pb);
            double E = 0.0;
            std::vector<double> Faf(K * K), Fbf(K * K);
            for (int i = 0; i < K * K; ++i) {
                Faf[i] = H[i] + J[i] - Ka[i];
                Fbf[i] = H[i] + J[i] - Kb[i];
            }
            E = energy(Pa, Faf, H) + energy(Pb, Fbf, H);
            out.E_ele = E;
            out.E_tot = E_nuc + E;
        }
    }
    out.iterations = n_it;
    out.P = Pa;
    out.P2 = Pb;
    out.e = Ea;
    out.e2 = Eb;
    out.C = Ca;
    if (!std::isfinite(out.E_tot)) throw Error(HFX_ERR_NUMERIC, "non-finite SCF energy");
    out.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return out;
}

}  // namespace hfx
