// hfx_api.cpp -- the extern "C" boundary of libhfx (include/hfx.h).  Every
// entry point converts engine exceptions into an hfx_status plus a
// thread-local message; nothing terminates the process (the reference's
// cuda_check calls std::exit, cuda/src/eri.cu:8-14).
#include <cstring>
#include <memory>
#include <string>

#include "hfx_dscf.hpp"
#include "hfx_engine.hpp"
#include "hfx_scf.hpp"

struct hfx_job {
    std::unique_ptr<hfx::Job> job;
    std::unique_ptr<hfx::ScfSetup> setup;   // S, H, X, E_nuc; made on first SCF
    std::unique_ptr<hfx::DeviceScf> dscf_rhf, dscf_uhf;   // device SCF workspaces
    ~hfx_job()
    {
        dscf_rhf.reset();
        dscf_uhf.reset();
        job.reset();
    }
};

namespace hfx {
// density-weighted screening threshold of the FP64 builds of density changes
// in the mixed-precision SCF (Q_AB Q_CD max|dD| below this: quartet skipped)
constexpr double kDeltaThr = 1e-12;
void fock_rhf_noalloc(Job& job, int device, const double* dP, double* dG);   // hfx_noalloc.cu
void noalloc_prepare(int device);                                            // hfx_noalloc.cu
void grid_eval(const Basis& b, int device, const double* M, int column, const double* xyz, long long n, int res,
               const double* start, const double* step, double* out);                  // hfx_grid.cu
static thread_local std::string g_last_error;
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace hfx

using namespace hfx;

template <typename F>
static hfx_status guarded(F&& f)
{
    try {
        g_last_error.clear();
        f();
        return HFX_OK;
    } catch (const Error& e) {
        g_last_error = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        g_last_error = "host allocation failed";
        return HFX_ERR_OOM;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return HFX_ERR_INVALID;
    } catch (...) {
        g_last_error = "unknown error";
        return HFX_ERR_INVALID;
    }
}

static hfx_options default_options(const hfx_options* o)
{
    hfx_options r{};
    if (o) r = *o;
    return r;
}

extern "C" {

hfx_status hfx_last_error(char* buf, size_t n)
{
    if (!buf || n == 0) return HFX_ERR_INVALID;
    std::strncpy(buf, g_last_error.c_str(), n - 1);
    buf[n - 1] = 0;
    return HFX_OK;
}

hfx_status hfx_create(const hfx_functions* basis, const hfx_options* opt, hfx_job** job)
{
    return guarded([&] {
        if (!basis || !job) throw Error(HFX_ERR_INVALID, "null argument");
        *job = nullptr;
        auto j = std::make_unique<hfx_job>();
        j->job = std::make_unique<Job>(basis_from_functions(*basis), default_options(opt));
        noalloc_prepare(j->job->device());
        *job = j.release();
    });
}

hfx_status hfx_create_molecule(const hfx_molecule* mol, const hfx_options* opt, hfx_job** job)
{
    return guarded([&] {
        if (!mol || !job) throw Error(HFX_ERR_INVALID, "null argument");
        *job = nullptr;
        auto j = std::make_unique<hfx_job>();
        j->job = std::make_unique<Job>(build_basis(*mol), default_options(opt));
        noalloc_prepare(j->job->device());
        *job = j.release();
    });
}

hfx_status hfx_destroy(hfx_job* job)
{
    return guarded([&] { delete job; });
}

hfx_status hfx_nbasis(const hfx_job* job, int* K)
{
    return guarded([&] {
        if (!job || !K) throw Error(HFX_ERR_INVALID, "null argument");
        *K = job->job->K();
    });
}

static void export_basis(const Basis& b, double* centres, int* lmn, int* prim_offset, double* alpha, double* coeff,
                         double* norm, int* nprim_total)
{
    int off = 0;
    for (const auto& s : b.shells) {
        int nc = ncart(s.L), np = s.nprim();
        for (int c = 0; c < nc; ++c) {
            int f = s.bf0 + c;
            int lx, ly, lz;
            component(s.L, c, lx, ly, lz);
            if (centres) {
                centres[3 * f] = s.x;
                centres[3 * f + 1] = s.y;
                centres[3 * f + 2] = s.z;
            }
            if (lmn) {
                lmn[3 * f] = lx;
                lmn[3 * f + 1] = ly;
                lmn[3 * f + 2] = lz;
            }
            if (prim_offset) prim_offset[f] = off;
            for (int i = 0; i < np; ++i) {
                if (alpha) alpha[off + i] = s.exps[i];
                if (coeff) coeff[off + i] = s.coef[i];
                if (norm) norm[off + i] = s.coef[i] != 0.0 ? s.w[(size_t)c * np + i] / s.coef[i] : cart_norm(s.exps[i], lx, ly, lz);
            }
            off += np;
        }
    }
    if (prim_offset) prim_offset[b.K] = off;
    if (nprim_total) *nprim_total = off;
}

hfx_status hfx_export_functions(const hfx_job* job, double* centres, int* lmn, int* prim_offset, double* alpha,
                                double* coeff, double* norm, int* nprim_total)
{
    return guarded([&] {
        if (!job) throw Error(HFX_ERR_INVALID, "null job");
        export_basis(job->job->basis(), centres, lmn, prim_offset, alpha, coeff, norm, nprim_total);
    });
}

hfx_status hfx_build_functions(const hfx_molecule* mol, int* K, int* nprim_total, double* centres, int* lmn,
                               int* prim_offset, double* alpha, double* coeff, double* norm)
{
    return guarded([&] {
        if (!mol) throw Error(HFX_ERR_INVALID, "null molecule");
        Basis b = build_basis(*mol);
        if (K) *K = b.K;
        export_basis(b, centres, lmn, prim_offset, alpha, coeff, norm, nprim_total);
    });
}

hfx_status hfx_debug_pair_data(const hfx_molecule* mol, int* npairs, int* nprimpairs, long long* nepool, int* rec,
                               double* geo, double* epool)
{
    return guarded([&] {
        if (!mol) throw Error(HFX_ERR_INVALID, "null molecule");
        const Basis b = build_basis(*mol);
        PairData pd = build_pair_data(b, single_fragment(b));
        if (npairs) *npairs = (int)pd.dpairs.size();
        if (nprimpairs) *nprimpairs = (int)pd.geo.size();
        if (nepool) *nepool = (long long)pd.epool.size();
        if (rec)
            for (size_t p = 0; p < pd.dpairs.size(); ++p) {
                const DPair& d = pd.dpairs[p];
                int* r = rec + 10 * p;
                r[0] = d.bf0; r[1] = d.bf1; r[2] = d.l0; r[3] = d.l1; r[4] = d.pp0; r[5] = d.npp;
                r[6] = (int)(d.e_off & 0xffffffffLL); r[7] = (int)(d.e_off >> 32); r[8] = d.same; r[9] = d.id;
            }
        if (geo)
            for (size_t q = 0; q < pd.geo.size(); ++q) {
                geo[4 * q] = pd.geo[q].p; geo[4 * q + 1] = pd.geo[q].x;
                geo[4 * q + 2] = pd.geo[q].y; geo[4 * q + 3] = pd.geo[q].z;
            }
        if (epool) std::memcpy(epool, pd.epool.data(), pd.epool.size() * sizeof(double));
    });
}

hfx_status hfx_schwarz(hfx_job* job, double* Q)
{
    return guarded([&] {
        if (!job || !Q) throw Error(HFX_ERR_INVALID, "null argument");
        std::vector<double> q;
        job->job->schwarz_host(q);
        std::memcpy(Q, q.data(), q.size() * sizeof(double));
    });
}

hfx_status hfx_fock_rhf(hfx_job* job, const double* P, double* G)
{
    return guarded([&] {
        if (!job || !P || !G) throw Error(HFX_ERR_INVALID, "null argument");
        job->job->fock_rhf(P, G);
    });
}

hfx_status hfx_fock_uhf(hfx_job* job, const double* Pa, const double* Pb, double* J, double* Ka, double* Kb)
{
    return guarded([&] {
        if (!job || !Pa || !Pb || !J || !Ka || !Kb) throw Error(HFX_ERR_INVALID, "null argument");
        job->job->fock_uhf(Pa, Pb, J, Ka, Kb);
    });
}

hfx_status hfx_fock_rhf_device(hfx_job* job, const double* dP, double* dG)
{
    return guarded([&] {
        if (!job || !dP || !dG) throw Error(HFX_ERR_INVALID, "null argument");
        job->job->fock_rhf_device(dP, dG);
    });
}

hfx_status hfx_fock_uhf_device(hfx_job* job, const double* dPa, const double* dPb, double* dJ, double* dKa,
                               double* dKb)
{
    return guarded([&] {
        if (!job || !dPa || !dPb || !dJ || !dKa || !dKb) throw Error(HFX_ERR_INVALID, "null argument");
        job->job->fock_uhf_device(dPa, dPb, dJ, dKa, dKb);
    });
}

hfx_status hfx_fock_rhf_device_noalloc(hfx_job* job, const double* dP, double* dG)
{
    return guarded([&] {
        if (!job || !dP || !dG) throw Error(HFX_ERR_INVALID, "null argument");
        fock_rhf_noalloc(*job->job, job->job->device(), dP, dG);
    });
}

hfx_status hfx_eri_unique(hfx_job* job, double threshold, double* out)
{
    return guarded([&] {
        if (!job || !out) throw Error(HFX_ERR_INVALID, "null argument");
        job->job->eri_unique(threshold, out);
    });
}

hfx_status hfx_eri_gpu(const hfx_functions* basis, double threshold, double* out)
{
    return guarded([&] {
        if (!basis || !out) throw Error(HFX_ERR_INVALID, "null argument");
        hfx_options o{};
        o.screening_threshold = threshold;
        Job j(basis_from_functions(*basis), o);
        j.eri_unique(threshold, out);
    });
}

hfx_status hfx_autotune_fp32_threshold(hfx_job* job, const double* P, double target_dE, double* tau,
                                       double* dE, double* ms_fp64, double* ms_mixed)
{
    return guarded([&] {
        if (!job || !P) throw Error(HFX_ERR_INVALID, "null argument");
        if (!(target_dE > 0.0)) throw Error(HFX_ERR_INVALID, "target_dE must be positive");
        double t = job->job->autotune_fp32_threshold(P, target_dE, dE, ms_fp64, ms_mixed);
        if (tau) *tau = t;
    });
}

hfx_status hfx_get_launch_shape(const hfx_job* job, hfx_launch_shape* shape)
{
    return guarded([&] {
        if (!job || !shape) throw Error(HFX_ERR_INVALID, "null argument");
        *shape = job->job->launch_shape();
    });
}

hfx_status hfx_set_launch_shape(hfx_job* job, const hfx_launch_shape* shape)
{
    return guarded([&] {
        if (!job || !shape) throw Error(HFX_ERR_INVALID, "null argument");
        job->job->set_launch_shape(*shape);
    });
}

hfx_status hfx_autotune_launch_shape(hfx_job* job, const double* P, int builds, hfx_launch_shape* shape,
                                     double* best_ms)
{
    return guarded([&] {
        if (!job || !P) throw Error(HFX_ERR_INVALID, "null argument");
        const double ms = job->job->autotune_launch_shape(P, builds, shape);
        if (best_ms) *best_ms = ms;
    });
}

hfx_status hfx_last_build_stats(const hfx_job* job, hfx_build_stats* stats)
{
    return guarded([&] {
        if (!job || !stats) throw Error(HFX_ERR_INVALID, "null argument");
        *stats = job->job->stats;
    });
}

// The reference's box_points (cube.hpp:137-168): linspace(c - L/2, c + L/2, res) per axis.
static void box_eval(const Basis& b, int device, const double* M, int column, const double* center, double L, int res,
                     double* out)
{
    if (res < 2) throw Error(HFX_ERR_INVALID, "resolution must be at least 2");
    if (res > 2048) throw Error(HFX_ERR_INVALID, "resolution above 2048");
    double start[3], step[3];
    for (int d = 0; d < 3; ++d) {
        const double lo = center[d] - L / 2, hi = center[d] + L / 2;
        start[d] = lo;
        step[d] = (hi - lo) / (res - 1);
    }
    grid_eval(b, device, M, column, nullptr, (long long)res * res * res, res, start, step, out);
}

static void fill_result(const ScfOutput& o, hfx_scf_result* r, double fock_ms)
{
    if (!r) return;
    std::memset(r, 0, sizeof(*r));
    r->E_tot = o.E_tot;
    r->E_ele = o.E_ele;
    r->E_nuc = o.E_nuc;
    r->iterations = o.iterations;
    r->converged = o.converged ? 1 : 0;
    r->K = o.K;
    r->n_electrons = o.n_electrons;
    r->seconds = o.seconds;
    r->fock_ms = fock_ms;
    r->fock_builds = o.fock_builds;
    r->mixed_builds = o.mixed_builds;
    r->fp64_builds = o.fp64_builds;
    r->delta_builds = o.delta_builds;
    r->projections = o.projections;
    r->projection_fallbacks = o.projection_fallbacks;
}

static hfx_options job_options(const hfx_scf_options* o)
{
    hfx_options j{};
    if (o) {
        j.screening_threshold = o->screening_threshold;
        j.precision = o->precision;
        j.fp32_threshold = o->fp32_threshold;
    }
    return j;
}

hfx_status hfx_rhf_diis(const hfx_molecule* mol, const hfx_scf_options* opt, const double* P0, hfx_scf_result* res,
                        double* density, double* coefficient, double* mo_energy)
{
    hfx_status st = guarded([&] {
        if (!mol) throw Error(HFX_ERR_INVALID, "null molecule");
        hfx_scf_options o{};
        if (opt) o = *opt;
        Basis b = build_basis(*mol);
        Job job(b, job_options(&o));
        ScfSetup setup = scf_setup(b, true);
        DeviceScf d(job, setup, 1);
        ScfOutput out = d.run(b, setup, o, 0, 0, P0, nullptr, kDeltaThr);
        fill_result(out, res, out.fock_ms);
        int K = out.K;
        if (density) std::memcpy(density, out.P.data(), sizeof(double) * K * K);
        if (coefficient && !out.C.empty()) std::memcpy(coefficient, out.C.data(), sizeof(double) * K * K);
        if (mo_energy && !out.e.empty()) std::memcpy(mo_energy, out.e.data(), sizeof(double) * K);
        if (!out.converged) throw Error(HFX_ERR_NOT_CONVERGED, "SCF did not converge within max_iterations");
    });
    return st;
}

hfx_status hfx_uhf_diis(const hfx_molecule* mol, const hfx_scf_options* opt, int n_alpha, int n_beta,
                        const double* Pa0, const double* Pb0, hfx_scf_result* res, double* Pa, double* Pb,
                        double* mo_energy_a, double* mo_energy_b)
{
    return guarded([&] {
        if (!mol) throw Error(HFX_ERR_INVALID, "null molecule");
        hfx_scf_options o{};
        if (opt) o = *opt;
        Basis b = build_basis(*mol);
        Job job(b, job_options(&o));
        ScfSetup setup = scf_setup(b, true);
        DeviceScf d(job, setup, 2);
        ScfOutput out = d.run(b, setup, o, n_alpha, n_beta, Pa0, Pb0, kDeltaThr);
        fill_result(out, res, out.fock_ms);
        int K = out.K;
        if (Pa) std::memcpy(Pa, out.P.data(), sizeof(double) * K * K);
        if (Pb) std::memcpy(Pb, out.P2.data(), sizeof(double) * K * K);
        if (mo_energy_a && !out.e.empty()) std::memcpy(mo_energy_a, out.e.data(), sizeof(double) * K);
        if (mo_energy_b && !out.e2.empty()) std::memcpy(mo_energy_b, out.e2.data(), sizeof(double) * K);
        if (!out.converged) throw Error(HFX_ERR_NOT_CONVERGED, "SCF did not converge within max_iterations");
    });
}

static const ScfSetup& job_setup(hfx_job* job)
{
    if (job->job->basis().atom_Z.empty())
        throw Error(HFX_ERR_INVALID, "SCF needs a job created from a molecule (nuclear charges)");
    if (!job->setup) job->setup = std::make_unique<ScfSetup>(scf_setup(job->job->basis(), true));
    return *job->setup;
}

hfx_status hfx_job_rhf(hfx_job* job, const hfx_scf_options* opt, const double* P0, hfx_scf_result* res,
                       double* density, double* coefficient, double* mo_energy)
{
    return guarded([&] {
        if (!job) throw Error(HFX_ERR_INVALID, "null job");
        hfx_scf_options o{};
        if (opt) o = *opt;
        const ScfSetup& setup = job_setup(job);
        Job& j = *job->job;
        if (!job->dscf_rhf) job->dscf_rhf = std::make_unique<DeviceScf>(j, setup, 1);
        ScfOutput out = job->dscf_rhf->run(j.basis(), setup, o, 0, 0, P0, nullptr, kDeltaThr);
        fill_result(out, res, out.fock_ms);
        int K = out.K;
        if (density) std::memcpy(density, out.P.data(), sizeof(double) * K * K);
        if (coefficient && !out.C.empty()) std::memcpy(coefficient, out.C.data(), sizeof(double) * K * K);
        if (mo_energy && !out.e.empty()) std::memcpy(mo_energy, out.e.data(), sizeof(double) * K);
        if (!out.converged) throw Error(HFX_ERR_NOT_CONVERGED, "SCF did not converge within max_iterations");
    });
}

hfx_status hfx_job_uhf(hfx_job* job, const hfx_scf_options* opt, int n_alpha, int n_beta, const double* Pa0,
                       const double* Pb0, hfx_scf_result* res, double* Pa, double* Pb)
{
    return guarded([&] {
        if (!job) throw Error(HFX_ERR_INVALID, "null job");
        hfx_scf_options o{};
        if (opt) o = *opt;
        const ScfSetup& setup = job_setup(job);
        Job& j = *job->job;
        if (!job->dscf_uhf) job->dscf_uhf = std::make_unique<DeviceScf>(j, setup, 2);
        ScfOutput out = job->dscf_uhf->run(j.basis(), setup, o, n_alpha, n_beta, Pa0, Pb0, kDeltaThr);
        fill_result(out, res, out.fock_ms);
        int K = out.K;
        if (Pa) std::memcpy(Pa, out.P.data(), sizeof(double) * K * K);
        if (Pb) std::memcpy(Pb, out.P2.data(), sizeof(double) * K * K);
        if (!out.converged) throw Error(HFX_ERR_NOT_CONVERGED, "SCF did not converge within max_iterations");
    });
}

hfx_status hfx_rhf_diis_with_builder(const hfx_molecule* mol, const hfx_scf_options* opt, const double* P0,
                                     hfx_g_builder gb, void* user, hfx_scf_result* res, double* density,
                                     double* mo_energy)
{
    return guarded([&] {
        if (!mol || !gb) throw Error(HFX_ERR_INVALID, "null argument");
        hfx_scf_options o{};
        if (opt) o = *opt;
        Basis b = build_basis(*mol);
        GBuilder g = [&](const double* P, double* G, int) {
            if (gb(user, P, G) != 0) throw Error(HFX_ERR_INVALID, "caller G builder failed");
        };
        ScfOutput out = rhf_diis(b, o, P0, g);
        fill_result(out, res, 0.0);
        if (density) std::memcpy(density, out.P.data(), sizeof(double) * out.K * out.K);
        if (mo_energy && !out.e.empty()) std::memcpy(mo_energy, out.e.data(), sizeof(double) * out.K);
        if (!out.converged) throw Error(HFX_ERR_NOT_CONVERGED, "SCF did not converge within max_iterations");
    });
}

hfx_status hfx_uhf_diis_with_builder(const hfx_molecule* mol, const hfx_scf_options* opt, int n_alpha, int n_beta,
                                     hfx_jk_builder jkb, void* user, hfx_scf_result* res, double* Pa, double* Pb)
{
    return guarded([&] {
        if (!mol || !jkb) throw Error(HFX_ERR_INVALID, "null argument");
        hfx_scf_options o{};
        if (opt) o = *opt;
        Basis b = build_basis(*mol);
        JKBuilder jk = [&](const double* a, const double* bb, double* J, double* Ka, double* Kb, int) {
            if (jkb(user, a, bb, J, Ka, Kb) != 0) throw Error(HFX_ERR_INVALID, "caller JK builder failed");
        };
        ScfOutput out = uhf_diis(b, o, n_alpha, n_beta, nullptr, nullptr, jk);
        fill_result(out, res, 0.0);
        if (Pa) std::memcpy(Pa, out.P.data(), sizeof(double) * out.K * out.K);
        if (Pb) std::memcpy(Pb, out.P2.data(), sizeof(double) * out.K * out.K);
        if (!out.converged) throw Error(HFX_ERR_NOT_CONVERGED, "SCF did not converge within max_iterations");
    });
}

hfx_status hfx_debug_packed_pairs(const hfx_molecule* mols, int n, int* npairs, int* rec, long long* offs)
{
    return guarded([&] {
        if (!mols || n <= 0) throw Error(HFX_ERR_INVALID, "null molecules or n <= 0");
        std::vector<Basis> bases;
        for (int i = 0; i < n; ++i) bases.push_back(build_basis(mols[i]));
        Fragments fr;
        const Basis all = concat_basis(bases, fr);
        const PairData pd = build_pair_data(all, fr);
        if (npairs) *npairs = (int)pd.dpairs.size();
        for (size_t p = 0; p < pd.dpairs.size(); ++p) {
            const DPair& d = pd.dpairs[p];
            if (rec) {
                int* r = rec + 10 * p;
                r[0] = d.frag; r[1] = d.kdim; r[2] = d.pbase; r[3] = d.id; r[4] = d.sh0;
                r[5] = d.sh1; r[6] = d.bf0; r[7] = d.bf1; r[8] = d.l0; r[9] = d.l1;
            }
            if (offs) {
                offs[3 * p] = d.moff;
                offs[3 * p + 1] = d.qoff;
                offs[3 * p + 2] = d.npp;
            }
        }
    });
}

hfx_status hfx_debug_plan(const hfx_job* job, int mixed, int* ngroups, double* rows)
{
    return guarded([&] {
        if (!job || !ngroups) throw Error(HFX_ERR_INVALID, "null argument");
        const auto& groups = job->job->plan_groups(mixed != 0);
        *ngroups = (int)groups.size();
        if (!rows) return;
        for (size_t g = 0; g < groups.size(); ++g) {
            const LaunchGroup& x = groups[g];
            double* r = rows + 10 * g;
            r[0] = x.kind; r[1] = x.pcb; r[2] = x.pck; r[3] = x.fp32 ? 1 : 0; r[4] = (double)x.n;
            r[5] = x.flops; r[6] = x.prims; r[7] = x.grid; r[8] = x.slice; r[9] = x.warps_per_cta;
        }
    });
}

hfx_status hfx_one_electron(const hfx_molecule* mol, double* S, double* T, double* V, int* K)
{
    return guarded([&] {
        if (!mol) throw Error(HFX_ERR_INVALID, "null molecule");
        Basis b = build_basis(*mol);
        if (K) *K = b.K;
        if (!S && !T && !V) return;
        std::vector<double> s, t, v;
        one_electron(b, s, t, v);
        if (S) std::memcpy(S, s.data(), s.size() * sizeof(double));
        if (T) std::memcpy(T, t.data(), t.size() * sizeof(double));
        if (V) std::memcpy(V, v.data(), v.size() * sizeof(double));
    });
}

static void check_device(int device)
{
    int ndev = 0;
    cuda_check(cudaGetDeviceCount(&ndev), "cudaGetDeviceCount");
    if (device < 0 || device >= ndev) throw Error(HFX_ERR_INVALID, "invalid CUDA device ordinal");
}

hfx_status hfx_grid_density(const hfx_functions* basis, int device, const double* P, const double* center, double L,
                            int res, double* rho)
{
    return guarded([&] {
        if (!basis || !P || !center || !rho) throw Error(HFX_ERR_INVALID, "null argument");
        check_device(device);
        box_eval(basis_from_functions(*basis), device, P, -1, center, L, res, rho);
    });
}

hfx_status hfx_grid_orbital(const hfx_functions* basis, int device, const double* C, int column, const double* center,
                            double L, int res, double* psi)
{
    return guarded([&] {
        if (!basis || !C || !center || !psi) throw Error(HFX_ERR_INVALID, "null argument");
        if (column < 0 || column >= basis->K) throw Error(HFX_ERR_INVALID, "orbital index out of range");
        check_device(device);
        box_eval(basis_from_functions(*basis), device, C, column, center, L, res, psi);
    });
}

hfx_status hfx_points_eval(const hfx_functions* basis, int device, const double* M, int column, const double* xyz,
                           long long n, double* out)
{
    return guarded([&] {
        if (!basis || !M || (n > 0 && (!xyz || !out))) throw Error(HFX_ERR_INVALID, "null argument");
        if (n < 0) throw Error(HFX_ERR_INVALID, "negative point count");
        if (column >= basis->K) throw Error(HFX_ERR_INVALID, "orbital index out of range");
        check_device(device);
        if (n == 0) return;
        grid_eval(basis_from_functions(*basis), device, M, column < 0 ? -1 : column, xyz, n, 0, nullptr, nullptr, out);
    });
}

hfx_status hfx_one_electron_gpu(const hfx_molecule* mol, int device, double* S, double* T, double* V, int* K)
{
    return guarded([&] {
        if (!mol) throw Error(HFX_ERR_INVALID, "null molecule");
        int ndev = 0;
        cuda_check(cudaGetDeviceCount(&ndev), "cudaGetDeviceCount");
        if (device < 0 || device >= ndev) throw Error(HFX_ERR_INVALID, "invalid CUDA device ordinal");
        cuda_check(cudaSetDevice(device), "cudaSetDevice");
        Basis b = build_basis(*mol);
        if (K) *K = b.K;
        if (!S && !T && !V) return;
        std::vector<double> s, t, v;
        one_electron_gpu(b, s, t, v);
        if (S) std::memcpy(S, s.data(), s.size() * sizeof(double));
        if (T) std::memcpy(T, t.data(), t.size() * sizeof(double));
        if (V) std::memcpy(V, v.data(), v.size() * sizeof(double));
    });
}

}  // extern "C"
