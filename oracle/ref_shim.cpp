// ref_shim.cpp -- extern "C" access to the reference's own integral code,
// compiled UNCHANGED from a checkout of KLYYCYNN/hartree_fock_cpp
// (include/integrals.hpp, include/basis.hpp, include/indexing.hpp and the
// vendored rapidcsv).  TEST INFRASTRUCTURE ONLY: it is built by
// oracle/Makefile into oracle/_ref/ where that checkout exists, and is used
// to pin the C restatement (hf_oracle.c) and to generate the golden fixtures
// under tests/golden/.  Nothing in the engine links it.
#include "integrals.hpp"   // brings basis.hpp, atoms.hpp, types.hpp, indexing.hpp
#include <atomic>
#include <cstring>
#include <thread>

static std::vector<basis_function> g_basis;
static std::vector<atom> g_atoms;

extern "C" {

// basis.hpp:157-262 basis_construction; returns K or -1 on error.
int ref_build_basis(int natom, const char* const* symbols, const double* xyz,
                    const char* basis_set, const char* basis_path)
{
    std::vector<std::pair<std::string, vector3>> config;
    for (int i = 0; i < natom; ++i)
        config.push_back({symbols[i], position_vector(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2])});
    try {
        g_basis = basis_construction(config, basis_set, basis_path).first;
        g_atoms = configuration(config);
    } catch (...) {
        return -1;
    }
    return (int)g_basis.size();
}

int ref_nprims_total()
{
    int n = 0;
    for (auto& f : g_basis) n += (int)f.prims.size();
    return n;
}

// flat export: centres (3K), lmn (3K), prim_off (K+1), alpha/coeff/norm
void ref_export_basis(double* centres, int* lmn, int* prim_off, double* alpha, double* coeff, double* norm)
{
    int o = 0;
    for (size_t i = 0; i < g_basis.size(); ++i) {
        const auto& f = g_basis[i];
        centres[3 * i] = f.center.x; centres[3 * i + 1] = f.center.y; centres[3 * i + 2] = f.center.z;
        lmn[3 * i] = f.lx; lmn[3 * i + 1] = f.ly; lmn[3 * i + 2] = f.lz;
        prim_off[i] = o;
        for (auto& p : f.prims) { alpha[o] = p.alpha; coeff[o] = p.coeff; norm[o] = p.norm; ++o; }
    }
    prim_off[g_basis.size()] = o;
}

double ref_boys(int m, double T) { return boys(m, T); }

double ref_basis_repulsion(int a, int b, int c, int d)
{
    return basis_repulsion(g_basis[a], g_basis[b], g_basis[c], g_basis[d]);
}

void ref_schwarz_bounds(double* out)
{
    auto b = schwarz_bounds(g_basis);
    std::memcpy(out, b.data(), b.size() * sizeof(double));
}

void ref_repulsion_tensor(double threshold, double* out)
{
    auto e = repulsion_tensor(g_basis, threshold);
    std::memcpy(out, e.data(), e.size() * sizeof(double));
}

// repulsion_tensor (integrals.hpp:754-787) with its Schwarz pass and quartet
// loop spread over nthreads host threads (harness only: each element is still
// one call of the reference's basis_repulsion, with the reference's own
// schwarz test and index helpers, so the array equals repulsion_tensor's).
void ref_repulsion_tensor_mt(double threshold, double* out, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    const int K = (int)g_basis.size();
    const size_t n_pairs = (size_t)K * (K + 1) / 2;
    const size_t n_quartets = n_pairs * (n_pairs + 1) / 2;
    std::vector<double> bounds(n_pairs);
    auto par = [&](size_t n, size_t block, auto body) {
        std::atomic<size_t> next{0};
        std::vector<std::thread> th;
        for (int t = 0; t < nthreads; ++t)
            th.emplace_back([&] {
                for (;;) {
                    size_t b = next.fetch_add(block);
                    if (b >= n) break;
                    size_t e = std::min(n, b + block);
                    for (size_t i = b; i < e; ++i) body(i);
                }
            });
        for (auto& t : th) t.join();
    };
    par(n_pairs, 8, [&](size_t i) {
        std::pair<int, int> idx = pair_to_indices((int)i);
        double b = basis_repulsion(g_basis[idx.first], g_basis[idx.second], g_basis[idx.first], g_basis[idx.second]);
        bounds[i] = std::sqrt(std::max(b, 0.0));
    });
    par(n_quartets, 1024, [&](size_t i) {
        std::pair<int, int> q = quartet_to_pairs(i);
        std::pair<int, int> p1 = pair_to_indices(q.first);
        std::pair<int, int> p2 = pair_to_indices(q.second);
        if (bounds[q.first] * bounds[q.second] < threshold) {
            out[i] = 0.0;
            return;
        }
        out[i] = basis_repulsion(g_basis[p1.first], g_basis[p1.second], g_basis[p2.first], g_basis[p2.second]);
    });
}

void ref_one_electron(double* S, double* T, double* V)
{
    auto s = overlap_matrix(g_basis);
    auto t = kinetic_matrix(g_basis);
    auto v = attraction_matrix(g_basis, g_atoms);
    std::memcpy(S, s.data(), s.size() * sizeof(double));
    std::memcpy(T, t.data(), t.size() * sizeof(double));
    std::memcpy(V, v.data(), v.size() * sizeof(double));
}

}  // extern "C"
