// ref_grid_shim.cpp -- extern "C" access to the reference's own grid
// evaluation (include/cube.hpp: function_eval :9-40, electron_density :43-93,
// orbital_wf :96-135, box_points :137-168), compiled UNCHANGED from a checkout
// of KLYYCYNN/hartree_fock_cpp.  TEST INFRASTRUCTURE ONLY: built by
// oracle/Makefile into oracle/_ref/ where that checkout exists, and used to
// generate tests/golden/grid_golden.json, which pins the oracle's grid
// restatement and the engine's grid kernels.  cube.hpp includes save.hpp,
// which includes a JSON library that is not installed here; oracle/stub
// supplies a compile-only stand-in (the JSON writers are never called).
#include "cube.hpp"

#include <cstring>

static std::vector<basis_function> g_basis;

// cube.hpp calls the reference's CUDA evaluators (defined in its CUDA
// sources, cube.hpp:223-230) from its GPU branches, which this shim never
// takes; these definitions only satisfy the linker.
std::vector<double> density_gpu(const std::vector<basis_function>&, const std::vector<double>&,
                                const std::vector<vector3>&)
{
    throw std::runtime_error("density_gpu is not part of the grid shim");
}
std::vector<double> orbital_gpu(const std::vector<basis_function>&, const std::vector<double>&, int,
                                const std::vector<vector3>&)
{
    throw std::runtime_error("orbital_gpu is not part of the grid shim");
}

extern "C" {

// basis.hpp:157-262 basis_construction; returns K or -1 on error.
int refg_build_basis(int natom, const char* const* symbols, const double* xyz, const char* basis_set,
                     const char* basis_path)
{
    std::vector<std::pair<std::string, vector3>> config;
    for (int i = 0; i < natom; ++i)
        config.push_back({symbols[i], position_vector(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2])});
    try {
        g_basis = basis_construction(config, basis_set, basis_path).first;
    } catch (...) {
        return -1;
    }
    return (int)g_basis.size();
}

// column < 0: electron_density(basis, M, points); else orbital_wf(basis, M, column, points).
// M is K x K row-major (index2d order); xyz holds n points.
void refg_points(const double* M, int column, const double* xyz, int n, double* out)
{
    const int K = (int)g_basis.size();
    std::vector<double> m(M, M + (size_t)K * K);
    std::vector<vector3> r(n);
    for (int i = 0; i < n; ++i) r[i] = position_vector(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
    std::vector<double> v = column < 0 ? electron_density(g_basis, m, r) : orbital_wf(g_basis, m, column, r);
    std::memcpy(out, v.data(), sizeof(double) * n);
}

// box_points(center, L, res): res^3 points, 3 doubles each
void refg_box_points(double cx, double cy, double cz, double L, int res, double* out)
{
    std::vector<vector3> r = box_points(position_vector(cx, cy, cz), L, res);
    for (size_t i = 0; i < r.size(); ++i) {
        out[3 * i] = r[i].x;
        out[3 * i + 1] = r[i].y;
        out[3 * i + 2] = r[i].z;
    }
}

}  // extern "C"
