// hfx_internal.hpp -- host-side types shared by the libhfx translation units.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "hfx.h"

namespace hfx {

// Error carried from the engine internals to the C ABI, where it becomes an
// hfx_status plus a thread-local message (hfx_last_error).
struct Error : std::runtime_error {
    hfx_status code;
    Error(hfx_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& msg);

constexpr int kMaxL = 3;                   // up to f, as the reference (integrals.hpp:325)
constexpr int kMaxLTot = 4 * kMaxL;        // (ff|ff) -> 12
constexpr int ncart(int l) { return (l + 1) * (l + 2) / 2; }
constexpr int nherm(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }

// One contracted Cartesian shell.  Components follow angmom_partition order
// (basis.hpp:52-64): for lx = 0..L, ly = 0..L-lx: (lx, ly, L-lx-ly).
struct Shell {
    double x, y, z;
    int L;
    int bf0;                    // first basis function (reference order)
    int atom;                   // atom index (informational)
    std::vector<double> exps;   // nprim exponents
    std::vector<double> coef;   // nprim contraction coefficients
    // w[c * nprim + i] = coeff_i * norm_i(component c): the per-component
    // primitive weight the reference applies in basis_repulsion
    // (integrals.hpp:719-721).
    std::vector<double> w;
    int nprim() const { return (int)exps.size(); }
};

struct Basis {
    std::vector<Shell> shells;
    int K = 0;
    std::vector<int> atom_Z;            // per atom (0 if unknown)
    std::vector<double> atom_xyz;       // 3 per atom
};

// Reference cart_norm (basis.hpp:28-49).
double cart_norm(double alpha, int lx, int ly, int lz);

// Component (lx,ly,lz) of index c in a shell of angular momentum L.
void component(int L, int c, int& lx, int& ly, int& lz);

// basis.hpp:157-262 equivalent: atoms in order -> CSV shells -> components.
Basis build_basis(const hfx_molecule& mol);

// Group a flat basis-function list (reference basis_function records) into
// shells; throws Error(HFX_ERR_BASIS) if the list does not form complete
// Cartesian shells.
Basis basis_from_functions(const hfx_functions& f);

int element_Z(const std::string& sym);

// Host one-electron matrices (K x K row-major).
void one_electron(const Basis& b, std::vector<double>& S, std::vector<double>& T, std::vector<double>& V);
// The same matrices computed on the current CUDA device (hfx_onee_gpu.cu).
void one_electron_gpu(const Basis& b, std::vector<double>& S, std::vector<double>& T, std::vector<double>& V);

// 1-D Hermite expansion coefficients E^{ij}_t (integrals.hpp:269-322
// recursion) for i <= imax, j <= jmax, stored
// E[(i*(jmax+1)+j)*(imax+jmax+1)+t].
void hermite_1d(int imax, int jmax, double a, double b, double A, double B, std::vector<double>& E);

// Nuclear repulsion energy (scf.hpp:64-78).
double nuclear_repulsion(const Basis& b);

// Accurate Boys function on the host (series / asymptotic), used for the
// device table and host one-electron integrals.
double boys_host(int m, double T);

// ---- dense linear algebra (linalg.cpp) ----
// Symmetric eigen-decomposition: A (n x n, row-major) -> eigenvalues
// ascending in w, eigenvectors as columns of V (row-major n x n).
void sym_eig(int n, const double* A, double* w, double* V);
// Solve A x = b with LU and complete pivoting (Eigen fullPivLu stand-in).
void solve_full_piv(int n, const double* A, const double* b, double* x);
void matmul(int n, const double* A, const double* B, double* C);   // C = A B
void matmul_tn(int n, const double* A, const double* B, double* C); // C = A^T B

}  // namespace hfx
