// hfx_basis.cpp -- basis construction with the reference's conventions.
//
// Reads the reference's per-element CSV tables (columns
// shell_id,L,primitive_id,exponent,coefficient; basis.hpp:180-231) and builds
// Cartesian shells in the reference's order: atoms in input order, shells in
// CSV order, components in angmom_partition order (basis.hpp:52-64), with the
// per-component primitive norm cart_norm (basis.hpp:28-49) and the
// contraction left unnormalised, as basis.hpp:67-113 does.
#include <dlfcn.h>

#include <cmath>
#include <fstream>
#include <map>
#include <sstream>

#include "hfx_internal.hpp"

namespace hfx {

static const char* kElements[] = {"H",  "He", "Li", "Be", "B",  "C",  "N",  "O",  "F",  "Ne", "Na", "Mg",
                                  "Al", "Si", "P",  "S",  "Cl", "Ar", "K",  "Ca", "Sc", "Ti", "V",  "Cr",
                                  "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge", "As", "Se", "Br", "Kr"};

int element_Z(const std::string& sym)
{
    for (int i = 0; i < 36; ++i)
        if (sym == kElements[i]) return i + 1;
    return 0;
}

static int double_factorial(int n)
{
    int r = 1;
    for (int k = n; k > 0; k -= 2) r *= k;
    return r;
}

double cart_norm(double alpha, int lx, int ly, int lz)
{
    int L = lx + ly + lz;
    double num = std::pow(4.0 * alpha, L);
    double den = double(double_factorial(2 * lx - 1)) * double_factorial(2 * ly - 1) * double_factorial(2 * lz - 1);
    return std::pow(2.0 * alpha / M_PI, 0.75) * std::sqrt(num / den);
}

void component(int L, int c, int& lx, int& ly, int& lz)
{
    int n = 0;
    for (int a = 0; a <= L; ++a)
        for (int b = 0; b <= L - a; ++b) {
            if (n == c) {
                lx = a;
                ly = b;
                lz = L - a - b;
                return;
            }
            ++n;
        }
    lx = ly = lz = -1;
}

static std::string default_basis_path()
{
    Dl_info info;
    if (dladdr((void*)&default_basis_path, &info) && info.dli_fname) {
        std::string so = info.dli_fname;
        auto pos = so.find_last_of('/');
        std::string dir = pos == std::string::npos ? std::string(".") : so.substr(0, pos);
        return dir + "/basis";
    }
    return "basis";
}

struct CsvShell {
    int L;
    std::vector<double> e, c;
};

static std::vector<CsvShell> read_element(const std::string& path, const std::string& set, const std::string& el)
{
    std::string fn = path + "/" + set + "/" + el + ".csv";
    std::ifstream in(fn);
    if (!in.is_open())
        throw Error(HFX_ERR_BASIS, "Critical Error: File does not exist or is invalid at path: " + fn);
    std::string line;
    std::getline(in, line);  // header
    // column positions from the header
    std::vector<std::string> cols;
    {
        std::stringstream ss(line);
        std::string t;
        while (std::getline(ss, t, ',')) {
            while (!t.empty() && (t.back() == '\r' || t.back() == ' ')) t.pop_back();
            cols.push_back(t);
        }
    }
    auto col = [&](const char* name) {
        for (size_t i = 0; i < cols.size(); ++i)
            if (cols[i] == name) return (int)i;
        throw Error(HFX_ERR_BASIS, "basis file " + fn + " lacks column " + name);
    };
    int c_sid = col("shell_id"), c_L = col("L"), c_pid = col("primitive_id"), c_e = col("exponent"),
        c_c = col("coefficient");
    std::vector<CsvShell> shells;
    std::vector<int> maxpid;
    int cur = -1;
    while (std::getline(in, line)) {
        if (line.empty() || line == "\r") continue;
        std::vector<std::string> f;
        std::stringstream ss(line);
        std::string t;
        while (std::getline(ss, t, ',')) f.push_back(t);
        if ((int)f.size() < (int)cols.size()) throw Error(HFX_ERR_BASIS, "malformed row in " + fn);
        int sid = std::stoi(f[c_sid]);
        std::string Ls = f[c_L];
        while (!Ls.empty() && (Ls.back() == ' ' || Ls.back() == '\r')) Ls.pop_back();
        static const std::string sym = "SPDFGH";
        int L = (int)sym.find(Ls);
        if (Ls.size() != 1 || L < 0) throw Error(HFX_ERR_BASIS, "unknown angular momentum '" + Ls + "' in " + fn);
        if (sid != cur) {
            if (sid != (int)shells.size())
                throw Error(HFX_ERR_BASIS, "building shells in the wrong order");  // basis.hpp:222-225
            shells.push_back({L, {}, {}});
            maxpid.push_back(-1);
            cur = sid;
        }
        shells.back().e.push_back(std::stod(f[c_e]));
        shells.back().c.push_back(std::stod(f[c_c]));
        maxpid.back() = std::max(maxpid.back(), std::stoi(f[c_pid]));
    }
    for (size_t j = 0; j < shells.size(); ++j)
        if (maxpid[j] + 1 != (int)shells[j].e.size())
            throw Error(HFX_ERR_BASIS, "wrong primitive number");  // basis.hpp:215-217
    return shells;
}

static void finish_shell(Shell& s)
{
    int nc = ncart(s.L), np = s.nprim();
    s.w.assign((size_t)nc * np, 0.0);
    for (int c = 0; c < nc; ++c) {
        int lx, ly, lz;
        component(s.L, c, lx, ly, lz);
        for (int i = 0; i < np; ++i) s.w[(size_t)c * np + i] = s.coef[i] * cart_norm(s.exps[i], lx, ly, lz);
    }
}

Basis build_basis(const hfx_molecule& mol)
{
    if (mol.natom <= 0 || !mol.symbols || !mol.xyz || !mol.basis_set)
        throw Error(HFX_ERR_INVALID, "hfx_molecule: natom, symbols, xyz and basis_set are required");
    std::string path = mol.basis_path && mol.basis_path[0] ? std::string(mol.basis_path) : default_basis_path();
    std::map<std::string, std::vector<CsvShell>> cache;
    Basis b;
    int bf = 0;
    for (int a = 0; a < mol.natom; ++a) {
        std::string el = mol.symbols[a];
        int Z = element_Z(el);
        if (Z == 0) throw Error(HFX_ERR_BASIS, "unknown element symbol '" + el + "'");
        b.atom_Z.push_back(Z);
        for (int k = 0; k < 3; ++k) b.atom_xyz.push_back(mol.xyz[3 * a + k]);
        auto it = cache.find(el);
        if (it == cache.end()) it = cache.emplace(el, read_element(path, mol.basis_set, el)).first;
        for (const auto& cs : it->second) {
            if (cs.L > kMaxL)
                throw Error(HFX_ERR_UNSUPPORTED, "angular momentum above f is not supported (element " + el + ")");
            Shell s;
            s.x = mol.xyz[3 * a];
            s.y = mol.xyz[3 * a + 1];
            s.z = mol.xyz[3 * a + 2];
            s.L = cs.L;
            s.bf0 = bf;
            s.atom = a;
            s.exps = cs.e;
            s.coef = cs.c;
            finish_shell(s);
            bf += ncart(s.L);
            b.shells.push_back(std::move(s));
        }
    }
    b.K = bf;
    return b;
}

Basis basis_from_functions(const hfx_functions& f)
{
    if (f.K <= 0 || !f.centres || !f.lmn || !f.prim_offset || !f.alpha || !f.coeff || !f.norm)
        throw Error(HFX_ERR_INVALID, "hfx_functions: all arrays are required and K > 0");
    Basis b;
    int i = 0;
    while (i < f.K) {
        int L = f.lmn[3 * i] + f.lmn[3 * i + 1] + f.lmn[3 * i + 2];
        if (L < 0 || L > kMaxL) throw Error(HFX_ERR_UNSUPPORTED, "basis function with L outside 0..3");
        int nc = ncart(L);
        if (i + nc > f.K) throw Error(HFX_ERR_BASIS, "basis functions do not form complete Cartesian shells");
        int p0 = f.prim_offset[i], np = f.prim_offset[i + 1] - p0;
        if (np <= 0) throw Error(HFX_ERR_BASIS, "basis function without primitives");
        Shell s;
        s.x = f.centres[3 * i];
        s.y = f.centres[3 * i + 1];
        s.z = f.centres[3 * i + 2];
        s.L = L;
        s.bf0 = i;
        s.atom = -1;
        s.exps.assign(f.alpha + p0, f.alpha + p0 + np);
        s.coef.assign(f.coeff + p0, f.coeff + p0 + np);
        s.w.assign((size_t)nc * np, 0.0);
        for (int c = 0; c < nc; ++c) {
            int fi = i + c;
            int lx, ly, lz;
            component(L, c, lx, ly, lz);
            if (f.lmn[3 * fi] != lx || f.lmn[3 * fi + 1] != ly || f.lmn[3 * fi + 2] != lz ||
                f.centres[3 * fi] != s.x || f.centres[3 * fi + 1] != s.y || f.centres[3 * fi + 2] != s.z ||
                f.prim_offset[fi + 1] - f.prim_offset[fi] != np)
                throw Error(HFX_ERR_BASIS, "basis functions do not form complete Cartesian shells");
            int q0 = f.prim_offset[fi];
            for (int k = 0; k < np; ++k) {
                if (f.alpha[q0 + k] != s.exps[k])
                    throw Error(HFX_ERR_BASIS, "basis functions of one shell have different exponents");
                s.w[(size_t)c * np + k] = f.coeff[q0 + k] * f.norm[q0 + k];
            }
        }
        b.shells.push_back(std::move(s));
        i += nc;
    }
    b.K = f.K;
    return b;
}

double nuclear_repulsion(const Basis& b)
{
    double E = 0.0;
    int n = (int)b.atom_Z.size();
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) {
            double dx = b.atom_xyz[3 * i] - b.atom_xyz[3 * j], dy = b.atom_xyz[3 * i + 1] - b.atom_xyz[3 * j + 1],
                   dz = b.atom_xyz[3 * i + 2] - b.atom_xyz[3 * j + 2];
            E += b.atom_Z[i] * b.atom_Z[j] / std::sqrt(dx * dx + dy * dy + dz * dz);
        }
    return E;
}

}  // namespace hfx
