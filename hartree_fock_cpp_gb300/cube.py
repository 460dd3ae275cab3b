"""Electron density and orbitals on grids, and cube files.

GPU counterparts of the reference's density3d / homo_lumo_3d / orbital_wf
(cube.hpp:137-380) and write_cube_file (cube.hpp:383-450): the values come
from hfx_grid_density / hfx_grid_orbital / hfx_points_eval (csrc/hfx_grid.cu);
a cube is a dict {field, origin, dx, res} like the reference's cube_data
(types.hpp:108), field in (i * res + j) * res + k order.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import HfxError, check, lib, ptr

_ELEMENTS = ["H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na", "Mg", "Al", "Si", "P", "S", "Cl", "Ar",
             "K", "Ca", "Sc", "Ti", "V", "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge", "As", "Se", "Br", "Kr"]


def _mat(M, K):
    M = np.ascontiguousarray(M, dtype=np.float64).reshape(-1)
    if M.size != K * K:
        raise HfxError(1, "Mismatch between matrix and basis sizes")
    return M


def density3d(basis, density_matrix, center, L, resolution, device=0):
    """rho on the res^3 box around center (cube.hpp:221-258)."""
    P = _mat(density_matrix, basis.K)
    c = np.ascontiguousarray(center, dtype=np.float64)
    out = np.zeros(int(resolution) ** 3)
    check(lib.hfx_grid_density(basis.ref(), int(device), ptr(P), ptr(c), float(L), int(resolution), ptr(out)))
    return {"field": out, "origin": c - L / 2, "dx": L / (resolution - 1), "res": int(resolution)}


def orbital3d(basis, coeff_matrix, index, center, L, resolution, device=0):
    """psi_index on the res^3 box (the evaluation inside homo_lumo_3d)."""
    C = _mat(coeff_matrix, basis.K)
    if index < 0 or index >= basis.K:
        raise HfxError(1, "orbital index out of range")
    c = np.ascontiguousarray(center, dtype=np.float64)
    out = np.zeros(int(resolution) ** 3)
    check(lib.hfx_grid_orbital(basis.ref(), int(device), ptr(C), int(index), ptr(c), float(L), int(resolution),
                               ptr(out)))
    return {"field": out, "origin": c - L / 2, "dx": L / (resolution - 1), "res": int(resolution)}


def homo_lumo_3d(basis, coeff_mats, occupation, center, L, res, homo_or_lumo=True, alpha_or_beta=True, device=0):
    """cube.hpp:271-380: the HOMO (occupation - 1) or LUMO (occupation) of
    the alpha (first) or beta (second) coefficients."""
    Ca, Cb = coeff_mats
    if np.size(Ca) != np.size(Cb):
        raise HfxError(1, "Coefficient matrices dimension mismatch")
    if res < 2:
        raise HfxError(1, "resolution must be at least 2")
    occ = occupation[0] if alpha_or_beta else occupation[1]
    C = Ca if alpha_or_beta else Cb
    idx = occ - 1 if homo_or_lumo else occ
    return orbital3d(basis, C, idx, center, L, res, device)


def points_eval(basis, matrix, xyz, index=-1, device=0):
    """rho (index < 0, matrix = P) or psi_index (matrix = C) at explicit points
    (n x 3, bohr), e.g. the planes of square_points (cube.hpp:171-218)."""
    M = _mat(matrix, basis.K)
    r = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
    n = r.size // 3
    out = np.zeros(n)
    check(lib.hfx_points_eval(basis.ref(), int(device), ptr(M), int(index), ptr(r), ctypes.c_longlong(n), ptr(out)))
    return out


def write_cube_file(filename, cube, atoms, comment="Generated by HF code"):
    """Gaussian cube file in the layout of the reference's write_cube_file
    (cube.hpp:383-450): two comment lines, atom count + origin, the three
    grid vectors, one line per atom (Z, charge, x, y, z), then the values in
    (i, j, k) order, z fastest, six per line.  atoms: [(symbol, (x, y, z))]."""
    N = cube["res"]
    field = np.asarray(cube["field"]).reshape(-1)
    if field.size != N ** 3:
        raise HfxError(1, "cube field size does not match resolution")
    o = cube["origin"]
    dx = cube["dx"]
    with open(filename, "w") as f:
        f.write(comment + "\n")
        f.write("Electron density / molecular orbital cube\n")
        f.write("%d %g %g %g\n" % (len(atoms), o[0], o[1], o[2]))
        f.write("%d %g 0.0 0.0\n" % (N, dx))
        f.write("%d 0.0 %g 0.0\n" % (N, dx))
        f.write("%d 0.0 0.0 %g\n" % (N, dx))
        for sym, R in atoms:
            Z = _ELEMENTS.index(sym) + 1
            f.write("%d %g %g %g %g\n" % (Z, float(Z), R[0], R[1], R[2]))
        vals = ["%.8e " % v for v in field]
        for s in range(0, len(vals), 6):
            f.write("".join(vals[s:s + 6]) + ("\n" if s + 6 <= len(vals) else ""))
        f.write("\n")
