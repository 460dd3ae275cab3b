"""Generate tests/golden/grid_golden.json from the reference's own grid
evaluation: include/cube.hpp (function_eval, electron_density, orbital_wf,
box_points) compiled unchanged into oracle/_ref/libhfref_grid.so.

TEST INFRASTRUCTURE.  Nothing at test time reads the reference.  The density
and coefficient matrices are closed-form (platform-independent) functions of
the indices, restated in the tests that read the fixture:
  P_ij = cos(0.37 i + 0.53 j) + cos(0.37 j + 0.53 i)   (symmetric)
  C_ij = sin(0.11 i j + 0.7 i)
Run from the repository root:
  HF_REFERENCE=<reference checkout> python tests/golden/make_grid_golden.py
"""
import importlib.util
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
import oracle as O  # noqa: E402

_spec = importlib.util.spec_from_file_location("hfx_workloads",
                                               os.path.join(REPO, "hartree_fock_cpp_gb300", "workloads.py"))
W = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(W)


def matrices(K):
    i, j = np.meshgrid(np.arange(K), np.arange(K), indexing="ij")
    P = np.cos(0.37 * i + 0.53 * j) + np.cos(0.37 * j + 0.53 * i)
    C = np.sin(0.11 * i * j + 0.7 * i)
    return P, C


CASES = [("water_ccpvdz", W.water(), "cc-pVDZ", (0.1, -0.2, 0.3), 6.0, 5, 4),
         ("nacl_ccpvtz", W.nacl_scan(8)[3], "cc-pVTZ", (0.0, 0.2, 2.0), 8.0, 5, 13)]
POINTS = [[0.0, 0.0, 0.0], [0.3, -0.2, 0.5], [1.1, 0.7, -0.4], [-0.8, 1.9, 2.2], [2.5, -1.5, 4.0],
          [0.05, 0.0, 4.46], [-3.0, 0.4, 1.0]]


def main():
    if O.reference_checkout() is None:
        sys.exit("set HF_REFERENCE to a checkout of the reference")
    O.build_oracle()
    out = []
    for name, cfg, basis, center, L, res, col in CASES:
        r = O.RefGridLib()
        K = r.build(cfg, basis, O.BASIS_PATH)
        P, C = matrices(K)
        box = r.box_points(center, L, res)
        out.append(dict(name=name, config=cfg, basis=basis, K=K, center=center, L=L, res=res, column=col,
                        box=box.tolist(), rho_box=r.points(P, -1, box).tolist(),
                        psi_box=r.points(C, col, box).tolist(), points=POINTS,
                        rho_points=r.points(P, -1, np.array(POINTS)).tolist(),
                        psi_points=r.points(C, col, np.array(POINTS)).tolist()))
    json.dump(out, open(os.path.join(HERE, "grid_golden.json"), "w"))


if __name__ == "__main__":
    main()
