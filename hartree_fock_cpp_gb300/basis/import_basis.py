"""Copy the per-element basis-set tables (STO-3G, 6-31G, 6-31G*, cc-pVDZ,
cc-pVTZ; H-Ar) out of a checkout of KLYYCYNN/hartree_fock_cpp into this
package, so that the library finds its basis sets on machines where that
checkout does not exist.

The tables are published basis-set data (contraction exponents and
coefficients), kept in the reference's own CSV layout
(`shell_id,L,primitive_id,exponent,coefficient`, one primitive per row; see
the reference's basis/<set>/<El>.csv and its reader basis.hpp:157-262), because
the engine must build exactly the same basis functions as the reference for
its ERIs to agree.  Conversion reports (`_summary.csv`, `_block_report.json`,
`n_basis.csv`) are not copied.

Usage: python import_basis.py <reference checkout root>
"""
import os
import shutil
import sys

SETS = ["STO-3G", "6-31G", "6-31G*", "cc-pVDZ", "cc-pVTZ"]


def main(root):
    here = os.path.dirname(os.path.abspath(__file__))
    for s in SETS:
        src = os.path.join(root, "basis", s)
        dst = os.path.join(here, s)
        os.makedirs(dst, exist_ok=True)
        for name in sorted(os.listdir(src)):
            if not name.endswith(".csv") or name.startswith("_") or name == "n_basis.csv":
                continue
            shutil.copyfile(os.path.join(src, name), os.path.join(dst, name))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python import_basis.py <reference checkout root>")
    main(sys.argv[1])
