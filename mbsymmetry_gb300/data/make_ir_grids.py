"""Regenerate the committed IR sampling grids (``ir_<nts>.npz``).

The grids are deterministic outputs of :mod:`mbsymmetry_gb300.irbasis`;
they are committed because the singular value expansion takes tens of
seconds per grid.  Run:  python -m mbsymmetry_gb300.data.make_ir_grids
"""
import os

import numpy as np

from mbsymmetry_gb300.irbasis import make_ir_grid

HERE = os.path.dirname(os.path.abspath(__file__))
GRIDS = (62, 100, 120, 150)


def main():
    for nts in GRIDS:
        lam, ir = make_ir_grid(nts)
        np.savez_compressed(os.path.join(HERE, f"ir_{nts}.npz"), Lambda=lam,
                            **{k.replace("/", "__"): v for k, v in ir.items()})
        print(nts, lam)


if __name__ == "__main__":
    main()
