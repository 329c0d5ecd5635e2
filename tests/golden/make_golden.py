"""Generates the golden fixtures of this directory from the CPU oracle.

The reference (Julia) cannot run here, so the fixtures come from the oracle
(oracle/gridap_oracle.py), which tests/test_oracle_kats.py pins against the
reference's own known-answer tests (test/FESpacesTests.jl, test/PoissonTests.jl,
test/sequential/PeriodicBCsTests.jl).  Run:  python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent / "oracle"))
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE))
import gridap_oracle as go  # noqa: E402
from helpers import make_problem  # noqa: E402

CASES = {
    # test/FESpacesTests.jl: (0,4)^2, 4x4 cells, Q1, u = x+y on the boundary, l = 0
    "fespaces_q1_2x2": dict(dim=2, n=(4, 4), parts=(2, 2), order=1, f=0.0, u=lambda x, y: x + y,
                            domain=(0, 4, 0, 4)),
    # test/PoissonTests.jl (all-Dirichlet variant): Q2, u = (x+y)^2, f = -4
    "poisson_q2_2x2": dict(dim=2, n=(4, 4), parts=(2, 2), order=2, f=-4.0, u=lambda x, y: (x + y) ** 2,
                           domain=(0, 4, 0, 4)),
    # 3D Q1 lognormal kappa, f = 1, homogeneous Dirichlet, parts (2,2,2)
    "diffusion_q1_3d": dict(dim=3, n=(6, 5, 4), parts=(2, 2, 2), order=1, seed=7, f=1.0),
}


def dump(name, spec, strategy):
    pb = make_problem(**spec)
    fe = go.build_fespace(pb)
    mats = go.assemble(pb, fe, strategy)
    x = go.solve_lu(mats, fe.dofs[0].ngdofs)
    out = {"ngdofs": fe.dofs[0].ngdofs, "x": x}
    for p, (d, M) in enumerate(zip(fe.dofs, mats)):
        out[f"p{p}_gid"] = d.ldof_to_gdof
        out[f"p{p}_owner"] = d.ldof_to_owner
        out[f"p{p}_rowptr"] = M.rowptr
        out[f"p{p}_colidx"] = M.colidx
        out[f"p{p}_vals"] = M.vals
        out[f"p{p}_b"] = M.b
        out[f"p{p}_grow_gid"] = M.row_ghost_gids
        out[f"p{p}_grow_owner"] = M.row_ghost_owner
        out[f"p{p}_gcol_gid"] = M.col_ghost_gids
        out[f"p{p}_gcol_owner"] = M.col_ghost_owner
    np.savez_compressed(HERE / f"{name}_{strategy}.npz", **out)


if __name__ == "__main__":
    for name, spec in CASES.items():
        for strategy in ("sub", "full"):
            dump(name, spec, strategy)
            print("wrote", name, strategy)
