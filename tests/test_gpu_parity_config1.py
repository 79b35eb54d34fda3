"""Per-result parity at the first benchmarked configuration: the R = 2 nm, H = 8 nm nanotip on
a 20 x 20 x 2 nm slab with the vacuum up to 60 nm (Q1, 2.8e5 DoFs), applied field 1 GV/m,
phi = 0 on the metal, field interpolated onto all of its surface atoms (rank 1, the
reference default).

The oracle solves the reference's system with deal.II's SSOR(1.2)-CG restated
(src/DealSolver.cpp:443-459), restarted from its true residual until that stops falling,
recovers and smooths the nodal field (src/Interpolator.cpp:125-170) and locates/interpolates
the atoms sequentially (src/SolutionReader.cpp:136-165). Against it, per solver and tolerance:

* the relative residual of the GPU solution in the oracle's own system, evaluated
  compensated (Dot2), within the tolerance plus twice the FP64 floor 2^-53 |(|b| + |A||x|)|
  / |b| (the two assemblies sum element contributions in different orders, which moves the
  system by that much; on this mesh the floor is ~2e-12, so a 1e-12 solve ends on it);
* the solver's status: converged (1) or at the FP64 floor (2);
* located cells: bit-exact;
* max |dphi| at the atoms below 0.01 x t x max |phi| and max relative |dE| at the atoms
  (points whose field is above 1e-3 of the largest; atoms located in metal carry the empty
  value 0) below 5 x t, with t = max(tol, 2 x floor).

The bounds are several times the errors measured on a GB300 (stated in the design notes).
Solvers: the default FP64 CG with the FP32 multigrid preconditioner (precision 2) and FP32
Jacobi-PCG with FP64 refinement (precision 1), at 1e-9 and 1e-12.
"""
import json
import os

import numpy as np
import pytest

import femocs_gb300 as fg
import oracle as orc
from oracle import pipeline

pytestmark = pytest.mark.gpu
E0 = 0.1  # the Neumann value -E0 of a 1 GV/m applied field, E0 = -0.1 V/A


@pytest.fixture(scope="module")
def config1():
    m = fg.Mesh.synthetic(**fg.CONFIG1)
    atoms, types = fg.synth_atoms(fg.CONFIG1, seed=12345)
    surf = np.ascontiguousarray(atoms[types == 2])
    sol, info = pipeline.reference_solution(m, E0, rel_tol=1e-13)
    ref_cells, ref_out = orc.locate_interpolate(pipeline.tables(m, sol), 1, surf)
    return m, surf, sol, info, ref_cells, ref_out


@pytest.mark.parametrize("precision,tol", [(2, 1e-9), (2, 1e-12), (1, 1e-9), (1, 1e-12)])
def test_config1_results_match_reference_solve(config1, precision, tol):
    m, surf, sol, info, ref_cells, ref_out = config1
    f = fg.Field(m)
    f.setup(E0)
    f.assemble(True, False)
    rc, st = f.solve(precision=precision, rel_tol=tol, max_iter=100000)
    assert rc > 0 and st["status"] in (1, 2), st
    system, v2n = info["system"], info["vertex2node"]
    x = f.phi_nodes()[v2n]
    bnorm = float(np.linalg.norm(system.rhs))
    r_abs, floor_abs = system.residual(x)
    r, floor = r_abs / bnorm, floor_abs / bnorm
    f.extract(smoothen=True)
    cells, out = f.interpolate(surf, rank=1)
    p = pipeline.point_parity(cells, out, ref_cells, ref_out)
    p.update(precision=precision, tol=tol, status=st["status"], iterations=st["iterations"],
             rel_residual_gpu=st["rel_residual"], rel_residual_oracle=r, rel_floor=floor,
             oracle_ssor_iterations=info["ssor_iterations"], oracle_rel_residual=info["rel_residual"])
    print(json.dumps(p))
    out_dir = os.environ.get("FGB_PARITY_OUT")
    if out_dir:
        with open(os.path.join(out_dir, f"parity_config1_p{precision}_{tol:g}.json"), "w") as fh:
            json.dump(p, fh)
    assert r <= 1.1 * tol + 2 * floor, (r, floor)
    assert st["status"] == 1 or tol < 2 * floor, st  # the floor status only where the floor is above tol
    assert p["cells_bit_exact"], p["cells_differing"]
    t = max(tol, 2 * floor)
    assert p["max_abs_dphi"] <= 0.01 * t * np.abs(sol[:, 4]).max(), p
    assert p["max_rel_dE"] <= 5 * t, p
