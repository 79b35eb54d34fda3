"""Iterations of the reference's solver to a 1e-9 relative residual on the benchmarked
systems -- TEST INFRASTRUCTURE ONLY.

    python -m oracle.ssor_iterations config2 [--order 2] [--tol 1e-9]

Builds the workload entirely in the oracle (oracle/workload.py mesh, oracle/mesh_prep.py
split, the Q1 system of oracle/femocs_oracle.c or the Q2 system of oracle/q2_oracle.c, both
numbered the way the reference's DoF handler meets the cells), runs deal.II's SolverCG +
PreconditionSSOR(1.2) restated (src/DealSolver.cpp:443-459) from phi = 0 until
||b - A x|| <= tol ||b||, and records the iteration count with the true residual in
oracle/ssor_iterations.json. The benchmark's CPU reference arm times a bounded number of
iterations of the same solver on the same system and scales by this count, because a full
solve of the Q2 system takes over an hour on one core.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import time

import numpy as np

from . import oracle_lib as orc
from . import mesh_prep, workload

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "ssor_iterations.json")
E0 = -0.1  # 1 GV/m; the Neumann value on the top is -E0


def build_system(spec, order):
    """(oracle mesh, system) of a workload, Q1 or Q2, the top Neumann value -E0"""
    om = mesh_prep.OracleMesh(*workload.tet_mesh(spec))
    xyz = om.export("node_xyz").reshape(-1, 3)
    cells = om.export("hex_nodes").reshape(-1, 8)[om.export("vac_cells")]
    if order == 2:
        return om, orc.Q2CSystem(xyz, cells, -E0)
    from .pipeline import vacuum_inputs
    vx, vc, _ = vacuum_inputs(om)
    return om, orc.System(vx, vc, -E0)


def load_fixture():
    try:
        with open(FIXTURE) as f:
            return json.load(f)
    except OSError:
        return {}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("workload", choices=["config1", "config2"])
    ap.add_argument("--order", type=int, default=0, help="element order (default: 2 for config2, 1 for config1)")
    ap.add_argument("--tol", type=float, default=1e-9)
    args = ap.parse_args()
    order = args.order or (2 if args.workload == "config2" else 1)
    spec = workload.CONFIG2 if args.workload == "config2" else workload.CONFIG1
    t0 = time.perf_counter()
    _, s = build_system(spec, order)
    t_build = time.perf_counter() - t0
    bnorm = float(np.linalg.norm(s.rhs))
    t0 = time.perf_counter()
    it, x = s.ssor_cg(1.2, args.tol * bnorm, 100000)
    t_solve = time.perf_counter() - t0
    r = float(np.linalg.norm(s.spmv(x) - s.rhs) / bnorm)
    rec = {"workload": args.workload, "order": order, "n_dofs": int(s.n), "nnz": int(len(s.col)),
           "rel_tol": args.tol, "iterations": int(it), "true_rel_residual": r, "solve_s": t_solve,
           "s_per_iteration": t_solve / max(abs(it), 1), "build_s": t_build, "threads": 1,
           "host": f"{platform.machine()} {platform.processor() or ''}".strip(),
           "how": "oracle SSOR(1.2)-CG from phi = 0 on the oracle-built system, stop ||b - A x|| <= tol ||b|| "
                  "(recursive residual, as deal.II's SolverCG)"}
    print(json.dumps(rec), flush=True)
    fx = load_fixture()
    fx[f"{args.workload}_q{order}"] = rec
    with open(FIXTURE, "w") as f:
        json.dump(fx, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
