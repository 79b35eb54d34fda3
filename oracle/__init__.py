"""CPU oracle of the femocs_gb300 field-solve path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's parity and CPU legs may import this
package; the product path never does. The FEM solve (assembly, boundary conditions,
SSOR-CG) cannot be pinned bit for bit against the reference (it runs in deal.II 9.2, which
is absent); it is pinned to the reference's own analytic answer for a hemisphere on a plane
(tests/test_oracle_analytic.py). Location, interpolation, nodal field and smoothing are
pinned against golden vectors produced by the reference's own compiled sources (see
oracle/ref_driver.cpp and tests/golden/make_golden.py). The workload, the tet -> hex split,
the tables and the Q1/Q2 systems can be built here without the product (workload.py,
mesh_prep.py, q2_oracle.c) for the CPU reference arm of the benchmark.
"""
from .oracle_lib import *  # noqa: F401,F403
from . import pipeline  # noqa: F401,E402
