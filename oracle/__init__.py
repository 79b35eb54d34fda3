"""CPU oracle of the femocs_gb300 field-solve path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline arm may import this
package; the product path never does. Parity of the FEM solve (assembly, boundary
conditions, SSOR-CG) is unpinned against the reference (it runs in deal.II 9.2, which is
absent); location, interpolation, nodal field and smoothing are pinned against golden
vectors produced by the reference's own compiled sources (see oracle/ref_driver.cpp and
tests/golden/make_golden.py).
"""
from .oracle_lib import *  # noqa: F401,F403
from . import pipeline  # noqa: F401
