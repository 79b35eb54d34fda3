"""The oracle's numpy restatement of the synthetic workload (oracle/workload.py) against the
product's generator: the tet mesh, the atoms with their surface types and the vacuum probes
must be identical bit for bit, so the CPU reference arm of the benchmark can build its inputs
without the product's library."""
import numpy as np
import pytest

import femocs_gb300 as fg
from oracle import workload

SMALL = dict(radius=6.0, height=24.0, box_half=24.0, slab=6.0, top=60.0, h=3.0, growth=1.5, margin=4.0)


@pytest.mark.parametrize("spec", [SMALL, fg.CONFIG1], ids=["small", "config1"])
def test_tet_mesh_equals_product(spec):
    xyz, tets, marker = workload.tet_mesh(spec)
    m = fg.Mesh.synthetic(**spec)
    s = m.sizes()
    assert len(tets) == s["n_tets"] and len(xyz) == s["n_tetnodes"]
    np.testing.assert_array_equal(tets.reshape(-1), m.export("tet_nodes"))
    np.testing.assert_array_equal(marker, m.export("tet_marker"))
    assert np.array_equal(xyz.reshape(-1).view(np.int64), m.export("node_xyz")[: 3 * len(xyz)].view(np.int64))


@pytest.mark.parametrize("spec", [SMALL, fg.CONFIG1], ids=["small", "config1"])
def test_atoms_and_probes_equal_product(spec):
    pos, types = workload.atoms(spec, seed=12345)
    pa, ta = fg.synth_atoms(spec, seed=12345)
    assert pos.shape == pa.shape
    assert np.array_equal(pos.view(np.int64), pa.view(np.int64))
    np.testing.assert_array_equal(types, ta)
    pr = workload.probes(spec, 3000, seed=777)
    assert np.array_equal(pr.view(np.int64), fg.synth_probes(spec, 3000, seed=777).view(np.int64))


def test_benchmark_specs_equal_product():
    assert workload.CONFIG1 == fg.CONFIG1 and workload.CONFIG2 == fg.CONFIG2
