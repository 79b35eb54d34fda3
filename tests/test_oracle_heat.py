"""Known answers of the oracle's current/heat restatement on the bulk hexahedra (no GPU):
a uniform surface current through a flat slab gives a potential linear in z (exact for Q1), and
a body without current and heat flux stays at the ambient temperature."""
import numpy as np

import femocs_gb300 as fg
from oracle.heat_oracle import BulkSystem

FLAT = dict(radius=0.0, height=0.0, box_half=20.0, slab=8.0, top=40.0, h=4.0, growth=1.4, margin=0.0)
SMALL = dict(radius=5.0, height=14.0, box_half=18.0, slab=4.0, top=40.0, h=4.0, growth=1.6, margin=3.0)
TAB_T = np.array([200.0, 400.0, 800.0, 1600.0])
TAB_RHO = np.array([1.0e-8, 1.7e-8, 3.5e-8, 7.0e-8])


def bulk(spec):
    m = fg.Mesh.synthetic(**spec)
    return m, BulkSystem(m.export("node_xyz"), m.export("hex_nodes"), m.export("hex_marker"))


def test_flat_slab_potential_is_linear():
    m, b = bulk(FLAT)
    j = 0.01
    phi = b.current(np.full(len(b.surface), j))
    z = b.xyz[:, 2]
    assert len(b.surface) > 0 and b.fixed.any()
    np.testing.assert_allclose(phi, j * (z - z.min()), rtol=0, atol=1e-10)


def test_unheated_body_stays_at_ambient():
    m, b = bulk(SMALL)
    T0 = np.full(b.n, 300.0)
    T = b.heat(T0, np.zeros(b.n), 1e-12, np.zeros(len(b.surface)), TAB_T, TAB_RHO, 2.44e-8, 3.4496e-24, 300.0)
    np.testing.assert_allclose(T, 300.0, rtol=1e-12)


def test_bulk_marking_follows_the_reference_rules():
    m, b = bulk(SMALL)
    c = b.surface_centroids
    # the copper bottom is at z min; the surface covers the slab top and the tip
    assert np.isclose(b.xyz[b.fixed, 2], b.xyz[:, 2].min()).all()
    assert c[:, 2].max() > 0.9 * SMALL["height"] and (c[:, 2] > b.xyz[:, 2].min() + 1e-6).all()
