"""Serving loop: MD runs with resident meshes submit solves that are batched continuously.

Checks: a request's result is the same alone and in the mix (bit for bit with the autotuner
off: per-mesh reductions make a mesh's arithmetic independent of the other meshes in a
launch); served results match the single-mesh pipeline within the solve tolerance (cells
identical); Poisson arrivals complete with ordered timestamps, overlap on the device and
warm starts cut iterations; runs that free memory does not admit stay pending."""
import numpy as np
import pytest

import femocs_gb300 as fg

pytestmark = pytest.mark.gpu
SPECS = [
    dict(radius=8.0, height=25.0, box_half=30.0, slab=6.0, top=80.0, h=4.0, growth=1.4, margin=4.0),
    dict(radius=10.0, height=35.0, box_half=40.0, slab=8.0, top=120.0, h=4.0, growth=1.35, margin=5.0),
    dict(radius=6.0, height=30.0, box_half=25.0, slab=5.0, top=70.0, h=3.5, growth=1.45, margin=4.0),
    dict(radius=12.0, height=30.0, box_half=40.0, slab=6.0, top=90.0, h=5.0, growth=1.4, margin=5.0),
]
FIELDS = [0.1, 0.2, 0.05, 0.15]
TOL = 1e-10


@pytest.fixture(scope="module")
def meshes():
    return [fg.Mesh.synthetic(**s) for s in SPECS]


def atoms_of(spec, n=1500, seed=3):
    atoms, types = fg.synth_atoms(spec, seed=seed)
    surf = atoms[types == 2]
    return np.ascontiguousarray(np.r_[surf, fg.synth_probes(spec, max(0, n - len(surf)), seed=seed)][:n])


def make_server(meshes, autotune=False, iters=3, **kw):
    b = fg.Batch(autotune=autotune)
    s = fg.Server(b, rel_tol=TOL, max_iter=400, iters_per_launch=iters, **kw)
    for i, (m, spec) in enumerate(zip(meshes, SPECS)):
        assert s.add_run(m, atoms_of(spec), seed=100 + i) == i
    assert s.place_pending() == len(meshes)
    return b, s


def test_alone_and_in_the_mix(meshes):
    b, s = make_server(meshes)
    s.start()
    s.submit(1, FIELDS[1], sigma=0.02)
    assert s.drain(120)
    s.stop()
    cells_alone, out_alone = s.last_result(1)
    rec = s.records()
    it_alone = int(rec["iterations"][0])
    for r in range(len(meshes)):
        s.reset_run(r)
    s.clear_records()
    s.start()
    # the same request for run 1 arrives while the other runs' requests are in flight
    s.submit(0, FIELDS[0], sigma=0.02)
    s.submit(2, FIELDS[2], sigma=0.02)
    s.submit(1, FIELDS[1], sigma=0.02)
    s.submit(3, FIELDS[3], sigma=0.02)
    assert s.drain(120)
    s.stop()
    rec = s.records()
    assert len(rec["id"]) == 4 and np.all(rec["status"] == 1)
    cells_mix, out_mix = s.last_result(1)
    assert int(rec["iterations"][rec["run"] == 1][0]) == it_alone
    np.testing.assert_array_equal(cells_mix, cells_alone)
    np.testing.assert_array_equal(out_mix, out_alone)


def test_alone_and_in_the_mix_autotuned(meshes):
    b, s = make_server(meshes, autotune=True)
    s.start()
    s.submit(2, FIELDS[2], sigma=0.02)
    assert s.drain(120)
    s.stop()
    cells_alone, out_alone = s.last_result(2)
    for r in range(len(meshes)):
        s.reset_run(r)
    s.start()
    for r in (0, 1, 2, 3):
        s.submit(r, FIELDS[r], sigma=0.02)
    assert s.drain(120)
    s.stop()
    cells_mix, out_mix = s.last_result(2)
    np.testing.assert_array_equal(cells_mix, cells_alone)
    scale_phi = np.abs(out_alone[:, 4]).max()
    scale_e = np.linalg.norm(out_alone[:, :3], axis=1).max()
    assert np.abs(out_mix[:, 4] - out_alone[:, 4]).max() <= 2e3 * TOL * scale_phi
    assert np.linalg.norm(out_mix[:, :3] - out_alone[:, :3], axis=1).max() <= 2e3 * TOL * scale_e


def test_served_result_matches_single_mesh_pipeline(meshes):
    b, s = make_server(meshes)
    s.start()
    s.submit(3, FIELDS[3], sigma=0.0)  # atoms not displaced: compare at the initial positions
    assert s.drain(120)
    s.stop()
    cells, out = s.last_result(3)
    f = fg.Field(meshes[3])
    f.setup(-FIELDS[3])
    f.assemble(True, False)
    rc, st = f.solve(precision=2, rel_tol=1e-12)
    f.extract(smoothen=True)
    cells_f, out_f = f.interpolate(atoms_of(SPECS[3]), rank=1)
    np.testing.assert_array_equal(cells, cells_f)
    assert np.abs(out[:, 4] - out_f[:, 4]).max() <= 2e3 * TOL * np.abs(out_f[:, 4]).max()
    e = np.linalg.norm(out_f[:, :3], axis=1).max()
    assert np.linalg.norm(out[:, :3] - out_f[:, :3], axis=1).max() <= 2e3 * TOL * e


def test_poisson_arrivals(meshes):
    b, s = make_server(meshes, autotune=True)
    s.start()
    s.run_poisson(rate=400.0, n=60, base_fields=FIELDS, sigma=0.02, seed=11)
    s.stop()
    rec = s.records()
    assert len(rec["id"]) == 60
    assert np.all(rec["status"] == 1)
    assert np.all(rec["rel_residual"] <= TOL)
    assert np.all(rec["t_submit"] <= rec["t_admit"]) and np.all(rec["t_admit"] <= rec["t_solved"])
    assert np.all(rec["t_solved"] <= rec["t_done"])
    info = s.info()
    assert info["max_in_flight"] >= 2 and info["solver_launches"] > 0
    # warm starts: a run's later requests (field within ~1% of its last one) need fewer
    # iterations than its first (cold) request
    order = np.argsort(rec["id"])
    runs, iters = rec["run"][order], rec["iterations"][order]
    first, later = [], []
    for r in range(len(meshes)):
        its = iters[runs == r]
        if len(its) > 1:
            first.append(its[0])
            later.extend(its[1:])
    assert np.median(later) < np.median(first)


def test_admission_by_free_memory(meshes):
    b = fg.Batch()
    s = fg.Server(b, rel_tol=TOL, hbm_reserve=1e15)
    s.add_run(meshes[0], atoms_of(SPECS[0]))
    assert s.place_pending() == 0 and s.run_info(0)["slot"] == -1
