"""Host-side pieces that need no GPU: C ABI exports, mesh import, configuration parsing,
synthetic workload determinism."""
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

import femocs_gb300 as fg
import oracle as orc
from femocs_gb300._lib import LIB_PATH, exported_symbols

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "femocs_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(\w+)\s*\([^;{]*\)\s*;", txt)))


def test_library_exports_every_declared_symbol():
    out = subprocess.run(["nm", "-D", "--defined-only", LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = set(line.split()[-1] for line in out.splitlines() if line.strip())
    declared = header_functions()
    assert len(declared) >= 40
    missing = [f for f in declared if f not in exported]
    assert not missing, missing
    # the Python binding declares prototypes for all of them
    assert set(declared) <= set(exported_symbols())


def test_reference_wrapper_names_present():
    # the symbols of the reference's include/Femocs_wrap.h
    names = ["create_femocs", "delete_femocs", "femocs_run", "femocs_import_file", "femocs_import_parcas",
             "femocs_import_atoms", "femocs_interpolate_elfield", "femocs_interpolate_surface_elfield",
             "femocs_interpolate_phi", "femocs_export_data", "femocs_export_int", "femocs_interpolate",
             "femocs_parse_int", "femocs_parse_double", "femocs_parse_string"]
    assert set(names) <= set(header_functions())


def test_library_loads_without_gpu():
    lib = fg.load()
    assert lib.femocs_last_error() is not None


def test_gmsh_roundtrip_and_arrays_agree():
    m = fg.Mesh.synthetic(radius=5.0, height=15.0, box_half=15.0, slab=5.0, top=40.0, h=4.0, growth=1.5, margin=3.0)
    s = m.sizes()
    xyz = m.export("node_xyz").reshape(-1, 3)[: s["n_tetnodes"]]
    tets = m.export("tet_nodes")
    mk = m.export("tet_marker")
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "m.msh")
        orc.write_msh(p, xyz, tets, mk)
        m2 = fg.Mesh.read_gmsh(p)
    m3 = fg.Mesh.from_arrays(xyz, tets, mk)
    for name in ("hex_nodes", "hex_marker", "tet_nbor", "node_xyz", "tet_det", "hex_coeffs", "voro_idx"):
        a = m.export(name)
        assert np.array_equal(a, m2.export(name)), name
        assert np.array_equal(a, m3.export(name)), name


def test_mesh_invariants():
    m = fg.Mesh.synthetic(radius=8.0, height=25.0, box_half=30.0, slab=6.0, top=80.0, h=4.0, growth=1.4, margin=4.0)
    s = m.sizes()
    assert s["n_hexs"] == 4 * s["n_tets"]
    hexs = m.export("hex_nodes").reshape(-1, 8)
    hm = m.export("hex_marker")
    tets = m.export("tet_nodes").reshape(-1, 4)
    # hex 4t+k carries tet vertex k and the marker +-(1+vertex)
    k = np.arange(len(hexs)) % 4
    v = tets[np.arange(len(hexs)) // 4, k]
    assert np.all(np.abs(hm) == v + 1)
    assert np.all((hexs == v[:, None]).sum(1) == 1)
    nb = m.export("tet_nbor").reshape(-1, 4)
    # neighbour j shares the face opposite vertex j
    for t in range(0, len(tets), 97):
        for j in range(4):
            u = nb[t, j]
            if u >= 0:
                assert set(np.delete(tets[t], j)) <= set(tets[u])
    # every vacuum tet has at least one vacuum hex node set; vacuum cells = positive markers
    assert np.array_equal(np.flatnonzero(hm > 0), m.export("vac_cells"))


def test_invalid_mesh_is_rejected():
    with pytest.raises(RuntimeError):
        fg.Mesh.from_arrays(np.zeros((3, 3)), np.array([[0, 1, 2, 7]]), np.array([3]))
    with pytest.raises(RuntimeError):
        fg.Mesh.read_gmsh("/nonexistent/file.msh")


def test_synthetic_workloads_are_deterministic():
    kw = dict(radius=10.0, height=30.0, box_half=30.0, slab=8.0, top=100.0, h=5.0, growth=1.4, margin=5.0)
    a1, t1 = fg.synth_atoms(kw, seed=5)
    a2, t2 = fg.synth_atoms(kw, seed=5)
    assert np.array_equal(a1, a2) and np.array_equal(t1, t2)
    assert (t1 == 2).sum() > 100
    p = fg.synth_probes(kw, 500, seed=3)
    assert p.shape == (500, 3)
    assert np.all(p[:, 2] >= 0) and np.all(np.abs(p[:, :2]) <= kw["box_half"])


def test_config_parser_semantics(tmp_path):
    conf = tmp_path / "femocs.in"
    conf.write_text("ELFIELD = -0.12   ! comment\nfield_ncg 77\n# hidden 5\nsmoothen_field false\n"
                    "mesh_file  /x/y.msh\nfemocs_end\nradius 9\n")
    f = fg.Femocs(str(conf))
    assert f.parse_double("elfield") == (0, -0.12)
    assert f.parse_double("field_ncg") == (0, 77.0)
    assert f.parse_double("hidden")[0] == 1
    assert f.parse_double("radius")[0] == 1  # after femocs_end


def test_q2_structure_matches_independent_enumeration():
    """Host Q2 structure (DoF count, sparsity) against the numpy restatement's own
    enumeration of vertex/edge/face/interior entities on a small mesh."""
    from oracle.q2_oracle import Q2System
    spec = dict(radius=3.0, height=8.0, box_half=10.0, slab=3.0, top=20.0, h=3.0, growth=1.7, margin=2.0)
    m = fg.Mesh.synthetic(**spec)
    q = m.q2_sizes()
    s = Q2System(m.export("node_xyz"), m.export("hex_nodes"), m.export("vac_cells"), -0.1)
    assert q["n_dofs"] == s.n and q["nnz"] == s.nnz_pattern
    assert q["n_top_faces"] > 0 and s.fixed.sum() > 0


def test_structure_builders_do_not_depend_on_thread_count():
    """The parallel phases of the Q1 (vacuum, bulk) and Q2 structure builders give the same
    structure as a single thread (every array hashed by fgb_mesh_structure_digest)."""
    import subprocess
    import sys
    code = ("import femocs_gb300 as fg; from femocs_gb300._lib import load; "
            "m = fg.Mesh.synthetic(radius=5.0, height=14.0, box_half=18.0, slab=4.0, top=40.0, h=3.0, growth=1.5, "
            "margin=3.0); print([load().fgb_mesh_structure_digest(m.h, o, r) for o, r in ((1, 0), (1, 1), (2, 0))])")
    env_root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    outs = []
    for nt in ("1", "5"):
        env = dict(os.environ, OMP_NUM_THREADS=nt, PYTHONPATH=env_root)
        outs.append(subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, check=True,
                                   timeout=300).stdout.strip())
    assert outs[0] == outs[1] and outs[0].startswith("[")
    # and the structures themselves are pinned: the numbering (Morton order, windows by row
    # length) and every table of this mesh, for Q1 vacuum, Q1 bulk and Q2
    pinned = [0x91bc05e014367b7f, 0x45728c20f1713063, 0xe384d55500756846]
    assert [int(v) & 0xffffffffffffffff for v in eval(outs[0])] == pinned


@pytest.mark.parametrize("cells,max_dofs", [(256, 4096), (64, 1024), (16, 200), (1, 27)])
def test_cell_blocks_invariants(cells, max_dofs):
    """The Q2 cell blocks (host-built) pass every invariant the element-by-element kernels rely
    on (validated in the library), for the default limits and for limits that force blocks to
    be halved down to a single hex: every DoF is complete in one block or split with one slot
    per block."""
    m = fg.Mesh.synthetic(radius=5.0, height=14.0, box_half=18.0, slab=4.0, top=40.0, h=3.0, growth=1.5, margin=3.0)
    q = m.q2_sizes()
    cb = m.cell_blocks(cells, max_dofs)
    assert cb["n_complete"] + cb["n_split"] == q["n_dofs"]
    assert cb["max_cells"] <= cells and cb["max_dofs"] <= max_dofs
    assert cb["n_local"] >= q["n_dofs"] and cb["n_slots"] >= 2 * cb["n_split"]
    if cells == 1:
        assert cb["n_blocks"] == m.sizes()["n_vac_cells"]


def test_cell_blocks_reject_bad_limits():
    m = fg.Mesh.synthetic(radius=5.0, height=14.0, box_half=18.0, slab=4.0, top=40.0, h=4.0, growth=1.6, margin=3.0)
    with pytest.raises(RuntimeError):
        m.cell_blocks(4096, 4096)   # 27 x 4096 items do not fit 16 bits
    with pytest.raises(RuntimeError):
        m.cell_blocks(256, 8192)    # a block's DoFs must fit the kernels' 4096


def test_cell_blocks_do_not_depend_on_thread_count():
    import subprocess
    import sys
    code = ("import femocs_gb300 as fg; m = fg.Mesh.synthetic(radius=5.0, height=14.0, box_half=18.0, slab=4.0, "
            "top=40.0, h=3.0, growth=1.5, margin=3.0); print(m.cell_blocks(64, 1024))")
    env_root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    outs = []
    for nt in ("1", "5"):
        env = dict(os.environ, OMP_NUM_THREADS=nt, PYTHONPATH=env_root)
        outs.append(subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, check=True,
                                   timeout=300).stdout.strip())
    assert outs[0] == outs[1] and "digest" in outs[0]
    # pinned: the block cuts, local DoFs, items and slot numbering of this mesh
    assert eval(outs[0])["digest"] == 1488237973323863000
