"""Shared helpers of the test suite (golden loading, oracle tables from a product mesh)."""
import os

import numpy as np

import femocs_gb300 as fg
import oracle as orc  # noqa: F401
from oracle import pipeline

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SPEC_KEYS = ("radius", "height", "box_half", "slab", "top", "h", "growth", "margin")


def golden_cases():
    return sorted(f[len("golden_"):-4] for f in os.listdir(GOLDEN_DIR) if f.startswith("golden_") and f.endswith(".npz"))


def load_golden(name):
    g = dict(np.load(os.path.join(GOLDEN_DIR, f"golden_{name}.npz")))
    g["spec_kw"] = dict(zip(SPEC_KEYS, [float(v) for v in g["spec"]]))
    return g


def surface_cases():
    return sorted(f[len("surface_"):-4] for f in os.listdir(GOLDEN_DIR) if f.startswith("surface_") and f.endswith(".npz"))


def load_surface(name):
    g = dict(np.load(os.path.join(GOLDEN_DIR, f"surface_{name}.npz")))
    g["spec_kw"] = dict(zip(SPEC_KEYS, [float(v) for v in g["spec"]]))
    return g


def oracle_tables(mesh, sol):
    return pipeline.tables(mesh, sol)


def vacuum_system_inputs(mesh):
    """Vertex coordinates and vacuum cells in the reference's vertex numbering
    (ascending mesh node ids of the vacuum hexes, src/DealSolver.cpp:192-208)."""
    return pipeline.vacuum_inputs(mesh)


def bits_equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return a.shape == b.shape and bool((a.view(np.int64) == b.view(np.int64)).all())
