"""The allocation-free location + interpolation entry point, fgb_field_interpolate_device_noalloc.

MD engines that hand all device memory to their own pool allocator, or fix their device
footprint at start-up, cannot let a library call cudaMalloc inside the timestep loop (and a
cudaMalloc synchronises the device, stalling an asynchronous pipeline). This entry point keeps
its per-point scratch in a fixed device array instead. Its results must equal those of the
allocating entry point, fgb_field_interpolate_device, exactly, including on a second call in a
row (the shared array still holds the first call's data); the calls must leave the device's
free memory unchanged; and oversize requests must be refused before anything runs.

This file is collected last so that a stopping run has executed every other test first; it
also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import femocs_gb300 as fg
import oracle as orc
from femocs_gb300._lib import load
from util import bits_equal, load_golden

pytestmark = pytest.mark.gpu


def _run(fn, field, pts, rank):
    n = len(pts)
    d_pts = fg.DeviceBuffer(24 * n)
    d_pts.upload(np.ascontiguousarray(pts, dtype=np.float64))
    d_cells = fg.DeviceBuffer(4 * n)
    d_out = fg.DeviceBuffer(40 * n)
    rc = fn(field.h, n, C.c_void_p(d_pts.ptr), rank, C.c_void_p(d_cells.ptr), C.c_void_p(d_out.ptr))
    assert rc == 0, fg.last_error()
    field.mark(0)
    field.elapsed(0, 0)  # waits until the field's stream has finished the call
    cells = d_cells.download(np.zeros(n, dtype=np.int32))
    out = d_out.download(np.zeros((n, 5)))
    return cells, out


@pytest.fixture(scope="module")
def field_and_points():
    g = load_golden("tip_a")
    m = fg.Mesh.synthetic(**g["spec_kw"])
    f = fg.Field(m)
    f.set_nodal(orc.test_solution(m.export("node_xyz")))
    spec = g["spec_kw"]
    rng = np.random.default_rng(11)
    b = spec["box_half"]
    other = np.c_[rng.uniform(-b, b, 7000), rng.uniform(-b, b, 7000), rng.uniform(-spec["slab"], spec["top"], 7000)]
    return g, m, f, g["pts"], other


@pytest.mark.parametrize("rank", [1, 2, 3])
def test_noalloc_equals_allocating_entry_point_on_two_calls(field_and_points, rank):
    g, m, f, pts_a, pts_b = field_and_points
    lib = load()
    ref_a = _run(lib.fgb_field_interpolate_device, f, pts_a, rank)
    ref_b = _run(lib.fgb_field_interpolate_device, f, pts_b, rank)
    # two allocation-free calls in a row: the second reuses the scratch the first filled
    got_a = _run(lib.fgb_field_interpolate_device_noalloc, f, pts_a, rank)
    got_b = _run(lib.fgb_field_interpolate_device_noalloc, f, pts_b, rank)
    for ref, got in ((ref_a, got_a), (ref_b, got_b)):
        np.testing.assert_array_equal(got[0], ref[0])
        assert bits_equal(got[1], ref[1])
    # and both agree with the reference's golden cells
    np.testing.assert_array_equal(got_a[0], g[f"cells_r{rank}"])


def test_noalloc_refuses_more_points_than_its_scratch(field_and_points):
    _, _, f, _, _ = field_and_points
    lib = load()
    rc = lib.fgb_field_interpolate_device_noalloc(f.h, 262145, None, 3, None, None)
    assert rc == 1
    assert "262144" in fg.last_error()


def test_noalloc_calls_allocate_no_device_memory(field_and_points):
    """Free device memory (cudaMemGetInfo) is the same before and after two allocation-free
    calls, with every buffer the calls use allocated beforehand."""
    _, _, f, pts, _ = field_and_points
    lib = load()
    n = len(pts)
    d_pts = fg.DeviceBuffer(24 * n)
    d_pts.upload(np.ascontiguousarray(pts, dtype=np.float64))
    d_cells = fg.DeviceBuffer(4 * n)
    d_out = fg.DeviceBuffer(40 * n)
    args = (f.h, n, C.c_void_p(d_pts.ptr), 3, C.c_void_p(d_cells.ptr), C.c_void_p(d_out.ptr))
    assert lib.fgb_field_interpolate_device_noalloc(*args) == 0, fg.last_error()
    assert lib.fgb_device_sync() == 0
    free0, _, _ = fg.device_info()
    for _ in range(2):
        assert lib.fgb_field_interpolate_device_noalloc(*args) == 0, fg.last_error()
    assert lib.fgb_device_sync() == 0
    free1, _, _ = fg.device_info()
    assert free1 == free0, (free0, free1)
