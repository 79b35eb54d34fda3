"""The tensor-core (tcgen05) path: a self check of the descriptors and the TMEM layout, and the
Q2 element matrices computed on the tensor cores by error-free BF16 splitting against the
FP32-pair kernel."""
import ctypes as C

import pytest

from femocs_gb300._lib import load

pytestmark = pytest.mark.gpu


def test_tensor_core_self_check_is_exact():
    """One 128 x 48 x 32 product of small integers (BF16 in, FP32 accumulated in tensor memory,
    two MMAs) equals the host's exactly."""
    err = C.c_double(-1.0)
    assert load().fgb_tc_selftest(C.byref(err)) == 0
    assert err.value == 0.0


import numpy as np  # noqa: E402

import femocs_gb300 as fg  # noqa: E402

TIP = dict(radius=8.0, height=25.0, box_half=30.0, slab=6.0, top=80.0, h=4.0, growth=1.4, margin=4.0)


@pytest.mark.parametrize("spec", [TIP, dict(fg.CONFIG2, h=22.0, growth=1.3)], ids=["small", "probe"])
def test_tensor_core_element_matrices_match(spec):
    """The Q2 element matrices from the tensor cores (error-free BF16 slices) equal the FP32-pair
    kernel's within 1e-12 of each cell's largest entry -- the bound the element matrices are
    held to against the numpy restatement -- and the solve is unchanged."""
    m = fg.Mesh.synthetic(**spec)
    f = fg.Field(m, order=2)
    out = {}
    for tc in (False, True):
        f.set_ke_tensor(tc)
        f.setup(0.1)
        f.assemble(True, False)
        K = f.element_matrices().reshape(-1, 378)
        rc, st = f.solve(precision=2, rel_tol=1e-10)
        assert rc > 0 and st["status"] == 1, st
        out[tc] = (K, st["iterations"], f.solution())
    K0, K1 = out[False][0], out[True][0]
    scale = np.abs(K0).max(axis=1)
    err = (np.abs(K1 - K0).max(axis=1) / scale).max()
    assert err <= 1e-12, err
    assert abs(out[True][1] - out[False][1]) <= 1
    x = out[False][2]
    assert np.abs(out[True][2] - x).max() <= 2e3 * 1e-10 * np.abs(x).max()
