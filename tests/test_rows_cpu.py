"""Row runs on the CPU: the oracle's restatement of the row path's sample
preparation pinned by the reference's own Stokes-I KATs, and the library's
plane-to-polarization selection (a host function of the C ABI) against the
oracle's derive_pair_selection restatement."""
import numpy as np
import pytest

import casars_cuda as cc
from oracle import rows as OR


def _pair_runs(v0, v1, w0, w1, f0, f1):
    n = len(v0)
    data = np.zeros((n, 1, 2), np.complex64)
    data[:, 0, 0], data[:, 0, 1] = v0, v1
    flag = np.zeros((n, 1, 2), np.uint8)
    flag[:, 0, 0], flag[:, 0, 1] = f0, f1
    weight = np.stack([w0, w1], 1).astype(np.float32)
    uvw = np.zeros((n, 3))
    uvw[:, 0] = 10.0
    uvw[:, 1] = 5.0
    return uvw, data, flag, weight


def test_stokes_i_collapse_kats():
    # lib.rs:88688-88703: a flagged hand drops its logical sample
    uvw, data, flag, weight = _pair_runs([1 + 0j, 1 + 0j], [1 + 0j, 1 + 0j], [1.0, 1.0],
                                         [1.0, 1.0], [0, 1], [0, 0])
    out = OR.prepare(uvw, np.array([1.0]), data, flag, weight, None, None, 0, 1, "half_sum", 2.0)
    assert len(out["u"]) == 1
    # lib.rs:88705-88726: half-sum visibility, CASA-style mean weight, factor 2
    uvw, data, flag, weight = _pair_runs([2 + 1j], [6 - 1j], [1.5], [3.0], [0], [0])
    out = OR.prepare(uvw, np.array([1.0]), data, flag, weight, None, None, 0, 1, "half_sum", 2.0)
    assert abs(out["vis"][0].real - 4.0) < 1e-6 and abs(out["vis"][0].imag) < 1e-6
    assert abs(out["weight"][0] - 2.25) < 1e-6
    assert abs(out["sumwt_factor"][0] - 2.0) < 1e-6
    assert out["u"][0] == 10.0 and out["v"][0] == 5.0


def test_transforms_follow_complex_arithmetic():
    a, b = 3 + 2j, 1 - 4j
    assert OR.collapse(a, b, "half_sum") == (a + b) / 2
    assert OR.collapse(a, b, "half_difference") == (a - b) / 2
    assert OR.collapse(a, b, "positive_half_imag_difference") == (a - b) * 0.5j
    assert OR.collapse(a, b, "negative_half_imag_difference") == (a - b) * -0.5j


LINEAR, CIRCULAR = [9, 10, 11, 12], [5, 6, 7, 8]


@pytest.mark.parametrize("corr", [LINEAR, CIRCULAR, [9, 12], [5, 8], [12, 9], [10, 11],
                                  [6, 7], [9, 9, 12]])
@pytest.mark.parametrize("plane", ["I", "Q", "U", "V", "XX", "YY", "RR", "LL"])
def test_plane_polarization_matches_oracle(corr, plane):
    try:
        ref = OR.plane_polarization(plane, corr)
    except ValueError:
        with pytest.raises(cc.CasarsCudaError):
            cc.Polarization.for_plane(plane, corr)
        return
    p = cc.Polarization.for_plane(plane, corr)
    assert (p.corr0, p.corr1, p.transform, p.sumwt_factor) == ref
