"""The oracle's robust RMS (n-sigma threshold) against the reference's tests.

robust_rms_jy_per_beam (crates/casa-imaging/src/lib.rs:74130-74183) takes the
finite residual values, clips them with Chauvenet's criterion (automatic z,
at most 5 iterations) when no clean mask restricts them, and returns
f32(MADFM) * 1.4826.  The oracle restates it in C; these tests pin it to the
reference's known answers: the Chauvenet fixture and its counts, the sample
variance, and casacore's MADFM of 0..63.  The masked path (values outside
the clean mask, no clipping) is checked against a sort-based restatement on
the fixture of the reference's radix-MADFM test.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
KATS = {k["name"]: k for k in json.load(open(os.path.join(HERE, "golden", "reference_kats.json")))["kats"]}


def test_chauvenet_clipping_counts():
    k = KATS["chauvenet_clipping_counts"]
    vals = np.array(k["input"]["values"], np.float32)
    assert len(vals) == 107
    cases = {"zscore_3.5_iterations_0": (3.5, 0), "zscore_3.5_iterations_1": (3.5, 1),
             "zscore_3.5_until_converged": (3.5, -1),
             "automatic_zscore_until_converged": (-1.0, -1)}
    for name, (z, it) in cases.items():
        kept = O.chauvenet_clip(vals, z, it)
        exp = k["expected"][name]
        assert len(kept) == exp["len"], name
        assert abs(float(kept.max()) - exp["max"]) < 1e-6, name


def test_mean_stddev_sample_variance():
    k = KATS["mean_stddev_sample_variance"]
    m, s = O.mean_stddev(k["input"]["values"])
    assert abs(m - k["expected"]["mean"]) < 1e-12
    assert abs(s - k["expected"]["stddev"]) < 1e-12


def test_madfm_indgen():
    k = KATS["madfm_indgen_64"]
    med, mad = O.madfm(np.arange(64, dtype=np.float32))
    assert med == k["expected"]["median"] and mad == k["expected"]["madfm"]


def test_chauvenet_zscore_table_and_bisection():
    # table entries are returned exactly; between entries the bisection
    # finds z whose 0.5 / erfc(z / sqrt 2) truncates to npts
    table = {0: 0.5, 1: 1.0, 3: 1.5, 10: 2.0, 40: 2.5, 185: 3.0, 1074: 3.5, 7893: 4.0}
    for n, z in table.items():
        assert O.chauvenet_max_zscore(n) == z
    from math import erfc, sqrt
    prev = 0.0
    for n in (2, 5, 100, 5000, 100000, 4194304, 10 ** 9):
        z = O.chauvenet_max_zscore(n)
        assert z > prev
        prev = z
        assert int(0.5 / erfc(z / sqrt(2.0))) == n


def _sorted_madfm(v):
    w = np.sort(np.asarray(v, np.float64))
    n = len(w)
    n2 = (n - 1) // 2
    med = (w[n2] + w[n2 + 1]) / 2.0 if n % 2 == 0 else w[n2]
    d = np.sort(np.abs(np.asarray(v, np.float64) - med))
    return (d[n2] + d[n2 + 1]) / 2.0 if n % 2 == 0 else d[n2]


def test_masked_path_excludes_the_clean_region():
    # the 4 x 5 residual of the reference's radix-MADFM test
    # (lib.rs:76006-76035); True marks the clean mask
    res = np.array([-8.0, 4.0, -2.0, 1.0, 0.0, 7.0, -3.0, 9.0, -1.0, 5.0, -6.0, 2.0, -4.0, 8.0,
                    3.0, -7.0, 6.0, -5.0, 10.0, -9.0], np.float32).reshape(4, 5)
    for masked in ([(0, 0), (3, 4)], [(0, 0), (1, 1), (3, 4)],
                   [(0, 4), (1, 4), (2, 4), (3, 4)]):
        mask = np.zeros((4, 5), np.uint8)
        for p in masked:
            mask[p] = 1
        rms, mad, n = O.robust_rms(res, mask)
        sel = res[mask == 0]
        assert n == len(sel)
        assert mad == _sorted_madfm(sel)
        assert rms == float(np.float32(mad) * np.float32(1.4826))


@pytest.mark.parametrize("seed", [0, 1])
def test_full_mask_path_clips_then_madfm(seed):
    rng = np.random.default_rng(seed)
    img = rng.normal(0.0, 0.01, (96, 80)).astype(np.float32)
    img[10, 10] = 5.0
    img[40, 20] = -3.0
    img[5, 7] = np.nan
    rms, mad, n = O.robust_rms(img)
    finite = img[np.isfinite(img)]
    kept = O.chauvenet_clip(finite, -1.0, 5)
    assert n == len(kept) < len(finite)
    assert mad == _sorted_madfm(kept)
    assert rms == float(np.float32(mad) * np.float32(1.4826))
    # an all-true mask is the full-mask path
    assert O.robust_rms(img, np.ones(img.shape, np.uint8)) == (rms, mad, n)
    assert O.nsigma_threshold(img, 3.0) == float(np.float32(3.0) * np.float32(rms))
    assert O.nsigma_threshold(img, 0.0) == 0.0
