"""focss_field_power against Field::average_power / peak_power
(src/focss/field.cpp:164-187) for one and two modes: reference outputs in
tests/golden/field_power_golden.npz (written by the unmodified field.cpp,
tests/golden/make_golden.py) on inputs exactly representable in complex64.
The average is an FP64 sum of FP32 |A|^2 (one rounding each, 6e-8); the
peak is the FP32 maximum of the summed |A|^2."""
import os

import numpy as np
import pytest

import focss_gb300 as fg
from conftest import ROOT

pytestmark = pytest.mark.gpu

GOLD = os.path.join(ROOT, "tests", "golden", "field_power_golden.npz")


@pytest.mark.parametrize("modes", [1, 2])
def test_field_power_matches_reference(ctx, modes):
    g = dict(np.load(GOLD))
    a = g["power_in%d" % modes]
    avg_want, peak_want = g["power_out%d" % modes]
    batch = 3
    data = np.stack([a, a * 0.5, a * 2.0])  # realizations of different power
    f = fg.Field(fg.Domain(modes, a.shape[1], 1.0), data=data, batch=batch, ctx=ctx)
    avg, peak = f.power_stats()
    for b, s in enumerate((1.0, 0.25, 4.0)):
        assert abs(avg[b] - s * avg_want) < 1e-7 * s * avg_want
        assert abs(peak[b] - s * peak_want) < 2e-7 * s * peak_want
