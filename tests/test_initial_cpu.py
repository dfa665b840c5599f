"""Initial-condition helpers (CPU): the reference notebooks' helpers and the
host side of the device seeding."""

import math

import numpy as np


def test_notebook_helpers():
    from mantaray_gb300 import initial as I

    # utils.py:11-26 with g = 9.81: T = 10 s -> k = 4 pi^2 / 981
    assert abs(I.period_to_wavenumber_deep(10.0) - 4 * math.pi ** 2 / 981.0) < 1e-15
    k = I.period_to_wavenumber_deep(10.0)
    cg = I.deep_water_group_velocity(k)
    assert abs(cg - math.sqrt(9.81 / k) / 2) < 1e-12
    x = np.arange(0, 5001, 50.0)
    y = np.arange(0, 3001, 25.0)
    assert abs(I.cfl_time_step(x, y, k) - 25.0 / cg) < 1e-12
    assert I.duration_to_cross(x, k) == round(5000.0 / cg)
    # start line snapped to grid nodes, against the notebook's brute-force search
    xs, ys = I.start_line_points((12.0, 988.0), (3.0, 2017.0), x, y, 17)
    XX, YY = np.meshgrid(x, y)
    for px, py, gx, gy in zip(np.linspace(12, 988, 17), np.linspace(3, 2017, 17), xs, ys):
        d = np.sqrt((XX - px) ** 2 + (YY - py) ** 2)
        j = np.unravel_index(np.argmin(d), d.shape)
        assert (XX[j], YY[j]) == (gx, gy)


def test_splitmix_uniform_known_values():
    # SplitMix64 of 0 and seed 0: the generator's published first output
    # 0xE220A8397B1DCDAF, top 53 bits over 2^53
    from mantaray_gb300.initial import splitmix_uniform

    u = splitmix_uniform(0, np.array([0]))
    assert u[0] == float(0xE220A8397B1DCDAF >> 11) * 2.0 ** -53
    v = splitmix_uniform(12345, np.arange(100000))
    assert 0.0 <= v.min() and v.max() < 1.0 and abs(v.mean() - 0.5) < 0.01
