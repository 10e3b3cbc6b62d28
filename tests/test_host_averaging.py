"""Host-side averaging of the reference (src/main.ts:590-596) and the sweep order
(src/ui/aeromap.ts:79-84), through libwt's C entry points, against plain Python
restatements; both are host code and run without a GPU."""
import ctypes

import numpy as np


def ema_reference(readings, q):
    """main.ts:590-596: a = 0.15 for n < 20, 0.04 for n < 60, else 0.011; the
    first reading is taken as is."""
    cd = cl = 0.0
    for n, (drag, down) in enumerate(readings):
        a = 0.15 if n < 20 else 0.04 if n < 60 else 0.011
        r = 1.0 if n == 0 else a
        cd += (drag / q - cd) * r
        cl += (down / q - cl) * r
    return cd, cl


def test_coef_ema_matches_reference(wt_lib):
    from windtunnel import _abi
    _abi.load()
    rng = np.random.default_rng(0)
    readings = [(1500 + 200 * rng.standard_normal(), 3000 + 500 * rng.standard_normal()) for _ in range(150)]
    q = 0.5 * 1.225 * (250 / 3.6) ** 2
    e = _abi.CoefEma()
    for drag, down in readings:
        wt_lib.wt_coef_ema_update(ctypes.byref(e), drag, down, q)
    cd, cl = ema_reference(readings, q)
    assert e.n == 150 and e.cd == cd and e.cl == cl


def test_serpentine_order():
    """The order the C driver visits: front-major, rear reversed on odd rows."""
    from windtunnel.sweep import serpentine
    order = serpentine(5, 5)
    assert order[:6] == [(0, 0), (0, 1), (0, 2), (0, 3), (0, 4), (1, 4)]
    assert sorted(order) == [(i, j) for i in range(5) for j in range(5)]
