"""The texture-gather throughput probe the benchmark divides by
(xrp_probe_gather_rate): a positive rate, stable between calls."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def test_gather_probe_rate():
    import __graft_entry__ as g
    g.build()
    from xray_projection_render_gb300 import _lib as XL
    L = XL.load()
    rates = []
    for _ in range(2):
        r = ctypes.c_double(0.0)
        XL.check(L.xrp_probe_gather_rate(ctypes.byref(r)), "xrp_probe_gather_rate")
        rates.append(r.value)
    assert all(r > 1e9 for r in rates)
    assert abs(rates[0] - rates[1]) <= 0.2 * max(rates)
