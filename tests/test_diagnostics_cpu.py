"""Host side of the flow statistics: the per-shell spectrum comparison."""
import numpy as np

from padeops_gb300 import diagnostics as D


def test_compare_spectra_shells_and_floor():
    n = 48  # shells 1 .. 16
    ref = np.concatenate([[0.0], np.exp(-np.arange(1, 30, dtype=float))])
    e = ref.copy()
    e[3] *= 1.02
    c = D.compare_spectra(e, ref, n)
    assert c["kmax"] == 16
    assert abs(c["max"] - 0.02) < 1e-12
    assert c["per_shell"][2] == c["max"]
    # a floor drops the shells below 1e-5 of the peak (exp(-k) < 1e-5 e^-1 for k >= 13)
    e[14] = 10 * ref[14]
    c2 = D.compare_spectra(e, ref, n, floor=1e-5)
    assert c2["kmax"] == 12
    assert np.isnan(c2["per_shell"][13])
    assert abs(c2["max"] - 0.02) < 1e-12
