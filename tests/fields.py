"""Seeded synthetic fields with the shapes and spectra of the benchmark configurations.

All arrays are Fortran-ordered (x fastest), like the reference's fields.
"""
import numpy as np


from padeops_gb300.synthetic import hit_initial_field, random_modes  # noqa: F401


def relerr(a, b):
    """Normwise relative difference max|a-b| / max|b|."""
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))
