"""Helpers built on a throw-away context (src/python/pyparament/parament/debug_functions.py:22-38)."""
import numpy as np

from . import paramentlib
from .parament import Parament


def expm(m):
    """Matrix exponential e^m for matrices of modest norm.

    Loads H0 = i m and H1 = m with one zero-amplitude step of dt = 1, so the
    propagator exp(-i (i m)) equals e^m.
    """
    with Parament() as ctx:
        ctx.set_hamiltonian(1j * np.asarray(m), m, use_magnus=False, quadrature_mode='none')
        return ctx.equiprop(1.0, np.zeros(1))


def device_info():
    """Print the visible CUDA devices to stdout."""
    paramentlib.lib.device_info()
