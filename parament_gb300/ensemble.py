"""Batched ensembles of independent equiprop problems (one persistent launch
captured in a CUDA graph).  Wraps Parament_ensembleCreate / SetSamples / Run /
Tune / Destroy of libparament.so.

    ens = Ensemble([(H0, H1, dt), ...], precision='fp32', quadrature_mode='none')
    ens.set_samples([carr_0, carr_1, ...])   # carr_i: (K_i, pts_i)
    Us = ens.run()                            # list of (d_i, d_i) propagators
"""
import ctypes

import numpy as np

from . import paramentlib
from .constants import PARAMENT_QUADRATURE_MIDPOINT, PARAMENT_QUADRATURE_NONE, PARAMENT_QUADRATURE_SIMPSON

_lib = paramentlib.lib
_vp = ctypes.c_void_p
_lib.Parament_ensembleCreate.argtypes = [ctypes.POINTER(_vp), ctypes.c_int, ctypes.c_uint,
                                         ctypes.POINTER(ctypes.c_uint), ctypes.POINTER(ctypes.c_uint),
                                         ctypes.POINTER(ctypes.c_uint), ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.c_int]
_lib.Parament_ensembleSetSamples.argtypes = [_vp, ctypes.POINTER(_vp)]
_lib.Parament_ensembleRun.argtypes = [_vp, ctypes.POINTER(_vp)]
_lib.Parament_ensembleTune.argtypes = [_vp]
_lib.Parament_ensembleGranularity.argtypes = [_vp]
_lib.Parament_ensembleGranularity.restype = ctypes.c_double
_lib.Parament_ensembleLastMs.argtypes = [_vp]
_lib.Parament_ensembleLastMs.restype = ctypes.c_float
_lib.Parament_ensembleDestroy.argtypes = [_vp]

_QUAD = {'none': PARAMENT_QUADRATURE_NONE, 'midpoint': PARAMENT_QUADRATURE_MIDPOINT,
         'simpson': PARAMENT_QUADRATURE_SIMPSON}


class Ensemble:
    """Independent problems ``(H0, H1, dt, pts)`` run together on one GPU.

    ``H1`` is a (K, d, d) array (K may differ between problems), ``pts`` the
    number of samples per control.  All problems share the precision and the
    quadrature mode (no Magnus terms)."""

    def __init__(self, problems, precision='fp32', quadrature_mode='none'):
        if precision not in ('fp32', 'fp64'):
            raise ValueError("precision must be either 'fp32' or 'fp64'")
        if quadrature_mode not in _QUAD:
            raise ValueError('unknown quadrature mode selected')
        self._ct = np.complex128 if precision == 'fp64' else np.complex64
        n = len(problems)
        self._keep = []
        dims, amps, pts, dts, h0p, h1p = [], [], [], [], [], []
        for H0, H1, dt, p in problems:
            H0 = np.ascontiguousarray(np.atleast_2d(H0), dtype=self._ct)
            H1 = np.ascontiguousarray(np.asarray(H1).reshape(-1, H0.shape[0], H0.shape[0]), dtype=self._ct)
            self._keep += [H0, H1]
            dims.append(H0.shape[0])
            amps.append(H1.shape[0])
            pts.append(int(p))
            dts.append(float(dt))
            h0p.append(H0.ctypes.data)
            h1p.append(H1.ctypes.data)
        self.dims, self.amps, self.pts = dims, amps, pts
        u = ctypes.c_uint * n
        self._handle = _vp()
        code = _lib.Parament_ensembleCreate(ctypes.byref(self._handle), 1 if precision == 'fp64' else 0, n,
                                            u(*dims), u(*amps), u(*pts), (ctypes.c_double * n)(*dts),
                                            (_vp * n)(*h0p), (_vp * n)(*h1p), _QUAD[quadrature_mode])
        self._keep = []
        if code != 0:
            self._handle = None
            _raise(code)

    def set_samples(self, carrs):
        arrs = [np.ascontiguousarray(np.asarray(c, dtype=self._ct).reshape(k, p))
                for c, k, p in zip(carrs, self.amps, self.pts)]
        ptrs = (_vp * len(arrs))(*[a.ctypes.data for a in arrs])
        _check(_lib.Parament_ensembleSetSamples(self._handle, ptrs))

    def run(self, copy_out=True):
        outs = [np.zeros((d, d), dtype=self._ct) for d in self.dims] if copy_out else None
        ptrs = (_vp * len(self.dims))(*[o.ctypes.data for o in outs]) if copy_out else None
        _check(_lib.Parament_ensembleRun(self._handle, ptrs))
        return outs

    def tune(self):
        _check(_lib.Parament_ensembleTune(self._handle))
        return float(_lib.Parament_ensembleGranularity(self._handle))

    @property
    def last_ms(self):
        return float(_lib.Parament_ensembleLastMs(self._handle))

    def destroy(self):
        if self._handle is not None:
            _lib.Parament_ensembleDestroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.destroy()


def _raise(code):
    from .parament import _EXCEPTIONS
    msg = _lib.Parament_errorMessage(code).decode()
    raise _EXCEPTIONS.get(code, RuntimeError)(f"Error code {code}: {msg}")


def _check(code):
    if code != 0:
        _raise(code)
