"""The ``Parament`` context class: a drop-in for the reference's pyparament
wrapper (src/python/pyparament/parament/parament.py:48-314) over the GB300
library.

Same constructor, methods, argument meaning, exception types and messages.
Differences: ``dt`` is passed as a plain ``float`` (the reference's fp32 branch
calls ``np.float``, removed from NumPy), error messages for a stored code are
read with ``Parament_peekAtLastError`` (the reference calls a symbol that does
not exist), and the context exposes the cycle-control, precision-form and
device-tensor entry points of the library.
"""
import ctypes
import logging
from functools import wraps

import numpy as np

from . import paramentlib
from .constants import *  # noqa: F401,F403
from .constants import (PARAMENT_FAIL, PARAMENT_PRECISION_PLAIN, PARAMENT_PRECISION_SPLIT,
                        PARAMENT_QUADRATURE_MIDPOINT, PARAMENT_QUADRATURE_NONE, PARAMENT_QUADRATURE_SIMPSON,
                        PARAMENT_STATUS_CUBLAS_FAILED, PARAMENT_STATUS_CUBLAS_INIT_FAILED,
                        PARAMENT_STATUS_DEVICE_ALLOC_FAILED, PARAMENT_STATUS_HOST_ALLOC_FAILED,
                        PARAMENT_STATUS_INVALID_QUADRATURE_SELECTION, PARAMENT_STATUS_INVALID_VALUE,
                        PARAMENT_STATUS_KERNEL_TIMEOUT, PARAMENT_STATUS_NO_HAMILTONIAN,
                        PARAMENT_STATUS_SELECT_SMALLER_DT, PARAMENT_STATUS_SUCCESS)

logger = logging.getLogger('Parament')
logger.setLevel(logging.CRITICAL)

try:
    import qutip
except ImportError:
    from . import qutip_mock as qutip

_EXCEPTIONS = {
    PARAMENT_STATUS_HOST_ALLOC_FAILED: MemoryError,
    PARAMENT_STATUS_DEVICE_ALLOC_FAILED: MemoryError,
    PARAMENT_STATUS_CUBLAS_INIT_FAILED: RuntimeError,
    PARAMENT_STATUS_INVALID_VALUE: ValueError,
    PARAMENT_STATUS_CUBLAS_FAILED: RuntimeError,
    PARAMENT_STATUS_SELECT_SMALLER_DT: RuntimeError,
    PARAMENT_STATUS_NO_HAMILTONIAN: RuntimeError,
    PARAMENT_STATUS_INVALID_QUADRATURE_SELECTION: ValueError,
    PARAMENT_FAIL: RuntimeError,
    PARAMENT_STATUS_KERNEL_TIMEOUT: RuntimeError,
}

# Handle of CUDA's legacy default stream.  torch reports its default stream as
# handle 0, which the C-ABI reads as "the context's own stream"; passing the
# legacy handle keeps the work on the caller's stream.
_CUDA_STREAM_LEGACY = 1


def _pack_samples(carr, ctype, amps, pts):
    """The control samples as one C-contiguous (amps * pts) array of ``ctype``.

    When the rows are consecutive rows of one C-contiguous 2-D array of that
    type (``equiprop(dt, *samples)`` with ``samples`` of shape (amps, pts)),
    that array is passed on as it is; otherwise the rows are copied (and
    converted) into a new one, as the reference's wrapper does.
    """
    if amps and all(isinstance(c, np.ndarray) for c in carr):
        base = carr[0].base
        if (isinstance(base, np.ndarray) and base.dtype == ctype and base.ndim == 2 and base.shape == (amps, pts)
                and base.flags.c_contiguous):
            start = base.__array_interface__['data'][0]
            step = pts * base.itemsize
            if all(c.base is base and c.__array_interface__['data'][0] == start + k * step
                   for k, c in enumerate(carr)):
                return base.reshape(-1)
    return np.ascontiguousarray(np.ravel(np.asarray(carr, dtype=ctype).reshape(amps, pts), order='C'))


def _stream_handle(stream):
    return ctypes.c_void_p(stream.cuda_stream or _CUDA_STREAM_LEGACY)


_QUADRATURE = {
    'none': PARAMENT_QUADRATURE_NONE,
    'midpoint': PARAMENT_QUADRATURE_MIDPOINT,
    'simpson': PARAMENT_QUADRATURE_SIMPSON,
}


def _must_be_alive(f):
    @wraps(f)
    def wrapper(self, *args, **kwargs):
        if self._handle is None:
            raise RuntimeError("Attempting to use a context that has been destroyed")
        return f(self, *args, **kwargs)

    return wrapper


class Parament:
    """A Parament context: settings and device state between calls.

    Load the Hamiltonians with :meth:`set_hamiltonian`, then call
    :meth:`equiprop` to obtain the propagator of the piecewise-constant
    evolution.

    Parameters
    ----------
    precision : {'fp32', 'fp64'}
        Arithmetic of the context: complex64 or complex128.

    Examples
    --------
    >>> ctx = Parament()
    >>> ctx.set_hamiltonian(np.array([[1, 0], [0, -1]]), np.array([[0, 1], [1, 0]]))
    >>> ctx.equiprop(1.0, np.zeros(1))   # exp(-i diag(1, -1))
    array([[0.54030234-0.84147096j, 0.        +0.j        ],
           [0.        +0.j        , 0.54030234+0.84147096j]], dtype=complex64)

    The context frees its device memory on :meth:`destroy`, at garbage
    collection, or at the end of a ``with`` block.
    """

    def __init__(self, precision='fp32'):
        if precision not in ('fp32', 'fp64'):
            raise ValueError("precision must be either 'fp32' or 'fp64'")
        self._use_doubles = (precision == 'fp64')
        self._lib = paramentlib.lib
        self._handle = ctypes.c_void_p()
        create = self._lib.Parament_create_fp64 if self._use_doubles else self._lib.Parament_create
        code = create(ctypes.byref(self._handle))
        if code != PARAMENT_STATUS_SUCCESS:
            self._handle = None
            self._check_error(code)
        self.dim = -1
        self.amps = -1
        self._qutip_H0 = None
        self._use_qutip = False

    def _fn(self, name):
        return getattr(self._lib, name + ('_fp64' if self._use_doubles else ''))

    @property
    def _ctype(self):
        return np.complex128 if self._use_doubles else np.complex64

    @_must_be_alive
    def destroy(self):
        """Destroy the context and free its device memory."""
        self._check_error(self._fn('Parament_destroy')(self._handle))
        self._handle = None

    def __del__(self):
        if getattr(self, '_handle', None) is not None:
            try:
                self.destroy()
            except Exception:  # interpreter shutdown
                pass

    @_must_be_alive
    def set_hamiltonian(self, H0, *H1, use_magnus=False, quadrature_mode='none'):
        """Load the drift Hamiltonian ``H0`` and the control Hamiltonians ``H1``.

        ``H1`` is variadic: pass one matrix per control, or unpack a list or a
        3-D array whose first axis enumerates the controls.  ``use_magnus`` and
        ``quadrature_mode`` ('none', 'midpoint' or 'simpson') are keyword-only;
        the Magnus terms require 'simpson'.  A qutip ``Qobj`` drift makes
        :meth:`equiprop` return a ``Qobj``.
        """
        if isinstance(H0, qutip.Qobj):
            self._use_qutip = True
            self._qutip_H0 = H0
            H0 = H0.data.todense() if hasattr(H0.data, 'todense') else H0.full()
        else:
            self._use_qutip = False
        H0 = np.atleast_2d(H0)
        if quadrature_mode not in _QUADRATURE:
            raise ValueError('unknown quadrature mode selected')
        mode_sel = _QUADRATURE[quadrature_mode]
        dim = np.shape(H0)[0]
        if len(H1) == 0:
            raise ValueError('provide at least 1 control amplitude')
        H1 = [(Hi.data.todense() if hasattr(Hi.data, 'todense') else Hi.full()) if isinstance(Hi, qutip.Qobj)
              else Hi for Hi in H1]
        H1 = np.atleast_2d(H1)
        shape = np.shape(H1)
        amps = shape[0] if len(shape) > 2 else 1
        self.dim = dim
        self.amps = amps
        # C order keeps the time ordering of the samples without any flip.
        h0 = np.ascontiguousarray(np.ravel(H0, order='C'), dtype=self._ctype)
        h1 = np.ascontiguousarray(np.ravel(H1, order='C'), dtype=self._ctype)
        self._check_error(self._fn('Parament_setHamiltonian')(self._handle, h0, h1, dim, amps, bool(use_magnus),
                                                              mode_sel))

    @_must_be_alive
    def equiprop(self, dt, *carr):
        """Propagator of the loaded Hamiltonians under the control samples ``carr``.

        Pass one sample vector per control (``equiprop(dt, u1, u2)``) or unpack
        a 2-D array whose first axis enumerates the controls.  Fewer vectors
        than controls leave the remaining controls at zero amplitude.
        """
        if self.amps < 0:
            raise RuntimeError("No hamiltonian set")
        amps = len(carr)
        if len(carr) > self.amps:
            raise ValueError(f'Got {len(carr)} amplitude arrays, but there are only {self.amps} Hamiltonians.')
        pts = np.shape(carr[0])[0] if amps else 0
        if any(np.shape(c) != (pts,) for c in carr):
            raise ValueError("All amplitude arrays must have the same length.")
        output = np.zeros(self.dim ** 2, dtype=self._ctype)
        samples = _pack_samples(carr, self._ctype, amps, pts)
        if samples.size == 0:
            samples = np.zeros(1, dtype=self._ctype)
        self._check_error(self._fn('Parament_equiprop')(self._handle, samples, float(dt), pts, amps, output))
        out = np.ascontiguousarray(np.reshape(output, (self.dim, self.dim)))
        if self._use_qutip:
            out = qutip.Qobj(out, dims=self._qutip_H0.dims)
        return out

    # ---------------------------------------------------------------- extensions

    @_must_be_alive
    def set_iteration_cycles_manually(self, cycles):
        """Force the Chebyshev order (odd, 1..63) instead of the norm-based choice."""
        self._check_error(self._fn('Parament_setIterationCyclesManually')(self._handle, int(cycles)))

    @_must_be_alive
    def automatic_iteration_cycles(self):
        """Return to the norm-based choice of the Chebyshev order."""
        self._check_error(self._fn('Parament_automaticIterationCycles')(self._handle))

    @_must_be_alive
    def peek_at_last_error(self):
        """Error code of the last library call on this context."""
        return int(self._fn('Parament_peekAtLastError')(self._handle))

    @property
    @_must_be_alive
    def last_iteration_cycles(self):
        """Chebyshev order used by the last successful :meth:`equiprop`."""
        return int(self._fn('Parament_lastIterationCycles')(self._handle))

    @property
    @_must_be_alive
    def hamiltonian_norm(self):
        """Norm bound ||H0||_inf + sum_k ||H_k||_inf of the loaded Hamiltonians."""
        return float(self._fn('Parament_hamiltonianNorm')(self._handle))

    @_must_be_alive
    def set_precision_mode(self, mode):
        """'plain' (the reference scheme, default) or 'split' (complex64 contexts:
        U_j = I + E_j with X_j and the first-order term in double-float, the
        higher powers as sliced bf16 products with exact accumulation on the
        tensor cores at d = 64 (FP32 products below), a double-float running
        product per chunk of steps and a double-float tree of the chunks)."""
        if self._use_doubles and mode != 'plain':
            raise ValueError("the split precision form applies to 'fp32' contexts only")
        code = {'plain': PARAMENT_PRECISION_PLAIN, 'split': PARAMENT_PRECISION_SPLIT}.get(mode)
        if code is None:
            raise ValueError("precision mode must be 'plain' or 'split'")
        if not self._use_doubles:
            self._check_error(self._lib.Parament_setPrecisionMode(self._handle, code))

    @_must_be_alive
    def equiprop_device(self, dt, carr, out=None, stream=None):
        """equiprop on CUDA tensors: ``carr`` is an (amps, pts) complex tensor on
        the context's device; the result is written to ``out`` (allocated when
        None) on ``stream`` (the current torch stream when None) without a host
        round trip."""
        import torch

        want = torch.complex128 if self._use_doubles else torch.complex64
        if not (isinstance(carr, torch.Tensor) and carr.is_cuda):
            raise TypeError("carr must be a CUDA tensor")
        carr = carr.to(want)
        if carr.dim() == 1:
            carr = carr.unsqueeze(0)
        carr = carr.contiguous()
        amps, pts = carr.shape
        if amps > self.amps:
            raise ValueError(f'Got {amps} amplitude arrays, but there are only {self.amps} Hamiltonians.')
        if out is None:
            out = torch.empty((self.dim, self.dim), dtype=want, device=carr.device)
        if out.dtype != want or not out.is_contiguous() or out.numel() != self.dim ** 2:
            raise ValueError("out must be a contiguous (dim, dim) tensor of the context's complex type")
        if stream is None:
            stream = torch.cuda.current_stream(carr.device)
        code = self._fn('Parament_equipropDevice')(self._handle, ctypes.c_void_p(carr.data_ptr()), float(dt), pts,
                                                   amps, ctypes.c_void_p(out.data_ptr()), _stream_handle(stream))
        self._check_error(code)
        return out

    @_must_be_alive
    def synchronize(self):
        """Wait for the work queued by the device-buffer calls of this context;
        raises RuntimeError (code 1010) if a bounded wait of a tensor-core
        kernel gave up since the last report."""
        self._check_error(self._fn('Parament_synchronize')(self._handle))

    @property
    @_must_be_alive
    def device_memory_bytes(self):
        """Bytes of device memory held by this context's buffers."""
        return int(self._fn('Parament_deviceMemoryBytes')(self._handle))

    @_must_be_alive
    def vjp(self, dt, W, *carr):
        """Vector-Jacobian product of :meth:`equiprop`: for a seed ``W`` (dim x dim)
        returns ``grad`` with ``grad[k, i] = d/du_k[i] Re Tr(W^H U)`` for real
        control samples.  A loss with ``dL = Re Tr(G^H dU)`` has ``dL/du = grad``
        for ``W = G``."""
        if self.amps < 0:
            raise RuntimeError("No hamiltonian set")
        amps = len(carr)
        if amps > self.amps:
            raise ValueError(f'Got {amps} amplitude arrays, but there are only {self.amps} Hamiltonians.')
        pts = np.shape(carr[0])[0] if amps else 0
        if any(np.shape(c) != (pts,) for c in carr):
            raise ValueError("All amplitude arrays must have the same length.")
        samples = np.ascontiguousarray(np.asarray(carr, dtype=self._ctype).reshape(amps, pts).ravel())
        if samples.size == 0:
            samples = np.zeros(1, dtype=self._ctype)
        w = np.ascontiguousarray(np.asarray(W, dtype=self._ctype).reshape(self.dim, self.dim).ravel())
        grad = np.zeros(max(amps * pts, 1), dtype=np.float64 if self._use_doubles else np.float32)
        self._check_error(self._fn('Parament_equipropVJP')(self._handle, samples, float(dt), pts, amps, w, grad))
        return grad[:amps * pts].reshape(amps, pts)

    def fidelity_gradient(self, dt, U_target, *carr):
        """Loss ``1 - |Tr(V^H U)|^2 / d^2`` for the target ``V = U_target`` and its
        gradient with respect to every real control sample: ``(loss, grad)``."""
        U = np.asarray(self.equiprop(dt, *carr), dtype=np.complex128)
        V = np.asarray(U_target, dtype=np.complex128)
        d = self.dim
        g = np.trace(V.conj().T @ U)
        loss = 1.0 - abs(g) ** 2 / d ** 2
        W = -(2.0 / d ** 2) * g * V
        return loss, self.vjp(dt, W, *carr)

    @_must_be_alive
    def vjp_device(self, dt, carr, W, grad=None, stream=None):
        """:meth:`vjp` on CUDA tensors: ``carr`` (amps, pts) and ``W`` (dim, dim)
        on the context's device; ``grad`` (amps, pts) real, allocated when None."""
        import torch

        ct = torch.complex128 if self._use_doubles else torch.complex64
        rt = torch.float64 if self._use_doubles else torch.float32
        carr = carr.to(ct)
        if carr.dim() == 1:
            carr = carr.unsqueeze(0)
        carr = carr.contiguous()
        W = W.to(ct).contiguous()
        amps, pts = carr.shape
        if amps > self.amps:
            raise ValueError(f'Got {amps} amplitude arrays, but there are only {self.amps} Hamiltonians.')
        if grad is None:
            grad = torch.empty((amps, pts), dtype=rt, device=carr.device)
        if stream is None:
            stream = torch.cuda.current_stream(carr.device)
        code = self._fn('Parament_equipropVJPDevice')(self._handle, ctypes.c_void_p(carr.data_ptr()), float(dt),
                                                      pts, amps, ctypes.c_void_p(W.data_ptr()),
                                                      ctypes.c_void_p(grad.data_ptr()), _stream_handle(stream))
        self._check_error(code)
        return grad

    # ------------------------------------------------------------------ errors

    @_must_be_alive
    def _get_error_message(self, code=None):
        if code is None:
            code = self._fn('Parament_peekAtLastError')(self._handle)
        return self._lib.Parament_errorMessage(code).decode()

    def _check_error(self, error_code):
        """Raise the exception that matches a C error code."""
        if error_code == PARAMENT_STATUS_SUCCESS:
            return
        try:
            exception_class = _EXCEPTIONS[error_code]
        except KeyError as e:
            raise AssertionError('Unknown error code ') from e
        message = self._lib.Parament_errorMessage(error_code).decode()
        raise exception_class(f"Error code {error_code}: {message}")

    def __enter__(self):
        return self

    def __exit__(self, exc_type, exc_val, exc_tb):
        self.destroy()
