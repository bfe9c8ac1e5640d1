"""qutip interop of the Python wrapper (src/python/pyparament/parament/parament.py:162-166,
185-188, 274-275): a ``Qobj`` drift makes equiprop return a ``Qobj`` with the
drift's dims, and ``Qobj`` control Hamiltonians are converted to dense arrays.

qutip is not installed here, so the module's qutip binding is replaced by a
minimal type with the parts of the ``Qobj`` interface the wrapper uses:
``full()``, ``dims`` and the ``Qobj(array, dims=...)`` constructor.
"""
import types

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


class FakeQobj:
    def __init__(self, data, dims=None):
        self._a = np.asarray(data)
        n = self._a.shape[0]
        self.dims = dims if dims is not None else [[n], [n]]
        self.data = object()  # no todense(): the wrapper falls back to full()

    def full(self):
        return self._a


@pytest.fixture
def fake_qutip(monkeypatch):
    from parament_gb300 import parament as mod
    monkeypatch.setattr(mod, "qutip", types.SimpleNamespace(Qobj=FakeQobj))
    return mod


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-5)])
def test_qobj_in_qobj_out(built_lib, fake_qutip, precision, tol):
    rng = np.random.default_rng(4)
    from parament_gb300.workloads import hermitian
    H0 = hermitian(rng, 4, 1.0)
    H1 = hermitian(rng, 4, 1.0)
    carr = rng.standard_normal(50)
    with fake_qutip.Parament(precision) as ctx:
        ctx.set_hamiltonian(FakeQobj(H0, dims=[[2, 2], [2, 2]]), FakeQobj(H1))
        U = ctx.equiprop(1e-2, carr)
    assert isinstance(U, FakeQobj)
    assert U.dims == [[2, 2], [2, 2]]
    if precision == "fp32":
        H0, H1, carr = (x.astype(np.complex64).astype(np.complex128) for x in (H0, H1, carr))
    Uo = oracle.equiprop(H0, H1[None], carr[None], 1e-2, single=precision == "fp32")[0]
    assert np.linalg.norm(U.full() - Uo) / np.linalg.norm(Uo) < tol


def test_plain_arrays_return_arrays(built_lib, fake_qutip):
    rng = np.random.default_rng(5)
    H0 = rng.standard_normal((3, 3))
    H0 = H0 + H0.T
    with fake_qutip.Parament("fp64") as ctx:
        ctx.set_hamiltonian(H0, np.eye(3))
        U = ctx.equiprop(1e-2, np.zeros(4))
    assert isinstance(U, np.ndarray) and U.shape == (3, 3)
