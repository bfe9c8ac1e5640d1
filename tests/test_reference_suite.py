"""The reference's own pyparament test-suite, run against this library
(src/python/pyparament/parament/test/test_error.py, test_wrapper.py,
test_numerics.py), with the same inputs, messages and tolerances."""
import numpy as np
import pytest
import scipy.linalg

pytestmark = pytest.mark.gpu


@pytest.fixture
def parament(built_lib):
    import parament_gb300
    return parament_gb300


@pytest.fixture
def context(parament):
    with parament.Parament() as runner:
        yield runner


def random_hamiltonians(dim):
    np.random.seed(27)
    H0 = np.random.uniform(-1, 1, (dim, dim)) / dim + 1j * np.random.uniform(-1, 1, (dim, dim)) / 2
    H0 = H0 + H0.conj().T
    return H0, np.zeros((dim, dim), dtype=complex)


# ---- test_error.py
def test_use_after_destruction(parament):
    ctx = parament.Parament()
    ctx.destroy()
    with pytest.raises(RuntimeError, match='Attempting to use a context that has been destroyed'):
        ctx.set_hamiltonian(np.eye(2), np.eye(2))


def test_propagate_no_hamiltonian(context):
    with pytest.raises(RuntimeError, match='No hamiltonian set'):
        context.equiprop(1.0)


def test_invalid_quadrature_selection(context):
    with pytest.raises(ValueError, match='Invalid quadrature selection'):
        context.set_hamiltonian(np.eye(2), np.eye(2), use_magnus=True, quadrature_mode='none')
    with pytest.raises(ValueError, match='Invalid quadrature selection'):
        context.set_hamiltonian(np.eye(2), np.eye(2), use_magnus=True, quadrature_mode='midpoint')


def test_propagate_unset_amplitudes(context):
    context.set_hamiltonian(np.eye(2), np.eye(2))
    with pytest.raises(ValueError, match='Got 2 amplitude arrays, but there are only 1 Hamiltonians.'):
        context.equiprop(1.0, np.zeros(4), np.zeros(4))


def test_propagate_unequal_amplitude_size(context):
    context.set_hamiltonian(np.eye(2), np.eye(2), np.eye(2))
    with pytest.raises(ValueError, match='All amplitude arrays must have the same length.'):
        context.equiprop(1.0, np.zeros(4), np.zeros(5))


# ---- test_wrapper.py
def test_smoke(parament):
    runner = parament.Parament()
    runner.set_hamiltonian(np.array([[1, 0], [0, -1]]), np.array([[0, 1], [1, 0]]))
    runner.destroy()


def test_context_manager(parament):
    with parament.Parament() as runner:
        runner.set_hamiltonian(np.array([[1, 0], [0, -1]]), np.array([[0, 1], [1, 0]]))
        runner.equiprop(1.0, np.zeros(1))
    assert runner._handle is None


def test_device_info(parament, capfd):
    parament.device_info()
    out = capfd.readouterr().out
    assert "Total number of CUDA devices" in out


def test_docstring_example(parament):
    with parament.Parament() as runner:
        runner.set_hamiltonian(np.array([[1, 0], [0, -1]]), np.array([[0, 1], [1, 0]]))
        U = runner.equiprop(1.0, np.zeros(1))
    assert U.dtype == np.complex64
    assert np.allclose(U, np.diag([0.54030234 - 0.84147096j, 0.54030234 + 0.84147096j]), atol=1e-6)


# ---- test_numerics.py
@pytest.mark.parametrize("dim", [2, 16])
def test_fp32_expm_scipy_random(parament, dim):
    H0, H1 = random_hamiltonians(dim)
    with parament.Parament() as ctx:
        ctx.set_hamiltonian(H0, H1, use_magnus=False, quadrature_mode='none')
        U = ctx.equiprop(0.01, np.zeros(1))
    err = np.sum(np.abs(U - scipy.linalg.expm(-1j * 0.01 * H0)))
    assert err < np.finfo(np.float32).eps * dim * dim


@pytest.mark.parametrize("dim", [2, 4])
def test_fp32_expm_debug(parament, dim):
    H0, _ = random_hamiltonians(dim)
    err = np.sum(np.abs(parament.expm(H0) - scipy.linalg.expm(H0)))
    assert err < np.finfo(np.float32).eps * dim * dim


@pytest.mark.parametrize("dim", [2, 16])
def test_fp64_expm_scipy_random(parament, dim):
    H0, H1 = random_hamiltonians(dim)
    with parament.Parament(precision='fp64') as ctx:
        ctx.set_hamiltonian(H0, H1, use_magnus=False, quadrature_mode='none')
        U = ctx.equiprop(0.01, np.zeros(1))
    err = np.sum(np.abs(U - scipy.linalg.expm(-1j * 0.01 * H0)))
    assert err < np.finfo(np.float64).eps * dim * dim


@pytest.mark.parametrize("dim", [2, 16])
def test_fp32_multi_fields(parament, dim):
    H0, H1 = random_hamiltonians(dim)
    H2 = H0[:, :]
    c1, c2 = np.random.rand(10), np.random.rand(10)
    with parament.Parament(precision='fp32') as ctx:
        ctx.set_hamiltonian(H0, H1, H2, use_magnus=False, quadrature_mode='none')
        U = ctx.equiprop(0.01, c1, c2)
    ref = np.eye(dim, dtype=np.complex128)
    for i in range(len(c1)):
        ref = scipy.linalg.expm(-1j * (H0 + c1[i] * H1 + c2[i] * H2) * 0.01) @ ref
    assert np.linalg.norm(ref - U) < 1e-6
