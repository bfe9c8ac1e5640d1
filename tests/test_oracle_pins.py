"""Pins the CPU oracle before it is trusted as the checker.

Against the reference's own known answers (docstring example, the seed-27
problems of its test_numerics.py with its tolerances), the reference's host
functions (golden values taken from the reference built from its sources),
and an independent SciPy expm product for every quadrature mode.
"""
import os

import numpy as np
import pytest
import scipy.linalg

import oracle

from conftest import ROOT


def seed27(dim):
    np.random.seed(27)
    H0 = np.random.uniform(-1, 1, (dim, dim)) / dim + 1j * np.random.uniform(-1, 1, (dim, dim)) / 2
    return H0 + H0.conj().T


def test_docstring_known_answer():
    # src/python/pyparament/parament/parament.py:61-68
    U, M, hn, st = oracle.equiprop(np.diag([1.0, -1.0]), np.array([[0, 1], [1, 0]]), np.zeros(1), 1.0, single=True)
    assert st == 0
    want = np.diag([0.54030234 - 0.84147096j, 0.54030234 + 0.84147096j])
    assert np.allclose(U, want, atol=1e-7)


@pytest.mark.parametrize("dim", [2, 16])
@pytest.mark.parametrize("single", [True, False])
def test_seed27_single_step_vs_scipy(dim, single):
    # test_numerics.py:32-57 and :72-97: sum |diff| < eps * dim^2
    H0 = seed27(dim)
    U, M, hn, st = oracle.equiprop(H0, np.zeros((dim, dim)), np.zeros(1), 0.01, single=single)
    assert st == 0
    err = np.sum(np.abs(U - scipy.linalg.expm(-1j * 0.01 * H0)))
    eps = np.finfo(np.float32 if single else np.float64).eps
    assert err < eps * dim * dim


@pytest.mark.parametrize("dim", [2, 4])
def test_seed27_debug_expm(dim):
    # test_numerics.py:60-69: expm(m) through H0 = i m, H1 = m, dt = 1
    m = seed27(dim)
    U, M, hn, st = oracle.equiprop(1j * m, m, np.zeros(1), 1.0, single=True)
    assert st == 0
    err = np.sum(np.abs(U - scipy.linalg.expm(m)))
    assert err < np.finfo(np.float32).eps * dim * dim


@pytest.mark.parametrize("dim", [2, 16])
def test_seed27_multi_fields_time_ordering(dim):
    # test_numerics.py:100-117: ten steps, two fields, later step on the left
    H0 = seed27(dim)
    H1 = np.zeros((dim, dim), complex)
    c1, c2 = np.random.rand(10), np.random.rand(10)
    U, M, hn, st = oracle.equiprop(H0, np.stack([H1, H0]), np.stack([c1, c2]), 0.01, single=True)
    ref = np.eye(dim, dtype=complex)
    for i in range(10):
        ref = scipy.linalg.expm(-1j * 0.01 * (H0 + c1[i] * H1 + c2[i] * H0)) @ ref
    assert np.linalg.norm(ref - U) < 1e-6


@pytest.mark.parametrize("magnus,mode", [(False, oracle.NONE), (False, oracle.MIDPOINT),
                                         (False, oracle.SIMPSON), (True, oracle.SIMPSON)])
@pytest.mark.parametrize("K", [1, 2, 3, 5])
def test_modes_vs_scipy(magnus, mode, K):
    rng = np.random.default_rng(K + 10 * int(magnus) + mode % 7)
    d = 6
    def herm():
        a = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
        return (a + a.conj().T) / 2
    H0, H1 = herm(), np.stack([herm() for _ in range(K)])
    carr = rng.standard_normal((K, 15)) + 0.2j * rng.standard_normal((K, 15))
    U, M, hn, st = oracle.equiprop(H0, H1, carr, 0.01, magnus=magnus, mode=mode)
    R = oracle.scipy_expm_product(H0, H1, carr, 0.01, magnus=magnus, mode=mode)
    assert st == 0
    assert np.linalg.norm(U - R) / np.linalg.norm(R) < 1e-12


def test_magnus_commutator_orientation():
    # [H0,H_k] and [H_j,H_i] (j<i) as the reference forms them for row-major
    # data (src/cuda/parament.cpp:295-358)
    rng = np.random.default_rng(3)
    d, K = 4, 3
    H0 = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    H1 = rng.standard_normal((K, d, d)) + 1j * rng.standard_normal((K, d, d))
    st = oracle.build_stack(H0, H1, True)
    for k in range(K):
        assert np.allclose(st[1 + K + k], H0 @ H1[k] - H1[k] @ H0)
    slot = 1 + 2 * K
    for i in range(1, K):
        for j in range(i):
            assert np.allclose(st[slot + i * (i - 1) // 2 + j], H1[j] @ H1[i] - H1[i] @ H1[j])


def test_order_tables_match_reference(ref_host):
    for x, m32, m64 in ref_host["cycles"]:
        assert oracle.select_cycles(x, 1.0, fp64=False) == m32, x
        assert oracle.select_cycles(x, 1.0, fp64=True) == m64, x


def test_onenorm_matches_reference(ref_host):
    for n in ref_host["norms"]:
        d = n["d"]
        m = (np.array(n["re"]) + 1j * np.array(n["im"])).reshape(d, d)
        assert oracle.onenorm(m) == pytest.approx(n["onenorm_fp64"], rel=1e-15)
        m32 = m.astype(np.complex64).astype(np.complex128)
        assert oracle.onenorm(m32, single=True) == pytest.approx(n["onenorm_fp32"], rel=1e-6)


def test_golden_cases_reproduce(golden_cases):
    for c in golden_cases:
        U, M, hn, st = oracle.equiprop(c["H0"], c["H1"], c["carr"], c["dt"], magnus=c["magnus"], mode=c["mode"],
                                       single=(c["precision"] == "fp32"))
        assert st == 0 and M == c["M"], c["name"]
        assert np.allclose(U, c["U"], rtol=0, atol=1e-13), c["name"]


def test_live_reference_host_functions():
    """Only where the reference sources are present (the build container)."""
    so = os.path.join(ROOT, "oracle", "_ref", "libparament_ref.so")
    if not os.path.exists(so):
        pytest.skip("reference host library not built here")
    import ctypes
    L = ctypes.CDLL(so)
    L.Parament_selectIterationCycles_fp64.argtypes = [ctypes.c_double, ctypes.c_double]
    rng = np.random.default_rng(11)
    for _ in range(200):
        hn, dt = rng.uniform(0, 100), rng.uniform(0, 0.2)
        assert L.Parament_selectIterationCycles_fp64(hn, dt) == oracle.select_cycles(hn, dt, fp64=True)


def test_threads_do_not_change_result():
    rng = np.random.default_rng(5)
    d = 8
    a = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    H0 = (a + a.conj().T) / 2
    carr = rng.standard_normal((1, 101))
    U1 = oracle.equiprop(H0, H0 * 0.3, carr, 0.01, nthreads=1)[0]
    U4 = oracle.equiprop(H0, H0 * 0.3, carr, 0.01, nthreads=4)[0]
    assert np.array_equal(U1, U4)
