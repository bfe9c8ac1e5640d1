"""The tensor-core split kernel (d = 64, complex64 contexts in split mode)
against the FP64 oracle on the same complex64 inputs.

The kernel forms every product from bf16 slices with exact accumulation and
keeps the running product in double-float, so each case must land within the
split form's bar of 1e-6 relative Frobenius error.  The cases cover the
quadrature modes, the Magnus terms, complex samples (the general assembly
branch), fewer steps than SMs, constant controls, and step sizes that push the
Chebyshev order up to the split form's limit.
"""
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

QUAD = {oracle.NONE: "none", oracle.MIDPOINT: "midpoint", oracle.SIMPSON: "simpson"}
TOL = 1e-6


def c64(x):
    return np.asarray(x).astype(np.complex64).astype(np.complex128)


def relerr(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


def problem(K, n, seed, norm0=10.0, complex_samples=False):
    from parament_gb300.workloads import hermitian
    rng = np.random.default_rng(seed)
    H0 = hermitian(rng, 64, norm0)
    H1 = np.stack([hermitian(rng, 64, 1.0) for _ in range(K)]) if K else np.zeros((0, 64, 64), complex)
    carr = rng.standard_normal((K, n)) + (1j * rng.standard_normal((K, n)) if complex_samples else 0)
    return c64(H0), c64(H1), c64(carr)


def split_equiprop(H0, H1, carr, dt, magnus, mode):
    import parament_gb300 as parament
    with parament.Parament("fp32") as ctx:
        ctx.set_precision_mode("split")
        ctx.set_hamiltonian(H0, *H1, use_magnus=magnus, quadrature_mode=QUAD[mode])
        U = ctx.equiprop(dt, *carr)
        return U.astype(np.complex128), ctx.last_iteration_cycles


@pytest.mark.parametrize("magnus,mode", [(False, oracle.NONE), (False, oracle.MIDPOINT), (False, oracle.SIMPSON),
                                         (True, oracle.SIMPSON)])
@pytest.mark.parametrize("complex_samples", [False, True])
def test_modes_and_samples(built_lib, magnus, mode, complex_samples):
    H0, H1, carr = problem(3, 301, seed=11, complex_samples=complex_samples)
    U, M = split_equiprop(H0, H1, list(carr), 1e-3, magnus, mode)
    Uo = oracle.equiprop(H0, H1, carr, 1e-3, magnus=magnus, mode=mode, nthreads=os.cpu_count())[0]
    assert relerr(U, Uo) < TOL


@pytest.mark.parametrize("steps", [1, 7, 151, 152, 153])
def test_fewer_steps_than_sms(built_lib, steps):
    H0, H1, carr = problem(2, steps, seed=steps)
    U, _ = split_equiprop(H0, H1, list(carr), 1e-3, False, oracle.NONE)
    Uo = oracle.equiprop(H0, H1, carr, 1e-3)[0]
    assert relerr(U, Uo) < TOL


def test_constant_zero_controls(built_lib):
    """Zero amplitudes: every step has X = H0, the same roundings each step."""
    H0, H1, _ = problem(1, 1, seed=3, norm0=5.0)
    carr = np.zeros((1, 400), np.complex128)
    U, _ = split_equiprop(H0, H1, list(carr), 1e-3, False, oracle.NONE)
    Uo = oracle.equiprop(H0, H1, carr, 1e-3)[0]
    assert relerr(U, Uo) < TOL


@pytest.mark.parametrize("dt,order", [(1e-4, 3), (6e-3, 7), (1.6e-2, 9)])
def test_chebyshev_orders(built_lib, dt, order):
    """Larger steps raise the split order (more even powers in the kernel)."""
    H0, H1, carr = problem(2, 257, seed=5, norm0=5.0)
    U, M = split_equiprop(H0, H1, list(carr), dt, False, oracle.NONE)
    Uo = oracle.equiprop(H0, H1, carr, dt, nthreads=os.cpu_count())[0]
    assert M == order
    assert relerr(U, Uo) < TOL, (M, relerr(U, Uo))


def test_magnus_complex_samples_2048(built_lib):
    H0, H1, carr = problem(4, 2 * 2048 + 1, seed=21, complex_samples=True)
    U, M = split_equiprop(H0, H1, list(carr), 1e-3, True, oracle.SIMPSON)
    Uo = oracle.equiprop(H0, H1, carr, 1e-3, magnus=True, mode=oracle.SIMPSON, nthreads=os.cpu_count())[0]
    assert relerr(U, Uo) < TOL


def test_repeated_calls_agree(built_lib):
    """The kernel keeps no state between calls: two calls give the same bits."""
    H0, H1, carr = problem(2, 1000, seed=8)
    U1, _ = split_equiprop(H0, H1, list(carr), 1e-3, False, oracle.NONE)
    U2, _ = split_equiprop(H0, H1, list(carr), 1e-3, False, oracle.NONE)
    assert np.array_equal(U1, U2)


def test_fewer_sample_arrays_than_controls(built_lib):
    """Magnus with 4 controls loaded and 2 sample arrays: the rest are zero."""
    H0, H1, carr = problem(4, 2 * 300 + 1, seed=31)
    U, _ = split_equiprop(H0, H1, list(carr[:2]), 1e-3, True, oracle.SIMPSON)
    full = np.concatenate([carr[:2], np.zeros_like(carr[2:])])
    Uo = oracle.equiprop(H0, H1, full, 1e-3, magnus=True, mode=oracle.SIMPSON, nthreads=os.cpu_count())[0]
    assert relerr(U, Uo) < TOL


def test_matches_simt_split_kernel(built_lib):
    """The tensor-core kernel and the SIMT split kernel (tensor cores disabled
    through PARAMENT_DISABLE_TENSOR_CORES in a child process) agree within the
    split form's bar, on the d=64 Magnus workload at 4096 steps."""
    import subprocess
    import sys
    import tempfile
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys, numpy as np, parament_gb300 as p\n"
            "from parament_gb300 import workloads\n"
            "w = workloads.magnus_d64(4096)\n"
            "c = lambda x: x.astype(np.complex64)\n"
            "ctx = p.Parament('fp32'); ctx.set_precision_mode('split')\n"
            "ctx.set_hamiltonian(c(w['H0']), *c(w['H1']), use_magnus=True, quadrature_mode='simpson')\n"
            "np.save(sys.argv[1], ctx.equiprop(w['dt'], *c(w['carr'])))\n")
    outs = []
    with tempfile.TemporaryDirectory() as tmp:
        for tag, env in (("tc", {}), ("simt", {"PARAMENT_DISABLE_TENSOR_CORES": "1"})):
            f = os.path.join(tmp, tag + ".npy")
            r = subprocess.run([sys.executable, "-c", code, f], cwd=root, env=dict(os.environ, **env),
                               capture_output=True, text=True, timeout=600)
            assert r.returncode == 0, r.stderr
            outs.append(np.load(f).astype(np.complex128))
    assert relerr(outs[0], outs[1]) < TOL
    assert not np.array_equal(outs[0], outs[1])  # two different kernels ran


def test_two_step_batches(built_lib):
    """More steps than one batch of X planes (65536): the step kernel runs
    once per batch and the chunk products of both batches meet in the tree.
    Checked against the FP64 oracle on the same complex64 inputs."""
    H0, H1, carr = problem(2, 65536 + 257, seed=13, norm0=5.0)
    U, _ = split_equiprop(H0, H1, list(carr), 1e-3, False, oracle.NONE)
    Uo = oracle.equiprop(H0, H1, carr, 1e-3, nthreads=os.cpu_count())[0]
    assert relerr(U, Uo) < TOL


def test_wide_expansion_magnus_k5(built_lib):
    """Magnus with five controls: 20 expansion matrices (H_k, [H0, H_k] and the
    pair commutators), more than the assemble kernel keeps in registers, so its
    shared-memory form runs."""
    H0, H1, carr = problem(5, 2 * 700 + 1, seed=41)
    U, _ = split_equiprop(H0, H1, list(carr), 1e-3, True, oracle.SIMPSON)
    Uo = oracle.equiprop(H0, H1, carr, 1e-3, magnus=True, mode=oracle.SIMPSON, nthreads=os.cpu_count())[0]
    assert relerr(U, Uo) < TOL


@pytest.mark.parametrize("dt,magnus,order,n,seed", [(1e-3, True, 7, 2 * 1024 + 1, 17), (1.6e-2, False, 9, 257, 5)])
def test_hermitian_steps_bit_identical(built_lib, dt, magnus, order, n, seed):
    """Hermitian inputs with real samples take the kernel's Hermitian-step
    shortcut (the B operands of X X, X^2 X^2 and X^(2k-2) X^2 read from the A
    slices).  Those slices are the numbers the B slicing would produce, so the
    propagator is bit-identical to the general path's (shortcut switched off
    with PARAMENT_SPLIT_HERMITIAN=0); order 9 also covers X^8 = X^6 X^2."""
    K = 4 if magnus else 2
    H0, H1, carr = problem(K, n, seed=seed, norm0=5.0 if order == 9 else 10.0)
    mode = oracle.SIMPSON if magnus else oracle.NONE
    U1, M = split_equiprop(H0, H1, list(carr), dt, magnus, mode)
    old = os.environ.get("PARAMENT_SPLIT_HERMITIAN")
    os.environ["PARAMENT_SPLIT_HERMITIAN"] = "0"
    try:
        U0, _ = split_equiprop(H0, H1, list(carr), dt, magnus, mode)
    finally:
        if old is None:
            del os.environ["PARAMENT_SPLIT_HERMITIAN"]
        else:
            os.environ["PARAMENT_SPLIT_HERMITIAN"] = old
    assert M == order
    assert np.array_equal(U1, U0)
    Uo = oracle.equiprop(H0, H1, carr, dt, magnus=magnus, mode=mode, nthreads=os.cpu_count())[0]
    assert relerr(U1, Uo) < TOL


def test_non_hermitian_hamiltonian(built_lib):
    """A drift with a small anti-Hermitian part (a lossy system): no step is
    Hermitian, every product slices its B operand.  Against the FP64 oracle."""
    from parament_gb300.workloads import hermitian
    H0, H1, carr = problem(3, 2 * 500 + 1, seed=23)
    H0 = c64(H0 + 0.05j * hermitian(np.random.default_rng(24), 64, 1.0))
    U, _ = split_equiprop(H0, H1, list(carr), 1e-3, True, oracle.SIMPSON)
    Uo = oracle.equiprop(H0, H1, carr, 1e-3, magnus=True, mode=oracle.SIMPSON, nthreads=os.cpu_count())[0]
    assert relerr(U, Uo) < TOL


def test_hermitian_and_general_steps_mixed(built_lib):
    """Samples with imaginary parts on a few stretches only: steps touching
    them take the general path, the others the Hermitian one, within one
    chunk.  Against the FP64 oracle."""
    H0, H1, carr = problem(3, 2 * 3000 + 1, seed=29)
    rng = np.random.default_rng(30)
    for lo in (100, 2000, 4500):
        carr[:, lo:lo + 37] += 1j * rng.standard_normal((3, 37))
    carr = c64(carr)
    U, _ = split_equiprop(H0, H1, list(carr), 1e-3, True, oracle.SIMPSON)
    Uo = oracle.equiprop(H0, H1, carr, 1e-3, magnus=True, mode=oracle.SIMPSON, nthreads=os.cpu_count())[0]
    assert relerr(U, Uo) < TOL
