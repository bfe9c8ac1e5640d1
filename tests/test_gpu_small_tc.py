"""The plain complex64 form at d = 64 on the tensor cores (k_small_tc).

Checked against the oracle in the complex64 context (the reference's complex64
order table and norm moduli) on the same complex64-rounded inputs, within the
complex64 parity bar of 1e-5 relative Frobenius error, and against the FP32
SIMT kernel it replaces (tensor cores switched off through
PARAMENT_DISABLE_TENSOR_CORES in a child process).  Cases: every quadrature
mode with Magnus, complex samples, fewer steps than SMs, manual Chebyshev
orders from 1 to 15, more steps than one batch of X planes, and the fall-back
to the SIMT kernel when the plane buffer cannot be allocated.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

QUAD = {oracle.NONE: "none", oracle.MIDPOINT: "midpoint", oracle.SIMPSON: "simpson"}
TOL = 1e-5


def c64(x):
    return np.asarray(x).astype(np.complex64).astype(np.complex128)


def relerr(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


def problem(K, n, seed, norm0=10.0, complex_samples=False):
    from parament_gb300.workloads import hermitian
    rng = np.random.default_rng(seed)
    H0 = hermitian(rng, 64, norm0)
    H1 = np.stack([hermitian(rng, 64, 1.0) for _ in range(K)])
    carr = rng.standard_normal((K, n)) + (1j * rng.standard_normal((K, n)) if complex_samples else 0)
    return c64(H0), c64(H1), c64(carr)


def plain_equiprop(H0, H1, carr, dt, magnus=False, mode=oracle.NONE, cycles=None):
    import parament_gb300 as parament
    with parament.Parament("fp32") as ctx:
        ctx.set_hamiltonian(H0, *H1, use_magnus=magnus, quadrature_mode=QUAD[mode])
        if cycles is not None:
            ctx.set_iteration_cycles_manually(cycles)
        U = ctx.equiprop(dt, *carr)
        return U.astype(np.complex128), ctx.last_iteration_cycles


@pytest.mark.parametrize("magnus,mode", [(False, oracle.NONE), (False, oracle.MIDPOINT), (False, oracle.SIMPSON),
                                         (True, oracle.SIMPSON)])
@pytest.mark.parametrize("complex_samples", [False, True])
def test_modes_and_samples(built_lib, magnus, mode, complex_samples):
    H0, H1, carr = problem(3, 401, seed=51, complex_samples=complex_samples)
    U, M = plain_equiprop(H0, H1, list(carr), 1e-3, magnus, mode)
    Uo, Mo, _, _ = oracle.equiprop(H0, H1, carr, 1e-3, magnus=magnus, mode=mode, single=True,
                                   nthreads=os.cpu_count())
    assert M == Mo
    assert relerr(U, Uo) < TOL


@pytest.mark.parametrize("steps", [1, 7, 151, 152, 153])
def test_fewer_steps_than_sms(built_lib, steps):
    H0, H1, carr = problem(2, steps, seed=60 + steps)
    U, _ = plain_equiprop(H0, H1, list(carr), 1e-3)
    Uo = oracle.equiprop(H0, H1, carr, 1e-3, single=True)[0]
    assert relerr(U, Uo) < TOL


@pytest.mark.parametrize("cycles", [1, 3, 9, 15])
def test_manual_orders(built_lib, cycles):
    """Manual orders: M = 1 has no Clenshaw product (U = s J_1 X + J_0 I), the
    others 1 .. 14 of them per step."""
    H0, H1, carr = problem(2, 300, seed=70 + cycles, norm0=2.0)
    U, M = plain_equiprop(H0, H1, list(carr), 1e-3, cycles=cycles)
    Uo = oracle.equiprop(H0, H1, carr, 1e-3, single=True, M=cycles, nthreads=os.cpu_count())[0]
    assert M == cycles
    assert relerr(U, Uo) < TOL


def test_two_batches(built_lib):
    """More steps than one batch of X planes (65536): two assemble + step
    kernel launches whose chunk products meet in the double-float tree."""
    H0, H1, carr = problem(2, 65536 + 300, seed=81, norm0=5.0)
    U, M = plain_equiprop(H0, H1, list(carr), 1e-3)
    Uo, Mo, _, _ = oracle.equiprop(H0, H1, carr, 1e-3, single=True, nthreads=os.cpu_count())
    assert M == Mo
    assert relerr(U, Uo) < TOL


def test_matches_simt_kernel(built_lib):
    """The tensor-core kernel and the FP32 SIMT kernel it replaces agree within
    the complex64 bar on the d=64 Magnus workload at 4096 steps."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys, numpy as np, parament_gb300 as p\n"
            "from parament_gb300 import workloads\n"
            "w = workloads.magnus_d64(4096)\n"
            "c = lambda x: x.astype(np.complex64)\n"
            "ctx = p.Parament('fp32')\n"
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


_FALLBACK_CASE = """
import sys, numpy as np, torch
import parament_gb300 as p
from parament_gb300.workloads import hermitian
rng = np.random.default_rng(91)
c = lambda x: x.astype(np.complex64)
H0 = hermitian(rng, 64, 5.0)
H1 = np.stack([hermitian(rng, 64, 1.0) for _ in range(2)])
carr = rng.standard_normal((2, 20000))
ctx = p.Parament('fp32')
ctx.set_hamiltonian(c(H0), *c(H1))
U = ctx.equiprop_device(1e-3, torch.tensor(c(carr), device='cuda'))
torch.cuda.synchronize()
np.save(sys.argv[1], U.cpu().numpy())
print('BYTES', ctx.device_memory_bytes)
"""


def test_falls_back_when_planes_cannot_be_allocated(built_lib):
    """Host-side fault injection fails the X plane buffer (the fifth device
    allocation: stack, chunks, work, tree buffer, planes): the propagation runs
    on the FP32 SIMT kernel, which holds no planes, and still meets the bar."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    with tempfile.TemporaryDirectory() as tmp:
        f = os.path.join(tmp, "U.npy")
        env = dict(os.environ, PARAMENT_FAIL_ALLOC_AFTER="4")
        r = subprocess.run([sys.executable, "-c", _FALLBACK_CASE, f], cwd=root, env=env, capture_output=True,
                           text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        U = np.load(f).astype(np.complex128)
    held = int(r.stdout.split("BYTES")[1].split()[0])
    assert held < 200 << 20, held  # no plane buffer (it would take 696 MB)
    from parament_gb300.workloads import hermitian
    rng = np.random.default_rng(91)
    H0 = c64(hermitian(rng, 64, 5.0))
    H1 = c64(np.stack([hermitian(rng, 64, 1.0) for _ in range(2)]))
    carr = c64(rng.standard_normal((2, 20000)))
    Uo = oracle.equiprop(H0, H1, carr, 1e-3, single=True, nthreads=os.cpu_count())[0]
    assert relerr(U, Uo) < TOL
