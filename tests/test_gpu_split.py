"""The split-precision complex64 form against the FP64 oracle.

The split form targets the exact propagator, not the reference's complex64
rounding, so its parity bar is the FP64 oracle on the complex64 inputs:
relative Frobenius error <= 1e-6 (the bar of the precision workload).
"""
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

QUAD = {0: "none", 0x01000000: "midpoint", 0x02000000: "simpson"}


def relerr(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


def c64(x):
    return np.asarray(x).astype(np.complex64).astype(np.complex128)


def run_split(H0, H1, carr, dt, magnus=False, mode=0):
    import parament_gb300 as parament
    with parament.Parament("fp32") as ctx:
        ctx.set_precision_mode("split")
        ctx.set_hamiltonian(H0, *H1, use_magnus=magnus, quadrature_mode=QUAD[mode])
        U = ctx.equiprop(dt, *carr)
        return U.astype(np.complex128), ctx.last_iteration_cycles


def test_split_golden_cases(built_lib, golden_cases):
    bad = []
    for c in golden_cases:
        if c["precision"] != "fp32" or c["hnorm"] * c["dt"] * (2 if c["mode"] == oracle.SIMPSON else 1) > 0.5:
            continue
        U, M = run_split(c["H0"], c["H1"], list(c["carr"]), c["dt"], c["magnus"], c["mode"])
        Uo = oracle.equiprop(c["H0"], c["H1"], c["carr"], c["dt"], magnus=c["magnus"], mode=c["mode"])[0]
        # a single rounding of the complex64 output is the floor for one-step cases
        e = relerr(U, Uo)
        if e > 1e-6:
            bad.append((c["name"], e))
    assert not bad, bad


def test_split_magnus_d64_reduced(built_lib):
    from parament_gb300 import workloads
    w = workloads.magnus_d64(steps=512)
    H0, H1, carr = c64(w["H0"]), c64(w["H1"]), c64(w["carr"])
    U, M = run_split(H0, H1, list(carr), w["dt"], True, oracle.SIMPSON)
    Uo = oracle.equiprop(H0, H1, carr, w["dt"], magnus=True, mode=oracle.SIMPSON, nthreads=os.cpu_count())[0]
    assert relerr(U, Uo) < 1e-6


def test_split_constant_controls_no_drift(built_lib):
    """Constant amplitudes repeat every rounding at every step: the case where
    plain complex64 drifts coherently."""
    import parament_gb300 as parament
    from parament_gb300.workloads import hermitian
    rng = np.random.default_rng(4)
    H0 = c64(hermitian(rng, 16, 10.0))
    H1 = c64(np.stack([hermitian(rng, 16, 1.0) for _ in range(2)]))
    carr = np.ones((2, 20000))
    U, _ = run_split(H0, H1, list(carr), 1e-3)
    with parament.Parament("fp64") as ctx:
        ctx.set_hamiltonian(H0, *H1)
        U64 = ctx.equiprop(1e-3, *carr)
    with parament.Parament("fp32") as ctx:
        ctx.set_hamiltonian(H0, *H1)
        U32 = ctx.equiprop(1e-3, *carr).astype(np.complex128)
    e_split, e_plain = relerr(U, U64), relerr(U32, U64)
    assert e_split < 1e-6, (e_split, e_plain)
    assert e_split < e_plain / 10


def test_split_full_size_error_bar(built_lib):
    """65536-step Magnus workload: split complex64 within 1e-6 of FP64."""
    import parament_gb300 as parament
    from parament_gb300 import workloads
    w = workloads.magnus_d64()
    H0, H1, carr = c64(w["H0"]), c64(w["H1"]), c64(w["carr"])
    U, M = run_split(H0, H1, list(carr), w["dt"], True, oracle.SIMPSON)
    with parament.Parament("fp64") as ctx:
        ctx.set_hamiltonian(H0, *H1, use_magnus=True, quadrature_mode="simpson")
        U64 = ctx.equiprop(w["dt"], *carr)
    assert relerr(U, U64) < 1e-6


def test_split_rejects_large_steps(built_lib):
    import parament_gb300 as parament
    with parament.Parament("fp32") as ctx:
        ctx.set_precision_mode("split")
        ctx.set_hamiltonian(np.diag([1.0, -1.0]), np.eye(2))
        with pytest.raises(RuntimeError, match="Timestep too large"):
            ctx.equiprop(0.5, np.zeros(4))  # Hnorm*dt = 1 > 0.5
        U = ctx.equiprop(0.1, np.zeros(4))
        assert np.allclose(U, np.diag(np.exp(-0.4j * np.array([1, -1]))), atol=1e-6)


def test_split_mode_only_for_fp32(built_lib):
    import parament_gb300 as parament
    with parament.Parament("fp64") as ctx:
        with pytest.raises(ValueError):
            ctx.set_precision_mode("split")


@pytest.mark.parametrize("d", [24, 40])
def test_split_partial_tiles(built_lib, d):
    """Dimensions that are not multiples of 16 (the SIMT split kernel and the
    double-float chunk tree with partial 16 x 16 tiles), Magnus with Simpson."""
    from parament_gb300.workloads import hermitian
    rng = np.random.default_rng(d)
    H0 = c64(hermitian(rng, d, 5.0))
    H1 = c64(np.stack([hermitian(rng, d, 1.0) for _ in range(2)]))
    carr = c64(rng.standard_normal((2, 2 * 500 + 1)))
    U, _ = run_split(H0, H1, list(carr), 1e-3, True, oracle.SIMPSON)
    Uo = oracle.equiprop(H0, H1, carr, 1e-3, magnus=True, mode=oracle.SIMPSON, nthreads=os.cpu_count())[0]
    assert relerr(U, Uo) < 1e-6
