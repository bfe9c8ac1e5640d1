"""Batched ensembles (one persistent launch in a CUDA graph) against the
single-problem path and the CPU oracle.

Tolerances: complex128 ensembles agree with the single-problem path to 1e-12
and with the oracle to 1e-10; complex64 ensembles with the single-problem
complex64 path to 1e-5 (relative Frobenius error; the chunking differs, so
the rounding does).
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

QUAD = {"none": oracle.NONE, "midpoint": oracle.MIDPOINT, "simpson": oracle.SIMPSON}


def relerr(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


def mixed_problems(seed, n=40):
    from parament_gb300.workloads import hermitian, sinusoid_controls
    rng = np.random.default_rng(seed)
    dims = [2, 3, 4, 5, 7, 8, 12, 16, 20, 31, 32, 40, 63, 64]
    out = []
    for i in range(n):
        d = dims[i % len(dims)]
        K = int(rng.integers(1, 5))
        pts = int(rng.integers(3, 400))
        H0 = hermitian(rng, d, float(rng.uniform(0.5, 3.0)))
        H1 = np.stack([hermitian(rng, d, 1.0) for _ in range(K)])
        out.append((H0, H1, 1e-2, sinusoid_controls(rng, K, pts, 1e-2)))
    return out


def single(H0, H1, dt, carr, precision, mode):
    import parament_gb300 as parament
    with parament.Parament(precision) as ctx:
        ctx.set_hamiltonian(H0, *H1, quadrature_mode=mode)
        return ctx.equiprop(dt, *carr).astype(np.complex128)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("mode", ["none", "midpoint", "simpson"])
def test_ensemble_matches_single_problem(built_lib, precision, mode):
    from parament_gb300.ensemble import Ensemble
    probs = mixed_problems(hash((precision, mode)) % 1000)
    with Ensemble([(H0, H1, dt, c.shape[1]) for H0, H1, dt, c in probs], precision, mode) as ens:
        ens.set_samples([c for *_, c in probs])
        Us = ens.run()
        for _ in range(2):  # graph replays give the same result
            again = ens.run()
            assert all(np.array_equal(a, b) for a, b in zip(Us, again))
    tol = 1e-12 if precision == "fp64" else 1e-5
    bad = []
    for (H0, H1, dt, carr), U in zip(probs, Us):
        ref = single(H0, H1, dt, carr, precision, mode)
        e = relerr(U, ref)
        if e > tol:
            bad.append((H0.shape[0], carr.shape, e))
    assert not bad, bad
    if precision == "fp64":
        for i in range(8):
            H0, H1, dt, carr = probs[i]
            Uo = oracle.equiprop(H0, H1, carr, dt, mode=QUAD[mode])[0]
            assert relerr(Us[i], Uo) < 1e-10


def test_ensemble_tune_keeps_results(built_lib):
    from parament_gb300.ensemble import Ensemble
    probs = mixed_problems(5, n=60)
    with Ensemble([(H0, H1, dt, c.shape[1]) for H0, H1, dt, c in probs], "fp64") as ens:
        ens.set_samples([c for *_, c in probs])
        before = ens.run()
        g = ens.tune()
        assert g in (1.0, 2.0, 4.0, 8.0, 16.0, 32.0, 64.0)
        after = ens.run()
        assert ens.last_ms > 0
    for a, b in zip(before, after):
        assert relerr(a, b) < 1e-12


def test_ensemble_workload_4096(built_lib):
    """The 4096-problem complex64 workload; 24 problems spot-checked."""
    from parament_gb300 import workloads
    from parament_gb300.ensemble import Ensemble
    probs = workloads.ensemble()
    with Ensemble([(H0, H1, dt, c.shape[1]) for H0, H1, dt, c in probs], "fp32") as ens:
        ens.set_samples([c for *_, c in probs])
        Us = ens.run()
    rng = np.random.default_rng(0)
    for i in rng.choice(len(probs), 24, replace=False):
        H0, H1, dt, carr = probs[i]
        ref = single(H0, H1, dt, carr, "fp32", "none")
        assert relerr(Us[i], ref) < 1e-5, (i, H0.shape[0], carr.shape)


def test_ensemble_rejects_bad_problems(built_lib):
    from parament_gb300.ensemble import Ensemble
    H = np.eye(65)
    with pytest.raises(ValueError, match="Invalid value"):
        Ensemble([(H, H[None], 0.1, 10)])
    H = np.eye(4)
    with pytest.raises(ValueError, match="Invalid value"):
        Ensemble([(H, np.stack([H] * 17), 0.1, 10)])
