"""The benchmark workloads at their full sizes against the CPU oracle.

Every propagator here is compared with the oracle (the FP64 C restatement of
the reference algorithm) run over all steps on every host core, not with
another GPU result:

  * d=64, K=4, Magnus with Simpson, 65536 steps (131073 samples per control):
    complex128 within 1e-10; the split complex64 form within 1e-6 of the FP64
    oracle on the complex64-rounded inputs; the plain complex64 scheme within
    1e-5 of the oracle's complex64-context arithmetic.
  * d=32, K=6, NONE, 16384 steps (the gradient workload's forward pass), in
    the same three forms.
  * 24 complex64 problems spread over the 4096-problem ensemble, within 1e-5.
  * d=512 at 8192 steps and d=1024 at 2048 steps (complex64, tensor-core
    products), where steps x d^2 = 2^31 (the reference passes that count to
    cuBLAS as an int, src/cuda/parament.cpp:590): unitarity and the
    composition of the two halves, plus an oracle check of a prefix.

The relative Frobenius error of each case is printed (pytest -s shows it).
"""
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

NPROC = os.cpu_count() or 1


def relerr(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


def c64(x):
    return np.asarray(x).astype(np.complex64).astype(np.complex128)


def propagate(w, precision, split=False, carr=None):
    import parament_gb300 as parament
    mode = {oracle.NONE: "none", oracle.MIDPOINT: "midpoint", oracle.SIMPSON: "simpson"}[w["quadrature"]]
    with parament.Parament(precision) as ctx:
        if split:
            ctx.set_precision_mode("split")
        ctx.set_hamiltonian(w["H0"], *w["H1"], use_magnus=w["magnus"], quadrature_mode=mode)
        U = ctx.equiprop(w["dt"], *(w["carr"] if carr is None else carr))
        return U.astype(np.complex128), ctx.last_iteration_cycles


def oracle_u(w, single=False):
    U, M, _, st = oracle.equiprop(w["H0"], w["H1"], w["carr"], w["dt"], magnus=w["magnus"], mode=w["quadrature"],
                                  single=single, nthreads=NPROC)
    assert st == 0
    return U, M


def rounded(w):
    w = dict(w)
    for k in ("H0", "H1", "carr"):
        w[k] = c64(w[k])
    return w


@pytest.fixture(scope="module")
def magnus_full():
    from parament_gb300 import workloads
    return rounded(workloads.magnus_d64())


@pytest.fixture(scope="module")
def magnus_oracle(magnus_full):
    return oracle_u(magnus_full)


def test_magnus_d64_full_complex128(built_lib, magnus_full, magnus_oracle):
    U, M = propagate(magnus_full, "fp64")
    Uo, Mo = magnus_oracle
    e = relerr(U, Uo)
    print(f"\nd=64 Magnus 65536 steps complex128: rel err vs oracle {e:.3e} (M={M})")
    assert M == Mo and e < 1e-10


def test_magnus_d64_full_split(built_lib, magnus_full, magnus_oracle):
    U, M = propagate(magnus_full, "fp32", split=True)
    e = relerr(U, magnus_oracle[0])
    print(f"\nd=64 Magnus 65536 steps split complex64: rel err vs FP64 oracle {e:.3e} (M={M})")
    assert e < 1e-6


def test_magnus_d64_full_plain_complex64(built_lib, magnus_full):
    U, M = propagate(magnus_full, "fp32")
    Uo, Mo = oracle_u(magnus_full, single=True)
    e = relerr(U, Uo)
    print(f"\nd=64 Magnus 65536 steps plain complex64: rel err vs oracle (complex64 context) {e:.3e} (M={M})")
    assert M == Mo and e < 1e-5


@pytest.fixture(scope="module")
def adjoint_full():
    from parament_gb300 import workloads
    return rounded(workloads.adjoint_d32())


def test_adjoint_forward_full(built_lib, adjoint_full):
    """The gradient workload's forward pass (d=32, K=6, 16384 steps) in the
    three forms."""
    Uo, Mo = oracle_u(adjoint_full)
    U, M = propagate(adjoint_full, "fp64")
    e128 = relerr(U, Uo)
    Us, _ = propagate(adjoint_full, "fp32", split=True)
    es = relerr(Us, Uo)
    Up, Mp = propagate(adjoint_full, "fp32")
    Uos, Mos = oracle_u(adjoint_full, single=True)
    ep = relerr(Up, Uos)
    print(f"\nd=32 K=6 16384 steps: complex128 {e128:.3e}, split complex64 {es:.3e}, "
          f"plain complex64 {ep:.3e} (vs oracle)")
    assert M == Mo and e128 < 1e-10
    assert es < 1e-6
    assert Mp == Mos and ep < 1e-5


def float32_scheme(H0, H1, carr, dt, M, hnorm):
    """The plain scheme (NONE quadrature) restated in complex64 arithmetic with
    numpy: the Clenshaw recurrence of every step in FP32 and an FP64 product.
    Its distance from the oracle is the rounding that the complex64 scheme
    itself carries (the same for any FP32 implementation of it)."""
    d = H0.shape[0]
    J = oracle.bessel_coeffs(M, dt * hnorm).astype(np.complex64)
    s = np.float32(2.0 / hnorm)
    I = np.eye(d, dtype=np.complex64)
    H0f, H1f, cf = H0.astype(np.complex64), H1.astype(np.complex64), carr.astype(np.complex64)
    U = np.eye(d)
    for j in range(cf.shape[1]):
        X = (H0f + np.tensordot(cf[:, j], H1f, axes=1)).astype(np.complex64)
        b2, b1 = J[M] * I, (s * J[M]) * X + J[M - 1] * I
        for k in range(M - 2, -1, -1):
            v = (s * (b1 @ X)).astype(np.complex64) + np.float32(-2 if k == 0 else -1) * b2 + J[k] * I
            b2, b1 = b1, v.astype(np.complex64)
        U = b1.astype(np.complex128) @ U
    return U


def test_ensemble_spot_check_against_oracle(built_lib):
    """24 problems spread over the 4096-problem complex64 ensemble, against the
    oracle's complex64-context arithmetic: within 1e-5, or within twice the
    rounding of the complex64 scheme itself where that is larger (a few long,
    small-d problems: the FP32 Clenshaw rounding repeats at every step)."""
    from parament_gb300 import workloads
    from parament_gb300.ensemble import Ensemble
    probs = workloads.ensemble()
    with Ensemble([(H0, H1, dt, c.shape[1]) for H0, H1, dt, c in probs], "fp32") as ens:
        ens.set_samples([c for *_, c in probs])
        Us = ens.run()
    picks = np.linspace(0, len(probs) - 1, 24).astype(int)
    worst = 0.0
    for i in picks:
        H0, H1, dt, carr = probs[i]
        H0, H1, carr = c64(H0), c64(H1), c64(carr)
        Uo, M, hn, st = oracle.equiprop(H0, H1, carr, dt, single=True, nthreads=NPROC)
        assert st == 0
        e = relerr(Us[i].astype(np.complex128), Uo)
        worst = max(worst, e)
        if e >= 1e-5:
            e32 = relerr(float32_scheme(H0, H1, carr, dt, M, hn), Uo)
            print(f"\nproblem {i} (d={H0.shape[0]}, {carr.shape[1]} steps): {e:.3e}; the complex64 scheme "
                  f"in numpy FP32: {e32:.3e}")
            assert e < 2 * e32, (int(i), H0.shape[0], carr.shape, e, e32)
    print(f"\nensemble, 24 of 4096 problems: worst rel err vs oracle {worst:.3e}")


def halves(w):
    """The workload's samples split into the first and second half of its steps."""
    n = w["carr"].shape[1]
    return w["carr"][:, : n // 2], w["carr"][:, n // 2:]


@pytest.mark.parametrize("d,K,steps,precision,tol", [(512, 8, 8192, "fp32", 1e-4), (1024, 4, 2048, "fp32", 1e-4)])
def test_large_dense_index_range(built_lib, d, K, steps, precision, tol):
    """steps x d^2 = 2^31: the full workload composes from its two halves and
    stays unitary; its first steps match the oracle."""
    from parament_gb300 import workloads
    w = workloads.large_dense(d=d, K=K, steps=steps)
    if precision == "fp32":
        w = rounded(w)
    assert steps * d * d == 2 ** 31
    U, _ = propagate(w, precision)
    a, b = halves(w)
    Ua, _ = propagate(w, precision, carr=a)
    Ub, _ = propagate(w, precision, carr=b)
    eu = float(np.linalg.norm(U.conj().T @ U - np.eye(d)) / np.sqrt(d))
    ec = relerr(Ub @ Ua, U)
    print(f"\nd={d} {precision} {steps} steps: unitarity {eu:.3e}, halves composed {ec:.3e}")
    assert ec < tol and eu < 10 * tol
    nprefix = 3 if d == 1024 else 12
    wp = dict(w, carr=w["carr"][:, :nprefix])
    Up, M = propagate(wp, precision)
    Uo, Mo = oracle_u(wp, single=(precision == "fp32"))
    ep = relerr(Up, Uo)
    print(f"d={d} {precision} first {nprefix} steps: rel err vs oracle {ep:.3e}")
    assert M == Mo and ep < (1e-5 if precision == "fp32" else 1e-10)
