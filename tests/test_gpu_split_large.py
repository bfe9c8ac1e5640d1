"""The split-precision complex64 form for d > 64 (split_large.cu).

Its parity bar is the FP64 oracle on the complex64-rounded inputs: relative
Frobenius error <= 1e-6, as for the d <= 64 split form.  Cases: d = 96 (FP32
SIMT GEMMs) with Magnus and Simpson, d = 192, 256 and 384 (the exact sliced
tensor-core GEMM) in the other quadratures, uneven chunk lengths, d = 1024
(sixteen K blocks) against the complex128 path, and the d=512, K=8 large dense
workload -- a prefix against the oracle and all 8192 steps against the GPU's
complex128 path (itself held to 1e-10 of the oracle).
"""
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

NPROC = os.cpu_count() or 1
QUAD = {0: "none", 0x01000000: "midpoint", 0x02000000: "simpson"}


def relerr(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


def c64(x):
    return np.asarray(x).astype(np.complex64).astype(np.complex128)


def run(H0, H1, carr, dt, magnus=False, mode=0, precision="fp32", split=True):
    import parament_gb300 as parament
    with parament.Parament(precision) as ctx:
        if split:
            ctx.set_precision_mode("split")
        ctx.set_hamiltonian(H0, *H1, use_magnus=magnus, quadrature_mode=QUAD[mode])
        U = ctx.equiprop(dt, *carr)
        return U.astype(np.complex128), ctx.last_iteration_cycles


@pytest.mark.parametrize("d,K,n,magnus,mode", [(96, 2, 101, True, oracle.SIMPSON), (256, 3, 211, False, oracle.NONE),
                                               (384, 2, 77, False, oracle.MIDPOINT), (192, 2, 301, True, oracle.SIMPSON)])
def test_split_large_against_oracle(built_lib, d, K, n, magnus, mode):
    from parament_gb300.workloads import hermitian, sinusoid_controls
    rng = np.random.default_rng(d)
    H0 = c64(hermitian(rng, d, 15.0))
    H1 = c64(np.stack([hermitian(rng, d, 1.0) for _ in range(K)]))
    carr = c64(sinusoid_controls(rng, K, n, 1e-3))
    U, M = run(H0, H1, list(carr), 1e-3, magnus, mode)
    Uo = oracle.equiprop(H0, H1, carr, 1e-3, magnus=magnus, mode=mode, nthreads=NPROC)[0]
    e = relerr(U, Uo)
    print(f"\nsplit d={d} K={K} {n} samples (M={M}): rel err vs FP64 oracle {e:.3e}")
    assert e < 1e-6


@pytest.fixture(scope="module")
def dense512():
    from parament_gb300 import workloads
    w = workloads.large_dense(d=512, K=8, steps=8192)
    for k in ("H0", "H1", "carr"):
        w[k] = c64(w[k])
    return w


def test_split_large_dense_prefix_against_oracle(built_lib, dense512):
    w = dense512
    carr = w["carr"][:, :48]
    U, M = run(w["H0"], w["H1"], list(carr), w["dt"])
    Uo = oracle.equiprop(w["H0"], w["H1"], carr, w["dt"], nthreads=NPROC)[0]
    e = relerr(U, Uo)
    print(f"\nsplit d=512 K=8 first 48 steps (M={M}): rel err vs FP64 oracle {e:.3e}")
    assert e < 1e-6


def test_split_large_dense_full_length(built_lib, dense512):
    """All 8192 steps: the split complex64 form against the complex128 path."""
    w = dense512
    U, M = run(w["H0"], w["H1"], list(w["carr"]), w["dt"])
    U128, _ = run(w["H0"], w["H1"], list(w["carr"]), w["dt"], precision="fp64", split=False)
    e = relerr(U, U128)
    print(f"\nsplit d=512 K=8 8192 steps (M={M}): rel err vs complex128 {e:.3e}")
    assert e < 1e-6


def test_split_large_d1024_against_complex128(built_lib):
    """d=1024 (sixteen K blocks of the exact sliced GEMM), 64 steps, against
    the complex128 path on the same complex64-rounded inputs."""
    from parament_gb300 import workloads
    w = workloads.large_dense(d=1024, K=4, steps=64)
    H0, H1, carr = c64(w["H0"]), c64(w["H1"]), c64(w["carr"])
    U, M = run(H0, H1, list(carr), w["dt"])
    U128, _ = run(H0, H1, list(carr), w["dt"], precision="fp64", split=False)
    e = relerr(U, U128)
    print(f"\nsplit d=1024 K=4 64 steps (M={M}): rel err vs complex128 {e:.3e}")
    assert e < 1e-6
