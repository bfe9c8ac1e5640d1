"""Seeded synthetic problems of the benchmark shapes.

Every generator returns a dict with H0 (d, d), H1 (K, d, d), carr (K, n)
complex128 arrays plus dt, magnus, quadrature and the number of steps P.

Common recipe (drawn in this order from ``numpy.random.default_rng(seed)``):
Hermitian matrices (A + A^H)/2 with A complex standard normal, rescaled to the
stated spectral norm -- H0 first, then H_1..H_K; then the control amplitudes
u_k[j] = sin(2 pi f_k j dt + phi_k) + 0.1 N(0, 1) with f_k ~ U[1, 20] and
phi_k ~ U[0, 2 pi).  Amplitudes are real numbers stored as complex.
"""
from __future__ import annotations

import numpy as np

NONE, MIDPOINT, SIMPSON = 0x00000000, 0x01000000, 0x02000000


def hermitian(rng, d: int, norm: float) -> np.ndarray:
    a = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    h = (a + a.conj().T) / 2
    return h * (norm / np.linalg.norm(h, 2))


def sinusoid_controls(rng, K: int, n: int, dt: float) -> np.ndarray:
    f = rng.uniform(1.0, 20.0, K)
    phi = rng.uniform(0.0, 2 * np.pi, K)
    t = np.arange(n) * dt
    u = np.sin(2 * np.pi * f[:, None] * t[None, :] + phi[:, None]) + 0.1 * rng.standard_normal((K, n))
    return u.astype(np.complex128)


def problem(d, K, n, dt, norm0=1.0, norm1=1.0, seed=0, magnus=False, quadrature=NONE):
    rng = np.random.default_rng(seed)
    H0 = hermitian(rng, d, norm0)
    H1 = np.stack([hermitian(rng, d, norm1) for _ in range(K)])
    carr = sinusoid_controls(rng, K, n, dt)
    if magnus or quadrature == SIMPSON:
        P = (n - 1) // 2
    elif quadrature == MIDPOINT:
        P = n - 1
    else:
        P = n
    return dict(H0=H0, H1=H1, carr=carr, dt=dt, magnus=magnus, quadrature=quadrature, P=P)


def plain_d16(steps=4096, seed=0):
    """Plain equiprop: d=16, K=2, NONE quadrature, dt=1e-3, norms 1."""
    return problem(16, 2, steps, 1e-3, seed=seed)


def magnus_d64(steps=65536, seed=0):
    """Precision workload: d=64, K=4, Magnus with Simpson (2 steps + 1 samples),
    ||H0|| = 10, ||H_k|| = 1, dt = 1e-3."""
    return problem(64, 4, 2 * steps + 1, 1e-3, norm0=10.0, norm1=1.0, seed=seed, magnus=True, quadrature=SIMPSON)


def adjoint_d32(steps=16384, seed=0):
    """Gradient workload: d=32, K=6, NONE quadrature, dt=1e-3, norms 1."""
    return problem(32, 6, steps, 1e-3, seed=seed)


def large_dense(d=512, K=8, steps=8192, norm0=20.0, seed=2, dt=1e-3):
    """Large dense: smooth amplitudes, each the sum of 8 random Fourier modes."""
    rng = np.random.default_rng(seed)
    H0 = hermitian(rng, d, norm0)
    H1 = np.stack([hermitian(rng, d, 1.0) for _ in range(K)])
    t = np.arange(steps) * dt
    u = np.zeros((K, steps))
    for k in range(K):
        amp = rng.standard_normal(8) / np.sqrt(8)
        freq = rng.uniform(0.5, 10.0, 8)
        ph = rng.uniform(0, 2 * np.pi, 8)
        u[k] = (amp[:, None] * np.sin(2 * np.pi * freq[:, None] * t[None, :] + ph[:, None])).sum(0)
    return dict(H0=H0, H1=H1, carr=u.astype(np.complex128), dt=dt, magnus=False, quadrature=NONE, P=steps)


def haar_unitary(d: int, seed: int = 1) -> np.ndarray:
    """Haar-random unitary: QR of a complex Gaussian matrix with the phases of
    R's diagonal moved into Q."""
    rng = np.random.default_rng(seed)
    z = (rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))) / np.sqrt(2)
    q, r = np.linalg.qr(z)
    ph = np.diag(r) / np.abs(np.diag(r))
    return q * ph[None, :]


def ensemble(nprob=4096, seed=3, dt=1e-3):
    """Batched workload: nprob problems with d in {4, 8, 16, 32, 64}
    (probabilities .3/.3/.2/.15/.05), pts ~ U[256, 8192], K ~ U{1..4}.  Each
    problem: H0 random Hermitian of norm 1 plus delta * Z_total with
    delta ~ N(0, 0.05) and Z_total = sum_q Z_q over the log2(d) qubits
    (diagonal entries sum_q (1 - 2 bit_q(i))); H_k random Hermitian of norm 1;
    sinusoid-plus-noise controls.  Returns a list of (H0, H1, dt, carr)."""
    rng = np.random.default_rng(seed)
    dims = rng.choice([4, 8, 16, 32, 64], size=nprob, p=[0.3, 0.3, 0.2, 0.15, 0.05])
    out = []
    for d in dims:
        d = int(d)
        pts = int(rng.integers(256, 8193))
        K = int(rng.integers(1, 5))
        q = int(np.log2(d))
        z = np.array([sum(1 - 2 * ((i >> b) & 1) for b in range(q)) for i in range(d)], dtype=float)
        H0 = hermitian(rng, d, 1.0) + rng.normal(0.0, 0.05) * np.diag(z)
        H1 = np.stack([hermitian(rng, d, 1.0) for _ in range(K)])
        carr = sinusoid_controls(rng, K, pts, dt)
        out.append((H0, H1, dt, carr))
    return out
