"""Adjoint gradient (vector-Jacobian product of equiprop) on the GPU.

Checked against:
- torch autograd through torch.linalg.matrix_exp (CPU, complex128) for every
  quadrature mode with and without Magnus terms (chain rule through weights);
- the exact Frechet derivative of exp from the block matrix [[A, E], [0, A]]
  (scipy.linalg.expm, FP64);
- central finite differences (eps = 1e-4, FP64 equiprop) on 64 random entries
  of the d=32, K=6 fidelity workload;
- the complex128 gradient, for the complex64 context;
- the torch.autograd.Function binding;
- the stored-checkpoint sweep (manual Chebyshev order) against the recomputing
  one (automatic order) at the same order;
- the device memory of the d=32, K=6, 16384-step gradient: no per-step
  matrices.
Tolerances are relative to the largest gradient entry.
"""
import numpy as np
import pytest
import scipy.linalg

import oracle

pytestmark = pytest.mark.gpu

QUAD = {0: "none", 0x01000000: "midpoint", 0x02000000: "simpson"}


def herm(rng, d, norm):
    from parament_gb300.workloads import hermitian
    return hermitian(rng, d, norm)


def torch_reference_grad(H0, H1, carr, dt, magnus, mode, W):
    """d/du Re Tr(W^H U) with U = prod_j expm(-i h X_j) built in torch."""
    import torch

    K = H1.shape[0]
    stack = torch.tensor(oracle.build_stack(H0, H1, magnus))
    u = torch.tensor(np.real(carr), dtype=torch.float64, requires_grad=True)
    uc = u.to(torch.complex128)
    h = 2 * dt if (magnus or mode == oracle.SIMPSON) else dt
    P = oracle.num_steps(mode, magnus, carr.shape[1])
    f = 1j * h / 12
    Ut = torch.eye(H0.shape[0], dtype=torch.complex128)
    for j in range(P):
        if magnus or mode == oracle.SIMPSON:
            w = [(uc[k, 2 * j] + 4 * uc[k, 2 * j + 1] + uc[k, 2 * j + 2]) / 6 for k in range(K)]
        elif mode == oracle.MIDPOINT:
            w = [0.5 * (uc[k, j] + uc[k, j + 1]) for k in range(K)]
        else:
            w = [uc[k, j] for k in range(K)]
        if magnus:
            w += [f * (uc[k, 2 * j + 2] - uc[k, 2 * j]) for k in range(K)]
            for i in range(1, K):
                for jj in range(i):
                    w.append(f * (uc[jj, 2 * j] * uc[i, 2 * j + 2] - uc[jj, 2 * j + 2] * uc[i, 2 * j]))
        X = stack[0] + sum(wm * stack[1 + m] for m, wm in enumerate(w))
        Ut = torch.linalg.matrix_exp(-1j * h * X) @ Ut
    val = torch.real(torch.trace(torch.tensor(W).conj().T @ Ut))
    val.backward()
    return u.grad.numpy()


@pytest.mark.parametrize("magnus,mode", [(False, oracle.NONE), (False, oracle.MIDPOINT), (False, oracle.SIMPSON),
                                         (True, oracle.SIMPSON)])
def test_vjp_matches_torch_autograd(built_lib, magnus, mode):
    import parament_gb300 as parament
    rng = np.random.default_rng(7 + mode % 5 + magnus)
    d, K, pts, dt = 4, 3, 13, 0.05
    H0 = herm(rng, d, 2.0)
    H1 = np.stack([herm(rng, d, 1.0) for _ in range(K)])
    carr = rng.standard_normal((K, pts))
    W = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    with parament.Parament("fp64") as ctx:
        ctx.set_hamiltonian(H0, *H1, use_magnus=magnus, quadrature_mode=QUAD[mode])
        g = ctx.vjp(dt, W, *carr)
    ref = torch_reference_grad(H0, H1, carr, dt, magnus, mode, W)
    assert np.abs(g - ref).max() <= 1e-9 * np.abs(ref).max()


def test_vjp_matches_block_matrix_frechet(built_lib):
    import parament_gb300 as parament
    rng = np.random.default_rng(11)
    d, K, P, dt = 6, 2, 5, 0.03
    H0 = herm(rng, d, 3.0)
    H1 = np.stack([herm(rng, d, 1.0) for _ in range(K)])
    carr = rng.standard_normal((K, P))
    W = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    Us = [scipy.linalg.expm(-1j * dt * (H0 + sum(carr[k, j] * H1[k] for k in range(K)))) for j in range(P)]
    ref = np.zeros((K, P))
    for j in range(P):
        A = -1j * dt * (H0 + sum(carr[k, j] * H1[k] for k in range(K)))
        Lj = np.eye(d, dtype=complex)
        for i in range(j + 1, P):
            Lj = Us[i] @ Lj
        Rj = np.eye(d, dtype=complex)
        for i in range(j):
            Rj = Us[i] @ Rj
        for k in range(K):
            big = np.zeros((2 * d, 2 * d), complex)
            big[:d, :d] = A
            big[d:, d:] = A
            big[:d, d:] = -1j * dt * H1[k]
            dU = scipy.linalg.expm(big)[:d, d:]
            ref[k, j] = np.real(np.trace(W.conj().T @ Lj @ dU @ Rj))
    with parament.Parament("fp64") as ctx:
        ctx.set_hamiltonian(H0, *H1)
        g = ctx.vjp(dt, W, *carr)
    assert np.abs(g - ref).max() <= 1e-10 * np.abs(ref).max()


def _fidelity(ctx, dt, Ut, carr):
    U = ctx.equiprop(dt, *carr)
    d = U.shape[0]
    return 1.0 - abs(np.trace(Ut.conj().T @ U)) ** 2 / d ** 2


def test_fidelity_gradient_d32_central_differences(built_lib):
    """d=32, K=6, 16384 steps: adjoint vs FP64 central differences on 64 entries."""
    import parament_gb300 as parament
    from parament_gb300 import workloads
    w = workloads.adjoint_d32()
    Ut = workloads.haar_unitary(32, seed=1)
    carr = w["carr"].real
    rng = np.random.default_rng(3)
    picks = [(int(rng.integers(0, 6)), int(rng.integers(0, carr.shape[1]))) for _ in range(64)]
    with parament.Parament("fp64") as ctx:
        ctx.set_hamiltonian(w["H0"], *w["H1"])
        loss, g64 = ctx.fidelity_gradient(w["dt"], Ut, *carr)
        eps = 1e-4
        fd = []
        for k, i in picks:
            cp, cm = carr.copy(), carr.copy()
            cp[k, i] += eps
            cm[k, i] -= eps
            fd.append((_fidelity(ctx, w["dt"], Ut, cp) - _fidelity(ctx, w["dt"], Ut, cm)) / (2 * eps))
    fd = np.array(fd)
    adj = np.array([g64[k, i] for k, i in picks])
    scale = np.abs(g64).max()
    assert np.abs(adj - fd).max() <= 1e-6 * scale, (np.abs(adj - fd).max(), scale)
    with parament.Parament("fp32") as ctx:
        ctx.set_hamiltonian(w["H0"], *w["H1"])
        loss32, g32 = ctx.fidelity_gradient(w["dt"], Ut, *carr)
    assert abs(loss32 - loss) < 1e-3
    assert np.linalg.norm(g32 - g64) <= 1e-3 * np.linalg.norm(g64)


def test_autograd_function_matches_vjp(built_lib):
    import torch

    import parament_gb300 as parament
    from parament_gb300 import autograd, workloads
    w = workloads.plain_d16(steps=300)
    Ut = workloads.haar_unitary(16, seed=1)
    with parament.Parament("fp64") as ctx:
        ctx.set_hamiltonian(w["H0"], *w["H1"])
        u = torch.tensor(w["carr"].real, dtype=torch.float64, device="cuda", requires_grad=True)
        U = autograd.propagate(ctx, w["dt"], u)
        loss = autograd.fidelity_loss(U, torch.tensor(Ut, device="cuda"))
        loss.backward()
        l2, g2 = ctx.fidelity_gradient(w["dt"], Ut, *w["carr"].real)
    assert abs(loss.item() - l2) < 1e-12
    assert np.abs(u.grad.cpu().numpy() - g2).max() <= 1e-9 * np.abs(g2).max()


def test_vjp_errors(built_lib):
    import parament_gb300 as parament
    with parament.Parament("fp64") as ctx:
        with pytest.raises(RuntimeError, match="No hamiltonian set"):
            ctx.vjp(0.1, np.eye(2), np.zeros(3))
        ctx.set_hamiltonian(np.eye(49), np.eye(49))
        with pytest.raises(ValueError, match="Invalid value"):
            ctx.vjp(0.01, np.eye(49), np.zeros(3))


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 1e-4)])
def test_recomputed_and_stored_sweeps_agree(built_lib, precision, tol):
    """The automatic order recomputes R_j = U_j^H R_(j+1) backward from the
    chunk-end checkpoint; a manual order (here the same order) stores every
    R_j of the forward sweep.  Both are the derivative of the same computed
    propagator."""
    import parament_gb300 as parament
    from parament_gb300 import workloads
    w = workloads.problem(12, 3, 2001, 1e-3, norm0=5.0, seed=4, magnus=True, quadrature=oracle.SIMPSON)
    rng = np.random.default_rng(2)
    W = rng.standard_normal((12, 12)) + 1j * rng.standard_normal((12, 12))
    with parament.Parament(precision) as ctx:
        ctx.set_hamiltonian(w["H0"], *w["H1"], use_magnus=True, quadrature_mode="simpson")
        g_rec = ctx.vjp(w["dt"], W, *w["carr"].real)
        M = ctx.last_iteration_cycles
        ctx.set_iteration_cycles_manually(M)
        g_sto = ctx.vjp(w["dt"], W, *w["carr"].real)
    assert np.abs(g_rec - g_sto).max() <= tol * np.abs(g_sto).max()


def test_gradient_memory_has_no_per_step_matrices(built_lib):
    """d=32, K=6, 16384 steps, complex64: the context's device memory after a
    gradient is the samples, the gradient, the per-step traces and a few
    matrices per chunk (about one chunk per SM; the chunk boundaries are the
    checkpoints) -- far below one d x d matrix per step."""
    import torch

    import parament_gb300 as parament
    from parament_gb300 import workloads
    w = workloads.adjoint_d32()
    d, K, P, sc = 32, 6, w["P"], 8
    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    free0 = torch.cuda.mem_get_info()[0]
    with parament.Parament("fp32") as ctx:
        ctx.set_hamiltonian(w["H0"], *w["H1"])
        g = ctx.vjp(w["dt"], np.eye(d), *w["carr"].real)
        held = ctx.device_memory_bytes
        torch.cuda.synchronize()
        used = free0 - torch.cuda.mem_get_info()[0]
    per_step_mats = P * d * d * sc
    io = K * P * sc + K * P * 4 + d * d * sc          # samples, gradient, seed
    # traces (Ke = K here), the Hamiltonian stack, and five matrices per chunk
    # (chunk product, prefix, suffix, two scan buffers) for at most eight
    # resident CTAs per SM
    budget = io + P * K * sc + (1 + K) * d * d * sc + 5 * 8 * nsm * d * d * sc
    print(f"\ngradient d=32 P=16384: context holds {held / 2**20:.2f} MiB (budget {budget / 2**20:.2f} MiB, "
          f"one matrix per step would be {per_step_mats / 2**20:.0f} MiB); driver reports {used / 2**20:.1f} MiB")
    assert np.isfinite(g).all()
    assert held <= budget
    assert used < per_step_mats / 4
