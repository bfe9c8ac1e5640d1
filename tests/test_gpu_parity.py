"""Parity of the CUDA equiprop path with the CPU oracle, through the C-ABI.

Tolerances (relative Frobenius error against the FP64 oracle):
complex128 contexts 1e-10, complex64 contexts 1e-5.  Full-size workloads are
checked through size-independent properties (unitarity, composition of two
halves, agreement of the two context precisions).
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
from conftest import ROOT

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-10, "fp32": 1e-5}
QUAD = {0: "none", 0x01000000: "midpoint", 0x02000000: "simpson"}


def relerr(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


def run(H0, H1, carr, dt, magnus=False, mode=0, precision="fp64", cycles=None):
    import parament_gb300 as parament
    with parament.Parament(precision) as ctx:
        ctx.set_hamiltonian(H0, *H1, use_magnus=magnus, quadrature_mode=QUAD[mode])
        if cycles:
            ctx.set_iteration_cycles_manually(cycles)
        U = ctx.equiprop(dt, *carr)
        return U.astype(np.complex128), ctx.last_iteration_cycles


def test_golden_cases(built_lib, golden_cases):
    bad = []
    for c in golden_cases:
        U, M = run(c["H0"], c["H1"], [r for r in c["carr"]], c["dt"], c["magnus"], c["mode"], c["precision"])
        e = relerr(U, c["U"])
        if e > TOL[c["precision"]] or M != c["M"]:
            bad.append((c["name"], e, M, c["M"]))
    assert not bad, bad


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_plain_d16_full_size(built_lib, precision):
    from parament_gb300 import workloads
    w = workloads.plain_d16()
    U, M = run(w["H0"], w["H1"], list(w["carr"]), w["dt"], precision=precision)
    Uo, Mo, _, st = oracle.equiprop(w["H0"], w["H1"], w["carr"], w["dt"], single=(precision == "fp32"),
                                    nthreads=os.cpu_count())
    assert st == 0 and M == Mo
    assert relerr(U, Uo) < TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_magnus_d64_reduced(built_lib, precision):
    from parament_gb300 import workloads
    w = workloads.magnus_d64(steps=384)
    U, M = run(w["H0"], w["H1"], list(w["carr"]), w["dt"], True, oracle.SIMPSON, precision)
    Uo, Mo, _, st = oracle.equiprop(w["H0"], w["H1"], w["carr"], w["dt"], magnus=True, mode=oracle.SIMPSON,
                                    single=(precision == "fp32"), nthreads=os.cpu_count())
    assert st == 0 and M == Mo
    assert relerr(U, Uo) < TOL[precision]


def test_magnus_d64_full_size_properties(built_lib):
    """65536 steps: unitarity, and the product of the two halves equals the whole."""
    from parament_gb300 import workloads
    w = workloads.magnus_d64()
    carr = w["carr"]
    U, _ = run(w["H0"], w["H1"], list(carr), w["dt"], True, oracle.SIMPSON, "fp64")
    d = U.shape[0]
    assert np.linalg.norm(U.conj().T @ U - np.eye(d)) < 1e-9
    half = (carr.shape[1] - 1) // 2  # Simpson pairs share the boundary sample
    Ua, _ = run(w["H0"], w["H1"], list(carr[:, :half + 1]), w["dt"], True, oracle.SIMPSON, "fp64")
    Ub, _ = run(w["H0"], w["H1"], list(carr[:, half:]), w["dt"], True, oracle.SIMPSON, "fp64")
    assert relerr(Ub @ Ua, U) < 1e-10
    U32, _ = run(w["H0"], w["H1"], list(carr), w["dt"], True, oracle.SIMPSON, "fp32")
    assert relerr(U32, U) < 1e-3


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("d", [65, 80, 130])
def test_large_dimension_path(built_lib, precision, d):
    rng = np.random.default_rng(d)
    from parament_gb300.workloads import hermitian
    H0 = hermitian(rng, d, 5.0)
    H1 = np.stack([hermitian(rng, d, 1.0) for _ in range(2)])
    carr = rng.standard_normal((2, 9))
    U, M = run(H0, H1, list(carr), 2e-3, False, oracle.MIDPOINT, precision)
    if precision == "fp32":
        H0, H1, carr = (x.astype(np.complex64).astype(np.complex128) for x in (H0, H1, carr))
    Uo, Mo, _, _ = oracle.equiprop(H0, H1, carr, 2e-3, mode=oracle.MIDPOINT, single=(precision == "fp32"),
                                   nthreads=os.cpu_count())
    assert M == Mo
    assert relerr(U, Uo) < TOL[precision]


_CLUSTER_CASE = """
import sys, numpy as np, parament_gb300 as p
from parament_gb300.workloads import hermitian, sinusoid_controls
d, magnus, n, prec = int(sys.argv[2]), sys.argv[3] == "1", int(sys.argv[4]), sys.argv[5]
rng = np.random.default_rng(d + n)
H0 = hermitian(rng, d, 8.0)
H1 = np.stack([hermitian(rng, d, 1.0) for _ in range(3)])
carr = sinusoid_controls(rng, 3, n, 1e-3)
with p.Parament(prec) as ctx:
    ctx.set_hamiltonian(H0, *H1, use_magnus=magnus, quadrature_mode="simpson" if magnus else "none")
    U = ctx.equiprop(1e-3, *carr)
    np.save(sys.argv[1], U)
    print("BYTES", ctx.device_memory_bytes, "M", ctx.last_iteration_cycles)
"""


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("d,magnus,n", [(96, True, 801), (128, False, 1500), (72, False, 37)])
def test_cluster_resident_path(built_lib, precision, d, magnus, n):
    """64 < d <= 128 when the batched path's buffers cannot be had (the fourth
    device allocation of the child process -- the first batch buffer -- is
    made to fail): clusters of four CTAs with the step resident in their
    shared memory (complex64 up to d = 128, complex128 up to d = 96; complex128
    at d = 128 then reports the allocation failure), against the oracle."""
    import tempfile
    if precision == "fp64" and d > 96:
        pytest.skip("complex128 at d = 128 has no cluster-resident form")
    with tempfile.TemporaryDirectory() as tmp:
        f = os.path.join(tmp, "U.npy")
        env = dict(os.environ, PARAMENT_FAIL_ALLOC_AFTER="3")
        r = subprocess.run([sys.executable, "-c", _CLUSTER_CASE, f, str(d), "1" if magnus else "0", str(n),
                            precision], cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stdout + r.stderr
        U = np.load(f).astype(np.complex128)
    held = int(r.stdout.split("BYTES")[1].split()[0])
    assert held < 100 << 20, held  # no batch buffers
    rng = np.random.default_rng(d + n)
    from parament_gb300.workloads import hermitian, sinusoid_controls
    H0 = hermitian(rng, d, 8.0)
    H1 = np.stack([hermitian(rng, d, 1.0) for _ in range(3)])
    carr = sinusoid_controls(rng, 3, n, 1e-3)
    mode = oracle.SIMPSON if magnus else oracle.NONE
    if precision == "fp32":
        H0, H1, carr = (x.astype(np.complex64).astype(np.complex128) for x in (H0, H1, carr))
    Uo, Mo, _, _ = oracle.equiprop(H0, H1, carr, 1e-3, magnus=magnus, mode=mode, single=(precision == "fp32"),
                                   nthreads=os.cpu_count())
    assert relerr(U, Uo) < TOL[precision]


@pytest.mark.parametrize("cycles", [1, 3, 5, 9, 21])
def test_manual_cycles(built_lib, cycles):
    rng = np.random.default_rng(cycles)
    from parament_gb300.workloads import hermitian
    H0, H1 = hermitian(rng, 7, 1.0), hermitian(rng, 7, 1.0)[None]
    carr = rng.standard_normal((1, 11))
    U, M = run(H0, H1, list(carr), 0.01, cycles=cycles)
    Uo, Mo, _, _ = oracle.equiprop(H0, H1, carr, 0.01, M=cycles)
    assert M == cycles
    assert relerr(U, Uo) < 1e-10


def test_cycle_control_errors(built_lib):
    import parament_gb300 as parament
    with parament.Parament("fp64") as ctx:
        with pytest.raises(ValueError, match="Invalid value"):
            ctx.set_iteration_cycles_manually(4)
        with pytest.raises(ValueError, match="Invalid value"):
            ctx.set_iteration_cycles_manually(0)
        ctx.set_hamiltonian(np.diag([1.0, -1.0]), np.eye(2))
        # Hnorm = 2, so dt = 7 gives Hnorm*dt = 14, past the fp64 table (12.7584).
        with pytest.raises(RuntimeError, match="Timestep too large"):
            ctx.equiprop(7.0, np.zeros(3))
        assert ctx.peek_at_last_error() == 70
        ctx.set_iteration_cycles_manually(41)
        U = ctx.equiprop(7.0, np.zeros(3))  # a manual order bypasses the table
        want = np.diag(np.exp(-1j * 21.0 * np.array([1.0, -1.0])))
        assert np.allclose(U, want, atol=1e-9)
        ctx.automatic_iteration_cycles()
        with pytest.raises(RuntimeError, match="Timestep too large"):
            ctx.equiprop(7.0, np.zeros(3))


def test_no_steps_after_quadrature_is_invalid(built_lib):
    import parament_gb300 as parament
    with parament.Parament("fp64") as ctx:
        ctx.set_hamiltonian(np.eye(2), np.eye(2), quadrature_mode="simpson")
        with pytest.raises(ValueError, match="Invalid value"):
            ctx.equiprop(0.1, np.zeros(2))
        ctx.set_hamiltonian(np.eye(2), np.eye(2), quadrature_mode="midpoint")
        with pytest.raises(ValueError, match="Invalid value"):
            ctx.equiprop(0.1, np.zeros(1))


def test_zero_hamiltonian_gives_identity(built_lib):
    U, _ = run(np.zeros((3, 3)), [np.zeros((3, 3))], [np.ones(5)], 0.1)
    assert np.array_equal(U, np.eye(3))


def test_context_reuse_across_modes_and_lengths(built_lib):
    import parament_gb300 as parament
    rng = np.random.default_rng(9)
    from parament_gb300.workloads import hermitian
    H0 = hermitian(rng, 6, 2.0)
    H1 = np.stack([hermitian(rng, 6, 1.0) for _ in range(3)])
    with parament.Parament("fp64") as ctx:
        for mode, magnus, pts in [("none", False, 40), ("simpson", True, 9), ("midpoint", False, 300),
                                  ("simpson", False, 41), ("none", False, 3)]:
            ctx.set_hamiltonian(H0, *H1, use_magnus=magnus, quadrature_mode=mode)
            carr = rng.standard_normal((3, pts))
            U = ctx.equiprop(0.01, *carr)
            m = {"none": oracle.NONE, "midpoint": oracle.MIDPOINT, "simpson": oracle.SIMPSON}[mode]
            Uo = oracle.equiprop(H0, H1, carr, 0.01, magnus=magnus, mode=m)[0]
            assert relerr(U, Uo) < 1e-10, (mode, magnus, pts)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_device_entry_point_matches_host(built_lib, precision):
    import torch

    import parament_gb300 as parament
    from parament_gb300 import workloads
    w = workloads.plain_d16(steps=1000)
    with parament.Parament(precision) as ctx:
        ctx.set_hamiltonian(w["H0"], *w["H1"])
        Uh = ctx.equiprop(w["dt"], *w["carr"])
        ct = torch.complex128 if precision == "fp64" else torch.complex64
        carr = torch.tensor(w["carr"], dtype=ct, device="cuda")
        Ud = ctx.equiprop_device(w["dt"], carr)
        ctx.synchronize()  # no bounded wait gave up
        torch.cuda.synchronize()
        assert np.array_equal(Ud.cpu().numpy(), Uh)


def test_device_allocation_failure_is_reported(built_lib):
    """Host-side fault injection: the third device allocation fails."""
    code = ("import numpy as np, parament_gb300 as p\n"
            "c = p.Parament('fp64')\n"
            "c.set_hamiltonian(np.eye(4), np.eye(4))\n"
            "try:\n"
            "    c.equiprop(0.1, np.zeros(50))\n"
            "except MemoryError as e:\n"
            "    print('MEMERR', e)\n")
    env = dict(os.environ, PARAMENT_FAIL_ALLOC_AFTER="2")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert "MEMERR Error code 20" in r.stdout, r.stdout + r.stderr


@pytest.mark.parametrize("d,P", [(256, 6), (384, 3)])
def test_tensor_core_large_dimension(built_lib, d, P):
    """complex64, d >= 256: the tcgen05 3xTF32 GEMM path against the oracle."""
    rng = np.random.default_rng(d + P)
    from parament_gb300.workloads import hermitian
    H0 = hermitian(rng, d, 5.0)
    H1 = np.stack([hermitian(rng, d, 1.0) for _ in range(2)])
    carr = rng.standard_normal((2, P))
    U, M = run(H0, H1, list(carr), 2e-3, precision="fp32")
    H0, H1, carr = (x.astype(np.complex64).astype(np.complex128) for x in (H0, H1, carr))
    Uo, Mo, _, _ = oracle.equiprop(H0, H1, carr, 2e-3, single=True, nthreads=os.cpu_count())
    assert M == Mo
    assert relerr(U, Uo) < TOL["fp32"]


@pytest.mark.parametrize("d,K,steps", [(512, 8, 5), (1024, 4, 2)])
def test_tensor_core_matches_simt_gemm(built_lib, d, K, steps):
    """d=512 and d=1024: the tcgen05 path and the SIMT GEMM path (tensor cores
    disabled through PARAMENT_DISABLE_TENSOR_CORES in a child process) agree."""
    code = ("import sys, numpy as np, parament_gb300 as p\n"
            "from parament_gb300 import workloads\n"
            f"w = workloads.large_dense(d={d}, K={K}, steps={steps})\n"
            "c = p.Parament('fp32'); c.set_hamiltonian(w['H0'], *w['H1'])\n"
            "np.save(sys.argv[1], c.equiprop(w['dt'], *w['carr']))\n")
    import tempfile
    outs = []
    with tempfile.TemporaryDirectory() as tmp:
        for tag, env in (("tc", {}), ("simt", {"PARAMENT_DISABLE_TENSOR_CORES": "1"})):
            f = os.path.join(tmp, tag + ".npy")
            r = subprocess.run([sys.executable, "-c", code, f], cwd=ROOT, env=dict(os.environ, **env),
                               capture_output=True, text=True, timeout=600)
            assert r.returncode == 0, r.stderr
            outs.append(np.load(f).astype(np.complex128))
    assert relerr(outs[0], outs[1]) < 1e-5


def test_tensor_core_magnus_simpson(built_lib):
    """complex64, d=256, Magnus with Simpson: the commutators [H0, H_k] and
    [H_j, H_k] are single products (one batch item, unbatched operands) on the
    tcgen05 GEMM, then the Clenshaw batch and the tree."""
    rng = np.random.default_rng(256)
    from parament_gb300.workloads import hermitian
    H0 = hermitian(rng, 256, 5.0)
    H1 = np.stack([hermitian(rng, 256, 1.0) for _ in range(2)])
    carr = rng.standard_normal((2, 2 * 4 + 1))
    U, M = run(H0, H1, list(carr), 1e-3, magnus=True, mode=oracle.SIMPSON, precision="fp32")
    H0, H1, carr = (x.astype(np.complex64).astype(np.complex128) for x in (H0, H1, carr))
    Uo, Mo, _, _ = oracle.equiprop(H0, H1, carr, 1e-3, magnus=True, mode=oracle.SIMPSON, single=True,
                                   nthreads=os.cpu_count())
    assert M == Mo
    assert relerr(U, Uo) < TOL["fp32"]


def test_tensor_core_d512_against_oracle(built_lib):
    """complex64, d=512 (16 tiles of 128 x 128 complex per product): two steps
    against the oracle, including the tree's single product."""
    rng = np.random.default_rng(512)
    from parament_gb300.workloads import hermitian
    H0 = hermitian(rng, 512, 8.0)
    H1 = hermitian(rng, 512, 1.0)[None]
    carr = rng.standard_normal((1, 2))
    U, M = run(H0, H1, list(carr), 1e-3, precision="fp32")
    H0, H1, carr = (x.astype(np.complex64).astype(np.complex128) for x in (H0, H1, carr))
    Uo, Mo, _, _ = oracle.equiprop(H0, H1, carr, 1e-3, single=True, nthreads=os.cpu_count())
    assert M == Mo
    assert relerr(U, Uo) < TOL["fp32"]
