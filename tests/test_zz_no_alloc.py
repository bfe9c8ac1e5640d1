"""Parament_equipropNoAlloc_fp64: equiprop for callers that may not allocate
device memory while they propagate (real-time loops, applications that own
their GPU memory pool, plug-ins where cudaMalloc is forbidden).

Called through the C-ABI with ctypes and compared with the regular
device-buffer entry point, Parament_equipropDevice_fp64, on two calls in a row
with different samples, within the complex128 parity tolerance (1e-10
relative Frobenius).  Also: dt = 0 gives the identity, a scratch limit that
forces fewer chunks than the regular path gives the same product, and the
size limit is reported.  Kept in a file that pytest collects last.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _lib(path):
    lib = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    lib.Parament_create_fp64.argtypes = [ctypes.POINTER(vp)]
    lib.Parament_destroy_fp64.argtypes = [vp]
    c128 = np.ctypeslib.ndpointer(np.complex128, flags="C_CONTIGUOUS")
    lib.Parament_setHamiltonian_fp64.argtypes = [vp, c128, c128, ctypes.c_uint, ctypes.c_uint, ctypes.c_bool,
                                                 ctypes.c_int]
    for name in ("Parament_equipropDevice_fp64", "Parament_equipropNoAlloc_fp64"):
        getattr(lib, name).argtypes = [vp, vp, ctypes.c_double, ctypes.c_uint, ctypes.c_uint, vp, vp]
    lib.Parament_errorMessage.argtypes = [ctypes.c_int]
    lib.Parament_errorMessage.restype = ctypes.c_char_p
    lib.Parament_deviceMemoryBytes_fp64.argtypes = [vp]
    lib.Parament_deviceMemoryBytes_fp64.restype = ctypes.c_ulonglong
    lib.Parament_lastLaunchCount_fp64.argtypes = [vp]
    lib.Parament_lastLaunchCount_fp64.restype = ctypes.c_int
    return lib


def _problem(d, K, seed):
    rng = np.random.default_rng(seed)
    from parament_gb300.workloads import hermitian
    H0 = hermitian(rng, d, 10.0)
    H1 = np.stack([hermitian(rng, d, 1.0) for _ in range(K)])
    return np.ascontiguousarray(H0.ravel()), np.ascontiguousarray(H1.ravel())


@pytest.mark.parametrize("d,K,magnus,mode,pts", [(64, 4, True, 0x02000000, 2049), (16, 2, False, 0, 3000),
                                                 (5, 3, False, 0x01000000, 101)])
def test_no_alloc_matches_device_entry_point(built_lib, d, K, magnus, mode, pts):
    import torch

    lib = _lib(built_lib)
    ctx = ctypes.c_void_p()
    assert lib.Parament_create_fp64(ctypes.byref(ctx)) == 0
    try:
        H0, H1 = _problem(d, K, d)
        assert lib.Parament_setHamiltonian_fp64(ctx, H0, H1, d, K, magnus, mode) == 0
        stream = torch.cuda.current_stream().cuda_stream
        rng = np.random.default_rng(100 + d)
        for call in range(2):
            carr = torch.tensor(rng.standard_normal((K, pts)), dtype=torch.complex128, device="cuda")
            ref = torch.empty((d, d), dtype=torch.complex128, device="cuda")
            out = torch.full((d, d), float("nan"), dtype=torch.complex128, device="cuda")
            assert lib.Parament_equipropDevice_fp64(ctx, carr.data_ptr(), 1e-3, pts, K, ref.data_ptr(), stream) == 0
            torch.cuda.synchronize()
            held = lib.Parament_deviceMemoryBytes_fp64(ctx)
            free_before = torch.cuda.mem_get_info()[0]
            assert lib.Parament_equipropNoAlloc_fp64(ctx, carr.data_ptr(), 1e-3, pts, K, out.data_ptr(), stream) == 0
            torch.cuda.synchronize()
            # The context's buffers are untouched; the driver's free memory is a
            # second, looser check (it counts other processes on the GPU too).
            assert lib.Parament_deviceMemoryBytes_fp64(ctx) == held
            assert lib.Parament_lastLaunchCount_fp64(ctx) >= 1
            if call == 1:  # after the first call's one-time set-up, nothing is allocated
                assert torch.cuda.mem_get_info()[0] >= free_before
            R, U = ref.cpu().numpy(), out.cpu().numpy()
            err = np.linalg.norm(U - R) / np.linalg.norm(R)
            assert err < TOL, (call, err)
    finally:
        lib.Parament_destroy_fp64(ctx)


def test_no_alloc_rejects_dimensions_past_its_scratch(built_lib):
    import torch

    lib = _lib(built_lib)
    ctx = ctypes.c_void_p()
    assert lib.Parament_create_fp64(ctypes.byref(ctx)) == 0
    try:
        H0, H1 = _problem(65, 1, 1)
        assert lib.Parament_setHamiltonian_fp64(ctx, H0, H1, 65, 1, False, 0) == 0
        carr = torch.zeros((1, 8), dtype=torch.complex128, device="cuda")
        out = torch.empty((65, 65), dtype=torch.complex128, device="cuda")
        code = lib.Parament_equipropNoAlloc_fp64(ctx, carr.data_ptr(), 1e-3, 8, 1, out.data_ptr(), None)
        assert code == 1020
        assert b"no-allocation" in lib.Parament_errorMessage(code)
    finally:
        lib.Parament_destroy_fp64(ctx)


def test_no_alloc_zero_dt_gives_identity(built_lib):
    import torch

    lib = _lib(built_lib)
    ctx = ctypes.c_void_p()
    assert lib.Parament_create_fp64(ctypes.byref(ctx)) == 0
    try:
        H0, H1 = _problem(8, 2, 3)
        assert lib.Parament_setHamiltonian_fp64(ctx, H0, H1, 8, 2, False, 0) == 0
        carr = torch.ones((2, 10), dtype=torch.complex128, device="cuda")
        out = torch.full((8, 8), float("nan"), dtype=torch.complex128, device="cuda")
        assert lib.Parament_equipropNoAlloc_fp64(ctx, carr.data_ptr(), 0.0, 10, 2, out.data_ptr(), None) == 0
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), np.eye(8))
        assert lib.Parament_lastLaunchCount_fp64(ctx) == 1
    finally:
        lib.Parament_destroy_fp64(ctx)


_FEWER_CHUNKS = """
import ctypes, sys
import numpy as np, torch
sys.path[:0] = [sys.argv[2], sys.argv[3]]
from test_zz_no_alloc import _lib, _problem
lib = _lib(sys.argv[1])
ctx = ctypes.c_void_p()
assert lib.Parament_create_fp64(ctypes.byref(ctx)) == 0
d, K, pts = 64, 4, 2049
H0, H1 = _problem(d, K, 11)
assert lib.Parament_setHamiltonian_fp64(ctx, H0, H1, d, K, True, 0x02000000) == 0
carr = torch.tensor(np.random.default_rng(5).standard_normal((K, pts)), dtype=torch.complex128, device="cuda")
ref = torch.empty((d, d), dtype=torch.complex128, device="cuda")
out = torch.empty((d, d), dtype=torch.complex128, device="cuda")
assert lib.Parament_equipropDevice_fp64(ctx, carr.data_ptr(), 1e-3, pts, K, ref.data_ptr(), None) == 0
assert lib.Parament_equipropNoAlloc_fp64(ctx, carr.data_ptr(), 1e-3, pts, K, out.data_ptr(), None) == 0
torch.cuda.synchronize()
R, U = ref.cpu().numpy(), out.cpu().numpy()
print("ERR", np.linalg.norm(U - R) / np.linalg.norm(R))
lib.Parament_destroy_fp64(ctx)
"""


def test_no_alloc_fewer_chunks_than_the_regular_path(built_lib):
    """With the usable scratch cut to 13 chunk pairs at d=64 (the reduced chunk
    count a GPU with more SMs than chunks that fit would get), the product of
    fewer, longer chunks equals the regular entry point's."""
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    env = dict(os.environ, PARAMENT_NOALLOC_SCRATCH_BYTES=str(13 * 2 * 16 * 64 * 64))
    r = subprocess.run([sys.executable, "-c", _FEWER_CHUNKS, built_lib, here, root], cwd=root, env=env,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    err = float(r.stdout.split("ERR")[1].split()[0])
    assert err < TOL, err
