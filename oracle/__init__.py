"""CPU oracle for the equiprop path -- test infrastructure, not product code.

The oracle is a plain-C restatement (``paramentref.c``) of the reference
algorithm: norm bound, order tables, Bessel coefficients, quadrature/Magnus
expansion, Clenshaw recurrence and the pairwise tree product.  Only the tests,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use it,
always as the checker or the baseline, never as the thing measured or shipped.

Each helper cites the reference file:line it follows (paths inside the
parament project).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "paramentref.c")

NONE, MIDPOINT, SIMPSON = 0x00000000, 0x01000000, 0x02000000
MODES = {"none": NONE, "midpoint": MIDPOINT, "simpson": SIMPSON}

_lib = None
_lock = threading.Lock()


def build(force: bool = False) -> str:
    """Compile the C restatement into ``oracle/liboracle.so`` with gcc."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(SRC):
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        subprocess.check_call(
            ["gcc", "-O3", "-std=gnu11", "-Wall", "-Werror", "-fcx-limited-range", "-fPIC", "-shared", "-pthread", SRC, "-o", tmp, "-lm"]
        )
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    """Load (building if needed) the oracle shared library."""
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            c128 = np.ctypeslib.ndpointer(np.complex128, flags="C_CONTIGUOUS")
            L.pr_select_cycles.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double]
            L.pr_select_cycles.restype = ctypes.c_int
            L.pr_onenorm.argtypes = [c128, ctypes.c_uint, ctypes.c_int]
            L.pr_onenorm.restype = ctypes.c_double
            L.pr_bessel_coeffs.argtypes = [ctypes.c_int, ctypes.c_double, c128]
            L.pr_num_steps.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint]
            L.pr_num_steps.restype = ctypes.c_long
            L.pr_expansion_count.argtypes = [ctypes.c_uint, ctypes.c_int]
            L.pr_expansion_count.restype = ctypes.c_uint
            L.pr_build_stack.argtypes = [c128, c128, ctypes.c_uint, ctypes.c_uint, ctypes.c_int, c128]
            L.pr_step_weights.argtypes = [c128, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_double, ctypes.c_long, c128]
            L.pr_clenshaw.argtypes = [c128, ctypes.c_uint, ctypes.c_int, c128, ctypes.c_double, c128, c128]
            L.pr_equiprop.argtypes = [c128, c128, ctypes.c_uint, ctypes.c_uint, ctypes.c_int, ctypes.c_int, c128,
                                      ctypes.c_double, ctypes.c_uint, ctypes.c_uint, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_int, c128, ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_double)]
            L.pr_equiprop.restype = ctypes.c_int
            L.pr_step_exponentials.argtypes = [c128, c128, ctypes.c_uint, ctypes.c_uint, ctypes.c_int, ctypes.c_int,
                                               c128, ctypes.c_double, ctypes.c_uint, ctypes.c_uint, ctypes.c_int,
                                               ctypes.c_double, ctypes.c_long, ctypes.c_long, ctypes.c_int, c128]
            L.pr_step_exponentials.restype = ctypes.c_int
            L.pr_tree_product.argtypes = [c128, ctypes.c_long, ctypes.c_uint, ctypes.c_int]
            _lib = L
    return _lib


def _c128(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.complex128))


def select_cycles(hnorm: float, dt: float, fp64: bool) -> int:
    """Order table lookup (src/cuda/parament.cpp:723-766)."""
    return int(lib().pr_select_cycles(1 if fp64 else 0, float(hnorm), float(dt)))


def onenorm(m, single: bool = False) -> float:
    """Max absolute row sum (src/cuda/mathhelper.cpp:82-114)."""
    m = _c128(m)
    return float(lib().pr_onenorm(m, m.shape[0], 1 if single else 0))


def bessel_coeffs(M: int, x: float) -> np.ndarray:
    """(-i)^k J_k(x) for k=0..M (src/cuda/mathhelper.cpp:35-80)."""
    out = np.zeros(M + 1, np.complex128)
    lib().pr_bessel_coeffs(int(M), float(x), out)
    return out


def num_steps(mode: int, magnus: bool, pts: int) -> int:
    return int(lib().pr_num_steps(int(mode), 1 if magnus else 0, int(pts)))


def expansion_count(K: int, magnus: bool) -> int:
    return int(lib().pr_expansion_count(int(K), 1 if magnus else 0))


def build_stack(H0, H1, magnus: bool) -> np.ndarray:
    """[H0, H_1..H_K, ([H0,H_k])_k, ([H_j,H_i])_(j<i)] (src/cuda/parament.cpp:289-359)."""
    H0 = _c128(H0)
    H1 = _c128(H1).reshape(-1, H0.shape[0], H0.shape[0])
    d, K = H0.shape[0], H1.shape[0]
    out = np.zeros((1 + expansion_count(K, magnus), d, d), np.complex128)
    lib().pr_build_stack(H0, H1, d, K, 1 if magnus else 0, out)
    return out


def step_weights(carr, K: int, mode: int, magnus: bool, h: float, s: int) -> np.ndarray:
    carr = _c128(np.atleast_2d(carr))
    amps, pts = carr.shape
    out = np.zeros(expansion_count(K, magnus), np.complex128)
    lib().pr_step_weights(carr, pts, amps, K, int(mode), 1 if magnus else 0, float(h), int(s), out)
    return out


def clenshaw(X, M: int, J, s: float) -> np.ndarray:
    X = _c128(X)
    d = X.shape[0]
    U = np.zeros_like(X)
    work = np.zeros(3 * d * d, np.complex128)
    lib().pr_clenshaw(X, d, int(M), _c128(J), float(s), U, work)
    return U


def equiprop(H0, H1, carr, dt: float, magnus: bool = False, mode: int = NONE, single: bool = False,
             M: int = 0, nthreads: int = 1):
    """Full restatement of Parament_equiprop (src/cuda/parament.cpp:791-851).

    Returns (U, M_used, hnorm, status).  ``single`` selects the complex64
    context's order table and norm moduli; arithmetic stays FP64.
    """
    H0 = _c128(H0)
    d = H0.shape[0]
    H1 = _c128(H1).reshape(-1, d, d)
    K = H1.shape[0]
    carr = _c128(np.atleast_2d(carr))
    amps, pts = carr.shape
    out = np.zeros((d, d), np.complex128)
    Mu = ctypes.c_int(0)
    hn = ctypes.c_double(0.0)
    st = lib().pr_equiprop(H0, H1, d, K, 1 if magnus else 0, int(mode), carr, float(dt), pts, amps,
                           1 if single else 0, int(M), int(nthreads), out, ctypes.byref(Mu), ctypes.byref(hn))
    return out, Mu.value, hn.value, st


def step_exponentials(H0, H1, carr, dt, magnus, mode, M, hnorm, s0, s1, nthreads=1) -> np.ndarray:
    H0 = _c128(H0)
    d = H0.shape[0]
    H1 = _c128(H1).reshape(-1, d, d)
    carr = _c128(np.atleast_2d(carr))
    amps, pts = carr.shape
    U = np.zeros((s1 - s0, d, d), np.complex128)
    st = lib().pr_step_exponentials(H0, H1, d, H1.shape[0], 1 if magnus else 0, int(mode), carr, float(dt), pts,
                                    amps, int(M), float(hnorm), int(s0), int(s1), int(nthreads), U)
    if st:
        raise MemoryError("oracle allocation failed")
    return U


def tree_product(mats, nthreads: int = 1) -> np.ndarray:
    m = _c128(mats).copy()
    lib().pr_tree_product(m, m.shape[0], m.shape[1], int(nthreads))
    return m[0]


def scipy_expm_product(H0, H1, carr, dt, magnus=False, mode=NONE, s0=0, s1=None):
    """Independent cross-check: scipy.linalg.expm of every step, multiplied in
    time order (later step on the left), with the same expansion stack.  With
    s0, s1 only the steps [s0, s1) are propagated (their ordered product)."""
    import scipy.linalg

    H0 = _c128(H0)
    d = H0.shape[0]
    H1 = _c128(H1).reshape(-1, d, d)
    K = H1.shape[0]
    carr = _c128(np.atleast_2d(carr))
    h = 2.0 * dt if (magnus or mode == SIMPSON) else dt
    stack = build_stack(H0, H1, magnus)
    P = num_steps(mode, magnus, carr.shape[1])
    s1 = P if s1 is None else min(s1, P)
    U = np.eye(d, dtype=np.complex128)
    for s in range(s0, s1):
        w = step_weights(carr, K, mode, magnus, h, s)
        X = stack[0] + np.tensordot(w, stack[1:], axes=1)
        U = scipy.linalg.expm(-1j * h * X) @ U
    return U


def _scipy_chunk(args):
    """Worker of scipy_baseline: (seconds, product) of the steps [s0, s1)."""
    import time
    H0, H1, carr, dt, magnus, mode, s0, s1 = args
    t0 = time.perf_counter()
    U = scipy_expm_product(H0, H1, carr, dt, magnus, mode, s0, s1)
    return time.perf_counter() - t0, U


def scipy_baseline(H0, H1, carr, dt, magnus=False, mode=NONE, steps=None, procs=1):
    """The NumPy/SciPy FP64 expm-product of the scheme timed on the host: the
    first `steps` steps split into `procs` contiguous chunks, one process each
    (spawned, with one BLAS/OpenMP thread per process), then the ordered
    product of the chunk products.  Returns (steps/s, steps, wall seconds)."""
    import concurrent.futures as cf
    import multiprocessing as mp
    import time

    carr = _c128(np.atleast_2d(carr))
    P = num_steps(mode, magnus, carr.shape[1])
    S = P if steps is None else min(P, int(steps))
    bounds = [S * i // procs for i in range(procs + 1)]
    jobs = [(H0, H1, carr, dt, magnus, mode, bounds[i], bounds[i + 1]) for i in range(procs)]
    keep = {k: os.environ.get(k) for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")}
    for k in keep:
        os.environ[k] = "1"
    try:
        # A worker that fails to start breaks the executor (an exception here),
        # where a multiprocessing.Pool would restart it forever.
        with cf.ProcessPoolExecutor(procs, mp_context=mp.get_context("spawn")) as pool:
            list(pool.map(_scipy_chunk, [(H0, H1, carr, dt, magnus, mode, 0, 1)] * procs))  # start-up, imports
            t0 = time.perf_counter()
            parts = list(pool.map(_scipy_chunk, jobs))
            U = np.eye(np.shape(H0)[0], dtype=np.complex128)
            for _, Ui in parts:
                U = Ui @ U
            wall = time.perf_counter() - t0
    finally:
        for k, v in keep.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    return S / wall, S, wall
