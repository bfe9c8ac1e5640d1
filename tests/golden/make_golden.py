"""Generates the golden fixtures under tests/golden/.

equiprop_cases.npz
    Small equiprop problems covering every quadrature mode, Magnus on/off,
    K = 1..4 controls, fewer sample arrays than controls, odd/even step counts
    and both context precisions, plus the reference's own known-answer cases
    (the docstring example of src/python/pyparament/parament/parament.py:61-68
    and the seed-27 problems of src/python/pyparament/parament/test/test_numerics.py).
    Expected outputs come from the CPU oracle in FP64 and are checked here
    against an independent SciPy expm product before being written.

ref_host.json
    Outputs of the reference library's host-side functions -- the order tables
    (Parament_selectIterationCycles_fp32/_fp64), the norm bound (OneNorm,
    OneNorm_fp64) and the error strings (Parament_errorMessage) -- taken from
    the reference built from its own sources by oracle/build_ref.sh.  These
    functions need no GPU, so they run in the build container.

Run from the repository root:  python tests/golden/make_golden.py
"""
import ctypes
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def herm(rng, d, norm=1.0):
    a = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    h = (a + a.conj().T) / 2
    return h * (norm / np.linalg.norm(h, 2))


def seed27_hamiltonians(dim):
    """The generator of test_numerics.py:24-29 (legacy NumPy seed 27)."""
    np.random.seed(27)
    H0 = np.random.uniform(-1, 1, (dim, dim)) / dim + 1j * np.random.uniform(-1, 1, (dim, dim)) / 2
    H0 = H0 + H0.conj().T
    return H0, np.zeros((dim, dim), dtype=complex)


def make_cases():
    cases = []

    def add(name, H0, H1, carr, dt, magnus, mode, precision, K=None):
        H0 = np.asarray(H0, np.complex128)
        d = H0.shape[0]
        H1 = np.asarray(H1, np.complex128).reshape(-1, d, d)
        carr = np.asarray(carr, np.complex128)
        carr = carr.reshape(-1, carr.shape[-1]) if carr.size else np.zeros((0, 1), np.complex128)
        if precision == "fp32":  # what the complex64 API receives
            H0 = H0.astype(np.complex64).astype(np.complex128)
            H1 = H1.astype(np.complex64).astype(np.complex128)
            carr = carr.astype(np.complex64).astype(np.complex128)
        U, M, hn, st = oracle.equiprop(H0, H1, carr, dt, magnus=magnus, mode=mode, single=(precision == "fp32"))
        assert st == 0, (name, st)
        R = oracle.scipy_expm_product(H0, H1, carr, dt, magnus=magnus, mode=mode)
        err = np.linalg.norm(U - R) / np.linalg.norm(R)
        # The complex64 order table truncates at about the float epsilon.
        assert err < (1e-6 if precision == "fp32" else 1e-12), (name, err)
        cases.append(dict(name=name, H0=H0, H1=H1, carr=carr, dt=float(dt), magnus=bool(magnus), mode=int(mode),
                          precision=precision, U=U, M=int(M), hnorm=float(hn)))

    # Known answers of the reference.
    add("docstring_kat", np.diag([1.0, -1.0]), np.array([[0, 1], [1, 0]]), np.zeros((1, 1)), 1.0, False,
        oracle.NONE, "fp32")
    for prec in ("fp32", "fp64"):
        for dim in (2, 16):
            H0, H1 = seed27_hamiltonians(dim)
            add(f"seed27_expm_{prec}_d{dim}", H0, H1, np.zeros((1, 1)), 0.01, False, oracle.NONE, prec)
    for dim in (2, 4):
        H0, _ = seed27_hamiltonians(dim)
        add(f"seed27_debug_expm_d{dim}", 1j * H0, H0, np.zeros((1, 1)), 1.0, False, oracle.NONE, "fp32")
    for dim in (2, 16):
        H0, H1 = seed27_hamiltonians(dim)
        c1 = np.random.rand(10)
        c2 = np.random.rand(10)
        add(f"seed27_multifield_d{dim}", H0, np.stack([H1, H0]), np.stack([c1, c2]), 0.01, False, oracle.NONE,
            "fp32")

    # Mode sweep.
    rng = np.random.default_rng(2024)
    combos = [(False, oracle.NONE), (False, oracle.MIDPOINT), (False, oracle.SIMPSON), (True, oracle.SIMPSON)]
    for prec in ("fp32", "fp64"):
        for magnus, mode in combos:
            for K in (1, 2, 3, 4):
                for d in (3, 8):
                    H0 = herm(rng, d, 2.0)
                    H1 = np.stack([herm(rng, d, 1.0) for _ in range(K)])
                    pts = 17
                    carr = rng.standard_normal((K, pts)) + 0.3j * rng.standard_normal((K, pts))
                    tag = f"{prec}_{'magnus' if magnus else 'plain'}_{mode:x}_K{K}_d{d}"
                    add("sweep_" + tag, H0, H1, carr, 0.02, magnus, mode, prec)
            # Fewer sample arrays than controls: the rest have zero amplitude.
            H0 = herm(rng, 5, 2.0)
            H1 = np.stack([herm(rng, 5, 1.0) for _ in range(3)])
            carr = rng.standard_normal((2, 9))
            add(f"fewer_amps_{prec}_{'magnus' if magnus else 'plain'}_{mode:x}", H0, H1, carr, 0.03, magnus, mode,
                prec)
    # Tree shapes: odd leftovers at every level.
    for P in (1, 2, 3, 5, 7, 12):
        H0 = herm(rng, 4, 3.0)
        H1 = herm(rng, 4, 1.0)[None]
        add(f"tree_P{P}", H0, H1, rng.standard_normal((1, P)), 0.05, False, oracle.NONE, "fp64")
    # cfg1-like, short.
    H0 = herm(rng, 16, 1.0)
    H1 = np.stack([herm(rng, 16, 1.0) for _ in range(2)])
    add("d16_K2_P64", H0, H1, rng.standard_normal((2, 64)), 1e-3, False, oracle.NONE, "fp64")
    return cases


def save_cases(cases):
    arrays = {}
    meta = []
    for i, c in enumerate(cases):
        for k in ("H0", "H1", "carr", "U"):
            arrays[f"c{i}_{k}"] = c[k]
        meta.append({k: c[k] for k in ("name", "dt", "magnus", "mode", "precision", "M", "hnorm")})
    arrays["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(OUT, "equiprop_cases.npz"), **arrays)


def ref_host_values():
    so = os.path.join(ROOT, "oracle", "_ref", "libparament_ref.so")
    if not os.path.exists(so):
        # the reference root comes from $PARAMENT_REFERENCE_ROOT (build_ref.sh)
        subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh")])
    L = ctypes.CDLL(so)
    for n in ("Parament_selectIterationCycles_fp32", "Parament_selectIterationCycles_fp64"):
        getattr(L, n).argtypes = [ctypes.c_double, ctypes.c_double]
        getattr(L, n).restype = ctypes.c_int
    L.Parament_errorMessage.argtypes = [ctypes.c_int]
    L.Parament_errorMessage.restype = ctypes.c_char_p
    L.OneNorm.argtypes = [np.ctypeslib.ndpointer(np.complex64), ctypes.c_uint]
    L.OneNorm.restype = ctypes.c_double
    L.OneNorm_fp64.argtypes = [np.ctypeslib.ndpointer(np.complex128), ctypes.c_uint]
    L.OneNorm_fp64.restype = ctypes.c_double
    # Probe points: each threshold and its two neighbouring doubles, plus a sweep.
    lim32 = [0.032516793, 0.219062571, 0.619625593, 1.218059203, 1.979888284, 2.873301187, 3.872963682,
             4.959398466, 6.117657121, 7.336154907, 8.605792444, 9.919320831, 11.27088616, 12.65570085]
    lim64 = [0.000213616, 0.00768149, 0.0501474, 0.162592, 0.368382, 0.676861, 1.08784, 1.59605, 2.19402, 2.87366,
             3.62716, 4.44725, 5.3274, 6.26179, 7.2453, 8.27338, 9.34206, 10.4478, 11.5875, 12.7584]
    xs = sorted(set([np.nextafter(t, -1) for t in lim32 + lim64] + lim32 + lim64 +
                    [np.nextafter(t, 2 * t + 1) for t in lim32 + lim64] + list(np.linspace(0, 14, 141))))
    cycles = [[float(x), L.Parament_selectIterationCycles_fp32(float(x), 1.0),
               L.Parament_selectIterationCycles_fp64(float(x), 1.0)] for x in xs]
    rng = np.random.default_rng(7)
    norms = []
    for d in (1, 2, 5, 16, 33):
        m = (rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))) * 3.0
        m64 = np.ascontiguousarray(m.ravel())
        m32 = np.ascontiguousarray(m.astype(np.complex64).ravel())
        norms.append({"d": d, "re": m.real.ravel().tolist(), "im": m.imag.ravel().tolist(),
                      "onenorm_fp32": L.OneNorm(m32, d), "onenorm_fp64": L.OneNorm_fp64(m64, d)})
    codes = [0, 10, 20, 30, 50, 60, 70, 80, 90, 1000, 12345]
    messages = {str(c): L.Parament_errorMessage(c).decode() for c in codes}
    return {"cycles": cycles, "norms": norms, "messages": messages}


if __name__ == "__main__":
    cases = make_cases()
    save_cases(cases)
    print(f"wrote {len(cases)} equiprop cases")
    with open(os.path.join(OUT, "ref_host.json"), "w") as f:
        json.dump(ref_host_values(), f)
    print("wrote ref_host.json")
