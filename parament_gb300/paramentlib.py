"""ctypes binding of libparament.so (the GB300 build).

Library lookup follows the reference wrapper
(src/python/pyparament/parament/paramentlib.py:21-46): ``$PARAMENT_LIB_DIR``
first, else the package directory, else (with ``$USE_SHARED_PARAMENT`` set) the
system search path.  Argument types mirror the reference's
(paramentlib.py:51-72) and add the entry points the reference lacks.
"""
import ctypes
import os
import pathlib

import numpy as np

USE_SHARED_PARAMENT = os.environ.get("USE_SHARED_PARAMENT")
PARAMENT_LIB_DIR = os.environ.get("PARAMENT_LIB_DIR")

if os.name != "posix":
    raise RuntimeError("Don't know how to load library on " + os.name)

if PARAMENT_LIB_DIR:
    lib_path = str(pathlib.Path(PARAMENT_LIB_DIR) / "libparament.so")
elif not USE_SHARED_PARAMENT:
    lib_path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libparament.so")
else:
    lib_path = "libparament.so"

if not USE_SHARED_PARAMENT and not os.path.exists(lib_path):
    raise ImportError(
        f"libparament.so not found at {lib_path}: build it first "
        "(python -c 'import __graft_entry__ as g; g.build()' or python parament_gb300/build.py)")

lib = ctypes.cdll.LoadLibrary(lib_path)

c_ParamentContext_p = ctypes.c_void_p
c_cuComplex_p = np.ctypeslib.ndpointer(np.complex64)
c_cuDoubleComplex_p = np.ctypeslib.ndpointer(np.complex128)

lib.Parament_create.argtypes = [ctypes.POINTER(c_ParamentContext_p)]
lib.Parament_destroy.argtypes = [c_ParamentContext_p]
lib.Parament_setHamiltonian.argtypes = [c_ParamentContext_p, c_cuComplex_p, c_cuComplex_p, ctypes.c_uint,
                                        ctypes.c_uint, ctypes.c_bool, ctypes.c_int]
lib.Parament_equiprop.argtypes = [c_ParamentContext_p, c_cuComplex_p, ctypes.c_double, ctypes.c_uint, ctypes.c_uint,
                                  c_cuComplex_p]
lib.Parament_errorMessage.argtypes = [ctypes.c_int]
lib.Parament_errorMessage.restype = ctypes.c_char_p
lib.Parament_peekAtLastError.argtypes = [c_ParamentContext_p]
lib.Parament_setIterationCyclesManually.argtypes = [c_ParamentContext_p, ctypes.c_uint]
lib.Parament_automaticIterationCycles.argtypes = [c_ParamentContext_p]
lib.Parament_selectIterationCycles_fp32.argtypes = [ctypes.c_double, ctypes.c_double]
lib.Parament_selectIterationCycles_fp32.restype = ctypes.c_int

lib.Parament_create_fp64.argtypes = [ctypes.POINTER(c_ParamentContext_p)]
lib.Parament_destroy_fp64.argtypes = [c_ParamentContext_p]
lib.Parament_setHamiltonian_fp64.argtypes = [c_ParamentContext_p, c_cuDoubleComplex_p, c_cuDoubleComplex_p,
                                             ctypes.c_uint, ctypes.c_uint, ctypes.c_bool, ctypes.c_int]
lib.Parament_equiprop_fp64.argtypes = [c_ParamentContext_p, c_cuDoubleComplex_p, ctypes.c_double, ctypes.c_uint,
                                       ctypes.c_uint, c_cuDoubleComplex_p]
lib.Parament_peekAtLastError_fp64.argtypes = [c_ParamentContext_p]
lib.Parament_setIterationCyclesManually_fp64.argtypes = [c_ParamentContext_p, ctypes.c_uint]
lib.Parament_automaticIterationCycles_fp64.argtypes = [c_ParamentContext_p]
lib.Parament_selectIterationCycles_fp64.argtypes = [ctypes.c_double, ctypes.c_double]
lib.Parament_selectIterationCycles_fp64.restype = ctypes.c_int

lib.OneNorm.argtypes = [c_cuComplex_p, ctypes.c_uint]
lib.OneNorm.restype = ctypes.c_double
lib.OneNorm_fp64.argtypes = [c_cuDoubleComplex_p, ctypes.c_uint]
lib.OneNorm_fp64.restype = ctypes.c_double
lib.device_info.argtypes = []

# Extensions
lib.Parament_setPrecisionMode.argtypes = [c_ParamentContext_p, ctypes.c_int]
lib.Parament_getPrecisionMode.argtypes = [c_ParamentContext_p]
lib.Parament_getPrecisionMode.restype = ctypes.c_int
lib.Parament_lastIterationCycles.argtypes = [c_ParamentContext_p]
lib.Parament_lastIterationCycles.restype = ctypes.c_int
lib.Parament_lastIterationCycles_fp64.argtypes = [c_ParamentContext_p]
lib.Parament_lastIterationCycles_fp64.restype = ctypes.c_int
lib.Parament_hamiltonianNorm.argtypes = [c_ParamentContext_p]
lib.Parament_hamiltonianNorm.restype = ctypes.c_double
lib.Parament_hamiltonianNorm_fp64.argtypes = [c_ParamentContext_p]
lib.Parament_hamiltonianNorm_fp64.restype = ctypes.c_double
for _name in ("Parament_equipropDevice", "Parament_equipropDevice_fp64"):
    getattr(lib, _name).argtypes = [c_ParamentContext_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_uint,
                                    ctypes.c_uint, ctypes.c_void_p, ctypes.c_void_p]
for _sfx in ("", "_fp64"):
    getattr(lib, "Parament_synchronize" + _sfx).argtypes = [c_ParamentContext_p]
    getattr(lib, "Parament_deviceMemoryBytes" + _sfx).argtypes = [c_ParamentContext_p]
    getattr(lib, "Parament_deviceMemoryBytes" + _sfx).restype = ctypes.c_ulonglong
    getattr(lib, "Parament_setKernelTiming" + _sfx).argtypes = [c_ParamentContext_p, ctypes.c_int]
    getattr(lib, "Parament_lastKernelMs" + _sfx).argtypes = [c_ParamentContext_p]
    getattr(lib, "Parament_lastKernelMs" + _sfx).restype = ctypes.c_float
    getattr(lib, "Parament_lastLaunchCount" + _sfx).argtypes = [c_ParamentContext_p]
    getattr(lib, "Parament_lastLaunchCount" + _sfx).restype = ctypes.c_int
lib.Parament_equipropVJP.argtypes = [c_ParamentContext_p, c_cuComplex_p, ctypes.c_double, ctypes.c_uint,
                                     ctypes.c_uint, c_cuComplex_p, np.ctypeslib.ndpointer(np.float32)]
lib.Parament_equipropVJP_fp64.argtypes = [c_ParamentContext_p, c_cuDoubleComplex_p, ctypes.c_double, ctypes.c_uint,
                                          ctypes.c_uint, c_cuDoubleComplex_p, np.ctypeslib.ndpointer(np.float64)]
for _name in ("Parament_equipropVJPDevice", "Parament_equipropVJPDevice_fp64"):
    getattr(lib, _name).argtypes = [c_ParamentContext_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_uint,
                                    ctypes.c_uint, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
