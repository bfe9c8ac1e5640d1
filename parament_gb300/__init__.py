"""parament_gb300: GB300-native drop-in for the Parament equiprop path.

Same Python surface as the reference's ``parament`` package
(src/python/pyparament/parament/__init__.py:15-16): ``Parament``, ``expm``,
``device_info`` and the ``constants`` module, over ``libparament.so`` built
from ``csrc/`` for sm_103a.  ``import parament_gb300 as parament`` switches an
existing script over.

The shared library is loaded on first use of those names, so that
``parament_gb300.build`` can compile it in a fresh checkout.
"""
from . import constants

__all__ = ["Parament", "expm", "device_info", "constants"]


def __getattr__(name):
    if name == "Parament":
        from .parament import Parament
        return Parament
    if name in ("expm", "device_info"):
        from . import debug_functions
        return getattr(debug_functions, name)
    if name in ("paramentlib", "parament", "debug_functions"):
        import importlib
        return importlib.import_module("." + name, __name__)
    raise AttributeError(name)
