"""parament_gb300: GB300-native drop-in for the Parament equiprop path.

Same Python surface as the reference's ``parament`` package
(src/python/pyparament/parament/__init__.py:15-16): ``Parament``, ``expm``,
``device_info`` and the ``constants`` module, over ``libparament.so`` built
from ``csrc/`` for sm_103a.  ``import parament_gb300 as parament`` switches an
existing script over.
"""
from . import constants
from .parament import Parament
from .debug_functions import device_info, expm

__all__ = ["Parament", "expm", "device_info", "constants"]
