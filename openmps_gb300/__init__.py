"""GB300-native MPS time step with OpenMps's compute-class interface.

The product is ``libopenmps_gb300.so`` (C ABI in ``include/mps.h``): hand-written
sm_103a kernels for every stage of ``Computer::ForwardTime`` plus the host code that
orchestrates them.  This package holds its sources (``csrc/``), its build recipe
(``build.py``), a Python mirror of the ``Computer`` class over the C ABI
(``computer.py``) and the seeded scene generators used by tests and benchmarks
(``scenes.py``).
"""
from . import _abi as abi  # noqa: F401
from .computer import Computer, ComputerError, create_computer, load_library  # noqa: F401

__all__ = ["abi", "Computer", "ComputerError", "create_computer", "load_library"]
