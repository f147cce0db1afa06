"""GB300-native chunk generation for UnderwaterWorld terrain.

The compute path is ``libuww_gb300.so`` (CUDA, sm_103a) behind the C ABI of
``include/uww.h``.  This package holds its ctypes binding (:mod:`.abi`), the
host-side mirror of the reference's ``Chunk`` / ``perlin_util`` interface
(:mod:`.chunk`) and the build script (:mod:`.build`).
"""
from . import abi  # noqa: F401

__all__ = ["abi"]
