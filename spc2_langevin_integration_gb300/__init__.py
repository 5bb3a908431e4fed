"""GB300-native (sm_103a) particle-update path of raven91/spc2_langevin_integration.

The product is the CUDA library behind ``include/spc_gb300.h`` (built from
``csrc/`` into ``_build/libspc_gb300.so``); ``abi`` is its Python binding and
``host/`` holds the C++ adapters with the reference's class names.
"""
from . import abi, build  # noqa: F401

__all__ = ["abi", "build"]
