"""neslgpu_gb300 -- a GB300-native CVL vector library for NESL's VCODE
interpreter.

The product is ``libcvl_gb300.so``: the C ABI of the reference's
``nesl/include/cvl.h`` implemented with hand-written sm_103a kernels
(sources in ``csrc/``, declarations in ``include/cvl_gb300.h``).  This
package holds the build driver and a ctypes binding of that ABI.
"""
from .cvl import CVL, CVLError, DeviceVector, check, load, segdes  # noqa: F401

__all__ = ["CVL", "CVLError", "DeviceVector", "check", "load", "segdes"]
