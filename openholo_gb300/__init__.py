"""GB300-native hologram generation (OpenHologram hot path).

Hand-written sm_103a CUDA kernels behind the C ABI in include/oh.h; this
package is the Python host side (ctypes over liboh_gb300.so).  Importing it
does not load the library; the first call does, and fails loudly if the
library has not been built.
"""
from ._lib import Context, OhError, launch_count, lib  # noqa: F401

__all__ = ["Context", "OhError", "launch_count", "lib"]
__version__ = "0.1.0"
