"""GB300-native discrete-velocity Shakhov solver (Hybrid2D kinetic hot path).

The compute path is the CUDA library built from csrc/ (libhyb_gb300.so),
reached through the C ABI declared in include/hyb_dvm.h.  This package holds
the thin Python host side: ctypes struct mirrors (hyb_types), case set-up
(cases), the ABI binding (abi) and the build recipe (build).
"""
__all__ = ["hyb_types", "cases", "abi", "build"]
