"""GB300-native (sm_103a) backend for palinstrophy's pseudo-spectral 2D DNS step.

``palinstrophy_gb300.turbo_simulator`` mirrors the reference module's stepping
and initialisation API; ``palinstrophy_gb300._lib`` is the ctypes binding of
the C ABI in include/palgpu.h.
"""
__version__ = "0.1.0"
