"""GB300-native Kerr null-geodesic batch tracer (libbhk) for the photon path of Black_simulation.

The compute lives in libbhk.so (hand-written sm_103a CUDA behind the C ABI in include/bhk.h);
`black_simulation_gb300.bhk` is the Python host layer over it.
"""
from . import bhk  # noqa: F401

__all__ = ["bhk"]
