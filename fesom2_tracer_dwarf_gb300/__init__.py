"""GB300-native FESOM2 tracer-advection step (do_oce_adv_tra) with the
reference dwarf's C-ABI and Python wrapper.

- ``mesh.Mesh``: analytic mesh set-up and device upload
- ``engine.TracerAdvection``: K tracers stepped on the GPU (FP64 / FP32 forms)
- ``demo_tracer.FESOMTracerAdvection``: the reference's ctypes wrapper class
- ``synthetic``: seeded flows and fields of the benchmark configurations
"""
from . import _lib  # noqa: F401

__all__ = ["mesh", "engine", "synthetic", "demo_tracer"]
