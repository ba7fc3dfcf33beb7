"""GB300-native FIM Newton-step hot path of OpenCAEPoroX.

The compute lives in libocpx_gb300.so (hand-written CUDA for sm_103a behind
the C ABI declared in include/ocpx.h); this package builds it and mirrors the
reference's IsoT_FIM calls on top of it (see ``fim.FimContext``).
"""
from .fim import FimContext, Grid, Model, OcpxError, load_library, model_and_grid_from_dump  # noqa: F401

__all__ = ["FimContext", "Grid", "Model", "OcpxError", "load_library", "model_and_grid_from_dump"]
