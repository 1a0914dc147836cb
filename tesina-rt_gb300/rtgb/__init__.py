"""Host-side Python glue for librt_cuda.so (the GB300 Whitted ray tracer)."""
from . import abi, scenes  # noqa: F401
