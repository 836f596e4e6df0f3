"""GB300-native Malevich draw path: a Direct3D-11-flavoured C ABI (include/malevich.h) over
hand-written CUDA kernels for sm_103a. `api` is the Python front end of that ABI; `scenes`
holds frame descriptions and the seeded synthetic scenes."""
from . import scenes  # noqa: F401

__all__ = ["scenes", "api", "build"]
