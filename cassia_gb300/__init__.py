"""cassia_gb300: GB300-native surpass/mold rasterize -> sort -> paint.

The compute path is the in-tree CUDA library (include/cassia_gb300.h) driven
through its C ABI; this package is the host-side mirror of mold's API
(Composition, Layer, Path, Props, Style).  There is no CPU fallback: the
native library must be built (cassia_gb300.build.build()) and a GPU present.
"""
from .abi import CassiaError  # noqa: F401
from .types import (BlendMode, FillRule, Gradient, GradientType, Path, Point, Props, Style,  # noqa: F401
                    solid)

__version__ = "0.1.0"


def __getattr__(name):
    # The native-backed classes import lazily so that the pure types above
    # are usable (and tests collectable) without the CUDA library.
    if name in ("Composition", "Layer", "Buffer"):
        from . import composition
        return getattr(composition, name)
    raise AttributeError(name)
