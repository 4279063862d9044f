"""mold's scene types: Path, Props, Style, Fill, Gradient, BlendMode, FillRule.

Pure Python mirrors of mold/src/path/mod.rs:13-179 (Path commands) and
surpass/src/painter/style.rs / painter/mod.rs:125-141 (Props, Func, Style,
Fill, Gradient).  They marshal into the C ABI's plain-data layout
(cassia_gb300.abi) and load no native code.
"""
import ctypes
import enum
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

from . import abi


class FillRule(enum.IntEnum):
    """surpass FillRule (surpass/src/painter/style.rs:10-13)."""
    NonZero = 0
    EvenOdd = 1


class BlendMode(enum.IntEnum):
    """surpass BlendMode (surpass/src/painter/style.rs:190-203)."""
    Over = 0
    Multiply = 1
    Screen = 2
    Overlay = 3
    Darken = 4
    Lighten = 5
    ColorDodge = 6
    ColorBurn = 7
    HardLight = 8
    SoftLight = 9
    Difference = 10
    Exclusion = 11


class GradientType(enum.IntEnum):
    Linear = 0
    Radial = 1


@dataclass(frozen=True)
class Point:
    x: float
    y: float


@dataclass
class Gradient:
    """GradientBuilder + Gradient (style.rs:29-93): stops are (rgba, stop);
    a stop of None is spread evenly as GradientBuilder::build does."""
    start: Tuple[float, float]
    end: Tuple[float, float]
    stops: List[Tuple[Tuple[float, float, float, float], Optional[float]]]
    type: GradientType = GradientType.Linear


@dataclass
class Style:
    """surpass Style (style.rs:427-432); fill is an RGBA tuple (Fill::Solid)
    or a Gradient (Fill::Gradient)."""
    fill: object = (0.0, 0.0, 0.0, 1.0)
    blend_mode: BlendMode = BlendMode.Over
    is_clipped: bool = False


@dataclass
class Props:
    """surpass Props { fill_rule, func } (painter/mod.rs:137-141).  `func` is a
    Style (Func::Draw) or an int n (Func::Clip(n))."""
    fill_rule: FillRule = FillRule.NonZero
    func: object = field(default_factory=Style)

    def to_c(self):
        """Returns (CgbProps, keepalive) — keepalive owns the stops array."""
        p = abi.CgbProps()
        p.fill_rule = int(self.fill_rule)
        keep = None
        if isinstance(self.func, Style):
            st = self.func
            p.func = abi.FUNC_DRAW
            p.is_clipped = 1 if st.is_clipped else 0
            p.blend_mode = int(st.blend_mode)
            if isinstance(st.fill, Gradient):
                g = st.fill
                p.fill_kind = abi.FILL_GRADIENT
                p.gradient_type = int(g.type)
                p.gradient_start[0], p.gradient_start[1] = g.start
                p.gradient_end[0], p.gradient_end[1] = g.end
                flat = []
                for rgba, stop in g.stops:
                    flat += list(rgba) + [(-0.0 if stop is None else float(stop))]
                keep = (ctypes.c_float * len(flat))(*flat)
                p.n_stops = len(g.stops)
                p.stops = ctypes.cast(keep, ctypes.POINTER(ctypes.c_float))
            else:
                p.fill_kind = abi.FILL_SOLID
                for i in range(4):
                    p.color[i] = float(st.fill[i])
        else:
            p.func = abi.FUNC_CLIP
            p.clip_layers = int(self.func)
        return p, keep


def solid(color, fill_rule=FillRule.NonZero, blend_mode=BlendMode.Over) -> Props:
    return Props(fill_rule=fill_rule, func=Style(fill=tuple(color), blend_mode=blend_mode))


class Path:
    """mold Path (mold/src/path/mod.rs:23-179): one contour of commands."""

    def __init__(self):
        self.kinds: List[int] = []
        self.points: List[float] = []

    @staticmethod
    def _xy(p):
        return (float(p.x), float(p.y)) if isinstance(p, Point) else (float(p[0]), float(p[1]))

    def line(self, p0, p1):
        self.kinds.append(abi.CMD_LINE)
        self.points += [*self._xy(p0), *self._xy(p1)]
        return self

    def quad(self, p0, p1, p2):
        self.kinds.append(abi.CMD_QUAD)
        self.points += [*self._xy(p0), *self._xy(p1), *self._xy(p2)]
        return self

    def cubic(self, p0, p1, p2, p3):
        self.kinds.append(abi.CMD_CUBIC)
        self.points += [*self._xy(p0), *self._xy(p1), *self._xy(p2), *self._xy(p3)]
        return self

    def rat_quad(self, p0, p1, p2):
        """Each argument is (point, weight)."""
        self.kinds.append(abi.CMD_RAT_QUAD)
        for p, w in (p0, p1, p2):
            self.points += [*self._xy(p), float(w)]
        return self

    def rat_cubic(self, p0, p1, p2, p3):
        self.kinds.append(abi.CMD_RAT_CUBIC)
        for p, w in (p0, p1, p2, p3):
            self.points += [*self._xy(p), float(w)]
        return self

    def close(self):
        self.kinds.append(abi.CMD_CLOSE)
        return self

    def c_arrays(self):
        k = (ctypes.c_uint32 * max(1, len(self.kinds)))(*self.kinds)
        p = (ctypes.c_float * max(1, len(self.points)))(*self.points)
        return k, p


def transform_array(t: Optional[Sequence[float]], n: int):
    if t is None:
        return None
    if len(t) != n:
        raise ValueError(f"expected {n} transform values")
    return (ctypes.c_float * n)(*[float(v) for v in t])
