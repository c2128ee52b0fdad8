"""Boundary kinds (src/pmmoto/core/boundary_types.py:11-17).

Values are the reference's strings, so a ``pmmoto.BoundaryType`` member and
this one compare equal by ``.value`` and either may be passed in.
"""

from enum import Enum


class BoundaryType(str, Enum):
    """Allowable boundary types."""

    END = "end"
    WALL = "wall"
    PERIODIC = "periodic"
    INTERNAL = "internal"


def bt_value(b) -> str:
    """String value of a boundary kind given as either enum or string."""
    return str(getattr(b, "value", b))


def boundary_order(boundaries) -> BoundaryType:
    """Kind of an edge or corner from its faces (boundary_types.py:20-37)."""
    vals = [bt_value(b) for b in boundaries]
    if "end" in vals:
        return BoundaryType.END
    if "wall" in vals:
        return BoundaryType.WALL
    return BoundaryType.PERIODIC
