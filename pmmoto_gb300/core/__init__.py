"""Single-rank geometry: boundary kinds, the padded subdomain, initialize()."""

from .boundary_types import BoundaryType  # noqa: F401
from .subdomain import PaddedSubdomain, initialize  # noqa: F401
from . import geometry  # noqa: F401

__all__ = ["BoundaryType", "PaddedSubdomain", "initialize", "geometry"]
