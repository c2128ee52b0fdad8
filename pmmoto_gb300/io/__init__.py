"""File input for the sphere packs (``pmmoto.io.data_read``)."""

from .data_read import read_sphere_pack_xyzr_domain  # noqa: F401

__all__ = ["read_sphere_pack_xyzr_domain"]
