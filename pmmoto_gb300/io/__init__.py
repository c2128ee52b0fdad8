"""File input for the sphere packs (``pmmoto.io.data_read``) and image
output (``pmmoto.io.output``)."""

from . import output  # noqa: F401
from .data_read import read_sphere_pack_xyzr_domain  # noqa: F401
from .output import save_img  # noqa: F401

__all__ = ["read_sphere_pack_xyzr_domain", "save_img", "output"]
