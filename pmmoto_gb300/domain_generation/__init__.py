"""GPU drop-ins for ``pmmoto.domain_generation`` (sphere packs, porous media,
multiphase images)."""

from . import domain_generation, multiphase, porousmedia  # noqa: F401
from .domain_generation import gen_mp_constant, gen_pm_shape, gen_pm_spheres_domain  # noqa: F401
from .multiphase import Multiphase  # noqa: F401
from .porousmedia import PorousMedia, gen_pm  # noqa: F401

__all__ = ["gen_pm_spheres_domain", "gen_pm_shape", "gen_mp_constant", "Multiphase", "PorousMedia", "gen_pm",
           "domain_generation", "multiphase", "porousmedia"]
