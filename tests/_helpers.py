"""Small helpers shared by the tests."""


def geom_from_meta(mod, m):
    """Build a single-rank geometry from a golden_meta.json entry with
    ``mod.Geom`` (the oracle's) -- keyword names follow pmmoto.initialize."""
    return mod.Geom(tuple(m["voxels"]), boundary_types=tuple(tuple(b) for b in m["boundary_types"]),
                    box=tuple(tuple(b) for b in m["box"]), inlet=tuple(tuple(bool(x) for x in i) for i in m["inlet"]),
                    outlet=tuple(tuple(bool(x) for x in o) for o in m["outlet"]),
                    reservoir_voxels=m["reservoir_voxels"])


def sd_from_meta(m):
    """The package's own subdomain for a golden_meta.json geometry entry."""
    from pmmoto_gb300.core import initialize

    return initialize(tuple(m["voxels"]), box=tuple(tuple(b) for b in m["box"]),
                      boundary_types=tuple(tuple(b) for b in m["boundary_types"]),
                      inlet=tuple(tuple(bool(x) for x in i) for i in m["inlet"]),
                      outlet=tuple(tuple(bool(x) for x in o) for o in m["outlet"]),
                      reservoir_voxels=m["reservoir_voxels"])
