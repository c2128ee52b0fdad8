"""read_sphere_pack_xyzr_domain (src/pmmoto/io/data_read.py:26-84)."""

from __future__ import annotations

import logging
import os

import numpy as np

__all__ = ["read_sphere_pack_xyzr_domain"]

logger = logging.getLogger(__name__)


def read_sphere_pack_xyzr_domain(input_file: str):
    """Sphere pack file: three lines "min max" (x, y, z), then one
    "x y z r" line per sphere.  Returns (spheres (N, 4) float64, domain box
    ((x_min, x_max), (y_min, y_max), (z_min, z_max)))."""
    if not os.path.isfile(input_file):
        # io_utils.check_file logs and exits through utils.raise_error
        logger.error("%s does not exist!", input_file)
        raise SystemExit(1)
    with open(input_file, "r", encoding="utf-8") as f:
        lines = f.readlines()
    num_spheres = len(lines) - 3
    sphere_data = np.zeros([num_spheres, 4], dtype=np.double)
    domain_data = np.zeros([3, 2], dtype=np.double)
    count = 0
    for n_line, line in enumerate(lines):
        if n_line < 3:
            domain_data[n_line, 0] = float(line.split(" ")[0])
            domain_data[n_line, 1] = float(line.split(" ")[1])
        else:
            parts = line.split()
            if len(parts) != 4:
                raise ValueError(f"Invalid sphere line (expected 4 values): {line.strip()}")
            try:
                sphere_data[count] = [float(p) for p in parts]
            except ValueError as exc:
                raise ValueError(f"Non-numeric value in sphere line: {line.strip()}") from exc
            count += 1
    return sphere_data, tuple(map(tuple, domain_data))
