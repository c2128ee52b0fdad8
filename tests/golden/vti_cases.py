"""Seeded inputs of the image-writer fixtures (shared by make_golden.py and
the tests): each case is (name, initialize kwargs, {image name: array})."""

from __future__ import annotations

import numpy as np


def cases():
    rng = np.random.default_rng(2024)
    out = []
    out.append(("u8_default_box", dict(voxels=(4, 3, 2)),
                {"img": np.arange(24, dtype=np.uint8).reshape(4, 3, 2)}))
    vox = (6, 5, 4)
    box = ((0.0, 2.0), (1.0, 3.0), (-1.5, 0.5))
    out.append(("f64_box_extra", dict(voxels=vox, box=box),
                {"img": rng.random(vox),
                 "labels": rng.integers(0, 2**40, vox, dtype=np.uint64),
                 "dist": rng.random(vox).astype(np.float32),
                 "a_phase": rng.integers(-5, 5, vox, dtype=np.int32)}))
    vox = (8, 7, 9)
    out.append(("i64_periodic", dict(voxels=vox, box=((0, 1.0), (0, 1.0), (0, 1)),
                                      boundary_types="periodic"),
                {"img": rng.integers(-(2**40), 2**40, vox, dtype=np.int64),
                 "mask": rng.integers(0, 2, vox, dtype=np.uint8)}))
    return out
