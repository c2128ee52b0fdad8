"""Image output as VTK XML ImageData (``pmmoto.io.output.save_img``).

Mirrors ``save_img`` / ``_save_img`` of src/pmmoto/io/output.py:133-262 for a
single subdomain: the image and any additional images of the same shape are
written as cell data of one ``<file_name>.vti`` file in the reference's
layout -- XML header, arrays in sorted name order with the first as the
active scalars, raw appended data with a little-endian UInt64 byte count in
front of each array, values in Fortran (x fastest) order.  Number fields are
printed as Python's ``repr`` of the values the reference holds: the box's
lower corner as it was given to ``initialize`` and the voxel size as a
float64 scalar.  Host-side file I/O only; device tensors are copied to the
host first.
"""

from __future__ import annotations

import os

import numpy as np

__all__ = ["save_img"]

# numpy dtype -> VTK XML type name (the VTK file format's names)
_VTK_TYPES = {
    np.dtype(np.int8): "Int8",
    np.dtype(np.uint8): "UInt8",
    np.dtype(np.int16): "Int16",
    np.dtype(np.uint16): "UInt16",
    np.dtype(np.int32): "Int32",
    np.dtype(np.uint32): "UInt32",
    np.dtype(np.int64): "Int64",
    np.dtype(np.uint64): "UInt64",
    np.dtype(np.float32): "Float32",
    np.dtype(np.float64): "Float64",
}


def _host(a):
    if hasattr(a, "detach") and hasattr(a, "cpu"):
        return a.detach().cpu().numpy()
    return a


def _fields(values) -> str:
    return "".join(repr(v) + " " for v in values)


def _check_file_path(file_name: str) -> None:
    """io_utils.check_file_path(file_name, create_folder=False): make the
    file's folder if it is missing."""
    d = os.path.dirname(file_name)
    if d and not os.path.isdir(d):
        os.makedirs(d)


def save_img(file_name: str, subdomain, img, additional_img=None, **kwargs) -> None:
    """Save ``img`` (and ``additional_img``, a dict name -> array of the same
    shape) of ``subdomain`` as ``<file_name>.vti``.

    Raises TypeError for an additional image that is not an array and
    ValueError for one whose shape differs from ``img`` (output.py:238-253).
    """
    if isinstance(subdomain, dict) or isinstance(img, dict):
        raise NotImplementedError("save_img: one subdomain per process (no decomposed image sets)")
    if subdomain.domain.num_subdomains > 1:
        raise NotImplementedError("save_img: one subdomain per process (no parallel .pvti output)")
    _check_file_path(file_name)
    img = _host(img)
    data = {"img": np.asarray(img)}
    if additional_img is not None:
        for key, value in additional_img.items():
            value = _host(value)
            if not isinstance(value, np.ndarray):
                raise TypeError(f"Expected numpy array for {key}, but got {type(value)}")
            if value.shape != data["img"].shape:
                raise ValueError(f"Invalid img size! {key} has shape {value.shape}. "
                                 f"Required shape is {data['img'].shape} ")
            data[key] = value
    start = [int(s) for s in subdomain.start]
    end = [s + int(v) for s, v in zip(start, subdomain.voxels)]
    extent = " ".join(f"{s} {e}" for s, e in zip(start, end))
    origin = [subdomain.domain.box_input[d][0] for d in range(3)]
    spacing = [np.float64(r) for r in subdomain.domain.resolution]
    names = sorted(data)
    arrays, lines, offset = [], [], 0
    for name in names:
        a = np.asarray(data[name])
        if a.dtype not in _VTK_TYPES:
            raise TypeError(f"save_img: dtype {a.dtype} of {name} has no VTK type")
        raw = np.ascontiguousarray(a.reshape(a.shape, order="C").ravel(order="F")).tobytes()
        lines.append(f'<DataArray Name="{name}" NumberOfComponents="1" type="{_VTK_TYPES[a.dtype]}" '
                     f'format="appended" offset="{offset}"/>\n')
        arrays.append(np.uint64(len(raw)).astype("<u8").tobytes() + raw)
        offset += 8 + len(raw)
    head = ('<?xml version="1.0"?>\n'
            '<VTKFile type="ImageData" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n'
            f'<ImageData WholeExtent="{extent}" Origin="{_fields(origin)}" Spacing="{_fields(spacing)}">\n'
            f'<Piece Extent="{extent}">\n'
            f'<CellData scalars="{names[0]}">\n' + "".join(lines) +
            '</CellData>\n</Piece>\n</ImageData>\n<AppendedData encoding="raw">\n_')
    with open(file_name + ".vti", "wb") as f:
        f.write(head.encode("ascii"))
        for a in arrays:
            f.write(a)
        f.write(b'\n</AppendedData>\n</VTKFile>')
