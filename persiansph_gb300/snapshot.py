"""Reader of the snapshots Solve writes (the reference's WriteXDMF output,
Source/Domain.cpp:1869-2064, as <key>.xmf + <key>.bin).

The .bin holds the reference's HDF5 datasets back to back: NP, Position,
Velocity, Acceleration, Tag, Pressure, Density, the three OutputName
properties, Mass, h, Sigma, Strain (float32; NP and Tag int32; little
endian). The .xmf describes them for a viewer (each DataItem at its byte
offset). `read_snapshot` returns every dataset as a numpy array keyed by its
name (the properties under their OutputName; vectors (n, 3); Sigma and Strain
(n, 6), components 00 01 02 11 12 22) and checks the .xmf offsets against the
layout.
"""
from __future__ import annotations

import os
import xml.etree.ElementTree as ET

import numpy as np

# (name, values per particle, int32); None: the k-th OutputName property
LAYOUT = (("Position", 3, False), ("Velocity", 3, False), ("Acceleration", 3, False), ("Tag", 1, True),
          ("Pressure", 1, False), ("Density", 1, False), (None, 1, False), (None, 1, False), (None, 1, False),
          ("Mass", 1, False), ("h", 1, False), ("Sigma", 6, False), ("Strain", 6, False))


def read_snapshot(key: str) -> dict:
    """Datasets of <key>.bin, named as in <key>.xmf (key without extension)."""
    root = ET.parse(key + ".xmf").getroot()
    grid = root.find("Domain").find("Grid")
    attrs = grid.findall("Attribute")
    prop_names = [a.get("Name") for a in attrs[6:9]]
    seeks = {a.get("Name"): int(a.find("DataItem").get("Seek")) for a in attrs}
    with open(key + ".bin", "rb") as f:
        raw = f.read()
    n = int(np.frombuffer(raw[:4], "<i4")[0])
    out = {"NP": n}
    off = 4
    k_prop = 0
    for name, width, is_int in LAYOUT:
        if name is None:
            name = prop_names[k_prop]
            k_prop += 1
        arr = np.frombuffer(raw, dtype="<i4" if is_int else "<f4", count=n * width, offset=off)
        out[name] = arr.reshape(n, width) if width > 1 else arr
        if name in seeks and seeks[name] != off:
            raise ValueError(f"{key}.xmf: {name} at byte {seeks[name]}, the file has it at {off}")
        off += 4 * n * width
    if off != len(raw):
        raise ValueError(f"{key}.bin: {len(raw)} bytes, the layout needs {off}")
    return out
