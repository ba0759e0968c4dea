"""A small reader of the VTU files the frame writers produce (ASCII and binary
appended raw data with UInt64 or UInt32 headers): {array name: numpy array},
the point coordinates under "Points", the field data TIME and STEP as
numbers."""
from __future__ import annotations

import re

import numpy as np

_TYPES = {"Float32": "<f4", "Float64": "<f8", "Int32": "<i4", "Int64": "<i8", "UInt8": "u1", "UInt32": "<u4",
          "UInt64": "<u8"}


def read_vtu(path):
    raw = open(path, "rb").read()
    cut = raw.find(b"<AppendedData")
    head = raw[: cut if cut >= 0 else len(raw)].decode()
    base = raw.index(b"_", cut) + 1 if cut >= 0 else None
    header_type = re.search(r'header_type="(\w+)"', head)
    hdt = np.dtype(_TYPES[header_type.group(1)] if header_type else "<u4")
    out = {"_header": head}
    points = (head.find("<Points>"), head.find("</Points>"))
    for m in re.finditer(r"<DataArray([^>]*?)(/?)>", head):
        attrs = dict(re.findall(r'(\w+)="([^"]*)"', m.group(1)))
        name = attrs.get("Name") or ("Points" if points[0] < m.start() < points[1] else "?")
        dt = np.dtype(_TYPES[attrs["type"]])
        comps = int(attrs.get("NumberOfComponents", "1"))
        if attrs.get("format") == "appended":
            at = base + int(attrs["offset"])
            nbytes = int(np.frombuffer(raw, dtype=hdt, count=1, offset=at)[0])
            a = np.frombuffer(raw, dtype=dt, count=nbytes // dt.itemsize, offset=at + hdt.itemsize).copy()
        else:
            end = head.index("</DataArray>", m.end())
            a = np.array(head[m.end():end].split(), dtype=dt)
        out[name] = a.reshape(-1, comps) if comps > 1 else a
    for k in ("TIME", "STEP"):
        if k in out and len(out[k]) == 1:
            out[k] = out[k][0].item()
    return out
