"""Reader for the VTK XML UnstructuredGrid files the project writes (appended
raw data, UInt64 headers, optionally zlib-compressed blocks in VTK's layout),
used by the tests to check the files' content."""
import re
import zlib

import numpy as np

_TYPES = {"Float64": np.float64, "Float32": np.float32, "Int64": np.int64, "Int32": np.int32, "UInt8": np.uint8}


def read_vtu(path):
    """{'points', 'connectivity', 'offsets', 'types', <cell array name>...,
    'compressed'} as numpy arrays."""
    raw = open(path, "rb").read()
    start = raw.index(b"<AppendedData")
    head = raw[:start].decode("utf-8")
    assert 'header_type="UInt64"' in head
    compressed = "vtkZLibDataCompressor" in head
    data = raw[raw.index(b"_", start) + 1:]
    npts = int(re.search(r'NumberOfPoints="(\d+)"', head).group(1))
    ncells = int(re.search(r'NumberOfCells="(\d+)"', head).group(1))

    def block(off):
        if not compressed:
            n = int(np.frombuffer(data, np.uint64, 1, off)[0])
            return data[off + 8:off + 8 + n]
        nb, bs, last = (int(x) for x in np.frombuffer(data, np.uint64, 3, off))
        sizes = np.frombuffer(data, np.uint64, nb, off + 24).astype(np.int64)
        pos = off + 24 + 8 * nb
        out = []
        for k, cs in enumerate(sizes):
            chunk = zlib.decompress(data[pos:pos + cs])
            assert len(chunk) == (last if k == nb - 1 else bs)
            out.append(chunk)
            pos += cs
        return b"".join(out)

    out = {"compressed": compressed, "n_points": npts, "n_cells": ncells}
    for m in re.finditer(r"<DataArray ([^>]*)/>", head):
        attrs = dict(re.findall(r'(\w+)="([^"]*)"', m.group(1)))
        arr = np.frombuffer(block(int(attrs["offset"])), _TYPES[attrs["type"]])
        ncomp = int(attrs.get("NumberOfComponents", "1"))
        if ncomp > 1:
            arr = arr.reshape(-1, ncomp)
        out[attrs.get("Name", "points")] = arr
    return out
