"""Minimal reader for the VTK XML ImageData files the CLI writes (appended raw data)."""
import re

import numpy as np

_TYPES = {"UInt8": np.uint8, "UInt16": np.uint16, "Float32": np.float32, "Float64": np.float64}


def read_vti(path):
    data = open(path, "rb").read()
    head_end = data.index(b"<AppendedData")
    head = data[:head_end].decode()
    ext = [int(v) for v in re.search(r'WholeExtent="([^"]+)"', head).group(1).split()]
    I, J, K = ext[1] + 1, ext[3] + 1, ext[5] + 1
    start = data.index(b"_", head_end) + 1
    arrays = {}
    for m in re.finditer(r'<DataArray type="(\w+)" Name="(\w+)"(?: NumberOfComponents="(\d)")? '
                         r'format="appended" offset="(\d+)"/>', head):
        typ, name, ncomp, off = m.group(1), m.group(2), int(m.group(3) or 1), int(m.group(4))
        pos = start + off
        nbytes = int(np.frombuffer(data[pos:pos + 8], dtype=np.uint64)[0])
        arr = np.frombuffer(data[pos + 8:pos + 8 + nbytes], dtype=_TYPES[typ])
        # VTK point order is i fastest: reshape to (K, J, I[, c]) and transpose to (I, J, K)
        if ncomp == 1:
            arrays[name] = arr.reshape(K, J, I).transpose(2, 1, 0)
        else:
            arrays[name] = arr.reshape(K, J, I, ncomp).transpose(2, 1, 0, 3)
    return (I, J, K), arrays
