"""Reader for material bundles (.ncgb), the on-disk form of a material's
host-side loading results (see ncgb_export.cc for the producer and the record
layout).  Used by tests and tooling; the C++ loader in csrc/ncgb_bundle.cc is
the one the library itself uses."""
import struct

import numpy as np

_DT = {1: np.float64, 2: np.int64, 3: np.uint32}


def read_bundle(path):
    """Return {name: numpy array | str} for every record of a bundle file."""
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:8] != b"NCGBNDL1":
        raise ValueError(f"{path}: not a material bundle")
    (n,) = struct.unpack_from("<I", buf, 8)
    pos = 12
    out = {}
    for _ in range(n):
        (nl,) = struct.unpack_from("<I", buf, pos)
        pos += 4
        name = buf[pos:pos + nl].decode()
        pos += nl
        dt, cnt = struct.unpack_from("<IQ", buf, pos)
        pos += 12
        if dt == 4:
            out[name] = buf[pos:pos + cnt].decode()
            pos += cnt
        else:
            t = _DT[dt]
            sz = np.dtype(t).itemsize * cnt
            out[name] = np.frombuffer(buf, dtype=t, count=cnt, offset=pos).copy()
            pos += sz
    return out
