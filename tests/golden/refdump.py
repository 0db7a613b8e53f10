"""Reader for ref_dump.bin, the state dump of the reference program built for
the CPU by oracle/ref_build.py (see oracle/ref_harness.cpp for the format)."""
import struct

import numpy as np


def read_dump(path) -> dict:
    out = {}
    with open(path, "rb") as f:
        while True:
            head = f.read(41)
            if len(head) < 41:
                break
            name = head[:32].split(b"\0", 1)[0].decode()
            typ = chr(head[32])
            (count,) = struct.unpack("<q", head[33:41])
            dt = {"f": np.float32, "i": np.int32, "d": np.float64}[typ]
            out[name] = np.frombuffer(f.read(count * np.dtype(dt).itemsize), dtype=dt).copy()
    return out
