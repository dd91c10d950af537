"""Reader for the binary state dumps written by tests/drivers/dump.h.

Record: char name[64]; int32 kind (0 float32, 1 complex64, 2 float64,
3 complex128); int32 n0, n1, n2; then the elements in C order.
"""
import numpy as np

_DT = {0: np.float32, 1: np.complex64, 2: np.float64, 3: np.complex128}


def read_dump(path):
    out = {}
    with open(path, "rb") as f:
        buf = f.read()
    pos = 0
    while pos < len(buf):
        name = buf[pos:pos + 64].split(b"\0", 1)[0].decode()
        kind, n0, n1, n2 = np.frombuffer(buf, dtype="<i4", count=4, offset=pos + 64)
        pos += 80
        dt = np.dtype(_DT[int(kind)])
        count = int(n0) * int(n1) * int(n2)
        arr = np.frombuffer(buf, dtype=dt, count=count, offset=pos).reshape(int(n0), int(n1), int(n2))
        pos += count * dt.itemsize
        out[name] = arr.copy()
    return out
