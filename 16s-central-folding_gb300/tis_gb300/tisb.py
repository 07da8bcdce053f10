"""Reader and writer for TISB record files (system, state, list and force dumps).

Layout: 8-byte magic ``TISB0001`` followed by records
``name[32] (NUL padded) | dtype[4] ("f8"/"i4"/"i8") | int64 count | data``.
"""
import numpy as np

_DT = {"f8": np.float64, "i4": np.int32, "i8": np.int64}


def read(path):
    out = {}
    with open(path, "rb") as f:
        if f.read(8) != b"TISB0001":
            raise ValueError(f"{path}: not a TISB file")
        while True:
            head = f.read(40)
            if len(head) < 40:
                break
            name = head[:32].split(b"\0", 1)[0].decode()
            dt = head[32:36].split(b"\0", 1)[0].decode()
            n = int(np.frombuffer(head[36:40] + f.read(4), dtype=np.int64)[0])
            arr = np.frombuffer(f.read(n * np.dtype(_DT[dt]).itemsize), dtype=_DT[dt]).copy()
            out[name] = arr
    return out


def write(path, records):
    with open(path, "wb") as f:
        f.write(b"TISB0001")
        for name, arr in records.items():
            arr = np.ascontiguousarray(arr)
            if arr.dtype == np.float64:
                dt = b"f8"
            elif arr.dtype == np.int32:
                dt = b"i4"
            elif arr.dtype == np.int64:
                dt = b"i8"
            else:
                raise TypeError(f"{name}: unsupported dtype {arr.dtype}")
            f.write(name.encode().ljust(32, b"\0")[:32])
            f.write(dt.ljust(4, b"\0"))
            f.write(np.int64(arr.size).tobytes())
            f.write(arr.reshape(-1).tobytes())
