"""SEP datasets from Python: a text header of name=value pairs plus a binary
file of 4-byte floats named by the header's in= (big-endian for
data_format="xdr_float", the default, little-endian for "native_float").

The same format the command-line programs (seismic_gb300/cli) read and
write; arrays are returned with axis 1 fastest, i.e. shape (..., n2, n1).
"""
from __future__ import annotations

import os
import re

import numpy as np

# A name=value word: the name starts a blank-separated word.
_PAIR = re.compile(r"""(?:^|(?<=\s))([A-Za-z0-9_.\-]+)=("[^"\n]*"|'[^'\n]*'|\S+)""")


def parse_header(text: str) -> dict[str, str]:
    """name=value pairs of a header; a later definition wins."""
    out: dict[str, str] = {}
    for k, v in _PAIR.findall(text):
        if v[:1] in "\"'" and v[-1:] == v[:1]:
            v = v[1:-1]
        out[k] = v
    return out


def read(path: str) -> tuple[np.ndarray, dict[str, str]]:
    """Returns (samples shaped (..., n2, n1), header)."""
    with open(path, "rb") as f:
        raw = f.read()
    mark = raw.find(b"\x0c\x04")
    text = (raw[:mark] if mark >= 0 else raw).decode("latin-1")
    h = parse_header(text)
    dims = []
    for a in range(1, 10):
        n = int(float(h.get(f"n{a}", "1")))
        dims.append(n)
    while len(dims) > 1 and dims[-1] == 1:
        dims.pop()
    count = int(np.prod(dims))
    fmt = h.get("data_format", "xdr_float")
    if fmt not in ("xdr_float", "native_float"):
        raise ValueError(f"{path}: unsupported data_format {fmt}")
    dt = np.dtype(">f4" if fmt == "xdr_float" else "<f4")
    src = h.get("in")
    if src is None or src == "stdin":
        if mark < 0:
            raise ValueError(f"{path}: no in= and no embedded samples")
        data = np.frombuffer(raw[mark + 2:], dtype=dt, count=count)
    else:
        if not os.path.isabs(src) and not os.path.exists(src):
            src = os.path.join(os.path.dirname(path), src)
        data = np.fromfile(src, dtype=dt, count=count)
        if data.size != count:
            raise ValueError(f"{path}: {data.size} samples in {src}, header promises {count}")
    return data.astype(np.float32).reshape(dims[::-1]), h


def write(path: str, data, axes: dict[str, float | int] | None = None,
          data_format: str = "xdr_float", program: str = "seismic_gb300.sep") -> str:
    """Writes data (shape (..., n2, n1)) to path + "@" with a header at path.
    n1.. are taken from the array's shape unless given in `axes`; other
    `axes` entries (o1, d1, ...) are written as they are."""
    a = np.ascontiguousarray(data, np.float32)
    hdr: dict[str, float | int | str] = {}
    for i, n in enumerate(a.shape[::-1], start=1):
        hdr[f"n{i}"] = int(n)
    hdr.update(axes or {})
    bin_path = path + "@"
    dt = ">f4" if data_format == "xdr_float" else "<f4"
    a.astype(dt).tofile(bin_path)
    lines = [f"\n{program}:", f'\t\tin="{bin_path}"', "\t\tesize=4",
             f'\t\tdata_format="{data_format}"']
    lines += [f"\t\t{k}={v}" for k, v in hdr.items()]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path


def command(program: str, **params) -> list[str]:
    """argv for a command-line program: name=value words."""
    return [program] + [f"{k}={v}" for k, v in params.items()]
