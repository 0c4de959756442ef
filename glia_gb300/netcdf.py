"""netCDF classic-format fields and label maps: the reference's data-in path in front of the
reaction-diffusion solver.

- `read` / `write`: one 3-D variable ("data", dims x, y, z) in the classic netCDF format —
  CDF-1 (32-bit offsets), CDF-2 (64-bit offsets) and CDF-5 (64-bit data) are read; `write`
  produces CDF-2 with the reference's layout (dataIn / dataOut, src/utils/IO.cpp:511-652:
  variable "data", dims "x", "y", "z", NC_DOUBLE or NC_FLOAT, global attribute "CDF-5 mode").
  The format is the published netCDF classic specification (big-endian header of dimension,
  attribute and variable lists, then the variable data); no netCDF library is needed.
- `parse_labels`: the `atlas_labels` / `patient_labels` setting "[wm=6,gm=5,vt=7,csf=8,...]"
  (src/utils/IO.cpp:126-168) -> [wm, gm, vt, csf, tc, nec, en, ed], -1 where absent.
- `split_segmentation`: label map -> tissue probability maps (splitSegmentation,
  src/utils/Utils.cpp:592-658).
- `load_atlas`: read + split + the Weierstrass smoothing of SolverInterface::initializeAtlas-
  style set-up (src/SolverInterface.cpp:506-566), on a context of the CUDA library.
"""
from __future__ import annotations

import struct

import numpy as np

_TYPES = {1: ("b", 1), 2: ("S1", 1), 3: (">i2", 2), 4: (">i4", 4), 5: (">f4", 4), 6: (">f8", 8),
          7: ("u1", 1), 8: (">u2", 2), 9: (">u4", 4), 10: (">i8", 8), 11: (">u8", 8)}
_NC_DIMENSION, _NC_VARIABLE, _NC_ATTRIBUTE = 0x0A, 0x0B, 0x0C


class _Reader:
    def __init__(self, buf: bytes):
        self.b = buf
        self.o = 0
        if buf[:3] != b"CDF" or buf[3] not in (1, 2, 5):
            raise ValueError("not a classic netCDF file (magic CDF\\x01, \\x02 or \\x05)")
        self.version = buf[3]
        self.o = 4

    def i4(self):
        v = struct.unpack_from(">i", self.b, self.o)[0]
        self.o += 4
        return v

    def i8(self):
        v = struct.unpack_from(">q", self.b, self.o)[0]
        self.o += 8
        return v

    def count(self):  # NON_NEG: 4 bytes, 8 in CDF-5
        return self.i8() if self.version == 5 else self.i4()

    def offset(self):  # OFFSET: 4 bytes in CDF-1, 8 in CDF-2 and CDF-5
        return self.i4() if self.version == 1 else self.i8()

    def name(self):
        n = self.count()
        s = self.b[self.o:self.o + n].decode()
        self.o += (n + 3) // 4 * 4
        return s

    def values(self, nc_type, n):
        dt, size = _TYPES[nc_type]
        raw = self.b[self.o:self.o + n * size]
        self.o += (n * size + 3) // 4 * 4
        return np.frombuffer(raw, dtype=dt)

    def att_list(self):
        tag, n = self.i4(), self.count()
        if tag == 0:
            return {}
        if tag != _NC_ATTRIBUTE:
            raise ValueError("bad attribute list")
        out = {}
        for _ in range(n):
            nm = self.name()
            t = self.i4()
            out[nm] = self.values(t, self.count())
        return out


def read_header(buf: bytes):
    """(version, dims [(name, length)], global attributes, variables {name: dict})."""
    r = _Reader(buf)
    r.count()  # numrecs
    dims = []
    tag, n = r.i4(), r.count()
    if tag not in (0, _NC_DIMENSION):
        raise ValueError("bad dimension list")
    for _ in range(n if tag else 0):
        dims.append((r.name(), r.count()))
    gatts = r.att_list()
    tag, n = r.i4(), r.count()
    if tag not in (0, _NC_VARIABLE):
        raise ValueError("bad variable list")
    variables = {}
    for _ in range(n if tag else 0):
        nm = r.name()
        dimids = [r.count() for _ in range(r.count())]
        atts = r.att_list()
        t = r.i4()
        vsize = r.count()
        begin = r.offset()
        variables[nm] = {"dimids": dimids, "atts": atts, "type": t, "vsize": vsize,
                         "begin": begin, "shape": tuple(dims[d][1] for d in dimids)}
    return r.version, dims, gatts, variables


def read(path: str, var: str = "data") -> np.ndarray:
    """The variable `var` (default the reference's "data"; the only variable if there is one)
    as a float64 array in file order (x slowest)."""
    with open(path, "rb") as f:
        buf = f.read()
    _, dims, _, variables = read_header(buf)
    if var not in variables:
        if len(variables) != 1:
            raise KeyError(f"{path}: no variable {var!r} (have {sorted(variables)})")
        var = next(iter(variables))
    v = variables[var]
    if any(d == 0 for d in v["shape"]):
        raise ValueError("record variables are not supported")
    dt, size = _TYPES[v["type"]]
    count = int(np.prod(v["shape"]))
    raw = buf[v["begin"]:v["begin"] + count * size]
    return np.frombuffer(raw, dtype=dt).astype(np.float64).reshape(v["shape"])


def write(path: str, data: np.ndarray, single: bool = False, dims=("x", "y", "z")):
    """CDF-2 file with one variable "data" (NC_DOUBLE, or NC_FLOAT if `single`), the layout of
    the reference's dataOut."""
    data = np.asarray(data)
    if data.ndim != len(dims):
        raise ValueError("data rank must match dims")
    t = 5 if single else 6
    dt = ">f4" if single else ">f8"

    def name(s):
        b = s.encode()
        return struct.pack(">i", len(b)) + b + b"\0" * ((4 - len(b) % 4) % 4)

    head = b"CDF\x02" + struct.pack(">i", 0)
    head += struct.pack(">ii", _NC_DIMENSION, len(dims))
    for d, n in zip(dims, data.shape):
        head += name(d) + struct.pack(">i", n)
    head += struct.pack(">ii", _NC_ATTRIBUTE, 1) + name("CDF-5 mode") + struct.pack(">iii", 4, 1, 0)
    vsize = data.size * (4 if single else 8)
    var = name("data") + struct.pack(">i", len(dims))
    for i in range(len(dims)):
        var += struct.pack(">i", i)
    var += struct.pack(">ii", 0, 0)  # no variable attributes
    var += struct.pack(">ii", t, min(vsize, 2 ** 32 - 4))
    begin = len(head) + 8 + len(var) + 8
    var += struct.pack(">q", begin)
    out = head + struct.pack(">ii", _NC_VARIABLE, 1) + var + np.ascontiguousarray(data, dt).tobytes()
    with open(path, "wb") as f:
        f.write(out)


LABEL_KEYS = ("wm", "gm", "vt", "csf", "tc", "nec", "en", "ed")


def parse_labels(value: str) -> list:
    """"[wm=6,gm=5,vt=7,csf=8]" -> [6, 5, 7, 8, -1, -1, -1, -1] (keys wm gm vt csf tc nec en
    ed). As in src/utils/IO.cpp:126-168 a key must match exactly: unknown keys, and keys with
    surrounding spaces, are ignored."""
    body = value[value.find("[") + 1:]
    body = body[:body.find("]")] if "]" in body else body
    labels = [-1] * 8
    for item in body.split(","):
        if "=" not in item:
            continue
        k, v = item.split("=", 1)
        if k in LABEL_KEYS:
            labels[LABEL_KEYS.index(k)] = int(v)
    return labels


def split_segmentation(seg: np.ndarray, labels, with_csf=True, with_tumor=False,
                       with_edema=False) -> dict:
    """splitSegmentation (src/utils/Utils.cpp:592-658): indicator maps of the labelled tissues.
    Tumor labels (tc, or nec and en together) and edema count as white matter; `tu` / `ed`
    are returned when requested, as the reference fills them when its vectors exist."""
    seg = np.asarray(seg)
    wm_l, gm_l, vt_l = labels[0], labels[1], labels[2]
    csf_l, tc_l, nec_l, en_l, ed_l = (v if v > 0 else -1 for v in labels[3:8])
    out = {k: np.zeros(seg.shape) for k in ("wm", "gm", "vt")}
    if wm_l > 0:
        out["wm"][seg == wm_l] = 1
    if gm_l > 0:
        out["gm"][seg == gm_l] = 1
    if vt_l > 0:
        out["vt"][seg == vt_l] = 1
    if with_csf:
        out["csf"] = np.zeros(seg.shape)
        if csf_l > 0:
            out["csf"][seg == csf_l] = 1
    if with_tumor:
        out["tu"] = np.zeros(seg.shape)
        if tc_l > 0:
            m = seg == tc_l
        elif nec_l > 0 and en_l > 0:
            m = (seg == nec_l) | (seg == en_l)
        else:
            m = np.zeros(seg.shape, bool)
        out["wm"][m] = 1
        out["tu"][m] = 1
        if ed_l > 0:
            m = seg == ed_l
            out["wm"][m] = 1
            if with_edema:
                out["ed"] = np.zeros(seg.shape)
                out["ed"][m] = 1
    return out


def load_atlas(ctx, path: str, labels, smoothing_factor: float = 1.0) -> dict:
    """Label map from `path` -> tissue maps (split, then each map smoothed with the Weierstrass
    filter of width smoothing_factor * 2 pi / n when smoothing_factor > 0, as
    src/SolverInterface.cpp:506-566) -> glia_set_tissue on `ctx`. Returns the maps."""
    seg = read(path)
    n = seg.shape[0]
    if seg.shape != (n, n, n) or n != ctx.n:
        raise ValueError(f"{path}: shape {seg.shape}, context grid {ctx.n}^3")
    if min(labels[0], labels[1], labels[2]) <= 0:
        raise ValueError("wm, gm and vt labels are required")
    maps = split_segmentation(seg, labels, with_csf=True)
    if smoothing_factor > 0:
        sigma = smoothing_factor * 2 * np.pi / n
        for k in ("gm", "wm", "vt", "csf"):
            maps[k] = ctx.smooth(maps[k].reshape(-1), sigma).reshape(seg.shape)
    ctx.set_tissue(maps["wm"].reshape(-1), maps["gm"].reshape(-1), maps["csf"].reshape(-1),
                   maps["vt"].reshape(-1))
    return maps
