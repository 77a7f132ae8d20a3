"""NetCDF classic-format files (CDF-1 and CDF-2), read and written with numpy.

The reference keeps its grid and its lat-lon index map in netCDF files written through the
netCDF4 package (plot.py:477-703), which this image does not have.  This module writes the
classic format of the netCDF specification (header of dimensions, attributes and variables,
then each variable's values big-endian, padded to 4 bytes), which netCDF4 and every other
netCDF reader open, and reads classic files (fixed and record variables).  Files in the HDF5-based
netCDF-4 format are recognised and refused.

    write(path, dims, variables, attrs=None, version=2)
        dims: {name: length}; variables: [(name, array, dim_names)] (dim_names () for a scalar);
        attrs: global attributes {name: str | number | array}
    read(path) -> Dataset with .dims, .variables {name: ndarray}, .attrs
"""
import struct

import numpy as np

_ABSENT = b"\0" * 8
_DIMENSION, _VARIABLE, _ATTRIBUTE = 10, 11, 12
# nc_type codes of the specification and their big-endian numpy types
_TYPES = {1: ">i1", 2: "S1", 3: ">i2", 4: ">i4", 5: ">f4", 6: ">f8"}
_CODES = {np.dtype("int8"): 1, np.dtype("int16"): 3, np.dtype("int32"): 4, np.dtype("float32"): 5,
          np.dtype("float64"): 6}
_HDF5_MAGIC = b"\x89HDF\r\n\x1a\n"


def _pad4(n):
    return (4 - n % 4) % 4


def _name(s):
    b = s.encode("utf-8")
    return struct.pack(">i", len(b)) + b + b"\0" * _pad4(len(b))


def _attr_values(v):
    if isinstance(v, str):
        b = v.encode("utf-8")
        return 2, len(b), b + b"\0" * _pad4(len(b))
    a = np.atleast_1d(np.asarray(v))
    if a.dtype.kind == "f":
        a = a.astype(np.float64)
    elif a.dtype.kind in "iu":
        a = a.astype(np.int32)
    code = _CODES[a.dtype]
    b = a.astype(_TYPES[code]).tobytes()
    return code, a.size, b + b"\0" * _pad4(len(b))


def _att_list(attrs):
    if not attrs:
        return _ABSENT
    out = struct.pack(">ii", _ATTRIBUTE, len(attrs))
    for k, v in attrs.items():
        code, n, b = _attr_values(v)
        out += _name(k) + struct.pack(">ii", code, n) + b
    return out


def write(path, dims, variables, attrs=None, version=2):
    """Write a classic netCDF file (version 1: 32-bit offsets, 2: 64-bit offsets)."""
    if version not in (1, 2):
        raise ValueError("version must be 1 or 2")
    dnames = list(dims)
    prepared = []
    for name, data, vdims in variables:
        a = np.asarray(data)
        if a.dtype.kind == "f" and a.dtype != np.float32:
            a = a.astype(np.float64)
        elif a.dtype.kind in "iub" and a.dtype not in (np.dtype("int8"), np.dtype("int16")):
            a = a.astype(np.int32)
        shape = tuple(dims[d] for d in vdims)
        if a.shape != shape:
            raise ValueError("variable %s: shape %s, dimensions give %s" % (name, a.shape, shape))
        if any(dims[d] == 0 for d in vdims):
            raise ValueError("record (unlimited) dimensions are not written")
        prepared.append((name, [dnames.index(d) for d in vdims], _CODES[a.dtype], a))
    head = b"CDF" + bytes([version]) + struct.pack(">i", 0)
    if dims:
        head += struct.pack(">ii", _DIMENSION, len(dims))
        for d in dnames:
            head += _name(d) + struct.pack(">i", dims[d])
    else:
        head += _ABSENT
    head += _att_list(attrs)
    osize = 4 if version == 1 else 8
    # variable entries, then the offsets once the header length is known
    entries = []
    for name, ids, code, a in prepared:
        e = _name(name) + struct.pack(">i", len(ids)) + b"".join(struct.pack(">i", i) for i in ids)
        e += _ABSENT + struct.pack(">i", code)
        nb = a.size * a.dtype.itemsize
        vsize = min(nb + _pad4(nb), 2**32 - 1)
        entries.append((e + struct.pack(">I", vsize), a, nb))
    hlen = len(head) + 8 + sum(len(e) + osize for e, _, _ in entries)  # + the variable list's tag and count
    out = [head]
    out.append(struct.pack(">ii", _VARIABLE, len(prepared)) if prepared else _ABSENT)
    begin = hlen
    for e, _, nb in entries:
        if version == 1 and begin >= 2**31:
            raise ValueError("data past 2 GiB: use version 2")
        out.append(e + (struct.pack(">i", begin) if version == 1 else struct.pack(">q", begin)))
        begin += nb + _pad4(nb)
    with open(path, "wb") as f:
        f.write(b"".join(out))
        for _, a, nb in entries:  # one variable at a time, big-endian
            f.write(np.ascontiguousarray(a).astype(_TYPES[_CODES[a.dtype]]).tobytes())
            f.write(b"\0" * _pad4(nb))


class Dataset:
    """Contents of a classic netCDF file: dims {name: length}, variables {name: ndarray},
    attrs (global) and var_attrs {variable: {name: value}}."""

    def __init__(self, dims, variables, attrs, var_attrs):
        self.dims, self.variables, self.attrs, self.var_attrs = dims, variables, attrs, var_attrs

    def __getitem__(self, name):
        return self.variables[name]


class _Reader:
    def __init__(self, buf):
        self.b, self.o = buf, 0

    def int(self):
        v = struct.unpack_from(">i", self.b, self.o)[0]
        self.o += 4
        return v

    def uint(self):
        v = struct.unpack_from(">I", self.b, self.o)[0]
        self.o += 4
        return v

    def name(self):
        n = self.int()
        s = self.b[self.o:self.o + n].decode("utf-8")
        self.o += n + _pad4(n)
        return s

    def values(self, code, n):
        dt = np.dtype(_TYPES[code])
        nb = dt.itemsize * n
        raw = self.b[self.o:self.o + nb]
        self.o += nb + _pad4(nb)
        if code == 2:
            return raw.rstrip(b"\0").decode("utf-8", "replace")
        v = np.frombuffer(raw, dtype=dt).astype(dt.newbyteorder("="))
        return v[0] if n == 1 else v

    def atts(self):
        tag, n = self.int(), self.int()
        if tag == 0 and n == 0:
            return {}
        if tag != _ATTRIBUTE:
            raise ValueError("malformed attribute list")
        out = {}
        for _ in range(n):
            k = self.name()
            code, m = self.int(), self.int()
            out[k] = self.values(code, m)
        return out


def read(path):
    """Read a classic (CDF-1 or CDF-2) netCDF file."""
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:8] == _HDF5_MAGIC:
        raise ValueError("%s is an HDF5-based netCDF-4 file; only the classic format is read here" % path)
    if buf[:3] != b"CDF" or buf[3] not in (1, 2):
        raise ValueError("%s is not a classic netCDF file" % path)
    osize = 4 if buf[3] == 1 else 8
    r = _Reader(buf)
    r.o = 4
    numrecs = r.int()
    tag, n = r.int(), r.int()
    dims = {}
    if not (tag == 0 and n == 0):
        if tag != _DIMENSION:
            raise ValueError("malformed dimension list")
        for _ in range(n):
            k = r.name()
            dims[k] = r.int()
    dnames = list(dims)
    attrs = r.atts()
    tag, n = r.int(), r.int()
    specs = []
    if not (tag == 0 and n == 0):
        if tag != _VARIABLE:
            raise ValueError("malformed variable list")
        for _ in range(n):
            name = r.name()
            nd = r.int()
            ids = [r.int() for _ in range(nd)]
            vatts = r.atts()
            code = r.int()
            vsize = r.uint()
            begin = struct.unpack_from(">i" if osize == 4 else ">q", buf, r.o)[0]
            r.o += osize
            specs.append((name, ids, vatts, code, vsize, begin))
    rec = [s for s in specs if s[1] and dims[dnames[s[1][0]]] == 0]
    if len(rec) == 1:  # a lone record variable's records follow one another unpadded
        name, ids, _, code, _, _ = rec[0]
        recsize = int(np.prod([dims[dnames[i]] for i in ids[1:]], dtype=np.int64)) * np.dtype(_TYPES[code]).itemsize
    else:
        recsize = sum(s[4] for s in rec)
    variables, var_attrs = {}, {}
    for name, ids, vatts, code, vsize, begin in specs:
        dt = np.dtype(_TYPES[code]) if code != 2 else np.dtype("S1")
        shape = [dims[dnames[i]] for i in ids]
        if ids and shape[0] == 0:  # record variable: one slab per record
            shape[0] = numrecs
            per = int(np.prod(shape[1:], dtype=np.int64)) * dt.itemsize
            slabs = [buf[begin + k * recsize:begin + k * recsize + per] for k in range(numrecs)]
            raw = b"".join(slabs)
        else:
            nb = int(np.prod(shape, dtype=np.int64)) * dt.itemsize
            raw = buf[begin:begin + nb]
        a = np.frombuffer(raw, dtype=dt).reshape(shape)
        variables[name] = a.astype(dt.newbyteorder("=")) if code != 2 else a.copy()
        var_attrs[name] = vatts
    return Dataset(dims, variables, attrs, var_attrs)
