"""stablebear's binary file format for the results of the pairwise path.

``save`` / ``load`` read and write the same bytes as the reference's
``stablebear.save`` / ``stablebear.load`` (``stablebear/io.py:162-203``), so a
result saved by either library loads in the other:

* header (``include/sbear/io.hpp:127-160``): the five bytes ``"\\x01MPCF"``,
  the endianness byte ``"e"``, an ``int32`` format version (2), then three
  strings (``u64`` length + bytes): library version, build date, and (version
  2 only) platform.  Readers skip the strings.
* a ``u32`` format type: 1 single tensor, 2 single object (``io.hpp:165-169``).
* an object (``io.hpp:260-270``): ``int32`` base format and sub format
  (``io/tensor_io.hpp:96-128``: SymmetricMatrix 1100, DistanceMatrix 1120;
  sub format 32 or 64), then the matrix body
  (``io/compressed_matrix_io.hpp:10-32``): ``u64`` n and the condensed storage.
* a tensor of floats (``io/tensor_io.hpp:171-195``, ``io.hpp:188-194``):
  base/sub format (1, 32|64), ``u64`` rank, per axis ``u64`` extent and
  ``u64`` stride (elements, row-major), then the values.  ``cdist`` results
  are such tensors.

Only what the pairwise path produces is handled: DistanceMatrix,
SymmetricMatrix and float32/float64 arrays.  Other stablebear objects raise
``TypeError``.
"""
from __future__ import annotations

import io as _io
import platform as _platform
import struct
import time as _time

import numpy as np

from .matrices import DistanceMatrix, SymmetricMatrix

HEADER_ID = b"\x01MPCF"
FORMAT_VERSION = 2
SINGLE_TENSOR = 1
SINGLE_OBJECT = 2
_MAX_STRING = 32767

# (base format, sub format) of each object type, and back
_OBJECT_FORMATS = {
    (SymmetricMatrix, np.dtype(np.float32)): (1100, 32),
    (SymmetricMatrix, np.dtype(np.float64)): (1100, 64),
    (DistanceMatrix, np.dtype(np.float32)): (1120, 32),
    (DistanceMatrix, np.dtype(np.float64)): (1120, 64),
}
_OBJECT_TYPES = {v: k for k, v in _OBJECT_FORMATS.items()}
_SCALAR_FORMATS = {np.dtype(np.float32): (1, 32), np.dtype(np.float64): (1, 64)}
_SCALAR_TYPES = {v: k for k, v in _SCALAR_FORMATS.items()}


def _version_string() -> str:
    from . import __version__
    return "stablebear_gb300-" + __version__


def _platform_string() -> str:
    system = {"Linux": "linux", "Windows": "windows", "Darwin": "osx"}.get(_platform.system(), "other")
    arch = {"x86_64": "x86_64", "AMD64": "x86_64", "aarch64": "arm64", "arm64": "arm64"}.get(_platform.machine(),
                                                                                            _platform.machine())
    return system + "-" + arch


def _write_string(fh, s: str) -> None:
    b = s.encode()
    fh.write(struct.pack("<Q", len(b)))
    fh.write(b)


def _read_exact(fh, n: int) -> bytes:
    b = fh.read(n)
    if len(b) != n:
        raise ValueError("Incorrect number of bytes returned (file may be corrupted)")
    return b


def _read_string(fh) -> str:
    (n,) = struct.unpack("<Q", _read_exact(fh, 8))
    if n > _MAX_STRING:
        raise ValueError(f"Read string of length {n} which exceeds the {_MAX_STRING} limit "
                         "(this is likely a corrupted file).")
    return _read_exact(fh, n).decode(errors="replace")


def write_header(fh) -> None:
    fh.write(HEADER_ID)
    fh.write(b"e")
    fh.write(struct.pack("<i", FORMAT_VERSION))
    _write_string(fh, _version_string())
    _write_string(fh, _time.strftime("%Y-%m-%d"))
    _write_string(fh, _platform_string())


def read_header(fh) -> int:
    if _read_exact(fh, len(HEADER_ID)) != HEADER_ID:
        raise ValueError("Unrecognized file format.")
    if _read_exact(fh, 1) != b"e":
        raise ValueError("Data were saved on a platform with different endianness and cannot be read on this "
                         "platform.")
    (version,) = struct.unpack("<i", _read_exact(fh, 4))
    if version < 1 or version > FORMAT_VERSION:
        raise ValueError(f"Input file has format version {version}. This version reads format versions 1 "
                         f"through {FORMAT_VERSION}.")
    _read_string(fh)  # library version
    _read_string(fh)  # build date
    if version >= 2:
        _read_string(fh)  # platform
    return version


def _write_matrix(fh, m) -> None:
    base, sub = _OBJECT_FORMATS[(type(m), m.data.dtype)]
    fh.write(struct.pack("<IiiQ", SINGLE_OBJECT, base, sub, m.size))
    fh.write(np.ascontiguousarray(m.data).astype(m.data.dtype.newbyteorder("<"), copy=False).tobytes())


def _write_array(fh, a: np.ndarray) -> None:
    a = np.ascontiguousarray(a)
    if a.dtype not in _SCALAR_FORMATS:
        raise TypeError(f"Unsupported array dtype {a.dtype}; float32 or float64 arrays are saved")
    base, sub = _SCALAR_FORMATS[a.dtype]
    fh.write(struct.pack("<IiiQ", SINGLE_TENSOR, base, sub, a.ndim))
    stride = 1
    strides = []
    for ext in reversed(a.shape):
        strides.append(stride)
        stride *= ext
    for ext, st in zip(a.shape, reversed(strides)):
        fh.write(struct.pack("<QQ", ext, st))
    fh.write(a.astype(a.dtype.newbyteorder("<"), copy=False).tobytes())


def _save(item, fh) -> None:
    write_header(fh)
    if isinstance(item, (DistanceMatrix, SymmetricMatrix)):
        _write_matrix(fh, item)
    elif isinstance(item, np.ndarray):
        _write_array(fh, item)
    else:
        raise TypeError(f"Cannot save an object of type {type(item).__name__} (DistanceMatrix, SymmetricMatrix "
                        "or a float array)")


def _load(fh):
    read_header(fh)
    (ftype,) = struct.unpack("<I", _read_exact(fh, 4))
    base, sub = struct.unpack("<ii", _read_exact(fh, 8))
    if ftype == SINGLE_OBJECT:
        key = _OBJECT_TYPES.get((base, sub))
        if key is None:
            raise TypeError(f"File contains unsupported object of format ({base}, {sub})")
        cls, dt = key
        (n,) = struct.unpack("<Q", _read_exact(fh, 8))
        count = cls.storage_size(n)
        data = np.frombuffer(_read_exact(fh, count * dt.itemsize), dtype=dt.newbyteorder("<")).astype(dt)
        return cls._wrap(n, data)
    if ftype == SINGLE_TENSOR:
        dt = _SCALAR_TYPES.get((base, sub))
        if dt is None:
            raise TypeError(f"File contains an unsupported tensor of format ({base}, {sub})")
        (rank,) = struct.unpack("<Q", _read_exact(fh, 8))
        shape, strides = [], []
        for _ in range(rank):
            ext, st = struct.unpack("<QQ", _read_exact(fh, 16))
            shape.append(ext)
            strides.append(st)
        want, s = [], 1
        for ext in reversed(shape):
            want.append(s)
            s *= ext
        if strides != list(reversed(want)):
            raise ValueError(f"Incorrect strides in saved data (expected {list(reversed(want))} but got {strides})")
        count = int(np.prod(shape, dtype=np.uint64)) if shape else 1
        data = np.frombuffer(_read_exact(fh, count * dt.itemsize), dtype=dt.newbyteorder("<")).astype(dt)
        return data.reshape(shape)
    raise ValueError(f"Unknown format type {ftype}")


def save(item, file) -> None:
    """Save a DistanceMatrix, SymmetricMatrix or float array (a cdist result)
    in stablebear's binary format.  ``file`` is a path or a binary file object."""
    if isinstance(file, (str, bytes)) or hasattr(file, "__fspath__"):
        with open(file, "wb") as fh:
            _save(item, fh)
    else:
        _save(item, file)


def load(file):
    """Load what ``save`` (or the reference's ``save``) wrote: a
    DistanceMatrix, SymmetricMatrix or float array."""
    if isinstance(file, (str, bytes)) or hasattr(file, "__fspath__"):
        with open(file, "rb") as fh:
            return _load(fh)
    return _load(file)


def to_bytes(item) -> bytes:
    buf = _io.BytesIO()
    _save(item, buf)
    return buf.getvalue()


def from_bytes(buf: bytes):
    return _load(_io.BytesIO(buf))
