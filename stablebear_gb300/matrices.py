"""Condensed result containers: ``DistanceMatrix`` and ``SymmetricMatrix``.

Storage order is the reference's, so a result is bit-for-bit what
``sb::DistanceMatrix<T>`` / ``sb::SymmetricMatrix<T>`` hold:

* DistanceMatrix: ``n(n-1)/2`` values; ``(i, j)``, ``i != j`` at
  ``max(i,j) * (max(i,j) - 1) / 2 + min(i,j)``; zero diagonal; entries must be
  nonnegative (``include/sbear/distance_matrix.hpp:27-150``,
  ``stablebear/distance_matrix.py:32-179``).
* SymmetricMatrix: ``n(n+1)/2`` values; ``(i, j)`` at
  ``max(i,j) * (max(i,j) + 1) / 2 + min(i,j)``
  (``include/sbear/symmetric_matrix.hpp:25-107``,
  ``stablebear/symmetric_matrix.py:32-165``).

The storage is a contiguous numpy array (``.data``), which the native library
fills in place.
"""
from __future__ import annotations

import numpy as np

float32 = np.float32
float64 = np.float64

def _dense_input(array) -> np.ndarray:
    a = np.asarray(array)
    if a.dtype not in (np.float32, np.float64):
        raise TypeError(f"Unsupported dtype {a.dtype}")
    if a.ndim != 2:
        raise ValueError("Expected a 2-D array")
    if a.shape[0] != a.shape[1]:
        raise ValueError("Expected a square array")
    return a


def _check_dtype(dtype):
    dt = np.dtype(dtype if dtype is not None else np.float64)
    if dt not in (np.dtype(np.float32), np.dtype(np.float64)):
        raise TypeError(f"Unsupported dtype {dtype}; use float32 or float64")
    return dt


class _Condensed:
    _diag: bool  # True: diagonal stored (SymmetricMatrix)

    def __init__(self, n_or_data, dtype=None):
        if isinstance(n_or_data, type(self)):
            self._n = n_or_data._n
            self._data = n_or_data._data
            return
        if isinstance(n_or_data, (int, np.integer)) and not isinstance(n_or_data, bool):
            n = int(n_or_data)
            if n < 0:
                raise ValueError("matrix size must be nonnegative")
            self._n = n
            self._data = np.zeros(self.storage_size(n), dtype=_check_dtype(dtype))
            return
        raise TypeError(f"Expected int or {type(self).__name__}; got {type(n_or_data)}")

    @classmethod
    def _wrap(cls, n: int, data: np.ndarray):
        obj = cls.__new__(cls)
        obj._n = int(n)
        if data.shape != (cls.storage_size(n),):
            raise ValueError("storage has the wrong length")
        obj._data = data
        return obj

    @classmethod
    def storage_size(cls, n: int) -> int:
        return n * (n + 1) // 2 if cls._diag else (n * (n - 1) // 2 if n > 0 else 0)

    @property
    def size(self) -> int:
        return self._n

    @property
    def storage_count(self) -> int:
        return int(self._data.shape[0])

    @property
    def dtype(self):
        return self._data.dtype.type

    @property
    def data(self) -> np.ndarray:
        """The condensed storage (a view, not a copy)."""
        return self._data

    def _resolve_ij(self, ij):
        i, j = ij
        n = self._n
        i = int(i)
        j = int(j)
        if i < 0:
            i += n
        if j < 0:
            j += n
        if not (0 <= i < n and 0 <= j < n):
            raise IndexError(f"index ({ij[0]}, {ij[1]}) is out of bounds for a {n}x{n} matrix")
        return i, j

    def _index(self, i, j):
        r, c = (i, j) if i >= j else (j, i)
        return r * (r + 1) // 2 + c if self._diag else r * (r - 1) // 2 + c

    def to_dense(self) -> np.ndarray:
        """The full ``n x n`` matrix (vectorised scatter of the condensed
        storage; the reference does an O(n^2) host loop,
        src/python/py_distance_matrix.hpp:37-49)."""
        n = self._n
        out = np.zeros((n, n), dtype=self._data.dtype)
        if n == 0:
            return out
        k = 0 if self._diag else -1
        rows, cols = np.tril_indices(n, k=k)
        out[rows, cols] = self._data  # tril_indices is row-major: (0,0),(1,0),(1,1),... == storage order
        out[cols, rows] = self._data
        return out

    def to_numpy(self) -> np.ndarray:
        return self.to_dense()

    def __array__(self, dtype=None, copy=None):
        arr = self.to_dense()
        if dtype is not None:
            arr = arr.astype(dtype, copy=False)
        return arr

    def copy(self):
        return type(self)._wrap(self._n, self._data.copy())

    def __eq__(self, other):
        return type(other) is type(self) and self._n == other._n and np.array_equal(self._data, other._data)

    def allclose(self, other, atol=1e-8, rtol=1e-5) -> bool:
        """Whether every stored element satisfies ``|a - b| <= atol + rtol |b|``
        (b from ``other``), evaluated in the element type; False when the
        storage sizes differ.  As in the reference
        (include/sbear/tensor.tpp:1702-1718, bound in
        src/python/py_distance_matrix.hpp:76-78), an element fails only when
        the difference exceeds the tolerance, so NaN entries do not fail."""
        if type(other) is not type(self) or other._data.dtype != self._data.dtype:
            raise TypeError(f"allclose needs another {type(self).__name__} of the same element type")
        a, b = self._data, other._data
        if a.shape != b.shape:
            return False
        dt = a.dtype
        return not bool(np.any(np.abs(a - b) > dt.type(atol) + dt.type(rtol) * np.abs(b)))

    def __repr__(self):
        # as the reference's bound classes print (py_distance_matrix.hpp:78-83)
        suffix = "_f32" if self._data.dtype == np.float32 else "_f64"
        return f"{type(self).__name__}{suffix}(size={self._n})"

    # --- serialisation: stablebear's binary format (see ``io.py``) ----------

    def to_bytes(self) -> bytes:
        from . import io as _sbio
        return _sbio.to_bytes(self)

    @classmethod
    def from_bytes(cls, buf: bytes):
        from . import io as _sbio
        obj = _sbio.from_bytes(buf)
        if type(obj) is not cls:
            raise ValueError(f"serialised object is a {type(obj).__name__}, not a {cls.__name__}")
        return obj

    def save(self, path):
        from . import io as _sbio
        _sbio.save(self, path)

    @classmethod
    def load(cls, path):
        from . import io as _sbio
        obj = _sbio.load(path)
        if type(obj) is not cls:
            raise ValueError(f"file holds a {type(obj).__name__}, not a {cls.__name__}")
        return obj

    def __reduce__(self):
        return (type(self).from_bytes, (self.to_bytes(),))


class DistanceMatrix(_Condensed):
    """Compressed distance matrix (symmetric, zero diagonal, nonnegative)."""

    _diag = False

    def __getitem__(self, ij):
        i, j = self._resolve_ij(ij)
        if i == j:
            return self._data.dtype.type(0)
        return self._data[self._index(i, j)]

    def __setitem__(self, ij, value):
        i, j = self._resolve_ij(ij)
        if value < 0:
            raise ValueError("Distance matrix entries must be nonnegative")
        if i == j:
            if value != 0:
                raise ValueError("Diagonal entries of a distance matrix must be zero")
            return
        self._data[self._index(i, j)] = value

    @classmethod
    def from_dense(cls, array) -> "DistanceMatrix":
        """Checks as the reference does (src/python/py_distance_matrix.hpp:50-73):
        the diagonal first, then the strict upper triangle in row-major order,
        where the first entry that is negative or differs from its mirror
        decides the message."""
        a = _dense_input(array)
        n = a.shape[0]
        if np.any(np.diag(a) != 0):
            raise ValueError("Diagonal entries must be zero")
        iu, ju = np.triu_indices(n, k=1)
        up = a[iu, ju]
        bad = (up < 0) | (up != a[ju, iu])
        if bad.any():
            k = int(np.argmax(bad))
            raise ValueError("Entries must be nonnegative" if up[k] < 0 else "Matrix must be symmetric")
        rows, cols = np.tril_indices(n, k=-1)
        return cls._wrap(n, np.ascontiguousarray(a[rows, cols]))


class SymmetricMatrix(_Condensed):
    """Compressed symmetric matrix (lower-triangular storage with diagonal)."""

    _diag = True

    def __getitem__(self, ij):
        i, j = self._resolve_ij(ij)
        return self._data[self._index(i, j)]

    def __setitem__(self, ij, value):
        i, j = self._resolve_ij(ij)
        self._data[self._index(i, j)] = value

    @classmethod
    def from_dense(cls, array) -> "SymmetricMatrix":
        """As the reference (src/python/py_symmetric_matrix.hpp:62-81)."""
        a = _dense_input(array)
        if not np.array_equal(a, a.T):
            raise ValueError("Matrix must be symmetric")
        n = a.shape[0]
        rows, cols = np.tril_indices(n)
        return cls._wrap(n, np.ascontiguousarray(a[rows, cols]))
