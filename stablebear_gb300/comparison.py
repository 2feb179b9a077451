"""``allclose`` for the result types of the pairwise path, as
stablebear/comparison.py:8-48 provides it."""
from __future__ import annotations

import numpy as np

from .matrices import DistanceMatrix, SymmetricMatrix


def allclose(a, b, atol=1e-8, rtol=1e-5) -> bool:
    """Whether two objects of the same type are element-wise equal within
    ``|a_i - b_i| <= atol + rtol |b_i|``.

    DistanceMatrix and SymmetricMatrix compare their storage (NaN entries do
    not fail, include/sbear/tensor.tpp:1702-1718).  Dense float arrays (what
    ``cdist`` returns) compare element-wise with the same formula, evaluated
    in their element type; a NaN entry fails, as for the reference's tensors
    (tensor.tpp:1687-1700), and different shapes give False.  Any other
    combination raises TypeError, as the reference does.
    """
    if isinstance(a, DistanceMatrix) and isinstance(b, DistanceMatrix):
        return a.allclose(b, atol=atol, rtol=rtol)
    if isinstance(a, SymmetricMatrix) and isinstance(b, SymmetricMatrix):
        return a.allclose(b, atol=atol, rtol=rtol)
    if (isinstance(a, np.ndarray) and isinstance(b, np.ndarray) and a.dtype.kind == "f" and b.dtype.kind == "f"
            and a.dtype == b.dtype):
        if a.shape != b.shape:
            return False
        dt = a.dtype
        return bool(np.all(np.abs(a - b) <= dt.type(atol) + dt.type(rtol) * np.abs(b)))
    raise TypeError(
        f"allclose requires two objects of the same supported type "
        f"(float array, DistanceMatrix, or SymmetricMatrix), "
        f"got {type(a).__name__} and {type(b).__name__}"
    )
