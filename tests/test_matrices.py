"""DistanceMatrix / SymmetricMatrix on the host: construction, element
access, dense conversion and from_dense checks, with the behaviour and
messages of the reference's containers (include/sbear/distance_matrix.hpp,
src/python/py_distance_matrix.hpp, src/python/py_symmetric_matrix.hpp,
stablebear/distance_matrix.py, stablebear/symmetric_matrix.py)."""
import numpy as np
import pytest

import stablebear_gb300 as sb

DTYPES = [np.float32, np.float64]


@pytest.mark.parametrize("dt", DTYPES)
def test_sizes_and_storage(dt):
    for n, want in ((0, 0), (1, 0), (5, 10)):
        m = sb.DistanceMatrix(n, dtype=dt)
        assert m.size == n and m.storage_count == want and m.data.dtype == dt
    for n, want in ((0, 0), (1, 1), (5, 15)):
        assert sb.SymmetricMatrix(n, dtype=dt).storage_count == want
    assert sb.DistanceMatrix(3).dtype == np.float64
    with pytest.raises(TypeError, match="Unsupported dtype"):
        sb.DistanceMatrix(3, dtype=np.int32)


@pytest.mark.parametrize("dt", DTYPES)
def test_distance_access(dt):
    m = sb.DistanceMatrix(4, dtype=dt)
    m[2, 1] = 1.5
    assert m[1, 2] == 1.5 and m[2, 1] == 1.5
    assert m[3, 3] == 0
    m[3, 3] = 0.0  # writing zero to the diagonal is allowed
    m[-1, 0] = 2.0
    assert m[3, 0] == 2.0
    # storage order: max(i,j) * (max(i,j) - 1) / 2 + min(i,j)
    assert m.data[2 * 1 // 2 + 1] == 1.5 and m.data[3 * 2 // 2 + 0] == 2.0
    with pytest.raises(ValueError, match="nonnegative"):
        m[0, 1] = -1.0
    with pytest.raises(ValueError, match="Diagonal"):
        m[1, 1] = 1.0
    with pytest.raises(IndexError):
        _ = m[4, 0]


@pytest.mark.parametrize("dt", DTYPES)
def test_symmetric_access(dt):
    m = sb.SymmetricMatrix(3, dtype=dt)
    m[1, 1] = -2.0
    m[0, 2] = 3.0
    assert m[2, 0] == 3.0 and m[1, 1] == -2.0
    assert m.data[1 * 2 // 2 + 1] == -2.0 and m.data[2 * 3 // 2 + 0] == 3.0


@pytest.mark.parametrize("dt", DTYPES)
def test_dense_round_trips(dt):
    rng = np.random.default_rng(0)
    a = rng.uniform(0, 5, (6, 6)).astype(dt)
    a = a + a.T
    np.fill_diagonal(a, 0)
    dm = sb.DistanceMatrix.from_dense(a)
    np.testing.assert_array_equal(dm.to_dense(), a)
    np.testing.assert_array_equal(np.asarray(dm), a)
    np.testing.assert_array_equal(dm.to_numpy(), a)
    b = rng.normal(size=(5, 5)).astype(dt)
    b = b + b.T
    km = sb.SymmetricMatrix.from_dense(b)
    np.testing.assert_array_equal(km.to_dense(), b)
    assert sb.DistanceMatrix(0, dtype=dt).to_dense().shape == (0, 0)


def test_from_dense_messages():
    with pytest.raises(ValueError, match="Expected a 2-D array"):
        sb.DistanceMatrix.from_dense(np.zeros(3))
    with pytest.raises(ValueError, match="Expected a square array"):
        sb.SymmetricMatrix.from_dense(np.zeros((2, 3)))
    with pytest.raises(TypeError, match="Unsupported dtype"):
        sb.DistanceMatrix.from_dense(np.zeros((2, 2), np.int64))
    a = np.zeros((3, 3))
    a[1, 1] = 1
    with pytest.raises(ValueError, match="Diagonal entries must be zero"):
        sb.DistanceMatrix.from_dense(a)
    a = np.zeros((3, 3))
    a[0, 2], a[2, 0] = 1, 2
    with pytest.raises(ValueError, match="Matrix must be symmetric"):
        sb.DistanceMatrix.from_dense(a)
    with pytest.raises(ValueError, match="Matrix must be symmetric"):
        sb.SymmetricMatrix.from_dense(a)
    # the first violation in row-major order of the upper triangle decides
    a = np.zeros((3, 3))
    a[0, 1] = a[1, 0] = -1.0
    a[1, 2], a[2, 1] = 1, 2
    with pytest.raises(ValueError, match="Entries must be nonnegative"):
        sb.DistanceMatrix.from_dense(a)
    a = np.zeros((3, 3))
    a[0, 1], a[1, 0] = 1, 2
    a[1, 2] = a[2, 1] = -1.0
    with pytest.raises(ValueError, match="Matrix must be symmetric"):
        sb.DistanceMatrix.from_dense(a)


def test_repr_as_the_reference():
    assert repr(sb.DistanceMatrix(3, dtype=np.float32)) == "DistanceMatrix_f32(size=3)"
    assert repr(sb.SymmetricMatrix(4)) == "SymmetricMatrix_f64(size=4)"


def test_allclose_as_the_reference():
    """allclose: |a - b| <= atol + rtol |b| element-wise, in the element type
    (include/sbear/tensor.tpp:1687-1718); matrices compare their storage and
    let NaN entries pass, dense arrays do not."""
    import stablebear_gb300 as sb
    a = sb.DistanceMatrix(4, dtype=np.float32)
    a.data[:] = np.arange(1, 7, dtype=np.float32)
    b = a.copy()
    assert sb.allclose(a, b) and a.allclose(b)
    b.data[3] += np.float32(1e-4)  # |a - b| = 1e-4 > 1e-8 + 1e-5 * 4.0001
    assert not sb.allclose(a, b)
    assert sb.allclose(a, b, rtol=1e-4)
    assert sb.allclose(a, b, atol=1e-4)
    b = a.copy()
    b.data[0] = np.nan
    assert sb.allclose(a, b)  # a NaN does not exceed the tolerance
    assert not sb.allclose(a, sb.DistanceMatrix(5, dtype=np.float32))
    with pytest.raises(TypeError):
        sb.allclose(a, sb.SymmetricMatrix(4, dtype=np.float32))
    with pytest.raises(TypeError):
        a.allclose(sb.DistanceMatrix(4, dtype=np.float64))
    k = sb.SymmetricMatrix(3, dtype=np.float64)
    k.data[:] = 1.0
    k2 = k.copy()
    k2.data[:] += 5e-6
    assert sb.allclose(k, k2) and not sb.allclose(k, k2, rtol=1e-6)
    x = np.ones((2, 3), np.float32)
    y = x.copy()
    assert sb.allclose(x, y)
    y[0, 0] = np.nan
    assert not sb.allclose(x, y)  # dense arrays: a NaN fails
    assert not sb.allclose(x, np.ones((3, 2), np.float32))
    with pytest.raises(TypeError):
        sb.allclose(x, a)
