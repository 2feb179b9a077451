"""stablebear's binary format for DistanceMatrix / SymmetricMatrix / float
arrays: the matrix body against the reference's own writer (golden bytes),
header layout, round trips and the reader's errors."""
import io
import os
import pickle
import struct

import numpy as np
import pytest

import stablebear_gb300 as sb
from stablebear_gb300 import io as sbio
from tests.conftest import GOLDEN


def _skip_to_payload(buf):
    fh = io.BytesIO(buf)
    version = sbio.read_header(fh)
    return version, fh


@pytest.mark.parametrize("name", ["dist", "sym", "dist_empty", "sym_one"])
@pytest.mark.parametrize("tag", ["f32", "f64"])
def test_matrix_body_matches_reference_writer(name, tag):
    d = np.load(os.path.join(GOLDEN, "reference_matrix_io.npz"))
    st = d[f"{name}_{tag}_storage"]
    n = int(d[f"{name}_{tag}_n"][0])
    cls = sb.DistanceMatrix if name.startswith("dist") else sb.SymmetricMatrix
    m = cls._wrap(n, st.copy())
    version, fh = _skip_to_payload(sbio.to_bytes(m))
    assert version == 2
    ftype, base, sub = struct.unpack("<Iii", fh.read(12))
    assert ftype == sbio.SINGLE_OBJECT
    assert base == (1120 if cls is sb.DistanceMatrix else 1100)
    assert sub == (32 if tag == "f32" else 64)
    assert fh.read() == d[f"{name}_{tag}_body"].tobytes()


def test_header_layout():
    buf = sbio.to_bytes(sb.DistanceMatrix(3, dtype=np.float32))
    assert buf[:5] == b"\x01MPCF" and buf[5:6] == b"e"
    assert struct.unpack("<i", buf[6:10])[0] == 2
    fh = io.BytesIO(buf[10:])
    strings = []
    for _ in range(3):
        (k,) = struct.unpack("<Q", fh.read(8))
        strings.append(fh.read(k).decode())
    assert strings[0].startswith("stablebear_gb300-")
    assert "-" in strings[2]


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_round_trips(tmp_path, dt):
    rng = np.random.default_rng(1)
    dm = sb.DistanceMatrix(7, dtype=dt)
    dm.data[:] = rng.uniform(0, 3, dm.data.size).astype(dt)
    km = sb.SymmetricMatrix(6, dtype=dt)
    km.data[:] = rng.normal(size=km.data.size).astype(dt)
    arr = rng.normal(size=(3, 4)).astype(dt)
    for obj in (dm, km):
        p = tmp_path / f"{type(obj).__name__}.sb"
        sb.save(obj, str(p))
        back = sb.load(str(p))
        assert type(back) is type(obj) and back == obj and back.data.dtype == dt
        assert type(obj).load(p) == obj
        assert pickle.loads(pickle.dumps(obj)) == obj
        bio = io.BytesIO()
        sb.save(obj, bio)
        bio.seek(0)
        assert sb.load(bio) == obj
    p = tmp_path / "arr.sb"
    sb.save(arr, p)
    back = sb.load(p)
    assert back.dtype == dt and back.shape == arr.shape
    np.testing.assert_array_equal(back, arr)
    # a 0-d and a 1-d array
    for a in (np.array(2.5, dt), np.arange(5, dtype=dt)):
        np.testing.assert_array_equal(sbio.from_bytes(sbio.to_bytes(a)), a)


def test_tensor_layout():
    a = np.arange(6, dtype=np.float64).reshape(2, 3)
    version, fh = _skip_to_payload(sbio.to_bytes(a))
    ftype, base, sub, rank = struct.unpack("<IiiQ", fh.read(20))
    assert (ftype, base, sub, rank) == (sbio.SINGLE_TENSOR, 1, 64, 2)
    assert struct.unpack("<QQQQ", fh.read(32)) == (2, 3, 3, 1)
    np.testing.assert_array_equal(np.frombuffer(fh.read(), np.float64), np.arange(6))


def test_reads_format_version_1():
    m = sb.SymmetricMatrix(2, dtype=np.float64)
    m.data[:] = [1.0, 2.0, 3.0]
    body = struct.pack("<IiiQ", sbio.SINGLE_OBJECT, 1100, 64, 2) + m.data.tobytes()
    strs = b"".join(struct.pack("<Q", len(s)) + s for s in (b"1.0", b"2020-01-01"))
    buf = b"\x01MPCF" + b"e" + struct.pack("<i", 1) + strs + body
    assert sbio.from_bytes(buf) == m


def test_reader_errors():
    good = sbio.to_bytes(sb.DistanceMatrix(4, dtype=np.float32))
    with pytest.raises(ValueError, match="Unrecognized"):
        sbio.from_bytes(b"\x01XPCF" + good[5:])
    with pytest.raises(ValueError, match="endianness"):
        sbio.from_bytes(good[:5] + b"E" + good[6:])
    with pytest.raises(ValueError, match="format version 3"):
        sbio.from_bytes(good[:6] + struct.pack("<i", 3) + good[10:])
    with pytest.raises(ValueError, match="corrupted"):
        sbio.from_bytes(good[:-1])
    with pytest.raises(ValueError, match="not a SymmetricMatrix"):
        sb.SymmetricMatrix.from_bytes(good)
    with pytest.raises(TypeError):
        sbio.to_bytes([1, 2, 3])
    with pytest.raises(TypeError):
        sbio.to_bytes(np.arange(3, dtype=np.int32))
    other = sbio.to_bytes(sb.DistanceMatrix(2, dtype=np.float32))
    hdr = len(other) - 12 - 8 - 4
    bad = other[:hdr] + struct.pack("<Iii", sbio.SINGLE_OBJECT, 100, 32) + other[hdr + 12:]
    with pytest.raises(TypeError, match="unsupported object"):
        sbio.from_bytes(bad)
