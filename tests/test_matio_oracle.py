"""CPU tests of the matrix-file oracle (oracle/matio.py): the COSMIC_UPPER_PACKED
header as the reference documents it (src/core/upper_packed_binary.h), round trips,
and the reader's rejections."""
import struct

import numpy as np
import pytest

from oracle.matio import grm_gcta_bytes, read_upper_packed, upper_packed_bytes, upper_packed_header


def test_header_layout():
    h = upper_packed_header(5)
    assert len(h) == 60
    assert h[:19] == b"COSMIC_UPPER_PACKED" and h[19:32] == b"\0" * 13
    assert struct.unpack("<iqiiii", h[32:]) == (1, 5, 1, 1, 1, 1)


def test_upper_column_order_and_round_trip():
    A = np.arange(16, dtype=float).reshape(4, 4)
    A = A + A.T
    b = upper_packed_bytes(A)
    vals = np.frombuffer(b, dtype="<f8", offset=60)
    # A(0,0), A(0,1), A(1,1), A(0,2), A(1,2), A(2,2), ...
    expect = [A[0, 0], A[0, 1], A[1, 1], A[0, 2], A[1, 2], A[2, 2], A[0, 3], A[1, 3], A[2, 3], A[3, 3]]
    assert vals.tolist() == expect
    assert np.array_equal(read_upper_packed(b), A)


def test_reader_rejections():
    b = upper_packed_bytes(np.eye(3))
    with pytest.raises(ValueError):
        read_upper_packed(b + b"\0")
    with pytest.raises(ValueError):
        read_upper_packed(b[:-1])
    bad = bytearray(b)
    bad[36:44] = struct.pack("<q", 0)
    with pytest.raises(ValueError):
        read_upper_packed(bytes(bad))
    bad = bytearray(b)
    bad[44:48] = struct.pack("<i", 0)  # index base
    with pytest.raises(ValueError):
        read_upper_packed(bytes(bad))


def test_gcta_lower_row_order():
    G = np.array([[1.0, 0.5, 0.25], [0.5, 2.0, 0.125], [0.25, 0.125, 3.0]])
    g, nb = grm_gcta_bytes(G, 77)
    assert np.frombuffer(g, "<f4").tolist() == [1.0, 0.5, 2.0, 0.25, 0.125, 3.0]
    assert np.frombuffer(nb, "<f4").tolist() == [77.0] * 6
