"""Oracle: relationship-matrix file formats (test infrastructure).

* COSMIC_UPPER_PACKED, restating io::write_upper_packed_binary / read_upper_packed_binary
  (src/core/upper_packed_binary.cpp:27-68, 89-138; layout documented in
  src/core/upper_packed_binary.h): 32-byte NUL-padded magic, int32 version 1, int64 n,
  int32 index base 1, int32 storage code 1, int32 dtype code 1, int32 endian code 1,
  then A(i, j) for i <= j column by column as little-endian FP64.  The reader expands
  symmetrically and rejects other metadata and trailing bytes.
* GCTA .grm.bin / .grm.N.bin, restating GrmBuilder::save (src/core/grm_builder.cpp:
  1873-1922): G(i, j) for j <= i row by row as float32, N_snps in the same layout.
"""
from __future__ import annotations

import struct

import numpy as np

MAGIC = b"COSMIC_UPPER_PACKED".ljust(32, b"\0")


def upper_packed_header(n: int) -> bytes:
    return MAGIC + struct.pack("<iqiiii", 1, n, 1, 1, 1, 1)


def upper_packed_bytes(A: np.ndarray) -> bytes:
    """File bytes of write_upper_packed_binary for the dense matrix A."""
    n = A.shape[0]
    if A.shape != (n, n):
        raise ValueError("upper-packed binary output requires a square matrix")
    cols = [A[: j + 1, j] for j in range(n)]
    payload = np.concatenate(cols).astype("<f8").tobytes() if n else b""
    return upper_packed_header(n) + payload


def read_upper_packed(data: bytes) -> np.ndarray:
    """read_upper_packed_binary on the file bytes."""
    if len(data) < 60 or data[:32] != MAGIC:
        raise ValueError("unsupported binary matrix header")
    version, n, base, storage, dtype, endian = struct.unpack("<iqiiii", data[32:60])
    if (version, base, storage, dtype, endian) != (1, 1, 1, 1, 1):
        raise ValueError("unsupported upper-packed binary matrix metadata")
    if n <= 0 or n > 2**31 - 1:
        raise ValueError("invalid upper-packed binary matrix dimension")
    cnt = n * (n + 1) // 2
    if len(data) < 60 + 8 * cnt:
        raise ValueError("truncated upper-packed binary matrix file")
    if len(data) > 60 + 8 * cnt:
        raise ValueError("upper-packed binary matrix file has trailing bytes")
    vals = np.frombuffer(data, dtype="<f8", count=cnt, offset=60)
    A = np.zeros((n, n))
    k = 0
    for j in range(n):
        A[: j + 1, j] = vals[k: k + j + 1]
        A[j, : j + 1] = vals[k: k + j + 1]
        k += j + 1
    return A


def grm_gcta_bytes(G: np.ndarray, n_valid: int) -> tuple[bytes, bytes]:
    """(.grm.bin, .grm.N.bin) bytes of GrmBuilder::save."""
    n = G.shape[0]
    rows = [G[i, : i + 1] for i in range(n)]
    g = np.concatenate(rows).astype("<f4")
    return g.tobytes(), np.full(g.size, np.float32(n_valid), dtype="<f4").tobytes()
