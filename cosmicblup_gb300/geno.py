"""Genotype matrix-free products on the device (PlinkReader's RHE / PCG support).

Reference interfaces mirrored:
* ``PlinkReader::computeStats`` / ``getMeans`` / ``getInvStds``
  (src/core/plink_reader.cpp:186-237, src/core/plink_reader.h:103-108);
* ``GenotypeMatrix::multiply_Z_v`` / ``multiply_Zt_v`` as PlinkReader implements
  them (src/core/plink_reader.cpp:239-293, 341-392), ``rows()`` / ``cols()``;
* the SNP-effect back-solve of the result writer (src/solve/result_writer.cpp:565-623).
The arithmetic runs in libcbx (``cbx_geno_*``, ``cbx_snp_effects``); the BED payload
stays on the device after the first call.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import Handle, lib, ptr


class DeviceGenotypes:
    """A PLINK BED payload resident on the GPU with its per-SNP statistics."""

    def __init__(self, bed: bytes, n: int, m: int, handle: Handle | None = None):
        self._own = handle is None
        self.handle = handle or Handle(0)
        self.n, self.m = int(n), int(m)
        buf = np.frombuffer(bed, dtype=np.uint8)
        self.snp_means = np.empty(self.m)
        self.snp_inv_stds = np.empty(self.m)
        self.handle.check(lib().cbx_geno_attach(self.handle.raw, ptr(buf), buf.size, self.n, self.m,
                                                ptr(self.snp_means), ptr(self.snp_inv_stds)))

    # GenotypeMatrix interface (rows = samples, cols = SNPs)
    def rows(self) -> int:
        return self.n

    def cols(self) -> int:
        return self.m

    def getMeans(self) -> np.ndarray:
        return self.snp_means

    def getInvStds(self) -> np.ndarray:
        return self.snp_inv_stds

    def _product(self, fn, v: np.ndarray, n_in: int, n_out: int, what: str) -> np.ndarray:
        v = np.asarray(v, dtype=np.float64)
        if v.shape[0] != n_in:
            raise ValueError(f"Dimension mismatch in {what}")
        cols = v.reshape(n_in, -1)
        k = cols.shape[1]
        vin = np.ascontiguousarray(cols.T)  # column-major n_in x k
        out = np.empty((k, n_out))
        self.handle.check(fn(self.handle.raw, k, ptr(vin), ptr(out)))
        return out.T.reshape((n_out,) + v.shape[1:])

    def multiply_Zt_v(self, v: np.ndarray) -> np.ndarray:
        """y (m) = Z^T v (v: n), or one column per column of a 2-D v."""
        return self._product(lib().cbx_geno_zt_v, v, self.n, self.m, "multiply_Zt_v")

    def multiply_Z_v(self, v: np.ndarray) -> np.ndarray:
        """y (n) = Z v (v: m), or one column per column of a 2-D v."""
        return self._product(lib().cbx_geno_z_v, v, self.m, self.n, "multiply_Z_v")

    def snp_effects(self, u_g: np.ndarray, Ginv: np.ndarray | None = None):
        """Back-solved SNP effects: returns (effect, freq, total_2pq).

        Ginv=None uses the handle's device G^-1 (``invert_psd``) or its dense Q^-1.
        """
        u = np.ascontiguousarray(u_g, dtype=np.float64)
        G = None if Ginv is None else np.ascontiguousarray(Ginv, dtype=np.float64)
        if G is not None and G.shape != (u.size, u.size):
            raise ValueError("Ginv must be n_g x n_g")
        effect = np.empty(self.m)
        freq = np.empty(self.m)
        t2 = C.c_double()
        self.handle.check(lib().cbx_snp_effects(self.handle.raw, ptr(u), u.size, ptr(G), ptr(effect),
                                                ptr(freq), C.byref(t2)))
        return effect, freq, t2.value

    def close(self) -> None:
        if self._own and self.handle is not None:
            self.handle.close()
        self.handle = None
