"""GRM host API mirroring the reference's PlinkReader / GrmBuilder.

Reference interfaces mirrored:
* ``PlinkReader::load(prefix)`` reads .fam/.bim and opens the .bed
  (src/core/plink_reader.cpp:27-91);
* ``GrmBuilder(Options).compute(reader)`` then ``getGrm()``, ``getSum2pq()``,
  ``getTotalSnps()``, ``getAlleleFreqs()`` (src/core/grm_builder.h:14-58).
The arithmetic runs in libcbx (``cbx_grm_bed``); this module only moves bytes.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from ._lib import Handle, lib, ptr


class PlinkReader:
    """Holds the raw .bed bytes plus sample / SNP counts from .fam / .bim."""

    def __init__(self):
        self.bed = b""
        self.num_samples = 0
        self.num_snps = 0
        self.fam_ids: list[str] = []
        self.bim_ids: list[str] = []

    @classmethod
    def from_bytes(cls, bed: bytes, n: int, m: int) -> "PlinkReader":
        r = cls()
        r.bed, r.num_samples, r.num_snps = bytes(bed), int(n), int(m)
        return r

    def load(self, prefix: str) -> "PlinkReader":
        fam = [ln.split() for ln in open(prefix + ".fam") if ln.strip()]
        if not fam:
            raise RuntimeError("No samples found in .fam file")
        bim = [ln.split() for ln in open(prefix + ".bim") if ln.strip()]
        self.fam_ids = [f[1] for f in fam]
        self.fam_fids = [f[0] for f in fam]
        self.bim_ids = [b[1] for b in bim]
        self.num_samples, self.num_snps = len(fam), len(bim)
        with open(prefix + ".bed", "rb") as f:
            self.bed = f.read()
        return self

    def getNumSamples(self) -> int:
        return self.num_samples

    def getNumSnps(self) -> int:
        return self.num_snps

    def getBytesPerSnp(self) -> int:
        return (self.num_samples + 3) // 4

    # RHE / PCG support (src/core/plink_reader.h:100-125): the payload moves to
    # the device on the first call and the products run there.
    def computeStats(self, handle: Handle | None = None) -> None:
        from .geno import DeviceGenotypes
        if getattr(self, "_dev", None) is None:
            self._dev = DeviceGenotypes(self.bed, self.num_samples, self.num_snps, handle)

    def getMeans(self) -> np.ndarray:
        self.computeStats()
        return self._dev.getMeans()

    def getInvStds(self) -> np.ndarray:
        self.computeStats()
        return self._dev.getInvStds()

    def multiply_Z_v(self, v: np.ndarray) -> np.ndarray:
        self.computeStats()
        return self._dev.multiply_Z_v(v)

    def multiply_Zt_v(self, v: np.ndarray) -> np.ndarray:
        self.computeStats()
        return self._dev.multiply_Zt_v(v)


@dataclass
class GrmOptions:
    """Subset of GrmBuilder::Options honoured by the GPU path (grm_builder.h:14-29)."""
    thread_num: int = 1
    block_size: int = 2048
    min_maf: float = 0.01
    min_hwe: float = 0.0
    algorithm: int = 1


class GrmBuilder:
    def __init__(self, options: GrmOptions | None = None, handle: Handle | None = None):
        self.options = options or GrmOptions()
        self._own = handle is None
        self.handle = handle or Handle(0)
        self.G = None
        self.xx = None
        self.total_sum_2pq = 0.0
        self.total_valid_snps_count = 0
        self.allele_freqs = None

    def compute(self, reader: PlinkReader, keep_xx_counts: bool = False) -> None:
        if self.options.min_hwe > 0:
            raise NotImplementedError("HWE filtering is not part of the GPU GRM path")
        n, m = reader.num_samples, reader.num_snps
        bed = np.frombuffer(reader.bed, dtype=np.uint8)
        G = np.empty((n, n), dtype=np.float64)
        xx = np.empty((n, n), dtype=np.int32) if keep_xx_counts else None
        freqs = np.empty(m, dtype=np.float32)
        s2pq = C.c_double(0.0)
        nvalid = C.c_int64(0)
        rc = lib().cbx_grm_bed(self.handle.raw, ptr(bed), bed.size, n, m,
                               C.c_float(self.options.min_maf), self.options.algorithm,
                               self.options.block_size, ptr(G), ptr(xx), ptr(freqs),
                               C.byref(s2pq), C.byref(nvalid))
        self.handle.check(rc)
        self.G, self.xx, self.allele_freqs = G, xx, freqs
        self.total_sum_2pq = s2pq.value
        self.total_valid_snps_count = nvalid.value
        n_ids = len(getattr(reader, "fam_ids", []))
        self.sample_iids = list(reader.fam_ids) if n_ids == n else [str(i + 1) for i in range(n)]
        self.sample_fids = (list(reader.fam_fids) if len(getattr(reader, "fam_fids", [])) == n
                            else list(self.sample_iids))

    def save(self, out_prefix: str) -> None:
        """GrmBuilder::save (src/core/grm_builder.cpp:1873-1922): writes .grm.id here
        and .grm.bin / .grm.N.bin from the device GRM (cbx_write_grm_gcta)."""
        with open(out_prefix + ".grm.id", "w") as f:
            for fid, iid in zip(self.sample_fids, self.sample_iids):
                f.write(f"{fid}\t{iid}\n")
        self.handle.check(lib().cbx_write_grm_gcta(self.handle.raw, (out_prefix + ".grm.bin").encode(),
                                                   (out_prefix + ".grm.N.bin").encode(),
                                                   int(self.total_valid_snps_count)))

    def getGrm(self) -> np.ndarray:
        return self.G

    def getSum2pq(self) -> float:
        return self.total_sum_2pq

    def getTotalSnps(self) -> int:
        return self.total_valid_snps_count

    def getAlleleFreqs(self) -> np.ndarray:
        return self.allele_freqs

    def getXXCounts(self) -> np.ndarray:
        return self.xx


def bed_snp_counts(handle: Handle, bed: bytes, n: int, m: int) -> dict:
    """Per-SNP integer tallies (n_obs, sum_x, n_hom1, n_het, n_hom2) from the device."""
    buf = np.frombuffer(bed, dtype=np.uint8)
    outs = {k: np.empty(m, dtype=np.int32) for k in ("n_obs", "sum_x", "n_hom1", "n_het", "n_hom2")}
    rc = lib().cbx_bed_snp_counts(handle.raw, ptr(buf), buf.size, n, m, ptr(outs["n_obs"]),
                                  ptr(outs["sum_x"]), ptr(outs["n_hom1"]), ptr(outs["n_het"]),
                                  ptr(outs["n_hom2"]))
    handle.check(rc)
    return outs


def write_matrix_bin(handle: Handle, which: int, bin_path: str, id_path: str | None = None,
                     ids: list[str] | None = None) -> None:
    """write_matrix_bin (src/core/matrix_io.cpp:479-484) for a device matrix: which = 0
    the GRM left by cbx_grm_bed, 1 the G^-1 left by cbx_invert_psd (COSMIC_UPPER_PACKED)."""
    if id_path is not None and ids is not None:
        with open(id_path, "w") as f:
            for i in ids:
                f.write(f"{i}\n")
    handle.check(lib().cbx_write_upper_packed(handle.raw, int(which), bin_path.encode()))

