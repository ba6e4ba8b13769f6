"""Oracle: matrix-free genotype products and the SNP-effect back-solve (test infrastructure).

Restates, in FP64 numpy, the reference's standardized-genotype operators:

* ``PlinkReader::computeStats`` (src/core/plink_reader.cpp:186-237): per SNP the
  observed calls' mean, p = mean / 2, var = 2p(1-p), inv_std = 1/sqrt(var), with
  inv_std = 0 when var < 1e-9 and mean = inv_std = 0 when nothing is observed;
* ``PlinkReader::multiply_Zt_v`` (:341-392): y_j = (sum_obs x_ij v_i - mean_j
  sum_obs v_i) inv_std_j;
* ``PlinkReader::multiply_Z_v`` (:239-293): per SNP the float val_map
  ``(float)((code value - mean) * v_j inv_std_j)`` (0 for a missing call), summed
  over SNPs in FP64;
* the back-solve of the result writer (src/solve/result_writer.cpp:565-623):
  q = G^-1 u_g, effect_j = ((Z^T q)_j / inv_std_j) / total_2pq, freq_j = mean_j / 2.

Genotypes come in as ``oracle.plink.decode_bed`` gives them: (m, n) int8, allele-1
copies 2 / 1 / 0 and -1 for a missing call.  The sums run in numpy's order, not
the reference's sequential one; tests allow for the difference (a few FP64
roundings of the sums of magnitudes).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build


def compute_stats(geno: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """(mean, inv_std) per SNP, src/core/plink_reader.cpp:192-236."""
    m = geno.shape[0]
    mean = np.zeros(m)
    inv_std = np.zeros(m)
    for j in range(m):
        g = geno[j]
        obs = g >= 0
        count = int(obs.sum())
        if count == 0:
            continue
        s = float(g[obs].astype(np.int64).sum())  # the float codes summed in double: exact
        mu = s / count
        p = mu / 2.0
        var = 2.0 * p * (1.0 - p)
        mean[j] = mu
        inv_std[j] = 0.0 if var < 1e-9 else 1.0 / np.sqrt(var)
    return mean, inv_std


def multiply_zt_v(geno: np.ndarray, mean: np.ndarray, inv_std: np.ndarray, v: np.ndarray) -> np.ndarray:
    """Z^T v, src/core/plink_reader.cpp:341-392."""
    obs = geno >= 0
    x = np.where(obs, geno, 0).astype(np.float64)
    sum_xv = x @ v
    sum_v_obs = obs.astype(np.float64) @ v
    y = (sum_xv - mean * sum_v_obs) * inv_std
    return np.where(inv_std == 0.0, 0.0, y)


def val_maps(mean: np.ndarray, inv_std: np.ndarray, v: np.ndarray) -> np.ndarray:
    """Per-SNP float terms by code (00, 01, 10, 11), src/core/plink_reader.cpp:258-270."""
    weight = v * inv_std
    vm = np.zeros((mean.size, 4), np.float32)
    for c, x in ((0, 2.0), (2, 1.0), (3, 0.0)):
        vm[:, c] = ((x - mean) * weight).astype(np.float32)
    vm[inv_std == 0.0] = 0.0  # skipped SNPs (the reference's `continue`)
    return vm


def multiply_z_v(geno: np.ndarray, mean: np.ndarray, inv_std: np.ndarray, v: np.ndarray) -> np.ndarray:
    """Z v with float-rounded terms, src/core/plink_reader.cpp:239-293."""
    vm = val_maps(mean, inv_std, v).astype(np.float64)
    code = np.select([geno == 2, geno == -1, geno == 1], [0, 1, 2], 3)  # genotype -> 2-bit code
    terms = np.take_along_axis(vm, code, axis=1)
    return terms.sum(axis=0)


def total_2pq(mean: np.ndarray) -> float:
    """src/solve/result_writer.cpp:604-609 (sequential order)."""
    t = 0.0
    for mu in mean:
        p = mu / 2.0
        var = 2.0 * p * (1.0 - p)
        if var >= 1e-9:
            t += var
    return t


def snp_effects(geno: np.ndarray, Ginv: np.ndarray, u_g: np.ndarray):
    """(effect, freq, total_2pq), src/solve/result_writer.cpp:590-620 (--bfile branch)."""
    mean, inv_std = compute_stats(geno)
    q = Ginv @ u_g
    zt = multiply_zt_v(geno, mean, inv_std, q)
    t2 = total_2pq(mean)
    effect = np.zeros(mean.size)
    ok = (inv_std > 0.0) & (t2 > 0.0)
    effect[ok] = (zt[ok] / inv_std[ok]) / t2
    return effect, mean / 2.0, t2


def multiply_zt_v_c(bed: bytes, n: int, m: int, mean: np.ndarray, inv_std: np.ndarray, v: np.ndarray,
                    threads: int | None = None, j0: int = 0, j1: int | None = None) -> np.ndarray:
    """Z^T v for SNPs [j0, j1) by the C restatement of the reference's loop
    (oracle/csrc/oracle_geno.c), SNP ranges split over ``threads`` host threads (ctypes
    releases the GIL), as the reference splits them over OpenMP threads."""
    import concurrent.futures as cf
    if not os.path.exists(_build.LIB):
        _build.build()
    L = C.CDLL(_build.LIB)
    f = L.oracle_multiply_zt_v
    f.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.c_int64, C.c_int64]
    j1 = m if j1 is None else j1
    bps = (n + 3) // 4
    buf = np.frombuffer(bed, dtype=np.uint8)
    mean = np.ascontiguousarray(mean, dtype=np.float64)
    inv_std = np.ascontiguousarray(inv_std, dtype=np.float64)
    v = np.ascontiguousarray(v, dtype=np.float64)
    y = np.zeros(m)
    threads = threads or os.cpu_count() or 1
    cuts = np.linspace(j0, j1, threads + 1).astype(np.int64)
    base = buf.ctypes.data + 3
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(lambda k: f(base, n, bps, mean.ctypes.data, inv_std.ctypes.data, v.ctypes.data,
                                y.ctypes.data, int(cuts[k]), int(cuts[k + 1])), range(threads)))
    return y[j0:j1]

