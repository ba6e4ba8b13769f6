"""Why the dense H^-1 block of the PCG bulk is FP32 and not BF16 (CPU, oracle only).

Mixed-precision PCG runs the inner solves on a low-precision copy of the dense
block (Qd - c, c the mean off-diagonal entry) and refines on the FP64 residual
b - A x.  With an exact inner solve on the perturbed operator, each refinement
shrinks the residual by about the relative perturbation the block's rounding
makes in A^-1.  On a scaled single-step problem (pedigree A^-1 plus
(0.95 G + 0.05 A22)^-1 - A22^-1 on the genotyped animals, the reference's
SplitMatrixAdapter operator, src/core/matrix_adapter.h:252-278) the FP32 block
reaches relres 1e-10 after one refinement; a BF16 block contracts by only about
1e-3 per refinement and needs three, each of which costs an FP64-accurate block
product.
"""
import numpy as np
import pytest
import scipy.sparse as sp
from scipy.sparse.linalg import splu

from cosmicblup_gb300.synth import simulate_bed_gene_drop, simulate_gblup_records, simulate_pedigree
from oracle.grm import vanraden_grm
from oracle.mme import build_fixed_design, invert_psd_matrix, sparse_data_part
from oracle.ped import a_columns, ainv_henderson, tune_g


def _round_bf16(a):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    b = np.asarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


@pytest.fixture(scope="module")
def system():
    n_gen, per_gen, ng, m = 6, 500, 500, 3000
    sire, dam = simulate_pedigree(n_gen, per_gen, 25, 250, seed=5101, p_unknown=0.05)
    q = sire.size
    gmap = np.arange(q - ng, q, dtype=np.int32)
    bed, _ = simulate_bed_gene_drop(sire, dam, per_gen, m, seed=5100, p_lo=0.01, miss=0.02)
    G = vanraden_grm(bed, ng, m)["G"]
    ptr, col, val, _, dii = ainv_henderson(dam, sire)
    A22 = a_columns(dam, sire, dii, gmap)[gmap]
    Gt, _, _ = tune_g(G, A22)
    Gd = invert_psd_matrix(0.95 * Gt + 0.05 * A22) - np.linalg.inv(A22)
    rec = simulate_gblup_records(q, 30, np.random.default_rng(5102).normal(0, 0.6, q), seed=5103, var_e=0.65)
    p, rows, _ = build_fixed_design(rec["cats"])
    _, W = sparse_data_part(rec["aid"], rows, p, q)
    W = sp.csr_matrix(W)
    Ainv = sp.csr_matrix((val, col, ptr), shape=(q, q))
    lam = 1.2

    def lhs(D):
        Ds = sp.csr_matrix((D.ravel(), (np.repeat(gmap, ng), np.tile(gmap, ng))), shape=(q, q))
        return ((W.T @ W) + sp.block_diag([sp.csr_matrix((p, p)), lam * (Ainv + Ds)])).tocsc()

    return dict(Gd=Gd, lhs=lhs, b=W.T @ rec["y"], ng=ng)


def _refine(system, D, n=4):
    A, b = system["lhs"](system["Gd"]), system["b"]
    lu = splu(system["lhs"](D), permc_spec="MMD_AT_PLUS_A")
    x, r, hist = np.zeros_like(b), b.copy(), []
    for _ in range(n):
        x = x + lu.solve(r)
        r = b - A @ x
        hist.append(np.linalg.norm(r) / np.linalg.norm(b))
    return hist


def test_fp32_block_needs_one_refinement_bf16_three(system):
    Gd, ng = system["Gd"], system["ng"]
    c = (Gd.sum() - np.trace(Gd)) / (ng * ng - ng)
    fp32 = _refine(system, (Gd - c).astype(np.float32).astype(np.float64) + c)
    bf16 = _refine(system, _round_bf16(Gd - c) + c)
    assert fp32[0] < 1e-10
    assert bf16[0] > 1e-8 and bf16[1] > 1e-10 and bf16[2] < 1e-10
    # contraction per refinement of the BF16 block: about 1e-3
    assert 1e-4 < bf16[1] / bf16[0] < 1e-2
