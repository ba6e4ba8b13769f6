"""Generate ``toy_grm.json``: known answers for the reference's 6 x 4 toy BED.

Run from the repository root: ``python tests/golden/make_toy_golden.py [REFERENCE_DIR]``
(default: the checkout oracle/build.py uses).

The reference ships ``tests/fixtures/toy_plink/toy.bed`` (6 samples, 4 SNPs,
SNP-major).  This script reads that file from the reference checkout, checks
that the oracle decodes it to the genotypes the reference documents and that
this repository's BED writer reproduces it byte for byte, and stores:

* the decoded genotypes (so tests rebuild the BED without the reference tree),
* the integer cross-products X X^T (exact, the bit-exact target of the GRM),
* the FP64 VanRaden G and sum 2pq as restated by the oracle from
  src/core/grm_builder.cpp:166-404 (a restatement, not reference output).
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.plink import decode_bed  # noqa: E402
from oracle.grm import vanraden_grm, vanraden_grm_exact, xx_counts  # noqa: E402
from cosmicblup_gb300.synth import encode_bed  # noqa: E402

from oracle.build import REFERENCE  # noqa: E402

REF_BED = os.path.join(sys.argv[1] if len(sys.argv) > 1 else REFERENCE, "tests", "fixtures", "toy_plink",
                       "toy.bed")
DOCUMENTED = [[0, 1, 2, 0, 1, 2], [1, 1, 0, 2, 2, 1], [2, 2, 1, 0, 1, 0], [0, 1, 2, 1, 0, 2]]


def main() -> None:
    bed = open(REF_BED, "rb").read()
    geno = decode_bed(bed, 6, 4)
    assert geno.tolist() == DOCUMENTED, geno
    assert encode_bed(geno) == bed, "BED writer does not reproduce the reference fixture"
    r = vanraden_grm(bed, 6, 4)
    e = vanraden_grm_exact(bed, 6, 4)
    out = {
        "source": "reference tests/fixtures/toy_plink/toy.bed (6 samples x 4 SNPs)",
        "n": 6, "m": 4,
        "bed_hex": bed.hex(),
        "genotypes_snp_major": geno.tolist(),
        "xx_counts": xx_counts(bed, 6, 4).tolist(),
        "sum2pq": r["sum2pq"],
        "n_valid": r["n_valid"],
        "allele_freqs": [float(v) for v in r["freq"]],
        "G_restated": r["G"].tolist(),
        "G_exact_rounded": e["G"].tolist(),
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "toy_grm.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
