"""CPU oracle for the GBLUP/ssGBLUP hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, in numpy (and a little C), the arithmetic of the
CosmicBLUP reference path so that the CUDA implementation in
``cosmicblup_gb300`` can be checked against it.  It is imported only by
``tests/``, by ``__graft_entry__.smoke()`` and by the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py``; the product never calls it.

Parity status
-------------
The reference (C++17 + Eigen 3) cannot be built in this environment (no Eigen
headers), so most of this restatement is *pinned only partially*:

* BED decoding, SNP statistics and the VanRaden GRM are pinned against the
  reference's own fixture ``tests/fixtures/toy_plink/toy.bed`` (bytes and
  decoded genotypes) and the known-answer integer cross-products of that
  fixture; the FP64 GRM values for it are a restatement, not reference output.
* The Rademacher probe stream is pinned against the reference's own
  ``src/core/rng.h`` and ``src/core/adaptive_trace_estimator.cpp``, compiled
  from the reference tree with a minimal vector shim (``oracle/ref_trace``).
* PCG, MME assembly, EM/AI-REML and A-inverse are restatements of the cited
  reference lines; no reference output exists to pin them ("parity unpinned").
"""
