"""cosmicblup_gb300 -- GB300-native GBLUP / ssGBLUP hot path behind a C ABI.

The compute lives in ``libcbx.so`` (CUDA for sm_103a + C++ host code, built by
``cosmicblup_gb300.build``); this package is a thin Python mirror of the
reference interfaces used by tests and benchmarks.
"""
from ._lib import CbxError, Handle, lib  # noqa: F401
from .grm import GrmBuilder, GrmOptions, PlinkReader, bed_snp_counts, write_matrix_bin  # noqa: F401
from .mme import DeviceMME  # noqa: F401
from .vce import AIREML, RemlConfig, final_solve, invert_psd, reml_gradient, reml_logl_dense  # noqa: F401
from .ped import ainv_henderson, ssgblup_qinv  # noqa: F401
from .mt import MvEigenVce, MvOptions, solve_multi_trait  # noqa: F401
from .batch import BatchProblem, BatchResult, batch_reml  # noqa: F401
from .geno import DeviceGenotypes  # noqa: F401
from .results import write_beta, write_rand, write_vars  # noqa: F401

__all__ = ["CbxError", "Handle", "lib", "GrmBuilder", "GrmOptions", "PlinkReader",
           "bed_snp_counts", "write_matrix_bin", "DeviceMME", "AIREML", "RemlConfig", "final_solve", "invert_psd",
           "reml_gradient", "reml_logl_dense",
           "ainv_henderson", "ssgblup_qinv", "MvEigenVce", "MvOptions", "solve_multi_trait",
           "BatchProblem", "BatchResult", "batch_reml", "DeviceGenotypes"]
