"""ctypes binding of libcbx.so (the C ABI declared in include/cbx.h).

The library is loaded from the package directory.  There is no fallback:
if it is missing or cannot be loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcbx.so")

CBX_OK = 0
STATUS_NAMES = {
    1: "CBX_ERR_ARG", 2: "CBX_ERR_CUDA", 3: "CBX_ERR_FORMAT", 4: "CBX_ERR_TIMEOUT",
    5: "CBX_ERR_BREAKDOWN", 6: "CBX_ERR_NONFINITE", 7: "CBX_ERR_NOTCONV", 8: "CBX_ERR_FACTOR",
    9: "CBX_ERR_STATE", 10: "CBX_ERR_UNSUPPORTED",
}

_lib = None

i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")

# (name, restype, argtypes) for every C ABI entry point
SIGNATURES = [
    ("cbx_version", C.c_int, []),
    ("cbx_create", C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    ("cbx_destroy", C.c_int, [C.c_void_p]),
    ("cbx_last_error", C.c_char_p, [C.c_void_p]),
    ("cbx_launch_count", C.c_int64, [C.c_void_p]),
    ("cbx_sync", C.c_int, [C.c_void_p]),
    ("cbx_bed_snp_counts", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int64,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("cbx_geno_attach", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_void_p,
                                  C.c_void_p]),
    ("cbx_geno_zt_v", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    ("cbx_geno_z_v", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    ("cbx_snp_effects", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.POINTER(C.c_double)]),
    ("cbx_grm_bed", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_float,
                              C.c_int, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                              C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    ("cbx_write_upper_packed", C.c_int, [C.c_void_p, C.c_int32, C.c_char_p]),
    ("cbx_write_grm_gcta", C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_int64]),
    ("cbx_mme_create", C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.c_void_p, C.c_void_p]),
    ("cbx_mme_set_qinv_dense", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    ("cbx_mme_set_qinv_split", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_int64, C.c_void_p]),
    ("cbx_pcg_solve", C.c_int, [C.c_void_p, C.c_double, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32,
                                C.c_double, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    ("cbx_qinv_apply", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    ("cbx_invert_psd", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_double, C.c_void_p]),
    ("cbx_reml_config_default", None, [C.c_void_p]),
    ("cbx_reml_iterate", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_double),
                                   C.POINTER(C.c_double), C.c_void_p]),
    ("cbx_reml_iterate_grad", C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_double),
                                        C.POINTER(C.c_double), C.c_void_p, C.c_void_p, C.POINTER(C.c_double),
                                        C.POINTER(C.c_int64), C.c_void_p]),
    ("cbx_reml_solve", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                 C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_void_p, C.c_void_p]),
    ("cbx_mme_keep_warm", C.c_int, [C.c_void_p, C.c_int32]),
    ("cbx_profile_enable", C.c_int, [C.c_void_p, C.c_int32]),
    ("cbx_profile_read", C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int64), C.POINTER(C.c_double),
                                   C.POINTER(C.c_double)]),
    ("cbx_timer_start", C.c_int, [C.c_void_p]),
    ("cbx_range_push", C.c_int, [C.c_char_p]),
    ("cbx_range_pop", C.c_int, []),
    ("cbx_timer_stop", C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    ("cbx_ainv_henderson", C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.POINTER(C.c_int64),
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("cbx_ssgblup_qinv", C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                   C.c_void_p, C.c_double, C.c_int32, C.c_double, C.c_double, C.c_double,
                                   C.c_void_p, C.c_void_p]),
    ("cbx_final_solve", C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int32, C.c_double, C.c_int32,
                                  C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("cbx_reml_gradient", C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int32, C.c_int32, C.c_int32,
                                    C.c_int32, C.c_double, C.c_int32, C.c_void_p, C.POINTER(C.c_double),
                                    C.POINTER(C.c_int64)]),
    ("cbx_reml_logl_dense", C.c_int, [C.c_void_p, C.c_double, C.c_double, C.POINTER(C.c_double)]),
    ("cbx_mt_vce", C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                             C.c_int32, C.c_double, C.c_void_p, C.c_void_p, C.POINTER(C.c_int32),
                             C.POINTER(C.c_int32)]),
    ("cbx_mt_solve", C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("cbx_host_register", C.c_int, [C.c_void_p, C.c_int64]),
    ("cbx_host_unregister", C.c_int, [C.c_void_p]),
    ("cbx_tune_enable", C.c_int, [C.c_int32]),
    ("cbx_tune_reset", C.c_int, []),
    ("cbx_tune_report", C.c_int, [C.c_char_p, C.c_int64]),
    ("cbx_dense_apply_noalloc", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    ("cbx_write_vars", C.c_int, [C.c_char_p, C.c_char_p, C.c_double, C.c_double, C.c_double, C.c_double]),
    ("cbx_write_beta", C.c_int, [C.c_char_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("cbx_write_rand", C.c_int, [C.c_char_p, C.c_char_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p,
                                 C.c_void_p]),
    ("cbx_batch_reml", C.c_int, [C.c_int, C.c_int32, C.c_void_p, C.c_float, C.c_void_p, C.c_int32, C.c_void_p]),
    # diagnostics and self-test exports (not in the public header)
    ("cbx_trace_enable", C.c_int, [C.c_void_p, C.c_int32]),
    ("cbx_trace_read", C.c_int, [C.c_void_p, C.c_char_p, C.c_int64]),
    ("cbx_selftest_umma", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("cbx_selftest_dense_ff", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_int32,
                                        C.c_int32, C.c_int32, C.c_void_p, C.POINTER(C.c_double)]),
    ("cbx_selftest_dense_tc", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_int32,
                                        C.c_void_p]),
    ("cbx_selftest_dense_fx", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_int32,
                                        C.c_int32, C.c_void_p, C.POINTER(C.c_double)]),
    ("cbx_selftest_wait_timeout", C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_double)]),
]


class CbxError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def lib() -> C.CDLL:
    """Load libcbx.so once; raise if it is not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is not built; run `python -m cosmicblup_gb300.build`")
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def ptr(a: np.ndarray | None) -> C.c_void_p | None:
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "arrays passed to libcbx must be C-contiguous"
    return C.c_void_p(a.ctypes.data)


class Handle:
    """Owns one cbx_handle (one CUDA stream on one device)."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        rc = lib().cbx_create(device, C.byref(self._h))
        if rc != CBX_OK:
            msg = lib().cbx_last_error(self._h).decode() if self._h else "cbx_create failed"
            if self._h:
                lib().cbx_destroy(self._h)
            self._h = None
            raise CbxError(rc, msg)

    @property
    def raw(self) -> C.c_void_p:
        if self._h is None:
            raise RuntimeError("handle closed")
        return self._h

    def check(self, rc: int) -> None:
        if rc != CBX_OK:
            raise CbxError(rc, lib().cbx_last_error(self._h).decode())

    def keep_warm(self, on: bool) -> None:
        """MMEs rebuilt later with the same shape start their solves from the
        previous MME's last data and probe solutions (cbx_mme_keep_warm)."""
        self.check(lib().cbx_mme_keep_warm(self.raw, 1 if on else 0))

    def profile(self, on: bool) -> None:
        self.check(lib().cbx_profile_enable(self.raw, 1 if on else 0))

    def profile_read(self, bucket: int) -> tuple[int, float, float]:
        n, ms, b = C.c_int64(0), C.c_double(0), C.c_double(0)
        self.check(lib().cbx_profile_read(self.raw, bucket, C.byref(n), C.byref(ms), C.byref(b)))
        return n.value, ms.value, b.value

    def timer_start(self) -> None:
        self.check(lib().cbx_timer_start(self.raw))

    def timer_stop(self) -> float:
        ms = C.c_double(0)
        self.check(lib().cbx_timer_stop(self.raw, C.byref(ms)))
        return ms.value

    def trace(self, on: bool) -> None:
        """Start (or stop) the per-launch trace of this handle's stream."""
        self.check(lib().cbx_trace_enable(self.raw, 1 if on else 0))

    def trace_read(self) -> list[tuple[str, int, float]]:
        """(kernel, launches, ms) since the trace started, most expensive first;
        each launch is charged the time since the previous one finished."""
        buf = C.create_string_buffer(1 << 16)
        self.check(lib().cbx_trace_read(self.raw, buf, len(buf)))
        out = []
        for line in buf.value.decode().splitlines():
            name, cnt, ms = line.split("\t")
            out.append((name, int(cnt), float(ms)))
        return out

    def launches(self) -> int:
        return int(lib().cbx_launch_count(self.raw))

    def sync(self) -> None:
        self.check(lib().cbx_sync(self.raw))

    def close(self) -> None:
        if self._h is not None:
            lib().cbx_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tune_enable(on: bool) -> None:
    """Switch the launch-shape autotuner on or off for the whole process."""
    lib().cbx_tune_enable(1 if on else 0)


def tune_reset() -> None:
    lib().cbx_tune_reset()


def tune_report() -> list[str]:
    """One line per autotuner decision (kernel, device, size classes, width, choice, ms)."""
    buf = C.create_string_buffer(1 << 16)
    lib().cbx_tune_report(buf, len(buf))
    return [ln for ln in buf.value.decode().splitlines() if ln]


class pinned:
    """Context manager page-locking numpy arrays for the duration (cbx_host_register):
    the library's host <-> device copies of them then run at the link's full rate.
    Arrays that cannot be registered are left pageable."""

    def __init__(self, *arrays):
        self.arrays = [a for a in arrays if a is not None and a.nbytes > 0]
        self.done = []

    def __enter__(self):
        for a in self.arrays:
            if lib().cbx_host_register(C.c_void_p(a.ctypes.data), a.nbytes) == CBX_OK:
                self.done.append(a)
        return self

    def __exit__(self, *exc):
        for a in self.done:
            lib().cbx_host_unregister(C.c_void_p(a.ctypes.data))
        self.done = []

