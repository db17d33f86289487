"""ctypes binding of ``libfftso3_gb300.so`` (the C ABI in include/fftso3_gb300.h).

The shared library is the only compute path: if it is missing this module
raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfftso3_gb300.so")

# constants mirrored from include/fftso3_gb300.h
SUCCESS = 0
ERR_INVALID_ARG = 1
ERR_CUDA = 2
ERR_OOM = 3
ERR_UNSUPPORTED = 4
ERR_NO_DEVICE = 5

SO3_COMPLEX = 0
SO3_REAL = 1
S2_COMPLEX = 2
S2_REAL = 3

PREC_FP64 = 0
PREC_TC_BF16X3 = 1
PREC_FP32 = 2

RECURSION_REFERENCE = 0
RECURSION_STABLE = 1

FLAG_REFINE = 0x1
FLAG_GRAPH = 0x2
FLAG_AUTOTUNE = 0x4
FLAG_EXACT_INVERSE = 0x8

PRECISIONS = {"fp64": PREC_FP64, "tc_bf16x3": PREC_TC_BF16X3, "fp32": PREC_FP32}
RECURSIONS = {"reference": RECURSION_REFERENCE, "stable": RECURSION_STABLE}

# every symbol the header declares: name -> (restype, argtypes)
_vp = ctypes.c_void_p
_i = ctypes.c_int
_ll = ctypes.c_longlong
_d = ctypes.c_double
_dp = ctypes.POINTER(ctypes.c_double)
SIGNATURES = {
    "fftso3_last_error_string": (ctypes.c_char_p, []),
    "fftso3_version": (_i, []),
    "fftso3_grid_elems": (_ll, [_i, _i]),
    "fftso3_coeff_elems": (_ll, [_i, _i]),
    "fftso3_weights": (_i, [_i, _i, _dp]),
    "fftso3_plan_create": (_i, [ctypes.POINTER(_vp), _i, _i, _i, _i, _i, ctypes.c_uint]),
    "fftso3_plan_destroy": (_i, [_vp]),
    "fftso3_plan_device_bytes": (_ll, [_vp]),
    "fftso3_plan_check": (_i, [_vp]),
    "fftso3_plan_set_timing": (_i, [_vp, _i]),
    "fftso3_stage_count": (_i, []),
    "fftso3_stage_name": (ctypes.c_char_p, [_i]),
    "fftso3_plan_stage_times": (_i, [_vp, _dp, ctypes.POINTER(_ll), _i]),
    "fftso3_forward": (_i, [_vp, _vp, _vp, _vp]),
    "fftso3_inverse": (_i, [_vp, _vp, _vp, _vp]),
    "fftso3_forward_host": (_i, [_vp, _vp, _vp, _vp]),
    "fftso3_inverse_host": (_i, [_vp, _vp, _vp, _vp]),
    "fftso3_inverse_points": (_i, [_vp, _vp, _i, _dp, _i, _vp, _vp]),
    "fftso3_wigner_d": (_i, [_d, _i, _i, _dp]),
    "fftso3_derivative": (_i, [_vp, _vp, _i, _vp, _vp]),
    "fftso3_clebsch_gordan": (_i, [_i, _i, _i, _vp]),
    "fftso3_forward_noalloc": (_i, [_i, _vp, _vp, _vp]),
    "fftso3_correlate_s2": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "fftso3_grid_argmax": (_i, [_vp, _vp, ctypes.POINTER(_ll), _dp, _vp]),
    "fftso3_batch_create": (_i, [ctypes.POINTER(_vp), _i, ctypes.POINTER(_i), _i, _i, _i, ctypes.c_uint]),
    "fftso3_batch_destroy": (_i, [_vp]),
    "fftso3_batch_grid_offset": (_ll, [_vp, _i]),
    "fftso3_batch_coeff_offset": (_ll, [_vp, _i]),
    "fftso3_batch_bucket_count": (_i, [_vp]),
    "fftso3_batch_stream_count": (_i, [_vp]),
    "fftso3_batch_graph_kernels": (_i, [_vp, _i]),
    "fftso3_batch_device_bytes": (_ll, [_vp]),
    "fftso3_batch_forward": (_i, [_vp, _vp, _vp, _vp]),
    "fftso3_batch_inverse": (_i, [_vp, _vp, _vp, _vp]),
    "fftso3_batch_bucket_info": (_i, [_vp, _i, ctypes.POINTER(_i), ctypes.POINTER(_i)]),
    "fftso3_batch_set_timing": (_i, [_vp, _i]),
    "fftso3_batch_stage_times": (_i, [_vp, _i, _dp, ctypes.POINTER(_ll), _i]),
    "fftso3_batch_check": (_i, [_vp]),
    "fftso3_grid_fft_workspace_bytes": (ctypes.c_size_t, [_i, _ll]),
    "fftso3_grid_fft": (_i, [_i, _ll, _i, _i, _vp, _vp, _vp, _vp]),
    "fftso3_grid_fft_check": (_i, [_vp, _vp]),
    "fftso3_grid_fft_reset": (_i, [_vp, _vp]),
}

_lib = None


class FFTSO3Error(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"fftso3 error {code}: {msg}")
        self.code = code


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build the CUDA library first "
                "(python -m fftso3_gb300.build, or __graft_entry__.build())"
            )
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != SUCCESS:
        msg = lib().fftso3_last_error_string().decode(errors="replace")
        raise FFTSO3Error(rc, msg)


def grid_fft_workspace_bytes(N: int, nf: int) -> int:
    """Device workspace (bytes) of grid_fft for nf grids of N^3 samples (0: unsupported N)."""
    return int(lib().fftso3_grid_fft_workspace_bytes(int(N), int(nf)))


def grid_fft(N: int, nf: int, direction: int, real: bool, src: int, dst: int, workspace: int, stream: int = 0) -> None:
    """The grid FFT stage alone (fftso3_grid_fft): direction 1 grids -> pencils, -1 pencils -> grids;
    device pointers, asynchronous on `stream`; workspace zeroed before its first use."""
    check(lib().fftso3_grid_fft(int(N), int(nf), int(direction), 1 if real else 0, src, dst, workspace, stream))


def grid_fft_check(workspace: int, stream: int = 0) -> None:
    check(lib().fftso3_grid_fft_check(workspace, stream))


def clebsch_gordan(l1: int, l2: int, real: bool = False):
    """The Clebsch-Gordan matrix of (l1, l2) computed on the GPU (fftso3_clebsch_gordan): (n, n) float64 for
    the complex harmonics, complex128 for the real harmonics, n = (2 l1 + 1)(2 l2 + 1)."""
    import numpy as np

    n = (2 * int(l1) + 1) * (2 * int(l2) + 1)
    out = np.empty((n, n), dtype=np.complex128 if real else np.float64, order="F")
    check(lib().fftso3_clebsch_gordan(int(l1), int(l2), 1 if real else 0, out.ctypes.data))
    return out


class Plan:
    """Owns one ``fftso3_plan`` (tables and workspace on the current device)."""

    def __init__(self, kind: int, l_max: int, batch: int = 1, precision: str | int = "fp64",
                 recursion: str | int = "reference", flags: int = 0):
        self.kind = kind
        self.l_max = int(l_max)
        self.batch = int(batch)
        self.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        self.recursion = RECURSIONS[recursion] if isinstance(recursion, str) else int(recursion)
        self.flags = int(flags)
        h = _vp()
        check(lib().fftso3_plan_create(ctypes.byref(h), kind, self.l_max, self.batch, self.precision,
                                       self.recursion, ctypes.c_uint(self.flags)))
        self._h = h

    @property
    def handle(self):
        return self._h

    @property
    def grid_elems(self) -> int:
        return int(lib().fftso3_grid_elems(self.kind, self.l_max))

    @property
    def coeff_elems(self) -> int:
        return int(lib().fftso3_coeff_elems(self.kind, self.l_max))

    @property
    def device_bytes(self) -> int:
        return int(lib().fftso3_plan_device_bytes(self._h))

    def forward(self, grid_ptr: int, coeff_ptr: int, stream: int = 0) -> None:
        check(lib().fftso3_forward(self._h, _vp(grid_ptr), _vp(coeff_ptr), _vp(stream)))

    def inverse(self, coeff_ptr: int, grid_ptr: int, stream: int = 0) -> None:
        check(lib().fftso3_inverse(self._h, _vp(coeff_ptr), _vp(grid_ptr), _vp(stream)))

    def forward_host(self, grid_ptr: int, coeff_ptr: int, stream: int = 0) -> None:
        check(lib().fftso3_forward_host(self._h, _vp(grid_ptr), _vp(coeff_ptr), _vp(stream)))

    def inverse_host(self, coeff_ptr: int, grid_ptr: int, stream: int = 0) -> None:
        check(lib().fftso3_inverse_host(self._h, _vp(coeff_ptr), _vp(grid_ptr), _vp(stream)))

    def inverse_points(self, coeff_ptr: int, index: int, pts, n: int, out_ptr: int, stream: int = 0) -> None:
        check(lib().fftso3_inverse_points(self._h, _vp(coeff_ptr), int(index), pts, int(n), _vp(out_ptr),
                                          _vp(stream)))

    def derivative(self, coeff_ptr: int, axis: int, out_ptr: int, stream: int = 0) -> None:
        """Coefficients of d/dt f(R exp(t e_axis)) for the batch (fftso3_derivative)."""
        check(lib().fftso3_derivative(self._h, _vp(coeff_ptr), int(axis), _vp(out_ptr), _vp(stream)))

    def correlate_s2(self, F_ptr: int, G_ptr: int, grid_ptr: int, stream: int = 0) -> None:
        check(lib().fftso3_correlate_s2(self._h, _vp(F_ptr), _vp(G_ptr), _vp(grid_ptr), _vp(stream)))

    def grid_argmax(self, grid_ptr: int, stream: int = 0) -> tuple:
        """(flat indices, values) of the maximum of each of the batch's real grids."""
        idx = (_ll * self.batch)()
        val = (ctypes.c_double * self.batch)()
        check(lib().fftso3_grid_argmax(self._h, _vp(grid_ptr), idx, val, _vp(stream)))
        return list(idx), list(val)

    def set_timing(self, enable: bool = True) -> None:
        check(lib().fftso3_plan_set_timing(self._h, 1 if enable else 0))

    def stage_times(self, reset: bool = False) -> dict:
        """{stage name: (total ms, launches)} of the timed launches so far."""
        n = lib().fftso3_stage_count()
        ms = (ctypes.c_double * n)()
        cnt = (_ll * n)()
        check(lib().fftso3_plan_stage_times(self._h, ms, cnt, 1 if reset else 0))
        return {lib().fftso3_stage_name(i).decode(): (ms[i], cnt[i]) for i in range(n) if cnt[i]}

    def check(self) -> None:
        """Synchronise and raise if an earlier asynchronous call failed."""
        check(lib().fftso3_plan_check(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and _lib is not None:
            _lib.fftso3_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Owns one ``fftso3_batch``: functions of one kind with per-function l_max.

    The batch chooses where each function lives in the grid and coefficient
    buffers (``grid_offset(i)`` / ``coeff_offset(i)``, in elements; ``i = n``
    gives the totals).
    """

    def __init__(self, kind: int, l_max, precision: str | int = "fp64", recursion: str | int = "reference",
                 flags: int = 0):
        self.kind = kind
        self.l_max = [int(x) for x in l_max]
        self.n = len(self.l_max)
        self.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        self.recursion = RECURSIONS[recursion] if isinstance(recursion, str) else int(recursion)
        self.flags = int(flags)
        arr = (_i * max(self.n, 1))(*self.l_max)
        h = _vp()
        check(lib().fftso3_batch_create(ctypes.byref(h), kind, arr, self.n, self.precision, self.recursion,
                                        ctypes.c_uint(self.flags)))
        self._h = h

    def grid_offset(self, i: int) -> int:
        return int(lib().fftso3_batch_grid_offset(self._h, int(i)))

    def coeff_offset(self, i: int) -> int:
        return int(lib().fftso3_batch_coeff_offset(self._h, int(i)))

    @property
    def grid_elems(self) -> int:
        return self.grid_offset(self.n)

    @property
    def coeff_elems(self) -> int:
        return self.coeff_offset(self.n)

    @property
    def buckets(self) -> int:
        return int(lib().fftso3_batch_bucket_count(self._h))

    @property
    def streams(self) -> int:
        return int(lib().fftso3_batch_stream_count(self._h))

    @property
    def device_bytes(self) -> int:
        return int(lib().fftso3_batch_device_bytes(self._h))

    def graph_kernels(self, direction: int) -> int:
        """Kernel nodes of the captured CUDA graph of direction 0 (forward) / 1 (inverse); -1 if none."""
        return int(lib().fftso3_batch_graph_kernels(self._h, int(direction)))

    def forward(self, grid_ptr: int, coeff_ptr: int, stream: int = 0) -> None:
        check(lib().fftso3_batch_forward(self._h, _vp(grid_ptr), _vp(coeff_ptr), _vp(stream)))

    def inverse(self, coeff_ptr: int, grid_ptr: int, stream: int = 0) -> None:
        check(lib().fftso3_batch_inverse(self._h, _vp(coeff_ptr), _vp(grid_ptr), _vp(stream)))

    def bucket_info(self, k: int) -> tuple:
        L, c = _i(), _i()
        check(lib().fftso3_batch_bucket_info(self._h, int(k), ctypes.byref(L), ctypes.byref(c)))
        return L.value, c.value

    def set_timing(self, enable: bool = True) -> None:
        check(lib().fftso3_batch_set_timing(self._h, 1 if enable else 0))

    def stage_times(self, bucket: int = -1, reset: bool = False) -> dict:
        """{stage name: (total ms, launches)} summed over buckets (bucket = -1) or for one bucket."""
        n = lib().fftso3_stage_count()
        ms = (ctypes.c_double * n)()
        cnt = (_ll * n)()
        check(lib().fftso3_batch_stage_times(self._h, int(bucket), ms, cnt, 1 if reset else 0))
        return {lib().fftso3_stage_name(i).decode(): (ms[i], cnt[i]) for i in range(n) if cnt[i]}

    def check(self) -> None:
        check(lib().fftso3_batch_check(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and _lib is not None:
            _lib.fftso3_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
