"""Host buffers for the host-buffer calls (fftso3_forward_host / fftso3_inverse_host).

host_empty(n, dtype) returns a CPU tensor of n elements in page-locked memory backed by transparent huge pages:
an anonymous mapping aligned to 2 MB, advised MADV_HUGEPAGE, touched, then registered with CUDA
(cudaHostRegister).  Copies to and from such a buffer run at the host link's speed every time; page-locked memory
made of 4 KB pages (what cudaHostAlloc returns once the host's memory is fragmented) was measured to cross the
link at half that speed in some calls.  The registration is undone and the mapping released when the tensor is
garbage-collected.
"""
from __future__ import annotations

import ctypes
import mmap
import weakref

_HUGE = 2 << 20
_MADV_HUGEPAGE = 14
_libc = None


class _HostMapping:
    """an aligned, registered anonymous mapping; owns its release"""

    def __init__(self, nbytes: int):
        import torch

        global _libc
        if _libc is None:
            _libc = ctypes.CDLL(None, use_errno=True)
        if not torch.cuda.is_available():
            raise RuntimeError("host_empty: page-locked host buffers need a CUDA device")
        self.size = max(int(nbytes), 1)
        span = (self.size + _HUGE - 1) // _HUGE * _HUGE
        self.map = mmap.mmap(-1, span + _HUGE, flags=mmap.MAP_PRIVATE | mmap.MAP_ANONYMOUS)
        base = ctypes.addressof(ctypes.c_char.from_buffer(self.map))
        self.addr = (base + _HUGE - 1) // _HUGE * _HUGE
        self.offset = self.addr - base
        _libc.madvise(ctypes.c_void_p(self.addr), ctypes.c_size_t(span), _MADV_HUGEPAGE)
        view = memoryview(self.map)[self.offset:self.offset + span]
        for i in range(0, span, _HUGE):  # fault the pages in (one touch per 2 MB)
            view[i] = 0
        view.release()
        rc = torch.cuda.cudart().cudaHostRegister(self.addr, span, 0)
        if int(rc) != 0:
            self.map.close()
            raise RuntimeError(f"host_empty: cudaHostRegister failed ({rc})")
        self.span = span

    def release(self):
        import torch

        if self.map is not None:
            torch.cuda.cudart().cudaHostUnregister(self.addr)
            self.map = None


def host_empty(n: int, dtype=None):
    """A CPU tensor of n elements of dtype (default complex64) in registered, huge-page-backed host memory."""
    import torch

    dtype = dtype or torch.complex64
    esize = torch.empty(0, dtype=dtype).element_size()
    m = _HostMapping(n * esize)
    buf = (ctypes.c_char * (n * esize)).from_address(m.addr)
    t = torch.frombuffer(buf, dtype=torch.uint8, count=n * esize).view(dtype)
    t._fftso3_host_mapping = m  # keep the mapping alive as long as the tensor
    weakref.finalize(t, m.release)
    return t
