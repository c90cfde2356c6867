"""Page-locked host arrays for the host-buffer entry points.

`idg_imaging_cycle` (and the server's jobs) copy visibilities between host
buffers and the device while the kernels run, so the cycle's end-to-end rate
follows the host copy rate.  Memory from cudaHostAlloc (torch's
``pin_memory=True``) is locked in base pages, 64 KB on the Arm hosts of GB300
systems.  Once a process has churned host memory, copies from such buffers
were measured at 64-124 GB/s, against 211 GB/s host to device and 193 GB/s
device to host when the same bytes sit in transparent huge pages (512 MB on
those hosts).  `pinned_empty` maps anonymous memory, advises it for huge pages,
touches it and registers it with cudaHostRegister; `release` unregisters it.
"""
from __future__ import annotations

import mmap
import threading

import numpy as np

_registered: dict[int, int] = {}  # data pointer -> registered bytes
_lock = threading.Lock()


def _cudart():
    import torch

    return torch.cuda.cudart()


def pinned_empty(shape, dtype, register: bool = True) -> np.ndarray:
    """A zeroed C-contiguous numpy array in huge-page-advised memory, registered
    with CUDA (page-locked, mapped for copies) unless ``register`` is False.
    Raises RuntimeError when the registration fails."""
    dtype = np.dtype(dtype)
    shape = tuple(int(s) for s in (shape if isinstance(shape, (tuple, list)) else (shape,)))
    nbytes = int(np.prod(shape, dtype=np.int64)) * dtype.itemsize
    size = max(nbytes, 1)
    m = mmap.mmap(-1, size, flags=mmap.MAP_PRIVATE | mmap.MAP_ANONYMOUS)
    if hasattr(m, "madvise") and hasattr(mmap, "MADV_HUGEPAGE"):
        try:
            m.madvise(mmap.MADV_HUGEPAGE)
        except OSError:
            pass  # no transparent huge pages: base pages still work, at the base-page rate
    flat = np.frombuffer(m, dtype=np.uint8, count=size)
    flat[:] = 0  # fault the pages in before they are locked
    arr = flat[:nbytes].view(dtype).reshape(shape)
    if register:
        ptr = flat.ctypes.data
        rc = _cudart().cudaHostRegister(ptr, size, 0)
        if int(getattr(rc, "value", rc)) != 0:
            raise RuntimeError(f"cudaHostRegister of {size} bytes failed: {rc}")
        with _lock:
            _registered[ptr] = size
    return arr


def pinned_copy(a: np.ndarray, register: bool = True) -> np.ndarray:
    """`pinned_empty` filled with a copy of ``a``."""
    a = np.asarray(a)
    out = pinned_empty(a.shape, a.dtype, register)
    out[...] = a
    return out


def release(arr: np.ndarray) -> None:
    """Unregister an array from `pinned_empty` (no-op for one that was not
    registered).  The mapping is freed with the last reference to the array."""
    base = arr
    while isinstance(base.base, np.ndarray):
        base = base.base
    ptr = base.ctypes.data
    with _lock:
        size = _registered.pop(ptr, None)
    if size is not None:
        _cudart().cudaHostUnregister(ptr)


def huge_page_bytes() -> int:
    """Anonymous memory of this host currently in transparent huge pages
    (AnonHugePages of /proc/meminfo), in bytes; 0 where it is not reported."""
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("AnonHugePages:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 0
