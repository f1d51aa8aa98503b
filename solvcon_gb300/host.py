"""Page-locked host tables the device maps (not in the reference).

A table exchanged with a core every step (the state a host loop feeds in and
reads back) moves fastest from page-locked memory the device can address:
``scg_euler_set`` / ``scg_euler_get`` then copy it with one kernel and no
staging table, ``EulerCore.deliver`` has a march write its new state into it
as it computes, and ``EulerCore.march_from_host`` uploads it while the
march's first substep already runs.  ``HostTable`` is such a table as a
numpy array (``scg_host_alloc``).
"""

import ctypes

import numpy as np

from ._lib import check, lib

__all__ = ["HostTable"]


class HostTable:
    """A float64 numpy array in page-locked, device-mapped host memory.

    :param shape: the table's shape (an EulerCore array's, ghost rows first).

    ``array`` is valid until :meth:`free` (or the object's collection): keep
    the HostTable alive while the array, or a core it is registered with,
    uses it.
    """

    def __init__(self, shape):
        self.shape = tuple(int(x) for x in np.atleast_1d(shape))
        n = int(np.prod(self.shape))
        self._p = ctypes.c_void_p()
        check(lib.scg_host_alloc(8 * max(n, 1), ctypes.byref(self._p)))
        raw = (ctypes.c_double * max(n, 1)).from_address(self._p.value)
        self.array = np.ctypeslib.as_array(raw)[:n].reshape(self.shape)

    @property
    def address(self):
        """The table's host address (for the C ABI)."""
        return self._p.value

    @property
    def size(self):
        return self.array.size

    def free(self):
        """Release the memory (the array must no longer be used)."""
        if self._p is not None and self._p.value:
            check(lib.scg_host_free(self._p))
        self._p = None
        self.array = None

    def __del__(self):
        try:
            self.free()
        except Exception:  # interpreter shutdown
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.free()
