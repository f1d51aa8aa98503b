"""Ghost-aware array view with the indexing rules of solvcon's SimpleArray.

solvcon's ``SimpleArray`` (cpp/solvcon/buffer/SimpleArray.hpp, bound in
cpp/solvcon/buffer/pymod/wrap_SimpleArray.hpp:97-214 and
array_common.hpp:180-460) stores ghost rows before the body rows of its first
axis and addresses them with negative indices: ``arr[-1]`` is the last ghost
row, ``arr[0]`` the first body row.  ``arr.ndarray`` is the whole buffer,
ghost rows first.  This class gives the same view over a numpy buffer, which
is either a live host table (mesh arrays) or a host mirror of a device table
kept coherent by its owner (solver arrays).
"""

import numpy as np

__all__ = ["SimpleArray"]


class SimpleArray:
    """A view of one table with ``nghost`` leading ghost rows.

    :param fetch: callable returning the whole numpy buffer (ghost rows
        first); it is called on every access so the owner can refresh it.
    :param nghost: ghost rows on the first axis.
    :param on_write: called after every write made through this view.
    :param on_expose: called whenever :attr:`ndarray` hands the buffer out
        (the caller may keep it and write through it at any time); defaults
        to ``on_write``.
    """

    def __init__(self, fetch, nghost=0, on_write=None, on_expose=None):
        self._fetch = fetch
        self._nghost = int(nghost)
        self._on_write = on_write
        self._on_expose = on_expose if on_expose is not None else on_write

    # -- buffer -------------------------------------------------------------

    def _buf(self):
        return self._fetch()

    @property
    def ndarray(self):
        """The whole buffer, ghost rows first (writes go to the table)."""
        buf = self._buf()
        if self._on_expose is not None:
            self._on_expose()
        return buf

    def __array__(self, dtype=None, copy=None):
        buf = self._buf()
        return buf if dtype is None else buf.astype(dtype)

    @property
    def nghost(self):
        return self._nghost

    @property
    def nbody(self):
        return self.shape[0] - self._nghost

    @property
    def shape(self):
        return tuple(self._buf().shape)

    @property
    def ndim(self):
        return self._buf().ndim

    @property
    def size(self):
        return self._buf().size

    @property
    def dtype(self):
        return self._buf().dtype

    @property
    def body(self):
        """The body rows (a view; writes go to the table)."""
        return self.ndarray[self._nghost:]

    def __len__(self):
        return self._buf().shape[0]

    def __repr__(self):
        return "SimpleArray(shape=%s, nghost=%d)" % (self.shape, self._nghost)

    # -- indexing -----------------------------------------------------------

    def _row(self, i, nrow):
        j = int(i) + self._nghost
        if j < 0 or j >= nrow:
            raise IndexError("index %d out of range [%d, %d)" % (
                int(i), -self._nghost, nrow - self._nghost))
        return j

    def _map(self, key, nrow):
        if self._nghost == 0:
            return key
        tup = isinstance(key, tuple)
        first = key[0] if tup else key
        rest = key[1:] if tup else ()
        if isinstance(first, (int, np.integer)):
            first = self._row(first, nrow)
        elif isinstance(first, slice):
            start = None if first.start is None else first.start + self._nghost
            stop = None if first.stop is None else first.stop + self._nghost
            first = slice(start, stop, first.step)
        elif first is Ellipsis:
            pass
        else:
            arr = np.asarray(first)
            if arr.dtype.kind in "iu":
                first = arr + self._nghost
        return (first,) + rest if tup else first

    def __getitem__(self, key):
        buf = self._buf()
        out = buf[self._map(key, buf.shape[0])]
        return out.item() if isinstance(out, np.generic) else out

    def __setitem__(self, key, value):
        buf = self._buf()
        buf[self._map(key, buf.shape[0])] = value
        if self._on_write is not None:
            self._on_write()

    def copy(self):
        """A numpy copy of the whole buffer."""
        return np.array(self._buf(), copy=True)

    def tolist(self):
        return self._buf().tolist()

    def fill(self, value):
        buf = self._buf()
        buf.fill(value)
        if self._on_write is not None:
            self._on_write()

    # numpy-style comparisons return boolean arrays over the whole buffer.
    def __lt__(self, other):
        return self._buf() < other

    def __le__(self, other):
        return self._buf() <= other

    def __gt__(self, other):
        return self._buf() > other

    def __ge__(self, other):
        return self._buf() >= other
