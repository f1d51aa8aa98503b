"""Solution tables exchanged through page-locked, mapped host blocks.

``scg_euler_get`` / ``scg_euler_set`` on a host table that lies inside a
block from ``scg_host_alloc`` skip the device staging copy: one kernel
gathers the records straight into the host table (or scatters the host
table into the records) over the host link.  Every other host pointer goes
through the staging copy.  Both routes must give the same tables, bit for
bit, and a march continued after either route must give the same state.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RECORD_TABLES = {"so0c": 4, "so0n": 5, "so0t": 6, "so1c": 7, "so1n": 8}


class _Block:
    """A scg_host_alloc block with a float64 view starting ``skip`` values
    into it (skip = 1 gives a table that is 8- but not 16-byte aligned)."""

    def __init__(self, nvalue, skip=0):
        from solvcon_gb300._lib import check, lib
        self._lib = lib
        self.ptr = ctypes.c_void_p()
        check(lib.scg_host_alloc(8 * (nvalue + skip), ctypes.byref(self.ptr)))
        raw = (ctypes.c_double * (nvalue + skip)).from_address(self.ptr.value)
        self.view = np.ctypeslib.as_array(raw)[skip:]
        self.addr = self.ptr.value + 8 * skip

    def free(self):
        from solvcon_gb300._lib import check
        check(self._lib.scg_host_free(self.ptr))


def _marched_core(precision, ndim):
    import solvcon_gb300 as sg
    from solvcon_gb300 import meshgen
    if ndim == 2:
        x, t, c = meshgen.tri_square(24, 0.2, 3)
    else:
        x, t, c = meshgen.tet_cube(6, 0.15, 3)
    mesh = meshgen.build_mesh(ndim, x, t, c)
    ec = sg.EulerCore(mesh=mesh, time_increment=2e-3, precision=precision)
    clcnd = np.array(mesh.clcnd.ndarray)[mesh.ngstcell:]
    state = (meshgen.quadrant_state(clcnd, seed=5) if ndim == 2
             else meshgen.blast_state(clcnd))
    ec.add_slipwall([int(f) for f in mesh.bndfcs.ndarray[:, 0]])
    meshgen.set_state(ec, mesh, state, 1.4)
    ec.march(3)
    # From here on the tables move only through the C ABI calls below.
    ec.release_views()
    return ec


def _get(core, which, shape):
    """A table through the staging route (a pageable numpy table)."""
    from solvcon_gb300._lib import check, lib, ptr
    out = np.empty(shape, dtype="float64")
    check(lib.scg_euler_get(core.handle, which, ptr(out), out.size))
    return out


def _shape(core, name):
    total = core.ncell + core.ngstcell
    if name.startswith("so1"):
        return (total, core.neq, core.ndim)
    if name.startswith("so0"):
        return (total, core.neq)
    return (total,)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("ndim", [2, 3])
@pytest.mark.parametrize("skip", [0, 1])
def test_get_through_mapped_block_equals_staged(precision, ndim, skip):
    from solvcon_gb300._lib import check, lib
    ec = _marched_core(precision, ndim)
    for name, which in RECORD_TABLES.items():
        staged = _get(ec, which, _shape(ec, name))
        blk = _Block(staged.size, skip)
        try:
            blk.view[...] = np.nan
            check(lib.scg_euler_get(ec.handle, which, ctypes.c_void_p(blk.addr),
                                    staged.size))
            np.testing.assert_array_equal(blk.view.reshape(staged.shape),
                                          staged, err_msg=name)
        finally:
            blk.free()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("ndim", [2, 3])
@pytest.mark.parametrize("skip", [0, 1])
def test_set_through_mapped_block_equals_staged(precision, ndim, skip):
    from solvcon_gb300._lib import check, lib, ptr
    a = _marched_core(precision, ndim)
    b = _marched_core(precision, ndim)
    rng = np.random.default_rng(11)
    for name in ("so0n", "so1n"):
        which = RECORD_TABLES[name]
        cur = _get(a, which, _shape(a, name))
        new = cur * (1.0 + 1e-3 * rng.standard_normal(cur.shape))
        # a: staging route (a pageable numpy table).
        check(lib.scg_euler_set(a.handle, which, ptr(new), new.size))
        # b: mapped route.
        blk = _Block(new.size, skip)
        try:
            blk.view[...] = new.ravel()
            check(lib.scg_euler_set(b.handle, which, ctypes.c_void_p(blk.addr),
                                    new.size))
        finally:
            blk.free()
        np.testing.assert_array_equal(_get(b, which, new.shape),
                                      _get(a, which, new.shape), err_msg=name)
        # so0t is untouched by either route (the mapped so1n route makes
        # the new state's so0t in the record the march reads next).
        np.testing.assert_array_equal(_get(b, 6, _shape(b, "so0t")),
                                      _get(a, 6, _shape(a, "so0t")))
    a.march(2)
    b.march(2)
    for name in ("so0n", "so1n", "cflo"):
        which = {"so0n": 5, "so1n": 8, "cflo": 10}[name]
        shape = _shape(a, name)
        np.testing.assert_array_equal(_get(b, which, shape),
                                      _get(a, which, shape), err_msg=name)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_mapped_so1n_after_update_keeps_so0t(precision):
    """After update() the logical so0t lives in the buffer so1n is written
    to; the mapped route must then leave it alone."""
    from solvcon_gb300._lib import check, lib, ptr
    a = _marched_core(precision, 2)
    b = _marched_core(precision, 2)
    a.update()
    b.update()
    a.release_views()
    b.release_views()
    new = _get(a, 8, _shape(a, "so1n")) * 1.001
    check(lib.scg_euler_set(a.handle, 8, ptr(new), new.size))
    blk = _Block(new.size)
    try:
        blk.view[...] = new.ravel()
        check(lib.scg_euler_set(b.handle, 8, ctypes.c_void_p(blk.addr),
                                new.size))
    finally:
        blk.free()
    for which, name in ((6, "so0t"), (8, "so1n"), (5, "so0n")):
        np.testing.assert_array_equal(_get(b, which, _shape(b, name)),
                                      _get(a, which, _shape(a, name)),
                                      err_msg=name)
    a.march(1)
    b.march(1)
    np.testing.assert_array_equal(_get(b, 5, _shape(b, "so0n")),
                                  _get(a, 5, _shape(a, "so0n")))


def _delivery_core(precision, kind):
    """A marched core: triangles or tetrahedra (the simplex kernels), quads
    (the generic kernel), or triangles with slip walls on half of the
    boundary faces (ghost rows without a condition)."""
    import solvcon_gb300 as sg
    from solvcon_gb300 import meshgen
    if kind == "tet":
        return _marched_core(precision, 3)
    if kind == "tri":
        return _marched_core(precision, 2)
    if kind == "quad":
        x, t, c = meshgen.quad_square(12, 0.15, 2)
    else:
        x, t, c = meshgen.tri_square(16, 0.2, 4)
    mesh = meshgen.build_mesh(2, x, t, c)
    ec = sg.EulerCore(mesh=mesh, time_increment=2e-3, precision=precision)
    clcnd = np.array(mesh.clcnd.ndarray)[mesh.ngstcell:]
    faces = [int(f) for f in mesh.bndfcs.ndarray[:, 0]]
    ec.add_slipwall(faces if kind == "quad" else faces[::2])
    meshgen.set_state(ec, mesh, meshgen.quadrant_state(clcnd, seed=7), 1.4)
    ec.march(2)
    ec.release_views()
    return ec


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("kind", ["tri", "tet", "quad", "partial_bc"])
def test_march_delivers_so0n_so1n(precision, kind):
    """scg_euler_deliver: a march leaves so0n and so1n of its last substep
    in the registered host blocks, every row (ghost rows with and without a
    boundary condition included) equal bit for bit to scg_euler_get; the
    blocks are written only by marches, and no longer once deregistered."""
    from solvcon_gb300._lib import check, lib
    ec = _delivery_core(precision, kind)
    h = ec.handle
    blocks = {}
    try:
        for name in ("so0n", "so1n"):
            shape = _shape(ec, name)
            blk = _Block(int(np.prod(shape)))
            blk.view[...] = np.nan
            check(lib.scg_euler_deliver(h, RECORD_TABLES[name],
                                        ctypes.c_void_p(blk.addr),
                                        blk.view.size))
            blocks[name] = (blk, shape)
        for steps in (1, 3):
            check(lib.scg_euler_march(h, steps))
            check(lib.scg_euler_sync(h))
            for name, (blk, shape) in blocks.items():
                np.testing.assert_array_equal(
                    blk.view.reshape(shape),
                    _get(ec, RECORD_TABLES[name], shape), err_msg=name)
        # Operations other than march leave the blocks alone.
        for blk, _ in blocks.values():
            blk.view[...] = np.nan
        ec.calc_soln()
        ec.release_views()
        for blk, _ in blocks.values():
            assert np.isnan(blk.view).all()
        for name in blocks:
            check(lib.scg_euler_deliver(h, RECORD_TABLES[name], None, 0))
        check(lib.scg_euler_march(h, 1))
        check(lib.scg_euler_sync(h))
        for blk, _ in blocks.values():
            assert np.isnan(blk.view).all()
    finally:
        for blk, _ in blocks.values():
            blk.free()


def test_deliver_rejects_bad_targets():
    from solvcon_gb300._lib import check, lib, ptr
    ec = _marched_core("fp64", 2)
    h = ec.handle
    n0 = int(np.prod(_shape(ec, "so0n")))
    pageable = np.zeros(n0)
    with pytest.raises(ValueError):  # not a mapped block
        check(lib.scg_euler_deliver(h, 5, ptr(pageable), n0))
    blk = _Block(n0 + 1, skip=1)
    try:
        with pytest.raises(ValueError):  # only 8-byte aligned
            check(lib.scg_euler_deliver(h, 5, ctypes.c_void_p(blk.addr), n0))
        with pytest.raises(ValueError):  # not the array's size
            check(lib.scg_euler_deliver(h, 5, ctypes.c_void_p(blk.ptr.value),
                                        n0 - 1))
        with pytest.raises(ValueError):  # so0c is not delivered
            check(lib.scg_euler_deliver(h, 4, ctypes.c_void_p(blk.ptr.value),
                                        n0))
    finally:
        blk.free()


def test_batched_march_refuses_a_delivering_core():
    """A batched march does not write registered host blocks: it refuses a
    core that has one (ValueError, nothing marched), and marches it once
    the block is unregistered."""
    from solvcon_gb300._lib import check, lib
    from solvcon_gb300.batch import EulerBatch
    a = _marched_core("fp32", 2)
    b = _marched_core("fp32", 2)
    batch = EulerBatch([a, b], block=64, persistent=True)
    shape = _shape(b, "so0n")
    blk = _Block(int(np.prod(shape)))
    try:
        before = _get(b, RECORD_TABLES["so0n"], shape)
        check(lib.scg_euler_deliver(b.handle, RECORD_TABLES["so0n"],
                                    ctypes.c_void_p(blk.addr),
                                    blk.view.size))
        with pytest.raises(ValueError, match="scg_euler_deliver"):
            batch.march(1)
        np.testing.assert_array_equal(
            _get(b, RECORD_TABLES["so0n"], shape), before)
        check(lib.scg_euler_deliver(b.handle, RECORD_TABLES["so0n"], None, 0))
        batch.march(1)
        assert not np.array_equal(_get(b, RECORD_TABLES["so0n"], shape),
                                  before)
    finally:
        blk.free()


def _chunked_core(precision, kind):
    """A core large enough for several upload chunks (65,536 cells each), a
    quadrilateral one (the generic kernel, one chunk), or one whose cells
    are numbered at random (every chunk then needs the whole upload); half
    of the boundary faces carry a slip wall, so ghost rows without a
    condition are marched too."""
    import solvcon_gb300 as sg
    from solvcon_gb300 import meshgen
    if kind == "tet":
        x, t, c = meshgen.tet_cube(28, 0.15, 3)
        ndim = 3
    elif kind == "quad":
        x, t, c = meshgen.quad_square(40, 0.15, 2)
        ndim = 2
    else:
        x, t, c = meshgen.tri_square(260, 0.2, 3)
        ndim = 2
        if kind == "shuffled":
            perm = np.random.default_rng(9).permutation(len(t))
            t, c = t[perm], c[perm]
    mesh = meshgen.build_mesh(ndim, x, t, c)
    ec = sg.EulerCore(mesh=mesh, time_increment=1e-3 if ndim == 2 else 5e-4,
                      precision=precision)
    clcnd = np.array(mesh.clcnd.ndarray)[mesh.ngstcell:]
    state = (meshgen.quadrant_state(clcnd, seed=5) if ndim == 2
             else meshgen.blast_state(clcnd))
    ec.add_slipwall([int(f) for f in mesh.bndfcs.ndarray[::2, 0]])
    meshgen.set_state(ec, mesh, state, 1.4)
    ec.march(2)
    ec.release_views()
    return ec


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("kind", ["tri", "tet", "quad", "shuffled"])
def test_march_from_host_equals_set_and_march(precision, kind):
    """scg_euler_march_from_host overlaps the upload of the state from host
    blocks with the first substep, in chunks; what it leaves (the tables,
    the delivered blocks, and a march continued from it) equals
    scg_euler_set(so0n), scg_euler_set(so1n), scg_euler_march bit for
    bit."""
    from solvcon_gb300._lib import check, lib
    cores = [_chunked_core(precision, kind) for _ in range(2)]
    shapes = {n: _shape(cores[0], n) for n in ("so0n", "so1n")}
    rng = np.random.default_rng(4)
    start = {n: _get(cores[0], RECORD_TABLES[n], shapes[n]) *
             (1 + 1e-6 * rng.uniform(-1, 1, shapes[n])) for n in shapes}
    blocks = []
    try:
        ins, outs = [], []
        for ec in cores:
            inp, out = {}, {}
            for n, shape in shapes.items():
                size = int(np.prod(shape))
                bi, bo = _Block(size), _Block(size)
                blocks += [bi, bo]
                bo.view[...] = np.nan
                check(lib.scg_euler_deliver(ec.handle, RECORD_TABLES[n],
                                            ctypes.c_void_p(bo.addr), size))
                inp[n], out[n] = bi, bo
            ins.append(inp)
            outs.append(out)
        for steps in (1, 3):
            for inp in ins:
                for n in shapes:
                    inp[n].view[...] = start[n].ravel()
            a, b = cores
            for n in ("so0n", "so1n"):
                check(lib.scg_euler_set(a.handle, RECORD_TABLES[n],
                                        ctypes.c_void_p(ins[0][n].addr),
                                        ins[0][n].view.size))
            check(lib.scg_euler_march(a.handle, steps))
            check(lib.scg_euler_sync(a.handle))
            check(lib.scg_euler_march_from_host(
                b.handle, ctypes.c_void_p(ins[1]["so0n"].addr),
                ins[1]["so0n"].view.size, ctypes.c_void_p(ins[1]["so1n"].addr),
                ins[1]["so1n"].view.size, steps))
            check(lib.scg_euler_sync(b.handle))
            for n, shape in shapes.items():
                np.testing.assert_array_equal(
                    _get(b, RECORD_TABLES[n], shape),
                    _get(a, RECORD_TABLES[n], shape), err_msg=n)
                np.testing.assert_array_equal(outs[1][n].view, outs[0][n].view,
                                              err_msg=n)
            for ec in cores:
                check(lib.scg_euler_march(ec.handle, 1))
                check(lib.scg_euler_sync(ec.handle))
            for n, shape in shapes.items():
                np.testing.assert_array_equal(
                    _get(b, RECORD_TABLES[n], shape),
                    _get(a, RECORD_TABLES[n], shape), err_msg=n + " after")
        for ec in cores:
            for n in shapes:
                check(lib.scg_euler_deliver(ec.handle, RECORD_TABLES[n], None, 0))
    finally:
        for blk in blocks:
            blk.free()


def test_march_from_host_pageable_tables_and_bad_sizes():
    """Tables outside scg_host_alloc blocks are set as scg_euler_set sets
    them (same result as set + march); wrong sizes raise ValueError."""
    from solvcon_gb300._lib import check, lib, ptr
    a, b = (_chunked_core("fp64", "quad") for _ in range(2))
    so0 = _get(a, RECORD_TABLES["so0n"], _shape(a, "so0n")) * 1.000001
    so1 = _get(a, RECORD_TABLES["so1n"], _shape(a, "so1n"))
    check(lib.scg_euler_set(a.handle, RECORD_TABLES["so0n"], ptr(so0), so0.size))
    check(lib.scg_euler_set(a.handle, RECORD_TABLES["so1n"], ptr(so1), so1.size))
    check(lib.scg_euler_march(a.handle, 2))
    check(lib.scg_euler_sync(a.handle))
    check(lib.scg_euler_march_from_host(b.handle, ptr(so0), so0.size, ptr(so1),
                                        so1.size, 2))
    check(lib.scg_euler_sync(b.handle))
    for n in ("so0n", "so1n"):
        np.testing.assert_array_equal(_get(b, RECORD_TABLES[n], _shape(b, n)),
                                      _get(a, RECORD_TABLES[n], _shape(a, n)))
    with pytest.raises(ValueError):
        check(lib.scg_euler_march_from_host(b.handle, ptr(so0), so0.size - 1,
                                            ptr(so1), so1.size, 1))


def test_march_from_host_on_a_caller_stream():
    """With the core on a stream of the caller's (scg_euler_set_stream), the
    chunked first substep runs on that stream and a second one, joined back
    onto the caller's before the call's later work: the result still equals
    set + march on the core's own stream."""
    torch = pytest.importorskip("torch")
    from solvcon_gb300._lib import check, lib
    a, b = (_chunked_core("fp64", "tri") for _ in range(2))
    shapes = {n: _shape(a, n) for n in ("so0n", "so1n")}
    start = {n: _get(a, RECORD_TABLES[n], shapes[n]) * 1.000001
             for n in shapes}
    blocks = {}
    stream = torch.cuda.Stream()
    try:
        check(lib.scg_euler_set_stream(b.handle,
                                       ctypes.c_void_p(stream.cuda_stream)))
        for n, shape in shapes.items():
            blocks[n] = _Block(int(np.prod(shape)))
            blocks[n].view[...] = start[n].ravel()
        for n in shapes:
            check(lib.scg_euler_set(a.handle, RECORD_TABLES[n],
                                    ctypes.c_void_p(blocks[n].addr),
                                    blocks[n].view.size))
        check(lib.scg_euler_march(a.handle, 2))
        check(lib.scg_euler_sync(a.handle))
        check(lib.scg_euler_march_from_host(
            b.handle, ctypes.c_void_p(blocks["so0n"].addr),
            blocks["so0n"].view.size, ctypes.c_void_p(blocks["so1n"].addr),
            blocks["so1n"].view.size, 2))
        check(lib.scg_euler_sync(b.handle))
        stream.synchronize()
        for n, shape in shapes.items():
            np.testing.assert_array_equal(_get(b, RECORD_TABLES[n], shape),
                                          _get(a, RECORD_TABLES[n], shape),
                                          err_msg=n)
        check(lib.scg_euler_set_stream(b.handle, None))
    finally:
        for blk in blocks.values():
            blk.free()


def test_python_host_tables_deliver_and_march_from_host():
    """The same route from Python: HostTable state fed to
    EulerCore.march_from_host and read back through EulerCore.deliver gives
    the state of setting the arrays and calling march."""
    import solvcon_gb300 as sg
    a, b = (_chunked_core("fp64", "tri") for _ in range(2))
    start = {n: np.array(getattr(a, n).ndarray) * 1.000001
             for n in ("so0n", "so1n")}
    ins = {n: b.host_table(n) for n in start}
    outs = {n: b.host_table(n) for n in start}
    try:
        assert isinstance(ins["so0n"], sg.HostTable)
        for n in start:
            ins[n].array[...] = start[n]
            outs[n].array[...] = np.nan
            getattr(a, n).ndarray[...] = start[n]
        a.release_views()
        a.march(2)
        b.deliver(so0n=outs["so0n"], so1n=outs["so1n"])
        b.march_from_host(ins["so0n"], ins["so1n"], 2)
        for n in start:
            want = np.array(getattr(a, n).ndarray)
            np.testing.assert_array_equal(np.array(getattr(b, n).ndarray), want,
                                          err_msg=n)
            np.testing.assert_array_equal(outs[n].array, want, err_msg=n)
        with pytest.raises(ValueError):
            b.march_from_host(ins["so1n"], ins["so0n"], 1)
    finally:
        b.deliver()
        for t in list(ins.values()) + list(outs.values()):
            t.free()
