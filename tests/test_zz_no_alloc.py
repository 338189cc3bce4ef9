"""The allocation-free internal force (msx_internal_force_noalloc), for callers
that cannot call cudaMalloc: a host application whose own allocator owns all
device memory, code that must not cause the device synchronisation
cudaMalloc/cudaFree can trigger, or work enqueued during stream capture.

Collected last (file name) so that a run stopping at the first failure has run
every other test.  The test itself allocates the device buffers it passes in;
the entry point keeps its corner forces in a fixed array inside the library.
It checks the result against msx_internal_force on an FP64_EXACT handle, bit
for bit (both run the reference's operation order), on two calls in a row with
different displacements (the second call finds the first call's scratch).  The
argument checks (sizes, alignment) run before any CUDA call and are tested on
the CPU as well."""
import ctypes as C

import numpy as np
import pytest

import msx


@pytest.fixture(scope="module")
def lib():
    import build
    build.build()
    L = msx.load()
    f = L.msx_internal_force_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p,
                  C.POINTER(msx.Material_), C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return L


def cudart():
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            rt = C.CDLL(name)
            break
        except OSError:
            continue
    rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
    rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    rt.cudaFree.argtypes = [C.c_void_p]
    return rt


class DeviceArrays:
    """Caller-side device buffers (the caller's memory, not the library's)."""

    def __init__(self):
        self.rt = cudart()
        self.ptrs = []

    def put(self, a):
        a = np.ascontiguousarray(a)
        p = C.c_void_p()
        assert self.rt.cudaMalloc(C.byref(p), a.nbytes) == 0
        assert self.rt.cudaMemcpy(p, a.ctypes.data, a.nbytes, 1) == 0
        self.ptrs.append(p)
        return p

    def get(self, p, shape, dtype=np.float64):
        out = np.zeros(shape, dtype)
        assert self.rt.cudaMemcpy(out.ctypes.data, p, out.nbytes, 2) == 0
        return out

    def free(self):
        for p in self.ptrs:
            self.rt.cudaFree(p)


def csr(conn, nn):
    """node -> e*4+corner incidences, increasing element id per node."""
    inc = np.arange(conn.size, dtype=np.int64)
    order = np.argsort(conn.reshape(-1), kind="stable")
    ptr = np.zeros(nn + 1, np.int32)
    np.add.at(ptr, conn.reshape(-1) + 1, 1)
    return np.cumsum(ptr).astype(np.int32), inc[order].astype(np.int32)


@pytest.mark.gpu
@pytest.mark.parametrize("law", [msx.COMPRESSIBLE_NH, msx.NEO_HOOKEAN, msx.STVK, msx.LINEAR_ELASTIC])
def test_noalloc_internal_force_matches_handle_twice(lib, law):
    X, conn = msx.mesh_cube(8, seed=21)          # 3072 elements
    nn, ne = X.shape[1], conn.shape[0]
    mat = (law, 2e6, 0.35, 1100.0)
    S = msx.Solver(X, conn, [mat], [], 0.0, 1.0, 0.5, precision=msx.FP64_EXACT)
    ptr, inc = csr(conn, nn)
    dev = DeviceArrays()
    try:
        dX, dconn, dptr, dinc = dev.put(X), dev.put(conn), dev.put(ptr), dev.put(inc)
        dfint = dev.put(np.zeros(3 * nn))
        m = msx.Material_(law, 0, *mat[1:])
        rng = np.random.default_rng(law)
        for call in range(2):
            u = (1e-3 if call == 0 else 4e-3) * rng.standard_normal(3 * nn)
            du = dev.put(u)
            st = lib.msx_internal_force_noalloc(dX, dconn, nn, ne, dptr, dinc, C.byref(m), du, dfint, None)
            assert st == 0, lib.msx_last_error()
            assert cudart().cudaDeviceSynchronize() == 0
            f = dev.get(dfint, 3 * nn)
            ref = S.internal_force(u)
            assert np.isfinite(ref).all()
            # the same operation order on both paths: equal bits
            assert np.array_equal(f.view(np.uint64), ref.view(np.uint64)), \
                (call, np.abs(f - ref).max() / np.abs(ref).max())
    finally:
        dev.free()
        S.close()


def test_noalloc_rejects_sizes_beyond_scratch(lib):
    m = msx.Material_(1, 0, 1e6, 0.3, 1000.0)
    fake = C.c_void_p(256)      # never dereferenced: the size check comes first
    st = lib.msx_internal_force_noalloc(fake, fake, 10, 65537, fake, fake, C.byref(m), fake, fake, None)
    assert st == 1
    assert b"exceed the scratch maximum of 65536" in lib.msx_last_error()


@pytest.mark.parametrize("arg,addr,msg", [
    ("conn", 264, b"conn must be 16-byte aligned"),
    ("X", 260, b"X, u and fint must be 8-byte aligned"),
    ("u", 260, b"X, u and fint must be 8-byte aligned"),
    ("fint", 252, b"X, u and fint must be 8-byte aligned"),
    ("node_ptr", 258, b"node_ptr and node_inc must be 4-byte aligned"),
    ("node_inc", 257, b"node_ptr and node_inc must be 4-byte aligned"),
])
def test_noalloc_rejects_misaligned_pointers(lib, arg, addr, msg):
    """A caller's own allocator may hand out sub-allocations at any offset:
    misaligned arrays come back as MSX_ERR_ARG before anything touches the
    GPU (the fake addresses are never dereferenced)."""
    m = msx.Material_(1, 0, 1e6, 0.3, 1000.0)
    args = {k: C.c_void_p(256) for k in ("X", "conn", "node_ptr", "node_inc", "u", "fint")}
    args[arg] = C.c_void_p(addr)
    st = lib.msx_internal_force_noalloc(args["X"], args["conn"], 10, 8, args["node_ptr"], args["node_inc"],
                                        C.byref(m), args["u"], args["fint"], None)
    assert st == 1
    assert msg in lib.msx_last_error()


def test_noalloc_takes_every_law_and_rejects_bad_materials(lib):
    """The law parameters come from the same routine as every other entry
    point: an unknown law or an invalid constant is refused up front."""
    fake = C.c_void_p(256)
    for bad in (msx.Material_(4, 0, 1e6, 0.3, 1000.0), msx.Material_(1, 0, -1.0, 0.3, 1000.0),
                msx.Material_(2, 0, 1e6, 0.5, 1000.0)):
        st = lib.msx_internal_force_noalloc(fake, fake, 10, 8, fake, fake, C.byref(bad), fake, fake, None)
        assert st == 1
        assert b"material needs law 0..3" in lib.msx_last_error()
