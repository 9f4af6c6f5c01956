"""ctypes front end of the CPU oracle (oracle/lbm_oracle.c) and of the
reference kernels built from kernels.cl (oracle/_ref).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py, as the checker or the timed CPU baseline.  The
product package (lbmcl_gb300) never imports it.

Array conventions follow the reference host (lbmcl.hpp:76-90): f buffers are
flat CSoA arrays of dim^3*19 values (stride = 1 << stride_log2), rho is
dim^3, u is 3*dim^3 (planar ux, uy, uz), map is int32 dim^3.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build", "liblbm_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")

Q = 19
# D3Q19 in the reference's ordering (kernels.cl:131-205) and opposites (kernels.cl:208-226)
EX = np.array([0, 1, 0, -1, 0, 0, 0, 1, -1, -1, 1, 1, 0, -1, 0, 1, 0, -1, 0])
EY = np.array([0, 0, 1, 0, -1, 0, 0, 1, 1, -1, -1, 0, 1, 0, -1, 0, 1, 0, -1])
EZ = np.array([0, 0, 0, 0, 0, -1, 1, 0, 0, 0, 0, -1, -1, -1, -1, 1, 1, 1, 1])
OPP = np.array([0, 3, 4, 1, 2, 6, 5, 9, 10, 7, 8, 17, 18, 15, 16, 13, 14, 11, 12])

FLUID, MOVING, CORNER, WALL = 0x1, 0x2, 0x4, 0x8
LEFT, RIGHT, TOP, BOTTOM, FRONT, BACK = 0x10, 0x20, 0x40, 0x80, 0x100, 0x200


class _Params(C.Structure):
    _fields_ = [
        ("dim", C.c_int),
        ("stride_log2", C.c_int),
        ("viscosity", C.c_double),
        ("velocity", C.c_double),
        ("lid", C.POINTER(C.c_double)),
        ("seed", C.c_uint64),
        ("noise_sigma", C.c_double),
        ("threads", C.c_int),
        ("order", C.c_int),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, seconds)."""
    if force or not os.path.exists(BUILD):
        subprocess.check_call(["make", "-s", "-C", HERE, "all"])
    return BUILD


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(BUILD)
        P = C.POINTER(_Params)
        fp = C.c_void_p
        for sfx in ("f32", "f64"):
            getattr(L, f"lbmo_init_{sfx}").argtypes = [P, fp, fp, fp, fp, fp]
            getattr(L, f"lbmo_init_{sfx}").restype = None
            getattr(L, f"lbmo_compute_{sfx}").argtypes = [P, fp, fp, fp, fp, fp, C.c_int, C.c_int, C.c_int]
            getattr(L, f"lbmo_compute_{sfx}").restype = None
            getattr(L, f"lbmo_run_{sfx}").argtypes = [P, C.c_int, C.c_int, C.c_int, fp, fp, fp, fp, fp,
                                                      C.POINTER(C.c_int)]
            getattr(L, f"lbmo_run_{sfx}").restype = C.c_double
        L.lbmo_cell_type.argtypes = [C.c_int] * 4
        L.lbmo_cell_type.restype = C.c_int
        L.lbmo_gauss.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32]
        L.lbmo_gauss.restype = C.c_double
        L.lbmo_log.argtypes = [C.c_double]
        L.lbmo_log.restype = C.c_double
        L.lbmo_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.lbmo_philox4x32_10.restype = None
        L.lbmo_max_threads.restype = C.c_int
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    assert a.flags.c_contiguous
    return a.ctypes.data_as(C.c_void_p)


def stride_log2(stride: int) -> int:
    s = int(stride)
    assert s > 0 and (s & (s - 1)) == 0, "stride must be a power of two"
    return s.bit_length() - 1


class OracleLattice:
    """Reference-semantics lattice on the CPU: buffers, init, push steps.

    `state` is always the newest post-stream buffer R_t, i.e. what the
    reference's step t wrote (and what step t+1 reads).
    """

    def __init__(self, dim, viscosity, velocity, precision="f32", stride=None, lid=None,
                 seed=0, noise_sigma=0.0, threads=0, order="reference"):
        self.dim = int(dim)
        self.n = self.dim ** 3
        self.dtype = np.float32 if precision == "f32" else np.float64
        self.sfx = "f32" if precision == "f32" else "f64"
        stride = self.n if stride is None else int(stride)
        self.stride = stride
        self._lid = None if lid is None else np.ascontiguousarray(lid, dtype=np.float64).reshape(-1)
        if self._lid is not None:
            assert self._lid.size == self.dim * self.dim
        self.p = _Params(self.dim, stride_log2(stride), float(viscosity), float(velocity),
                         self._lid.ctypes.data_as(C.POINTER(C.c_double)) if self._lid is not None else None,
                         int(seed) & 0xFFFFFFFFFFFFFFFF, float(noise_sigma), int(threads),
                         1 if order == "sailfish" else 0)
        self.fa = np.empty(self.n * Q, self.dtype)
        self.fb = np.empty(self.n * Q, self.dtype)
        self.rho = np.empty(self.n, self.dtype)
        self.u = np.empty(3 * self.n, self.dtype)
        self.map = np.empty(self.n, np.int32)
        self.it = 0
        L = lib()
        getattr(L, f"lbmo_init_{self.sfx}")(C.byref(self.p), _ptr(self.fb), _ptr(self.fa), _ptr(self.rho),
                                           _ptr(self.u), _ptr(self.map))
        self.cur, self.nxt = self.fa, self.fb

    @property
    def state(self) -> np.ndarray:
        return self.cur

    def step(self, n=1, every=0):
        L = lib()
        which = C.c_int(0)
        secs = getattr(L, f"lbmo_run_{self.sfx}")(C.byref(self.p), self.it + 1, int(n), int(every),
                                                 _ptr(self.cur), _ptr(self.nxt), _ptr(self.rho), _ptr(self.u),
                                                 _ptr(self.map), C.byref(which))
        if which.value == 1:
            self.cur, self.nxt = self.nxt, self.cur
        self.it += int(n)
        return secs

    def compute_slab(self, z0, z1, update_macro=0):
        """One push step restricted to z-planes [z0, z1) (used for bounded CPU samples)."""
        getattr(lib(), f"lbmo_compute_{self.sfx}")(C.byref(self.p), _ptr(self.nxt), _ptr(self.cur),
                                                  _ptr(self.rho), _ptr(self.u), _ptr(self.map),
                                                  int(update_macro), int(z0), int(z1))

    def f_soa(self, buf=None) -> np.ndarray:
        """Newest state as [19, z, y, x] (de-indexed from CSoA)."""
        return csoa_to_soa(self.cur if buf is None else buf, self.dim, self.stride)


def csoa_to_soa(f: np.ndarray, dim: int, stride: int) -> np.ndarray:
    """CSoA (kernels.cl:64) -> [19, z, y, x]."""
    n = dim ** 3
    blk = f.reshape(n // stride, Q, stride)  # [block, q, lane]
    return np.ascontiguousarray(blk.transpose(1, 0, 2).reshape(Q, dim, dim, dim))


def soa_to_csoa(f: np.ndarray, dim: int, stride: int) -> np.ndarray:
    n = dim ** 3
    g = f.reshape(Q, n // stride, stride).transpose(1, 0, 2)
    return np.ascontiguousarray(g.reshape(-1))


def cell_types(dim: int) -> np.ndarray:
    L = lib()
    out = np.empty(dim ** 3, np.int32)
    i = 0
    for z in range(dim):
        for y in range(dim):
            for x in range(dim):
                out[i] = L.lbmo_cell_type(dim, x, y, z)
                i += 1
    return out


def gauss(seed, site, q):
    return lib().lbmo_gauss(int(seed) & 0xFFFFFFFFFFFFFFFF, int(site), int(q))


def philox(ctr, key):
    L = lib()
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    L.lbmo_philox4x32_10(c, k, o)
    return list(o)


# ---------------------------------------------------------------------------
# The reference's own kernels.cl compiled for the CPU (oracle/_ref), available
# only where the reference tree was present at build time.
# ---------------------------------------------------------------------------

def ref_available(precision="f32") -> bool:
    return os.path.exists(os.path.join(REF_DIR, f"libref_{precision}.so"))


class RefLattice:
    """Same interface as OracleLattice, executing the reference kernel source."""

    _libs: dict = {}

    def __init__(self, dim, viscosity, velocity, precision="f32", stride=None, lid=None):
        path = os.path.join(REF_DIR, f"libref_{precision}.so")
        if precision not in RefLattice._libs:
            L = C.CDLL(path)
            L.ref_configure.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.POINTER(C.c_double)]
            L.ref_initialize.argtypes = [C.c_void_p] * 5
            L.ref_compute.argtypes = [C.c_void_p] * 5 + [C.c_int]
            RefLattice._libs[precision] = L
        self.L = RefLattice._libs[precision]
        self.dim = int(dim)
        self.n = self.dim ** 3
        self.dtype = np.float32 if precision == "f32" else np.float64
        stride = self.n if stride is None else int(stride)
        self.stride = stride
        self._lid = None if lid is None else np.ascontiguousarray(lid, dtype=np.float64).reshape(-1)
        self.params = (self.dim, stride_log2(stride), float(viscosity), float(velocity))
        self.fa = np.empty(self.n * Q, self.dtype)
        self.fb = np.empty(self.n * Q, self.dtype)
        self.rho = np.empty(self.n, self.dtype)
        self.u = np.empty(3 * self.n, self.dtype)
        self.map = np.empty(self.n, np.int32)
        self.it = 0
        self._configure()
        self.L.ref_initialize(_ptr(self.fb), _ptr(self.fa), _ptr(self.rho), _ptr(self.u), _ptr(self.map))
        self.cur, self.nxt = self.fa, self.fb

    def _configure(self):
        lid = self._lid.ctypes.data_as(C.POINTER(C.c_double)) if self._lid is not None else None
        self.L.ref_configure(*self.params, lid)

    @property
    def state(self):
        return self.cur

    def step(self, n=1, every=0):
        self._configure()
        for _ in range(int(n)):
            self.it += 1
            upd = 1 if (every and self.it % every == 0) else 0
            self.L.ref_compute(_ptr(self.nxt), _ptr(self.cur), _ptr(self.rho), _ptr(self.u), _ptr(self.map), upd)
            self.cur, self.nxt = self.nxt, self.cur
