"""ctypes binding of liblbm_gb300.so (include/lbm.h).

The product path: every call goes to the sm_103a library.  There is no CPU
fallback; if the library is missing or no GPU is present the calls fail
loudly (ImportError / LbmError).
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "liblbm_gb300.so")
HEADER = os.path.join(os.path.dirname(PKG), "include", "lbm.h")

FP32, FP64, FP16, BF16 = 0, 1, 2, 3
PRECISIONS = {"fp32": FP32, "fp64": FP64, "fp16": FP16, "bf16": BF16}
KERNELS = {"auto": 0, "direct": 1, "staged": 2, "narrow": 3, "aa": 4}
ORDERS = {"reference": 0, "sailfish": 1}
DUMP_F, DUMP_RHO, DUMP_U, DUMP_MAP, DUMP_MAP_U8, DUMP_F_RAW = 0, 1, 2, 3, 4, 5
OK, EINVAL, ENOMEM, ECUDA, ESTATE, EDIVERGED, ETIMEOUT = 0, 1, 2, 3, 4, 5, 6
Q = 19


class LbmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"lbm status {code}: {msg}")
        self.code = code


class Config(C.Structure):
    _fields_ = [
        ("dim", C.c_int),
        ("viscosity", C.c_double),
        ("velocity", C.c_double),
        ("precision", C.c_int),
        ("stride", C.c_int),
        ("block_threads", C.c_int),
        ("seed", C.c_uint64),
        ("noise_sigma", C.c_double),
        ("lid_profile", C.POINTER(C.c_double)),
        ("tau", C.c_double),
        ("max_device_bytes", C.c_size_t),
        ("device", C.c_int),
        ("profile_steps", C.c_int),
        ("kernel", C.c_int),
        ("stages", C.c_int),
        ("adjoint_steps", C.c_int),
        ("adjoint_max_states", C.c_int),
        ("graph_iterations", C.c_int),
        ("adjoint_full_states", C.c_int),
        ("adjoint_fp64", C.c_int),
        ("order", C.c_int),
        ("adjoint_kernel", C.c_int),
        ("adjoint_tail_segments", C.c_int),
    ]


_lib = None


def declared_functions(header: str = HEADER) -> list:
    """Names of the functions include/lbm.h declares."""
    txt = open(header).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(lbm_[a-z0-9_]+)\s*\(", txt)))


def lib():
    """Load the library (ImportError when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m lbmcl_gb300.build` "
                          "(there is no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    vp, sz = C.c_void_p, C.c_size_t
    L.lbm_config_default.argtypes = [C.POINTER(Config)]
    L.lbm_config_default.restype = None
    L.lbm_init.argtypes = [C.POINTER(vp), C.POINTER(Config)]
    L.lbm_step.argtypes = [vp, C.c_int, C.c_int]
    L.lbm_dump.argtypes = [vp, C.c_int, vp, sz]
    L.lbm_load.argtypes = [vp, C.c_int, vp, sz]
    L.lbm_size.argtypes = [vp, C.c_int]
    L.lbm_size.restype = sz
    L.lbm_sync.argtypes = [vp]
    L.lbm_timing.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.lbm_iteration.argtypes = [vp, C.POINTER(C.c_int64)]
    L.lbm_stream.argtypes = [vp]
    L.lbm_stream.restype = vp
    L.lbm_reduce.argtypes = [vp, C.POINTER(C.c_double)]
    L.lbm_destroy.argtypes = [vp]
    L.lbm_destroy.restype = None
    L.lbm_last_error.restype = C.c_char_p
    L.lbm_device_name.argtypes = [vp]
    L.lbm_device_name.restype = C.c_char_p
    L.lbm_adjoint_set_loss.argtypes = [vp, C.c_int, C.POINTER(C.c_double)]
    L.lbm_adjoint_forward.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_double)]
    L.lbm_adjoint_backward.argtypes = [vp, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double), vp, sz]
    for name in ("lbm_init", "lbm_step", "lbm_dump", "lbm_load", "lbm_sync", "lbm_timing", "lbm_iteration",
                 "lbm_reduce", "lbm_adjoint_set_loss", "lbm_adjoint_forward", "lbm_adjoint_backward"):
        getattr(L, name).restype = C.c_int
    _lib = L
    return L


def check(rc: int) -> None:
    if rc != OK:
        raise LbmError(rc, lib().lbm_last_error().decode(errors="replace"))


def default_config() -> Config:
    c = Config()
    lib().lbm_config_default(C.byref(c))
    return c


class Lattice:
    """One D3Q19 lid-driven cavity on the GPU (a handle of the C library).

    precision: "fp32" | "fp64" | "fp16" | "bf16".  stride: CSoA stride of F
    dumps (None = dim^3).  lid: optional per-column lid u_x, shape (dim, dim)
    indexed [y, x] or flat x + y*dim.  adjoint_steps: adjoint steps per
    launch of the backward sweep (0 = default, 1, 2).  adjoint_max_states:
    cap on the backward sweep's recomputed state buffers (0 = as many as fit).
    graph_iterations: iterations per CUDA graph replay in step() (0 = 16,
    1 = no graphs).  adjoint_full_states: recompute full states in a backward
    sweep without a tau gradient too (default: only the velocity / density
    the adjoint needs).  adjoint_fp64: FP64 adjoint arithmetic over FP32 /
    16-bit storage.  order: "reference" | "sailfish" summation order of rho
    and u (FP32 / FP64).  adjoint_kernel: data movement of the FP32
    two-step adjoint in the stored-point sweep (0 = default, "direct" =
    per-thread loads, "staged" = TMA-staged planes; same results).
    adjoint_tail_segments: checkpoint segments at the end of an adjoint
    forward whose linearisation points it records, so a backward sweep
    without a tau gradient skips recomputing them (0 = as many as fit, n = at
    most n, -1 = none; same results).
    """

    def __init__(self, dim, viscosity=0.0089, velocity=0.05, precision="fp32", stride=None, lid=None,
                 seed=0, noise_sigma=0.0, tau=0.0, block_threads=0, max_device_bytes=0, device=0,
                 profile_steps=False, kernel=0, stages=0, adjoint_steps=0, adjoint_max_states=0,
                 graph_iterations=0, adjoint_full_states=False, adjoint_fp64=False, order="reference",
                 adjoint_kernel=0, adjoint_tail_segments=0):
        L = lib()
        c = default_config()
        c.dim = int(dim)
        c.viscosity = float(viscosity)
        c.velocity = float(velocity)
        c.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        c.stride = 0 if stride is None else int(stride)
        c.block_threads = int(block_threads)
        c.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        c.noise_sigma = float(noise_sigma)
        self._lid = None
        if lid is not None:
            self._lid = np.ascontiguousarray(np.asarray(lid, np.float64).reshape(-1))
            c.lid_profile = self._lid.ctypes.data_as(C.POINTER(C.c_double))
        c.tau = float(tau)
        c.max_device_bytes = int(max_device_bytes)
        c.device = int(device)
        c.profile_steps = 1 if profile_steps else 0
        c.kernel = KERNELS[kernel] if isinstance(kernel, str) else int(kernel)
        c.stages = int(stages)
        c.adjoint_steps = int(adjoint_steps)
        c.adjoint_max_states = int(adjoint_max_states)
        c.graph_iterations = int(graph_iterations)
        c.adjoint_full_states = 1 if adjoint_full_states else 0
        c.adjoint_fp64 = 1 if adjoint_fp64 else 0
        c.order = ORDERS[order] if isinstance(order, str) else int(order)
        c.adjoint_kernel = KERNELS[adjoint_kernel] if isinstance(adjoint_kernel, str) else int(adjoint_kernel)
        c.adjoint_tail_segments = int(adjoint_tail_segments)
        self.cfg = c
        self.dim = int(dim)
        self.n = self.dim ** 3
        self.precision = c.precision
        self.h = C.c_void_p()
        check(L.lbm_init(C.byref(self.h), C.byref(c)))
        self.fdtype = np.float64 if self.precision == FP64 else np.float32
        self.mdtype = self.fdtype

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            lib().lbm_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- stepping ----------------------------------------------------------
    def step(self, n=1, every=0):
        check(lib().lbm_step(self.h, int(n), int(every)))

    def sync(self):
        check(lib().lbm_sync(self.h))

    @property
    def iteration(self) -> int:
        it = C.c_int64()
        check(lib().lbm_iteration(self.h, C.byref(it)))
        return it.value

    @property
    def stream(self) -> int:
        return lib().lbm_stream(self.h)

    def timing(self):
        tot, ker = C.c_double(), C.c_double()
        check(lib().lbm_timing(self.h, C.byref(tot), C.byref(ker)))
        return tot.value, ker.value

    @property
    def device_name(self) -> str:
        return lib().lbm_device_name(self.h).decode()

    def reduce(self):
        out = (C.c_double * 3)()
        check(lib().lbm_reduce(self.h, out))
        return out[0], out[1], out[2]

    # -- dumps ---------------------------------------------------------------
    def size(self, what) -> int:
        return lib().lbm_size(self.h, int(what))

    def _dump(self, what, dtype, out=None):
        nbytes = self.size(what)
        if out is None:
            out = np.empty(nbytes // np.dtype(dtype).itemsize, dtype)
        assert out.flags.c_contiguous and out.nbytes == nbytes
        check(lib().lbm_dump(self.h, int(what), out.ctypes.data_as(C.c_void_p), nbytes))
        return out

    def f(self, out=None) -> np.ndarray:
        """Reference post-stream buffer after the iterations run so far (CSoA, handle stride)."""
        return self._dump(DUMP_F, self.fdtype, out)

    def rho(self, out=None) -> np.ndarray:
        return self._dump(DUMP_RHO, self.mdtype, out)

    def u(self, out=None) -> np.ndarray:
        return self._dump(DUMP_U, self.mdtype, out)

    def cell_map(self) -> np.ndarray:
        return self._dump(DUMP_MAP, np.int32)

    def cell_map_u8(self) -> np.ndarray:
        return self._dump(DUMP_MAP_U8, np.uint8)

    def raw(self) -> np.ndarray:
        return self._dump(DUMP_F_RAW, np.uint8)

    def load_f(self, f: np.ndarray):
        f = np.ascontiguousarray(f, self.fdtype)
        check(lib().lbm_load(self.h, DUMP_F, f.ctypes.data_as(C.c_void_p), f.nbytes))

    # -- gradients -------------------------------------------------------------
    def adjoint_set_loss(self, plane_y: int, target_ux=None):
        """Loss = mean over the FLUID sites of plane y of (u_x - target)^2;
        target_ux indexed [z, x] (or flat x + z*dim), None = 0."""
        t = None
        if target_ux is not None:
            self._target = np.ascontiguousarray(np.asarray(target_ux, np.float64).reshape(-1))
            assert self._target.size == self.dim * self.dim
            t = self._target.ctypes.data_as(C.POINTER(C.c_double))
        check(lib().lbm_adjoint_set_loss(self.h, int(plane_y), t))

    def adjoint_forward(self, iterations: int, checkpoint_every: int) -> float:
        loss = C.c_double()
        check(lib().lbm_adjoint_forward(self.h, int(iterations), int(checkpoint_every), C.byref(loss)))
        return loss.value

    def adjoint_backward(self, dloss: float = 1.0, want_f0: bool = True, want_tau: bool = True):
        """Returns (dL/dtau or None, dL/dlid as [y, x], dL/dR_0 in the F layout
        or None).  Without want_tau the sweep stores only the adjoint's
        linearisation points (unless adjoint_full_states)."""
        gt = C.c_double()
        glid = np.zeros(self.dim * self.dim, np.float64)
        gf0 = np.empty(self.size(DUMP_F) // np.dtype(self.fdtype).itemsize, self.fdtype) if want_f0 else None
        check(lib().lbm_adjoint_backward(self.h, float(dloss), C.byref(gt) if want_tau else None,
                                         glid.ctypes.data_as(C.POINTER(C.c_double)),
                                         gf0.ctypes.data_as(C.c_void_p) if gf0 is not None else None,
                                         gf0.nbytes if gf0 is not None else 0))
        return (gt.value if want_tau else None), glid.reshape(self.dim, self.dim), gf0

    def load_raw(self, raw: np.ndarray):
        raw = np.ascontiguousarray(raw)
        check(lib().lbm_load(self.h, DUMP_F_RAW, raw.ctypes.data_as(C.c_void_p), raw.nbytes))
