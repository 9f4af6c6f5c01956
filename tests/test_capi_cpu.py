"""The C-ABI library without a GPU: it loads, exports every function
include/lbm.h declares, and rejects bad arguments before touching CUDA."""
import ctypes as C
import os
import subprocess

import pytest


def test_exports_every_declared_symbol(libonly):
    names = libonly.declared_functions()
    assert {"lbm_init", "lbm_step", "lbm_dump", "lbm_destroy", "lbm_last_error"} <= set(names)
    L = libonly.lib()
    for n in names:
        assert hasattr(L, n), f"{n} declared in include/lbm.h but not exported"
    out = subprocess.run(["nm", "-D", "--defined-only", libonly.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in names if n not in exported]
    assert not missing, missing


def test_config_defaults_are_the_reference_cli_defaults(libonly):
    c = libonly.default_config()
    # lbm_options.hpp:83-101
    assert (c.dim, c.viscosity, c.velocity, c.precision, c.stride) == (8, 0.0089, 0.05, libonly.FP32, 32)
    assert c.noise_sigma == 0.0 and c.block_threads == 0 and not c.lid_profile


def _init(libonly, **kw):
    c = libonly.default_config()
    for k, v in kw.items():
        setattr(c, k, v)
    h = C.c_void_p()
    rc = libonly.lib().lbm_init(C.byref(h), C.byref(c))
    return rc, libonly.lib().lbm_last_error().decode()


@pytest.mark.parametrize("kw,frag", [
    (dict(dim=3), "dim"),
    (dict(dim=10), "multiple of 4"),
    (dict(dim=12, precision=2), "multiple of 8"),
    (dict(dim=4096), "dim"),
    (dict(precision=7), "precision"),
    (dict(stride=24), "stride"),
    (dict(stride=1024), "stride"),       # > dim^3 = 512
    (dict(stride=-1), "stride"),
    (dict(dim=12, stride=1024), "stride"),  # does not divide 1728
    (dict(viscosity=-1.0), "viscosity"),
    (dict(velocity=float("inf")), "velocity"),
    (dict(noise_sigma=-1.0), "noise"),
    (dict(block_threads=4096), "block_threads"),
    (dict(adjoint_steps=3), "adjoint_steps"),
    (dict(adjoint_steps=-1), "adjoint_steps"),
    (dict(adjoint_max_states=-2), "adjoint_max_states"),
    (dict(graph_iterations=3), "graph_iterations"),
    (dict(graph_iterations=512), "graph_iterations"),
    (dict(order=2), "summation order"),
    (dict(order=1, precision=3), "Sailfish"),   # FP16 storage: its own deviation sums
    (dict(adjoint_kernel=3), "adjoint_kernel"),  # only auto, direct or staged
    (dict(adjoint_kernel=-1), "adjoint_kernel"),
    (dict(adjoint_tail_segments=-2), "adjoint_tail_segments"),
])
def test_init_rejects_bad_arguments(libonly, kw, frag):
    rc, msg = _init(libonly, **kw)
    assert rc == libonly.EINVAL
    assert frag in msg


def test_init_respects_device_budget(libonly):
    # fault injection on the host: an allocation that would exceed the
    # configured budget fails cleanly with ENOMEM before any CUDA call
    rc, msg = _init(libonly, dim=64, max_device_bytes=1 << 20)
    assert rc == libonly.ENOMEM
    assert "budget" in msg


def test_null_arguments(libonly):
    L = libonly.lib()
    assert L.lbm_init(None, None) == libonly.EINVAL
    assert L.lbm_step(None, 1, 0) == libonly.EINVAL
    assert L.lbm_dump(None, 0, None, 0) == libonly.EINVAL
    assert L.lbm_sync(None) == libonly.EINVAL
    assert L.lbm_size(None, 0) == 0
    assert L.lbm_stream(None) is None
    L.lbm_destroy(None)


def test_lid_profile_must_be_finite(libonly):
    import numpy as np
    lid = np.full(64, 0.05)
    lid[7] = np.nan
    rc, msg = _init(libonly, lid_profile=lid.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == libonly.EINVAL and "lid_profile" in msg


def test_header_is_plain_c(tmp_path):
    """include/lbm.h compiles as C99 (callers bind it from C, cgo, JNI ...)."""
    import shutil
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    src = tmp_path / "use.c"
    src.write_text('#include "lbm.h"\nint main(void) { lbm_config c; lbm_config_default(&c); return c.dim; }\n')
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I" + inc, "-fsyntax-only",
                        str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("which", ["f", "map", "lid", "dim"])
def test_noalloc_checks_arguments_before_cuda(libonly, which):
    """lbm_reduce_noalloc refuses misaligned buffers and oversized lattices on
    the host, before any CUDA call (nothing is dereferenced)."""
    L = libonly.lib()
    fn = L.lbm_reduce_noalloc
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_double)]
    fn.restype = C.c_int
    ptrs = {"f": 1 << 20, "map": 1 << 20, "lid": 1 << 20}
    dim = 32
    if which == "dim":
        dim = 4096
    else:
        ptrs[which] += 1 if which == "map" else 2
    out = (C.c_double * 3)()
    rc = fn(C.c_void_p(ptrs["f"]), C.c_void_p(ptrs["map"]), C.c_void_p(ptrs["lid"]), dim, libonly.FP32, None, out)
    assert rc == libonly.EINVAL
    assert ("dim 4096" if which == "dim" else "misaligned") in L.lbm_last_error().decode()


def test_config_layout_matches_the_binding(tmp_path):
    """The ctypes Config of the Python binding has the C struct's size and
    every field at the C offset (fields are only ever appended)."""
    import shutil
    from lbmcl_gb300 import capi
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    names = [f for f, _ in capi.Config._fields_]
    body = "".join(f'    printf("%s %zu\\n", "{f}", offsetof(lbm_config, {f}));\n' for f in names)
    src = tmp_path / "layout.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "lbm.h"\nint main(void) {\n'
                   '    printf("sizeof %zu\\n", sizeof(lbm_config));\n' + body + "    return 0;\n}\n")
    exe = tmp_path / "layout"
    r = subprocess.run([cc, "-std=c99", "-I" + inc, str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                        check=True).stdout.splitlines())
    import ctypes as C
    assert int(out["sizeof"]) == C.sizeof(capi.Config)
    for f in names:
        assert int(out[f]) == getattr(capi.Config, f).offset, f
