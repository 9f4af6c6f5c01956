"""lbm_reduce_noalloc: the reduction for callers that cannot allocate device
memory (device memory owned by another allocator, such as a framework's
caching pool or a fixed arena, or already fully committed).  It must give
what lbm_reduce gives for the same state, call after call, and the only
device memory it touches besides the caller's buffers is its fixed static
scratch array: device free memory stays the same across calls.

Collected last on purpose (file name), so a run that stops at the first
failure has run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(capi):
    L = capi.lib()
    fn = L.lbm_reduce_noalloc
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_double)]
    fn.restype = C.c_int
    return fn


@pytest.mark.parametrize("prec,dim", [("fp32", 32), ("fp64", 24), ("fp16", 40), ("bf16", 32), ("fp32", 132)])
def test_noalloc_reduce_matches_lbm_reduce(capi, prec, dim):
    import torch
    fn = _noalloc(capi)
    rng = np.random.default_rng(17)
    lid = 0.05 + 0.01 * rng.standard_normal(dim * dim)
    with capi.Lattice(dim, 0.0089, 0.05, precision=prec, lid=lid, seed=3, noise_sigma=1e-4) as L:
        L.step(17)
        want = L.reduce()
        raw = L.raw()
        cmap = L.cell_map_u8()
    # the caller owns the device buffers (here: torch allocates them); the
    # entry point itself allocates nothing
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    f_d = torch.from_numpy(raw).to(dev)
    m_d = torch.from_numpy(cmap).to(dev)
    lid_d = torch.tensor(lid, dtype=torch.float64 if prec == "fp64" else torch.float32, device=dev)
    torch.cuda.synchronize()
    free_before = None
    for call in range(4):
        if call == 1:
            # the first call may load the library's device code (lazy module
            # loading); from the second call on, nothing may be allocated
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info(dev)[0]
        out = (C.c_double * 3)()
        rc = fn(f_d.data_ptr(), m_d.data_ptr(), lid_d.data_ptr(), dim, capi.PRECISIONS[prec], None, out)
        assert rc == capi.OK, capi.lib().lbm_last_error().decode()
        # same tolerances as the lbm_reduce parity test: FP64 sums in another
        # summation order
        assert abs(out[0] - want[0]) <= 1e-12 * abs(want[0]), (call, out[0], want[0])
        assert abs(out[1] - want[1]) <= 1e-9 * abs(want[1]), (call, out[1], want[1])
        assert out[2] == want[2]
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(dev)[0] == free_before, "device free memory changed across calls"


def test_noalloc_rejects_sizes_beyond_its_maximum(capi):
    fn = _noalloc(capi)
    out = (C.c_double * 3)()
    dummy = C.c_void_p(1 << 20)  # never dereferenced: the argument checks come first
    rc = fn(dummy, dummy, dummy, 4096, capi.FP32, None, out)
    assert rc == capi.EINVAL
    assert "dim 4096" in capi.lib().lbm_last_error().decode()
    assert fn(None, dummy, dummy, 32, capi.FP32, None, out) == capi.EINVAL


@pytest.mark.parametrize("which", ["f", "map", "lid"])
def test_noalloc_rejects_misaligned_buffers(capi, which):
    """A view at an odd offset into a caller's pool is refused on the host,
    before any launch (nothing is dereferenced)."""
    fn = _noalloc(capi)
    out = (C.c_double * 3)()
    base = 1 << 20
    ptrs = {"f": base, "map": base, "lid": base}
    ptrs[which] += 2 if which != "map" else 1
    rc = fn(C.c_void_p(ptrs["f"]), C.c_void_p(ptrs["map"]), C.c_void_p(ptrs["lid"]), 32, capi.FP32, None, out)
    assert rc == capi.EINVAL
    assert "misaligned" in capi.lib().lbm_last_error().decode()
