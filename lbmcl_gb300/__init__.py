"""GB300 (sm_103a) D3Q19 BGK lid-driven cavity behind the C ABI of include/lbm.h.

    capi      ctypes binding of liblbm_gb300.so (Lattice); no CPU fallback
    adjoint   torch.autograd.Function over the hand-written adjoint
    build     nvcc / g++ recipe of the library and the lbmcl program
    run       one cavity run with MLUPS (and an adjoint run)
    validate  storage-accuracy and gradient reports of the specified workloads
    sweep     the benchmark sweep of the lbmcl program (trimmed means)
    vti       VTK ImageData reading and writing, the verify metrics
"""
