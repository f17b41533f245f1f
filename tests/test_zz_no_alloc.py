"""The allocation-free entry point lelph_gpu_run_device_noalloc, called
through the C ABI, against the allocating lelph_gpu_run_device on the same
context: two calls in a row, FP64 and mixed forms, one case spanning several
batches of the 64 MiB static scratch.  Some callers cannot allocate device
memory after set-up (their device memory belongs to another pool, or a run
must not meet an allocation failure); this entry point serves them."""
import ctypes as C

import numpy as np
import pytest

from letzelphc_gb300 import synth
from letzelphc_gb300.elph import OUT_C128, LelphGPU, load_library

pytestmark = pytest.mark.gpu
TOL = 1e-10  # the same device kernels on the same inputs: agreement at the FP64 bar


def _ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


@pytest.mark.parametrize("name,ov,prec", [
    ("c0", {"qpts": [(0.25, 0, 0), (0.5, 0.25, 0)]}, "fp64"),
    ("c0", {"qpts": [(0.25, 0, 0), (0.5, 0.25, 0)]}, "mixed"),
    ("c1", {"kgrid": (4, 4, 4), "qpts": [(0.25, 0, 0)]}, "mixed"),   # 64 pairs: several scratch batches
])
def test_noalloc_matches_run_device(name, ov, prec):
    torch = pytest.importorskip("torch")
    s = synth.make_system(name, ov)
    L = load_library()
    with LelphGPU(s, prec, route="real") as ctx:   # the route whose buffers are all set up in advance
        for iq in range(len(s.qpts)):
            ctx.set_q(iq, s.qpts[iq], s.eigVec[iq], s.dVscf[iq])
        ctx.prepare()
        nq, nk = len(s.qpts), s.nk_bz
        qs = np.repeat(np.arange(nq), nk).astype(np.int32)
        ks = np.tile(np.arange(nk), nq).astype(np.int32)
        n = len(qs)
        gsz = s.nmodes * s.nspin * s.nbnds * s.nbnds
        ref = torch.empty(n * gsz * 2, dtype=torch.float64, device="cuda")
        ctx.run_device(qs, ks, ref.data_ptr(), out=OUT_C128)
        torch.cuda.synchronize()
        scale = ref.abs().max().item()
        warm = torch.empty_like(ref)
        outs = [torch.full_like(ref, float("nan")) for _ in range(2)]
        # a warm-up call loads every kernel the entry point launches (modules load
        # lazily, on first launch, into device memory), so that free device
        # memory is steady around the two checked calls
        rc = L.lelph_gpu_run_device_noalloc(ctx.h, n, _ptr(qs), _ptr(ks), 1, 0, OUT_C128,
                                            C.c_void_p(warm.data_ptr()))
        assert rc == 0, L.lelph_gpu_last_error(ctx.h).decode()
        held0 = ctx.stats()["device_bytes"]
        for call in range(2):
            out = outs[call]
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            rc = L.lelph_gpu_run_device_noalloc(ctx.h, n, _ptr(qs), _ptr(ks), 1, 0, OUT_C128,
                                                C.c_void_p(out.data_ptr()))
            assert rc == 0, L.lelph_gpu_last_error(ctx.h).decode()
            torch.cuda.synchronize()
            # nothing was allocated during the call: neither by the context nor on the device
            assert torch.cuda.mem_get_info()[0] == free0
            assert ctx.stats()["device_bytes"] == held0
            err = (out - ref).abs().max().item() / scale
            assert err < TOL, (call, err)


def test_noalloc_requires_prepare():
    s = synth.make_system("c0", {"kgrid": (2, 2, 2), "qpts": [(0.5, 0, 0)], "nbnds": 2})
    L = load_library()
    with LelphGPU(s, "fp64", route="real") as ctx:
        ctx.set_q(0, s.qpts[0], s.eigVec[0], s.dVscf[0])
        qs = np.zeros(1, np.int32)
        ks = np.zeros(1, np.int32)
        rc = L.lelph_gpu_run_device_noalloc(ctx.h, 1, _ptr(qs), _ptr(ks), 1, 0, OUT_C128, C.c_void_p(1))
        assert rc == -6   # LELPH_GPU_ERR_STATE: the call never allocates, so it cannot prepare implicitly
