"""The allocation-free majorant build (er_build_majorant_device_noalloc).

It exists for callers that cannot allocate device memory where they rebuild a
majorant grid: applications that rebuild it inside a frame loop, where
cudaMalloc/cudaFree would synchronise the device, and hosts whose device
memory belongs to their own pool allocator.  The test calls it through the C
ABI twice in a row, on different volumes, and compares each result with the
allocating entry point er_build_majorant_device (bit-exact, like every
majorant test).  The file name makes pytest collect it last.
"""
import ctypes

import numpy as np
import pytest

import oracle_lib as OL

pytestmark = pytest.mark.gpu

C = OL.C
S = OL.PKG.scenes


def sigma_table(oracle, n, ds):
    plf = C.make_plf([(0.0, 0.0), (300.0, 0.0), (1200.0, 0.7), (3000.5, 1.0)])
    xs = np.arange(n, dtype=np.float32)
    op = np.zeros(n, np.float32)
    oracle.plf_evaluate(ctypes.byref(plf), n, OL.ptr(xs), OL.ptr(op))
    return (np.float32(ds) * op).astype(np.float32)


def build_both(torch, lib, oracle, shape, brick, seed):
    vol = S.blob_volume(shape, n_blobs=5, seed=seed)
    n = int(vol.max()) + 1
    sig = sigma_table(oracle, n, 100.0)
    res = np.array([shape[2], shape[1], shape[0]], np.int32)
    res_p = res.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    total = int(np.prod([(int(r) + brick - 1) // brick for r in res]))
    d_vol = torch.from_numpy(vol.view(np.int16).copy()).cuda()
    d_sig = torch.from_numpy(sig).cuda()
    d_a = torch.full((total,), -1.0, dtype=torch.float32, device="cuda")
    d_b = torch.full((total,), -2.0, dtype=torch.float32, device="cuda")
    C.check(lib.er_build_majorant_device(d_vol.data_ptr(), res_p, brick, d_sig.data_ptr(), n, 100.0, d_a.data_ptr(), None))
    C.check(lib.er_build_majorant_device_noalloc(d_vol.data_ptr(), res_p, brick, d_sig.data_ptr(), n, 100.0, d_b.data_ptr(), None))
    torch.cuda.synchronize()
    return d_a.cpu().numpy(), d_b.cpu().numpy()


def test_noalloc_majorant_matches_allocating_entry_point(oracle):
    import torch
    assert torch.cuda.is_available()
    lib = C.load_library()
    C.check(lib.er_set_device(0))
    # two calls in a row on different inputs: the second must not see the
    # first call's scratch contents
    a1, b1 = build_both(torch, lib, oracle, (40, 36, 44), 8, seed=21)
    a2, b2 = build_both(torch, lib, oracle, (17, 30, 23), 4, seed=22)
    assert np.array_equal(a1.view(np.uint32), b1.view(np.uint32)) and a1.max() > 0
    assert np.array_equal(a2.view(np.uint32), b2.view(np.uint32)) and a2.max() > 0


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = C.load_library()
    res = np.array([1024, 1024, 1024], np.int32)
    st = lib.er_build_majorant_device_noalloc(ctypes.c_void_p(16), res.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), 4,
                                              ctypes.c_void_p(16), 100, 100.0, ctypes.c_void_p(16), None)
    assert st == 2
    assert b"allocation-free limit" in lib.er_last_error_message()
    st = lib.er_build_majorant_device_noalloc(ctypes.c_void_p(16), res.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), 8,
                                              ctypes.c_void_p(16), 70000, 100.0, ctypes.c_void_p(16), None)
    assert st == 2
