"""The allocation-free ATM entry point (komd_gpu_atm_forces_noalloc).

It serves callers that may pass device pointers but cannot allocate device
memory themselves (their host application's allocator owns the device, or
their time-step loop must not trigger the implicit synchronisation of
cudaMalloc/cudaFree).  Its neighbour-list scratch is a fixed static device
array inside the library.  This test plays such a caller: it hands over
device buffers it already has and compares the result with the regular
entry point (komd_gpu_forces with the ATM term) through the C ABI, on two
calls in a row, since the calls share and overwrite the one scratch array.

The file is named to be collected last, so that a run stopping at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP32_FORCE_RMSE = 1e-5


def rel_rmse(a, b):
    return float(np.sqrt(((a - b) ** 2).sum(1).mean()) / np.sqrt((b ** 2).sum(1).mean()))


def _regular_forces(s, sign):
    from komd_gb300 import gpu
    cfg = gpu.make_config(s.low, s.high, 2.0, cutoff=2.0, cutoff_3b=2.0, nu=0.073, terms=gpu.TERM_ATM,
                          atm_sign=sign, atm_enum=gpu.ATM_ENUM_FULL)
    g = gpu.GpuSystem(s, cfg)
    g.update_container()
    g.forces()
    r, _, f = g.download()
    g.close()
    return r, f


def test_noalloc_matches_regular_entry_point_twice():
    import torch
    from komd_gb300 import gpu, lattice
    lib = gpu.load()
    for seed, sign in ((31, gpu.ATM_SIGN_PHYSICAL), (32, gpu.ATM_SIGN_REFERENCE)):
        s = lattice.argon_fcc(6, rho=0.8442, t_star=0.722, seed=seed, jitter=0.06)   # 864 sites
        r_wrapped, f_ref = _regular_forces(s, sign)
        # the caller's own device buffers (it can hold memory, it just may not call cudaMalloc here)
        r_dev = torch.tensor(r_wrapped, dtype=torch.float64, device="cuda")
        f_dev = torch.full((s.n, 3), float("nan"), dtype=torch.float64, device="cuda")
        low = np.ascontiguousarray(s.low, np.float64)
        high = np.ascontiguousarray(s.high, np.float64)
        stream = torch.cuda.current_stream().cuda_stream
        for call in range(2):
            f_dev.fill_(float("nan"))
            rc = lib.komd_gpu_atm_forces_noalloc(s.n, ctypes.c_void_p(r_dev.data_ptr()),
                                                 ctypes.c_void_p(f_dev.data_ptr()),
                                                 low.ctypes.data_as(ctypes.c_void_p),
                                                 high.ctypes.data_as(ctypes.c_void_p), 2.0, 0.073, sign,
                                                 ctypes.c_void_p(stream))
            assert rc == 0, lib.komd_gpu_last_error().decode()
            f = f_dev.cpu().numpy()
            assert np.isfinite(f).all()
            err = rel_rmse(f, f_ref)
            assert err < FP32_FORCE_RMSE, f"call {call}: rel RMSE {err:.3e}"


def test_noalloc_rejects_oversized_input():
    from komd_gb300 import gpu
    lib = gpu.load()
    low = np.zeros(3)
    high = np.full(3, 100.0)
    dummy = ctypes.c_void_p(1)     # never dereferenced: the size check comes first
    rc = lib.komd_gpu_atm_forces_noalloc(4097, dummy, dummy, low.ctypes.data_as(ctypes.c_void_p),
                                         high.ctypes.data_as(ctypes.c_void_p), 2.0, 0.073, 1, None)
    assert rc == 1
    assert b"at most 4096 sites" in lib.komd_gpu_last_error()


def test_noalloc_rejects_bad_sign():
    from komd_gb300 import gpu
    lib = gpu.load()
    low = np.zeros(3)
    high = np.full(3, 10.0)
    dummy = ctypes.c_void_p(1)     # never dereferenced: the argument checks come first
    for bad in (2, -1, 7):
        rc = lib.komd_gpu_atm_forces_noalloc(100, dummy, dummy, low.ctypes.data_as(ctypes.c_void_p),
                                             high.ctypes.data_as(ctypes.c_void_p), 2.0, 0.073, bad, None)
        assert rc == 1
        assert b"atm_sign" in lib.komd_gpu_last_error()


def test_noalloc_overflow_then_clean_call():
    """A packed system exceeds the fixed neighbour capacity: the call reports
    KOMD_ERR_OVERFLOW (its forces are undefined), and the next, normal call
    on the shared scratch clears the flag and matches the regular entry point."""
    import torch
    from komd_gb300 import gpu, lattice
    lib = gpu.load()
    # 7^3 = 343 sites on a simple-cubic grid of spacing 4/7 in a box of edge 4.0
    # (= 2 * cutoff_3b): about 140 neighbours inside 2.0 per site, over the 96 of the scratch
    g = (np.arange(7) + 0.5) * (4.0 / 7.0)
    dense = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    r_dense = torch.tensor(dense, dtype=torch.float64, device="cuda")
    f_dense = torch.zeros_like(r_dense)
    low = np.zeros(3)
    high = np.full(3, 4.0)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.komd_gpu_atm_forces_noalloc(len(dense), ctypes.c_void_p(r_dense.data_ptr()),
                                         ctypes.c_void_p(f_dense.data_ptr()), low.ctypes.data_as(ctypes.c_void_p),
                                         high.ctypes.data_as(ctypes.c_void_p), 2.0, 0.073, gpu.ATM_SIGN_PHYSICAL,
                                         ctypes.c_void_p(stream))
    assert rc == 3, lib.komd_gpu_last_error().decode()
    assert b"neighbours" in lib.komd_gpu_last_error()
    s = lattice.argon_fcc(6, rho=0.8442, t_star=0.722, seed=33, jitter=0.06)
    r_wrapped, f_ref = _regular_forces(s, gpu.ATM_SIGN_PHYSICAL)
    r_dev = torch.tensor(r_wrapped, dtype=torch.float64, device="cuda")
    f_dev = torch.full((s.n, 3), float("nan"), dtype=torch.float64, device="cuda")
    lo = np.ascontiguousarray(s.low, np.float64)
    hi = np.ascontiguousarray(s.high, np.float64)
    rc = lib.komd_gpu_atm_forces_noalloc(s.n, ctypes.c_void_p(r_dev.data_ptr()), ctypes.c_void_p(f_dev.data_ptr()),
                                         lo.ctypes.data_as(ctypes.c_void_p), hi.ctypes.data_as(ctypes.c_void_p),
                                         2.0, 0.073, gpu.ATM_SIGN_PHYSICAL, ctypes.c_void_p(stream))
    assert rc == 0, lib.komd_gpu_last_error().decode()
    err = rel_rmse(f_dev.cpu().numpy(), f_ref)
    assert err < FP32_FORCE_RMSE, f"rel RMSE {err:.3e}"
