"""The allocation-free step entry point against the context-based path.

adg_ader_step_noalloc is for callers that cannot allocate GPU memory when
they need a step: code running inside another framework's memory arena, or a
loop that must not touch the allocator after start-up.  It keeps every
intermediate array in one fixed device array of the library.  This file is
collected last so that a first failure here leaves every other test run.
"""
import ctypes

import numpy as np
import pytest

from parity import rel_err

pytestmark = pytest.mark.gpu

ADG_ERR_NOALLOC_CAPACITY = 6


def _entry():
    import adg_gb300 as G

    f = G.lib().adg_ader_step_noalloc
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                  ctypes.POINTER(ctypes.c_double), ctypes.c_double, ctypes.c_double, ctypes.c_void_p,
                  ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def test_noalloc_step_matches_context_step_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    import adg_gb300 as G

    step = _entry()
    D, P, nx, ny = 2, 3, 48, 40
    s = G.AmrDG(P=P, D=D)
    s.setGeometrySettings(prob_lo=(0, 0), prob_hi=(1.2, 1.0), n_cell=(nx, ny))
    s.settings(c_dt=0.5)
    s.init(G.Compressible_Euler().settings("kh_noise", seed=99, noise_amp=1e-3))
    dt = s.Dt
    u0 = s.get_U_w()
    dev = torch.from_numpy(u0.copy().reshape(-1)).to("cuda")
    n_cell = (ctypes.c_int * 3)(nx, ny, 1)
    lo = (ctypes.c_double * 3)(0.0, 0.0, 0.0)
    hi = (ctypes.c_double * 3)(1.2, 1.0, 1.0)
    for call in range(2):
        s.ADER()  # existing entry point, same Dt (adg_ader does not change Dt)
        rc = step(D, P, n_cell, lo, hi, 1.4, dt, ctypes.c_void_p(dev.data_ptr()), None)
        torch.cuda.synchronize()
        assert rc == 0, f"call {call}: status {rc}"
        got = dev.cpu().numpy().reshape(u0.shape)
        ref = s.get_U_w()
        assert rel_err(got, ref) < 1e-13, f"call {call}"
        assert not np.array_equal(got, u0)


def test_noalloc_rejects_problems_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    step = _entry()
    dev = torch.zeros(8, dtype=torch.float64, device="cuda")
    n_cell = (ctypes.c_int * 3)(512, 512, 1)
    lo = (ctypes.c_double * 3)(0.0, 0.0, 0.0)
    hi = (ctypes.c_double * 3)(1.0, 1.0, 1.0)
    rc = step(2, 3, n_cell, lo, hi, 1.4, 1e-3, ctypes.c_void_p(dev.data_ptr()), None)
    assert rc == ADG_ERR_NOALLOC_CAPACITY
    assert torch.count_nonzero(dev).item() == 0
