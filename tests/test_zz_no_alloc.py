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


CASES = {
    # (D, P): n_cell, prob_hi, initial condition
    (2, 3): ((48, 40, 1), (1.2, 1.0, 1.0), ("kh_noise", dict(seed=99, noise_amp=1e-3))),
    (2, 1): ((24, 20, 1), (10.0, 8.0, 1.0), ("isentropic_vortex", dict(u_inf=1.0, v_inf=0.5))),
    (3, 2): ((8, 6, 4), (1.0, 0.75, 0.5), ("blast3d", dict())),
}


@pytest.mark.parametrize("D,P,side_stream", [(2, 3, False), (2, 1, False), (3, 2, False), (2, 3, True)])
def test_noalloc_step_matches_context_step_two_calls_in_a_row(D, P, side_stream):
    torch = pytest.importorskip("torch")
    import adg_gb300 as G

    step = _entry()
    n, hi, (ic, icp) = CASES[(D, P)]
    s = G.AmrDG(P=P, D=D)
    s.setGeometrySettings(prob_lo=(0, 0, 0)[:D], prob_hi=hi[:D], n_cell=n[:D], periodic=(1, 1, 1)[:D])
    s.settings(c_dt=0.5)
    s.init(G.Compressible_Euler().settings(ic, **icp))
    dt = s.Dt
    u0 = s.get_U_w()
    dev = torch.from_numpy(u0.copy().reshape(-1)).to("cuda")
    n_cell = (ctypes.c_int * 3)(*n)
    lo = (ctypes.c_double * 3)(0.0, 0.0, 0.0)
    hi_c = (ctypes.c_double * 3)(*hi)
    stream = torch.cuda.Stream() if side_stream else None
    handle = ctypes.c_void_p(stream.cuda_stream) if stream is not None else None
    for call in range(2):
        s.ADER()  # existing entry point, same Dt (adg_ader does not change Dt)
        if stream is not None:
            stream.wait_stream(torch.cuda.current_stream())
        rc = step(D, P, n_cell, lo, hi_c, 1.4, dt, ctypes.c_void_p(dev.data_ptr()), handle)
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
