"""The allocation-free mass-fixer entry point (csadv_mass_fixer_noalloc) against the plan-based
path, through the C ABI, on two calls in a row and a third in place.

Callers that cannot call cudaMalloc (a service whose device memory is fully committed to
resident solves, or a program whose device memory belongs to another runtime's pool) use
this entry point: it applies the divergence-projection mass fixer to device arrays they
own, with its scratch in a fixed array inside the library.

Reference result: the same divergence computed by a plan with the mass fixer (mf = 3)
versus without it (mf = 1) -- csadv_divergence returns both.  Tolerance: 1e-12 relative
to the field maximum, the FP64 parity bar of the other GPU tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build()


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_no_alloc_mass_fixer_matches_plan_divergence_twice():
    import torch
    from csadv import Plan, _lib
    from oracle.grid import CubedSphere

    N, dt = 48, 0.004
    scheme = dict(recon=2, dp=2, opsplit=1, et=3, mt=1, vf=2)
    g = CubedSphere(N)
    metric = torch.tensor(np.ascontiguousarray(g.metric_tensor_pc), dtype=torch.float64, device="cuda")
    L = _lib.lib()
    with Plan(N, dt, mf=1, **scheme) as raw, Plan(N, dt, mf=3, **scheme) as fixed:
        raw.init_tracer(3)
        fixed.init_tracer(3)
        for call in range(2):
            if call == 1:  # a new state: advance both, give the unfixed plan the same tracer
                fixed.advance(2)
                raw.advance(2)
                raw.set_tracer(fixed.get_tracer(full=True))
            div_raw = raw.divergence()
            div_ref = fixed.divergence()
            full = np.zeros((N + 8, N + 8, 6))
            full[4:N + 4, 4:N + 4] = div_raw
            d_in = torch.tensor(full, dtype=torch.float64, device="cuda")
            d_out = torch.empty_like(d_in)
            torch.cuda.synchronize()
            rc = L.csadv_mass_fixer_noalloc(d_in.data_ptr(), metric.data_ptr(), d_out.data_ptr(), N, None)
            assert rc == _lib.OK, _lib.status_string(rc)
            torch.cuda.synchronize()
            out = d_out.cpu().numpy()
            assert rel(out[4:N + 4, 4:N + 4], div_ref) <= RTOL
            np.testing.assert_array_equal(out[:4], full[:4])  # non-interior cells copied
        # in place (div_out == div_in), on the last state
        rc = L.csadv_mass_fixer_noalloc(d_in.data_ptr(), metric.data_ptr(), d_in.data_ptr(), N, None)
        assert rc == _lib.OK, _lib.status_string(rc)
        torch.cuda.synchronize()
        inplace = d_in.cpu().numpy()
        assert rel(inplace[4:N + 4, 4:N + 4], div_ref) <= RTOL
        np.testing.assert_array_equal(inplace[:4], full[:4])


def test_no_alloc_rejects_bad_sizes():
    from csadv import _lib
    L = _lib.lib()
    p = ctypes.c_void_p(16)
    assert L.csadv_mass_fixer_noalloc(p, p, p, 4, None) == _lib.ERR_ARG
    assert L.csadv_mass_fixer_noalloc(p, p, p, 4096, None) == _lib.ERR_TOO_LARGE
    assert L.csadv_mass_fixer_noalloc(None, p, p, 48, None) == _lib.ERR_ARG
