"""The allocation-free residual entry point (fqsb_residual_noalloc) through the C ABI.

Some callers cannot allocate device memory at the moment they need a residual -- inside a
global-mode stream capture, under a framework that owns all device memory, or in a loop that cannot
afford cudaFree's device synchronisation.  This entry point serves them: the caller passes device
arrays it owns, and the scratch lives in a fixed device array of the library.  The test compares it
with the handle's own residual (FQSB_SCALAR_RESIDUAL, same summation order, so bit for bit) on two
calls in a row with different inputs -- the second call must not see the first call's leftovers in
the shared scratch -- and checks that oversized inputs are rejected.  This file is collected last
so that a run stopping at the first failure has already run every other test.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [300001, 100000, 1000])
def test_residual_noalloc_matches_handle_residual(n):
    """n = 300001 fills more than 256 tiles of 1024 entries (the final pass sums the tile partials in a
    loop); 100000 and 1000 fit one CTA's tree of at most 256 partials."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from frictionqpotspringblock_gb300 import Line1d, _capi

    lib = _capi.lib()
    system = Line1d.System_Cuspy_Laplace(m=1.0, eta=0.1, mu=1.0, k_interactions=1.0, k_frame=1.0 / n, dt=0.1,
                                         shape=[n], seed=7, distribution="weibull", parameters=[2.0, 1.0, 1e-5],
                                         offset=-100.0, nchunk=200)
    rng = np.random.default_rng(11)
    system.u = rng.normal(0.0, 0.3, n)
    system.v = rng.normal(0.0, 0.01, n)
    f = torch.empty(n, dtype=torch.float64, device="cuda")
    f_frame = torch.empty(n, dtype=torch.float64, device="cuda")
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    seen = []
    for call in range(2):
        system.get_field_device(_capi.FIELD_F, f.data_ptr())
        system.get_field_device(_capi.FIELD_F_FRAME, f_frame.data_ptr())
        torch.cuda.synchronize()
        rc = lib.fqsb_residual_noalloc(ctypes.c_void_p(f.data_ptr()), ctypes.c_void_p(f_frame.data_ptr()), n,
                                       ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream))
        assert rc == _capi.OK, lib.fqsb_last_error(None)
        torch.cuda.synchronize()
        value = float(out.item())
        assert value == system.residual, (call, value, system.residual)
        seen.append(value)
        system.timeSteps(25)  # a different state for the second call
    assert seen[0] != seen[1]

    rc = lib.fqsb_residual_noalloc(ctypes.c_void_p(f.data_ptr()), ctypes.c_void_p(f_frame.data_ptr()),
                                   _capi.NOALLOC_MAX_N + 1, ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream))
    assert rc == _capi.ERR_INVALID
    assert "must be in" in lib.fqsb_last_error(None).decode()
