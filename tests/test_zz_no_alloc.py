"""The allocation-free per-shot entry point (sf_time_propagation_noalloc),
called through the C ABI. It is for callers that may not allocate device
memory during a call; its scratch is a static device array shared by every
call. Two calls in a row must each equal the allocating entry point
(sf_time_propagation) bit for bit, the tolerance of every traveltime test
here. This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from helpers import smooth_model

pytestmark = pytest.mark.gpu


def test_noalloc_matches_time_propagation_twice(engine_lib, cuda):
    import torch
    from seisfat2d_gb300 import Engine
    from seisfat2d_gb300._lib import SF_OK
    nx, nz, dx, dz = 161, 75, 10.0, 7.5
    m = smooth_model(nx, nz, 10.0, seed=77, noise=0.03)
    e = Engine(nx, nz, dx, dz)
    e.set_slowness(m)
    S = torch.tensor(e.get_slowness(), device="cuda")
    for sx, sz in [(800.0, 0.0), (123.4, 300.0)]:
        ref = e.time_propagation(sx, sz)
        T = torch.full((e.nxx, e.nzz), -1.0, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        st = engine_lib.sf_time_propagation_noalloc(C.c_void_p(S.data_ptr()), nx, nz, dx, dz, sx, sz,
                                                    C.c_void_p(T.data_ptr()), None)
        assert st == SF_OK
        assert np.array_equal(T.cpu().numpy(), ref)


def test_noalloc_sequence_of_grids_matches_time_propagation(engine_lib, cuda):
    """Calls that change the grid between them, each equal to the allocating
    entry point bit for bit: a tall square-cell grid (10 strips, more than the
    8 warps of the call's CTA, so warps run several strips), a small grid
    with dx != dz, then the tall grid again (the per-call epoch keeps the
    second call from taking pairs the first left in the shared array)."""
    import torch
    from seisfat2d_gb300 import Engine
    from seisfat2d_gb300._lib import SF_OK
    cases = [(200, 300, 10.0, 10.0, 77, (650.0, 0.0)), (90, 40, 12.5, 7.5, 78, (400.0, 120.0)),
             (200, 300, 10.0, 10.0, 77, (1300.0, 1700.0))]
    for nx, nz, dx, dz, seed, (sx, sz) in cases:
        m = smooth_model(nx, nz, 10.0, seed=seed, noise=0.03)
        e = Engine(nx, nz, dx, dz)
        e.set_slowness(m)
        S = torch.tensor(e.get_slowness(), device="cuda")
        ref = e.time_propagation(sx, sz)
        T = torch.full((e.nxx, e.nzz), -1.0, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        st = engine_lib.sf_time_propagation_noalloc(C.c_void_p(S.data_ptr()), nx, nz, dx, dz, sx, sz,
                                                    C.c_void_p(T.data_ptr()), None)
        assert st == SF_OK
        assert np.array_equal(T.cpu().numpy(), ref), (nx, nz, dx, dz)
        del e


def test_noalloc_rejects_sizes_beyond_its_scratch(engine_lib, cuda):
    from seisfat2d_gb300._lib import SF_ERR_RANGE
    # ceil(1006/32) * 8506 = 32 * 8506 > 262144 values: refused before any GPU work
    st = engine_lib.sf_time_propagation_noalloc(C.c_void_p(16), 8500, 1000, 10.0, 10.0, 0.0, 0.0,
                                                C.c_void_p(16), None)
    assert st == SF_ERR_RANGE
