"""Failure detection without a GPU fault: every device-side wait is bounded.

The tree sweeps wait on per-node flags and the cost volume waits on TMA
mbarriers.  deeds_selftest_bounded_waits runs both production wait helpers on a
flag / an mbarrier that nothing ever releases: each must give up within its
bound (about 0.13 s and 1 s), report it through its status word, and leave the
context usable for the next registration.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_bounded_waits_give_up_and_report():
    from deedsbcv_gb300 import api, phantom
    ctx = api.context(0)
    sweep, tma, secs = C.c_int(0), C.c_int(0), C.c_double(0.0)
    ctx.check(ctx._L.deeds_selftest_bounded_waits(ctx.handle, C.byref(sweep), C.byref(tma), C.byref(secs)))
    assert sweep.value == 1 and tma.value == 1
    assert secs.value < 30.0, secs.value
    # the context is still usable: a small registration and a soft level
    m, n, o = 32, 24, 40
    pr = phantom.make_pair((m, n, o), seed=4, max_disp=2.0)
    params = api.default_params(grid=(5, 4), radius=(3, 2), quant=(2, 1))
    flow, _ = api.register(pr["fixed"], pr["moving"], dims=(m, n, o), params=params)
    assert np.isfinite(flow).all()
    f = torch.from_numpy(pr["fixed"].ravel(order="F").astype(np.float32)).cuda()
    mv = torch.from_numpy(pr["moving"].ravel(order="F").astype(np.float32)).cuda()
    d = api.soft_level(f, mv, 1.6, (m, n, o), grid=4, radius=2, quant=1, tau=0.5)
    assert torch.isfinite(d).all()
