"""The bounded waits of the kernels that stage their inputs by bulk copies (the mixed form's
persistent kernels): a wait for copies that never arrive must give up after its poll limit, record
the timeout and let the block return, so that the host reads DG_ERR_TIMEOUT and the context stays
usable.  The failure is a barrier armed for bytes that no copy delivers: nothing faults and nothing
waits without a limit."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def test_bulk_copy_wait_runs_out_and_reports_timeout():
    import torch
    from galaexi_gb300 import _native as nat

    assert torch.cuda.is_available()
    lib = nat.lib()
    secs = ctypes.c_double(-1.0)
    rc = lib.dg_selftest_bulk_wait(ctypes.c_longlong(2000), ctypes.byref(secs))
    assert rc == nat.DG_ERR_TIMEOUT, (rc, lib.dg_last_error())
    assert secs.value >= 0.0
    # the limit bounds the wait: 2000 polls end well inside a second
    assert secs.value < 1.0, secs.value
    print("bulk-copy wait of 2000 polls ran out after %.3e s (%.1f ns per poll)" % (secs.value, secs.value / 2000 * 1e9))
    # the device is still usable afterwards
    x = torch.ones(1 << 20, device="cuda")
    assert float(x.sum()) == float(1 << 20)


def test_kernels_after_a_timeout_still_match():
    """After the self-test's timeout, an operator evaluation on the same device runs normally."""
    import math

    import numpy as np
    import torch

    import galaexi_gb300 as gx
    from galaexi_gb300 import _native as nat

    secs = ctypes.c_double()
    assert nat.lib().dg_selftest_bulk_wait(ctypes.c_longlong(100), ctypes.byref(secs)) == nat.DG_ERR_TIMEOUT
    cfg = gx.config(N=7, NodeType="gauss-lobatto", Riemann="roe", SplitDG="pi", parabolic=True, mu0=6.25e-4,
                    R=71.42857, precision="mixed")
    mesh = gx.Mesh(7, 2, 2, 2, 2, (-math.pi,) * 3, (math.pi,) * 3)
    U = torch.from_numpy(gx.tgv_state(mesh, mach=0.1, R=71.42857)).cuda()
    op = gx.DG(cfg, mesh)
    dt, bad = op.CalcTimeStep(U, 0.8, 0.8)  # reads the kernels' wait flag: no timeout here
    assert bad == 0 and dt > 0
    Ut = op.DGTimeDerivative_weakForm(0.0, U)
    assert bool(torch.isfinite(Ut).all())
    op.close()
