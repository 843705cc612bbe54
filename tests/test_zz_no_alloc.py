"""The allocation-free time-step entry point (dg_calc_timestep_noalloc) against dg_calc_timestep.

dg_calc_timestep_noalloc serves callers that cannot allocate device memory (device arrays owned by
another runtime's allocator, a fixed memory budget during the time loop): it takes the state and
metric arrays the caller already holds on the device and keeps its scratch in a static device array
of the library.  This test calls it through the C ABI, twice in a row on different states, and
checks each result against the context-based entry point within the tolerance the time-step parity
test uses (1e-14 relative).  It also checks that a bad state is reported and that an oversized
mesh is rejected.  The file is named to run last in a collected session.
"""
import ctypes
import math

import numpy as np
import pytest

import galaexi_gb300 as gx
from galaexi_gb300 import _native as nat

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

RTOL = 1e-14


def noalloc_dt(cfg, mesh, U, Mf, Mg, Mh, sJ, cfl, dfl):
    dt = ctypes.c_double()
    rc = nat.lib().dg_calc_timestep_noalloc(
        cfg.N, cfg.node_type, mesh.nElems, cfg.parabolic, cfg.kappa, cfg.mu0, cfg.Pr,
        ctypes.c_void_p(U.data_ptr()), ctypes.c_void_p(Mf.data_ptr()), ctypes.c_void_p(Mg.data_ptr()),
        ctypes.c_void_p(Mh.data_ptr()), ctypes.c_void_p(sJ.data_ptr()), float(cfl), float(dfl), ctypes.byref(dt),
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return rc, dt.value


def test_noalloc_timestep_matches_context_entry_point_twice():
    cfg = gx.config(N=7, Riemann="roe", SplitDG="pi", parabolic=True, mu0=6.25e-4, R=71.42857)
    mesh = gx.Mesh(7, 2, 3, 2, 4, (-math.pi,) * 3, (math.pi,) * 3)
    op = gx.DG(cfg, mesh)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    Mf, Mg, Mh, sJ = dev(mesh.Metrics_fTilde), dev(mesh.Metrics_gTilde), dev(mesh.Metrics_hTilde), dev(mesh.sJ)
    U1 = gx.tgv_state(mesh, mach=0.1, R=71.42857)
    rng = np.random.default_rng(5)
    U2 = gx.tgv_state(mesh, mach=0.3, R=71.42857)
    U2 = U2 + 1e-2 * rng.standard_normal(U2.shape) * np.abs(U2).mean(axis=(0, 1, 2, 3))
    for U, (cfl, dfl) in ((U1, (0.8, 0.8)), (U2, (0.9, 0.5))):
        Ud = dev(U)
        rc, dt = noalloc_dt(cfg, mesh, Ud, Mf, Mg, Mh, sJ, cfl, dfl)
        assert rc == nat.DG_OK, nat.lib().dg_last_error()
        ref, err = op.CalcTimeStep(Ud, cfl, dfl)
        assert err == 0
        assert abs(dt - ref) <= RTOL * ref, (dt, ref)
    op.close()


def test_noalloc_timestep_allocates_nothing():
    """After one call, further calls leave the device's free memory unchanged (cudaMemGetInfo): the
    entry point allocates nothing, neither directly nor through a library."""
    cfg = gx.config(N=5, Riemann="roe", SplitDG="pi", parabolic=True, mu0=1e-3, R=71.42857)
    mesh = gx.Mesh(5, 2, 4, 4, 4, (-math.pi,) * 3, (math.pi,) * 3)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    Mf, Mg, Mh, sJ = dev(mesh.Metrics_fTilde), dev(mesh.Metrics_gTilde), dev(mesh.Metrics_hTilde), dev(mesh.sJ)
    U = dev(gx.tgv_state(mesh, mach=0.1, R=71.42857))
    rc, dt0 = noalloc_dt(cfg, mesh, U, Mf, Mg, Mh, sJ, 0.8, 0.8)
    assert rc == nat.DG_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        rc, dt = noalloc_dt(cfg, mesh, U, Mf, Mg, Mh, sJ, 0.8, 0.8)
        assert rc == nat.DG_OK and dt == dt0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_timestep_reports_bad_state_and_limit():
    cfg = gx.config(N=3, Riemann="lf")
    mesh = gx.Mesh(3, 2, 2, 2, 2)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    Mf, Mg, Mh, sJ = dev(mesh.Metrics_fTilde), dev(mesh.Metrics_gTilde), dev(mesh.Metrics_hTilde), dev(mesh.sJ)
    U = gx.fill_ini(mesh, 1, [1.0, 0.1, 0.0, 0.0, 1.0])
    bad = U.copy()
    bad[1, 0, 2, 3, 0] = np.nan
    rc, _ = noalloc_dt(cfg, mesh, dev(bad), Mf, Mg, Mh, sJ, 0.9, 0.0)
    assert rc == nat.DG_ERR_NAN
    # the counter is cleared per call: a good state afterwards succeeds
    rc, dt = noalloc_dt(cfg, mesh, dev(U), Mf, Mg, Mh, sJ, 0.9, 0.0)
    assert rc == nat.DG_OK and dt > 0
    # more elements than the static scratch holds: rejected before any device work
    dtv = ctypes.c_double()
    rc = nat.lib().dg_calc_timestep_noalloc(3, 2, (1 << 19) + 1, 0, 1.4, 0.0, 0.72, ctypes.c_void_p(U.ctypes.data),
                                            ctypes.c_void_p(1), ctypes.c_void_p(1), ctypes.c_void_p(1),
                                            ctypes.c_void_p(1), 0.9, 0.0, ctypes.byref(dtv), None)
    assert rc == nat.DG_ERR_ARG and b"static scratch" in nat.lib().dg_last_error()
