"""End-to-end pin against the reference's own Taylor-Green vortex regression run.

The reference's regression check tgv/split runs the NS TGV at Re 1600, Mach 0.1 on the periodic
8^3 box [0, 2 pi]^3 with N = 7 Gauss-Lobatto, split form PI, RoeEntropyFix, BR1 lifting,
mu0 = 6.25e-4, R = 71.42857, CFLscale = DFLscale = 0.8, tEnd = 13, and compares its
TGVAnalysis.csv (a row every 10 time steps) with the committed reference file at 1e-4 relative
(regressioncheck/checks/tgv/split/{parameter.ini,analyze.ini}).  The same run goes through the
GB300 operator here: the time step from dg_calc_timestep, LSERK steps from dg_lserk_step, the
lifted gradients from dg_get_gradients, and the analysis of AnalyzeTestcase on the device.

The CPU test pins the analysis restatement and the oracle's lifting on the first row (t = 0).  A
GPU test runs the same 5,527 steps through the GPU path and through the oracle and compares the two
runs row by row (the reference's file comes from another build, so the GPU path and the oracle must
agree with each other much more closely than either agrees with the file).
"""
import math
import os

import numpy as np
import pytest

import galaexi_gb300 as gx
from tests.tgv_analysis import COLUMNS, TGVAnalysis, TimeControl, read_csv

CSV = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                   "TGV_Re1600_Split_TGVAnalysis_Reference.csv")
# the reference's own comparison tolerance (analyze.ini: compare_data_file_tolerance, relative)
RTOL = 1e-4
RTOL_VORT_MAX = 5e-4
MU0, R_GAS, KAPPA, MACH, TEND = 6.25e-4, 71.42857, 1.4, 0.1, 13.0


MESH_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "CART_HEX_PERIODIC_008_mesh.h5")


def tgv_setup(mesh_source="generated"):
    """mesh_source: "generated" (gx.Mesh box) or "file" (the regression run's own HOPR mesh file)."""
    cfg = gx.config(N=7, NodeType="gauss-lobatto", Riemann="roeentropyfix", SplitDG="pi", parabolic=True,
                    mu0=MU0, R=R_GAS, kappa=KAPPA)
    if mesh_source == "file":
        mesh = gx.Mesh.from_hopr(MESH_FILE, 7, 2)
    else:
        mesh = gx.Mesh(7, 2, 8, 8, 8, (0.0,) * 3, (2 * math.pi,) * 3)
    U0 = gx.tgv_state(mesh, mach=MACH, kappa=KAPPA, R=R_GAS)
    return cfg, mesh, U0


def column_errors(ours, ref, ref_all):
    """Relative error per entry, with a floor of 1e-2 of the column's largest magnitude over the
    whole run for columns that start at round-off level (DR_p, ED_D at t = 0)."""
    ours, ref = np.asarray(ours), np.asarray(ref)
    scale = np.maximum(np.abs(ref), 1e-2 * np.abs(ref_all).max(axis=0, keepdims=True))
    return np.abs(ours - ref) / scale


def test_first_row_from_oracle_gradients():
    from oracle.oracle import Oracle
    cfg, mesh, U0 = tgv_setup()
    times, ref = read_csv(CSV)
    orc = Oracle(cfg, mesh)
    orc.rhs(U0)
    n = 8
    g = [orc.work(1 + d, (mesh.nElems, n, n, n, 5)) for d in range(3)]
    ana = TGVAnalysis(np, gx.basis(7, 2)["xGP"], mesh.sJ, (2 * math.pi) ** 3, mu0=MU0, R=R_GAS, kappa=KAPPA)
    row = ana.row(U0, *g)
    err = column_errors([row], ref[:1], ref)[0]
    assert times[0] == 0.0
    bad = {COLUMNS[c]: (row[c], ref[0, c]) for c in range(15) if not err[c] <= 1e-9}
    assert not bad, bad


@pytest.mark.gpu
@pytest.mark.parametrize("mesh_source", ["generated", "file"])
def test_tgv_run_matches_reference_csv(mesh_source):
    torch = pytest.importorskip("torch")
    cfg, mesh, U0 = tgv_setup(mesh_source)
    times, ref = read_csv(CSV)
    op = gx.DG(cfg, mesh)
    U = torch.from_numpy(U0).cuda()
    Ut_tmp = torch.zeros_like(U)
    sJ = torch.from_numpy(np.ascontiguousarray(mesh.sJ)).cuda()
    ana = TGVAnalysis(torch, gx.basis(7, 2)["xGP"], sJ, (2 * math.pi) ** 3, mu0=MU0, R=R_GAS, kappa=KAPPA, like=U)
    op.DGTimeDerivative_weakForm(0.0, U)
    rows, row_t = [ana.row(U, *op.gradients())], [0.0]
    tc = TimeControl(TEND)
    while True:
        dt_cfl, err_type = op.CalcTimeStep(U, 0.8, 0.8)
        assert err_type == 0, "bad state at t=%g" % tc.t
        dt = tc.update(dt_cfl)
        op.TimeStepByLSERKW2(tc.t, dt, U, Ut_tmp)
        fresh, write = tc.advance(dt)
        if fresh:
            op.DGTimeDerivative_weakForm(tc.t, U)
        if write:
            rows.append(ana.row(U, *op.gradients()))
            row_t.append(tc.t)
        if tc.doFinalize:
            break
    op.close()
    assert len(rows) == len(ref), (len(rows), len(ref))
    t_err = np.abs(np.array(row_t) - times) / np.maximum(times, 1e-300)
    err = column_errors(rows, ref, ref)
    worst = {COLUMNS[c]: float(err[:, c].max()) for c in range(15)}
    print("%s mesh: max relative time error %.3e (t <= 4: %.3e); early columns %.3e; per column %s" % (
        mesh_source, t_err.max(), t_err[times <= 4.0].max(), err[times <= 4.0].max(), worst))
    # before the transition (t <= 4) the run follows the reference to round-off level
    early = times <= 4.0
    assert t_err[early].max() <= 1e-12, t_err[early].max()
    assert err[early].max() <= 1e-7, err[early].max()
    # over the whole run (5,400 steps to t = 13) the reference's own tolerance holds for every
    # integral column; the pointwise maximum of the vorticity amplifies round-off differences in the
    # turbulent phase (the CPU oracle deviates from the reference file by the same 2.7e-4 at t ~ 12.4)
    assert t_err.max() <= RTOL, t_err.max()
    bad = {k: v for k, v in worst.items() if not v <= (RTOL_VORT_MAX if k == "Maximum Vorticity" else RTOL)}
    assert not bad, bad


def _oracle_rows(cfg, mesh, U0, ana):
    """The regression run through the oracle: dt from its CALCTIMESTEP, its LSERK steps, the lifted
    gradients of its last RHS evaluation (from the last RK stage, or a fresh RHS at the analysis time)."""
    from oracle.oracle import Oracle, set_threads
    set_threads(os.cpu_count() or 1)
    orc = Oracle(cfg, mesh)
    n = mesh.N + 1
    shape = (mesh.nElems, n, n, n, 5)
    grads = lambda: [orc.work(1 + d, shape) for d in range(3)]
    U, Ut_tmp = np.array(U0), np.zeros_like(U0)
    orc.rhs(U)
    rows, row_t = [ana.row(U, *grads())], [0.0]
    tc = TimeControl(TEND)
    while True:
        dt_cfl, err_type = orc.calc_timestep(U, 0.8, 0.8)
        assert err_type == 0
        dt = tc.update(dt_cfl)
        orc.lserk_steps_inplace(U, Ut_tmp, dt, 1, t=tc.t)
        fresh, write = tc.advance(dt)
        if fresh:
            orc.rhs(U)
        if write:
            rows.append(ana.row(U, *grads()))
            row_t.append(tc.t)
        if tc.doFinalize:
            break
    orc.close()
    return np.array(row_t), np.array(rows)


def _gpu_rows(cfg, mesh, U0):
    torch = pytest.importorskip("torch")
    op = gx.DG(cfg, mesh)
    U = torch.from_numpy(U0).cuda()
    Ut_tmp = torch.zeros_like(U)
    sJ = torch.from_numpy(np.ascontiguousarray(mesh.sJ)).cuda()
    ana = TGVAnalysis(torch, gx.basis(7, 2)["xGP"], sJ, (2 * math.pi) ** 3, mu0=MU0, R=R_GAS, kappa=KAPPA, like=U)
    op.DGTimeDerivative_weakForm(0.0, U)
    rows, row_t = [ana.row(U, *op.gradients())], [0.0]
    tc = TimeControl(TEND)
    while True:
        dt_cfl, err_type = op.CalcTimeStep(U, 0.8, 0.8)
        assert err_type == 0, "bad state at t=%g" % tc.t
        dt = tc.update(dt_cfl)
        op.TimeStepByLSERKW2(tc.t, dt, U, Ut_tmp)
        fresh, write = tc.advance(dt)
        if fresh:
            op.DGTimeDerivative_weakForm(tc.t, U)
        if write:
            rows.append(ana.row(U, *op.gradients()))
            row_t.append(tc.t)
        if tc.doFinalize:
            break
    op.close()
    return np.array(row_t), np.array(rows)


# Agreement of the GPU run with the oracle's run over the whole regression (t = 0..13, 5,527 steps).
# Round-off differences of the two evaluation orders grow in the turbulent phase; they reach the
# time step (dt follows the state), so the times drift apart too.  Measured: time 3.6e-15 up to t = 4
# and 4.7e-10 at t = 13; every column 1.3e-10 up to t = 4; over the whole run kinetic energy 9.5e-10,
# maximum vorticity 2.0e-7, DR_p 1.4e-8, the other columns <= 1.2e-8.  Bounds:
GPU_VS_ORACLE_EARLY_TIME = 1e-12  # time, t <= 4 (relative to tEnd)
GPU_VS_ORACLE_EARLY = 1e-9        # every column, t <= 4
GPU_VS_ORACLE_TIME = 1e-8         # time, whole run (relative to tEnd)
GPU_VS_ORACLE_KE = 1e-8           # kinetic energy (incompressible and compressible), whole run
GPU_VS_ORACLE_ALL = 1e-5          # every column, whole run


@pytest.mark.gpu
def test_tgv_run_gpu_matches_oracle_run():
    cfg, mesh, U0 = tgv_setup("generated")
    times, ref = read_csv(CSV)
    t_gpu, rows_gpu = _gpu_rows(cfg, mesh, U0)
    ana = TGVAnalysis(np, gx.basis(7, 2)["xGP"], mesh.sJ, (2 * math.pi) ** 3, mu0=MU0, R=R_GAS, kappa=KAPPA)
    t_orc, rows_orc = _oracle_rows(cfg, mesh, U0, ana)
    assert len(t_gpu) == len(t_orc) == len(ref)
    t_err = np.abs(t_gpu - t_orc) / TEND
    err = column_errors(rows_gpu, rows_orc, rows_orc)
    early = t_orc <= 4.0
    print("GPU vs oracle: time %.3e (t <= 4: %.3e); columns t <= 4 %.3e; whole run per column %s" % (
        t_err.max(), t_err[early].max(), err[early].max(), {COLUMNS[c]: float(err[:, c].max()) for c in range(15)}))
    assert t_err[early].max() <= GPU_VS_ORACLE_EARLY_TIME, t_err[early].max()
    assert t_err.max() <= GPU_VS_ORACLE_TIME, t_err.max()
    assert err[early].max() <= GPU_VS_ORACLE_EARLY, err[early].max()
    assert err[:, 2:4].max() <= GPU_VS_ORACLE_KE, err[:, 2:4].max()
    assert err.max() <= GPU_VS_ORACLE_ALL, err.max()
