"""Taylor-Green vortex analysis and time-loop control of the reference's TGV regression run.

Restates, as test infrastructure, what the reference computes for each row of its
TGV_Re1600_Split_TGVAnalysis.csv:

  AnalyzeTestcase        testcase/taylorgreenvortex/testcase.f90:283-510  (interpolation of U, sJ and
                         the lifted velocity gradients to NAnalyze Gauss-Lobatto points, quadrature,
                         normalisation by Vol and rho0)
  InitAnalyzeBasis       analyze/analyze.f90:239-270  (GL points/weights, Vandermonde N -> NAnalyze)
  UpdateTimeStep         timedisc/timedisc_func.f90:246-296  (dt = min(CFL step, tAnalyze-t, tEnd-t),
                         stretched to hit tAnalyze/tEnd when the remainder is below dt/100;
                         nCalcTimeStepMax = 1 recomputes dt every step)
  TimeDisc loop          timedisc/timedisc.f90 (row after iterations that are multiples of
                         nAnalyzeTestCase = 10, and after the final step at tEnd)

Array arguments may be numpy arrays or torch tensors (xp = numpy or torch); states use the C-order
reversed Fortran layout (nElems, n, n, n, 5).
"""
import numpy as np

COLUMNS = ["Dissipation Rate Incompressible", "Dissipation Rate Compressible", "Ekin incomp", "Ekin comp",
           "Enstrophy comp", "DR_u", "DR_S", "DR_Sd", "DR_p", "Maximum Vorticity", "Mean Temperature",
           "uprime", "Mean Entropy", "ED_S", "ED_D"]


def read_csv(path):
    """Time column and the 15 analysis columns of a TGVAnalysis.csv."""
    with open(path) as f:
        head = f.readline().strip().split(",")
        rows = [[float(x) for x in line.split(",")] for line in f if line.strip()]
    assert head[0] == "Time" and head[1:] == COLUMNS, head
    a = np.array(rows)
    return a[:, 0], a[:, 1:]


def gl_nodes_weights(N):
    """Gauss-Lobatto nodes and weights on [-1, 1] (N+1 points)."""
    P = np.polynomial.legendre.Legendre.basis(N)
    x = np.concatenate([[-1.0], np.sort(P.deriv().roots().real), [1.0]])
    w = 2.0 / (N * (N + 1) * P(x) ** 2)
    return x, w


def vandermonde(x_from, x_to):
    """Lagrange interpolation matrix V[a, i] = l_i(x_to[a]) on the nodes x_from."""
    V = np.zeros((len(x_to), len(x_from)))
    for a, xa in enumerate(x_to):
        for i, xi in enumerate(x_from):
            num = [xa - xj for j, xj in enumerate(x_from) if j != i]
            den = [xi - xj for j, xj in enumerate(x_from) if j != i]
            V[a, i] = np.prod(num) / np.prod(den)
    return V


def change_basis(xp, V, X):
    """ChangeBasis3D of X (E, k, j, i, v) with the 1D matrix V in each direction."""
    X = xp.einsum("ai,ekjiv->ekjav", V, X)
    X = xp.einsum("bj,ekjiv->ekbiv", V, X)
    return xp.einsum("ck,ekjiv->ecjiv", V, X)


class TGVAnalysis:
    def __init__(self, xp, xGP, sJ, vol, NAnalyze=10, kappa=1.4, R=71.42857, mu0=6.25e-4, rho0=1.0, like=None):
        """xGP: the DG nodes; sJ (E, n, n, n) on the DG nodes; vol: the domain volume.  `like`
        (a torch tensor) places the matrices on its device when xp is torch."""
        self.xp = xp
        xa, wa = gl_nodes_weights(NAnalyze)
        V = vandermonde(np.asarray(xGP), xa)
        w3 = np.einsum("k,j,i->kji", wa, wa, wa)
        conv = (lambda a: xp.as_tensor(a, dtype=like.dtype, device=like.device)) if like is not None else np.asarray
        self.V = conv(V)
        self.w3 = conv(w3)
        sJa = change_basis(xp, self.V, sJ[..., None])[..., 0]
        self.intf = self.w3[None] / sJa
        self.vol, self.kappa, self.R, self.mu0, self.rho0 = vol, kappa, R, mu0, rho0

    def row(self, U, gradUx, gradUy, gradUz):
        """The 15 analysis columns of AnalyzeTestcase for one state and its lifted gradients."""
        xp, f = self.xp, self.intf
        Ua = change_basis(xp, self.V, U)
        rho = Ua[..., 0]
        vel = Ua[..., 1:4] / rho[..., None]
        v2 = (vel * vel).sum(-1)
        p = (self.kappa - 1.0) * (Ua[..., 4] - 0.5 * rho * v2)
        T = p / (rho * self.R)
        # GradVel(a, b) = d u_a / d x_b from the velocity entries (1:4) of the lifting variables
        gx, gy, gz = [change_basis(xp, self.V, g[..., 1:4]) for g in (gradUx, gradUy, gradUz)]
        G = xp.stack([gx, gy, gz], -1)                        # (..., a, b)
        divU = G[..., 0, 0] + G[..., 1, 1] + G[..., 2, 2]
        S = 0.5 * (G + G.swapaxes(-1, -2))
        Sd2 = (S * S).sum((-1, -2)) - divU ** 2 / 3.0          # |S - divU/3 I|^2
        om = xp.stack([G[..., 2, 1] - G[..., 1, 2], G[..., 0, 2] - G[..., 2, 0], G[..., 1, 0] - G[..., 0, 1]], -1)
        om2 = (om * om).sum(-1)
        s = lambda a: float((f * a).sum())
        vol, rho0, mu0 = self.vol, self.rho0, self.mu0
        Ekin = s(0.5 * v2) / vol
        Ekin_comp = s(0.5 * rho * v2) / vol / rho0
        T_mean = s(T) / vol
        Entropy = s(-1.0 / (self.kappa - 1.0) * rho * (xp.log(p) - self.kappa * xp.log(rho))) / vol
        Enstr = s(0.5 * rho * om2) / (rho0 * vol)
        DR_u = s((G * G).sum((-1, -2))) * mu0 / vol
        DR_S = s((S * S).sum((-1, -2))) * 2.0 * mu0 / (rho0 * vol)
        DR_Sd = s(Sd2) * 2.0 * mu0 / (rho0 * vol)
        DR_p = -s(p * divU) / (rho0 * vol)
        ED_S = s(mu0 * om2) / vol
        ED_D = s(mu0 * divU ** 2) * 4.0 / 3.0 / vol
        vort_max = float(om2.max()) ** 0.5
        uprime = (2.0 / 3.0 * Ekin) ** 0.5
        return [DR_S, DR_Sd + DR_p, Ekin, Ekin_comp, Enstr, DR_u, DR_S, DR_Sd, DR_p, vort_max, T_mean, uprime,
                Entropy, ED_S, ED_D]


class TimeControl:
    """UpdateTimeStep / AnalyzeTimeStep bookkeeping for tStart = 0, Analyze_dt = tEnd (one analysis
    interval), nCalcTimeStepMax = 1 and nAnalyzeTestCase = 10."""

    def __init__(self, tEnd, nAnalyzeTestCase=10):
        self.t, self.tEnd, self.tAnalyze, self.iter = 0.0, tEnd, tEnd, 0
        self.nAnalyzeTestCase = nAnalyzeTestCase
        self.doAnalyze = self.doFinalize = False

    def update(self, dt_cfl):
        """dt for the next step from the CFL time step (timedisc_func.f90:246-296)."""
        dmin = [dt_cfl, self.tAnalyze - self.t, self.tEnd - self.t]
        dt = min(dmin)
        if dt == dmin[1]:
            self.doAnalyze = True
        if dt == dmin[2]:
            self.doAnalyze = self.doFinalize = True
        dt = min(d for d in dmin if d > 0)
        if dmin[1] - dt < dt / 100.0 and dmin[1] > 0:
            dt, self.doAnalyze = dmin[1], True
        if dmin[2] - dt < dt / 100.0 and dmin[2] > 0:
            dt, self.doAnalyze, self.doFinalize = dmin[2], True, True
        return dt

    def advance(self, dt):
        """After TimeStep: returns (needs a fresh RHS at t, writes a row)."""
        self.iter += 1
        self.t = self.t + dt
        row = self.iter % self.nAnalyzeTestCase == 0 or self.doAnalyze
        return self.doAnalyze, row
