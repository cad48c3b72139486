"""Differentiation form: nf_adjoint against FP64 central finite differences and
through a torch.autograd.Function.

The gradient is defined with the accepted set and the contact topology held
fixed, and with each contact point held at its barycentric position along its
rod (for an unclamped closest-point pair that is the exact derivative of the
distance, by the envelope theorem). The finite-difference model below is that
definition written out in FP64 on the host: gaps from the endpoint
coordinates, G = G0 exp(-(max(gap, d_c) - d_c) / lambda), Norton assembly and
G_eff = sum over source contacts of G (1 - V), solved by a direct sparse
factorisation. Steps: h = 1e-3 nm on the endpoint coordinates of 64 random
rods, h = 1e-6 relative on lambda and G0.
"""
import numpy as np
import pytest

from conftest import rods_struct

pytestmark = pytest.mark.gpu

SRC, SNK = 0xFFFFFFFF, 0xFFFFFFFE
H_END = 1e-6  # um (1e-3 nm)


def endpoints(rods):
    c = np.stack([rods["x"], rods["y"], rods["z"]], 1).astype(np.float64)
    d = np.stack([rods["cx"], rods["cy"], rods["cz"]], 1).astype(np.float64)
    h = 0.5 * rods["l"].astype(np.float64)[:, None]
    return np.concatenate([c - h * d, c + h * d], 1)  # N x 6: e0, e1


class FixedTopology:
    """G_eff(endpoints, lambda, G0) with contacts and contact points frozen."""

    def __init__(self, cfg, rods, ct):
        self.cfg = cfg
        self.n = len(rods["x"])
        self.a = rods["a"].astype(np.float64)
        self.l = rods["l"].astype(np.float64)
        self.I = ct["I"].astype(np.int64)
        self.J = ct["J"].astype(np.int64)
        self.uI = ct["tI"] / self.l[self.I] + 0.5
        jj = np.where(self.J < self.n, self.J, 0)
        self.uJ = ct["tJ"] / self.l[jj] + 0.5
        self.shift = ct["image"].astype(np.float64) * np.asarray(cfg["box"], np.float64)
        self.D0 = ct["D"].astype(np.float64)
        self.axis = {1: 0, 2: 1, 4: 2}[cfg["field_dir"]]
        self.internal = self.J < self.n
        self.x0 = None

    def _dist(self, E):
        """Model distances up to a constant per contact (the baseline is D0)."""
        pa = E[self.I, :3] * (1 - self.uI)[:, None] + E[self.I, 3:] * self.uI[:, None]
        out = np.empty(len(self.I))
        m = self.internal
        jj = self.J[m]
        pb = E[jj, :3] * (1 - self.uJ[m])[:, None] + E[jj, 3:] * self.uJ[m][:, None] + self.shift[m]
        out[m] = np.linalg.norm(pa[m] - pb, axis=1)
        f = self.axis
        out[self.J == SRC] = pa[self.J == SRC, f]
        out[self.J == SNK] = -pa[self.J == SNK, f]
        return out

    def G_eff(self, E, lam=None, g0=None):
        import scipy.sparse as sp
        import scipy.sparse.linalg as spl
        lam = self.cfg["lambda_"] if lam is None else lam
        g0 = self.cfg["G0"] if g0 is None else g0
        if self.x0 is None:
            self.x0 = self._dist(E)
        D = self.D0 + (self._dist(E) - self.x0)
        gap = D - self.a[self.I] - np.where(self.internal, self.a[np.where(self.internal, self.J, 0)], 0.0)
        dc = self.cfg["d_c"]
        G = g0 * np.exp(-(np.maximum(gap, dc) - dc) / lam)
        m = self.internal
        # active set: components touching both electrodes
        A = sp.coo_matrix((np.ones(m.sum()), (self.I[m], self.J[m])), shape=(self.n, self.n))
        ncomp, lab = sp.csgraph.connected_components(A, directed=False)
        src = np.zeros(ncomp, bool)
        snk = np.zeros(ncomp, bool)
        src[lab[self.I[self.J == SRC]]] = True
        snk[lab[self.I[self.J == SNK]]] = True
        act = (src & snk)[lab]
        idx = -np.ones(self.n, np.int64)
        idx[act] = np.arange(act.sum())
        na = int(act.sum())
        if na == 0:
            return 0.0
        ei = m & act[self.I]
        i, j, g = idx[self.I[ei]], idx[self.J[ei]], G[ei]
        diag = np.zeros(na)
        np.add.at(diag, i, g)
        np.add.at(diag, j, g)
        b = np.zeros(na)
        for role in (SRC, SNK):
            sel = (self.J == role) & act[self.I]
            np.add.at(diag, idx[self.I[sel]], G[sel])
            if role == SRC:
                np.add.at(b, idx[self.I[sel]], G[sel])
        K = sp.coo_matrix((np.concatenate([diag, -g, -g]),
                           (np.concatenate([np.arange(na), i, j]), np.concatenate([np.arange(na), j, i]))),
                          shape=(na, na)).tocsc()
        V = spl.spsolve(K, b)
        sel = (self.J == SRC) & act[self.I]
        return float(np.sum(G[sel] * (1.0 - V[idx[self.I[sel]]])))


@pytest.fixture(scope="module")
def network(gpu, oracle):
    # the percolating jammed box (9 481 rods, ~1 200 active nodes): the medium
    # agglomerate network does not percolate with a 1.4 nm cutoff
    cfg = dict(gpu.configs.JAMMED)
    sim = gpu.Simulation(cfg)
    sim.generate()
    sim.contacts()
    sol = sim.solve()
    rods = sim.rods()
    ct = oracle.contacts(cfg, rods_struct(rods))  # bit-identical to the GPU list (FP64 tI, tJ)
    ctg = sim.contact_list()
    assert np.array_equal(ctg["I"], ct["I"]) and np.array_equal(ctg["D"], ct["D"])
    grad, dl, dg0 = sim.adjoint()
    yield dict(cfg=cfg, sim=sim, sol=sol, rods=rods, ct=ct, grad=grad, dl=dl, dg0=dg0)
    sim.close()


def test_model_reproduces_gpu_conductance(network):
    M = FixedTopology(network["cfg"], network["rods"], network["ct"])
    G = M.G_eff(endpoints(network["rods"]))
    assert network["sol"]["percolating"]
    assert G == pytest.approx(network["sol"]["G_eff"], rel=1e-6)


def test_adjoint_endpoints_vs_fd(network):
    cfg, rods, ct, grad = network["cfg"], network["rods"], network["ct"], network["grad"]
    M = FixedTopology(cfg, rods, ct)
    E0 = endpoints(rods)
    M.G_eff(E0)
    n = len(rods["x"])
    # skip rods with a contact within 3h of the gap floor (the law has a kink there)
    gap = ct["D"] - rods["a"][ct["I"]] - np.where(ct["J"] < n, rods["a"][np.where(ct["J"] < n, ct["J"], 0)], 0)
    near_kink = set(ct["I"][np.abs(gap - cfg["d_c"]) < 3 * H_END].tolist())
    near_kink |= set(ct["J"][(np.abs(gap - cfg["d_c"]) < 3 * H_END) & (ct["J"] < n)].tolist())
    rng = np.random.default_rng(64)
    live = np.flatnonzero(np.abs(grad).max(1) > 0)
    pool = np.array([r for r in live if r not in near_kink])
    pick = rng.choice(pool, size=min(56, len(pool)), replace=False)
    dead = np.setdiff1d(np.arange(n), live)
    pick = np.concatenate([pick, rng.choice(dead, size=min(64 - len(pick), len(dead)), replace=False)])
    assert len(pick) == 64
    scale = np.abs(grad).max()
    for r in pick:
        for k in range(6):
            Ep, Em = E0.copy(), E0.copy()
            Ep[r, k] += H_END
            Em[r, k] -= H_END
            fd = (M.G_eff(Ep) - M.G_eff(Em)) / (2 * H_END)
            assert abs(fd - grad[r, k]) <= 2e-4 * scale + 1e-3 * abs(fd), (r, k, fd, grad[r, k])


def test_adjoint_lambda_g0_vs_fd(network):
    cfg = network["cfg"]
    M = FixedTopology(cfg, network["rods"], network["ct"])
    E0 = endpoints(network["rods"])
    lam, g0 = cfg["lambda_"], cfg["G0"]
    hl, hg = 1e-6 * lam, 1e-6 * g0
    fd_l = (M.G_eff(E0, lam=lam + hl) - M.G_eff(E0, lam=lam - hl)) / (2 * hl)
    fd_g = (M.G_eff(E0, g0=g0 + hg) - M.G_eff(E0, g0=g0 - hg)) / (2 * hg)
    assert network["dl"] == pytest.approx(fd_l, rel=1e-5)
    assert network["dg0"] == pytest.approx(fd_g, rel=1e-6)
    # G_eff is homogeneous of degree one in G0
    assert network["dg0"] * g0 == pytest.approx(network["sol"]["G_eff"], rel=1e-6)


def rods_from_endpoints(E, a):
    e0, e1 = E[:, :3], E[:, 3:]
    d = e1 - e0
    l = np.linalg.norm(d, axis=1)
    c = d / l[:, None]
    m = 0.5 * (e0 + e1)
    return dict(x=m[:, 0], y=m[:, 1], z=m[:, 2], cx=c[:, 0], cy=c[:, 1], cz=c[:, 2], l=l, a=a)


def test_autograd_function_wraps_the_adjoint(gpu, network):
    torch = pytest.importorskip("torch")
    base = network["cfg"]
    a = network["rods"]["a"]

    class Geff(torch.autograd.Function):
        """G_eff of the rods with the given endpoints, through the C ABI
        (set rods, contacts, solve); backward = nf_adjoint of that network."""

        @staticmethod
        def forward(ctx, ends, lam, g0):
            cfg = dict(base, lambda_=float(lam), G0=float(g0))
            with gpu.Simulation(cfg) as sim:
                sim.set_rods(rods_from_endpoints(ends.detach().numpy(), a))
                sim.contacts()
                s = sim.solve()
                g, dl, dg0 = sim.adjoint()
            ctx.save_for_backward(torch.as_tensor(g, dtype=torch.float64),
                                  torch.tensor(dl, dtype=torch.float64), torch.tensor(dg0, dtype=torch.float64))
            return torch.tensor(s["G_eff"], dtype=torch.float64)

        @staticmethod
        def backward(ctx, go):
            g, dl, dg0 = ctx.saved_tensors
            return go * g, go * dl, go * dg0

    E0 = endpoints(network["rods"])
    ends = torch.tensor(E0, dtype=torch.float64, requires_grad=True)
    lam = torch.tensor(base["lambda_"], dtype=torch.float64, requires_grad=True)
    g0 = torch.tensor(base["G0"], dtype=torch.float64, requires_grad=True)
    G = Geff.apply(ends, lam, g0)
    (2.0 * G).backward()
    assert float(G.detach()) > 0
    # the same network computed directly gives the same value and gradient
    with gpu.Simulation(base) as sim:
        sim.set_rods(rods_from_endpoints(E0, a))
        sim.contacts()
        s = sim.solve()
        g, dl, dg0 = sim.adjoint()
    assert float(G.detach()) == pytest.approx(s["G_eff"], rel=1e-12)
    np.testing.assert_array_equal(ends.grad.numpy(), 2.0 * g.astype(np.float64))
    assert float(lam.grad) == pytest.approx(2.0 * dl, rel=1e-12)
    assert float(g0.grad) == pytest.approx(2.0 * dg0, rel=1e-12)
    # lambda moves no rod: a central difference through the GPU forward path
    h = 1e-6 * base["lambda_"]
    with torch.no_grad():
        fd = (Geff.apply(ends, lam + h, g0) - Geff.apply(ends, lam - h, g0)) / (2 * h)
    assert float(fd) == pytest.approx(dl, rel=1e-3)
