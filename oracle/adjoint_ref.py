"""FP64 numpy restatement of the evolution step and its hand-written discrete adjoint.

TEST INFRASTRUCTURE ONLY: the "FP64 adjoint" the GPU adjoint is checked against, and the
subject of the central-finite-difference tests. The reference has no adjoint; the forward
map restated here is the reference's step without the R_Q2C mask (evolve_VV,
evolution.cpp:607-694, equivalently evolve_VV_k_nopad with SIMULATE_INFLATION off),
scalar fields only (the GW tensors do not feed back into the fields or the background, so
they drop out of any scalar-field observable).

State: half-spectrum arrays f_k, pi_k [nf, N, N, N/2+1] (f_k = r2c(f(x)), FFTW/numpy rfftn
convention), background a, b = a', add = a''. Parameters theta = (gsq, mu) of
V = mu phi^2/2 + gsq phi^2 chi^2/2 (one field: V = mu phi^2/2). With GWs (gw=True) the state
also holds u_k, pi_u_k [6, N, N, N/2+1] (components 00,01,02,11,12,22), kicked with
F_u = a^(1+al) (-kIR^2 k^2 u + r2c(S)), S_ab = 2 sum_f d_a f d_b f (spectral derivatives, Nyquist
zeroed: kernel_GW evolution.cpp:581-601, field_1st_derivative :466-578), and drifted with the
fields' a_half^(al-3) (evolve_VV :635-684); the observable rho_GW is energy()'s GW energy
(output.cpp:1030-1060): (fStar/MPl)^2 / (4 N^6 a^6) [sum' w_k q_k(pi_u_k) + hz], q_k the
P-projected norm of spectra() (output.cpp:18-53) and hz the unprojected k = 0 norm.

Adjoint convention: the adjoint of a real field x(x) is carried in k-space as
Lambda = r2c(lambda(x)); <lambda, y> = sum_x lambda y = (1/N^3) sum' w Re(conj(Lambda) Y) with
w = 2 for 0 < kz < N/2, 1 on kz = 0, N/2. The gradient of an observable O with respect to
the stored half spectrum is g_k = dO/dRe f_k + i dO/dIm f_k = (w_k / N^3) Lambda_k.
"""
from __future__ import annotations

import numpy as np

YOSHIDA = {2: [1.0], 4: [1.351207191959657771818, -1.702414403875838200264, 1.351207191959657771818]}


class Model:
    def __init__(self, nf, gsq, mu=1.0):
        self.nf, self.gsq, self.mu = nf, gsq, mu

    def V(self, f):
        if self.nf == 1:
            return 0.5 * self.mu * f[0] ** 2
        return 0.5 * self.mu * f[0] ** 2 + 0.5 * self.gsq * f[0] ** 2 * f[1] ** 2

    def dV(self, f):
        if self.nf == 1:
            return np.stack([self.mu * f[0]])
        return np.stack([self.mu * f[0] + self.gsq * f[0] * f[1] ** 2, self.gsq * f[0] ** 2 * f[1]])

    def hess_apply(self, f, lam):
        if self.nf == 1:
            return np.stack([self.mu * lam[0]])
        p, c = f
        h00 = self.mu + self.gsq * c ** 2
        h01 = 2 * self.gsq * p * c
        h11 = self.gsq * p ** 2
        return np.stack([h00 * lam[0] + h01 * lam[1], h01 * lam[0] + h11 * lam[1]])

    def dV_dtheta(self, f):
        """d/d(gsq), d/d(mu) of V (real space)."""
        if self.nf == 1:
            return np.zeros_like(f[0]), 0.5 * f[0] ** 2
        return 0.5 * f[0] ** 2 * f[1] ** 2, 0.5 * f[0] ** 2

    def dVp_dtheta(self, f):
        """d/d(gsq), d/d(mu) of V' per field."""
        if self.nf == 1:
            return np.stack([np.zeros_like(f[0])]), np.stack([f[0]])
        return (np.stack([f[0] * f[1] ** 2, f[0] ** 2 * f[1]]),
                np.stack([f[0], np.zeros_like(f[1])]))


SYM = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]


def sym_index(a, b):
    return SYM.index((min(a, b), max(a, b)))


class Lattice:
    def __init__(self, N, kIR, nf, gsq, mu=1.0, alpha=0, fs_over_mpl2=1.0, vv=2, gw=False):
        self.N, self.kIR, self.nf, self.alpha, self.gw = N, kIR, nf, alpha, gw
        self.model = Model(nf, gsq, mu)
        self.C = fs_over_mpl2 / 3.0
        self.fs2 = fs_over_mpl2
        self.w = YOSHIDA[vv]
        H = N // 2 + 1
        i = np.arange(N)
        p = np.where(i <= N // 2, i, i - N)
        kz = np.arange(H)
        self.k2 = (p[:, None, None] ** 2 + p[None, :, None] ** 2 + kz[None, None, :] ** 2).astype(np.float64)
        self.wk = np.where((kz == 0) | (kz == N // 2), 1.0, 2.0)[None, None, :] * np.ones((N, N, 1))
        self.N3 = float(N ** 3)
        # i k_a multipliers of the spectral first derivatives, Nyquist zeroed
        px = np.where(i == N // 2, 0, p).astype(np.float64)
        pz = np.where(kz == N // 2, 0, kz).astype(np.float64)
        self.dk = [kIR * px[:, None, None] * np.ones((1, N, H)), kIR * px[None, :, None] * np.ones((N, 1, H)),
                   kIR * pz[None, None, :] * np.ones((N, N, 1))]
        # the wave vector of each stored mode, for the P projection of rho_GW
        self.kv = [kIR * p[:, None, None] * np.ones((1, N, H)), kIR * p[None, :, None] * np.ones((N, 1, H)),
                   kIR * kz[None, None, :] * np.ones((N, N, 1))]
        # weights of spectra()'s GW walk (output.cpp:780-1062) per stored mode: the interior
        # at 2; on the kz = 0, N/2 planes the "+" half at 2 (its partners, never read, at 0) and
        # the real corners at 1. The walk's k of a stored mode is (pcoord(i), pcoord(j), kz).
        wq = np.where((kz == 0) | (kz == N // 2), 0.0, 2.0)[None, None, :] * np.ones((N, N, 1))
        h = N // 2
        for kk in (0, h):
            for i0 in (0, h):
                wq[i0, 1:h, kk] = 2.0
            for j0 in (0, h):
                wq[1:h, j0, kk] = 2.0
            wq[1:h, 1:h, kk] = 2.0
            wq[1:h, h + 1:, kk] = 2.0
            for i0 in (0, h):
                for j0 in (0, h):
                    wq[i0, j0, kk] = 1.0
        self.wq = wq

    # -- transforms (numpy's irfftn includes 1/N^3: irfftn(r2c(x)) = x)
    def real(self, Xk):
        return np.fft.irfftn(Xk, s=(self.N,) * 3, axes=(-3, -2, -1))

    def kspace(self, x):
        return np.fft.rfftn(x, axes=(-3, -2, -1))

    def dot(self, L, Y):
        return float(np.sum(self.wk * np.real(np.conj(L) * Y)) / self.N3)

    # -- forward pieces
    def force(self, fk, a):
        al = self.alpha
        f = self.real(fk)
        Vpk = self.kspace(self.model.dV(f))
        F = -a ** (1 + al) * self.kIR ** 2 * self.k2 * fk - a ** (3 + al) * Vpk
        return F, Vpk, f

    # -- GW pieces
    def grads(self, fk):
        """d_a f(x) for every field and axis: [nf][3] real arrays."""
        return [[self.real(1j * self.dk[ax] * fk[i]) for ax in range(3)] for i in range(self.nf)]

    def source(self, fk):
        """S_ab(x) = 2 sum_f d_a f d_b f, six components."""
        d = self.grads(fk)
        return np.stack([2 * sum(d[i][a] * d[i][b] for i in range(self.nf)) for (a, b) in SYM])

    def force_u(self, uk, fk, a):
        al = self.alpha
        Sk = self.kspace(self.source(fk))
        return a ** (1 + al) * (-self.kIR ** 2 * self.k2 * uk + Sk), Sk

    def js(self, fk, a, L):
        """(dS_k/df)^T applied to a^(1+al) L (six components, k-space rep): per field
        -a^(1+al) sum_a i k_a r2c(T_a), T_a = 2 sum_b (1 + delta_ab) lambda_ab d_b f."""
        al = self.alpha
        lam = self.real(L)
        d = self.grads(fk)
        out = []
        for i in range(self.nf):
            acc = 0
            for a_ in range(3):
                T = 2 * sum((2.0 if a_ == b else 1.0) * lam[sym_index(a_, b)] * d[i][b] for b in range(3))
                acc = acc - 1j * self.dk[a_] * self.kspace(T)
            out.append(a ** (1 + al) * acc)
        return np.stack(out)

    def dot6(self, L, Y):
        return sum(self.dot(L[c], Y[c]) for c in range(L.shape[0]))

    def rho_gw(self, puk, a):
        return self.fs2 / (4 * self.N3 ** 2 * a ** 6) * self._qsum(puk)

    def _proj(self):
        kn = np.sqrt(sum(k ** 2 for k in self.kv))
        kn[0, 0, 0] = 1.0
        kh = [k / kn for k in self.kv]
        return [[(1.0 if i == j else 0.0) - kh[i] * kh[j] for j in range(3)] for i in range(3)]

    def _qsum(self, puk):
        P = self._proj()
        U = [[puk[sym_index(i, j)] for j in range(3)] for i in range(3)]
        V = [[sum(P[i][k] * U[k][j] for k in range(3)) for j in range(3)] for i in range(3)]
        tr = V[0][0] + V[1][1] + V[2][2]
        q = sum(np.abs(V[i][j]) ** 2 for i in range(3) for j in range(3)) - np.abs(tr) ** 2 / 2
        q[0, 0, 0] = sum((1.0 if a == b else 2.0) * np.abs(puk[c][0, 0, 0]) ** 2 for c, (a, b) in enumerate(SYM))
        return float(np.sum(self.wq * q))

    def rho_gw_seed(self, puk, a):
        """Lambda (k-space rep) of d rho_GW / d pi_u_k and d rho_GW / da."""
        P = self._proj()
        U = [[puk[sym_index(i, j)] for j in range(3)] for i in range(3)]
        V = [[sum(P[i][k] * U[k][j] for k in range(3)) for j in range(3)] for i in range(3)]
        tr = V[0][0] + V[1][1] + V[2][2]
        G = [[V[i][j] - 0.5 * tr * P[i][j] for j in range(3)] for i in range(3)]
        g = np.stack([G[i][j] + G[j][i] if i != j else G[i][i] for (i, j) in SYM])
        for c, (i, j) in enumerate(SYM):
            g[c][0, 0, 0] = (1.0 if i == j else 2.0) * puk[c][0, 0, 0]
        fac = self.fs2 / (4 * self.N3 ** 2 * a ** 6)
        # gradient wrt stored modes = fac wq 2 g; Lambda = gradient N^3 / w_k
        Lpu = fac * 2 * g * self.N3 * self.wq / self.wk
        return Lpu, -6 * self.rho_gw(puk, a) / a

    def energies(self, fk, pik, a):
        K = 0.5 * sum(np.sum(self.wk * np.abs(pik[i]) ** 2) for i in range(self.nf)) / a ** 6 / self.N3 ** 2
        G = 0.5 * self.kIR ** 2 * sum(np.sum(self.wk * self.k2 * np.abs(fk[i]) ** 2) for i in range(self.nf)) \
            / self.N3 ** 2 / a ** 2
        V = float(np.mean(self.model.V(self.real(fk))))
        return K, G, V

    def A(self, fk, pik, a):
        al = self.alpha
        K, G, V = self.energies(fk, pik, a)
        return self.C * a ** (1 + 2 * al) * ((al - 2) * K + al * G + (al + 1) * V)

    def stage(self, st, w, dt):
        f, pi, a, b, add = st[:5]
        c1 = w * dt / 2
        bh = b + c1 * add
        F0, _, _ = self.force(f, a)
        ph = pi + c1 * F0
        if self.gw:
            u, pu = st[5], st[6]
            puh = pu + c1 * self.force_u(u, f, a)[0]
        ah = a + bh * w * dt / 2
        c2 = w * dt * ah ** (self.alpha - 3)
        f1 = f + c2 * ph
        a1 = ah + bh * w * dt / 2
        F1, _, _ = self.force(f1, a1)
        p1 = ph + c1 * F1
        add1 = self.A(f1, p1, a1)
        b1 = bh + c1 * add1
        out = [f1, p1, a1, b1, add1]
        if self.gw:
            u1 = u + c2 * puh
            pu1 = puh + c1 * self.force_u(u1, f1, a1)[0]
            out += [u1, pu1]
        return out

    def step(self, st, dt):
        for w in self.w:
            st = self.stage(st, w, dt)
        return st

    # -- adjoint of one stage: returns adjoints of the stage inputs and the theta gradient
    def stage_adjoint(self, st, w, dt, adj):
        al, kIR2 = self.alpha, self.kIR ** 2
        f, pi, a, b, add = st[:5]
        Lf1, Lp1, la1, lb1, ladd1 = [x.copy() if isinstance(x, np.ndarray) else x for x in adj[:5]]
        c1 = w * dt / 2
        # forward recompute
        bh = b + c1 * add
        F0, Vp0, fx0 = self.force(f, a)
        ph = pi + c1 * F0
        ah = a + bh * w * dt / 2
        c2 = w * dt * ah ** (al - 3)
        f1 = f + c2 * ph
        a1 = ah + bh * w * dt / 2
        F1, Vp1, fx1 = self.force(f1, a1)
        p1 = ph + c1 * F1
        K1, G1, V1 = self.energies(f1, p1, a1)
        if self.gw:
            u, pu = st[5], st[6]
            Lu1, Lpu1 = adj[5].copy(), adj[6].copy()
            Fu0, Sk0 = self.force_u(u, f, a)
            puh = pu + c1 * Fu0
            u1 = u + c2 * puh
            _, Sk1 = self.force_u(u1, f1, a1)
        gtheta = np.zeros(2)
        # b1 = bh + c1 add1
        lat = ladd1 + c1 * lb1
        lbh = lb1
        # add1 = A(f1, p1, a1)
        Cc = self.C * a1 ** (1 + 2 * al)
        Lf1 = Lf1 + lat * Cc * (al * kIR2 * self.k2 * f1 / (a1 ** 2 * self.N3) + (al + 1) * Vp1 / self.N3)
        Lp1 = Lp1 + lat * Cc * (al - 2) * p1 / (a1 ** 6 * self.N3)
        la1 = la1 + lat * (self.C * (1 + 2 * al) * a1 ** (2 * al) * ((al - 2) * K1 + al * G1 + (al + 1) * V1)
                           + Cc * ((al - 2) * (-6 * K1 / a1) + al * (-2 * G1 / a1)))
        dVg, dVm = self.model.dV_dtheta(fx1)
        gtheta += lat * Cc * (al + 1) * np.array([np.mean(dVg), np.mean(dVm)])
        # p1 = ph + c1 F1(f1, a1)
        Lph = Lp1.copy()
        Lf1 = Lf1 + c1 * self.jt(fx1, a1, Lp1)
        dFda1 = (1 + al) * a1 ** al * (-kIR2 * self.k2 * f1) - (3 + al) * a1 ** (2 + al) * Vp1
        la1 = la1 + c1 * sum(self.dot(Lp1[i], dFda1[i]) for i in range(self.nf))
        gtheta += c1 * self.dtheta(fx1, a1, Lp1)
        if self.gw:
            # pu1 = puh + c1 F_u(u1, f1, a1)
            Lpuh = Lpu1.copy()
            Lu1 = Lu1 + c1 * a1 ** (1 + al) * (-kIR2 * self.k2) * Lpu1
            Lf1 = Lf1 + c1 * self.js(f1, a1, Lpu1)
            la1 = la1 + c1 * (1 + al) * a1 ** al * self.dot6(Lpu1, -kIR2 * self.k2 * u1 + Sk1)
        # a1 = ah + bh w dt / 2
        lah = la1
        lbh = lbh + la1 * w * dt / 2
        # f1 = f + c2(ah) ph  [and u1 = u + c2(ah) puh]
        Lf = Lf1.copy()
        Lph = Lph + c2 * Lf1
        lah = lah + sum(self.dot(Lf1[i], ph[i]) for i in range(self.nf)) * w * dt * (al - 3) * ah ** (al - 4)
        if self.gw:
            Lu = Lu1.copy()
            Lpuh = Lpuh + c2 * Lu1
            lah = lah + self.dot6(Lu1, puh) * w * dt * (al - 3) * ah ** (al - 4)
        # ah = a + bh w dt / 2
        la = lah
        lbh = lbh + lah * w * dt / 2
        # ph = pi + c1 F0(f, a)
        Lp = Lph.copy()
        Lf = Lf + c1 * self.jt(fx0, a, Lph)
        dFda0 = (1 + al) * a ** al * (-kIR2 * self.k2 * f) - (3 + al) * a ** (2 + al) * Vp0
        la = la + c1 * sum(self.dot(Lph[i], dFda0[i]) for i in range(self.nf))
        gtheta += c1 * self.dtheta(fx0, a, Lph)
        out = [Lf, Lp, la, None, None]
        if self.gw:
            # puh = pu + c1 F_u(u, f, a)
            Lpu = Lpuh.copy()
            Lu = Lu + c1 * a ** (1 + al) * (-kIR2 * self.k2) * Lpuh
            out[0] = out[0] + c1 * self.js(f, a, Lpuh)
            out[2] = out[2] + c1 * (1 + al) * a ** al * self.dot6(Lpuh, -kIR2 * self.k2 * u + Sk0)
            out += [Lu, Lpu]
        # bh = b + c1 add
        out[3] = lbh
        out[4] = c1 * lbh
        return out, gtheta

    def jt(self, fx, a, L):
        """(dF/df)^T applied to L (k-space rep): -a^(1+al) kIR^2 k^2 L - a^(3+al) r2c(V''(f) lambda)."""
        al = self.alpha
        lam = self.real(L)
        return -a ** (1 + al) * self.kIR ** 2 * self.k2 * L - a ** (3 + al) * self.kspace(self.model.hess_apply(fx, lam))

    def dtheta(self, fx, a, L):
        """<lambda, dF/dtheta> for theta = (gsq, mu): dF/dtheta = -a^(3+al) dV'/dtheta."""
        lam = self.real(L)
        dg, dm = self.model.dVp_dtheta(fx)
        s = -a ** (3 + self.alpha)
        return np.array([s * np.sum(lam * dg), s * np.sum(lam * dm)])

    def initial_A_adjoint(self, st, adj):
        """Fold the adjoint of the initial a'' into the state (a''(0) = A(f, pi, a))."""
        al, kIR2 = self.alpha, self.kIR ** 2
        f, pi, a, b, add = st[:5]
        Lf, Lp, la, lb, ladd = adj[:5]
        K, G, V = self.energies(f, pi, a)
        Cc = self.C * a ** (1 + 2 * al)
        _, Vp, fx = self.force(f, a)
        Lf = Lf + ladd * Cc * (al * kIR2 * self.k2 * f / (a ** 2 * self.N3) + (al + 1) * Vp / self.N3)
        Lp = Lp + ladd * Cc * (al - 2) * pi / (a ** 6 * self.N3)
        la = la + ladd * (self.C * (1 + 2 * al) * a ** (2 * al) * ((al - 2) * K + al * G + (al + 1) * V)
                          + Cc * ((al - 2) * (-6 * K / a) + al * (-2 * G / a)))
        dVg, dVm = self.model.dV_dtheta(fx)
        gth = ladd * Cc * (al + 1) * np.array([np.mean(dVg), np.mean(dVm)])
        return [Lf, Lp, la, lb, 0.0] + list(adj[5:]), gth


def observable_chi2(lat: Lattice, st) -> float:
    """O = <chi^2> (the last field) over the lattice."""
    return float(np.mean(lat.real(st[0][-1]) ** 2))


def gradient(lat: Lattice, st0, dt: float, nsteps: int, observable: str = "chi2"):
    """O(final) and dO/d(f_k(0), pi_k(0), a0, b0), dO/d(gsq, mu) with a''(0) = A(state0);
    O = <chi^2> ("chi2") or rho_GW ("rho_gw", needs gw). With GWs the returned tuple ends
    with dO/d(u_k(0), pi_u_k(0)) (gradients wrt the stored modes)."""
    st0 = list(st0)
    st0[4] = lat.A(st0[0], st0[1], st0[2])
    # forward, storing stage inputs
    tape = []
    st = st0
    for _ in range(nsteps):
        for w in lat.w:
            tape.append((list(st), w))
            st = lat.stage(st, w, dt)
    Lf = np.zeros_like(st[0])
    la = 0.0
    if observable == "chi2":
        O = observable_chi2(lat, st)
        Lf[-1] = 2.0 * st[0][-1] / lat.N3        # r2c(2 chi(x) / N^3)
    else:
        O = lat.rho_gw(st[6], st[2])
    adj = [Lf, np.zeros_like(st[1]), la, 0.0, 0.0]
    if lat.gw:
        Lpu = np.zeros_like(st[6])
        if observable != "chi2":
            Lpu, adj[2] = lat.rho_gw_seed(st[6], st[2])
        adj += [np.zeros_like(st[5]), Lpu]
    gth = np.zeros(2)
    for sti, w in reversed(tape):
        adj, g = lat.stage_adjoint(sti, w, dt, adj)
        gth += g
    adj, g = lat.initial_A_adjoint(st0, adj)
    gth += g
    gf = lat.wk * adj[0] / lat.N3
    gp = lat.wk * adj[1] / lat.N3
    out = (O, gf, gp, adj[2], adj[3], gth)
    if lat.gw:
        out += (lat.wk * adj[5] / lat.N3, lat.wk * adj[6] / lat.N3)
    return out


def run_O(lat: Lattice, st0, dt, nsteps, observable: str = "chi2"):
    st = list(st0)
    st[4] = lat.A(st[0], st[1], st[2])
    for _ in range(nsteps):
        st = lat.step(st, dt)
    if observable == "chi2":
        return observable_chi2(lat, st)
    return lat.rho_gw(st[6], st[2])
