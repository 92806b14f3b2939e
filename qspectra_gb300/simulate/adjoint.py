"""Gradients of disorder-averaged absorption spectra (GPU adjoint).

The reference has no derivatives; this module differentiates its
absorption path (``absorption_spectra``, qspectra/simulate/response.py:
103-154, through ``linear_response`` :15-43, averaged over the ensemble,
decorators.py:40-64) with respect to the site energies, the couplings and
the bath reorganisation energy of a Redfield model (redfield.py:9-152).

* The Heisenberg-picture 'eg' generator of every sample is built in FP64
  torch ops so that autograd carries d L / d theta: eigh of the
  rotating-frame one-exciton Hamiltonian (the Jacobi kernel with an
  analytic backward), the Debye correlation function
  (bath.py:84-102, the reference's truncated Matsubara sum, with its
  derivative), and the operator-form Redfield tensor.
* The RK4 time loop and its adjoint are hand-written kernels behind
  ``ProjectedMeanRK4``: forward ``qsx_rk4_batched`` (ensemble-mean
  projection, checkpoints every K steps), backward
  ``qsx_rk4_adjoint_batched`` (lambda backward under P^H, gradient
  sum_k lambda_{k+1} y_k^H accumulated per sample, segments recomputed from
  the checkpoints).
* The transform to the frequency grid is ``qsx_dft_batched`` forward and,
  with the roles of time and frequency exchanged, backward.
"""
import numpy as np
import torch

from .. import _native
from ..constants import CM_FS, CM_K


# ------------------------------------------------------------- Debye bath
def _debye_unit(x, temperature, cutoff_freq, matsubara_cutoff, chunk=8192):
    """C(x) / lambda and dC/dx / lambda by the reference's truncated sum
    (bath.py:84-102); x = 0 takes the reference's limit lambda (2T/gamma - i)."""
    T, gam = float(temperature), float(cutoff_freq)
    flat = x.reshape(-1)
    nu = 2 * np.pi * T * torch.arange(1, matsubara_cutoff, dtype=torch.float64,
                                      device=x.device)
    w = nu / (nu ** 2 - gam ** 2)
    a = 1.0 / np.tan(gam / (2 * T)) - 1j
    val = torch.empty(flat.shape, dtype=torch.complex128, device=x.device)
    der = torch.empty_like(val)
    for s in range(0, flat.numel(), chunk):
        xs = flat[s:s + chunk].to(torch.complex128)
        r = 1.0 / (nu[None, :] - 1j * xs[:, None])
        base = 1.0 / (gam - 1j * xs)
        val[s:s + chunk] = gam * (a * base + 4 * T * (w[None, :] * r).sum(1))
        der[s:s + chunk] = gam * (1j * a * base ** 2 + 4j * T * (w[None, :] * r * r).sum(1))
    zero = flat == 0
    val[zero] = 2 * T / gam - 1j
    return val.reshape(x.shape), der.reshape(x.shape)


class DebyeCorr(torch.autograd.Function):
    """lambda * C_unit(x) with gradients for real x and lambda."""

    @staticmethod
    def forward(ctx, x, lam, temperature, cutoff_freq, matsubara_cutoff):
        c0, d0 = _debye_unit(x.detach(), temperature, cutoff_freq, matsubara_cutoff)
        ctx.save_for_backward(c0, d0, lam)
        return lam * c0

    @staticmethod
    def backward(ctx, g):
        c0, d0, lam = ctx.saved_tensors
        gx = (torch.conj(lam * d0) * g).real
        glam = (torch.conj(c0) * g).real.sum().reshape(lam.shape)
        return gx, glam, None, None, None


# --------------------------------------------------------------- eigensolve
class SymmetricEigh(torch.autograd.Function):
    """E, U of a batch of real symmetric matrices by the batched Jacobi
    kernel (qsx_eigh_batched, FP64, n <= 32), with the analytic backward
    gA = U (diag(gE) + F o (U^T gU)) U^T, F_ij = 1 / (E_j - E_i) (i != j),
    symmetrised."""

    @staticmethod
    def forward(ctx, A):
        A = A.detach().contiguous()
        n = A.shape[-1]
        E, U = _native.eigh(A, [0, n])
        ctx.save_for_backward(E, U)
        return E, U

    @staticmethod
    def backward(ctx, gE, gU):
        E, U = ctx.saved_tensors
        inner = torch.zeros_like(U)
        if gU is not None:
            diff = E[:, None, :] - E[:, :, None]          # E_j - E_i
            F = torch.where(diff.abs() > 0, 1.0 / torch.where(diff == 0, 1.0, diff), 0.0)
            inner = F * (U.transpose(1, 2) @ gU)
        if gE is not None:
            inner = inner + torch.diag_embed(gE)
        gA = U @ inner @ U.transpose(1, 2)
        return 0.5 * (gA + gA.transpose(1, 2))


# --------------------------------------------------------------- generator
def eg_heisenberg_generator(H1, lam, temperature, cutoff_freq, rw_freq, unit_convert,
                            matsubara_cutoff=1000, eigh=None):
    """Heisenberg-picture 'eg' Redfield generator L^T (S, N, N) complex128.

    H1 (S, N, N) float64 one-exciton Hamiltonians (not rotating).  In the
    site basis L_eg = -(G + i uc H) with H the rotating-frame Hamiltonian and
    G[a][b] = uc sum_{c,d} U[a][c]^2 C(E_d - E_c) U[a][d] U[b][d], the e block
    of sum_i diag(occ_i) U (Kt_i o C) U^T (redfield.py:41-104,
    liouville_space.py:316-341).  ``eigh`` defaults to the GPU Jacobi kernel
    (SymmetricEigh); a caller working on host tensors passes its own.
    """
    N = H1.shape[-1]
    eye = torch.eye(N, dtype=torch.float64, device=H1.device)
    H = H1 - rw_freq * eye
    E, U = (eigh or SymmetricEigh.apply)(H)
    x = E[:, None, :] - E[:, :, None]                 # x[c][d] = E_d - E_c
    C = DebyeCorr.apply(x, lam, temperature, cutoff_freq, matsubara_cutoff)
    Uc = U.to(torch.complex128)
    W = (U * U).to(torch.complex128) @ C              # W[a][d] = sum_c U[a][c]^2 C[c][d]
    G = unit_convert * ((W * Uc) @ Uc.transpose(1, 2))
    A = G + 1j * unit_convert * H.to(torch.complex128)
    return -A.transpose(1, 2)


def rk4_step_minus_identity(L, h):
    """D = P - I, P = sum_{k<=4} (hL)^k / k! (Paterson-Stockmeyer form)."""
    A = h * L
    A2 = A @ A
    return A + 0.5 * A2 + A2 @ (A / 6 + A2 / 24)


# ------------------------------------------------------------- time loop
class ProjectedMeanRK4(torch.autograd.Function):
    """x_n = (1/S) sum_s c^T (I + D_s)^n y0, n = 0..nsteps, with the
    hand-written adjoint kernel as backward (FP64)."""

    @staticmethod
    def forward(ctx, D, y0, c, nsteps, ck_every):
        D = D.detach().contiguous()
        S, m, _ = D.shape
        out = _native.rk4(D, y0, nsteps, 1, proj=c[None], per_sample=False, mean=True,
                          precision=_native.QSX_FP64)
        nck = max(1, -(-nsteps // ck_every))
        ck = _native.rk4(D, y0, (nck - 1) * ck_every, ck_every, state=True,
                         precision=_native.QSX_FP64)['state'] if nck > 1 else \
            y0.to(torch.complex128).expand(S, 1, m).contiguous()
        ctx.save_for_backward(D, ck, c)
        ctx.nsteps, ctx.ck_every = nsteps, ck_every
        return out['mean'][:, 0]

    @staticmethod
    def backward(ctx, g):
        D, ck, c = ctx.saved_tensors
        gradD = _native.rk4_adjoint(D, ck.contiguous(), ctx.ck_every, ctx.nsteps, c,
                                    g.contiguous(), 1.0 / D.shape[0])
        return gradD, None, None, None, None


class Dft(torch.autograd.Function):
    """X_k = dt sum_n x_n exp(i (f_k - rw) uc n dt) on a uniform frequency grid;
    backward applies the conjugate transpose with the same kernel."""

    @staticmethod
    def forward(ctx, x, dt, freqs, rw_freq, unit_convert):
        f = np.asarray(freqs, float)
        ctx.save_for_backward(torch.as_tensor(f))
        ctx.args = (len(x), dt, rw_freq, unit_convert)
        return _native.dft(x.detach(), 0.0, dt, torch.as_tensor(f), rw_freq, unit_convert, 1)

    @staticmethod
    def backward(ctx, g):
        (f,) = ctx.saved_tensors
        nt, dt, rw, uc = ctx.args
        f = f.numpy()
        df = (f[-1] - f[0]) / (len(f) - 1)
        t = torch.arange(nt, dtype=torch.float64) * dt
        gx = _native.dft(g.contiguous(), f[0] - rw, df, t, 0.0, uc, -1) * (dt / df)
        return gx, None, None, None, None


# ------------------------------------------------------------------ model
class AbsorptionFit:
    """Misfit of a disorder-averaged absorption spectrum on a frequency grid.

    Parameters theta (float64, N + N(N-1)/2 + 1 entries): N site
    energies, N(N-1)/2 couplings (upper triangle, row major) and lambda.
    ``offsets`` (S, N) are the disorder samples' site-energy shifts.
    """

    def __init__(self, n_sites, offsets, freqs, dipoles=None, temperature_K=77.0,
                 cutoff_freq=106.0, rw_freq=12300.0, dt=1.0, nsteps=2047, ck_every=64,
                 unit_convert=CM_FS, matsubara_cutoff=1000):
        self.N = n_sites
        self.offsets = torch.as_tensor(np.asarray(offsets, float)).cuda()
        self.freqs = np.asarray(freqs, float)
        df = np.diff(self.freqs)
        if len(self.freqs) < 2 or not np.allclose(df, df[0], rtol=1e-9, atol=0):
            raise ValueError('the frequency grid must be uniform')
        # exactly f_0 + k df, the grid the transposed transform assumes
        f = self.freqs
        self.freqs = f[0] + np.arange(len(f)) * ((f[-1] - f[0]) / (len(f) - 1))
        self.T = CM_K * temperature_K
        self.gamma = cutoff_freq
        self.rw = rw_freq
        self.dt = dt
        self.nsteps = nsteps
        self.ck_every = ck_every
        self.uc = unit_convert
        self.K = matsubara_cutoff
        mu = np.ones(n_sites) if dipoles is None else np.asarray(dipoles, float)[:, 0]
        # Heisenberg linear response (response.py:15-43) with V0 = mu^+ on
        # gg->eg and V1 = mu^- on eg->gg: v_rho0 = mu, y0 = -V1.bra = -mu.
        self.c = torch.as_tensor(mu, dtype=torch.complex128).cuda()
        self.y0 = -self.c.clone()
        iu = np.triu_indices(n_sites, 1)
        self._iu = (torch.as_tensor(iu[0]).cuda(), torch.as_tensor(iu[1]).cuda())

    def n_params(self):
        return self.N + self.N * (self.N - 1) // 2 + 1

    def pack(self, H1, lam):
        H1 = np.asarray(H1, float)
        iu = np.triu_indices(self.N, 1)
        return torch.as_tensor(np.concatenate([np.diag(H1), H1[iu], [lam]])).cuda()

    def hamiltonians(self, theta):
        N = self.N
        E = theta[:N]
        J = theta[N:-1]
        H = torch.zeros((N, N), dtype=torch.float64, device=theta.device)
        H = H.index_put((self._iu[0], self._iu[1]), J)
        H = H + H.T + torch.diag(E)
        return H[None] + torch.diag_embed(self.offsets)

    def generator(self, theta):
        return eg_heisenberg_generator(self.hamiltonians(theta), theta[-1], self.T,
                                       self.gamma, self.rw, self.uc, self.K)

    def signal(self, theta, impl='adjoint'):
        """x_n = ensemble-mean response at t_n = n dt (response.py:15-43)."""
        D = rk4_step_minus_identity(self.generator(theta), self.dt)
        if impl == 'adjoint':
            return ProjectedMeanRK4.apply(D, self.y0, self.c, self.nsteps, self.ck_every)
        if impl == 'autograd':
            y = self.y0.expand(D.shape[0], -1)
            out = [y @ self.c]
            for _ in range(self.nsteps):
                y = y + (D @ y[..., None])[..., 0]
                out.append(y @ self.c)
            return torch.stack(out, 1).mean(0)
        raise ValueError(impl)

    def spectrum(self, theta, impl='adjoint'):
        """Re X(omega) of -x on the grid (absorption_spectra, response.py:103-154)."""
        x = self.signal(theta, impl)
        if impl == 'adjoint':
            X = Dft.apply(-x, self.dt, self.freqs, self.rw, self.uc)
        else:
            t = torch.arange(len(x), dtype=torch.float64, device=x.device) * self.dt
            ph = (torch.as_tensor(self.freqs, device=x.device) - self.rw) * self.uc
            F = self.dt * torch.exp(1j * ph[:, None] * t[None, :])
            X = F @ (-x)
        return X.real

    def misfit(self, theta, target, impl='adjoint'):
        """Relative L2 misfit |S(theta) - target|^2 / |target|^2."""
        s = self.spectrum(theta, impl)
        return ((s - target) ** 2).sum() / (target ** 2).sum()

    def fit(self, theta0, target, steps=200, lr=1.0, impl='adjoint'):
        """Adam on the misfit from theta0; returns (theta, misfit history)."""
        theta = theta0.clone().requires_grad_(True)
        opt = torch.optim.Adam([theta], lr=lr)
        hist = []
        for _ in range(steps):
            opt.zero_grad()
            loss = self.misfit(theta, target, impl)
            loss.backward()
            opt.step()
            hist.append(float(loss.detach()))
        return theta.detach(), hist
