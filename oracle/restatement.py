"""Plain NumPy/SciPy restatement of QSpectra's Liouville-space propagation path.

TEST INFRASTRUCTURE ONLY.  This module is the oracle that the CUDA path is
checked against; the product package never imports it.  Every function cites
the reference file:line whose algorithm it restates (paths are relative to the
qspectra project root).  The reference integrates with SciPy's adaptive
``zvode``; this oracle replaces that one piece by a fixed-step classical RK4
loop (the integrator the GPU path implements), and the golden fixtures pin the
RK4 loop against the reference's own ``eom`` callables driven by the same RK4
loop, plus tight-tolerance ``zvode`` runs for the integrator gap.
"""
import itertools
from functools import lru_cache

import numpy as np
import scipy.linalg
import scipy.sparse as sps

# --------------------------------------------------------------------------
# constants (qspectra/constants.py:8-18)
# --------------------------------------------------------------------------
CM_FS_LINEAR = 2.99792458e-5
CM_FS = np.pi * 2 * CM_FS_LINEAR
CM_K = 0.69503476
GAUSSIAN_SD_FWHM = 1.0 / (2 * np.sqrt(2 * np.log(2)))


class SubspaceError(Exception):
    """Invalid Hilbert/Liouville subspace (operator_tools.py:273-276)."""


# --------------------------------------------------------------------------
# Hilbert-space bookkeeping (qspectra/operator_tools.py)
# --------------------------------------------------------------------------
def n_excitations(n_sites, n_vib=1):
    """Number of 0-, 1- and 2-excitation states (operator_tools.py:279-285)."""
    return np.array([1, n_sites, n_sites * (n_sites - 1) // 2]) * n_vib


def site_states(n_sites, subspace='gef'):
    """States as tuples of excited sites, hard-core bosons (operator_tools.py:122-152)."""
    out = []
    if 'g' in subspace:
        out.append(())
    if 'e' in subspace:
        out.extend((i,) for i in range(n_sites))
    if 'f' in subspace:
        out.extend(itertools.combinations(range(n_sites), 2))
    return out


def manifold_slices(n_sites, hilbert_subspace):
    """Slice of each manifold inside ``hilbert_subspace`` (operator_tools.py:311-335)."""
    counts = dict(zip('gef', n_excitations(n_sites)))
    out, start = {}, 0
    for letter in 'gef':
        if letter in hilbert_subspace:
            out[letter] = slice(start, start + counts[letter])
            start += counts[letter]
    return out


def two_exciton_operator(op1):
    """a†_n a_m operator lifted to the pair states (operator_tools.py:155-191)."""
    op1 = np.asarray(op1)
    pairs = np.array(list(itertools.combinations(range(len(op1)), 2)),
                     dtype=int).reshape(-1, 2)
    if len(pairs) == 0:
        return np.zeros((0, 0), dtype=op1.dtype)
    i, j = pairs[:, 0][:, None], pairs[:, 1][:, None]
    k, l = pairs[:, 0][None, :], pairs[:, 1][None, :]
    return (op1[j, l] * (i == k) + op1[j, k] * (i == l)
            + op1[i, l] * (j == k) + op1[i, k] * (j == l))


def extend_operator(op1, subspace='gef'):
    """Block-diagonal extension over the g/e/f manifolds (operator_tools.py:194-235)."""
    op1 = np.asarray(op1)
    blocks = []
    if 'g' in subspace:
        blocks.append(np.zeros((1, 1), dtype=op1.dtype))
    if 'e' in subspace:
        blocks.append(op1)
    if 'f' in subspace:
        blocks.append(two_exciton_operator(op1))
    return scipy.linalg.block_diag(*blocks).astype(op1.dtype)


def occupations(n_sites, subspace='gef'):
    """occ[i, s] = 1 when site i is excited in state s: the diagonals of the
    number operators used as system-bath couplings (hamiltonian.py:593-608)."""
    states = site_states(n_sites, subspace)
    occ = np.zeros((n_sites, len(states)))
    for s, st in enumerate(states):
        for i in st:
            occ[i, s] = 1.0
    return occ


def transition_matrix(site, n_sites, subspace='gef', transitions='-+'):
    """Create (+) / annihilate (-) an excitation on ``site`` (operator_tools.py:238-270)."""
    states = [tuple(s) for s in site_states(n_sites, subspace)]
    pos = {s: k for k, s in enumerate(states)}
    out = np.zeros((len(states), len(states)))
    for col, s in enumerate(states):
        if site in s:
            continue
        up = tuple(sorted(s + (site,)))
        if up in pos:
            if '+' in transitions:
                out[pos[up], col] = 1.0
            if '-' in transitions:
                out[col, pos[up]] = 1.0
    return out


COORD = {'x': np.array([1., 0, 0]), 'y': np.array([0., 1, 0]),
         'z': np.array([0., 0, 1])}


def polarization_vector(p):
    """polarization.py:14-36."""
    if isinstance(p, str):
        return COORD[p]
    if np.isscalar(p):
        return np.array([np.cos(p), np.sin(p), 0.0])
    p = np.asarray(p, float).reshape(-1)
    if len(p) != 3:
        raise ValueError('polarization vectors must have length 3')
    return p


def random_rotation_matrix(rng):
    """Uniformly distributed rotation from three uniforms (polarization.py:87-102;
    Arvo, Graphics Gems III, 1992): a rotation by 2 pi x1 about z, then the
    reflection through the plane normal to v(x2, x3), negated."""
    x1, x2, x3 = rng.rand(3)
    th, ph = 2 * np.pi * x1, 2 * np.pi * x2
    Rz = np.array([[np.cos(th), np.sin(th), 0.0],
                   [-np.sin(th), np.cos(th), 0.0],
                   [0.0, 0.0, 1.0]])
    v = np.array([np.cos(ph) * np.sqrt(x3), np.sin(ph) * np.sqrt(x3), np.sqrt(1 - x3)])
    return -(np.eye(3) - 2 * np.outer(v, v)) @ Rz


FOURTH_ORDER_PAIRINGS = (((0, 1), (2, 3)), ((0, 2), (1, 3)), ((0, 3), (1, 2)))


def isotropic_weights_4th(polarization):
    """Weights of the three fourth-rank invariants (polarization.py:55-70):
    (1/30)(5 I - 1) applied to the products of polarization dot products in
    each pairing (Hochstrasser 2001)."""
    e = np.array([polarization_vector(p) for p in polarization])
    c = e @ e.T
    prod = np.array([c[a] * c[b] for a, b in FOURTH_ORDER_PAIRINGS])
    return (5 * np.eye(3) - np.ones((3, 3))) @ prod / 30


def isotropic_average_4th(func, polarization, *args, **kw):
    """Exact isotropic average of a third-order signal (decorators.py:67-92):
    each invariant whose weight exceeds 1e-8 adds its weight times the sum of
    the signals over the nine lab polarizations whose paired indices agree."""
    signals, total, ticks = {}, 0, None
    for pairing, w in zip(FOURTH_ORDER_PAIRINGS, isotropic_weights_4th(polarization)):
        if w <= 1e-8:
            continue
        for p in itertools.product('xyz', repeat=4):
            if all(p[a] == p[b] for a, b in pairing):
                key = ''.join(p)
                if key not in signals:
                    ticks, signals[key] = func(*args, polarization=key, **kw)
                total = total + w * signals[key]
    return ticks, total


def isotropic_average_2nd(func, polarization, *args, **kw):
    """Exact isotropic average of a second-order signal (decorators.py:95-125):
    (e1 . e2) / 3 times the sum of the 'xx', 'yy' and 'zz' signals."""
    e = [polarization_vector(p) for p in polarization]
    total, ticks = 0, None
    for p in ('xx', 'yy', 'zz'):
        ticks, sig = func(*args, polarization=p, **kw)
        total = total + sig
    return ticks, total * (np.dot(e[0], e[1]) / 3.0)


def dipole_operator(dipoles, subspace, polarization, transitions='-+'):
    """Σ_n T_n (d_n · e) (hamiltonian.py:580-591)."""
    dipoles = np.asarray(dipoles, float)
    n = len(dipoles)
    proj = dipoles @ polarization_vector(polarization)
    return sum(proj[s] * transition_matrix(s, n, subspace, transitions)
               for s in range(n))


# --------------------------------------------------------------------------
# Liouville-space conventions (qspectra/dynamics/liouville_space.py)
# --------------------------------------------------------------------------
def ket_vec(m):
    """Column-stacked vectorisation (liouville_space.py:46-50)."""
    return np.asarray(m).reshape(-1, order='F')


def ket_mat(v):
    """Inverse of ``ket_vec`` (liouville_space.py:53-58)."""
    n = int(round(np.sqrt(np.size(v))))
    return np.asarray(v).reshape((n, n), order='F')


def bra_vec(m):
    """Row-stacked vectorisation (liouville_space.py:61-65)."""
    return np.asarray(m).reshape(-1, order='C')


def tensor_to_super(r):
    """S[a + N b, c + N d] = R[a, b, c, d] (liouville_space.py:68-90)."""
    n = r.shape[0]
    return np.ascontiguousarray(r.transpose(1, 0, 3, 2)).reshape(n * n, n * n)


def super_left(op):
    """vec(op ρ) = (I ⊗ op) vec ρ (liouville_space.py:102-115)."""
    return np.kron(np.eye(len(op)), op)


def super_right(op):
    """vec(ρ op) = (opᵀ ⊗ I) vec ρ (liouville_space.py:118-131)."""
    return np.kron(np.asarray(op).T, np.eye(len(op)))


def super_commutator(op):
    """liouville_space.py:93-99."""
    return super_left(op) - super_right(op)


def liouville_subspace_index(liouville_subspace, hilbert_subspace, n_sites):
    """Ascending column-stacked indices of the requested blocks (liouville_space.py:9-29)."""
    sl = manifold_slices(n_sites, hilbert_subspace)
    n = sum(s.stop - s.start for s in sl.values())
    keep = np.zeros((n, n), dtype=bool)
    for block in liouville_subspace.split(','):
        row, col = block
        if row not in sl or col not in sl:
            raise SubspaceError('{}{} not in subspace {!r}'.format(
                row, col, hilbert_subspace))
        keep[sl[row], sl[col]] = True
    return np.flatnonzero(ket_vec(keep))


def extract_subspace(s):
    """operator_tools.py:292-298."""
    return sorted(set(s) - {',', '-', '>'}, key='gef'.index)


def full_liouville_subspace(s):
    """operator_tools.py:301-308."""
    h = extract_subspace(s)
    return ','.join(a + b for a in h for b in h)


# --------------------------------------------------------------------------
# Electronic Hamiltonian (qspectra/hamiltonian.py:464-631)
# --------------------------------------------------------------------------
class ElectronicHamiltonianSpec:
    """The numbers the path needs from ``ElectronicHamiltonian``.

    ``H1`` is the NON-rotating 1-exciton matrix (sampled or not); ``rw_freq``
    the rotating-wave frequency, default mean(E_e) (hamiltonian.py:177-209,
    375-380).  Disorder follows ``_sample`` (hamiltonian.py:552-578).
    """

    def __init__(self, H1, dipoles=None, rw_freq=None, disorder=None,
                 random_seed=0, energy_spread_extra=None, bath=None):
        self.H1 = np.asarray(H1, float)
        self.dipoles = None if dipoles is None else np.asarray(dipoles, float)
        self.disorder = disorder
        self.random_seed = random_seed
        self.energy_spread_extra = energy_spread_extra
        self.bath = bath
        self.n_sites = len(self.H1)
        self._unsampled = self
        if rw_freq is None:
            rw_freq = float(np.mean(scipy.linalg.eigh(self.H1)[0]))
        self.rw_freq = rw_freq

    def sample(self, n, random_orientations=False):
        """hamiltonian.py:233-274 and :552-578 (diagonal Gaussian disorder,
        then, with random_orientations, a uniform rotation of the dipoles
        drawn from the same RandomState)."""
        seed = list(np.atleast_1d(self.random_seed)) + [n]
        rng = np.random.RandomState(seed)
        if self.disorder is None:
            shift = np.zeros((self.n_sites, self.n_sites))
        else:
            shift = np.diag((self.disorder * GAUSSIAN_SD_FWHM)
                            * rng.randn(self.n_sites))
        dipoles = self.dipoles
        if random_orientations:
            R = random_rotation_matrix(rng)
            dipoles = np.array([R @ d for d in self.dipoles])
        out = ElectronicHamiltonianSpec(
            self.H1 + shift, dipoles, self.rw_freq, self.disorder,
            seed, self.energy_spread_extra, self.bath)
        out._unsampled = self._unsampled
        return out

    def H(self, subspace):
        """Rotating-frame H (hamiltonian.py:539-550)."""
        return extend_operator(self.H1 - self.rw_freq * np.eye(self.n_sites),
                               subspace)

    def eig(self, subspace):
        """eigh of the NON-rotating H, then subtract k·rw (hamiltonian.py:310-328)."""
        E, U = scipy.linalg.eigh(extend_operator(self.H1, subspace))
        sl = manifold_slices(self.n_sites, subspace)
        if 'e' in sl:
            E[sl['e']] -= self.rw_freq
        if 'f' in sl:
            E[sl['f']] -= 2 * self.rw_freq
        return E, U

    def time_step(self, unit_convert=1.0):
        """Nyquist step, fixed under sampling (hamiltonian.py:382-412, base.py:130-136)."""
        base = self._unsampled
        E = base.eig('gef')[0]
        if self.energy_spread_extra is None:
            extra = 0.01 * float(np.mean(scipy.linalg.eigh(base.H1)[0]))
        else:
            extra = self.energy_spread_extra
        fmax = max(E.max(), -E.min()) + extra
        return 1.0 / (2 * fmax) / unit_convert

    def couplings(self, subspace):
        """Number operators n_i (hamiltonian.py:593-608)."""
        occ = occupations(self.n_sites, subspace)
        return np.array([np.diag(o) for o in occ])

    def dipole(self, subspace, polarization, transitions='-+'):
        return dipole_operator(self.dipoles, subspace, polarization,
                               transitions)

    def thermal_state(self, subspace, temperature):
        """exp(-H/T)/Z on the non-rotating H (hamiltonian.py:49-78, 163-175)."""
        H = extend_operator(self.H1, subspace)
        if temperature > 0:
            rho = scipy.linalg.expm(-H / float(temperature))
            tr = np.trace(rho)
            if tr == 0 or np.isnan(rho).any():
                raise OverflowError('temperature too low for thermal_state')
            rho = rho / tr
        else:
            E, U = scipy.linalg.eigh(H)
            rho = np.mean([np.outer(U[:, i], U[:, i])
                           for i in range(len(U)) if E[i] == E[0]], axis=0)
        return rho.astype(complex)


# --------------------------------------------------------------------------
# Debye bath (qspectra/bath.py)
# --------------------------------------------------------------------------
class DebyeBathSpec:
    def __init__(self, temperature, reorg_energy, cutoff_freq):
        self.temperature = float(temperature)
        self.reorg_energy = float(reorg_energy)
        self.cutoff_freq = float(cutoff_freq)

    def corr_complex(self, x, matsubara_cutoff=1000):
        """One-sided C(ω) with the truncated Matsubara sum (bath.py:84-102)."""
        T, lam, gam = self.temperature, self.reorg_energy, self.cutoff_freq
        if x == 0:
            return lam * (2 * T / gam - 1j)
        nu = 2 * np.pi * np.arange(matsubara_cutoff) * T
        tail = np.sum(nu / ((nu ** 2 - gam ** 2) * (nu - 1j * x)))
        return lam * gam * ((1 / np.tan(gam / (2 * T)) - 1j) / (gam - 1j * x)
                            + 4 * T * tail)

    def spectral_density(self, x):
        """bath.py:76-82."""
        return (2 * self.reorg_energy * self.cutoff_freq * x
                / (self.cutoff_freq ** 2 + x ** 2))

    def corr_real(self, x):
        """(n(x)+1) J_anti(x); T J'(0) at x = 0 (bath.py:17-31)."""
        T = self.temperature
        if x == 0:
            return T * 2 * self.reorg_energy / self.cutoff_freq
        janti = self.spectral_density(x) if x >= 0 else -self.spectral_density(-x)
        return (1 / np.expm1(x / T) + 1) * janti


# --------------------------------------------------------------------------
# Redfield theory (qspectra/dynamics/redfield.py)
# --------------------------------------------------------------------------
def secular_mask(n):
    """(a=b and c=d) or (a=c and b=d) (redfield.py:77-83)."""
    e = np.eye(n, dtype=bool)
    return e[:, :, None, None] & e[None, None, :, :] | \
        e[:, None, :, None] & e[None, :, None, :]


def redfield_tensor(E, U, couplings, corr, secular=False):
    """Eigenbasis Redfield tensor R_abcd (redfield.py:9-74).

    Γ_abcd = Σ_i K_i,ab K_i,cd C(E_d − E_c) and
    R_abcd = δ_ac conj(ΓS_bd) + δ_bd ΓS_ac − conj(Γ_cabd) − Γ_dbac
    with ΓS_ac = Σ_b Γ_abbc (May & Kuhn eqs. 3.319 and 3.322).
    """
    n = len(E)
    K = np.array([U.conj().T @ k @ U for k in couplings])
    Cw = np.array([[corr(E[c] - E[d]) for d in range(n)] for c in range(n)])
    gamma = np.einsum('iab,icd->abcd', K, K) * Cw.T[None, None, :, :]
    gs = np.einsum('abbc->ac', gamma)
    eye = np.eye(n)
    R = (eye[:, None, :, None] * gs.conj()[None, :, None, :]
         + gs[:, None, :, None] * eye[None, :, None, :]
         - gamma.conj().transpose(1, 2, 0, 3)
         - gamma.transpose(2, 1, 3, 0))
    if secular:
        R = R * secular_mask(n)
    return R


def redfield_liouvillian(E, U, couplings, corr, secular=False, basis='site'):
    """L = -i[diag E, ·] - R, then (U⊗U) L (U⊗U)† in the site basis (redfield.py:95-104)."""
    R = redfield_tensor(E, U, couplings, corr, secular)
    L = -1j * super_commutator(np.diag(E)) - tensor_to_super(R)
    if basis == 'site':
        W = np.kron(U, U)
        L = W @ L @ W.conj().T
    elif basis != 'eigen':
        raise ValueError('invalid basis')
    return L


class RedfieldSpec:
    """What ``RedfieldModel`` computes (redfield.py:107-152, liouville_space.py:212-349)."""

    def __init__(self, ham, bath, hilbert_subspace='gef', unit_convert=1.0,
                 secular=True, discard_imag_corr=False, evolve_basis='site'):
        self.ham = ham
        self.bath = bath
        self.hilbert_subspace = hilbert_subspace
        self.unit_convert = unit_convert
        self.secular = secular
        self.discard_imag_corr = discard_imag_corr
        self.evolve_basis = evolve_basis
        self._L = None

    @property
    def n_sites(self):
        return self.ham.n_sites

    def sample(self, n, random_orientations=False):
        return RedfieldSpec(self.ham.sample(n, random_orientations), self.bath,
                            self.hilbert_subspace, self.unit_convert,
                            self.secular, self.discard_imag_corr,
                            self.evolve_basis)

    @property
    def time_step(self):
        return self.ham.time_step(self.unit_convert)

    def evolution_super_operator(self):
        """unit_convert · redfield_evolve (redfield.py:146-152)."""
        if self._L is None:
            E, U = self.ham.eig(self.hilbert_subspace)
            corr = (self.bath.corr_real if self.discard_imag_corr
                    else self.bath.corr_complex)
            self._L = self.unit_convert * redfield_liouvillian(
                E, U, self.ham.couplings(self.hilbert_subspace), corr,
                self.secular, self.evolve_basis)
        return self._L

    def index(self, liouville_subspace):
        return liouville_subspace_index(liouville_subspace,
                                        self.hilbert_subspace, self.n_sites)

    def eom_matrix(self, liouville_subspace, heisenberg_picture=False):
        """L[idx, idx], transposed for the Heisenberg picture (liouville_space.py:316-341)."""
        idx = self.index(liouville_subspace)
        L = self.evolution_super_operator()[np.ix_(idx, idx)]
        return L.T if heisenberg_picture else L

    def map_between_subspaces(self, state, from_s, to_s):
        """liouville_space.py:343-349."""
        n = len(extend_operator(self.ham.H1, self.hilbert_subspace))
        full = np.zeros(n * n, dtype=complex)
        full[self.index(from_s)] = state
        return full[self.index(to_s)]

    def thermal_state(self, liouville_subspace):
        """liouville_space.py:300-309 (site basis)."""
        if self.evolve_basis != 'site':
            raise NotImplementedError('oracle thermal_state is site-basis only')
        rho0 = self.ham.thermal_state(liouville_subspace,
                                      self.bath.temperature)
        full = full_liouville_subspace(liouville_subspace)
        return self.map_between_subspaces(ket_vec(rho0), full,
                                          liouville_subspace)

    def operator(self, op, subspace_map):
        return LiouvilleOperator(op, subspace_map, self)

    def dipole(self, subspace_map, polarization, transitions):
        op = self.ham.dipole(self.hilbert_subspace, polarization, transitions)
        if self.evolve_basis == 'eigen':
            U = self.ham.eig(self.hilbert_subspace)[1]
            op = U.conj().T @ op @ U
        return LiouvilleOperator(op, subspace_map, self)


class LiouvilleOperator:
    """Dipole super-operators restricted to from/to subspaces (liouville_space.py:151-209)."""

    def __init__(self, op, subspace_map, model):
        self.op = np.asarray(op)
        parts = (subspace_map.split('->') if '->' in subspace_map
                 else [subspace_map, subspace_map])
        self.from_idx = model.index(parts[0])
        self.to_idx = model.index(parts[1])
        self.mesh = np.ix_(self.to_idx, self.from_idx)

    @property
    def bra_vector(self):
        return bra_vec(np.asarray(self.op, dtype=complex))[self.from_idx]

    @property
    def left_matrix(self):
        return super_left(self.op)[self.mesh]

    @property
    def right_matrix(self):
        return super_right(self.op)[self.mesh]

    @property
    def commutator_matrix(self):
        return super_commutator(self.op)[self.mesh]

    def commutator(self, state):
        return np.asarray(state) @ self.commutator_matrix.T

    def left_multiply(self, state):
        return np.asarray(state) @ self.left_matrix.T

    def right_multiply(self, state):
        return np.asarray(state) @ self.right_matrix.T

    @property
    def expectation_row(self):
        tr = np.eye(len(self.op)).reshape(-1)[self.to_idx]
        return tr @ self.left_matrix

    def expectation_value(self, state):
        return np.asarray(state) @ self.expectation_row


# --------------------------------------------------------------------------
# Time loop (qspectra/simulate/utils.py:16-109), zvode -> fixed-step RK4
# --------------------------------------------------------------------------
def rk4_step_matrix(L, h):
    """One RK4 step for dy/dt = L y as stages (simulate/utils.py:44-49 loop body)."""
    def step(Y):
        k1 = Y @ L.T
        k2 = (Y + 0.5 * h * k1) @ L.T
        k3 = (Y + 0.5 * h * k2) @ L.T
        k4 = (Y + h * k3) @ L.T
        return Y + (h / 6.0) * (k1 + 2 * k2 + 2 * k3 + k4)
    return step


def rk4_integrate(L, y0, t, t0=None, save=None, h=None):
    """Fixed-step RK4 output at the times ``t`` (simulate/utils.py:16-109).

    ``y0`` may carry leading batch axes (the reference loops over them
    serially, utils.py:106-109; the map is linear so batching is exact).
    ``h`` defaults to t[1] - t[0]; every output time must be a whole number
    of steps from ``t0`` (default t[0]).  ``save`` is a matrix S applied as
    S @ y (a linear ``save_func``) or None.
    """
    t = np.asarray(t, float)
    y = np.array(y0, dtype=complex)
    if t0 is None:
        t0 = t[0]
    if h is None:
        h = t[1] - t[0] if len(t) > 1 else 1.0
    step = rk4_step_matrix(np.asarray(L), h)
    out = []
    cur = t0
    for ti in t:
        nsteps = int(round((ti - cur) / h))
        for _ in range(nsteps):
            y = step(y)
        cur = cur + nsteps * h
        out.append(y if save is None else y @ np.asarray(save).T)
    return np.stack(out, axis=-2)


# --------------------------------------------------------------------------
# Fourier transform (qspectra/simulate/utils.py:122-219)
# --------------------------------------------------------------------------
def symmetrize(t, x, axis=-1):
    """Zero-pad to a time grid symmetric about 0 (simulate/utils.py:128-151)."""
    t = np.asarray(t, float)
    x = np.asarray(x)
    d = np.diff(t)
    if not (np.max(np.abs(d - d[0])) < 1e-7 and np.all(d > 0)):
        raise ValueError('sample times must differ by a positive constant')
    T = max(t[-1], -t[0])
    dt = t[1] - t[0]
    n_plus = int((T - t[-1]) / dt) + 1
    n_minus = int((T + t[0]) / dt) + 1
    t_sym = np.concatenate([t[0] - dt * np.arange(1, n_minus)[::-1], t,
                            t[-1] + dt * np.arange(1, n_plus)])
    axis = axis % x.ndim
    shape = list(x.shape)
    shape[axis] = t_sym.size
    x_sym = np.zeros(shape, dtype=x.dtype)
    start = np.searchsorted(t_sym, t[0])
    sl = [slice(None)] * x.ndim
    sl[axis] = slice(start, start + t.size)
    x_sym[tuple(sl)] = x
    return t_sym, x_sym


def fourier_transform(t, x, axis=-1, rw_freq=0, unit_convert=1, sign=1,
                      convention='angular'):
    """∫ exp(i(ω-ω0)t) x(t) dt by FFT (simulate/utils.py:154-219)."""
    if convention == 'angular':
        unit_convert = unit_convert / (2 * np.pi)
    elif convention != 'linear':
        raise ValueError("convention must be 'angular' or 'linear'")
    if sign not in (-1, 1):
        raise ValueError('sign must be +1 or -1')
    t, x = symmetrize(t, x, axis)
    n = x.shape[axis]
    dt = t[1] - t[0]
    f = np.fft.fftshift(np.fft.fftfreq(n, dt * unit_convert))
    X = np.fft.fftshift(np.fft.fft(np.fft.ifftshift(x * dt, axes=axis),
                                   axis=axis), axes=axis)
    if sign == 1:
        f = -f[::-1]
        X = np.flip(X, axis=axis)
    return f + rw_freq, X


# --------------------------------------------------------------------------
# Drivers (qspectra/simulate/eom.py, response.py)
# --------------------------------------------------------------------------
def time_grid(time_max, dt):
    """np.arange(0, time_max, time_step) as used by every driver (response.py:21)."""
    return np.arange(0, time_max, dt)


def simulate_dynamics(model, psi_or_rho, duration, liouville_subspace='ee',
                      dt=None):
    """eom.py:11-26: ρ0 → subspace vector → RK4 → (T, N, N) in F order."""
    rho0 = np.asarray(psi_or_rho)
    if rho0.ndim == 1:
        rho0 = np.outer(rho0.conj(), rho0)
    y0 = ket_vec(rho0)
    full = full_liouville_subspace(liouville_subspace)
    y0 = model.map_between_subspaces(y0, full, liouville_subspace) \
        if full != liouville_subspace else y0
    dt = model.time_step if dt is None else dt
    t = time_grid(duration, dt)
    L = model.eom_matrix(liouville_subspace)
    states = rk4_integrate(L, y0, t)
    n = int(round(np.sqrt(states.shape[-1])))
    return t, states.reshape(-1, n, n, order='F')


def linear_response(model, time_max, polarization='xx', path='gg->eg->gg',
                    dt=None, initial_state=None):
    """Heisenberg-picture linear response (response.py:15-43); the initial
    state defaults to the thermal state of the path's first subspace."""
    subs = path.split('->')
    rho0 = (model.thermal_state(subs[0]) if initial_state is None
            else np.asarray(initial_state))
    dt = model.time_step if dt is None else dt
    t = time_grid(time_max, dt)
    signal = 0
    for sim in subs[1].split(','):
        V0 = model.dipole('{}->{}'.format(subs[0], sim), polarization[0], '+')
        V1 = model.dipole('{}->{}'.format(sim, subs[2]), polarization[1], '-')
        v_rho0 = V0.commutator(rho0)
        LH = model.eom_matrix(sim, heisenberg_picture=True)
        v_gt = rk4_integrate(LH, -V1.bra_vector, t)
        signal = signal + v_gt @ v_rho0
    return t, signal


PUMP_PROBE_PATHWAYS = {'GSB': 'gg->eg->gg', 'ESE': 'ee->eg->gg', 'ESA': 'ee->fe->ee'}
"""Pump-probe Liouville pathways (response.py:157-160)."""


def impulsive_probe(model, state, time_max, polarization='xx',
                    initial_liouv_subspace='gg,ge,eg,ee', include_signal='GSB,ESE,ESA'):
    """response.py:174-244: the state minus the thermal state, split over the
    selected pump-probe pathways, each portion's linear response summed, then
    the Fourier transform (sign +1, rw_freq added)."""
    init = np.asarray(state) - model.thermal_state(initial_liouv_subspace)
    total, t = 0, None
    for name, path in PUMP_PROBE_PATHWAYS.items():
        if name not in include_signal:
            continue
        first = path.split('->')[0]
        portion = model.map_between_subspaces(init, initial_liouv_subspace, first)
        t, sig = linear_response(model, time_max, polarization, path, initial_state=portion)
        total = total + sig
    return fourier_transform(t, total, rw_freq=model.ham.rw_freq,
                             unit_convert=model.unit_convert)


def two_dimensional_spectra(model, coherence_time_max, population_times, geometry='-++',
                            polarization='xxxx', include_signal=None):
    """response.py:430-455: the third-order response transformed over t1
    (sign -1, axis 0) and then t3 (sign +1, axis 2)."""
    (t1, t2, t3), X = third_order_response(model, coherence_time_max, population_times,
                                           geometry, polarization, include_signal)
    rw, uc = model.ham.rw_freq, model.unit_convert
    f1, X1 = fourier_transform(t1, X, 0, rw_freq=rw, sign=-1, unit_convert=uc)
    f3, X3 = fourier_transform(t3, X1, 2, rw_freq=rw, unit_convert=uc)
    return (f1, t2, f3), X3


def absorption_spectra(model, time_max, polarization='xx', dt=None,
                       correlation_decay_time=None):
    """response.py:103-154."""
    t, x = linear_response(model, time_max, polarization, dt=dt)
    if correlation_decay_time is not None:
        x = x * np.exp(-t / correlation_decay_time)
    f, X = fourier_transform(t, -x, rw_freq=model.ham.rw_freq,
                             unit_convert=model.unit_convert)
    return f, X.real


THIRD_ORDER_PATHWAYS = {
    '-++': {'ESE': 'gg->ge->ee->eg->gg', 'GSB': 'gg->ge->gg->eg->gg',
            'ESA': 'gg->ge->ee->fe->ee'},
    '+-+': {'ESE': 'gg->eg->ee->eg->gg', 'GSB': 'gg->eg->gg->eg->gg',
            'ESA': 'gg->eg->ee->fe->ee'},
    '++-': {'ESA1': 'gg->eg->fg->fe->ee', 'ESA2': 'gg->eg->fg->eg->gg'},
}
"""Liouville pathways per geometry (response.py:252-264; Abramavicius et al. 2009)."""


def third_order_response(model, coherence_time_max, population_times,
                         geometry='-++', polarization='xxxx',
                         include_signal=None, dt=None):
    """Sum over pathways of t1 → t2 → Heisenberg t3 (response.py:267-337)."""
    dt = model.time_step if dt is None else dt
    t1 = time_grid(coherence_time_max, dt)
    t3 = time_grid(coherence_time_max, dt)
    t2 = np.asarray(population_times, float)
    rho0 = model.thermal_state('gg')
    total = 0
    for name, path in THIRD_ORDER_PATHWAYS[geometry].items():
        if include_signal is not None and name not in include_signal:
            continue
        subs = path.split('->')
        V = [model.dipole('{}->{}'.format(a, b), p, tr)
             for a, b, p, tr in zip(subs[:-1], subs[1:], polarization,
                                    geometry + '-')]
        L = [model.eom_matrix(s) for s in subs[1:-1]]
        v_rho0 = V[0].commutator(rho0)
        v_rho1 = rk4_integrate(L[0], v_rho0, t1,
                               save=V[1].commutator_matrix, h=dt)
        v_rho2 = rk4_integrate(L[1], v_rho1, t2, t0=0.0,
                               save=V[2].commutator_matrix, h=dt)
        LH = model.eom_matrix(subs[3], heisenberg_picture=True)
        v_gt3 = rk4_integrate(LH, V[3].bra_vector, t3, h=dt)
        total = total + np.einsum('ci,abi->abc', v_gt3, v_rho2)
    return (t1, t2, t3), total


class GaussianPulseSpec:
    """E(t) = scale exp(i fc (carrier - rw)(t - t_peak) - (t - t_peak)^2 / 2 sigma^2)
    on [t_peak - 3 sigma, t_peak + 3 sigma], sigma = fwhm GAUSSIAN_SD_FWHM
    (pulse.py:74-113)."""

    def __init__(self, carrier_freq, fwhm, t_peak=0.0, scale=1.0, freq_convert=1.0,
                 t_limits_multiple=3):
        sigma = GAUSSIAN_SD_FWHM * fwhm
        self.two_sigma_squared = 2 * sigma ** 2
        self.t_init = t_peak - t_limits_multiple * sigma
        self.t_final = t_peak + t_limits_multiple * sigma
        self.t_peak, self.carrier_freq = t_peak, carrier_freq
        self.scale, self.freq_convert = scale, freq_convert

    def __call__(self, t, rw_freq):
        d = t - self.t_peak
        return self.scale * np.exp(1j * self.freq_convert * (self.carrier_freq - rw_freq) * d
                                   - d ** 2 / self.two_sigma_squared)


def simulate_with_fields(model, pulses, geometry='-+', polarization='xx', time_extra=0.0,
                         times=None, liouville_subspace='gg,ge,eg,ee', dt=None):
    """RK4 form of _simulate_with_fields (eom.py:77-105): dy/dt = L y +
    sum_p (-i E_p(t)^(*)) [V_p, y], from the thermal state at the first
    pulse's start, outputs on arange(t0, tf + time_extra, time_step)."""
    dt = model.time_step if dt is None else dt
    L = model.eom_matrix(liouville_subspace)
    C = [model.dipole(liouville_subspace, pol, tr).commutator_matrix
         for pol, tr in zip(polarization, geometry)]

    def f(t, y):
        d = L @ y
        for pulse, tr, Cp in zip(pulses, geometry, C):
            E = pulse(t, model.ham.rw_freq)
            if tr == '+':
                E = np.conj(E)
            d = d + (-1j * E) * (Cp @ y)
        return d

    y = np.array(model.thermal_state(liouville_subspace), dtype=complex)
    t0 = min(p.t_init for p in pulses)
    tf = max(p.t_final for p in pulses)
    t = (np.arange(t0, tf + time_extra, model.time_step) if times is None
         else tf + np.asarray(times, float))
    out, cur = [], t0
    for ti in t:
        for _ in range(int(round((ti - cur) / dt))):
            k1 = f(cur, y)
            k2 = f(cur + dt / 2, y + dt / 2 * k1)
            k3 = f(cur + dt / 2, y + dt / 2 * k2)
            k4 = f(cur + dt, y + dt * k3)
            y = y + dt / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
            cur = cur + dt
        out.append(y.copy())
    return t, np.array(out)


def ensemble_average(model, n_samples, func, *args, random_orientations=False, **kw):
    """Serial ensemble loop then mean (decorators.py:40-64)."""
    acc = None
    ticks = None
    for n in range(n_samples):
        ticks, sig = func(model.sample(n, random_orientations), *args, **kw)
        acc = sig if acc is None else acc + sig
    return ticks, acc / n_samples


# --------------------------------------------------------------------------
# HEOM (qspectra/dynamics/heom.py)
# --------------------------------------------------------------------------
@lru_cache(maxsize=None)
def _stars_and_bars(n, c):
    """Enumerate n-bin occupations with total c in the order of
    ``multichoose`` (heom.py:155-174): first every vector whose first bin is
    empty (recursing on the remaining bins), then every vector of total c-1
    with its first bin incremented."""
    if c == 0:
        return ((0,) * n,)
    if n == 0:
        return ()
    if n == 1:
        return ((c,),)
    head0 = tuple((0,) + v for v in _stars_and_bars(n - 1, c))
    head1 = tuple((v[0] + 1,) + v[1:] for v in _stars_and_bars(n, c - 1))
    return head0 + head1


def ado_indices(n_sites, K, level_cutoff):
    """All N×(K+1) occupation matrices with sum < level_cutoff (heom.py:92-152)."""
    out = []
    for c in range(level_cutoff):
        out.extend(_stars_and_bars(n_sites * (K + 1), c))
    return [np.array(v).reshape(n_sites, K + 1) for v in out]


def matsubara_frequencies(K, gamma, T):
    """ν_0 = γ, ν_k = 2πkT (heom.py:61-67)."""
    v = 2 * np.pi * T * np.arange(K + 1)
    v[0] = gamma
    return v


def heom_coefficients(K, gamma, T, lam, nu, aki=False):
    """c_0 = λγ(cot(γ/2T) − i), c_k = 4λγTν_k/(ν_k² − γ²) (heom.py:69-89)."""
    if aki:
        c0 = lam * gamma * (1 / (gamma / (2 * T)) - 1j)
    else:
        c0 = lam * gamma * (1 / np.tan(gamma / (2 * T)) - 1j)
    out = [c0]
    for k in range(1, K + 1):
        out.append(4 * lam * gamma * T * nu[k] / (nu[k] ** 2 - gamma ** 2))
    return out


class HEOMSpec:
    """What ``HEOMModel`` computes (heom.py:177-443), site basis."""

    def __init__(self, ham, bath, hilbert_subspace='gef', unit_convert=1.0,
                 level_cutoff=3, K=1, low_temp_corr=True, modified_HEOM=False):
        self.ham = ham
        self.bath = bath
        self.hilbert_subspace = hilbert_subspace
        self.unit_convert = unit_convert
        self.level_cutoff = level_cutoff
        self.K = K
        self.low_temp_corr = low_temp_corr
        self.modified_HEOM = modified_HEOM
        self.ados = ado_indices(ham.n_sites, K, level_cutoff)
        self.ado_count = len(self.ados)
        self._pos = {tuple(a.reshape(-1)): i for i, a in enumerate(self.ados)}

    def sample(self, n):
        return HEOMSpec(self.ham.sample(n), self.bath, self.hilbert_subspace,
                        self.unit_convert, self.level_cutoff, self.K,
                        self.low_temp_corr, self.modified_HEOM)

    def index(self, liouville_subspace):
        return liouville_subspace_index(liouville_subspace,
                                        self.hilbert_subspace,
                                        self.ham.n_sites)

    def temp_corr_coeff(self):
        """Σ_{k>K} c_k/ν_k over 5000 extra Matsubara terms (heom.py:387-393)."""
        T, lam, g = (self.bath.temperature, self.bath.reorg_energy,
                     self.bath.cutoff_freq)
        nu_inf = matsubara_frequencies(self.K + 5000, g, T)
        c_inf = heom_coefficients(self.K + 5000, g, T, lam, nu_inf)
        return np.sum((np.array(c_inf) / nu_inf)[self.K + 1:])

    def heom_tensor(self, liouville_subspace):
        """Block-sparse HEOM generator over ADO nodes (heom.py:298-443)."""
        T, lam, g = (self.bath.temperature, self.bath.reorg_energy,
                     self.bath.cutoff_freq)
        idx = self.index(liouville_subspace)
        mesh = np.ix_(idx, idx)
        M = idx.size
        nu = matsubara_frequencies(self.K, g, T)
        c = heom_coefficients(self.K, g, T, lam, nu)
        H = self.ham.H(self.hilbert_subspace)
        comm = super_commutator(H)[mesh]
        ops = self.ham.couplings(self.hilbert_subspace)
        left = [super_left(k)[mesh] for k in ops]
        right = [super_right(k)[mesh] for k in ops]
        tcorr = 0
        if self.low_temp_corr:
            tcoef = self.temp_corr_coeff()
            dc = sum(l + r - 2 * l @ r for l, r in zip(left, right))
            tcorr = tcoef * dc
        rows, cols, vals = [], [], []

        def put(bi, bj, block):
            block = sps.coo_matrix(block)
            rows.append(block.row + bi * M)
            cols.append(block.col + bj * M)
            vals.append(block.data.astype(complex))

        eye = np.eye(M)
        for n, ado in enumerate(self.ados):
            shift = np.sum(ado.dot(nu))
            put(n, n, -1j * comm - shift * eye - tcorr)
            for (j, k), njk in np.ndenumerate(ado):
                up = ado.copy()
                up[j, k] += 1
                p = self._pos.get(tuple(up.reshape(-1)))
                if p is not None:
                    mod = (np.sqrt((njk + 1) * np.abs(c[k]))
                           if self.modified_HEOM else 1)
                    put(n, p, -1j * mod * (left[j] - right[j]))
                if njk > 0:
                    dn = ado.copy()
                    dn[j, k] -= 1
                    m = self._pos[tuple(dn.reshape(-1))]
                    mod = (np.sqrt(njk / np.abs(c[k])) if self.modified_HEOM
                           else njk)
                    put(n, m, -1j * mod * (c[k] * left[j]
                                           - np.conj(c[k]) * right[j]))
        N = self.ado_count * M
        L = sps.coo_matrix((np.concatenate(vals),
                            (np.concatenate(rows), np.concatenate(cols))),
                           shape=(N, N)).tocsr()
        L.sum_duplicates()
        return L

    def eom_matrix(self, liouville_subspace, heisenberg_picture=False):
        """heom.py:228-244."""
        L = self.unit_convert * self.heom_tensor(liouville_subspace)
        return L.T.tocsr() if heisenberg_picture else L

    def initial_state(self, rho0_vec):
        """Embed in node 0 (heom.py:278-286)."""
        out = np.zeros(rho0_vec.size * self.ado_count, dtype=complex)
        out[:rho0_vec.size] = rho0_vec
        return out


def rk4_integrate_sparse(L, y0, nsteps, h, save_every=1):
    """RK4 with a sparse generator; returns states every ``save_every`` steps."""
    y = np.array(y0, dtype=complex)
    out = [y.copy()]
    for s in range(1, nsteps + 1):
        k1 = L @ y
        k2 = L @ (y + 0.5 * h * k1)
        k3 = L @ (y + 0.5 * h * k2)
        k4 = L @ (y + h * k3)
        y = y + (h / 6.0) * (k1 + 2 * k2 + 2 * k3 + k4)
        if s % save_every == 0:
            out.append(y.copy())
    return np.array(out)


# --------------------------------------------------------------------------
# ZOFE master equation (qspectra/dynamics/zofe.py)
# --------------------------------------------------------------------------
class ZOFESpec:
    """ZOFE model with one pseudomode bath per site (zofe.py:44-229).

    The state is rho (n x n) followed by the auxiliary operators
    O (npm, n_sites, n, n), both flattened column-major (zofe.py:101-119).
    ``Omega``, ``gamma``, ``huang`` are (npm, n_sites).
    """

    def __init__(self, ham, Omega, gamma, huang, hilbert_subspace='ge', unit_convert=1.0,
                 rho_hermit=False, ham_hermit=False):
        self.ham = ham
        self.rho_hermit = rho_hermit
        self.ham_hermit = ham_hermit
        self.Omega = np.asarray(Omega, complex)
        self.gamma = np.asarray(gamma, complex)
        self.huang = np.asarray(huang, complex)
        self.hilbert_subspace = hilbert_subspace
        self.unit_convert = unit_convert
        self.npm = self.Omega.shape[0]
        self.n = len(site_states(ham.n_sites, hilbert_subspace))
        self.oop_shape = (self.npm, ham.n_sites, self.n, self.n)

    def sample(self, n, random_orientations=False):
        return ZOFESpec(self.ham.sample(n, random_orientations), self.Omega, self.gamma,
                        self.huang, self.hilbert_subspace, self.unit_convert,
                        self.rho_hermit, self.ham_hermit)

    @property
    def time_step(self):
        return self.ham.time_step(self.unit_convert)

    def split(self, y):
        n2 = self.n * self.n
        return (y[:n2].reshape((self.n, self.n), order='F'),
                y[n2:].reshape(self.oop_shape, order='F'))

    def join(self, rho, oop):
        return np.concatenate([rho.reshape(-1, order='F'), oop.reshape(-1, order='F')])

    def rhs(self, y):
        """zofe.py:121-202, times unit_convert; L_n = -(number operators)
        (zofe.py:219-222).  The rho^H forms follow zofe.py:179-192."""
        rho, oop = self.split(y)
        H = self.ham.H(self.hilbert_subspace)
        L = -np.array([np.diag(o) for o in occupations(self.ham.n_sites,
                                                        self.hilbert_subspace)])
        Gamma = self.Omega ** 2 * self.huang
        w = 1j * self.Omega + self.gamma
        S = oop.sum(axis=0)
        Lh = np.conj(np.transpose(L, (0, 2, 1)))
        a = np.einsum('sij,sjk->ik', Lh, S)
        b = -1j * H - a
        c = np.einsum('sij,jk,smk->im', L, rho, np.conj(S))
        if not self.rho_hermit:
            big = np.einsum('sij,jk,skm->im', S, rho, Lh)
            if self.ham_hermit:
                f = rho @ b.conj().T + big
            else:
                f = rho @ (1j * H - a.conj().T) + big
        elif self.ham_hermit:
            f = (b @ rho + c).conj().T
        else:
            f = rho @ (1j * H - a.conj().T) + c.conj().T
        rhodot = b @ rho + c + f
        oopdot = (Gamma[:, :, None, None] * L[None]
                  - w[:, :, None, None] * oop
                  + np.einsum('kj,psjl->pskl', b, oop)
                  - np.einsum('pskj,jl->pskl', oop, b))
        return self.unit_convert * self.join(rhodot, oopdot)

    def thermal_state(self, _=None):
        """Ground state (a pseudomode bath has no temperature,
        hamiltonian.py:164-175) with zero auxiliary operators."""
        H = extend_operator(self.ham.H1, self.hilbert_subspace)
        E, U = scipy.linalg.eigh(H)
        rho = np.outer(U[:, 0], U[:, 0].conj())
        return self.join(rho.astype(complex), np.zeros(self.oop_shape, complex))

    def dipole(self, polarization, transitions):
        return dipole_operator(self.ham.dipoles, self.hilbert_subspace, polarization,
                               transitions)

    def commutator(self, A, y):
        """[A, .] on rho and on every auxiliary operator (zofe.py:22-33)."""
        rho, oop = self.split(y)
        return self.join(A @ rho - rho @ A, A @ oop - oop @ A)

    def expectation(self, A, y):
        rho, _ = self.split(y)
        return np.trace(A @ rho)


def rk4_nonlinear(f, y0, t, t0=None, h=None):
    """Fixed-step RK4 for dy/dt = f(t, y), outputs at t (simulate/utils.py:16-109)."""
    t = np.asarray(t, float)
    y = np.array(y0, dtype=complex)
    t0 = t[0] if t0 is None else t0
    h = (t[1] - t[0]) if h is None else h
    out, cur = [], t0
    for ti in t:
        for _ in range(int(round((ti - cur) / h))):
            k1 = f(cur, y)
            k2 = f(cur + h / 2, y + h / 2 * k1)
            k3 = f(cur + h / 2, y + h / 2 * k2)
            k4 = f(cur + h, y + h * k3)
            y = y + h / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
            cur = cur + h
        out.append(y.copy())
    return np.array(out)


def zofe_dynamics(model, psi_or_rho, duration):
    """simulate_dynamics for a ZOFE model (eom.py:11-26): rho(t) (T, n, n)."""
    rho0 = np.asarray(psi_or_rho)
    if rho0.ndim == 1:
        rho0 = np.outer(rho0.conj(), rho0)
    y0 = model.join(rho0.astype(complex), np.zeros(model.oop_shape, complex))
    t = time_grid(duration, model.time_step)
    ys = rk4_nonlinear(lambda _, y: model.rhs(y), y0, t)
    return t, np.array([model.split(y)[0] for y in ys])


def zofe_linear_response(model, time_max, polarization='xx'):
    """_linear_response without a Heisenberg picture (response.py:15-43):
    -tr(V1 rho(t)) from rho(0) = [V0, rho_thermal] (the ZOFE maps ignore
    Liouville subspaces, zofe.py:98-99)."""
    t = time_grid(time_max, model.time_step)
    V0 = model.dipole(polarization[0], '+')
    V1 = model.dipole(polarization[1], '-')
    y0 = model.commutator(V0, model.thermal_state())
    ys = rk4_nonlinear(lambda _, y: model.rhs(y), y0, t)
    return t, -np.array([model.expectation(V1, y) for y in ys])


def zofe_with_fields(model, pulses, geometry='-+', polarization='xx', time_extra=0.0):
    """_simulate_with_fields for a ZOFE model (eom.py:77-105)."""
    V = [model.dipole(p, tr) for p, tr in zip(polarization, geometry)]
    rw = model.ham.rw_freq

    def f(t, y):
        d = model.rhs(y)
        for pulse, tr, A in zip(pulses, geometry, V):
            E = pulse(t, rw)
            if tr == '+':
                E = np.conj(E)
            d = d + (-1j * E) * model.commutator(A, y)
        return d
    t0 = min(p.t_init for p in pulses)
    tf = max(p.t_final for p in pulses)
    t = np.arange(t0, tf + time_extra, model.time_step)
    return t, rk4_nonlinear(f, model.thermal_state(), t, t0=t0, h=model.time_step)
