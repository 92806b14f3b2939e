"""Host-side logic of the ensemble drivers (no GPU): block-size choice for
the real blocked loop, Hermitian block detection and the coordinate map."""
import numpy as np

from qspectra_gb300.simulate import ensemble as ens


def tc_supported(m, K, nsel):
    """The shapes the tensor-core block build takes: m <= 64, K = 2^J or
    2^J + 1, and at most 64 selected rows entering its last row product."""
    if m > 64 or K < 2 or K > 64:
        return False
    if K & (K - 1) and ((K - 1) & (K - 2) or K <= 2):
        return False
    b = 1
    while 2 * b < K - 1:
        b *= 2
    return b * nsel <= 64


def test_block_size_covers_the_steps_and_prefers_cheap_builds():
    for nsteps in (999, 512, 300, 2047, 1023, 24, 997):
        K = ens.pick_block_k_real(nsteps, 49, 7)
        Kt = ens.pick_block_k_real(nsteps, 49, 7,
                                   tensor_core=lambda k: tc_supported(49, k, 7))
        for k in (K, Kt):
            assert 1 < k <= 64
            assert 49 + 7 * (k - 1) <= 512
            run = ens.padded_block_steps(nsteps, k)
            assert run % k == 0 and nsteps <= run < nsteps + k
    # a cheaper build only makes tensor-core shapes more attractive: when the
    # plain choice is one, so is the weighted choice (possibly a larger K)
    for nsteps in (512, 360, 720, 1000):
        K = ens.pick_block_k_real(nsteps, 49, 7)
        Kt = ens.pick_block_k_real(nsteps, 49, 7, tensor_core=lambda k: tc_supported(49, k, 7))
        if tc_supported(49, K, 7):
            assert tc_supported(49, Kt, 7) and Kt >= K


def test_padded_block_steps():
    assert ens.padded_block_steps(999, 9) == 999
    assert ens.padded_block_steps(999, 8) == 1000
    assert ens.padded_block_steps(997, 8) == 1000
    assert ens.padded_block_steps(8, 8) == 8


def test_hermitian_block_detection():
    n = 8   # ground + 7 sites
    ee = np.array([a + n * b for b in range(1, n) for a in range(1, n)])
    assert ens.hermitian_block_size(ee, n) == 7
    eg = np.array([a + n * 0 for a in range(1, n)])
    assert ens.hermitian_block_size(eg, n) is None


def test_hermitian_coordinates_round_trip():
    rng = np.random.RandomState(0)
    nb = 5
    A = rng.randn(nb, nb) + 1j * rng.randn(nb, nb)
    rho = A + A.conj().T
    y = rho.reshape(-1, order='F')
    x = ens.hermitian_coordinates(y, nb)
    assert x.dtype.kind == 'f' and x.shape == (nb * nb,)
    # populations are coordinates
    for a in range(nb):
        assert x[a + nb * a] == rho[a, a].real
    back = ens.from_hermitian_coordinates(x, nb)
    assert np.allclose(back, y, atol=1e-14)


def test_measured_block_k_candidates():
    """The candidates the real-path tuner times, ranked by the cost model, the
    model's own choice first; block sizes that do not divide the step count
    run whole blocks past it."""
    tc = lambda k: k in (3, 5, 8, 9, 17, 33)   # tensor-core shapes
    c = ens.block_k_real_candidates(999, 49, 7, tc)
    assert c[0] == ens.pick_block_k_real(999, 49, 7, tensor_core=tc)
    assert len(c) == ens.K_REAL_CANDIDATES and len(set(c)) == len(c)
    assert 8 in c and 9 in c     # 1000 = 125 x 8 steps against 999 = 111 x 9
    small = ens.block_k_real_candidates(7, 49, 7)
    assert len(small) == ens.K_REAL_CANDIDATES and all(2 <= K <= 7 for K in small)
    ens.set_block_k_real(3)
    try:
        assert ens._PINNED_K_REAL == 3
    finally:
        ens.set_block_k_real(None)
