"""Host side of the NewmarkBeta integrator (no GPU): band widths and the row
band storage the device solve reads, and the beam matrices of the coupling
example against their defining stencil."""
import numpy as np
import pytest


def _mods():
    from sph.Integrators import NewmarkBeta as NB
    from sph import scenarios as S
    return NB, S


def test_bandwidths_and_band_storage_round_trip():
    NB, _ = _mods()
    rng = np.random.default_rng(3)
    for n, kl, ku in [(7, 0, 0), (9, 2, 1), (12, 1, 3), (6, 5, 5)]:
        A = rng.normal(size=(n, n))
        mask = np.fromfunction(lambda i, j: ((i - j) <= kl) & ((j - i) <= ku), (n, n))
        A = np.where(mask, A, 0.0)
        A[n - 1, max(0, n - 1 - kl)] = 1.0  # the widest band is occupied
        A[0, min(n - 1, ku)] = 1.0
        assert NB._bandwidths(A, np.zeros_like(A)) == (kl, ku)
        B = NB._to_band(A, kl, ku)
        back = np.zeros_like(A)
        for i in range(n):
            for d in range(-kl, ku + 1):
                j = i + d
                if 0 <= j < n:
                    back[i, j] = B[i, d + kl]
        np.testing.assert_array_equal(back, A)


def test_beam_matrices_follow_the_example_stencil():
    _, S = _mods()
    n, E, I, A, rho, L = 8, 2e6, 1e-6, 0.02, 917.0, 0.025
    K, M = S.beam_matrices(n, E, I, A, rho, L)
    D = K / (E * I / L ** 4)
    # interior rows: the central fourth difference 1 -4 6 -4 1
    np.testing.assert_array_equal(D[3, 1:6], [1, -4, 6, -4, 1])
    # clamped first node, free last two (examples/IceBreak.py:80-108)
    assert D[0, 0] == 7 and D[n - 1, n - 1] == 2 and D[n - 1, n - 3] == 2
    assert D[n - 2, n - 1] == -2 and D[n - 2, n - 2] == 5
    np.testing.assert_array_equal(M, np.eye(n) * rho * A)


def test_newmark_requires_two_beta_at_least_gamma():
    NB, _ = _mods()
    with pytest.raises(AssertionError):
        NB.NewmarkBeta(0.1, 0.5, np.eye(2), np.eye(2), np.eye(2))
    it = NB.NewmarkBeta(0.25, 0.5, np.eye(2), np.eye(2), np.eye(2))
    assert not it.isMultiStage()
