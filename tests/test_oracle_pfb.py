"""CPU checks of the inverse-PFB oracle: the banded solver against
scipy.linalg.solveh_banded, the forward PFB against its polyphase form, and
the correlation-loss figures the reference reports for PFB-mode data
(docs/resampling/summary.tex:449-464: 34% loss for a plain iFFT of 4-tap PFB
spectra, 0.5% with Shaw's inversion)."""
import numpy as np
import pytest

from oracle import sdbe_oracle as O


def test_banded_solver_matches_scipy():
    la = pytest.importorskip("scipy.linalg")
    rng = np.random.default_rng(3)
    L, ntap, nb = 64, 4, 37
    w, a = O.pfb_band(L, ntap)
    y = rng.standard_normal((nb, L))
    z = O.banded_ldl_solve(a, y)
    for p in range(0, L, 7):
        ab = np.zeros((ntap, nb))
        for d in range(ntap):
            ab[ntap - 1 - d, d:] = a[d, p]
        ref = la.solveh_banded(ab, y[:, p])
        assert np.allclose(z[:, p], ref, rtol=1e-9, atol=1e-9 * np.abs(ref).max())


def test_forward_pfb_is_the_polyphase_dft():
    """rFFT of ntap*L windowed samples, every ntap-th bin == L-point DFT of
    the ntap-term polyphase sum."""
    rng = np.random.default_rng(4)
    L, ntap = 128, 4
    x = rng.standard_normal(L * 9)
    S = O.forward_pfb(x, L, ntap)
    w, _ = O.pfb_band(L, ntap)
    xb = x.reshape(-1, L)
    for i in range(S.shape[0]):
        y = sum(w[t] * xb[i + t] for t in range(ntap))
        assert np.allclose(S[i], np.fft.rfft(y), atol=1e-9)


def test_inverse_is_consistent_and_recovers_the_loss_figures():
    rng = np.random.default_rng(1)
    L, ntap, nb = 256, 4, 400
    x = rng.standard_normal((nb + ntap - 1) * L)
    S = O.forward_pfb(x, L, ntap)
    rec = O.inverse_pfb(S, ntap)
    xb = x.reshape(-1, L)
    # the recovered blocks reproduce the spectra exactly (least-squares solution)
    assert np.allclose(O.forward_pfb(rec.ravel(), L, ntap), S, atol=1e-8 * np.abs(S).max())
    rho = np.corrcoef(rec.ravel(), xb.ravel())[0, 1]
    rho_in = np.corrcoef(rec[8:-8].ravel(), xb[8:-8].ravel())[0, 1]
    assert rho > 0.995 and rho_in > 0.998            # summary.tex: ~0.5% loss
    y = np.fft.irfft(S, n=L, axis=1)                 # plain iFFT of the PFB spectra
    rho_plain = max(np.corrcoef(y.ravel(), xb[s:s + nb].ravel())[0, 1] for s in range(ntap))
    assert 0.62 < rho_plain < 0.70                   # summary.tex: 34% loss
