"""The FP64 learned-DBP adjoint (oracle/ldbp_ref.py) against central finite
differences.  CPU only."""
import numpy as np

from oracle import ldbp_ref as R


def test_adjoint_matches_finite_differences():
    rng = np.random.default_rng(0)
    spans, steps, T, Tm, N, B = 2, 2, 5, 7, 64, 2
    L = spans * steps
    h = (rng.standard_normal((L, T)) + 1j * rng.standard_normal((L, T))) * 0.4
    xi = rng.standard_normal(L) * 0.5
    hmf = (rng.standard_normal(Tm) + 1j * rng.standard_normal(Tm)) * 0.4
    x = rng.standard_normal((B, N)) + 1j * rng.standard_normal((B, N))
    tx = rng.standard_normal((B, N // 2)) + 1j * rng.standard_normal((B, N // 2))
    sc = 0.9
    loss, gh, gxi, ghmf = R.loss_grad(h, xi, hmf, x, tx, sc, spans, steps)
    eps = 1e-6

    def f(h_, xi_, hmf_):
        y = R.forward(h_, xi_, hmf_, x, sc, spans, steps)
        return np.mean(np.abs(y[..., 0::2] - tx) ** 2)

    for (k, t) in ((0, 0), (3, 4), (2, 2)):
        for unit, part in ((1.0, np.real), (1j, np.imag)):
            hp, hm = h.copy(), h.copy()
            hp[k, t] += unit * eps
            hm[k, t] -= unit * eps
            fd = (f(hp, xi, hmf) - f(hm, xi, hmf)) / (2 * eps)
            assert abs(fd - 2 * part(gh[k, t])) < 1e-6 * max(1, abs(fd))
    for k in range(L):
        xp, xm = xi.copy(), xi.copy()
        xp[k] += eps
        xm[k] -= eps
        fd = (f(h, xp, hmf) - f(h, xm, hmf)) / (2 * eps)
        assert abs(fd - gxi[k]) < 1e-6 * max(1, abs(fd))
    for t in (0, 3, 6):
        for unit, part in ((1.0, np.real), (1j, np.imag)):
            mp, mm = hmf.copy(), hmf.copy()
            mp[t] += unit * eps
            mm[t] -= unit * eps
            fd = (f(h, xi, mp) - f(h, xi, mm)) / (2 * eps)
            assert abs(fd - 2 * part(ghmf[t])) < 1e-6 * max(1, abs(fd))
