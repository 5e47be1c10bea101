"""The per-band regrouping of the optical Hall sums that the warp-per-k kernel
(mepinterp_gb300/csrc/bandsum.cu, opt_hall_warp_kernel) evaluates, restated in
numpy and checked against the oracle's velo_ahc_tens / kubo_ohc_tens
(src/kubo.f90:86-198) on random Hermitian velocities.

The kernel relies on V being Hermitian: lane n reads row n of V^i as the
conjugate of column n, and with c^ij = V^i_nm V^j_mn = v_i conj(v_j) the (m, n)
products are conj(c^ij) and c^ji = conj(c^ij), so per band it keeps 24 sums
(vah: 2 Im(c^ij) W for i < j; koh: A = Re c (g2r - g1r), B = Im c (g2i + g1i),
C = Re c (g2i - g1i), D = Im c (g2r + g1r) for i < j, and A, C for i = j) and
expands them to the 3 x 3 tensors: vah^ji = -vah^ij, vah^ii = 0,
koh^ij = (A + B) + i (C - D), koh^ji = (A - B) + i (C + D).
"""
import numpy as np

from oracle import ref_numpy as O

PAIRS = ((0, 1), (0, 2), (1, 2))


def regrouped(E, V, f, hw, eta):
    """E (N,), V (3, N, N) Hermitian, f (nE, N) -> vah, koh (3, 3, nE) complex."""
    N = E.size
    Yv = np.zeros((N, 3, 3), complex)
    Yk = np.zeros((N, 3, 3), complex)
    for n in range(N):
        acc = np.zeros(24)
        for m in range(N):
            if m == n:
                continue
            v = np.conj(V[:, m, n])                       # V^i(n, m), from column n
            d = E[n] - E[m]
            dm, dp = d - hw, d + hw
            ar, ai = dm * dp + eta * eta, 2.0 * hw * eta
            an = 1.0 / (ar * ar + ai * ai)
            wvr, wvi = ar * an, ai * an
            b1r, b1i, b2r, b2i = d * dp, d * eta, d * dm, -d * eta
            n1, n2 = 1.0 / (b1r * b1r + b1i * b1i), 1.0 / (b2r * b2r + b2i * b2i)
            g1r, g1i, g2r, g2i = b1i * n1, b1r * n1, b2i * n2, b2r * n2
            gar, gbi, gci, gdr = g2r - g1r, g2i + g1i, g2i - g1i, g2r + g1r
            for pq, (i, j) in enumerate(PAIRS):
                c = v[i] * np.conj(v[j])
                dv = 2.0 * c.imag
                acc[6 * pq:6 * pq + 6] += [dv * wvr, dv * wvi, c.real * gar, c.imag * gbi, c.real * gci,
                                           c.imag * gdr]
            for i in range(3):
                c = abs(v[i]) ** 2
                acc[18 + 2 * i] += c * gar
                acc[19 + 2 * i] += c * gci
        for pq, (i, j) in enumerate(PAIRS):
            vr, vi, ka, kb, kc, kd = acc[6 * pq:6 * pq + 6]
            Yv[n, i, j], Yv[n, j, i] = vr + 1j * vi, -(vr + 1j * vi)
            Yk[n, i, j], Yk[n, j, i] = (ka + kb) + 1j * (kc - kd), (ka - kb) + 1j * (kc + kd)
        for i in range(3):
            Yk[n, i, i] = acc[18 + 2 * i] + 1j * acc[19 + 2 * i]
    return np.einsum("en,nij->ije", f, Yv), np.einsum("en,nij->ije", f, Yk)


def test_regrouped_optical_hall_matches_oracle():
    rng = np.random.default_rng(5)
    N = 9
    E = np.sort(rng.uniform(-0.3, 0.3, N))
    X = rng.normal(size=(3, N, N)) + 1j * rng.normal(size=(3, N, N))
    V = 0.5 * (X + np.conj(np.swapaxes(X, 1, 2)))            # Hermitian velocity blocks
    ef = np.array([-0.05, 0.01, 0.12])
    for T_kelvin in (0.0, 290.1):
        f = O.fd_stat(E[None], ef, T_kelvin)[0]               # (nE, N)
        for hw, eta in ((0.0, 3.7e-5), (0.02, 0.002)):
            vah, koh = regrouped(E, V, f, hw, eta)
            ref_v = O.velo_ahc(E[None], V[None], f[None], np.array([hw]), eta)[0][:, :, 0, :]
            ref_k = O.kubo_ohc(E[None], V[None], f[None], np.array([hw]), eta)[0][:, :, 0, :]
            assert np.abs(vah - ref_v).max() <= 1e-12 * np.abs(ref_v).max()
            assert np.abs(koh - ref_k).max() <= 1e-12 * np.abs(ref_k).max()
