"""The FP32 velocity of the gauge step is Hermitian to the bit.

The warp-per-k optical Hall kernel reads row n of each velocity block as the
conjugate of column n, which is exact only if the gauge step's FP32 velocity
V_a(p, q) = Hbar_a(p, q) - i (E_q - E_p) (Abar_a(p, q) + i D_a(p, q)),
D_a(p, q) = Hbar_a(p, q) / (E_q - E_p), is exactly Hermitian.  It is: the
rotated blocks are stored Hermitian (mirrored, real diagonal), E_q - E_p is
formed from FP32 hi + lo energies and is exactly antisymmetric, the inverse
gaps are sign-symmetric, and every operation is an IEEE-rounded product or sum
that commutes with negation and conjugation.  This restates that arithmetic
(mepinterp_gb300/csrc/gauge.cu, FP32 form) in numpy float32 on random
Hermitian blocks and checks V^T == conj(V) bit for bit.
"""
import numpy as np

f32 = np.float32


def herm32(rng, N):
    X = (rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N))).astype(np.complex64)
    U = np.triu(X)
    H = U + np.conj(np.triu(X, 1)).T                    # mirrored from the upper triangle
    H[np.diag_indices(N)] = H.diagonal().real            # real diagonal
    return H.real.astype(f32), H.imag.astype(f32)


def test_fp32_velocity_is_hermitian_to_the_bit():
    rng = np.random.default_rng(11)
    N = 16
    E = np.sort(rng.uniform(-1.0, 1.0, N))
    E[5] = E[4] + 3e-6                                    # a pair below kuboTol
    kubo_tol = 1e-5
    Eh = E.astype(f32)
    El = (E - Eh.astype(np.float64)).astype(f32)
    ded = E[None, :] - E[:, None]                         # [n][m] = E_m - E_n (FP64 decision)
    mask = (np.abs(ded) > kubo_tol) & ~np.eye(N, dtype=bool)
    invd = np.where(mask, (f32(1.0) / np.where(mask, ded, 1.0).astype(f32)), f32(0.0)).astype(f32)
    de = ((Eh[None, :] - Eh[:, None]) + (El[None, :] - El[:, None])).astype(f32)   # [p][q] = E_q - E_p
    for _ in range(3):
        hr, hi = herm32(rng, N)
        ar, ai = herm32(rng, N)
        dr, di = hr * invd, hi * invd                     # D = Hbar * invd
        avr, avi = ar - di, ai + dr                       # A'' = Abar + i D
        vr = hr + de * avi                                # V = Hbar - i de A''
        vi = hi - de * avr
        assert np.array_equal(vr, vr.T)
        assert np.array_equal(vi, -vi.T)
