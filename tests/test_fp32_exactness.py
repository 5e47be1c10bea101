"""Exactness claims of the FP32 kernels, restated in numpy float32 arithmetic.

* The band sums read 1 / (E_n0 - E_m) as -(1 / (E_m - E_n0))
  (mepinterp_gb300/csrc/bandsum.cu): the energy differences are formed from FP32
  hi + lo pairs by a TwoSum difference (df_diff) that is exactly antisymmetric,
  and an IEEE reciprocal is sign-symmetric.
* The tensor-core rotation (mepinterp_gb300/csrc/rot_tc.cu) cuts each scaled
  operand row into balanced base-512 digits that FP16 holds exactly, and sums
  each level of digit products exactly in FP32 (every partial sum an integer
  below 2^24).  At K = 64 on random operands the product is within 2^-31 of the
  product of the row and column scales with four digits (levels 2..5) and
  within 2^-22 with three (levels 2..4); measured 2^-31.9 and 2^-23.0 here.
"""
import numpy as np

f32 = np.float32


def df_diff(ah, al, bh, bl):
    """(ah + al) - (bh + bl) as an FP32 pair, the operation order of df_diff."""
    s = f32(ah - bh)
    bp = f32(s - ah)
    t = f32(f32(ah - f32(s - bp)) + f32(-bh - bp))
    lo = f32(t + f32(al - bl))
    h = f32(s + lo)
    return h, f32(lo - f32(h - s))


def test_energy_differences_and_inverses_are_antisymmetric():
    rng = np.random.default_rng(3)
    E = rng.uniform(-2.0, 2.0, 64)
    E[1] = E[0] + 1e-9
    Eh = E.astype(f32)
    El = (E - Eh.astype(np.float64)).astype(f32)
    for a in range(E.size):
        for b in range(E.size):
            if a == b:
                continue
            d_ab, _ = df_diff(Eh[a], El[a], Eh[b], El[b])
            d_ba, _ = df_diff(Eh[b], El[b], Eh[a], El[a])
            assert d_ab == -d_ba
            assert f32(1.0) / d_ab == -(f32(1.0) / d_ba)


def digits(x, nd):
    """Balanced base-512 digits of rows already scaled to |x| < 256 (float64
    holds every partial remainder exactly)."""
    out, r = [], np.asarray(x, np.float64)
    for _ in range(nd):
        d = np.rint(r)
        out.append(d)
        r = (r - d) * 512.0
    return out


def sliced_product(X, Y, nd):
    """X (M, K) @ Y (K, N) by exact-slice digit products with per-row scales
    of X and per-column scales of Y, levels L = p + q = 2..nd + 1."""
    ex = np.ceil(np.log2(np.abs(X).max(axis=1) + 1e-300)) + 1     # 2^ex > |row|
    ey = np.ceil(np.log2(np.abs(Y).max(axis=0) + 1e-300)) + 1
    dx = digits(X * 2.0 ** (8 - ex)[:, None], nd)
    dy = digits(Y * 2.0 ** (8 - ey)[None, :], nd)
    acc = np.zeros((X.shape[0], Y.shape[1]))
    for L in range(2, nd + 2):
        lvl = np.zeros_like(acc, dtype=np.float32)
        for p in range(1, nd + 1):
            q = L - p
            if 1 <= q <= nd:
                part = dx[p - 1] @ dy[q - 1]
                assert np.abs(part).max() < 2.0 ** 24                 # exact in the FP32 accumulator
                lvl = (lvl + part.astype(np.float32)).astype(np.float32)
        assert np.abs(lvl.astype(np.float64)).max() <= 2.0 ** 24
        acc += lvl.astype(np.float64) * 512.0 ** -(L - 2)
    return acc * 2.0 ** (ex - 8)[:, None] * 2.0 ** (ey - 8)[None, :], ex, ey


def test_exact_slice_products_meet_their_bounds():
    rng = np.random.default_rng(9)
    K = 64
    X = rng.normal(size=(128, K)) * np.exp(rng.uniform(-8, 8, (128, 1)))
    Y = rng.normal(size=(K, 64)) * np.exp(rng.uniform(-4, 4, (1, 64)))
    exact = X @ Y
    for nd, bound in ((4, 2.0 ** -31), (3, 2.0 ** -22)):
        got, ex, ey = sliced_product(X, Y, nd)
        scale = 2.0 ** ex[:, None] * 2.0 ** ey[None, :]
        assert (np.abs(got - exact) <= scale * bound).all()
