"""The pair-symmetric tensor-core operator's decomposition, replayed in FP64 numpy against the
oracle's W x (smuthi/linearsystem/linear_system.py:958-973).

The kernel (``csrc/sg_tcsym.cu``) visits receiver pairs I = (2I, 2I + 1) and runs of emitters
j >= 2I (work items); per emitter it builds A = [Re W_i1j; Im W_i1j; Re W_i2j; Im W_i2j] (rows padded
to 32 per part), accumulates D1 += A [Re x_j | Im x_j] for y_i1, y_i2, and for j >= 2I + 2 forms
D2 = A [S x_i1 | S x_i2] (S = diag((-1)^m)), whose diagonal blocks sum to S (W_ji1 x_i1 + W_ji2 x_i2)
and are added to y_j. This test performs the same products, block sums, sign flips and real /
imaginary combinations on a seeded synthetic table (the identity W_ji = S W_ij S holds for any
table: phi_ji = phi_ij + pi) and compares with the oracle.
"""
import numpy as np
import pytest

import oracle.physics as ophys
import oracle.solve as osv

BP = 32


def _system(n, seed):
    rng = np.random.default_rng(seed)
    parts = [ophys.Sphere([float(x), float(y), 100.0], 1.5, 80.0, 3, 3)
             for x, y in rng.uniform(0, 3000, (n, 2))]
    grid = np.linspace(0.0, 4300.0, 60)
    bs = 30
    table = rng.standard_normal((len(grid), bs, bs)) + 1j * rng.standard_normal((len(grid), bs, bs))
    return parts, osv.RadialLookupCPU(parts, table, grid, "linear")


def _block(W, i, j):
    """W_ij[n1][n2] = L(rho_ij) e^{i (m2 - m1) phi_ij}, from the oracle's own interpolants."""
    bs = W.bs
    out = np.zeros((bs, bs), complex)
    for a in range(bs):
        for b in range(bs):
            out[a, b] = W._eval(a, b, W.rho[i, j]) * np.exp(1j * (W.m_of[b] - W.m_of[a]) * W.phi[i, j])
    return out


def _panel(v, R):
    """[Re v | Im v] with K = n2 rows padded to 32: shape (32, 2R)."""
    p = np.zeros((BP, 2 * R))
    p[:v.shape[0], :R] = v.real
    p[:v.shape[0], R:] = v.imag
    return p


def _combine(D, R, bs):
    """Re y = Wr xr - Wi xi, Im y = Wr xi + Wi xr from a 64-row block [Wr rows 0-31; Wi rows 32-63]."""
    return (D[:bs, :R] - D[BP:BP + bs, R:]) + 1j * (D[:bs, R:] + D[BP:BP + bs, :R])


@pytest.mark.parametrize("n,chunk", [(7, 3), (8, 256), (2, 1)])
def test_pair_symmetric_decomposition_matches_oracle(n, chunk):
    parts, W = _system(n, seed=n)
    bs, R = W.bs, 4
    rng = np.random.default_rng(1)
    X = rng.standard_normal((n * bs, R)) + 1j * rng.standard_normal((n * bs, R))
    ref = np.stack([W.matvec(X[:, r]) for r in range(R)], axis=1)
    blocks = {(i, j): _block(W, i, j) for i in range(n) for j in range(n)}
    s = np.where(W.m_of % 2 == 1, -1.0, 1.0)
    xs = X.reshape(n, bs, R)
    y = np.zeros((n, bs, R), complex)
    items = [(I, jb, min(n, jb + chunk)) for I in range((n + 1) // 2) for jb in range(2 * I, n, chunk)]
    for I, jb, je in items:
        i0 = 2 * I
        recv = [i for i in (i0, i0 + 1) if i < n]
        D1 = np.zeros((128, 2 * R))
        sx = np.zeros((BP, 4 * R))  # [S x_i1 | S x_i2]
        for r, i in enumerate(recv):
            sx[:, 2 * R * r:2 * R * (r + 1)] = _panel(s[:, None] * xs[i], R)
        for j in range(jb, je):
            A = np.zeros((128, BP))
            for r, i in enumerate(recv):
                A[64 * r:64 * r + bs, :bs] = blocks[i, j].real
                A[64 * r + BP:64 * r + BP + bs, :bs] = blocks[i, j].imag
            D1 += A @ _panel(xs[j], R)
            if j >= i0 + 2:
                D2 = A @ sx
                E = D2[0:64, 0:2 * R] + D2[64:128, 2 * R:4 * R]
                y[j] += s[:, None] * _combine(E, R, bs)
        for r, i in enumerate(recv):
            y[i] += _combine(D1[64 * r:64 * (r + 1)], R, bs)
    err = np.linalg.norm(y.reshape(ref.shape) - ref) / np.linalg.norm(ref)
    assert err < 1e-12, err
