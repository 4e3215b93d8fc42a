"""CPU check of the arithmetic behind the tensor-core element kernel
(waterscapes_gb300/csrc/elem_tc.cu), restated in numpy.

The displacement Gram blocks Mg_ij[k][l] = int d_k phi_i d_l phi_j of a
tetrahedron are |T| sum_pq C_ij^pq b_p[k] b_q[l] over the barycentric
gradients b_1..b_3, with 20 C a small-integer table.  The kernel forms the
element blocks mu Mg^T + lambda Mg + mu tr(Mg) I as one GEMM of combined
features with that table: it scales a cell's features by one power of two,
rounds them to integers below 2^54, cuts them into five 11-bit slices,
multiplies each slice by the integer table with FP32 accumulation on the
tensor cores and combines the five products in 64-bit integers.
Here: the table is integral with row sums of magnitude <= 224 (so every
partial sum of a slice product is an integer below 2^19, exact in FP32), and
the sliced evaluation agrees with the oracle's FP64 Gram matrices
(oracle/fem.py) to round-off on random and badly shaped tetrahedra.
"""
import numpy as np

from oracle import fem


def _table():
    g_unit = np.zeros((10, 4, 4))       # grad phi_i at vertex r = sum_p G[i, r, p] b_p
    for i in range(4):
        for r in range(4):
            g_unit[i, r, i] = 3.0 if r == i else -1.0
    for e, (a, b) in enumerate(fem.TET_EDGES):
        g_unit[4 + e, a, b] += 4.0
        g_unit[4 + e, b, a] += 4.0
    W = np.ones((4, 4)) + np.eye(4)      # 20 * int lambda_r lambda_s / |T|
    rows = []
    pairs = []
    for i in range(10):
        for j in range(i, 10):
            Ct = np.einsum("rs,rp,sq->pq", W, g_unit[i], g_unit[j])
            C = Ct[1:, 1:] - Ct[0:1, 1:] - Ct[1:, 0:1] + Ct[0, 0]   # b_0 = -(b_1 + b_2 + b_3)
            rows.append(C.ravel())
            pairs.append((i, j))
    return np.array(rows), pairs


def _sliced_blocks(b, vol, T, mu, lmbda):
    """B_ij[k][l] = mu Mg_ij[l][k] + lmbda Mg_ij[k][l] + [k == l] mu tr Mg_ij for every
    (cell, k, l, pair) by the kernel's evaluation: combined features
    y_pq = (mu x_qp + lmbda x_pq + [k == l] mu tr_pq) / 20, one power-of-two scale
    per cell from the bound (4 |mu| + |lmbda|)/20 |T| max|b|^2, rounding to
    integers below 2^54, five 11-bit slices, exact integer products with the table
    (below 2^19), the slices combined in int64 and converted once."""
    nc = b.shape[0]
    bb = b[:, 1:, :]                                                  # (nc, p, k)
    x = np.einsum("c,cpk,cql->cklpq", vol, bb, bb)                    # x_pq^{kl}
    tr = np.einsum("c,cpm,cqm->cpq", vol, bb, bb)
    y = mu * np.transpose(x, (0, 1, 2, 4, 3)) + lmbda * x
    for k in range(3):
        y[:, k, k] += mu * tr
    y = (y / 20.0).reshape(nc, 3, 3, 9)
    bound = (4 * abs(mu) + abs(lmbda)) / 20.0 * vol * np.abs(bb).reshape(nc, -1).max(axis=1) ** 2
    _, e = np.frexp(bound)
    e = e + 1                                                         # |y| 2^-e < 1/2
    Y = np.rint(np.ldexp(y, (55 - e)[:, None, None, None])).astype(np.int64)
    assert np.abs(Y).max() < 2 ** 54
    a = np.abs(Y)
    sg = np.sign(Y)
    Ti = T.astype(np.int64)
    X = np.zeros(y.shape[:-1] + (T.shape[0],), dtype=np.int64)
    for s in range(5):
        Q = sg * ((a >> (44 - 11 * s)) & 2047)
        D = np.einsum("cklf,nf->ckln", Q, Ti)                         # exact integers
        assert np.abs(D).max() < 2 ** 19
        X += D << (44 - 11 * s)
    return np.ldexp(X.astype(np.float64), (e - 55)[:, None, None, None])   # (nc, k, l, pair)


def test_table_is_small_integer():
    T, pairs = _table()
    assert T.shape == (55, 9)
    assert np.array_equal(T, np.round(T))
    assert np.abs(T).sum(axis=1).max() <= 224


def test_sliced_blocks_match_fp64():
    rng = np.random.default_rng(0)
    T, pairs = _table()
    nc = 400
    x = rng.standard_normal((nc, 4, 3))
    x[:100] *= 1e-3                                              # small cells
    x[100:200, 3] = x[100:200, 0] + 1e-4 * rng.standard_normal((100, 3))  # slivers
    b, vol = fem.simplex_geometry(x.reshape(-1, 3), np.arange(4 * nc).reshape(nc, 4))
    g = fem.p2_gradient_vertex_values(b)
    Mg = fem.local_gradient_products(g, vol)                        # (nc, 10, 10, 3, 3)
    mu, lmbda = 1.0e3, 1.0e4
    S = _sliced_blocks(b, vol, T, mu, lmbda)
    scale = (mu + lmbda) * np.abs(Mg).reshape(nc, -1).max(axis=1)[:, None, None]
    for n, (i, j) in enumerate(pairs):
        M = Mg[:, i, j]                                             # (nc, k, l)
        ref = mu * np.transpose(M, (0, 2, 1)) + lmbda * M
        ref += mu * np.trace(M, axis1=1, axis2=2)[:, None, None] * np.eye(3)
        assert np.all(np.abs(S[:, :, :, n] - ref) <= 1e-14 * scale)
