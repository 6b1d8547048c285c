"""The SVD's batched symmetric eigensolver (tridiagonalisation, bisection,
inverse iteration, Newton-Schulz, back-transformation) against numpy's eigh.

Bars: eigenvalues within 1e-14 of the matrix norm; eigenvectors orthonormal
to 1e-13 with residuals |A z - lambda z| within 1e-12 of the norm; isolated
eigenvectors equal to the reference's up to sign.
"""
import ctypes as C

import numpy as np
import pytest

from ultradmrg_gb300 import _lib, api

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from ultradmrg_gb300 import build
    build.build()
    c = api.Context(0)
    yield c
    c.close()


def sym_eig(ctx, mats, ks):
    ns = np.array([m.shape[0] for m in mats], np.int32)
    kk = np.array(ks, np.int32)
    flat = np.concatenate([np.ascontiguousarray(m, np.float64).ravel() for m in mats])
    lam = np.zeros(int(ns.sum()))
    vec = np.zeros(int(sum(int(n) * int(k) for n, k in zip(ns, kk))) or 1)
    _lib.call("udmrg_selftest_sym_eig", ctx.h, len(mats), ns.ctypes.data_as(_lib.c_int32_p),
              flat.ctypes.data_as(_lib.c_double_p), kk.ctypes.data_as(_lib.c_int32_p),
              lam.ctypes.data_as(_lib.c_double_p), vec.ctypes.data_as(_lib.c_double_p))
    out, lo, vo = [], 0, 0
    for n, k in zip(ns, kk):
        n, k = int(n), int(k)
        out.append((lam[lo:lo + n], vec[vo:vo + n * k].reshape(n, k)))
        lo += n
        vo += n * k
    return out


def _rand_orth(n, rng):
    q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    return q


def _cases():
    rng = np.random.default_rng(11)
    mats = []
    for n in (1, 2, 3, 10, 64, 159, 300):
        a = rng.normal(size=(n, n))
        mats.append(("random%d" % n, (a + a.T) / 2))
    # graded PSD Gram matrix (Schmidt-like spectrum over 16 decades)
    n = 200
    x = _rand_orth(n, rng) @ np.diag(10.0 ** (-np.linspace(0, 8, n))) @ _rand_orth(n, rng)
    mats.append(("graded_gram", x @ x.T))
    # exact degeneracies (multiplets) and a tight cluster
    lam = np.repeat([1.0, 0.5, 0.25, 0.1], [3, 2, 4, 91])
    q = _rand_orth(100, rng)
    mats.append(("degenerate", (q * lam) @ q.T))
    lam = 1.0 + 1e-12 * np.arange(50)
    q = _rand_orth(50, rng)
    mats.append(("cluster", (q * lam) @ q.T))
    # rank deficient and zero
    y = rng.normal(size=(120, 30))
    mats.append(("rank30", y @ y.T))
    mats.append(("zero", np.zeros((20, 20))))
    # the largest size the SVD may meet at D = 2000
    n = 640
    y = rng.normal(size=(n, n)) * np.exp(-np.arange(n) / 60.0)
    mats.append(("big_gram", y @ y.T))
    return mats


@pytest.mark.parametrize("kfrac", [1.0, 0.3])
def test_sym_eig_batch(ctx, kfrac):
    cases = _cases()
    mats = [m for _, m in cases]
    ks = [max(1, int(round(kfrac * m.shape[0]))) if m.shape[0] > 0 else 0 for m in mats]
    got = sym_eig(ctx, mats, ks)
    for (name, a), (lam, z), k in zip(cases, got, ks):
        n = a.shape[0]
        w_ref, v_ref = np.linalg.eigh(a)
        w_ref, v_ref = w_ref[::-1], v_ref[:, ::-1]
        nrm = max(np.abs(w_ref).max(), 1e-300)
        assert np.max(np.abs(lam - w_ref)) <= 1e-14 * nrm * max(1, np.sqrt(n) / 4), name
        assert z.shape == (n, k)
        orth = np.max(np.abs(z.T @ z - np.eye(k)))
        res = np.max(np.abs(a @ z - z * lam[:k])) / nrm
        print(f"{name}: n={n} k={k} orth {orth:.1e} residual {res:.1e}")
        assert orth <= 1e-13, name
        assert res <= 1e-12 * max(1, np.sqrt(n) / 4), name
        # isolated eigenvalues: the vector itself (up to sign)
        gaps = np.full(n, np.inf)
        if n > 1:
            d = np.abs(np.diff(w_ref))
            gaps[:-1] = np.minimum(gaps[:-1], d)
            gaps[1:] = np.minimum(gaps[1:], d)
        for i in range(k):
            if gaps[i] > 1e-3 * nrm:
                assert abs(abs(z[:, i] @ v_ref[:, i]) - 1) <= 1e-10, (name, i)


def _graded_block(rows, cols, decades, rng, dtype):
    k = min(rows, cols)
    s = 10.0 ** (-np.linspace(0, decades, k))

    def orth(n):
        a = rng.normal(size=(n, k))
        if dtype == np.complex128:
            a = a + 1j * rng.normal(size=(n, k))
        q, _ = np.linalg.qr(a)
        return q
    return (orth(rows) * s) @ orth(cols).conj().T


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
@pytest.mark.parametrize("dmax", [400, 150])
def test_svd_large_sectors(ctx, dtype, dmax):
    """Truncated SVD whose Gram sectors (n = 150 .. 300) exceed shared memory,
    so the reduction runs on several cooperating CTAs per sector; with
    Dmax = 150 only the leading eigenvalues are computed (the rest of the
    weight from the traces)."""
    from oracle import blocksparse as bs
    from ultradmrg_gb300.tensor_data import BlockTensorData, Index
    rng = np.random.default_rng(23)
    li = Index.make([((0,), 260), ((1,), 150), ((2,), 40)], -1)
    ri = Index.make([((0,), 300), ((1,), 180), ((2,), 60)], +1)
    blocks = {(0, 0): _graded_block(260, 300, 7, rng, dtype),
              (1, 1): 0.3 * _graded_block(150, 180, 9, rng, dtype),
              (2, 2): 0.1 * _graded_block(40, 60, 5, rng, dtype)}
    t = BlockTensorData([li, ri], blocks, dtype)
    bs.normalize(t)
    ldiv = (0,)
    u, s, vt, err, Dk = bs.svd(t, 1, ldiv, 1e-10, 1, dmax)
    gu, gs, gvt, gerr, gD = api.svd(ctx, api.DeviceTensor.from_data(ctx, t), 1, ldiv, 1e-10, 1,
                                    dmax)
    gu, gs, gvt = gu.to_data(), gs.to_data(), gvt.to_data()
    assert gD == Dk and abs(gerr - err) <= 1e-12
    w = np.concatenate([np.diag(b) for _, b in sorted(s.blocks.items())])
    gw = np.concatenate([np.diag(b) for _, b in sorted(gs.blocks.items())])
    assert np.allclose(gw ** 2, w ** 2, atol=1e-14)
    rec = bs.contract(bs.contract(u, s, [1], [0]), vt, [1], [0])
    grec = bs.contract(bs.contract(gu, gs, [1], [0]), gvt, [1], [0])
    for k, b in rec.blocks.items():
        assert np.max(np.abs(grec.blocks[k] - b)) <= 1e-11
    uu = bs.contract(bs.dag(gu), gu, [0], [0])
    for k, b in uu.blocks.items():
        assert np.allclose(b, np.eye(b.shape[0]), atol=1e-12)
