"""The mixed path's tensor-core front updates, each run alone on seeded random
complex fronts through elp_front_update_test and compared with the same
update computed in FP64 by NumPy.

The kernels compute C -= A B with tcgen05 kind::tf32 "3xTF32" products: every
FP32 operand x is split into TF32 parts hi + lo (x = hi + lo + d with
|d| <= 2^-22 |x|) and hi*hi' + hi*lo' + lo*hi' is accumulated in FP32. Per
real product the dropped lo*lo' and d terms are at most 3 * 2^-22 |a||b|; the
FP32 accumulation over depth K adds at most K * 2^-24 sum |a||b|; the
epilogue's FP32 subtraction from C (and, fused, its addition into the parent)
one rounding of each. A complex product has four real ones, so entry-wise

    |err| <= (4 * 3 * 2^-22 + 2 * K * 2^-24) (|A| |B|) + 2^-23 (|C| + |P|),

with |A| |B| the product of the entry-wise moduli. A factor that is wrong but
close (a split term dropped, a tile missing, a wrong offset) misses this by
orders of magnitude: one dropped hi*lo' term alone is ~2^-11 |a||b|.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GEMM_COL, GEMM_ROW, GEMM_SCHUR, PACKED_SCHUR, GEMM_SCHUR_32 = 0, 1, 2, 3, 4


def _fronts(rng, slots, m):
    """slots random complex64 m x m matrices (logical values; _col lays them out)."""
    return (rng.standard_normal((slots, m, m)) + 1j * rng.standard_normal((slots, m, m))).astype(np.complex64)


def _col(a):
    """slots x m x m complex64 as the column-major interleaved floats the C side takes."""
    return np.ascontiguousarray(a.transpose(0, 2, 1)).view(np.float32).reshape(-1)


def _uncol(buf, slots, m):
    return buf.view(np.complex64).reshape(slots, m, m).transpose(0, 2, 1)


def _bound(A, B, C, K, P=None):
    absab = np.abs(A.astype(np.complex128)) @ np.abs(B.astype(np.complex128))
    extra = np.abs(C.astype(np.complex128)) + (0 if P is None else np.abs(P.astype(np.complex128)))
    return (12 * 2.0 ** -22 + 2 * K * 2.0 ** -24) * absab + 2.0 ** -23 * extra


def _run(elp, kernel, p, b, step, F, parents=None, pmap=None):
    lib = elp.load_library()
    slots, m = F.shape[0], F.shape[1]
    fb = _col(F).copy()
    pb = None if parents is None else _col(parents).copy()
    mp = None if pmap is None else np.ascontiguousarray(pmap, dtype=np.int32)
    rc = lib.elp_front_update_test(kernel, p, b, step, slots, fb.ctypes.data_as(C.c_void_p),
                                   0 if parents is None else parents.shape[1],
                                   None if mp is None else mp.ctypes.data_as(C.c_void_p),
                                   None if pb is None else pb.ctypes.data_as(C.c_void_p))
    assert rc == 0, lib.elp_last_error()
    return _uncol(fb, slots, m), None if pb is None else _uncol(pb, slots, parents.shape[1])


@pytest.mark.parametrize("p,b,step", [(200, 300, 3), (97, 170, 1), (64, 0, 1)])
def test_crout_column_update(elp, p, b, step):
    rng = np.random.default_rng(100 + p)
    m, k0 = p + b, 32 * step
    F = _fronts(rng, 2, m)
    G, _ = _run(elp, GEMM_COL, p, b, step, F)
    w = min(32, p - k0)
    for s in range(2):
        A, B, Cb = F[s][k0:, :k0], F[s][:k0, k0:k0 + w], F[s][k0:, k0:k0 + w]
        want = Cb.astype(np.complex128) - A.astype(np.complex128) @ B.astype(np.complex128)
        got = G[s][k0:, k0:k0 + w]
        assert np.all(np.abs(got - want) <= _bound(A, B, Cb, k0)), np.max(np.abs(got - want))
        # nothing outside the block changes
        mask = np.ones((m, m), bool)
        mask[k0:, k0:k0 + w] = False
        assert np.array_equal(G[s][mask], F[s][mask])


@pytest.mark.parametrize("p,b,step", [(200, 300, 3), (97, 170, 2)])
def test_crout_row_update(elp, p, b, step):
    rng = np.random.default_rng(200 + p)
    m, k0 = p + b, 32 * step
    w = min(32, p - k0)
    F = _fronts(rng, 2, m)
    G, _ = _run(elp, GEMM_ROW, p, b, step, F)
    for s in range(2):
        A, B, Cb = F[s][k0:k0 + w, :k0], F[s][:k0, k0 + w:], F[s][k0:k0 + w, k0 + w:]
        want = Cb.astype(np.complex128) - A.astype(np.complex128) @ B.astype(np.complex128)
        got = G[s][k0:k0 + w, k0 + w:]
        assert np.all(np.abs(got - want) <= _bound(A, B, Cb, k0)), np.max(np.abs(got - want))
        mask = np.ones((m, m), bool)
        mask[k0:k0 + w, k0 + w:] = False
        assert np.array_equal(G[s][mask], F[s][mask])


@pytest.mark.parametrize("kernel", [GEMM_SCHUR, GEMM_SCHUR_32])
@pytest.mark.parametrize("p,b", [(200, 300), (45, 77)])
def test_schur_update_in_place(elp, kernel, p, b):
    rng = np.random.default_rng(300 + p)
    m = p + b
    F = _fronts(rng, 2, m)
    G, _ = _run(elp, kernel, p, b, 0, F)
    for s in range(2):
        A, B, Cb = F[s][p:, :p], F[s][:p, p:], F[s][p:, p:]
        want = Cb.astype(np.complex128) - A.astype(np.complex128) @ B.astype(np.complex128)
        assert np.all(np.abs(G[s][p:, p:] - want) <= _bound(A, B, Cb, p))
        assert np.array_equal(G[s][:p, :], F[s][:p, :]) and np.array_equal(G[s][:, :p], F[s][:, :p])


@pytest.mark.parametrize("kernel", [GEMM_SCHUR, PACKED_SCHUR, GEMM_SCHUR_32])
@pytest.mark.parametrize("p,b", [(200, 300), (300, 129), (40, 20)])
def test_schur_update_into_parent(elp, kernel, p, b):
    """The extend-add fused into the update: parent[pmap[i], pmap[j]] +=
    C[i, j] - (L21 U12)[i, j]; the child front stays as it was and parent
    entries outside the map are untouched."""
    rng = np.random.default_rng(400 + p + 7 * kernel)
    m, mp = p + b, b + 57
    F = _fronts(rng, 2, m)
    P = _fronts(rng, 2, mp)
    pmap = rng.permutation(mp)[:b].astype(np.int32)
    G, Q = _run(elp, kernel, p, b, 0, F, parents=P, pmap=pmap)
    for s in range(2):
        assert np.array_equal(G[s], F[s])
        A, B, Cb = F[s][p:, :p], F[s][:p, p:], F[s][p:, p:]
        S = Cb.astype(np.complex128) - A.astype(np.complex128) @ B.astype(np.complex128)
        want = P[s].astype(np.complex128)
        want[np.ix_(pmap, pmap)] += S
        bound = np.zeros((mp, mp))
        bound[np.ix_(pmap, pmap)] = _bound(A, B, Cb, p, P[s][np.ix_(pmap, pmap)])
        assert np.all(np.abs(Q[s] - want) <= bound), np.max(np.abs(Q[s] - want) - bound)
        untouched = np.ones((mp, mp), bool)
        untouched[np.ix_(pmap, pmap)] = False
        assert np.array_equal(Q[s][untouched], P[s][untouched])


def test_front_update_rejects_bad_arguments(elp):
    lib = elp.load_library()
    F = np.zeros(2 * 10 * 10, np.float32)
    pm = np.array([0, 0], np.int32)
    P = np.zeros(2 * 5 * 5, np.float32)
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    assert lib.elp_front_update_test(GEMM_COL, 8, 2, 1, 1, ptr(F), 0, None, None) == 1    # step beyond p
    assert lib.elp_front_update_test(PACKED_SCHUR, 8, 2, 0, 1, ptr(F), 0, None, None) == 1  # needs a parent
    assert lib.elp_front_update_test(GEMM_SCHUR, 8, 2, 0, 1, ptr(F), 5, ptr(pm), ptr(P)) == 1  # pmap not injective
