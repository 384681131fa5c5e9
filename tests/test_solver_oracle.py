"""CPU pins of the FP64 solver restatements (oracle/numerics.py) that the GPU
CGLS and split-Bregman tests use as their checker: solveCGLS.m:6-31 solves
the regularised normal equations, and solveSplitBregman.m:15-41 reaches the
least-squares solution without shrinkage and lowers the analysis-l1
objective with it."""
import numpy as np
import pytest

from oracle import numerics as N


def _problem(seed=0, m=40, n=20):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((m, n)), rng.standard_normal(m)


@pytest.mark.parametrize("lam", [0.0, 0.5])
def test_cgls_solves_the_regularised_normal_equations(lam):
    A, f = _problem()
    b = A.T @ f
    u, hist = N.cgls(lambda x: A.T @ (A @ x), b, np.zeros(A.shape[1]), lam, iters=40)
    want = np.linalg.solve(A.T @ A + lam * np.eye(A.shape[1]), b)
    assert np.linalg.norm(u - want) < 1e-8 * np.linalg.norm(want)
    assert hist[-1] < 1e-12 * hist[0]


def test_cgls_warm_start_and_early_stop():
    A, f = _problem(seed=1)
    b = A.T @ f
    normal = lambda x: A.T @ (A @ x)  # noqa: E731
    u5, _ = N.cgls(normal, b, np.zeros(A.shape[1]), 0.0, iters=5)
    u_warm, _ = N.cgls(normal, b, u5, 0.0, iters=40)
    want = np.linalg.lstsq(A, f, rcond=None)[0]
    assert np.linalg.norm(u_warm - want) < 1e-8 * np.linalg.norm(want)
    _, hist = N.cgls(normal, b, np.zeros(A.shape[1]), 0.0, iters=40, tol=1e-3)
    assert len(hist) < 40 and hist[-1] < 1e-3


def _frame(shape):
    W = lambda u: N.frame_dec(u.reshape(shape), 1, "linear")  # noqa: E731
    Wt = lambda c: N.frame_rec(c, "linear").reshape(-1)       # noqa: E731
    return W, Wt


def test_split_bregman_without_shrinkage_reaches_least_squares():
    A, f = _problem(seed=2)
    W, Wt = _frame((2, 2, 5))
    u = N.split_bregman(lambda x: A @ x, lambda y: A.T @ y, W, Wt, f, np.zeros(20), 0.0, 1.0,
                        outer=40, cg_iters=30)
    want = np.linalg.lstsq(A, f, rcond=None)[0]
    assert np.linalg.norm(u - want) < 1e-5 * np.linalg.norm(want)


def test_split_bregman_lowers_the_analysis_l1_objective():
    A, f = _problem(seed=3)
    W, Wt = _frame((2, 2, 5))
    lam = 5.0

    def objective(u):
        high = sum(np.abs(a).sum() for k, a in W(u)[0].items() if k != (0, 0, 0))
        return 0.5 * float(np.sum((A @ u - f) ** 2)) + lam * high

    u = N.split_bregman(lambda x: A @ x, lambda y: A.T @ y, W, Wt, f, np.zeros(20), lam, 1.0,
                        outer=60, cg_iters=30)
    ls = np.linalg.lstsq(A, f, rcond=None)[0]
    assert objective(u) < 0.5 * objective(ls)
