"""The oracle's host numerics for Chebyshev and PPCG (tqli, the Lanczos
eigenvalue estimate, the Chebyshev coefficients; tea_leaf_cheby.f90:46-174)
checked against an independent computation: the Ritz values of the CG
Lanczos tridiagonal from scipy's tridiagonal eigensolver, and the closed-form
limit of the Chebyshev recurrence.  The reference's own benchmarks pin only
CG, so this pins the oracle's Chebyshev/PPCG set-up on the CPU."""
import ctypes as C

import numpy as np
import pytest

from tests.oracle_lib import lib

_D = C.POINTER(C.c_double)


def _cg_coefficients(a, b, iters):
    """plain CG on the SPD matrix a: the alphas and betas of each iteration"""
    x = np.zeros_like(b)
    r = b - a @ x
    p = r.copy()
    rr = r @ r
    alphas, betas = [], []
    for _ in range(iters):
        w = a @ p
        alpha = rr / (p @ w)
        x += alpha * p
        r -= alpha * w
        rrn = r @ r
        beta = rrn / rr
        alphas.append(alpha)
        betas.append(beta)
        p = r + beta * p
        rr = rrn
    return np.array(alphas), np.array(betas)


def _oracle_eigenvalues(alphas, betas):
    l = lib()
    l.ora_calc_eigenvalues.argtypes = [_D, _D, C.c_int, _D, _D]
    l.ora_calc_eigenvalues.restype = C.c_int
    al = np.ascontiguousarray(alphas, dtype=np.float64)
    be = np.ascontiguousarray(betas, dtype=np.float64)
    emin, emax = C.c_double(), C.c_double()
    info = l.ora_calc_eigenvalues(al.ctypes.data_as(_D), be.ctypes.data_as(_D), len(al), C.byref(emin),
                                  C.byref(emax))
    return info, emin.value, emax.value


@pytest.mark.parametrize("n,iters", [(120, 20), (400, 60)])
def test_oracle_eigenvalues_are_the_lanczos_ritz_values(n, iters):
    scipy_linalg = pytest.importorskip("scipy.linalg")
    rng = np.random.default_rng(n)
    # a 1-D diffusion operator with random face coefficients, like one row
    # of the 5-point operator: I + sum K (x_c - x_nb)
    k = rng.uniform(0.1, 50.0, n + 1)
    k[0] = k[-1] = 0.0
    a = np.diag(1.0 + k[:-1] + k[1:]) - np.diag(k[1:-1], 1) - np.diag(k[1:-1], -1)
    b = rng.standard_normal(n)
    alphas, betas = _cg_coefficients(a, b, iters)
    # the Lanczos tridiagonal of tea_leaf_cheby.f90:106-113
    diag = 1.0 / alphas
    diag[1:] += betas[:-1] / alphas[:-1]
    off = np.sqrt(betas[:-1]) / alphas[:-1]
    ritz = scipy_linalg.eigvalsh_tridiagonal(diag, off)
    info, emin, emax = _oracle_eigenvalues(alphas, betas)
    assert info == 0
    assert emin == pytest.approx(ritz[0], rel=1e-12)
    assert emax == pytest.approx(ritz[-1], rel=1e-12)
    lam = np.linalg.eigvalsh(a)
    assert lam[0] * (1 - 1e-12) <= emin and emax <= lam[-1] * (1 + 1e-12)


@pytest.mark.parametrize("eigmin,eigmax", [(0.9, 2.5e4), (1.0, 100.0)])
def test_oracle_chebyshev_coefficients_follow_the_closed_form(eigmin, eigmax):
    """rho_k = 1 / (2 sigma - rho_{k-1}) from rho_0 = 1 / sigma is
    T_k(sigma) / T_{k+1}(sigma) (Chebyshev polynomials of the first kind);
    alpha_k = rho_{k+1} rho_k, beta_k = 2 rho_{k+1} / delta
    (tea_leaf_cheby.f90:147-174)"""
    l = lib()
    l.ora_calc_ch_coefs.argtypes = [_D, _D, C.c_double, C.c_double, _D, C.c_int]
    l.ora_calc_ch_coefs.restype = None
    n = 400
    al, be = np.zeros(n), np.zeros(n)
    theta = C.c_double()
    l.ora_calc_ch_coefs(al.ctypes.data_as(_D), be.ctypes.data_as(_D), eigmin, eigmax, C.byref(theta), n)
    assert theta.value == (eigmax + eigmin) / 2.0
    delta = (eigmax - eigmin) / 2.0
    sigma = theta.value / delta
    acs = np.arccosh(sigma)
    k = np.arange(n + 2, dtype=np.float64)
    # T_k(sigma) / T_{k+1}(sigma) without overflow: cosh(k a) / cosh((k+1) a)
    rho = (np.exp(-acs) * (1.0 + np.exp(-2.0 * k * acs)) / (1.0 + np.exp(-2.0 * (k + 1.0) * acs)))
    np.testing.assert_allclose(al, rho[1:n + 1] * rho[:n], rtol=1e-11)
    np.testing.assert_allclose(be, 2.0 * rho[1:n + 1] / delta, rtol=1e-11)
    if sigma > 1.01:
        limit = sigma - np.sqrt(sigma * sigma - 1.0)
        assert al[-1] == pytest.approx(limit * limit, rel=1e-12)


@pytest.mark.parametrize("method", [dict(tl_use_cg=True, tl_preconditioner_type="jac_diag"),
                                    dict(tl_use_cg=False, tl_use_ppcg=True, tl_preconditioner_type="jac_block",
                                         tl_ppcg_inner_steps=10, tl_ch_cg_presteps=10, tl_ch_cg_epslim=1.0e10)])
def test_oracle_is_independent_of_its_thread_count(method):
    """The oracle's sums run per row in x order, then over rows in y order,
    so a solve gives the same bits on 1 and on 4 threads (the grid is above
    the size where its loops go parallel)."""
    from tests import decks
    from tests.oracle_run import run_deck
    deck = decks.make_deck(n=300, end_step=2, summary_frequency=1, **method)
    one, _ = run_deck(deck, threads=1)
    four, _ = run_deck(deck, threads=4)
    keys = ("iterations", "ppcg_inner", "switch_n", "error_ratio", "vol", "mass", "ie", "temp")
    assert len(one) == len(four) == 3  # the step-0 summary and two timesteps
    assert all(r["iterations"] > 10 for r in one[1:])
    for a, b in zip(one, four):
        for k in keys:
            assert a.get(k) == b.get(k), k
