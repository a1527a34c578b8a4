"""The transient oracle's integrator formulas (oracle/xgo_tran.c) held to the
reference's own compiled time-integration and Newton code.

tests/golden/tia/steps.npz was written by the reference's N_TIA_OneStep
(updateCoeffs, obtainPredictor, obtainResidual, obtainJacobian), its
N_TIA_DataStore error weights and WRMS norm, N_NLS_DampedNewton::
converged_, and the step control of OneStep::completeStep and rejectStep
(oracle/_ref/libxyceref_tia.so, made by
tests/golden/make_golden_tia.py) over trapezoid steps of the 24-stage
inverter chain and the 7-stage ring oscillator, on the F, Q, limiter
vectors and matrices of their transient loads in the device fixtures.  The
oracle must reproduce every array bit for bit and every convergence
decision exactly; the same formulas drive its transient, which the GPU
stepper is held to at the benchmarked sizes.  Where the reference library
is built, a second test compares the two on fresh random inputs.
"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "tia", "steps.npz")


@pytest.fixture(scope="module")
def fx():
    return np.load(FIX)


@pytest.fixture(scope="module")
def integ(oracle_lib):
    from oracle.oracle import Integrator
    return Integrator()


@pytest.mark.parametrize("name", ["inverter_chain_24", "ring_7"])
def test_integrator_steps_match_reference(name, fx, integ):
    n_steps = int(fx[name + ".n_steps"][0])
    assert n_steps >= 3
    for s in range(n_steps):
        p = f"{name}.s{s}."
        g = lambda k: fx[p + k]  # noqa: E731
        order, h, h_sum = g("scalars")
        order = int(order)
        psi, beta, alphas, ck = integ.update_coeffs(order, h, h_sum, g("psi_in"))
        assert np.array_equal(psi, g("psi")) and np.array_equal(beta, g("beta")), s
        assert np.array_equal([alphas, ck], g("alphas_ck")), s
        xn0, qn0 = integ.predictor(order, beta, g("xh0"), g("xh1"), g("xh2"), g("qh0"))
        assert np.array_equal(xn0, g("xn0")) and np.array_equal(qn0, g("qn0")), s
        args = (g("Q"), qn0, g("F"), g("qh2"), g("dFdxdVp"), g("dQdxdVp"))
        assert np.array_equal(integ.residual(order, h, alphas, 1, *args), g("rhs")), s
        rhs0 = integ.residual(order, h, alphas, 0, *args)
        assert np.array_equal(rhs0, g("rhs_nolim")), s
        assert np.array_equal(integ.jacobian(order, h, alphas, g("dQdx"), g("dFdx")), g("jac")), s
        est = integ.error_estimate(ck, g("xh0"), g("x_next") - xn0, 1e-3, 1e-6)
        assert est == g("est")[0], (s, est, g("est")[0])


def test_newton_convergence_decisions_match_reference(fx, integ):
    ins, outs = fx["conv.inputs"], fx["conv.outputs"]
    seen = set()
    for row, want in zip(ins, outs):
        transient, step, max_step, rhs_tol, dx_tol, max_rhs, upd, rel, rate, count, tmp = row
        got = integ.converged(int(transient), int(step), int(max_step), rhs_tol, dx_tol, 1e-6, max_rhs,
                              upd, rel, rate, int(count), tmp)
        assert got[0] == int(want[0]) and got[1] == int(want[1]) and got[2] == want[2], (row, got, want)
        seen.add(got[0])
    # every verdict of the test was exercised
    assert seen >= {1, 2, 3, 4, -1, -2, -3, 0}, seen


def test_step_control_matches_reference(fx, integ):
    """Accepted steps: the next order and step, the breakpoint clip, the
    saved step, the rotated histories; failed steps: Newton failure, first
    and later local-error failures.  Every case bit for bit."""
    branches = set()
    for k in range(int(fx["acc.n"][0])):
        st = fx[f"acc{k}.state"]
        out, hs = integ.complete_step(st, list(fx[f"acc{k}.hist"]), *fx[f"acc{k}.xqf"])
        assert np.array_equal(out, fx[f"acc{k}.out"]), (k, out, fx[f"acc{k}.out"])
        assert np.array_equal(np.array(hs), fx[f"acc{k}.hist_out"]), k
        ratio = out[3] / st[4]
        branches.add("clip" if out[5] == st[7] else "grow" if ratio == 2.0 else
                     "shrink" if ratio < 1.0 else "keep" if ratio == 1.0 else "bounded")
        branches.add(f"order{int(out[0])}")
    assert branches >= {"clip", "grow", "shrink", "keep", "order1", "order2"}, branches
    seen = set()
    for st, want in zip(fx["rej.inputs"], fx["rej.outputs"]):
        got = integ.reject_step(st)
        assert np.array_equal(got, want), (st, got, want)
        seen.add("newton" if st[15] <= 0 else "first" if st[2] == 0 else "later")
    assert seen == {"newton", "first", "later"}, seen


def test_integrator_matches_live_reference_random(integ):
    from oracle import ref
    if not ref.tia_available():
        pytest.skip("oracle/_ref/libxyceref_tia.so not built (needs the reference source tree)")
    R = ref.integrator()
    rng = np.random.default_rng(7)
    for trial in range(20):
        n = int(rng.integers(1, 200))
        order = int(rng.integers(1, 3))
        h, h_sum = 10 ** rng.uniform(-14, -9), 10 ** rng.uniform(-13, -8)
        psi_in = 10 ** rng.uniform(-14, -9, 3)
        a, b = integ.update_coeffs(order, h, h_sum, psi_in), R.update_coeffs(order, h, h_sum, psi_in)
        assert all(np.array_equal(x, y) for x, y in zip(a, b)), trial
        _, beta, alphas, ck = a
        v = [rng.standard_normal(n) * 10 ** rng.uniform(-15, 1) for _ in range(8)]
        assert all(np.array_equal(x, y) for x, y in zip(integ.predictor(order, beta, *v[:4]),
                                                        R.predictor(order, beta, *v[:4]))), trial
        for lim in (0, 1):
            assert np.array_equal(integ.residual(order, h, alphas, lim, *v[:6]),
                                  R.residual(order, h, alphas, lim, *v[:6])), trial
        assert np.array_equal(integ.jacobian(order, h, alphas, v[6], v[7]),
                              R.jacobian(order, h, alphas, v[6], v[7])), trial
        x, corr = v[0], v[1] * 1e-3
        assert integ.error_estimate(ck, x, corr, 1e-3, 1e-6) == R.error_estimate(ck, x, corr, 1e-3, 1e-6)
