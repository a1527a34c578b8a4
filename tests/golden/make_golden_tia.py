"""Generates tia/steps.npz in this folder from the reference's own
time-integration and Newton-convergence code.

Runs oracle/_ref/libxyceref_tia.so (the reference's N_TIA_OneStep,
N_TIA_DataStore and N_NLS_DampedNewton compiled from its sources by
oracle/ref_build/build_ref.py, driven by oracle/ref_build/xref_tia.C) over
a few trapezoid steps of two golden circuits, the 24-stage inverter chain and
the 7-stage ring oscillator: each step's F, Q, limiter vectors and matrices
are those of the circuit's transient loads in the device fixtures
(inverter_chain_24.npz, ring_7.npz, made by the reference's own device code).
Per step it stores the inputs and the reference's updateCoeffs, predictor,
residual, Jacobian and error estimate; then a table of Newton convergence
decisions over every branch of DampedNewton::converged_, and one of the step
control after accepted and failed steps (completeStep, rejectStep).  Needs the
reference source tree; the tests only read the .npz.

    python tests/golden/make_golden_tia.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

from helpers import Golden  # noqa: E402
from oracle import ref  # noqa: E402

STEPS_H = [1.0e-12, 2.3e-12, 0.91e-12, 4.7e-12, 1.3e-12, 7.9e-13]


def steps_of(name, rng):
    g = Golden(os.path.join(HERE, name + ".npz"))
    R = ref.integrator()
    loads = [k for k in range(g.n_loads) if g.flags(k).transient]
    out = {}
    psi = np.array([STEPS_H[0], STEPS_H[0], STEPS_H[0]])
    h_sum = 2 * STEPS_H[0]
    for s in range(len(loads) - 1):
        prev, cur = g.outputs(loads[s]), g.outputs(loads[s + 1])
        sol = g.inputs(loads[s + 1])[0]
        n = len(cur["F"])
        order = 1 if s == 0 else 2
        h = STEPS_H[s % len(STEPS_H)]
        p = f"{name}.s{s}."
        out[p + "scalars"] = np.array([order, h, h_sum])
        out[p + "psi_in"] = psi.copy()
        psi, beta, alphas, ck = R.update_coeffs(order, h, h_sum, psi)
        out[p + "psi"], out[p + "beta"], out[p + "alphas_ck"] = psi, beta, np.array([alphas, ck])
        xh0, xh1 = sol[1][:n], sol[1][:n] - sol[2][:n]
        xh2 = 0.1 * rng.standard_normal(n)
        qh0 = prev["Q"]
        out[p + "xh0"], out[p + "xh1"], out[p + "xh2"], out[p + "qh0"] = xh0, xh1, xh2, qh0
        xn0, qn0 = R.predictor(order, beta, xh0, xh1, xh2, qh0)
        out[p + "xn0"], out[p + "qn0"] = xn0, qn0
        for key in ("Q", "F", "dFdxdVp", "dQdxdVp", "dFdx", "dQdx"):
            out[p + key] = cur[key]
        out[p + "qh2"] = prev["F"]
        out[p + "rhs"] = R.residual(order, h, alphas, 1, cur["Q"], qn0, cur["F"], prev["F"],
                                    cur["dFdxdVp"], cur["dQdxdVp"])
        out[p + "rhs_nolim"] = R.residual(order, h, alphas, 0, cur["Q"], qn0, cur["F"], prev["F"],
                                          cur["dFdxdVp"], cur["dQdxdVp"])
        out[p + "jac"] = R.jacobian(order, h, alphas, cur["dQdx"], cur["dFdx"])
        x_next = sol[0][:n]
        out[p + "x_next"] = x_next
        out[p + "est"] = np.array([R.error_estimate(ck, xh0, x_next - xn0, 1e-3, 1e-6)])
        h_sum = h + STEPS_H[(s + 1) % len(STEPS_H)]
    out[name + ".n_steps"] = np.array([len(loads) - 1])
    return out


def convergence_table(rng):
    """Cases over every branch of converged_: residual below machine
    precision, normal convergence, near convergence past the step limit,
    small update, too many steps, a huge update, and five-step stalls."""
    R = ref.integrator()
    rows, res = [], []
    for transient in (0, 1):
        max_step, rhs_tol, dx_tol = (20, 1e-2, 0.33) if transient else (200, 1e-6, 1.0)
        cases = [(3, 1e-17, 5.0, 0.5, 0.5), (3, 1e-3 * rhs_tol, 0.1, 0.5, 0.5),
                 (max_step + 1, 10 * rhs_tol, 2.0, 0.5, 0.9), (4, 10 * rhs_tol, 1e-7, 0.5, 0.9),
                 (max_step + 1, 10 * rhs_tol, 2.0, 0.95, 1.2), (5, 10 * rhs_tol, 2.0, 0.5, 1e308),
                 (2, 10 * rhs_tol, 2.0, 0.5, 0.5)]
        for _ in range(60):
            cases.append((int(rng.integers(1, max_step + 3)), 10 ** rng.uniform(-18, 1) * rhs_tol,
                          10 ** rng.uniform(-8, 1), rng.uniform(0, 2), 10 ** rng.uniform(-3, 1)))
        for step, max_rhs, upd, rhs_rel, rate in cases:
            r = R.converged(transient, step, max_step, rhs_tol, dx_tol, 1e-6, max_rhs, upd, rhs_rel, rate)
            rows.append([transient, step, max_step, rhs_tol, dx_tol, max_rhs, upd, rhs_rel, rate, 0, 0.0])
            res.append(list(r))
        # a stall: five steps with the rate within 1e-3 of 1, then the verdict
        for rel in (0.5, 0.95):
            count, tmp = 0, 0.0
            for k in range(6):
                rate = 1.0 + (k % 3 - 1) * 4e-4
                r = R.converged(transient, 2 + k, max_step, rhs_tol, dx_tol, 1e-6, 10 * rhs_tol, 2.0,
                                rel, rate, count, tmp)
                rows.append([transient, 2 + k, max_step, rhs_tol, dx_tol, 10 * rhs_tol, 2.0, rel, rate,
                             count, tmp])
                res.append(list(r))
                count, tmp = r[1], r[2]
    return {"conv.inputs": np.array(rows, float), "conv.outputs": np.array(res, float)}


def step_control_table(rng):
    """completeStep / rejectStep over accepted and failed steps: estimates
    around the acceptance bound, first and later failures, Newton failures,
    orders 1 and 2, steps clipped at a breakpoint and bounded by the min and
    max step; the histories of the accepted ones are random vectors."""
    R = ref.integrator()
    out = {}
    acc_in, acc_out, rej_in, rej_out = [], [], [], []
    n = 5
    for k in range(120):
        order = int(rng.integers(1, 3))
        steps = int(rng.integers(0, 6))
        h = 10 ** rng.uniform(-13, -10)
        t = rng.uniform(0, 5e-9)
        stop = t + h * (rng.choice([0.5, 1.0, 3.0, 50.0]) + rng.uniform(0, 1))
        state = [order, steps, int(rng.integers(0, 3)), 10 ** rng.uniform(-4, 1), h, t, t + h,
                 stop, t * 10 * 2.220446049250313e-16, rng.choice([1e-12, 1e-10, 1e-9]),
                 h * rng.uniform(0.3, 3), h * rng.uniform(1.5, 4),
                 h, h * rng.uniform(0.5, 2), h * rng.uniform(0.5, 2), int(rng.choice([-1, 0, 2])),
                 h * 2]
        hist = [rng.standard_normal(n) for _ in range(6)]
        x, q, f = rng.standard_normal(n), rng.standard_normal(n), rng.standard_normal(n)
        res, hs = R.complete_step(state, hist, x, q, f)
        out[f"acc{k}.state"] = np.array(state, float)
        out[f"acc{k}.hist"] = np.array(hist)
        out[f"acc{k}.xqf"] = np.array([x, q, f])
        out[f"acc{k}.out"] = res
        out[f"acc{k}.hist_out"] = np.array(hs)
        rej_in.append(state)
        rej_out.append(R.reject_step(state))
    out["rej.inputs"] = np.array(rej_in, float)
    out["rej.outputs"] = np.array(rej_out, float)
    out["acc.n"] = np.array([120])
    return out


def main():
    if not ref.tia_available():
        print("oracle/_ref/libxyceref_tia.so not built (needs the reference source tree)")
        return 1
    rng = np.random.default_rng(2024)
    out = {}
    for name in ("inverter_chain_24", "ring_7"):
        out.update(steps_of(name, rng))
    out.update(convergence_table(rng))
    out.update(step_control_table(rng))
    path = os.path.join(HERE, "tia", "steps.npz")
    np.savez_compressed(path, **out)
    print(path, len(out), "arrays")
    return 0


if __name__ == "__main__":
    sys.exit(main())
