"""The stopping rule of the oracle's LM (``oracle.solver.lm_solve``) clause by clause, on
scripted steps: the linearisation, damped solve, update and cost are replaced by fakes
that return a given sequence of candidate costs and predicted decreases, so each case
exercises one clause of the rule (the GPU's k_decide applies the same rule;
``test_stop_rho_matches_oracle`` compares the two on a real scene).

An accepted step whose relative decrease is below tol ends the solve when
  * stop_rho is 0 (the plain rule), or
  * its gain ratio rho = actual / predicted decrease is at least stop_rho, or
  * its predicted relative decrease is itself below tol, or
  * the accepted step before it also lowered the cost by less than tol."""
import types

import pytest

from oracle import solver as S

TOL = 1e-6


def run_script(monkeypatch, steps, stop_rho, F0=100.0):
    """steps: (relative decrease, predicted relative decrease) of each candidate, both
    relative to the cost before the step; returns the LMResult."""
    state = {"F": F0, "k": 0}
    monkeypatch.setattr(S, "linearize", lambda prob, loss: types.SimpleNamespace(cost=state["F"]))

    def solve_damped(lin, lam, eps):
        rel, pred_rel = steps[state["k"]]
        state["rel"] = rel
        return types.SimpleNamespace(ok=True, pred=pred_rel * lin.cost, delta=None, delta_a=None)

    def cost(prob, loss):
        Fn = state["F"] * (1.0 - state["rel"])
        state["k"] += 1
        state["F"] = Fn if Fn < state["F"] else state["F"]
        return Fn

    monkeypatch.setattr(S, "solve_damped", solve_damped)
    monkeypatch.setattr(S, "apply_update", lambda poses, alpha, *a, **k: (poses, alpha))
    monkeypatch.setattr(S, "cost", cost)
    prob = types.SimpleNamespace(poses=None, alpha=None)
    return S.lm_solve(prob, S.Loss(), max_iters=len(steps), tol=TOL, stop_rho=stop_rho)


@pytest.mark.parametrize("name,steps,stops_at", [
    # a well-modelled small step (rho = 1): every rule stops at once
    ("rho", [(5e-10, 5e-10), (1e-1, 1e-1)], {0.0: 1, 0.25: 1}),
    # a poorly modelled small step (rho = 5e-5) that promised 1 %: the plain rule stops,
    # the condition goes on; a large step, then a well-modelled small one stops it
    ("plateau", [(5e-7, 1e-2), (1e-1, 1.1e-1), (5e-10, 5e-10), (1e-1, 1e-1)], {0.0: 1, 0.25: 3}),
    # a poorly modelled small step (rho = 0.11) whose model promised less than tol
    ("pred", [(1e-7, 9e-7), (1e-1, 1e-1)], {0.0: 1, 0.25: 1}),
    # two poorly modelled small steps in a row: the second one stops it
    ("two_small", [(5e-7, 1e-2), (4e-7, 1e-2), (1e-1, 1e-1)], {0.0: 1, 0.25: 2}),
])
def test_stopping_rule_clauses(monkeypatch, name, steps, stops_at):
    for stop_rho, it in stops_at.items():
        r = run_script(monkeypatch, steps, stop_rho)
        assert r.converged and r.iterations == it, (name, stop_rho, r.iterations)
