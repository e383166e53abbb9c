"""Run-driver host logic against the reference's integration engine.

The golden file ``tests/golden/schedule_events.json`` holds the events the
reference's ``IntegrationScheduler`` / ``integrate`` produced (made by
``tests/golden/make_golden.py runs`` from src/planetary_sandbox/run/engine.py),
with every time and step length as an exact float (hex); the GB300 runner's
scheduler must reproduce them bit for bit, including the cases that raise.
No GPU is needed: the scheduler never touches the state.
"""
import json
import math

import pytest

from conftest import GOLDEN
from aeolus_gb300 import runner as RN

with open(GOLDEN / "schedule_events.json") as _f:
    G = json.load(_f)


def _hex_events(events):
    return [[k, float(dt).hex(), float(t).hex()] for k, dt, t in events]


@pytest.mark.parametrize("case", [c for c in G["cases"] if c["kind"] == "plan"], ids=lambda c: c["name"])
def test_constant_ceiling_plans_match_reference(case):
    ev = RN.integration_plan(case["t_end"], case["dt_cfl"], **case["kw"])
    assert _hex_events(ev) == case["events"]


@pytest.mark.parametrize("case", [c for c in G["cases"] if c["kind"] == "adaptive"], ids=lambda c: c["name"])
def test_state_adaptive_stepping_matches_reference(case):
    speeds, ls = case["speeds"], case["length_scale"]
    sch = RN.IntegrationScheduler(case["t_end"], **case["kw"])
    events = []

    def on_step(t0, t1, dt, k):
        events.append(("step", dt, t1))
        return speeds[(k - 1) % len(speeds)]

    out = RN.integrate(sch, RN.advective_cfl_timestep(ls, speeds[-1]), ls, on_step=on_step,
                       on_store=lambda t: events.append(("store", 0.0, t)))
    assert _hex_events(events) == case["events"]
    assert [float(out[0]).hex(), out[1]] == case["final"]


def test_stagnating_ceiling_raises_like_reference():
    case = next(c for c in G["cases"] if c["kind"] == "stagnation")
    sch = RN.IntegrationScheduler(1.0e6, mode="count", snapshot_times=[5.0e5, 1.0e6])
    got = []
    assert case["raises"] == "FloatingPointError"
    with pytest.raises(FloatingPointError):
        for dt in [5.0e5] + [1e-12] * 4:
            got.append(sch.next_event(dt))
    assert _hex_events(got) == case["events"]


def _outcome(fn, *a):
    try:
        return {"value": float(fn(*a)).hex()}
    except Exception as exc:
        return {"raises": type(exc).__name__}


def test_cfl_ceiling_matches_reference():
    for ls, sp, want in G["helpers"]["cfl"]:
        assert _outcome(RN.advective_cfl_timestep, ls, sp) == want, (ls, sp)


def test_schedule_helpers_match_reference():
    for times, t_end, want in G["helpers"]["validate"]:
        try:
            got = {"value": [float(x).hex() for x in RN.validate_snapshot_schedule(times, t_end)]}
        except Exception as exc:
            got = {"raises": type(exc).__name__}
        assert got == want, (times, t_end)
    for d, t, want in G["helpers"]["interval_times"]:
        assert [float(x).hex() for x in RN.interval_snapshot_times(d, t)] == want
    for n, t, want in G["helpers"]["count_times"]:
        assert [float(x).hex() for x in RN.count_snapshot_times(n, t)] == want
    for bad, want in G["helpers"]["bad_ceiling"]:
        with pytest.raises(ValueError):
            RN.IntegrationScheduler(100.0, mode="count", snapshot_times=[100.0]).next_event(bad)
        assert want == "ValueError"


def test_mode_errors():
    with pytest.raises(ValueError):
        RN.IntegrationScheduler(10.0, mode="bogus")
    with pytest.raises(ValueError):
        RN.IntegrationScheduler(10.0, mode="interval")
    with pytest.raises(ValueError):
        RN._resolve_schedule("count", None, None, 10.0)
    with pytest.raises(ValueError):
        RN._resolve_schedule("interval", None, None, 10.0)
    with pytest.raises(ValueError):
        RN._resolve_schedule("weekly", [1.0], None, 10.0)
    assert RN._resolve_schedule(None, [0.0, 10.0], None, 10.0) == ("count", [0.0, 10.0])
    assert RN._resolve_schedule(None, None, 5.0, 10.0) == ("interval", None)
    assert math.isclose(RN.integration_plan(10.0, 4.0, mode="count", snapshot_times=[10.0])[-1][2], 10.0)
