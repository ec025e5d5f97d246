"""The planner check tool (nbody_gb300.plancheck) on one small size: it
reports the planner's plan and a grid of forced plans, all timed."""
import pytest

pytestmark = pytest.mark.gpu


def test_plancheck_reports_plan_and_grid(cuda):
    from nbody_gb300 import force_config_names
    from nbody_gb300.plancheck import check
    r = check(4096, calls=2)
    assert r["n"] == 4096 and r["plan"]["config"] in force_config_names()
    assert r["plan"]["us"] > 0 and r["plan"]["nsplit"] >= 1
    assert len(r["grid_best"]) == 3 and all(g["us"] > 0 for g in r["grid_best"])
    assert r["plan_over_best"] > 0
