"""The host-only planner entry (nbgb_force_plan_on) given this GPU's own SM
count and occupancy table decides exactly as the planner on the device."""
import pytest

import nbody_gb300 as nb

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 1000, 4096, 16384, 65536, 155677, 262144, 1048576])
def test_host_planner_matches_device_planner(cuda, n):
    sms, occ = nb.force_device_info()
    assert sms > 0 and len(occ) == len(nb.force_config_names())
    c, s, f, w = nb.force_plan_on(n, sms, occ)
    assert (c, s, w) == nb.force_plan(n)
    for config, nsplit in ((0, 4), (45, -16), (32, 1)):
        r = nb.force_plan_on(n, sms, occ, config, nsplit)
        assert (r[0], r[1], r[3]) == nb.force_plan(n, config, nsplit)
