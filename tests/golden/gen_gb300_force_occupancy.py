"""Writes tests/golden/gb300_force_occupancy.json: the SM count and the
resident CTAs per SM of every force-kernel configuration on this GPU, as the
planner reads them (nbgb_force_device_info).  Run on a GB300:

    python tests/golden/gen_gb300_force_occupancy.py [OUT]

The CPU tests of the planner (tests/test_planner.py) plan against this table
with nbgb_force_plan_on, so they pin the planner's decisions for a GB300
without a GPU."""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import nbody_gb300 as nb  # noqa: E402


def main():
    import torch
    out = sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "gb300_force_occupancy.json")
    sms, occ = nb.force_device_info()
    rec = {"device": torch.cuda.get_device_name(0), "sms": sms,
           "configs": nb.force_config_names(), "occupancy": occ}
    with open(out, "w") as f:
        json.dump(rec, f, indent=1)
    print(out, sms, occ)


if __name__ == "__main__":
    main()
