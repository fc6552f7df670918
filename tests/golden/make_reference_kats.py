"""Generate tests/golden/reference_kats.json from the reference's own tests.

The reference (ClassicalSpinMC.jl) is Julia and cannot run in this
environment, so its known-answer tests are read as text: each case below names
the file and line of the reference test it restates, and this script checks
that the cited line really contains the expected value before writing the
JSON.  Run from the repository root with the reference checked out at
``$CSMC_REFERENCE`` (default: a sibling checkout path given on the command line).
"""
from __future__ import annotations

import json
import os
import sys
from pathlib import Path

CASES = [
    {
        "name": "zeeman_energy",
        "source": "test/latticetests.jl:17",
        "needle": "-1.0 == total_energy(lat)",
        "model": {"bravais": "Square", "shape": [1, 1], "S": 1.0, "field": [[1, [1.0, 0.0, 0.0]]],
                  "spins": [[1.0, 0.0, 0.0]]},
        "expect": {"total_energy": -1.0},
    },
    {
        "name": "zeeman_local_field",
        "source": "test/latticetests.jl:18",
        "needle": "tuple((-h)...) == get_local_field(lat, 1)",
        "model": {"bravais": "Square", "shape": [1, 1], "S": 1.0, "field": [[1, [1.0, 0.0, 0.0]]],
                  "spins": [[1.0, 0.0, 0.0]]},
        "expect": {"local_field_site1": [-1.0, -0.0, -0.0]},
    },
    {
        "name": "bilinear_fm_energy_density",
        "source": "test/latticetests.jl:30",
        "needle": "-2.0 == total_energy(lat) / lat.size",
        "model": {"bravais": "Square", "shape": [2, 2], "S": 1.0,
                  "bilinear": [[1, 1, "-I", [1, 0]], [1, 1, "-I", [-1, 0]], [1, 1, "-I", [0, 1]],
                               [1, 1, "-I", [0, -1]]],
                  "spins_all": [1.0, 0.0, 0.0]},
        "expect": {"energy_density": -2.0},
    },
    {
        "name": "honeycomb_kitaev_gamma_anneal",
        "source": "test/mctests.jl:49",
        "needle": "-0.6444 == round(E, digits=4)",
        "model": {"bravais": "Honeycomb", "shape": [4, 4], "S": 1.0, "J": 0.0, "K": -1.0, "G": 0.2, "Gp": -0.02,
                  "h": 0.1, "h_dir": "(1,1,1)/sqrt(3)", "bonds": "test/mctests.jl:14-29",
                  "T0": 1.0, "T": 1e-7, "schedule": "T0*0.9^x",
                  "params": {"t_thermalization": 10000, "overrelaxation_rate": 10, "t_deterministic": 1000000},
                  "alg": "Metropolis", "deterministic": True},
        "expect": {"energy_density_4dp": -0.6444},
    },
    {
        "name": "honeycomb_kitaev_gamma_anneal_adaptive",
        "source": "test/mctests.jl:57",
        "needle": "-0.6444 == round(E, digits=4)",
        "model": {"bravais": "Honeycomb", "shape": [4, 4], "S": 1.0, "J": 0.0, "K": -1.0, "G": 0.2, "Gp": -0.02,
                  "h": 0.1, "h_dir": "(1,1,1)/sqrt(3)", "bonds": "test/mctests.jl:14-29",
                  "T0": 1.0, "T": 1e-7, "schedule": "T0*0.9^x",
                  "params": {"t_thermalization": 10000, "overrelaxation_rate": 10, "t_deterministic": 1000000},
                  "alg": "MetropolisAdaptive", "deterministic": False},
        "expect": {"energy_density_4dp": -0.6444},
    },
]


def main(ref_root: Path) -> None:
    # the reference's tests live in one file per topic; line numbers cited
    # above are within those files
    for c in CASES:
        path, line = c["source"].split(":")
        text = (ref_root / path).read_text().splitlines()
        lineno = int(line)
        window = "\n".join(text[max(0, lineno - 3):lineno + 2])
        if c["needle"] not in window:
            raise SystemExit(f"{c['name']}: '{c['needle']}' not found near {c['source']}")
    out = Path(__file__).resolve().parent / "reference_kats.json"
    out.write_text(json.dumps({"reference": "ClassicalSpinMC.jl v1.0.0", "cases": CASES}, indent=1) + "\n")
    print("wrote", out)


if __name__ == "__main__":
    root = Path(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CSMC_REFERENCE", "."))
    main(root)
