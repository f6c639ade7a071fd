#!/usr/bin/env python3
"""Calibrate the oracle port of the reference's element loop against the reference itself.

The CPU baseline on machines without the reference sources (the GPU machines) times the port
(oracle/anifem_oracle.c, gradgrad_sym): the P2 GRAD.GRAD fem3Dtet loop with a per-tet symmetric
tensor at order 4.  Where the reference build exists (oracle/_ref, made by `make -C oracle ref`),
this script times both on the same tets and threads and writes the ratio to
oracle/port_calibration.json, which the benchmark reports beside its CPU baseline:

    python oracle/calibrate_port.py [ntets]
"""
import json
import os
import platform
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "inmost-fem_gb300"))

from anigpu import meshgen  # noqa: E402
from oracle.oracle import Reference, Restated  # noqa: E402


def cpu_model():
    try:
        with open("/proc/cpuinfo") as fh:
            for line in fh:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def main():
    nt = int(sys.argv[1]) if len(sys.argv) > 1 else 100000
    if not Reference.available():
        raise SystemExit("the reference build is missing: make -C oracle ref REF_ROOT=<reference checkout>")
    xyz, tets, D6 = meshgen.p2_aniso_workload(64)
    XY = meshgen.tet_coords(xyz, tets[:nt])
    D6 = D6[:nt]
    ref, port = Reference(), Restated()
    out = {"workload": f"P2 GRAD.GRAD, per-tet symmetric tensor, order 4, first {nt} tets of the 64^3 workload",
           "host": cpu_model(), "machine": platform.machine(), "threads": {}}
    for th in (1, os.cpu_count() or 1):
        best_r = min(ref.time_p2_sym(XY, D6, 4, th)[0] for _ in range(3))
        best_p = min(port.time_p2_sym(XY, D6, 4, th)[0] for _ in range(3))
        out["threads"][str(th)] = {"reference_us_per_tet": 1e6 * best_r / nt, "port_us_per_tet": 1e6 * best_p / nt,
                                   "port_over_reference": best_p / best_r}
    path = os.path.join(HERE, "port_calibration.json")
    with open(path, "w") as fh:
        json.dump(out, fh, indent=1)
        fh.write("\n")
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
