"""Writes the golden fixtures under tests/golden/ from the oracle.

config1_300steps.npz: seismograms (16 receivers x vx,vy,vz x 300 steps) and
every second point of the final vz field of config 1 (homogeneous elastic
12x12x8, lpd 4, moment-tensor Ricker source) after 300 steps.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [os.path.join(ROOT, "ses3d-nt_gb300"), os.path.join(ROOT, "oracle")]

import sesnt_oracle  # noqa: E402
import workloads  # noqa: E402

NT = 300


def main():
    wl = workloads.config1(nt=NT)
    o = sesnt_oracle.Oracle(wl.grid)
    sesnt_oracle.load_workload(o, wl)
    o.run(NT)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "config1_300steps.npz")
    np.savez_compressed(out, nt=NT, seismograms=o.seismograms(),
                        vz_sub=o.field(2)[::2, ::2, ::2, ::2, ::2, ::2])
    print("wrote", out)


if __name__ == "__main__":
    main()
