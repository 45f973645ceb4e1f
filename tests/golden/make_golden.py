"""Writes the golden fixtures of tests/golden from the oracle.

The reference (Fortran 90 + MPI) cannot be built or run on the machines this
library is developed and tested on, and it ships no test data, so these are
NOT outputs of the reference: they are outputs of the oracle (the C++ FP64
restatement in oracle/), committed so that any later change to the oracle or
the library that alters the results of these cases is caught.  Each fixture
holds the seeded start's recipe, the fields after 4 steps, the per-step
iteration counts and the recycling state.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from turbulentbl_gb300.synth import small_workload, make_state  # noqa: E402
from oracle.bind import OracleRunner  # noqa: E402

CASES = {
    # name: (variant, nproc, recycle_after, cum, nstep0, cnt2)
    "dnstbl2_p2": (0, 2, 2, 3, 0, 0),
    "original_p2": (1, 2, 2, 3, 0, 5000),
    "dnssetbl_p3": (2, 3, 2, 3, 4000, 0),
}
GRID = dict(nx=12, nz_span=6, ny_wall=14, kmax=10)
STEPS = 4


def case_setup(name):
    variant, P, rec_after, cum, nstep0, cnt2 = CASES[name]
    wl = small_workload(**GRID)
    mesh, rp, st = make_state(wl, nproc=P)
    rp.variant, rp.recycle_after, rp.cum = variant, rec_after, cum
    st = dict(st, nstep=nstep0, cnt2=cnt2)
    return mesh, rp, st


def run_oracle(name):
    mesh, rp, st = case_setup(name)
    o = OracleRunner(mesh, rp)
    o.upload(st)
    counts = []
    for _ in range(STEPS):
        o.step(1)
        counts.append(o.last_counts())
    d = o.download()
    return d, counts


def main():
    for name in CASES:
        d, counts = run_oracle(name)
        width = max(len(c) for c in counts)
        cnt = np.full((STEPS, width), -1, dtype=np.int32)
        for q, c in enumerate(counts):
            cnt[q, :len(c)] = c
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), u=d["u"], v=d["v"], w=d["w"], p=d["p"],
                            newk=d["newk"], wt=d["wt"], lamda=d["lamda"], nstep=d["nstep"], counts=cnt)
        print(name, "written")


if __name__ == "__main__":
    main()
