"""Writes tests/golden/rnp_ref_*.npz: outputs of the reference's own
RNPBond, Neighbor, Fracture, InteriorFlags and ULoading/FLoading sources
(oracle/refshim, compiled from the NLMech tree) on the problems of
tests/refcases.py, for the GPU tests to compare against on machines without
the reference tree.

    python tests/golden/make_rnp_golden.py [case ...]   (default: every case)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import oracle as orc  # noqa: E402
import refcases  # noqa: E402

CASES = refcases.GOLDEN_CASES


def main(names=None):
    for name, (make, steps) in CASES.items():
        if names and name not in names:
            continue
        p = make()
        r = orc.RefRNP(p)
        rowptr, cols = r.neighbors()
        pre = r.bond_state()
        r.run(steps)
        u, v, f = r.state()
        t, n = r.time()
        broken = r.bond_state()
        energies = r.energies()  # strain, work, kinetic, fracture (computePostProcFields)
        extra = {"reaction": r.reaction_force()} if p.dim == 2 else {}
        out = os.path.join(HERE, "rnp_ref_%s.npz" % name)
        np.savez_compressed(out, u=u, v=v, f=f, rowptr=rowptr, cols=cols, precrack=pre,
                            broken=broken, fixity=r.fixity(), time=t, steps=n,
                            energies=energies, **extra)
        print(out, os.path.getsize(out), "bytes,", int(r.bond_state().sum()), "broken")


if __name__ == "__main__":
    main(sys.argv[1:])
