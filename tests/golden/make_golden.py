"""Writes the golden fixtures in tests/golden/ from the reference itself.

Run where the reference sources are present (the reference library is built
from them by oracle/Makefile):

    python tests/golden/make_golden.py

For each case it writes the case directory (mesh and input.hamstr in the
reference's formats) and <case>.npz holding:
  freestream  uinf, vinf, einf the reference computed (set explicitly by the
              tests, so machines whose libm cos/sin differ in the last bit
              still compare against the same state)
  q0          the initial state
  hist        per-step norms: computeRHS L2, Linf, final linear L2, Linf
  q, dq, r, r0, sigma, ff   the reference's arrays after the last step
  end_rule    the chain end rule the case runs under

Cases on split (mixed tri/quad) meshes under the reference's own rule come
from the reference too.  The extended end rule has no reference
counterpart: its case is written by the C restatement (kind "port"), so it
pins later changes of the CUDA path and the restatement against each other.
"""
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from hamstr_oop_gb300 import meshgen  # noqa: E402
from oracle import oracle  # noqa: E402

CASES = {
    "ogrid16x4_o3": dict(ni=16, nj=4, order=3, CFL=10.0, msweep=2, steps=6),
    "ogrid16x4_o1": dict(ni=16, nj=4, order=1, CFL=10.0, msweep=2, steps=6),
    "ogrid16x5_o5": dict(ni=16, nj=5, order=5, CFL=20.0, msweep=2, steps=6),
    "ogrid16x4_o3_loop0": dict(ni=16, nj=4, order=3, CFL=10.0, msweep=3, steps=5, loop_start=0),
    "split32x12_light_o3": dict(ni=32, nj=12, order=3, CFL=2.0, msweep=2, steps=5, split=0.04, seed=29),
    "split24x8_half_o5_ext": dict(ni=24, nj=8, order=5, CFL=5.0, msweep=2, steps=5, split=0.5, seed=1,
                                  end_rule=1),
}


def main():
    oracle.build(reference=True)
    for name, c in CASES.items():
        d = os.path.join(HERE, name)
        if os.path.isdir(d):
            shutil.rmtree(d)
        mesh = meshgen.naca0012_ogrid(c["ni"], c["nj"], loop_start=c.get("loop_start"),
                                      split=c.get("split", 0.0), seed=c.get("seed", 0))
        meshgen.write_case(d, mesh, dict(order=c["order"], CFL=c["CFL"], msweep=c["msweep"], nsteps=c["steps"]))
        rule = c.get("end_rule", 0)
        ref = oracle.OracleCase(d, "reference" if rule == 0 else "port")
        ref.set_option("chain_end_rule", rule)
        p = ref.params
        q0 = ref.get("q")
        hist = ref.march(c["steps"])
        np.savez_compressed(os.path.join(HERE, name + ".npz"),
                            freestream=np.array([p["uinf"], p["vinf"], p["einf"]]), q0=q0, hist=hist,
                            q=ref.get("q"), dq=ref.get("dq"), r=ref.get("r"), r0=ref.get("r0"),
                            sigma=ref.get("sigma"), ff=ref.get("ff"), end_rule=np.array(rule))
        print(name, ref.sizes["nCell"], "cells, final L2", hist[-1, 0])


if __name__ == "__main__":
    main()
