"""Generates tests/golden/*.npz from the FP64 oracle.  These are regression fixtures of the
oracle itself (the reference cannot run here and ships no golden vectors): they catch
drift of the restatement across machines and edits.  Run: python tests/golden/make_golden.py"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "kitamr.jl_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import numpy as np  # noqa: E402

import oracle as O  # noqa: E402
from kitgpu import abi, cases  # noqa: E402


def main():
    n, nv, steps = 6, 12, 3
    p = cases.couette(n=n, nv=nv)
    topo, state = cases.build(p)
    st = O.OracleState(topo, state)
    st.run(abi.make_params(p, st_check_interval=1), p.dt(), 0, steps)
    np.savez_compressed(os.path.join(HERE, "couette_caidvm_3steps.npz"), n=n, nv=nv, steps=steps,
                        f=st.f, w=st.w, prim=st.prim, qf=st.qf)


if __name__ == "__main__":
    main()
