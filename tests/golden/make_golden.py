"""Generates the golden fixtures of tests/golden from the CPU oracle.

The Fortran reference cannot be compiled or run where these fixtures were
made (no Fortran compiler), so the fixtures pin the oracle itself: its
tendency and one RK4 step of Williamson case 2 on level-2 and level-3 grids,
and the local-truncation and 5-day error tables of case 2 that the
reference's own harnesses print (swm_horiz_loc_trunc_er, swm.f90:382-734;
swm_tests error table, swm.f90:2922-2990).  The tests compare fresh oracle
and GPU results with these files, on this machine and on the GPU host.

Run from the repository root:  python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from imodel_gb300 import _build, swm  # noqa: E402
from imodel_gb300.mesh import meshbuild  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
LTE_FIELDS = [("h_ed", 6), ("ke", 0), ("q_tr", 1), ("q_ed", 6), ("grad_ghbK", 6),
              ("uhq_perp", 6)]


def lte_table(levels):
    out = {}
    for L in levels:
        g = meshbuild(L)
        o = oracle.Oracle(g, 2)
        h, u = swm.initialize_fields_tc2(g)
        o.tendency(h, u)
        ex = swm.tc2_exact_operators(g)
        row = {}
        for name, pos in LTE_FIELDS:
            row[name] = list(o.error_calc(o.field(name), ex[name], pos))
        row["utg"] = list(o.error_calc(o.trsk_tangent(u), ex["utg"], 6))
        out[str(L)] = row
    return out


def run_table(cases):
    out = {}
    for L, dt in cases:
        g = meshbuild(L)
        o = oracle.Oracle(g, 2)
        h, u = swm.initialize_fields_tc2(g)
        n = swm.ntime_for(5.0, dt)
        h1, u1 = o.run(h, u, dt, n)
        out[str(L)] = {"dt": dt, "ntime": n, "h": list(o.error_calc(h1, h, 0)),
                       "u": list(o.error_calc(u1, u, 6))}
    return out


def main():
    _build.build_mesh_lib()
    oracle.build()
    with open(os.path.join(HERE, "tc2_tables.json"), "w") as f:
        json.dump({"lte": lte_table([2, 3, 4, 5, 6]),
                   "run5d": run_table([(3, 1800.0), (4, 900.0)])}, f, indent=1)
    for L, dt in [(2, 3600.0), (3, 1800.0)]:
        g = meshbuild(L)
        o = oracle.Oracle(g, 2)
        h, u = swm.initialize_fields_tc2(g)
        m, mo = o.tendency(h, u)
        h1, u1 = o.ode_rk4(h, u, dt)
        np.savez_compressed(os.path.join(HERE, f"tc2_l{L}.npz"), h=h, u=u, masseq=m,
                            momeq=mo, h1=h1, u1=u1, dt=dt,
                            hx_areag=g.hx_areag, ed_leng=g.ed_leng)


if __name__ == "__main__":
    main()
