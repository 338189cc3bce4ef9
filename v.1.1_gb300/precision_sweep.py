"""Mixed-precision (or double-word) error against the plain FP64 path, on the 6M-tet cube.

    python v.1.1_gb300/precision_sweep.py [--cube 100] [--steps 5000] [--every 100] [--vms-every 500]
                                          [--precision mixed|dword]

For each law (St-Venant-Kirchhoff, compressible neo-Hookean) and Poisson ratio
(0.3, 0.45, 0.49) the same seeded mesh and loading run side by side in
MSX_PREC_FP64 and MSX_PREC_MIXED (FP32 element kinematics, stress and B^T P;
FP64 nodal update, J-1, ln J and dt).  Every `every` steps the relative L2
displacement error of the mixed run against the FP64 run is recorded, every
`vms-every` steps the largest von Mises difference relative to the largest
von Mises stress.  Prints one JSON line per (law, nu) and a summary line.
With --precision dword the second run is MSX_PREC_DOUBLE_WORD instead.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import msx  # noqa: E402


def run(n, law, nu, steps, every, vms_every, E=1e6, rho=1000.0, v_top=0.1, ramp=200, precision=msx.MIXED):
    X, conn = msx.mesh_cube(n, 1234, 0.1)
    bcs = msx.cube_bcs(n, v_top, msx.BC_VEL_RAMP, ramp)
    mat = (law, E, nu, rho)
    A = msx.Solver(X, conn, [mat], bcs, 0.0, 1e30, 0.5, max_steps=steps, precision=msx.FP64)
    B = msx.Solver(X, conn, [mat], bcs, 0.0, 1e30, 0.5, max_steps=steps, precision=precision)
    hist, vhist, done = [], [], 0
    t0 = time.time()
    while done < steps:
        k = min(every, steps - done)
        ra, rb = A.run(k), B.run(k)
        done += ra.steps
        if ra.steps != k or rb.steps != k:
            raise RuntimeError("run stopped early: %s %s" % (ra, rb))
        ua, ub = A.state()[0], B.state()[0]
        hist.append((done, float(np.linalg.norm(ub - ua) / max(np.linalg.norm(ua), 1e-300))))
        if done % vms_every == 0 or done == steps:
            va, vb = A.element_fields()[2], B.element_fields()[2]
            vhist.append((done, float(np.abs(vb - va).max() / max(np.abs(va).max(), 1e-300))))
    A.close()
    B.close()
    return {"law": {msx.STVK: "St-Venant-Kirchhoff", msx.COMPRESSIBLE_NH: "3D-Compressible-Neo-Hookean",
                    msx.NEO_HOOKEAN: "Neo-Hookean"}[law], "nu": nu, "num_elems": int(conn.shape[0]),
            "steps": steps, "max_rel_l2_u": max(e for _, e in hist), "final_rel_l2_u": hist[-1][1],
            "max_rel_vms": max(e for _, e in vhist), "rel_l2_u_every": hist, "rel_vms_every": vhist,
            "wall_s": time.time() - t0}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--cube", type=int, default=100)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--every", type=int, default=100)
    ap.add_argument("--vms-every", type=int, default=500)
    ap.add_argument("--precision", choices=["mixed", "dword"], default="mixed")
    args = ap.parse_args()
    prec = msx.DOUBLE_WORD if args.precision == "dword" else msx.MIXED
    out = []
    for law in (msx.STVK, msx.COMPRESSIBLE_NH):
        for nu in (0.3, 0.45, 0.49):
            r = run(args.cube, law, nu, args.steps, args.every, args.vms_every, precision=prec)
            r["precision"] = args.precision
            print(json.dumps(r), flush=True)
            out.append(r)
    print(json.dumps({"summary": [{k: r[k] for k in ("law", "nu", "max_rel_l2_u", "final_rel_l2_u", "max_rel_vms")}
                                  for r in out],
                      "worst_rel_l2_u": max(r["max_rel_l2_u"] for r in out)}))


if __name__ == "__main__":
    main()
