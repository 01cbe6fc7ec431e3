"""Writes tests/golden/oracle_small.npz: small seeded cases computed by the CPU oracle.

The reference (dineshadepu/prestige) has no numeric path and no golden data, so these
fixtures are not reference outputs: they pin the oracle itself (its results must not drift
between builds, compilers or the x86 and Arm hosts) and give the GPU tests a stored target.
Every case is generated from the seeded workloads of prestige_gb300.workloads:
  lattice_*   3D jittered lattice, 1,000 particles: cell list, neighbour counts, SPH rates
              (f64), and the state after 5 SPH steps (f64 and f32)
  dam_*       2D dam break at dx = 0.1 (fluid + 3 wall layers): state after 5 steps
  dem_*       3D compressed sphere lattice (4 x 4 x 4): state after 10 steps, contact count
  dual_*      dual-number L, dL/dalpha, dL/dB, <dL/dv0, u> of a 512-particle run, 4 steps
Run:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import py_oracle  # noqa: E402
from prestige_gb300 import workloads  # noqa: E402

OUT = os.path.join(HERE, "oracle_small.npz")


def cases():
    out = {}
    w = workloads.sph_lattice_3d(n=1000, seed=2)
    cfg, f = w["config"], w["fields"]
    support = 2.0 * cfg["h"]
    cell, sid, start = py_oracle.cell_list(f["pos"], cfg["domain_lo"], cfg["domain_hi"], support)
    out["lattice_cell"], out["lattice_sorted_id"], out["lattice_cell_start"] = cell, sid, start
    out["lattice_counts"] = py_oracle.neighbor_counts(f["pos"], cfg["domain_lo"], cfg["domain_hi"], support)
    st = py_oracle.SphState(f["pos"], f["vel"], f["rho"], f["mass"])
    out["lattice_acc"], out["lattice_drho"] = py_oracle.sph_rates(cfg, st)
    py_oracle.sph_run(cfg, st, 5)
    out["lattice_pos5"], out["lattice_vel5"], out["lattice_rho5"] = st.pos, st.vel, st.rho
    st32 = py_oracle.SphState(f["pos"], f["vel"], f["rho"], f["mass"], f64=False)
    py_oracle.sph_run(dict(cfg, precision=0), st32, 5)
    out["lattice_pos5_f32"], out["lattice_rho5_f32"] = st32.pos, st32.rho
    w = workloads.dam_break_2d(dx=0.1)
    st = py_oracle.SphState(w["fields"]["pos"], w["fields"]["vel"], w["fields"]["rho"], w["fields"]["mass"])
    py_oracle.sph_run(w["config"], st, 5)
    out["dam_pos5"], out["dam_vel5"], out["dam_rho5"] = st.pos, st.vel, st.rho
    w = workloads.dem_compressed_lattice(nside=4)
    f = w["fields"]
    ds = py_oracle.DemState(f["pos"], f["vel"], f["omega"], f["radius"], f["mass"], 16)
    c, _ = py_oracle.dem_run(w["config"], ds, 10)
    out["dem_pos10"], out["dem_vel10"], out["dem_omega10"] = ds.pos, ds.vel, ds.omega
    out["dem_contacts10"] = np.array([c])
    w = workloads.differentiable_3d(n=512, seed=4, target_seed=5)
    f = w["fields"]
    st = py_oracle.SphState(f["pos"], f["vel"], f["rho"], f["mass"])
    u = np.random.default_rng(7).normal(size=f["vel"].shape)
    out["dual_4"] = py_oracle.sph_grad_dual(w["config"], st, u, w["target"], 4)
    return out


if __name__ == "__main__":
    np.savez_compressed(OUT, **cases())
    print(OUT, os.path.getsize(OUT), "bytes")
