"""Writes tests/golden/oracle_small.npz: small seeded cases and the CPU oracle's results on them.

The reference (dineshadepu/prestige) has no numeric path and no golden data, so these
fixtures are not reference outputs: they pin the oracle itself (its results must not drift
between builds, compilers or the x86 and Arm hosts) and give the GPU tests a stored target.
Inputs are stored with the results: the seeded generators use numpy's transcendental functions
(the dam break's hydrostatic density), which may differ by an ulp between hosts, so the
checks start from the stored arrays rather than from regenerated ones.
Cases (generated from prestige_gb300.workloads):
  lattice   3D jittered lattice, 1,000 particles: cell list, neighbour counts, SPH rates (f64),
            state after 5 SPH steps (f64 and f32)
  dam       2D dam break at dx = 0.1 (fluid + 3 wall layers): state after 5 steps
  dem       3D compressed sphere lattice (4 x 4 x 4): state after 10 steps, contact count
  dual      dual-number L, dL/dalpha, dL/dB, <dL/dv0, u> of a 512-particle run, 4 steps
Run:  python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import py_oracle  # noqa: E402

OUT = os.path.join(HERE, "oracle_small.npz")


def inputs():
    """The cases' configurations and input arrays, from the seeded workload generators."""
    from prestige_gb300 import workloads
    lat = workloads.sph_lattice_3d(n=1000, seed=2)
    dam = workloads.dam_break_2d(dx=0.1)
    dem = workloads.dem_compressed_lattice(nside=4)
    dif = workloads.differentiable_3d(n=512, seed=4, target_seed=5)
    cfgs = {"lattice": lat["config"], "dam": dam["config"], "dem": dem["config"], "dual": dif["config"]}
    arrays = {}
    for name, w in (("lattice", lat), ("dam", dam), ("dem", dem), ("dual", dif)):
        for k, v in w["fields"].items():
            arrays["%s_in_%s" % (name, k)] = np.asarray(v)
    arrays["dual_in_target"] = dif["target"]
    arrays["dual_in_u"] = np.random.default_rng(7).normal(size=dif["fields"]["vel"].shape)
    return cfgs, arrays


def results(cfgs, a):
    """The oracle's results from stored inputs (the function the tests rerun)."""
    out = {}
    cfg = cfgs["lattice"]
    pos, vel, rho, mass = (a["lattice_in_" + k] for k in ("pos", "vel", "rho", "mass"))
    support = 2.0 * cfg["h"]
    cell, sid, start = py_oracle.cell_list(pos, cfg["domain_lo"], cfg["domain_hi"], support)
    out["lattice_cell"], out["lattice_sorted_id"], out["lattice_cell_start"] = cell, sid, start
    out["lattice_counts"] = py_oracle.neighbor_counts(pos, cfg["domain_lo"], cfg["domain_hi"], support)
    st = py_oracle.SphState(pos, vel, rho, mass)
    out["lattice_acc"], out["lattice_drho"] = py_oracle.sph_rates(cfg, st)
    py_oracle.sph_run(cfg, st, 5)
    out["lattice_pos5"], out["lattice_vel5"], out["lattice_rho5"] = st.pos, st.vel, st.rho
    st32 = py_oracle.SphState(pos, vel, rho, mass, f64=False)
    py_oracle.sph_run(dict(cfg, precision=0), st32, 5)
    out["lattice_pos5_f32"], out["lattice_rho5_f32"] = st32.pos, st32.rho
    st = py_oracle.SphState(*(a["dam_in_" + k] for k in ("pos", "vel", "rho", "mass")))
    py_oracle.sph_run(cfgs["dam"], st, 5)
    out["dam_pos5"], out["dam_vel5"], out["dam_rho5"] = st.pos, st.vel, st.rho
    cap = cfgs["dem"]["contact_capacity"]
    ds = py_oracle.DemState(*(a["dem_in_" + k] for k in ("pos", "vel", "omega", "radius", "mass")), cap)
    c, _ = py_oracle.dem_run(cfgs["dem"], ds, 10)
    out["dem_pos10"], out["dem_vel10"], out["dem_omega10"] = ds.pos, ds.vel, ds.omega
    out["dem_contacts10"] = np.array([c])
    st = py_oracle.SphState(*(a["dual_in_" + k] for k in ("pos", "vel", "rho", "mass")))
    out["dual_4"] = py_oracle.sph_grad_dual(cfgs["dual"], st, a["dual_in_u"], a["dual_in_target"], 4)
    return out


if __name__ == "__main__":
    cfgs, arrays = inputs()
    res = results(cfgs, arrays)
    np.savez_compressed(OUT, configs=np.array(json.dumps(cfgs, sort_keys=True)), **arrays, **res)
    print(OUT, os.path.getsize(OUT), "bytes")
