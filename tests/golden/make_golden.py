"""Generates tests/golden/golden_v1.npz from the CPU restatement (oracle/).

The reference (Fortran + GSL) cannot be built or run in this environment, so the fixtures
are produced by the restatement, whose own pins are checked in tests/test_oracle_pins.py.
Every case is small and seeded; the inputs are stored next to the outputs so the GPU
tests replay exactly the same calls.

    python tests/golden/make_golden.py
"""
import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [REPO, os.path.join(REPO, "oracle")]
import oracle as O  # noqa: E402

pkg = importlib.import_module("2d_dvm_microflows_gb300")
ph = pkg.physics
OUT = os.path.join(HERE, "golden_v1.npz")


def grids():
    return {
        "even8": ph.VelocityGrid.uniform(8, -3.0, 3.0),
        "odd9": ph.VelocityGrid.uniform(9, -4.0, 4.0),
        "stretched": ph.VelocityGrid(np.array([-4.0, -2.5, -1.2, -0.3, 0.4, 1.5, 3.0]),
                                     np.array([-3.0, -1.9, -0.8, 0.1, 0.9, 2.1, 3.2, 4.0]),
                                     np.array([-3.5, -2.0, -0.7, 0.0, 0.6, 1.9, 3.1, 4.2, 5.0])),
    }


def pairlist_case(rng, nv, counts, num_repl, with_nodes=True):
    subs, arrays = [], {}
    for q, n in enumerate(counts):
        d = {"count": n, "num_repl": num_repl,
             "r_phi": rng.random(n * num_repl), "r_cos": rng.random(n * num_repl)}
        if with_nodes:
            d["glA"] = rng.integers(0, nv, n).astype(np.int32)
            d["glB"] = rng.integers(0, nv, n).astype(np.int32)
        else:
            d["rA"] = rng.random(n)
            d["rB"] = rng.random(n)
        subs.append(d)
        for k, v in d.items():
            if isinstance(v, np.ndarray):
                arrays["%s%d" % (k, q)] = v
        arrays["count%d" % q] = np.int64(n)
    return subs, arrays


def main():
    rng = np.random.default_rng(20261203)
    out = {}
    G = grids()
    # 1. remap on three grids, inside, near edges and outside the velocity box
    for name, g in G.items():
        lo = np.array([g.x[0], g.y[0], g.z[0]]) - 0.6
        hi = np.array([g.x[-1], g.y[-1], g.z[-1]]) + 0.6
        pts = rng.uniform(lo, hi, size=(96, 3))
        st = np.zeros((96, 7), np.int32)
        ms = np.zeros((96, 7))
        for t, (u, v, w) in enumerate(pts):
            st[t], ms[t], r = O.remap(g, u, v, w)
            assert r == 0
        out["remap_%s_pts" % name] = pts
        out["remap_%s_st" % name] = st
        out["remap_%s_mass" % name] = ms
    # 2. 0-D VR step from a recorded pair list (node indices), and with partner uniforms
    g = G["even8"]
    f0 = ph.bimodal(g)
    for tag, nodes, method in (("vr_nodes", True, pkg.DVM_COLL_VR),
                               ("vr_uniforms", False, pkg.DVM_COLL_VR),
                               ("fmc_uniforms", False, pkg.DVM_COLL_FMC)):
        counts = (300, 200, 100) if method == pkg.DVM_COLL_VR else (400,)
        subs, arrays = pairlist_case(rng, g.nv, counts, 2, with_nodes=nodes)
        cfg = pkg.DVMConfig(iColl=method, NRepl=2, deltat=0.05, seed=0)
        s = O.OracleSolver(cfg, g)
        s.initialize_dist_func(f0)
        s.compute_collision_integral(step=0, pairs=pkg.PairList(subs))
        out["%s_f1" % tag] = s.phi()[0]
        for k, v in arrays.items():
            out["%s_%s" % (tag, k)] = v
    out["zerod_f0"] = f0
    # 3. 2-D cavity convection (odd grid: zero-velocity nodes), lid moving, partial
    #    accommodation so both wall parts act
    g = G["odd9"]
    nxs, nys = 5, 4
    f2 = np.stack([ph.maxwellian(g, 1.0 + 0.05 * c, 0.1 * (c % 3), -0.05 * (c % 2), 0.0,
                                 1.0 + 0.02 * c) for c in range(nxs * nys)])
    walls = ((1.0, 0.0, 0.0, 0.0, 1.0), (1.0, 0.0, 0.0, 0.0, 1.2),
             (1.0, 0.0, 0.0, 0.0, 1.0), (1.0, 0.3, 0.0, 0.0, 1.0))
    cfg = pkg.DVMConfig(geometry=pkg.DVM_GEOM_2D, nx_space=nxs, ny_space=nys, dx=0.5, dy=0.5,
                        deltat=0.02, iColl=pkg.DVM_COLL_NONE, iConv=pkg.DVM_CONV_UPWIND1,
                        acc_coeff=0.8, walls=walls)
    s = O.OracleSolver(cfg, g)
    s.initialize_dist_func(f2)
    s.compute_convection()
    out["cav_f0"] = f2
    out["cav_f1"] = s.phi()
    s.calculate_physical_properties()
    out["cav_props1"] = s.properties()
    # 4. 1-D convection with diffuse ends
    g = G["even8"]
    n1 = 5
    f1d = np.stack([ph.maxwellian(g, 1.0 + 0.1 * c, -0.2 * c, 0.0, 0.0, 1.0 + 0.05 * c)
                    for c in range(n1)])
    walls = ((1.0, 0.0, 0.0, 0.0, 1.1), (1.0, 0.0, 0.0, 0.0, 0.9), (1, 0, 0, 0, 1), (1, 0, 0, 0, 1))
    cfg = pkg.DVMConfig(geometry=pkg.DVM_GEOM_1D, nx_space=n1, dx=0.4, deltat=0.03,
                        iColl=pkg.DVM_COLL_NONE, iConv=pkg.DVM_CONV_UPWIND1, acc_coeff=0.6,
                        bc=(pkg.DVM_BC1D_DIFFUSE, pkg.DVM_BC1D_DIFFUSE, 0, 0), walls=walls)
    s = O.OracleSolver(cfg, g)
    s.initialize_dist_func(f1d)
    s.compute_convection()
    out["d1_f0"] = f1d
    out["d1_f1"] = s.phi()
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
