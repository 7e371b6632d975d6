"""Writes the golden fixtures of tests/test_golden.py and
tests/test_gpu_golden.py: small seeded meshes and one pressure operator
computed by the CPU oracle (oracle/lvref.cpp, a restatement of the
reference's algorithms), together with an independent Voronoi of the same
seeds from scipy.spatial (Qhull).  The reference itself (Julia) does not run
here, and its repository holds no golden vectors; these fixtures pin the
oracle against regressions and against Qhull, and give the GPU path fixed
expected values.

Run from the repository root:  python tests/golden/make_golden.py
"""
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))
import lvref  # noqa: E402
import workloads as W  # noqa: E402

spec = importlib.util.spec_from_file_location("populate_golden",
                                              os.path.join(ROOT, "lagrangianvoronoi.jl_gb300", "populate.py"))
pop = importlib.util.module_from_spec(spec)
spec.loader.exec_module(pop)

CASES = {
    # name: (n, jitter, seed, periodic)
    "periodic_12": (12, 0.3, 7, True),
    "walls_10": (10, 0.2, 11, False),
}


def qhull_periodic(x):
    from scipy import spatial
    n = len(x)
    shifts = np.array([(a, b) for b in (-1, 0, 1) for a in (-1, 0, 1)], dtype=float)
    pts = np.concatenate([x + s for s in shifts])
    vor = spatial.Voronoi(pts)
    centre = 4 * n
    pairs = set()
    for (p, q), rv in zip(vor.ridge_points, vor.ridge_vertices):
        if -1 in rv:
            continue
        if np.linalg.norm(vor.vertices[rv[0]] - vor.vertices[rv[1]]) < 1e-12:
            continue
        if centre <= p < centre + n:
            pairs.add((p - centre, q % n))
        if centre <= q < centre + n:
            pairs.add((q - centre, p % n))
    area = np.zeros(n)
    for i in range(n):
        reg = vor.regions[vor.point_region[centre + i]]
        v = vor.vertices[reg]
        c = v.mean(axis=0)
        ang = np.arctan2(v[:, 1] - c[1], v[:, 0] - c[0])
        v = v[np.argsort(ang)]
        area[i] = 0.5 * abs(np.dot(v[:, 0], np.roll(v[:, 1], -1)) - np.dot(v[:, 1], np.roll(v[:, 0], -1)))
    return np.array(sorted(pairs), dtype=np.int64), area


def main():
    for name, (n, jitter, seed, periodic) in CASES.items():
        x = pop.jittered_lattice((0, 1), (0, 1), n, n, jitter, seed)
        g = lvref.OracleGrid((0, 1), (0, 1), 1.0 / n, n * n, xperiodic=periodic, yperiodic=periodic, max_edges=20)
        g.set("x", x)
        assert g.remesh() == 0
        F = g.faces()
        E = g.edges()
        out = dict(x=x, area=E["area"], centroid=E["centroid"], e_counts=E["counts"], e_verts=E["verts"],
                   e_labels=E["labels"], f_rowptr=F["rowptr"], f_nbr=F["nbr"], f_lrr=F["lrr"], f_len=F["len"],
                   f_mid=F["mid"], f_y=F["y"])
        if periodic:
            pairs, qarea = qhull_periodic(x)
            out["qhull_pairs"] = pairs
            out["qhull_area"] = qarea
            # a pressure operator and first-sweep right-hand side on this mesh
            flow = W.taylor_green(n)
            f = W.initial_fields(flow, x, E["area"])
            for k, v in f.items():
                g.set(k, v)
            g.stiffened_eos(flow.gamma, flow.P0)
            op = g.pressure_operator(flow.dt)
            b, gp = g.pressure_rhs(flow.dt, 0)
            out.update(op_diag=op["diag"], op_rowptr=op["rowptr"], op_col=op["col"], op_w=op["w"], rhs_b=b,
                       rhs_gp=gp, dt=np.array([flow.dt]))
        path = os.path.join(HERE, f"mesh_{name}.npz")
        np.savez_compressed(path, **out)
        print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    lvref.build()
    main()
