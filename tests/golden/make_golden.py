"""Generate the golden fixtures in this folder from the REFERENCE itself.

Runs the unmodified reference FMM (tbenthompson/3bem cpp/, compiled from its
own sources into oracle/_ref by oracle/ref/Makefile) through its C shim on
small seeded inputs, and stores inputs, reference outputs, the reference's
check-to-equivalent operators, trees and task lists.  The GPU tests compare
the product against these without needing the reference checkout.

    python tests/golden/make_golden.py [<reference checkout>] [all|2d|nearfield|icosphere15k|interior]

(the checkout defaults to $TBEM_REFERENCE_ROOT, else a `reference` folder
beside this repository)

("2d" writes only the 2D fixtures: fmm_*2_*.npz and kernels_2d.npz;
"nearfield" only the nearfield / farfield-correction matrices,
nearfield_*.npz, made by the reference's own construction with the
restated GTEngine queries of oracle/ref/gte_restated.cpp.)

The reference's LAPACK (scipy's OpenBLAS) is run single-threaded so that
the stored operators are reproducible.
"""
import os
import sys

os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
os.environ.setdefault("OMP_NUM_THREADS", "4")

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "3bem_gb300"))

import numpy as np  # noqa: E402

from oracle import oracle  # noqa: E402
from tbempy import meshes  # noqa: E402

# (name, kernel, n_src, n_obs (0 = same points), order, leaf, small_cells, seed, geometry)
CASES = [
    ("laps_cube", "LaplaceSingle", 600, 0, 35, 20, False, 1, "cube"),
    ("laps_cube_small", "LaplaceSingle", 600, 0, 35, 20, True, 2, "cube"),
    ("lapd_cube", "LaplaceDouble", 600, 0, 35, 20, False, 3, "cube"),
    ("eldisp_cube", "ElasticDisplacement", 400, 0, 12, 20, False, 4, "cube"),
    ("eltrac_cube_small", "ElasticTraction", 400, 0, 12, 20, True, 5, "cube"),
    ("eladj_cube", "ElasticAdjointTraction", 400, 0, 12, 20, False, 6, "cube"),
    ("laps_two_sets", "LaplaceSingle", 500, 300, 35, 20, False, 7, "cube"),
    ("laps_sphere", "LaplaceSingle", 960, 0, 35, 30, False, 8, "sphere2"),
    ("eldisp_fault", "ElasticDisplacement", 1536, 0, 12, 64, False, 9, "fault16"),
]

# 2D operators (FMMOperator<2,1,1> / <2,2,2>): points [n][2]
CASES_2D = [
    ("laps2_square", "LaplaceSingle", 600, 0, 20, 20, False, 11, "square"),
    ("lapd2_square_small", "LaplaceDouble", 600, 0, 20, 20, True, 12, "square"),
    ("laph2_two_sets", "LaplaceHypersingular", 500, 300, 20, 20, False, 13, "square"),
    ("eldisp2_square", "ElasticDisplacement", 400, 0, 12, 20, False, 14, "square"),
    ("eltrac2_square_small", "ElasticTraction", 400, 0, 12, 20, True, 15, "square"),
    ("eladj2_square", "ElasticAdjointTraction", 400, 0, 12, 20, False, 16, "square"),
    ("elhyp2_square", "ElasticHypersingular", 400, 0, 16, 20, False, 17, "square"),
    ("laps2_circle", "LaplaceSingle", 1024, 0, 20, 30, False, 18, "circle"),
]


def points(geom, n, seed):
    rng = np.random.default_rng(seed)
    if geom == "square":
        locs = rng.uniform(0, 1, (n, 2))
        nrm = rng.normal(size=(n, 2))
        nrm /= np.linalg.norm(nrm, axis=1)[:, None]
        w = rng.uniform(0.5, 1.0, n)
        return locs, nrm, w
    if geom == "circle":
        # midpoints of n equal segments of the unit circle, outward normals
        t = 2 * np.pi * (np.arange(n) + 0.5) / n
        nrm = np.stack([np.cos(t), np.sin(t)], axis=1)
        return nrm.copy(), nrm, np.full(n, 2 * np.pi / n)
    if geom == "cube":
        locs = rng.uniform(0, 1, (n, 3))
        nrm = rng.normal(size=(n, 3))
        nrm /= np.linalg.norm(nrm, axis=1)[:, None]
        w = rng.uniform(0.5, 1.0, n)
        return locs, nrm, w
    if geom == "sphere2":
        return meshes.sphere_points(2)
    if geom == "fault16":
        l, nn, w, _ = meshes.fault_points(16)
        return l, nn, w
    raise ValueError(geom)


def make_case(name, kernel, n_src, n_obs, order, leaf, small, seed, geom):
    locs, nrm, w = points(geom, n_src, seed)
    if n_obs:
        ol, on, _ = points("square" if locs.shape[1] == 2 else "cube", n_obs, seed + 100)
    else:
        ol, on = locs, nrm
    ref = oracle.RefFMM(kernel, ol, on, locs, nrm, w, 0.3, order, leaf, 0.05, small)
    R = ref.R
    rng = np.random.default_rng(seed + 1000)
    x = rng.uniform(-1, 1, R * len(locs))
    out = dict(kernel=kernel, order=order, leaf=leaf, small=int(small), mac=0.3, d=0.05,
               obs_locs=ol, obs_normals=on, src_locs=locs, src_normals=nrm, src_weights=w,
               x=x, y_ref=ref.apply(x),
               y_direct=oracle.direct(kernel, ol, on, locs, nrm, w, x),
               n_surf=ref.n_surf())
    for which in (0, 1):
        t = ref.tree(which)
        for k in ("level", "index", "center", "hw", "n_idx", "n_children"):
            out["tree%d_%s" % (which, k)] = t[k]
        out["tree%d_indices" % which] = np.concatenate(t["indices"])
        nl = ref.n_levels(which)
        out["c2e%d" % which] = np.stack([ref.c2e(which, lev) for lev in range(nl)])
    for kind in oracle.LISTS:
        a, b = ref.list(kind)
        out["list_%s_obs" % kind] = a
        out["list_%s_src" % kind] = b
    return out


def make_icosphere15k():
    """The plain FP64 Laplace single-layer workload at its stated size: an
    icosahedron subdivided 4 times (5,120 triangles, radius 1), 3 Gauss points
    per triangle (15,360 points, obs = src), weights area / 3, outward normals,
    density uniform[-1, 1] from seed 0; "order 6" read as 6 (6 - 1)^2 + 2 =
    152 requested surface points, MAC 0.3, 50 points per leaf, d = 0.05.
    Stores the reference's apply, its pseudo-inverses, trees, lists, its
    one-ulp sensitivity and the FP64 direct sum."""
    locs, nrm, w = meshes.sphere_points(4)
    x = np.random.default_rng(0).uniform(-1, 1, len(locs))
    ref = oracle.RefFMM("LaplaceSingle", locs, nrm, locs, nrm, w, 0.3, 152, 50, 0.05, False)
    out = dict(kernel="LaplaceSingle", order=152, leaf=50, small=0, mac=0.3, d=0.05,
               obs_locs=locs, obs_normals=nrm, src_locs=locs, src_normals=nrm, src_weights=w,
               x=x, y_ref=ref.apply(x), n_surf=ref.n_surf(),
               y_direct=oracle.direct("LaplaceSingle", locs, nrm, locs, nrm, w, x))
    for which in (0, 1):
        t = ref.tree(which)
        for k in ("level", "index", "n_idx", "n_children"):
            out["tree%d_%s" % (which, k)] = t[k].astype(np.int32)
        for k in ("center", "hw"):
            out["tree%d_%s" % (which, k)] = t[k]
        out["tree%d_indices" % which] = np.concatenate(t["indices"]).astype(np.int32)
        out["c2e%d" % which] = np.stack([ref.c2e(which, lev) for lev in range(ref.n_levels(which))])
    for kind in oracle.LISTS:
        a, b = ref.list(kind)
        out["list_%s_obs" % kind] = a.astype(np.int32)
        out["list_%s_src" % kind] = b.astype(np.int32)
    orc = oracle.OracleFMM("LaplaceSingle", locs, nrm, locs, nrm, w, 0.3, 152, 50, 0.05, False)
    out["ulp_floor"] = orc.ulp_floor(x)
    return out


def kernel_vectors():
    """Reference kernel tensors at seeded random configurations."""
    rng = np.random.default_rng(42)
    rows = []
    for k in range(6):
        for _ in range(40):
            obs, src = rng.uniform(-1, 1, 3), rng.uniform(-1, 1, 3)
            no, ns = rng.normal(size=3), rng.normal(size=3)
            no /= np.linalg.norm(no)
            ns /= np.linalg.norm(ns)
            mu, nu = rng.uniform(0.5, 40.0), rng.uniform(0.1, 0.45)
            K = oracle.kernel_tensor(k, obs, src, no, ns, mu, nu, lib="ref")
            rows.append(np.concatenate([[k, mu, nu], obs, src, no, ns, np.pad(K.ravel(), (0, 9 - K.size))]))
    # the self-pair rule: r^2 < 1e-12 gives a zero tensor
    for k in range(6):
        p = rng.uniform(-1, 1, 3)
        K = oracle.kernel_tensor(k, p, p + 1e-7, np.array([1.0, 0, 0]), np.array([0, 1.0, 0]),
                                 1.0, 0.25, lib="ref")
        rows.append(np.concatenate([[k, 1.0, 0.25], p, p + 1e-7, [1, 0, 0], [0, 1, 0],
                                    np.pad(K.ravel(), (0, 9 - K.size))]))
    # the hypersingular kernel (id 6), its own seed so the rows above stay put
    rng6 = np.random.default_rng(43)
    for _ in range(40):
        obs, src = rng6.uniform(-1, 1, 3), rng6.uniform(-1, 1, 3)
        no, ns = rng6.normal(size=3), rng6.normal(size=3)
        no /= np.linalg.norm(no)
        ns /= np.linalg.norm(ns)
        mu, nu = rng6.uniform(0.5, 40.0), rng6.uniform(0.1, 0.45)
        K = oracle.kernel_tensor(6, obs, src, no, ns, mu, nu, lib="ref")
        rows.append(np.concatenate([[6, mu, nu], obs, src, no, ns, K.ravel()]))
    p = rng6.uniform(-1, 1, 3)
    K = oracle.kernel_tensor(6, p, p + 1e-7, np.array([1.0, 0, 0]), np.array([0, 1.0, 0]), 1.0, 0.25,
                             lib="ref")
    rows.append(np.concatenate([[6, 1.0, 0.25], p, p + 1e-7, [1, 0, 0], [0, 1, 0], K.ravel()]))
    return np.array(rows)


def kernel_vectors_2d():
    """Reference 2D kernel tensors (ids 16-23) at seeded random configurations,
    the same row layout as kernel_vectors with z = 0 everywhere."""
    rng = np.random.default_rng(44)
    rows = []
    for k in range(16, 24):
        for _ in range(40):
            obs, src = rng.uniform(-1, 1, 2), rng.uniform(-1, 1, 2)
            no, ns = rng.normal(size=2), rng.normal(size=2)
            no /= np.linalg.norm(no)
            ns /= np.linalg.norm(ns)
            mu, nu = rng.uniform(0.5, 40.0), rng.uniform(0.1, 0.45)
            K = oracle.kernel_tensor(k, obs, src, no, ns, mu, nu, lib="ref")
            z = [0.0]
            rows.append(np.concatenate([[k, mu, nu], obs, z, src, z, no, z, ns, z,
                                        np.pad(K.ravel(), (0, 9 - K.size))]))
        p = rng.uniform(-1, 1, 2)
        K = oracle.kernel_tensor(k, p, p + 1e-7, np.array([1.0, 0]), np.array([0, 1.0]), 1.0, 0.25,
                                 lib="ref")
        rows.append(np.concatenate([[k, 1.0, 0.25], p, [0], p + 1e-7, [0], [1, 0, 0], [0, 1, 0],
                                    np.pad(K.ravel(), (0, 9 - K.size))]))
    return np.array(rows)


def nearfield_meshes():
    """Small seeded meshes for the nearfield fixtures: an icosphere, a dipping
    fault, a folded wedge (3D), a circle and a V-shaped wedge (2D)."""
    ico_v, ico_f = meshes.icosphere(1)
    flt_v, flt_f, _ = meshes.dipping_fault(4)
    wedge_v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0], [0, 0.1, 0.2], [1, 0.1, 0.2]], float)
    wedge_f = np.array([[0, 1, 2], [1, 3, 2], [0, 4, 1], [1, 4, 5]])
    n = 40
    t = 2 * np.pi * np.arange(n) / n
    circ_v = np.stack([np.cos(t), np.sin(t)], axis=1)
    circ_f = np.stack([np.arange(n), (np.arange(n) + 1) % n], axis=1)
    vw_v = np.array([[-1, 1], [-0.5, 0.5], [0, 0], [0.5, 0.5], [1, 1], [0.2, 0.05]], float)
    vw_f = np.array([[0, 1], [1, 2], [2, 3], [3, 4], [2, 5]])
    return {"ico": (ico_v, ico_f), "fault": (flt_v, flt_f), "wedge": (wedge_v, wedge_f),
            "circle": (circ_v, circ_f), "vwedge": (vw_v, vw_f)}


# (name, mesh, kernel, mu, nu, sinh_order, obs_near, obs_far, src_far, steps, far_threshold)
NEARFIELD_CASES = [
    ("lapd_ico", "ico", "LaplaceDouble", 1.0, 0.25, 5, 2, 2, 2, 8, 3.0),
    ("laps_wedge", "wedge", "LaplaceSingle", 1.0, 0.25, 4, 3, 2, 3, 6, 3.0),
    ("eltrac_fault", "fault", "ElasticTraction", 1.0, 0.25, 4, 2, 2, 3, 6, 3.0),
    ("elhyp_fault", "fault", "ElasticHypersingular", 30.0, 0.25, 4, 2, 2, 2, 6, 3.0),
    ("laps2_circle", "circle", "LaplaceSingle", 1.0, 0.25, 12, 3, 3, 3, 8, 3.0),
    ("eldisp2_vwedge", "vwedge", "ElasticDisplacement", 1.0, 0.25, 8, 3, 2, 3, 8, 3.0),
    ("elhyp2_circle", "circle", "ElasticHypersingular", 1.0, 0.3, 10, 2, 2, 3, 8, 3.0),
]


# the adaptive Gauss-Lobatto strategy (make_adaptive_integrator): (name, mesh,
# kernel, mu, nu, near_tol, obs_near, obs_far, src_far, steps, far_threshold)
ADAPTIVE_CASES = [
    ("adapt_laps_wedge", "wedge", "LaplaceSingle", 1.0, 0.25, 1e-4, 2, 2, 3, 6, 3.0),
    ("adapt_lapd_ico", "ico", "LaplaceDouble", 1.0, 0.25, 1e-4, 2, 2, 3, 6, 3.0),
    ("adapt_eltrac_fault", "fault", "ElasticTraction", 1.0, 0.25, 1e-4, 2, 2, 3, 6, 3.0),
    ("adapt_laps2_circle", "circle", "LaplaceSingle", 1.0, 0.25, 1e-5, 2, 2, 3, 6, 3.0),
    ("adapt_eldisp2_vwedge", "vwedge", "ElasticDisplacement", 1.0, 0.25, 1e-5, 2, 2, 3, 6, 3.0),
]


def make_nearfield_cases():
    ms = nearfield_meshes()
    cases = [(c, "sinh", 0.0) for c in NEARFIELD_CASES]
    cases += [((n, m, k, mu, nu, 0) + tuple(rest), "adaptive", tol)
              for n, m, k, mu, nu, tol, *rest in ADAPTIVE_CASES]
    for (name, mesh, kernel, mu, nu, so, on, of, sf, st, ft), strategy, tol in cases:
        v, f = ms[mesh]
        out = dict(kernel=kernel, mu=mu, nu=nu, vertices=v, facets=f, sinh_order=so,
                   obs_near_order=on, obs_far_order=of, src_far_order=sf, n_singular_steps=st,
                   far_threshold=ft, strategy=strategy, near_tol=tol)
        # the reference's own sensitivity: its matrix again with every vertex
        # coordinate moved by one ulp (random sign), max |change| / max |entry|
        vp = v * (1 + 2.0 ** -52 * np.random.default_rng(0).choice([-1, 1], size=v.shape))
        for which in (0, 1):
            nr, nc, vals, cols, rows = oracle.ref_nearfield(
                kernel, v, f, strategy, tol, so, on, of, sf, st, ft, which, mu, nu)
            out["shape%d" % which] = np.array([nr, nc])
            out["values%d" % which] = vals
            out["cols%d" % which] = cols
            out["rowptr%d" % which] = rows
            pr, pc, pv, pcols, prows = oracle.ref_nearfield(
                kernel, vp, f, strategy, tol, so, on, of, sf, st, ft, which, mu, nu)
            a = np.zeros((nr, nc))
            b = np.zeros((pr, pc))
            for r in range(nr):
                np.add.at(a[r], cols[rows[r]:rows[r + 1]], vals[rows[r]:rows[r + 1]])
                np.add.at(b[r], pcols[prows[r]:prows[r + 1]], pv[prows[r]:prows[r + 1]])
            out["ulp_floor%d" % which] = np.abs(a - b).max() / np.abs(a).max()
        loc, nrm, dirs = oracle.ref_obs_points(v, f, on)
        out["obs_loc"], out["obs_dir"] = loc, dirs
        np.savez_compressed(os.path.join(HERE, "nearfield_%s.npz" % name), **out)
        print("wrote nearfield", name, out["shape0"], len(out["values0"]), len(out["values1"]))


def _dense(nr, nc, vals, cols, rows):
    a = np.zeros((nr, nc))
    for r in range(nr):
        np.add.at(a[r], cols[rows[r]:rows[r + 1]], vals[rows[r]:rows[r + 1]])
    return a


def make_interior_cases():
    """dense_interior_operator's nearfield / correction for given points (on the
    surface, just off it, inside, far) and the mass operators, from the
    reference; plus the reference's one-ulp sensitivity as for the nearfield."""
    ms = nearfield_meshes()
    rng = np.random.default_rng(21)
    cases = [("lapd_ico", "ico", "LaplaceDouble", 1.0, 0.25, 5, 2, 2, 2, 8, 3.0),
             ("laps2_circle", "circle", "LaplaceSingle", 1.0, 0.25, 10, 2, 2, 3, 8, 3.0)]
    for name, mesh, kernel, mu, nu, so, on, of, sf, st, ft in cases:
        v, f = ms[mesh]
        dim = v.shape[1]
        loc, nrm, _ = oracle.ref_obs_points(v, f, 2)
        loc, nrm = loc[:, :dim], nrm[:, :dim]
        pts = np.concatenate([loc[:8], loc[8:16] * (1 + 1e-4), loc[16:24] * 0.97,
                              rng.normal(size=(6, dim)) * 0.3, rng.normal(size=(4, dim)) * 3])
        nrms = np.concatenate([nrm[:24], np.tile(np.eye(dim)[:1], (10, 1))])
        out = dict(kernel=kernel, mu=mu, nu=nu, vertices=v, facets=f, sinh_order=so,
                   obs_near_order=on, obs_far_order=of, src_far_order=sf, n_singular_steps=st,
                   far_threshold=ft, locs=pts, normals=nrms,
                   dirs=oracle.ref_interior_dirs(pts, v, f)[:, :dim])
        vp = v * (1 + 2.0 ** -52 * np.random.default_rng(0).choice([-1, 1], size=v.shape))
        for which in (0, 1):
            res = oracle.ref_nearfield_points(kernel, v, f, pts, nrms, so, on, of, sf, st, ft, which,
                                              mu, nu)
            out["shape%d" % which] = np.array(res[:2])
            out["values%d" % which], out["cols%d" % which], out["rowptr%d" % which] = res[2:]
            pr = oracle.ref_nearfield_points(kernel, vp, f, pts, nrms, so, on, of, sf, st, ft, which,
                                             mu, nu)
            a, b = _dense(*res), _dense(*pr)
            out["ulp_floor%d" % which] = np.abs(a - b).max() / max(np.abs(a).max(), 1e-300)
        # the reference's whole operator (nearfield + correction + interpolated
        # direct farfield), its apply to a seeded density, and that apply's
        # one-ulp sensitivity (the same vertex perturbation)
        args = (so, on, of, sf, st, ft, mu, nu)
        A = oracle.ref_dense_interior(kernel, v, f, pts, nrms, *args)
        Ap = oracle.ref_dense_interior(kernel, vp, f, pts, nrms, *args)
        x = np.random.default_rng(3).uniform(-1, 1, A.shape[1])
        out["dense"], out["apply_x"], out["apply_y"] = A, x, A @ x
        out["apply_ulp_floor"] = np.linalg.norm(A @ x - Ap @ x) / np.linalg.norm(A @ x)
        for R in sorted({1, dim}):
            for nq in (2, 3):
                res = oracle.ref_mass(v, f, R, nq)
                out["mass_%d_%d_shape" % (R, nq)] = np.array(res[:2])
                (out["mass_%d_%d_values" % (R, nq)], out["mass_%d_%d_cols" % (R, nq)],
                 out["mass_%d_%d_rowptr" % (R, nq)]) = res[2:]
        np.savez_compressed(os.path.join(HERE, "interior_%s.npz" % name), **out)
        print("wrote interior", name, out["shape0"], len(out["values0"]), out["ulp_floor0"])


def make_dense_boundary_cases():
    """The reference's dense_boundary_operator (sinh strategy) of two small
    meshes, with its one-ulp sensitivity."""
    ms = nearfield_meshes()
    cases = [("lapd_ico", "ico", "LaplaceDouble", 1.0, 0.25, 5, 3, 3, 3, 8, 3.0),
             ("eltrac2_circle", "circle", "ElasticTraction", 1.0, 0.25, 8, 3, 3, 3, 8, 3.0)]
    for name, mesh, kernel, mu, nu, so, on, of, sf, st, ft in cases:
        v, f = ms[mesh]
        A = oracle.ref_dense_boundary(kernel, v, f, so, on, of, sf, st, ft, mu, nu)
        vp = v * (1 + 2.0 ** -52 * np.random.default_rng(0).choice([-1, 1], size=v.shape))
        B = oracle.ref_dense_boundary(kernel, vp, f, so, on, of, sf, st, ft, mu, nu)
        np.savez_compressed(os.path.join(HERE, "dense_boundary_%s.npz" % name), kernel=kernel, mu=mu,
                            nu=nu, vertices=v, facets=f, sinh_order=so, obs_near_order=on,
                            obs_far_order=of, src_far_order=sf, n_singular_steps=st,
                            far_threshold=ft, matrix=A,
                            ulp_floor=np.abs(A - B).max() / np.abs(A).max())
        print("wrote dense boundary", name, A.shape, np.abs(A - B).max() / np.abs(A).max())


def main(ref_root=None, which="all"):
    ref_root = ref_root or oracle.REF_ROOT
    oracle.build()
    if oracle.build_ref(ref_root) is None:
        raise SystemExit("the reference checkout is needed to regenerate the fixtures")
    if which == "icosphere15k":
        data = make_icosphere15k()
        np.savez_compressed(os.path.join(HERE, "fmm_laps_icosphere15k.npz"), **data)
        print("wrote laps_icosphere15k", len(data["x"]), "points, ulp floor %.3g" % data["ulp_floor"])
        return
    if which == "interior":
        make_interior_cases()
        return
    if which == "nearfield":
        make_nearfield_cases()
        make_interior_cases()
        make_dense_boundary_cases()
        return
    for case in CASES_2D:
        data = make_case(*case)
        np.savez_compressed(os.path.join(HERE, "fmm_%s.npz" % case[0]), **data)
        print("wrote", case[0], {k: v.shape for k, v in data.items() if hasattr(v, "shape") and v.ndim})
    circ = {str(o): oracle.RefFMM("LaplaceSingle", np.zeros((1, 2)), np.zeros((1, 2)),
                                  np.zeros((1, 2)), np.zeros((1, 2)), np.ones(1), 0.3, o, 1,
                                  0.05, False).n_surf() for o in (1, 4, 12, 20, 64)}
    np.savez_compressed(os.path.join(HERE, "kernels_2d.npz"), rows=kernel_vectors_2d(),
                        surf_orders=np.array([int(k) for k in circ]),
                        surf_counts=np.array(list(circ.values())),
                        surf4=oracle.surface(4, 2, lib="ref"))
    if which == "2d":
        return
    for case in CASES:
        data = make_case(*case)
        np.savez_compressed(os.path.join(HERE, "fmm_%s.npz" % case[0]), **data)
        print("wrote", case[0], {k: v.shape for k, v in data.items() if hasattr(v, "shape") and v.ndim})
    np.savez_compressed(os.path.join(HERE, "kernels.npz"), rows=kernel_vectors())
    surf = {str(o): oracle.RefFMM("LaplaceSingle", np.zeros((1, 3)), np.zeros((1, 3)),
                                  np.zeros((1, 3)), np.zeros((1, 3)), np.ones(1), 0.3, o, 1,
                                  0.05, False).n_surf() for o in (1, 6, 8, 20, 35, 75, 100, 152, 296)}
    # the octree of the reference's degenerate-line test (unit_tests/test_octree.cpp:144-155),
    # restated in 3D: points i and i + 1 on the x axis, one point per cell
    line = np.array([[float(i), 0.0, 0.0] for i in range(10)] +
                    [[float(i + 1), 0.0, 0.0] for i in range(10)])
    ref = oracle.RefFMM("LaplaceSingle", line, np.ones_like(line), line, np.ones_like(line),
                        np.ones(len(line)), 0.3, 6, 1, 0.05, False)
    t = ref.tree(0)
    np.savez_compressed(os.path.join(HERE, "misc.npz"),
                        surf_orders=np.array([int(k) for k in surf]),
                        surf_counts=np.array(list(surf.values())),
                        line_pts=line, line_n_cells=len(t["level"]),
                        line_levels=t["level"], line_n_idx=t["n_idx"])
    print("surface counts", surf, "line cells", len(t["level"]))


if __name__ == "__main__":
    main(*sys.argv[1:])
