"""Seeded synthetic meshes and point sets for the BEM operator apply.

The reference builds point data from a triangle mesh with
``nbody_src_from_bem`` (cpp/nbody_operator.h:56-76): one point per (facet,
quadrature point), weight = w_q * jacobian with jacobian = 2 * area
(cpp/numerics.h:33-35), normal = facet normal.  The workloads here use a
3-point symmetric triangle rule (reference-triangle weights 1/6 each, i.e.
area/3 after the jacobian), which the reference does not ship
(``tri_gauss(n)`` gives n^2 points, cpp/gauss_quad.cpp:124-152).

Generators:
  * ``icosphere(n_subdiv)``  -- icosahedron refined 1->4, vertices projected
    to the unit sphere (5,120 triangles at n_subdiv=4);
  * ``dipping_fault(n, dip)`` -- planar 2 x 2 square dipping ``dip`` degrees,
    an n x n quad grid, each quad split into 2 triangles;
  * ``points_from_mesh`` -- the 3-point rule -> (locs, normals, weights).
"""
import numpy as np

# Barycentric coordinates of the 3-point rule (degree 2, interior points).
_TRI3_BARY = np.array([[2.0 / 3.0, 1.0 / 6.0, 1.0 / 6.0],
                       [1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0],
                       [1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0]])


def icosphere(n_subdiv, radius=1.0, center=(0.0, 0.0, 0.0)):
    """Icosahedron subdivided ``n_subdiv`` times, projected to a sphere.

    Returns (verts [nv,3] float64, tris [nt,3] int64) with outward orientation.
    """
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]],
                 dtype=np.int64)
    verts = [row for row in v]
    for _ in range(n_subdiv):
        cache = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            idx = cache.get(key)
            if idx is None:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                idx = len(verts) - 1
                cache[key] = idx
            return idx

        nf = np.empty((4 * len(f), 3), dtype=np.int64)
        for i, (a, b, c) in enumerate(f):
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf[4 * i + 0] = (a, ab, ca)
            nf[4 * i + 1] = (b, bc, ab)
            nf[4 * i + 2] = (c, ca, bc)
            nf[4 * i + 3] = (ab, bc, ca)
        f = nf
    verts = np.asarray(verts) * radius + np.asarray(center, dtype=np.float64)
    # orient outward: normal . (centroid - center) > 0
    p = verts[f]
    n = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    flip = np.einsum("ij,ij->i", n, p.mean(axis=1) - np.asarray(center)) < 0
    f[flip] = f[flip][:, ::-1]
    return verts, f


def dipping_fault(n, dip_deg=45.0, width=2.0, center=(0.0, 0.0, -1.0)):
    """Planar ``width`` x ``width`` square fault dipping ``dip_deg`` degrees.

    Strike along x; the down-dip direction is (0, cos(dip), -sin(dip)).  The
    n x n quad grid is split into 2 n^2 triangles (diagonal lower-left to
    upper-right).  Returns (verts, tris, uv) with uv in [-1,1]^2 per vertex.
    """
    s = np.linspace(-1.0, 1.0, n + 1)
    u, w = np.meshgrid(s, s, indexing="ij")
    dip = np.deg2rad(dip_deg)
    h = 0.5 * width
    x = h * u
    y = h * w * np.cos(dip)
    z = -h * w * np.sin(dip)
    verts = np.stack([x, y, z], axis=-1).reshape(-1, 3) + np.asarray(center)
    uv = np.stack([u, w], axis=-1).reshape(-1, 2)
    idx = np.arange((n + 1) * (n + 1)).reshape(n + 1, n + 1)
    a = idx[:-1, :-1].ravel()
    b = idx[1:, :-1].ravel()
    c = idx[1:, 1:].ravel()
    d = idx[:-1, 1:].ravel()
    tris = np.concatenate([np.stack([a, b, c], 1), np.stack([a, c, d], 1)])
    return verts, tris.astype(np.int64), uv


def points_from_mesh(verts, tris):
    """3-point rule on every triangle -> (locs [N,3], normals [N,3], weights [N]).

    Point order is facet-major (facet f, point q -> row 3 f + q), matching the
    reference's dof numbering obs_idx * n_quad + q (cpp/nbody_operator.h:62-70).
    """
    p = verts[tris]                                   # [nt, 3, 3]
    cr = np.cross(p[:, 2] - p[:, 0], p[:, 2] - p[:, 1])  # reference unscaled_normal
    nrm = np.linalg.norm(cr, axis=1)
    normals = cr / nrm[:, None]
    area = 0.5 * nrm
    locs = np.einsum("qk,tkd->tqd", _TRI3_BARY, p).reshape(-1, 3)
    normals = np.repeat(normals, 3, axis=0)
    # w_q * jacobian = (1/6) * (2 * area) = area / 3
    weights = np.repeat((1.0 / 6.0) * (2.0 * area), 3)
    return (np.ascontiguousarray(locs), np.ascontiguousarray(normals),
            np.ascontiguousarray(weights))


def sphere_points(n_subdiv=4):
    """Unit icosphere points: 3 per triangle (15,360 at n_subdiv=4)."""
    v, t = icosphere(n_subdiv)
    return points_from_mesh(v, t)


def real_sph_harm(lmax, theta, phi):
    """Real orthonormal spherical harmonics Y_lm(theta, phi) for 0 <= l <= lmax,
    -l <= m <= l (theta the polar angle): a dict {(l, m): values}.  The
    associated Legendre functions come from the standard three-term
    recurrences (P_m^m, P_{m+1}^m, then upward in l), normalised so that
    the Y_lm are orthonormal on the unit sphere."""
    from math import factorial
    x = np.cos(theta)
    s = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    P = {}
    pmm = np.ones_like(x)
    for m in range(lmax + 1):
        if m > 0:
            pmm = -(2 * m - 1) * s * pmm
        P[(m, m)] = pmm
        if m + 1 <= lmax:
            P[(m + 1, m)] = x * (2 * m + 1) * pmm
        for l in range(m + 2, lmax + 1):
            P[(l, m)] = ((2 * l - 1) * x * P[(l - 1, m)] - (l + m - 1) * P[(l - 2, m)]) / (l - m)
    Y = {}
    for l in range(lmax + 1):
        for m in range(-l, l + 1):
            am = abs(m)
            norm = np.sqrt((2 * l + 1) / (4 * np.pi) * factorial(l - am) / factorial(l + am))
            if m == 0:
                Y[(l, m)] = norm * P[(l, 0)]
            elif m > 0:
                Y[(l, m)] = np.sqrt(2.0) * norm * P[(l, am)] * np.cos(am * phi)
            else:
                Y[(l, m)] = np.sqrt(2.0) * norm * P[(l, am)] * np.sin(am * phi)
    return Y


def bumpy_sphere(n_subdiv=8, seed=4, amplitude=0.1, lmax=8):
    """The full-solve workload's surface: an icosphere subdivided ``n_subdiv``
    times (20 4^n triangles; 1,310,720 at 8) whose vertices are moved to
    r = 1 + amplitude Y(theta, phi), Y = sum over 1 <= l <= lmax, |m| <= l of
    c_lm Y_lm with c_lm ~ N(0, 1 / l^2) (real orthonormal harmonics) drawn
    from a generator seeded ``seed``.  Returns (verts, tris)."""
    v, t = icosphere(n_subdiv)
    rng = np.random.default_rng(seed)
    theta = np.arccos(np.clip(v[:, 2], -1.0, 1.0))
    phi = np.arctan2(v[:, 1], v[:, 0])
    Y = real_sph_harm(lmax, theta, phi)
    bump = np.zeros(len(v))
    for l in range(1, lmax + 1):
        for m in range(-l, l + 1):
            bump += rng.normal(0.0, 1.0 / l) * Y[(l, m)]
    return v * (1.0 + amplitude * bump)[:, None], t


def interior_charges(n=10, seed=4, radius=0.3):
    """``n`` unit point charges uniform in the ball of ``radius`` about the
    origin (inside the bumpy sphere), from a generator seeded ``seed`` + 1."""
    rng = np.random.default_rng(seed + 1)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    return d * (radius * rng.uniform(0, 1, n) ** (1.0 / 3.0))[:, None]


_SPHERE_CACHE = {}


def sphere_batch(n_meshes=200, seed=2, levels=(2, 6), n_rhs=64):
    """The batched Laplace workload: ``n_meshes`` icospheres with subdivision
    levels drawn uniformly from ``levels`` (inclusive; 320 to 81,920
    triangles), radii lognormal(0, 0.5), centres uniform in [-100, 100]^3, 3
    Gauss points per triangle, outward normals; then ``n_rhs`` densities
    uniform[-1, 1] over all points, all from one generator seeded ``seed``.
    Returns (locs [N,3], normals [N,3], weights [N], offsets [n_meshes + 1],
    x [n_rhs, N])."""
    rng = np.random.default_rng(seed)
    lev = rng.integers(levels[0], levels[1] + 1, n_meshes)
    rad = rng.lognormal(0.0, 0.5, n_meshes)
    cen = rng.uniform(-100.0, 100.0, (n_meshes, 3))
    L, Nm, W, off = [], [], [], [0]
    for m in range(n_meshes):
        k = int(lev[m])
        if k not in _SPHERE_CACHE:
            _SPHERE_CACHE[k] = sphere_points(k)
        l0, n0, w0 = _SPHERE_CACHE[k]
        L.append(l0 * rad[m] + cen[m])
        Nm.append(n0)
        W.append(w0 * rad[m] ** 2)
        off.append(off[-1] + len(l0))
    locs = np.ascontiguousarray(np.concatenate(L))
    x = rng.uniform(-1.0, 1.0, (n_rhs, len(locs)))
    return (locs, np.ascontiguousarray(np.concatenate(Nm)), np.ascontiguousarray(np.concatenate(W)),
            np.asarray(off, dtype=np.int64), x)


def misfit_workload(n=64, n_obs=16384, seed=3):
    """The differentiated workload's geometry and slips: an n x n-quad fault
    dipping 45 degrees (2 n^2 triangles, 3 Gauss points each) whose vertices
    are lifted by 0.05 sin(3x) cos(2y), ``n_obs`` observers uniform on the
    free surface z = 0 over [-3, 3]^2 (normals +z), and two 3-component
    slips uniform[-1, 1] (the one differentiated, and the one that makes the
    data) and the data's noise N(0, 1e-3) per observed component, all from
    one generator seeded ``seed``.  Returns (verts, tris, obs_locs,
    obs_normals, s, s2, noise) with slips component-major ([3 N])."""
    v, t, _ = dipping_fault(n, 45.0)
    v = v.copy()
    v[:, 2] += 0.05 * np.sin(3 * v[:, 0]) * np.cos(2 * v[:, 1])
    rng = np.random.default_rng(seed)
    obs = np.column_stack([rng.uniform(-3, 3, n_obs), rng.uniform(-3, 3, n_obs), np.zeros(n_obs)])
    on = np.tile([0.0, 0.0, 1.0], (n_obs, 1))
    n_pts = 3 * len(t)
    s = rng.uniform(-1, 1, 3 * n_pts)
    s2 = rng.uniform(-1, 1, 3 * n_pts)
    noise = rng.normal(0.0, 1e-3, 3 * n_obs)
    return v, t, obs, on, s, s2, noise


def fault_points(n=128, dip_deg=45.0):
    """Dipping-fault points (98,304 at n=128) plus each point's (u, v)."""
    v, t, uv = dipping_fault(n, dip_deg)
    locs, normals, weights = points_from_mesh(v, t)
    uvp = np.einsum("qk,tkd->tqd", _TRI3_BARY, uv[t]).reshape(-1, 2)
    return locs, normals, weights, uvp


def tapered_slip(uv, seed=1):
    """3-component slip: uniform[-1,1] times a cosine taper to zero at edges.

    Returned component-major ([3 * N], x[d * N + i]) like the reference's
    operator inputs (cpp/fmm.cpp:189-190).
    """
    rng = np.random.default_rng(seed)
    n = uv.shape[0]
    taper = np.cos(0.5 * np.pi * uv[:, 0]) * np.cos(0.5 * np.pi * uv[:, 1])
    s = rng.uniform(-1.0, 1.0, size=(3, n)) * taper[None, :]
    return np.ascontiguousarray(s.reshape(-1))


def points_from_mesh_torch(verts, tris):
    """points_from_mesh with torch tensors (differentiable in the vertices):
    3-point rule locations, unit normals and weights area / 3."""
    import torch
    t = torch.as_tensor(tris, dtype=torch.long, device=verts.device)
    p = verts[t]                                           # [nt, 3, 3]
    cr = torch.cross(p[:, 2] - p[:, 0], p[:, 2] - p[:, 1], dim=1)
    nrm = torch.linalg.norm(cr, dim=1)
    normals = cr / nrm[:, None]
    bary = torch.as_tensor(_TRI3_BARY, dtype=verts.dtype, device=verts.device)
    locs = torch.einsum("qk,tkd->tqd", bary, p).reshape(-1, 3)
    normals = normals.repeat_interleave(3, dim=0)
    weights = ((1.0 / 6.0) * nrm).repeat_interleave(3)    # (1/6) (2 area)
    return locs, normals, weights
