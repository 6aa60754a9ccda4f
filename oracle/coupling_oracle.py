"""CPU restatement of t4mesh::mesh_coupling (core/containers/t4mesh/util/
t4mesh_mesh_coupling.h) -- test infrastructure only: the library never
imports, links or runs it.

* barycentric(): geometry::barycentric_algebraic for tetrahedra
  (core/geometry/geometry_barycentric.h:343-385): w = P^-1 (p - x4) with the
  columns of P the edges x1 - x4, x2 - x4, x3 - x4; w4 = 1 - w1 - w2 - w3.
* bind(): bind_surface (t4mesh_mesh_coupling.h:129-236) with the embedding
  test of collision_policy::report (:84-111), all four weights in
  (-1e-4, 1 + 1e-4).  The reference's spatial-hash point query
  (collision/spatial_hashing/spatial_hashing_query.h:141-158) visits the
  tets in index order and report() keeps a point's first embedding tet, so
  the binding is the lowest tet index that embeds the point, which is what
  this restatement computes.  Stored per point: the tet and (m_w1, m_w2,
  m_w3).
* update(): update_surface (:238-275), p0 w0 + p1 w1 + p2 w2 + p3 w3 with
  w0 = 1 - w1 - w2 - w3.

Pinned to the reference: tests/golden/coupling.npz holds bind_surface and
update_surface of the unmodified reference headers (oracle/ref/
ref_coupling.cpp, tests/golden/make_coupling.py), and tests/test_coupling.py
checks this restatement against it (identical tets, weights to 1e-12).
"""
import numpy as np

DELTA = 10e-5  # t4mesh_mesh_coupling.h:91


def barycentric(x1, x2, x3, x4, p):
    """Weights (w1, w2, w3, w4) of p for the tets (x1, x2, x3, x4), batched
    over the leading dimension."""
    P = np.stack([x1 - x4, x2 - x4, x3 - x4], axis=-1)
    w = np.linalg.solve(P, (p - x4)[..., None])[..., 0]
    return np.concatenate([w, 1.0 - w.sum(axis=-1, keepdims=True)], axis=-1)


def bind(tets, x, points):
    """(tet per point, -1 if none; (w1, w2, w3) per point)."""
    xi, xj, xk, xm = (x[tets[:, k]] for k in range(4))
    tet = np.full(len(points), -1, np.int64)
    bary = np.zeros((len(points), 3))
    for n, p in enumerate(points):
        w = barycentric(xi, xj, xk, xm, np.broadcast_to(p, xi.shape))
        ok = np.all((w > -DELTA) & (w < 1.0 + DELTA), axis=1)
        hit = np.flatnonzero(ok)
        if hit.size:
            t = hit[0]
            tet[n] = t
            bary[n] = w[t, 1:]
    return tet, bary


def update(tets, x, tet, bary, rest):
    out = np.array(rest, dtype=np.float64, copy=True)
    for n, t in enumerate(tet):
        if t < 0:
            continue
        w1, w2, w3 = bary[n]
        w0 = 1.0 - w1 - w2 - w3
        p0, p1, p2, p3 = (x[tets[t, k]] for k in range(4))
        out[n] = p0 * w0 + p1 * w1 + p2 * w2 + p3 * w3
    return out
