"""Synthetic workloads of the benchmark configurations (seeded).

``random_beams`` draws the batched configuration: `count` cantilever beams of
nx x ny x nz unit blocks (edge 0.1 m, 5 tets per block) with nx ~ U{8..64},
ny, nz ~ U{3..16}, E ~ logU[1e5, 5e6] Pa, nu ~ U[0.25, 0.45], one of the 6
faces fixed (uniformly) and a tip force |F| ~ U[0, 50] N, direction uniform
on the sphere, spread evenly over the opposite face's nodes.
"""
import numpy as np

from .fem import generate_blocks


def face_nodes(I, J, K, face):
    """Node mask of a face of the block grid: 0/1 -> i = 0 / I, 2/3 -> j = 0 / J,
    4/5 -> k = 0 / K (node index (i*(J+1)+j)*(K+1)+k)."""
    i, j, k = np.meshgrid(np.arange(I + 1), np.arange(J + 1), np.arange(K + 1), indexing="ij")
    i, j, k = i.reshape(-1), j.reshape(-1), k.reshape(-1)
    axis, end = divmod(face, 2)
    g, n = ((i, I), (j, J), (k, K))[axis]
    return g == (n if end else 0)


def random_beams(count, seed, nx=(8, 64), nyz=(3, 16), edge=0.1):
    rng = np.random.default_rng(seed)
    beams = []
    for _ in range(count):
        I = int(rng.integers(nx[0], nx[1] + 1))
        J = int(rng.integers(nyz[0], nyz[1] + 1))
        K = int(rng.integers(nyz[0], nyz[1] + 1))
        tets, coord = generate_blocks(I, J, K, edge, edge, edge)
        face = int(rng.integers(6))
        fixed = face_nodes(I, J, K, face).astype(np.uint8)
        tip = face_nodes(I, J, K, face ^ 1)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        force = np.zeros_like(coord)
        force[tip] = rng.uniform(0, 50) * d / tip.sum()
        beams.append(dict(dims=(I, J, K), tets=tets, coord=coord, fixed=fixed, tip_force=force,
                          young=float(np.exp(rng.uniform(np.log(1e5), np.log(5e6)))),
                          poisson=float(rng.uniform(0.25, 0.45)), density=1000.0))
    return beams
