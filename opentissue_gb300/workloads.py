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


def jittered_beam(I, J, K, seed, jitter=0.01, edge=0.1):
    """A cantilever of I x J x K blocks (edge `edge`, 5 tets per block) with
    every node moved by U[-jitter, jitter] per coordinate (numpy PCG64 `seed`)
    and the x = 0 face (grid index i == 0) fixed."""
    tets, coord = generate_blocks(I, J, K, edge, edge, edge)
    rng = np.random.default_rng(seed)
    coord = coord + rng.uniform(-jitter, jitter, coord.shape)
    fixed = (np.arange(coord.shape[0]) < (J + 1) * (K + 1)).astype(np.uint8)
    return tets, coord, fixed


def gravity(mass, fixed, g=-9.81):
    """m_i * (0, g, 0) on the free nodes."""
    f = np.zeros((mass.shape[0], 3))
    free = fixed == 0
    f[free, 1] = g * mass[free]
    return f


class SineTip:
    """The time-varying tip load of the learned-start comparison: a force
    amp * sin(2 pi freq t) * d spread evenly over the free end face (grid
    index i == I) of an I x J x K beam, with amp ~ U[0, 100] N, freq ~
    U[0.5, 5] Hz and d uniform on the sphere, drawn from numpy PCG64 `seed`.
    Step k (0-based) of a run applies the load at t = k * dt."""

    def __init__(self, I, J, K, seed):
        rng = np.random.default_rng(seed)
        self.amp = float(rng.uniform(0, 100))
        self.freq = float(rng.uniform(0.5, 5))
        d = rng.normal(size=3)
        self.direction = d / np.linalg.norm(d)
        n = (I + 1) * (J + 1) * (K + 1)
        self.tip = np.arange(n) >= I * (J + 1) * (K + 1)

    def force(self, k, dt):
        f = np.zeros((self.tip.shape[0], 3))
        f[self.tip] = self.amp * np.sin(2 * np.pi * self.freq * k * dt) * self.direction / self.tip.sum()
        return f


# The configurations the fixtures, tests and benchmark share.
BEAM128 = dict(I=128, J=32, K=32, seed=20261203, dt=0.01, steps=200)           # single large mesh, gravity
BEAM64_SINE = dict(I=64, J=16, K=16, seed=20261208, load_seed=20261209, dt=0.01, steps=500)  # gravity + SineTip
BATCH = dict(count=256, seed=20261203, dt=0.005, freq_seed=20261210)


def batch_tip_frequencies(count, seed=BATCH["freq_seed"]):
    """Per-beam frequencies U[0.5, 5] Hz of the batch's sinusoidal tip loads."""
    return np.random.default_rng(seed).uniform(0.5, 5, count)


def batch_forces(beams, mass, k, dt, sine, freqs=None):
    """External forces of a batch (the beams' nodes one after another) at step
    k (0-based): gravity plus each beam's tip force, constant or scaled by
    sin(2 pi f_beam k dt); zero on fixed nodes."""
    out = []
    off = 0
    for b_i, bm in enumerate(beams):
        n = bm["coord"].shape[0]
        f = gravity(mass[off:off + n], bm["fixed"])
        s = np.sin(2 * np.pi * freqs[b_i] * k * dt) if sine else 1.0
        f = f + s * bm["tip_force"]
        f[bm["fixed"] == 1] = 0.0
        out.append(f)
        off += n
    return np.concatenate(out)
