"""Profiling driver for the learned warm start's kernels under `ncu`.

Collects the training set of a jittered 64x16x16 beam (plain solver, gravity
and a sinusoidal tip load), trains for `--epochs` (k_mlp_train, k_adam,
k_pack_params), then runs `--steps` learned-start steps (k_node_features,
k_smooth_correction) and prints what it launched.  Run it plainly first, then
under ncu, e.g.

  python opentissue_gb300/profile_mlp.py --samples 262144 --epochs 2 --steps 2
  ncu --set full --clock-control none -k regex:k_mlp_train -s 2 -c 1 -o mlp_train \\
      python opentissue_gb300/profile_mlp.py --samples 262144 --epochs 2 --steps 2
"""
import argparse
import ctypes
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from opentissue_gb300 import build, capi  # noqa: E402
from opentissue_gb300.fem import generate_blocks  # noqa: E402
from opentissue_gb300.warmstart import WarmStartNet  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dims", type=int, nargs=3, default=[64, 16, 16])
    ap.add_argument("--samples", type=int, default=262144)
    ap.add_argument("--epochs", type=int, default=2)
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--steps", type=int, default=2)
    args = ap.parse_args()
    build.build()
    lib = capi.lib()
    I, J, K = args.dims
    tets, coord = generate_blocks(I, J, K, 0.1, 0.1, 0.1)
    coord = coord + np.random.default_rng(20261203).uniform(-0.01, 0.01, coord.shape)
    fixed = (np.arange(coord.shape[0]) < (J + 1) * (K + 1)).astype(np.uint8)
    tip = np.arange(coord.shape[0]) >= I * (J + 1) * (K + 1)
    N = coord.shape[0]
    dp = ctypes.POINTER(ctypes.c_double)

    def make():
        desc = capi.MeshDesc(N, tets.shape[0], tets.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                             coord.ctypes.data_as(dp), coord.ctypes.data_as(dp),
                             fixed.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
        h = ctypes.c_void_p()
        capi.check(lib.otfem_create(ctypes.byref(desc), None, ctypes.byref(h)))
        capi.check(lib.otfem_init(h, 5e5, 0.33, 1000.0, 1e30, 0.0, 0.0))
        mass = np.zeros(N)
        capi.check(lib.otfem_get_nodes(h, capi.MASS, mass.ctypes.data_as(dp), N))
        g = np.zeros((N, 3))
        g[fixed == 0, 1] = -9.81 * mass[fixed == 0]
        return h, g

    net = WarmStartNet(capacity=args.samples, seed=1)
    h, g = make()
    WarmStartNet.collect(h)
    plain = capi.default_params(solver=capi.SOLVER_MIXED, max_iterations=5000, rtol=1e-6)
    k = 0
    while net.num_samples() < args.samples and k < 1000:
        f = g.copy()
        f[tip] += 60.0 * np.sin(2 * np.pi * 2.0 * k * 0.01) * np.array([0.0, -0.8, 0.6]) / tip.sum()
        capi.check(lib.otfem_set_nodes(h, capi.F_EXTERNAL, f.ctypes.data_as(dp), f.size))
        capi.check(lib.otfem_simulate_ex(h, 0.01, 1, ctypes.byref(plain), None))
        net.add_samples(h)
        k += 1
    net.fit_normalization()
    loss = net.train(args.epochs, batch=args.batch, lr=1e-3, seed=2)
    capi.check(lib.otfem_destroy(h))
    h, g = make()
    net.attach(h)
    learned = capi.default_params(solver=capi.SOLVER_MIXED, max_iterations=5000, rtol=1e-6,
                                  warm_start=capi.WARM_START_LEARNED)
    st = capi.StepStats()
    for s in range(args.steps):
        capi.check(lib.otfem_set_nodes(h, capi.F_EXTERNAL, g.ctypes.data_as(dp), g.size))
        capi.check(lib.otfem_simulate_ex(h, 0.01, 1, ctypes.byref(learned), ctypes.byref(st)))
    capi.check(lib.otfem_synchronize(h))
    batches = (net.num_samples() + args.batch - 1) // args.batch
    print(f"samples {net.num_samples()} ({k} steps), {args.epochs} epochs x {batches} minibatches, loss {loss:.4f}; "
          f"{args.steps} learned steps on {N} nodes, last {st.iterations} iterations")
    net.detach(h)
    capi.check(lib.otfem_destroy(h))
    net.close()


if __name__ == "__main__":
    main()
