"""The CPU oracle (C restatement of the reference) against the golden
fixtures generated from the unmodified reference headers, bit for bit."""
import os

import numpy as np
import pytest

from helpers import MATERIAL, beam, golden, gravity_force, step_hash
from opentissue_gb300.fem import generate_blocks


def _trajectory_hashes(po, tets, coord, fixed, steps, material=MATERIAL, warp=True, converged=False):
    m = po.OracleMesh(tets, coord, coord, fixed)
    m.init(*material)
    mass = m.get(po.MASS)
    hashes, its = [], []
    for _ in range(steps):
        m.set(po.F_EXTERNAL, gravity_force(mass, fixed))
        if converged:
            it, _ = m.simulate_converged(0.01, warp, 2.0, 1e-6, 100000)
            its.append(it)
        else:
            m.simulate(0.01, warp)
        hashes.append(step_hash(m.get(po.COORD), m.get(po.VELOCITY)))
    return m, hashes, its


def test_generate_blocks_matches_reference(oracle):
    g = golden("config1")
    tets, coord = generate_blocks(10, 4, 4, 0.1, 0.1, 0.1)
    assert np.array_equal(tets, g["tets"]) and np.array_equal(coord, g["coord"])
    for dims in [(1, 1, 1), (3, 2, 5), (7, 3, 2)]:
        a = generate_blocks(*dims, 0.1, 0.2, 0.3)
        b = oracle.generate_blocks(*dims, 0.1, 0.2, 0.3)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_config1_trajectory_bitwise(oracle):
    g = golden("config1")
    m, hashes, _ = _trajectory_hashes(oracle, g["tets"], g["coord"], g["fixed"], 100)
    assert hashes == list(g["hashes"])
    assert np.array_equal(m.get(oracle.COORD), g["x_final"])
    assert np.array_equal(m.get(oracle.MASS), g["mass"])


def test_config1_tip_value(oracle):
    # tip node after 100 steps, as measured on the reference
    g = golden("config1")
    tip = g["x_100"][-1]
    assert np.allclose(tip, [1.02712794204, 0.188507035986, 0.399908092627], atol=1e-11, rtol=0)


def test_k_rows_export_and_orientation_bitwise(oracle):
    g = golden("config1")
    m = oracle.OracleMesh(g["tets"], g["coord"], g["coord"], g["fixed"])
    m.init(*MATERIAL)
    r0, c0, v0 = m.export_k()
    assert len(v0) == 3 * int(g["fixed"].sum())  # before the first step only fixed rows export
    m.set(oracle.F_EXTERNAL, gravity_force(m.get(oracle.MASS), g["fixed"]))
    m.simulate(0.01, True)
    rp, cols = m.k_pattern()
    assert np.array_equal(rp, g["k_row_ptr"]) and np.array_equal(cols, g["k_cols"])
    assert np.array_equal(m.k_values(), g["k_values_1"])
    r, c, v = m.export_k()
    assert np.array_equal(r, g["export_rows_1"]) and np.array_equal(c, g["export_cols_1"])
    assert np.array_equal(v, g["export_vals_1"])
    assert np.array_equal(m.re(), g["re_1"])
    assert np.array_equal(m.get(oracle.F0), g["f0_1"]) and np.array_equal(m.get(oracle.B), g["b_1"])


def test_plastic_and_nowarp_bitwise(oracle):
    g = golden("plastic")
    m, hashes, _ = _trajectory_hashes(oracle, g["tets"], g["coord"], g["fixed"], 30,
                                      material=(5e5, 0.33, 1000.0, 1e-4, 50.0, 1e-2))
    assert hashes == list(g["hashes"])
    assert np.array_equal(m.plastic(), g["plastic_final"])
    assert np.abs(g["plastic_final"]).max() > 0
    g = golden("nowarp")
    _, hashes, _ = _trajectory_hashes(oracle, g["tets"], g["coord"], g["fixed"], 10, warp=False)
    assert hashes == list(g["hashes"])


def test_converged_cg_bitwise(oracle):
    g = golden("converged")
    tets, coord, fixed = beam(16, 6, 6, jitter_seed=7)
    assert np.array_equal(coord, g["coord"])
    _, hashes, its = _trajectory_hashes(oracle, tets, coord, fixed, 20, converged=True)
    assert hashes == list(g["hashes"])
    assert its == list(g["iterations"])


def test_update_original_coord(oracle):
    tets, coord, fixed = beam(4, 2, 2)
    m = oracle.OracleMesh(tets, coord, coord, fixed)
    m.init(*MATERIAL)
    m.set(oracle.F_EXTERNAL, gravity_force(m.get(oracle.MASS), fixed))
    m.simulate(0.01, True)
    m.update_original_coord()
    m.simulate(0.01, True)
    assert np.isfinite(m.get(oracle.COORD)).all()


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle",
                                                    "_ref", "libotfem_ref.so")),
                    reason="reference build not present on this machine")
def test_port_matches_live_reference_random_meshes(oracle):
    for seed, dims in [(1, (3, 2, 2)), (2, (5, 3, 4)), (3, (2, 5, 3))]:
        tets, coord, fixed = beam(*dims, jitter_seed=seed, jitter=0.02)
        out = {}
        for kind in ("port", "reference"):
            m = oracle.OracleMesh(tets, coord, coord, fixed, kind=kind)
            m.init(3e5, 0.4, 900.0, 1e-3, 20.0, 5e-2)
            mass = m.get(oracle.MASS)
            hs = []
            for s in range(5):
                m.set(oracle.F_EXTERNAL, gravity_force(mass, fixed))
                if s % 2:
                    m.simulate_converged(0.005, True, 1.5, 1e-8, 1000)
                else:
                    m.simulate(0.005, True)
                hs.append(step_hash(m.get(oracle.COORD), m.get(oracle.VELOCITY)))
            out[kind] = (hs, m.plastic())
        assert out["port"][0] == out["reference"][0]
        assert np.array_equal(out["port"][1], out["reference"][1])
