"""Unstructured meshes: TetGen files (t4mesh::tetgen_read) and Delaunay
meshes with scrambled node numbering, through the GPU pattern builder and the
solvers, against the C oracle."""
import os

import numpy as np
import pytest

from helpers import MATERIAL, GpuMesh, gravity_force, irregular_mesh
from opentissue_gb300 import capi
from opentissue_gb300.fem import tetgen_read, tetgen_write

# ---- TetGen files (CPU) -------------------------------------------------------


def test_tetgen_round_trip(tmp_path):
    tets, coord, _ = irregular_mesh((4, 3, 3), seed=1)
    base = os.path.join(tmp_path, "m")
    tetgen_write(base, tets, coord)
    t2, c2 = tetgen_read(base)
    assert np.array_equal(t2, tets) and np.array_equal(c2, coord)


def test_tetgen_read_attributes_markers_and_ids(tmp_path):
    """Point attributes and boundary markers are skipped, ids may start
    anywhere, '#' starts a comment (t4mesh_tetgen_read.h:62-83, 96-125)."""
    base = os.path.join(tmp_path, "a")
    with open(base + ".node", "w") as f:
        f.write("# four points\n4 3 1 1\n")
        f.write("10 0 0 0 7.5 1\n11 1 0 0 7.5 0\n12 0 1 0 7.5 0  # apex\n13 0 0 1 7.5 1\n")
    with open(base + ".ele", "w") as f:
        f.write("1 4 1\n5 10 11 12 13 3\n")
    tets, coord = tetgen_read(base)
    assert tets.tolist() == [[0, 1, 2, 3]]
    assert coord.tolist() == [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]]


def test_tetgen_read_rejects_what_the_reference_rejects(tmp_path):
    base = os.path.join(tmp_path, "b")
    with pytest.raises(ValueError, match="unable to open"):
        tetgen_read(base)
    with open(base + ".node", "w") as f:
        f.write("4 3 0 0\n1 0 0 0\n2 1 0 0\n3 0 1 0\n4 0 0 1\n")
    with open(base + ".ele", "w") as f:
        f.write("1 10 0\n1 1 2 3 4 1 2 3 4 1 2\n")  # 10-node tets
    with pytest.raises(ValueError, match="4 points"):
        tetgen_read(base)
    with open(base + ".ele", "w") as f:
        f.write("1 4 2\n1 1 2 3 4 0 0\n")  # two attributes
    with pytest.raises(ValueError, match="1 region"):
        tetgen_read(base)


def test_irregular_mesh_is_a_valid_fem_mesh(oracle):
    tets, coord, fixed = irregular_mesh((8, 4, 4), seed=2)
    e = coord[tets[:, 1:]] - coord[tets[:, :1]]
    assert (np.einsum("ij,ij->i", e[:, 0], np.cross(e[:, 1], e[:, 2])) > 0).all()
    assert len(np.unique(tets)) == len(coord) and 0 < fixed.sum() < len(coord)
    o = oracle.OracleMesh(tets, coord, coord, fixed)
    o.init(*MATERIAL)
    assert (o.get(oracle.MASS)[fixed == 0] > 0).all()
    o.close()

# ---- GPU against the oracle ---------------------------------------------------


@pytest.mark.gpu
def test_irregular_pattern_and_reference_solver_bitwise(gpu, oracle, tmp_path):
    """The K_row keys built on the GPU, and five reference-solver steps with
    sequential dot products, are bit-identical to the oracle on a mesh read
    from TetGen files."""
    tets, coord, fixed = irregular_mesh((10, 4, 4), seed=3)
    base = os.path.join(tmp_path, "irr")
    tetgen_write(base, tets, coord)
    tets, coord = tetgen_read(base)
    o = oracle.OracleMesh(tets, coord, coord, fixed)
    o.init(*MATERIAL)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    mass = m.get(capi.MASS)
    assert np.array_equal(mass, o.get(oracle.MASS))
    f = gravity_force(mass, fixed)
    for _ in range(5):
        m.set(capi.F_EXTERNAL, f)
        o.set(oracle.F_EXTERNAL, f)
        m.step(0.01, True, capi.default_params(sequential_dots=1))
        o.simulate(0.01, True)
    rp, cols = m.k_pattern()
    rp_o, cols_o = o.k_pattern()
    assert np.array_equal(rp, rp_o) and np.array_equal(cols, cols_o)
    assert np.array_equal(m.get(capi.COORD), o.get(oracle.COORD))
    assert np.array_equal(m.get(capi.VELOCITY), o.get(oracle.VELOCITY))
    o.close()
    m.close()


@pytest.mark.gpu
@pytest.mark.parametrize("variant", range(capi.NUM_APPLY_VARIANTS))
def test_irregular_matrix_free_vs_oracle(gpu, oracle, variant):
    """The matrix-free solver (every apply variant, plain and projected
    starts) against the converged FP64 oracle on a scrambled Delaunay mesh."""
    tets, coord, fixed = irregular_mesh((12, 4, 4), seed=4)
    o = oracle.OracleMesh(tets, coord, coord, fixed)
    o.init(*MATERIAL)
    mass = o.get(oracle.MASS)
    f = gravity_force(mass, fixed)
    ref = []
    for _ in range(8):
        o.set(oracle.F_EXTERNAL, f)
        o.simulate_converged(0.01, True, 2.0, 1e-11, 100000)
        ref.append(o.get(oracle.COORD))
    o.close()
    for warm in (capi.WARM_START_PREVIOUS, capi.WARM_START_PROJECTED, capi.WARM_START_EXTRAPOLATED):
        m = GpuMesh(tets, coord, fixed)
        m.init()
        capi.check(m.lib.otfem_set_apply_variant(m.h, variant))
        p = capi.default_params(solver=capi.SOLVER_MIXED, max_iterations=5000, rtol=1e-6, warm_start=warm)
        for s in range(8):
            m.set(capi.F_EXTERNAL, f)
            _, st = m.step(0.01, True, p)
            assert st.status == capi.OK and st.rel_residual <= 1e-6
            x = m.get(capi.COORD)
            disp = np.abs(ref[s] - coord).max()
            assert np.abs(x - ref[s]).max() <= 1e-5 * disp, (warm, s)
        m.close()
