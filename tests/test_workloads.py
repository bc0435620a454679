"""Seeded workload builders: sizes and structure of the configurations the
benchmark and the parity tests run (host only)."""
import numpy as np

from particlesolver_gb300 import workloads as W


def test_dam_break_one_million():
    sc = W.dam_break(128, 128, 64)
    assert sc.n == 1 << 20
    assert np.all(sc.phase == W.PHASE_FLUID)
    assert sc.params["grid_size"] == [256, 64, 32]


def test_mixed_scene_counts():
    sc = W.mixed_scene()
    assert sc.n == 65_536 + 128_000 + 640_000
    # cloth: stretch 2*256*255, shear 2*255^2, bend 2*256*254; ropes 63 links each
    assert len(sc.pairs) == 2 * 256 * 255 + 2 * 255 * 255 + 2 * 256 * 254 + 2000 * 63
    assert len(sc.bodies) == 10_000 and all(c == 64 for _, c, _ in sc.bodies)
    assert len(np.unique(sc.phase)) == 1 + 2000 + 10_000
    assert sc.pairs.max() < sc.n and np.all(sc.pairs[:, 0] != sc.pairs[:, 1])
    # each object's constraints stay inside the object
    assert np.all(sc.phase[sc.pairs[:, 0]] == sc.phase[sc.pairs[:, 1]])
    # the bodies sit above the ropes, the ropes above the cloth
    assert sc.pos_w[65_536:193_536, 1].min() > sc.pos_w[:65_536, 1].max()
    assert sc.pos_w[193_536:, 1].min() > sc.pos_w[65_536:193_536, 1].max()


def test_mixed_scene_is_seeded():
    a = W.mixed_scene(cloth=16, ropes=4, rope_particles=8, bodies=5)
    b = W.mixed_scene(cloth=16, ropes=4, rope_particles=8, bodies=5)
    np.testing.assert_array_equal(a.pos_w, b.pos_w)
    c = W.mixed_scene(cloth=16, ropes=4, rope_particles=8, bodies=5, seed=78)
    assert not np.array_equal(a.pos_w, c.pos_w)
