"""Emitters (pbd_add_emitter / pbd_emit): the CPU reference's FluidEmitter
and OpenSmokeEmitter on the CUDA system.  Emission is checked against the
emitter's timer and its seeded velocity jitter; the solidification against
its rule applied, tick by tick, to the lambdas, velocities and positions the
CUDA system had before the tick.  Both rules (tests/helpers.py:
emitter_counts, solidify_rule) are pinned to the reference's own
FluidEmitter::tick and OpenSmokeEmitter::tick
(tests/test_oracle_vs_reference.py, tests/test_golden_oracle.py)."""
import numpy as np
import pytest

from helpers import emitter_counts as expected_counts
from helpers import solidify_rule
from particlesolver_gb300 import ParticleSystem, PbdError, default_params
from particlesolver_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def block_system(capacity=4096):
    sc = W.pbf_block(512, seed=3)
    g = ParticleSystem(default_params(**sc.params), capacity)
    W.apply_to(sc, g)
    return sc, g


def test_fluid_emitter_emits_on_its_timer_with_seeded_jitter():
    sc, g = block_system()
    dt = float(np.float32(1 / 60))  # the step the C ABI receives
    pos, vel, jit, seed, rate, dur = [0.3, 2.0, 0.4], [0.0, 1.0, 0.0], [1.0, 0.0, 0.5], 7, 33.0, 0.5
    g.add_emitter(position=pos, rate=rate, duration=dur, phase=W.PHASE_FLUID, inverse_mass=1.0, rest_density=2.5,
                  velocity=vel, velocity_jitter=jit, seed=seed)
    want = expected_counts(rate, dur, dt, 60)
    got = [g.emit(dt) for _ in range(60)]
    assert got == want and sum(got) > 0
    total = sum(got)
    x, v, ph = g.positions()[sc.n:], g.velocities()[sc.n:], g.phases()[sc.n:]
    assert x.shape[0] == total
    np.testing.assert_array_equal(x, np.tile(np.float32(pos + [1.0]), (total, 1)))
    u = W.uniform(seed, (total, 3), 0.0, 1.0).astype(np.float32)
    np.testing.assert_allclose(v[:, :3], np.float32(vel) + u * np.float32(jit), rtol=0, atol=1e-6)
    assert np.all(ph == W.PHASE_FLUID)


def test_emission_stops_at_the_capacity():
    sc, g = block_system(capacity=530)
    g.add_emitter(position=[0.0, 2.0, 0.0], rate=1000.0, duration=0.0, phase=W.PHASE_FLUID)
    assert g.emit(0.1) == 530 - sc.n
    assert g.emit(0.1) == 0
    g.update(1 / 60)
    g.check_finite()


def test_smoke_emitter_feeds_an_open_gas():
    sc = W.smoke_box(open_gas=True, solid_floor=True)
    g = ParticleSystem(default_params(**sc.params), sc.n + 200)
    W.apply_to(sc, g)
    g.add_emitter(position=[0.0, -2.0, 0.0], rate=15.0, duration=0.0, phase=W.PHASE_GAS, rest_density=1.5,
                  open_gas=1, seed=11)
    added = 0
    for _ in range(30):
        g.update(sc.dt)
        added += g.emit(sc.dt)
    assert added == sum(expected_counts(15.0, 0.0, float(np.float32(sc.dt)), 30))
    g.update(sc.dt)
    g.check_finite()
    new = slice(sc.n, sc.n + added)
    assert np.all(g.phases()[new] == W.PHASE_GAS)
    assert np.max(np.abs(g.forces()[new, :3])) > 0.0  # open drag / vorticity reach the emitted gas



def test_gas_emitter_follows_the_smoke_emitter():
    """A gas emitter without a time limit emits as OpenSmokeEmitter::tick
    (opensmokeemitter.cpp:17-28; the rule pinned to it by
    tests/test_oracle_vs_reference.py and tests/test_golden_oracle.py): 6 s
    of ticks, past the fluid emitter's 5 s, each particle a gas particle of
    inverse mass 1 at rest at the emitter."""
    sc = W.smoke_box(open_gas=True, solid_floor=True)
    g = ParticleSystem(default_params(**sc.params), sc.n + 100)
    W.apply_to(sc, g)
    pos, rate, dt = [0.25, -1.5, 0.0], 7.0, float(np.float32(0.05))
    g.add_emitter(position=pos, rate=rate, duration=0.0, phase=W.PHASE_GAS, inverse_mass=1.0, rest_density=1.0,
                  open_gas=1, seed=5)
    ticks = int(np.ceil(6.0 / dt))
    got = [g.emit(dt) for _ in range(ticks)]
    assert got == expected_counts(rate, 0.0, dt, ticks) and sum(got) > rate * 5.0
    new = slice(sc.n, sc.n + sum(got))
    np.testing.assert_array_equal(g.positions()[new], np.tile(np.float32(pos + [1.0]), (sum(got), 1)))
    assert np.all(g.velocities()[new, :3] == 0.0) and np.all(g.phases()[new] == W.PHASE_GAS)

def test_solidification_follows_the_fluid_emitter_rule():
    """A resting fluid block whose particles all take part: every tick, the
    particles slower than the threshold at a low enough height count their
    timers down while lambda <= 0 (up by dt, at most 3, otherwise) and turn
    into solids pinned where they stopped -- checked tick by tick against
    the rule."""
    sc, g = block_system()
    speed, height, dt = 0.5, 100.0, float(np.float32(1 / 60))
    g.add_emitter(position=[0.0, 50.0, 0.0], rate=1.0, duration=1e-6, phase=W.PHASE_FLUID, solidify=1,
                  solidify_speed=speed, solidify_height=height, group_first=0, group_count=sc.n)
    timer = np.full(sc.n, 4.0)
    converted = 0
    for _ in range(12):
        g.update(dt)
        lam, v, x, ph = g.lambdas(), g.velocities(), g.positions(), g.phases()
        timer, turn = solidify_rule(x[:, 1], np.linalg.norm(v[:, :3], axis=1), lam, timer, ph == W.PHASE_FLUID,
                                    float(np.float32(dt)), speed, height)
        assert g.emit(dt) == 0
        ph2, x2 = g.phases(), g.positions()
        want = np.where(turn, W.PHASE_SOLID, ph)
        np.testing.assert_array_equal(ph2, want)
        assert np.all(x2[turn, 3] == 0.0) and np.all(g.velocities()[turn, :3] == 0.0)
        converted += int(turn.sum())
    assert converted > 0
    for _ in range(3):  # the census follows the conversions: contacts run for the new solids
        g.update(dt)
    g.check_finite()
    fixed = g.phases() == W.PHASE_SOLID
    np.testing.assert_array_equal(g.positions()[fixed], x2[fixed])  # pinned
    assert np.all(g.positions()[fixed, 3] == 0.0)


def test_emitter_arguments_validated():
    sc, g = block_system()
    with pytest.raises(PbdError):
        g.add_emitter(position=[0, 0, 0], rate=0.0, phase=W.PHASE_FLUID)
    with pytest.raises(PbdError):
        g.add_emitter(position=[0, 0, 0], rate=5.0, phase=W.PHASE_SOLID)
    with pytest.raises(PbdError):
        g.add_emitter(position=[0, 0, 0], rate=5.0, phase=W.PHASE_FLUID, solidify=1, group_first=0,
                      group_count=sc.n + 1)
