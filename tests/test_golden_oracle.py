"""The oracle against the golden fixtures made from the reference's own
kernels (tests/golden/make_golden.py).  Runs anywhere (no reference tree,
no GPU needed)."""
import numpy as np
import pytest

from helpers import check_against_golden, check_trajectory, golden_scene, params_nolib, run_stages
from conftest import GOLDEN
from oracle import Oracle
from particlesolver_gb300 import workloads as W

FIXTURES = sorted(GOLDEN.glob("ref_*.npz"))


class OracleSystem(Oracle):
    """Oracle with the CUDA system's method names for run_stages."""

    def grid(self):
        return super().grid()


def load_oracle(data):
    sc = golden_scene(data)
    o = OracleSystem(params_nolib(sc.params), sc.n)
    W.apply_to(sc, o)
    return sc, o


@pytest.mark.parametrize("path", FIXTURES, ids=[p.stem for p in FIXTURES])
def test_stages_match_reference_golden(path):
    data = np.load(path)
    sc, o = load_oracle(data)
    out = run_stages(o)
    check_against_golden(out, data, sc.pos_w)


@pytest.mark.parametrize("path", FIXTURES, ids=[p.stem for p in FIXTURES])
def test_updates_match_reference_golden(path):
    data = np.load(path)
    sc, o = load_oracle(data)
    for k in range(3):
        o.update(sc.dt)
        check_trajectory(o.positions(), data[f"update{k + 1}_pos"], sc.pos_w)


def test_fixtures_present():
    assert len(FIXTURES) >= 3
