"""Step-grid record and replay in the FP64 oracle (CPU).

The ADAPTIVE loop of the reference (src/focss/solver/ssfm.cpp:92-118) takes
each step size from the field's peak power after the Kerr step (:136-140).
Replaying a recorded list of step sizes through the same loop must reproduce
the recorded run bit for bit, so that a GPU run and the oracle can be put on
one grid.  The oracle's ADAPTIVE run itself is pinned bit for bit to the
reference build (test_oracle_pins.py).
"""
import numpy as np
import pytest

from conftest import ALPHA, BETA2, GAMMA, rel_l2


def _signal(n, p_mw, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * np.sqrt(p_mw * 1e-3 / 2)


@pytest.mark.parametrize("direction", [1.0, -1.0])
def test_adaptive_replay_is_bit_identical(oracle_cpu, direction):
    cpu = oracle_cpu
    fib = cpu.Fiber(ALPHA, BETA2, GAMMA, 20e3, 1.55e-6, 1.0)
    x = _signal(1024, 8.0, 3)
    want, steps = cpu.ssfm_run(x, 1 / 128e9, fib, cpu.ADAPTIVE, 1, 0.005, 1000.0, direction)
    got, rsteps, h = cpu.ssfm_run_recorded(x, 1 / 128e9, fib, cpu.ADAPTIVE, 1, 0.005, 1000.0, direction)
    assert rsteps == steps == h.size and steps > 20
    assert np.array_equal(got, want)
    assert abs(h.sum() - 20e3) < 1e-6 and np.all(h > 0) and np.all(h <= 1000.0)
    rep = cpu.ssfm_run_steps(x, 1 / 128e9, fib, h, direction)
    assert np.array_equal(rep, want)


def test_uniform_and_logarithmic_lists(oracle_cpu):
    cpu = oracle_cpu
    fib = cpu.Fiber(ALPHA, BETA2, GAMMA, 40e3, 1.55e-6, 1.0)
    x = _signal(512, 4.0, 4)
    want, steps, h = cpu.ssfm_run_recorded(x, 1 / 64e9, fib, cpu.UNIFORM, 25)
    assert steps == 25 and np.allclose(h, 40e3 / 25, rtol=0, atol=1e-9)
    # the same grid in the ADAPTIVE loop's Strang pattern: equal in exact arithmetic
    assert rel_l2(cpu.ssfm_run_steps(x, 1 / 64e9, fib, h), want) < 1e-12
    want, steps, h = cpu.ssfm_run_recorded(x, 1 / 64e9, fib, cpu.LOGARITHMIC, 1, 0.005, 1000.0)
    assert steps == h.size and abs(h.sum() - 40e3) < 1e-6
    assert rel_l2(cpu.ssfm_run_steps(x, 1 / 64e9, fib, h), want) < 1e-12


def test_replay_rejects_empty_list(oracle_cpu):
    cpu = oracle_cpu
    fib = cpu.Fiber(ALPHA, BETA2, GAMMA, 1e3, 1.55e-6, 1.0)
    with pytest.raises(ValueError):
        cpu.ssfm_run_steps(np.zeros(256, complex), 1e-12, fib, [])
