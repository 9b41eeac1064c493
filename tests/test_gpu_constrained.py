"""Centroid-constrained PIMD on the device stepper: the bead centroid stays
where it is while the internal modes move, and the accumulated mean centroid
force is the step average of (1/P) sum_b F_b."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _constrained(q, n=64, P=8, precision=None, seed=71, thermo=None):
    st = q.seeded_start(n, P, 298.0, seed=seed)
    ctx = q.Context([q.system_desc(n, P, st.box_bohr, propagator=q.TROTTER,
                                   thermostat=q.PILE_L if thermo is None else thermo, seed=seed)],
                    q.MIXED if precision is None else precision)
    s = ctx.systems[0]
    s.set_state(st.q, st.p)
    s.set_centroid_fixed(True)
    ctx.init_forces()
    return ctx, s, st


def _centroid(x, P):
    return x.reshape(P, -1).mean(axis=0)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_centroid_stays_fixed_while_beads_move(gpu_lib, prec):
    q = gpu_lib
    ctx, s, st = _constrained(q, precision=q.FP64 if prec == "fp64" else q.MIXED)
    c0 = _centroid(st.q.reshape(-1), 8)
    ctx.run_steps(200, is_nvt=True)
    ctx.sync()
    qn = s.get_state()["q"]
    assert np.abs(_centroid(qn, 8) - c0).max() < 1e-10
    assert np.abs(qn - st.q.reshape(-1)).max() > 1e-3  # internal modes moved
    assert np.all(np.isfinite(s.estimators()["conserved"]))


def test_mean_centroid_force_is_the_bead_averaged_force(gpu_lib):
    q = gpu_lib
    ctx, s, _ = _constrained(q, precision=q.FP64)
    s.reset_centroid_force()
    ctx.run_steps(1, is_nvt=True)
    ctx.sync()
    f, n = s.centroid_force()
    assert n == 1
    ref = _centroid(s.get_state()["fphys"], 8)
    assert np.abs(f - ref).max() < 1e-12 * max(1.0, np.abs(ref).max())
    # the running mean over several steps, and reset
    ctx.run_steps(9, is_nvt=True)
    ctx.sync()
    f10, n10 = s.centroid_force()
    assert n10 == 10 and np.all(np.isfinite(f10))
    s.reset_centroid_force()
    f0, n0 = s.centroid_force()
    assert n0 == 0 and not np.any(f0)


def test_unconstrained_systems_accumulate_nothing(gpu_lib):
    q = gpu_lib
    ctx, s, _ = _constrained(q, precision=q.MIXED)
    s.set_centroid_fixed(False)
    s.reset_centroid_force()
    ctx.run_steps(5, is_nvt=True)
    ctx.sync()
    f, n = s.centroid_force()
    assert n == 0
