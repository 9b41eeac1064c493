"""Device-resident stepping (CUDA-graph replay per step) against the oracle:
single systems, uneven batches of replicas, NVE conservation, thermostat
statistics and error states."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def oracle_steps(st, nsteps, trotter, temp=298.0, dt=0.25):
    from oracle.binding import Oracle

    o = Oracle(st.n_mols, st.n_beads, st.box_bohr, temp, dt)
    q, p = st.q.copy(), st.p.copy()
    point, lst, disp = o.build_lists(q)
    f = np.zeros_like(q)
    fp = np.zeros_like(q)
    if trotter:
        o.force_eval_trotter(q, f, point, lst)
        fp[:] = f
    else:
        o.force_eval_sc(q, f, point, lst, fp)
    for _ in range(nsteps):
        o.update_pimd(q, p, f, fp, point, lst, disp, is_nvt=False, trotter=trotter)
    return q, p, f


@pytest.mark.parametrize("prop", ["sc", "trotter"])
def test_device_steps_match_oracle(gpu_lib, prop):
    q = gpu_lib
    st = q.seeded_start(64, 4, 298.0, seed=41)
    s = q.System.create(64, 4, st.box_bohr, precision=q.FP64, dt_fs=0.25, seed=41,
                        propagator=q.SUZUKI_CHIN if prop == "sc" else q.TROTTER)
    s.set_state(st.q, st.p)
    s.ctx.init_forces()
    s.ctx.run_steps(4, is_nvt=False)
    s.ctx.sync()
    out = s.get_state()
    qo, po, fo = oracle_steps(st, 4, prop == "trotter")
    assert np.abs(out["q"].reshape(qo.shape) - qo).max() < 1e-10
    np.testing.assert_allclose(out["p"].reshape(po.shape), po, rtol=0, atol=1e-8 * np.abs(po).max())
    np.testing.assert_allclose(out["f"].reshape(fo.shape), fo, rtol=0, atol=1e-8 * np.abs(fo).max())
    est = s.estimators()
    assert len(est["step"]) == 5 and np.all(np.isfinite(est["conserved"]))


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-7)])
def test_uneven_replica_batch_matches_single_systems(gpu_lib, precision, tol):
    """Replicas of different N, P and T advance in one launch sequence; each must
    follow its own single-system oracle trajectory (mixed: a batch of second-order
    and Suzuki-Chin systems takes the forked force evaluation with the assembly
    kernel; positions in bohr)."""
    q = gpu_lib
    specs = [(64, 8, 250.0, 51, q.TROTTER), (27, 4, 330.0, 52, q.SUZUKI_CHIN), (125, 2, 298.0, 53, q.TROTTER)]
    starts = [q.seeded_start(n, p, t, seed=sd) for n, p, t, sd, _ in specs]
    descs = [q.system_desc(n, p, st.box_bohr, temp_K=t, dt_fs=0.25, seed=sd, propagator=pr)
             for (n, p, t, sd, pr), st in zip(specs, starts)]
    ctx = q.Context(descs, q.FP64 if precision == "fp64" else q.MIXED)
    for sys_, st in zip(ctx.systems, starts):
        sys_.set_state(st.q, st.p)
    ctx.init_forces()
    ctx.run_steps(3, is_nvt=False)
    ctx.sync()
    for sys_, st, spec in zip(ctx.systems, starts, specs):
        out = sys_.get_state()
        qo, _, _ = oracle_steps(st, 3, spec[4] == q.TROTTER, temp=spec[2])
        assert np.abs(out["q"].reshape(qo.shape) - qo).max() < tol, spec


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nve_conservation(gpu_lib, precision):
    """Ring-polymer Hamiltonian over 800 NVE steps (0.2 ps) of 64 waters, P=8, after
    600 PILE-G steps of equilibration (the protocol of simulation.cpp:880-937: the
    lattice start relaxes violently, so conservation is judged after equilibration)."""
    q = gpu_lib
    st = q.seeded_start(64, 8, 298.0, seed=61)
    s = q.System.create(64, 8, st.box_bohr, precision=q.FP64 if precision == "fp64" else q.MIXED, dt_fs=0.25,
                        propagator=q.TROTTER, thermostat=q.PILE_G, seed=61)
    s.set_state(st.q, st.p)
    s.ctx.init_forces()
    s.ctx.run_steps(600, is_nvt=True)
    s.ctx.reset_estimators()
    s.ctx.run_steps(800, is_nvt=False)
    s.ctx.sync()
    e = s.estimators()
    cons, kin = e["conserved"], e["kin"]
    assert np.all(np.isfinite(cons))
    slope = np.polyfit(np.arange(len(cons)), cons, 1)[0] * len(cons)
    # bounded fluctuation and drift, small against the kinetic-energy fluctuation scale
    assert np.abs(cons - cons.mean()).max() < 2e-3 * kin.mean()
    assert abs(slope) < 1e-3 * kin.mean()


def test_pile_g_samples_the_ring_polymer_temperature(gpu_lib):
    q = gpu_lib
    P, N, T = 4, 64, 298.0
    st = q.seeded_start(N, P, T, seed=71)
    s = q.System.create(N, P, st.box_bohr, precision=q.MIXED, temp_K=T, dt_fs=0.5, propagator=q.TROTTER,
                        thermostat=q.PILE_G, seed=71)
    s.set_state(st.q, st.p)
    s.ctx.init_forces()
    s.ctx.run_steps(400, is_nvt=True)
    s.ctx.reset_estimators()
    s.ctx.run_steps(1600, is_nvt=True)
    s.ctx.sync()
    e = s.estimators()
    beta_n = s.info.beta_n
    expect = 0.5 * P * 9 * N / beta_n  # bead kinetic energy at the ring-polymer temperature
    kin = e["kin"]
    assert abs(kin.mean() / expect - 1.0) < 0.03
    assert np.all(np.isfinite(e["conserved"])) and e["heat"][-1] != 0.0


def test_run_before_init_is_a_state_error(gpu_lib):
    q = gpu_lib
    st = q.seeded_start(27, 2, 298.0, seed=3)
    s = q.System.create(27, 2, st.box_bohr, precision=q.FP64)
    s.set_state(st.q, st.p)
    with pytest.raises(q.QtgError) as ei:
        s.ctx.run_steps(1)
    assert ei.value.status == 5


def test_counter_based_noise_is_reproducible(gpu_lib):
    """Two contexts with identical descriptors draw the same thermostat noise and
    sum their forces and system sums in a fixed order, so their NVT trajectories
    agree bit for bit."""
    q = gpu_lib
    st = q.seeded_start(27, 4, 298.0, seed=81)
    outs = []
    for _ in range(2):
        s = q.System.create(27, 4, st.box_bohr, precision=q.MIXED, propagator=q.TROTTER, seed=81)
        s.set_state(st.q, st.p)
        s.ctx.init_forces()
        s.ctx.run_steps(20, is_nvt=True)
        s.ctx.sync()
        outs.append(s.get_state()["q"])
    assert np.array_equal(outs[0], outs[1])
