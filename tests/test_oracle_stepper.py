"""CPU checks of the oracle's restatement of the device stepper's propagation:
the Philox4x32-10 generator against the known-answer vectors published with
the algorithm (Salmon et al., SC'11, Random123), the noise distributions, and
the invariants of the constrained and thermostatted steps."""
import numpy as np
import pytest

from oracle.binding import Oracle, lib, philox4x32_10


@pytest.mark.parametrize("ctr,key,expect", [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
])
def test_philox_known_answers(ctr, key, expect):
    assert philox4x32_10(ctr, key) == expect


def test_mode_noise_is_standard_normal():
    L = lib()
    rng = np.random.default_rng(0)
    w = rng.integers(0, 2 ** 32, size=(200000, 2), dtype=np.uint64)
    x = np.array([L.qo_stepper_normal_f32(int(a), int(b)) for a, b in w])
    assert abs(x.mean()) < 0.01 and abs(x.var() - 1.0) < 0.01
    assert abs(np.mean(x ** 4) - 3.0) < 0.05


def test_centroid_draws_have_the_chi_square_moments():
    import ctypes as C

    L = lib()
    n_dof = 576
    R, g2 = C.c_double(), C.c_double()
    rs, gs = [], []
    for st in range(4000):
        assert L.qo_stepper_centroid_draw(7, 0, n_dof, st, C.byref(R), C.byref(g2)) == 1
        rs.append(R.value)
        gs.append(g2.value)
    rs, gs = np.array(rs), np.array(gs)
    k = n_dof - 1
    assert abs(rs.mean()) < 0.06 and abs(rs.var() - 1.0) < 0.08
    assert abs(gs.mean() / k - 1.0) < 0.01 and abs(gs.var() / (2 * k) - 1.0) < 0.1


def _state(N, P, seed):
    import qtip4pf_water_gb300 as q

    st = q.seeded_start(N, P, 298.0, seed=seed)
    o = Oracle(N, P, st.box_bohr, 298.0, 0.25)
    qq, pp = st.q.copy().reshape(-1), st.p.copy().reshape(-1)
    point, lst, disp = o.build_lists(qq)
    f = np.zeros_like(qq)
    o.force_eval_trotter(qq, f, point, lst)
    return o, st, [qq, pp, f, f.copy(), point, lst, disp]


def test_constrained_step_keeps_the_centroid_and_averages_the_force():
    o, st, (qq, pp, f, fp, point, lst, disp) = _state(27, 4, 3)
    stp = o.stepper(11, thermostat=2, trotter=True, centroid_fixed=True)
    c0 = qq.reshape(4, -1).mean(axis=0)
    cf = np.zeros(9 * 27)
    acc = np.zeros(9 * 27)
    for _ in range(5):
        o.stepper_step(stp, qq, pp, f, fp, point, lst, disp, is_nvt=True, cf_acc=cf)
        acc += fp.reshape(4, -1).mean(axis=0)
    assert np.abs(qq.reshape(4, -1).mean(axis=0) - c0).max() < 1e-10
    assert stp.cf_samples == 5 and stp.step == 6
    np.testing.assert_allclose(cf, acc, rtol=1e-12, atol=1e-14)


def test_nve_stepper_step_is_the_reference_step():
    """With the thermostat off the stepper's step is update.cpp:271-401 (second
    order): the restatement equals qo_update_pimd."""
    o, st, a = _state(27, 4, 5)
    b = [x.copy() for x in a]
    stp = o.stepper(1, thermostat=1, trotter=True)
    for _ in range(3):
        o.stepper_step(stp, *a, is_nvt=False)
        o.update_pimd(*b, is_nvt=False, trotter=True)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_same_seed_same_trajectory_different_seed_differs():
    outs = []
    for seed in (21, 21, 22):
        o, st, a = _state(27, 2, 9)
        stp = o.stepper(seed, thermostat=1, trotter=True)
        for _ in range(3):
            o.stepper_step(stp, *a, is_nvt=True)
        outs.append(a[0].copy())
    assert np.array_equal(outs[0], outs[1]) and not np.array_equal(outs[0], outs[2])


def test_nvt_chains_in_spawned_workers_are_seeded_and_distinct():
    """The replica chains the statistical comparison runs in spawned worker
    processes: one (seed, system index) gives one run average, another seed or
    another system index another."""
    import multiprocessing as mp

    from oracle.nvt_chain import nvt_chain
    from qtip4pf_water_gb300.start import seeded_start

    st = seeded_start(64, 2, 298.0, seed=5)
    jobs = [(64, 2, st.box_bohr, st.q, st.p, 298.0, 0.5, s, 12, 2, k, 4) for s, k in ((7, 0), (7, 0), (8, 0), (7, 1))]
    with mp.get_context("spawn").Pool(2) as pool:
        a, b, c, d = pool.map(nvt_chain, jobs)
    assert a == b and a[:2] != c[:2]
    assert a[:2] != d[:2]  # the system index keys the noise too
    assert all(np.isfinite(x) for x in a[:2] + c[:2])
    assert len(a[2]) == len(a[3]) == 4 and a[2] != c[2]
