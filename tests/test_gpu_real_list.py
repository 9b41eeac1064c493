"""The mixed real space of large beads over the pair list (k_rlist_test,
k_rlist_rows, k_real_list) against the oracle's FP64 restatement of the
reference's all-pairs sum (forces.cpp:589-608) and against the all-pairs FP32
kernel (k_real_f32). Both forms take the same site pairs (those within r_c), so
the forces agree with the oracle at the mixed-mode tolerance (1e-4 relative RMS)
and with each other to FP32 summation order (1e-5 relative RMS). Energies
follow the mixed-mode convention of the parity tests: within 1e-6 of the Ewald
self-energy of the oracle's, and within 1e-7 of it of each other (the total is
a small difference of Ewald terms of that size). The list stays complete while
the system moves: the forces a run ends with, computed with whatever list the
displacement test kept, equal the all-pairs forces at the positions the run
reached. A configuration with a molecule wider than the spread bound of the
one-image-per-molecule-pair form takes a minimum image per site pair and gives
the same forces."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_rms(a, b):
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


def ewald_self(s):
    qc = s.charges()
    return float(np.sum(s.info.kappa / np.sqrt(np.pi) * qc * qc))


def _stepper(q, st, P, form, dt=0.25, seed=7):
    ctx = q.Context([q.system_desc(st.n_mols, P, st.box_bohr, dt_fs=dt, propagator=q.TROTTER,
                                   thermostat=q.PILE_G, seed=seed)], q.MIXED)
    ctx.set_real_space(form)
    s = ctx.systems[0]
    s.set_state(st.q, st.p)
    ctx.init_forces()
    return ctx, s


def test_eligibility(gpu_lib):
    q = gpu_lib
    for n_mols, eligible in ((512, False), (1000, True), (4096, True)):
        st = q.seeded_start(n_mols, 1, 298.0, seed=3)
        ctx = q.Context([q.system_desc(n_mols, 1, st.box_bohr)], q.MIXED)
        assert ctx.real_space() == (0, eligible), n_mols
        ctx.close()
    st = q.seeded_start(1000, 1, 298.0, seed=3)
    ctx = q.Context([q.system_desc(1000, 1, st.box_bohr)], q.FP64)
    assert ctx.real_space() == (0, False)
    with pytest.raises(q.QtgError):
        ctx.set_real_space(2)


@pytest.mark.parametrize("n_mols", [1000, 4096])
def test_list_forces_and_energy_match_the_oracle(gpu_lib, n_mols):
    from oracle.binding import Oracle

    q = gpu_lib
    st = q.seeded_start(n_mols, 1, 298.0, seed=40)
    x = st.q.reshape(-1).copy()
    s = q.System.create(n_mols, 1, st.box_bohr, precision=q.MIXED)
    point, lst, _ = s.build_lists(x)
    out = {}
    for form in (1, 0):
        s.ctx.set_real_space(form)
        f = np.zeros_like(x)
        e = s.get_forces_nospline(x, f, s.charges(), point, lst, 0)
        out[form] = (f, e)
    o = Oracle(n_mols, 1, st.box_bohr)
    po, lo, _ = o.build_lists(x)
    fo = np.zeros_like(x)
    eo = o.get_forces(x, fo, po, lo, 0)
    (fl, el), (fa, ea) = out[0], out[1]
    assert rel_rms(fl, fo) < 1e-4
    assert abs(el - eo) < 1e-6 * ewald_self(s)
    assert rel_rms(fl, fa) < 1e-5
    assert abs(el - ea) < 1e-7 * ewald_self(s)


def test_list_forces_of_several_beads_match_the_oracle(gpu_lib):
    from oracle.binding import Oracle

    q = gpu_lib
    P = 2
    st = q.seeded_start(1000, P, 298.0, seed=41)
    ctx, s = _stepper(q, st, P, 0)
    f_list = s.get_state()["fphys"]
    o = Oracle(1000, P, st.box_bohr, 298.0, 0.25)
    qq = st.q.reshape(-1).copy()
    point, lst, _ = o.build_lists(qq)
    fo = np.zeros_like(qq)
    o.force_eval_trotter(qq, fo, point, lst)
    assert rel_rms(f_list, fo) < 1e-4
    ctx.set_real_space(1)
    ctx.init_forces()
    assert rel_rms(f_list, s.get_state()["fphys"]) < 1e-5


def test_suzuki_chin_forces_of_large_beads_match_the_oracle(gpu_lib):
    """Suzuki-Chin assembly of 1000 waters, P = 4, mixed: the physical forces
    (real space over the pair list, Lennard-Jones over the list) and the
    propagating Suzuki-Chin forces (with the FP64 finite-difference gradient
    terms) against the oracle's restatement of force_eval_sc_nospline."""
    from oracle.binding import Oracle

    q = gpu_lib
    P = 4
    st = q.seeded_start(1000, P, 298.0, seed=47)
    ctx = q.Context([q.system_desc(1000, P, st.box_bohr, dt_fs=0.25, propagator=q.SUZUKI_CHIN,
                                   thermostat=q.PILE_G, seed=47)], q.MIXED)
    assert ctx.real_space() == (0, True)
    s = ctx.systems[0]
    s.set_state(st.q, st.p)
    ctx.init_forces()
    out = s.get_state()
    o = Oracle(1000, P, st.box_bohr, 298.0, 0.25)
    qq = st.q.reshape(-1).copy()
    point, lst, _ = o.build_lists(qq)
    f, fp = np.zeros_like(qq), np.zeros_like(qq)
    o.force_eval_sc(qq, f, point, lst, fp)
    assert rel_rms(out["fphys"], fp) < 1e-4
    assert rel_rms(out["f"], f) < 1e-4


def test_list_stays_complete_while_the_system_moves(gpu_lib):
    """Also the Lennard-Jones term of large beads, which the stepper takes over
    its symmetric Verlet list (rebuilt beside the forces): the forces at the
    positions a run reached against the oracle's at the same positions."""
    from oracle.binding import Oracle

    q = gpu_lib
    st = q.seeded_start(1000, 2, 298.0, seed=45)
    ctx, s = _stepper(q, st, 2, 0, dt=0.5)
    o = Oracle(1000, 2, st.box_bohr, 298.0, 0.5)
    for _ in range(3):
        ctx.run_steps(300, is_nvt=True)
        ctx.sync()
        state = s.get_state()
        point, lst, _ = o.build_lists(state["q"])
        fo = np.zeros_like(state["q"])
        o.force_eval_trotter(state["q"].copy(), fo, point, lst)
        assert rel_rms(state["fphys"], fo) < 1e-4
        ctx.set_real_space(1)
        ctx.init_forces()
        f_all = s.get_state()["fphys"]
        assert rel_rms(state["fphys"], f_all) < 1e-5
        ctx.set_real_space(0)
        ctx.init_forces()
        assert rel_rms(s.get_state()["fphys"], f_all) < 1e-5


def test_a_wide_molecule_takes_a_minimum_image_per_site_pair(gpu_lib):
    from oracle.binding import Oracle

    q = gpu_lib
    st = q.seeded_start(1000, 1, 298.0, seed=46)
    x = st.q.reshape(1000, 3, 3).copy()
    x[5, 1] = x[5, 0] + np.array([4.0, 0.0, 0.0])  # an O-H bond of 4 bohr: H1 ~3.5 bohr from M
    x = x.reshape(-1)
    s = q.System.create(1000, 1, st.box_bohr, precision=q.MIXED)
    point, lst, _ = s.build_lists(x)
    out = {}
    for form in (1, 0):
        s.ctx.set_real_space(form)
        f = np.zeros_like(x)
        out[form] = f, s.get_forces_nospline(x, f, s.charges(), point, lst, 0)
    o = Oracle(1000, 1, st.box_bohr)
    po, lo, _ = o.build_lists(x)
    fo = np.zeros_like(x)
    eo = o.get_forces(x, fo, po, lo, 0)
    assert rel_rms(out[0][0], out[1][0]) < 1e-5
    assert rel_rms(out[0][0], fo) < 1e-4
    assert abs(out[0][1] - eo) < 1e-6 * ewald_self(s)
