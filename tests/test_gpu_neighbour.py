"""The Verlet-list build in boxes large enough for its cell grid (five or more
cells of side >= r_skin / 2 a side, from ~850 waters): the CSR half list
bit-identical to the oracle's restatement of neighbour.cpp:12-62 (itself pinned
to the reference's build), for wrapped and unwrapped coordinates, and the
symmetric list the stepper keeps consistent with it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n_mols,P,unwrap", [(1000, 2, False), (1000, 1, True), (4096, 1, False)])
def test_cell_list_build_is_bit_exact(gpu_lib, n_mols, P, unwrap):
    from oracle.binding import Oracle

    q = gpu_lib
    st = q.seeded_start(n_mols, P, 298.0, seed=n_mols + P)
    x = st.q.reshape(-1).copy()
    if unwrap:
        rs = np.random.default_rng(3)
        shift = rs.integers(-2, 3, size=(P, n_mols, 1, 3)) * st.box_bohr[None, None, None, :]
        x = (x.reshape(P, n_mols, 3, 3) + shift).reshape(-1)
    s = q.System.create(n_mols, P, st.box_bohr, precision=q.FP64)
    point, lst, disp = s.new_lists()
    disp[:] = 1.0
    for b in range(P):
        s.neighbour_list(x, point, lst, disp, b)
    o = Oracle(n_mols, P, st.box_bohr)
    po, lo, do = o.new_lists()
    for b in range(P):
        assert o.neighbour_list(x, po, lo, do, b) >= 0
    assert np.array_equal(point, po)
    assert np.array_equal(lst, lo)
    assert not disp.any()


def test_stepper_with_cell_list_follows_the_oracle(gpu_lib):
    """A 1000-water system (cell grid active) stepped on the device: its
    rebuilds and forces keep the trajectory on the oracle's."""
    from oracle.binding import Oracle

    q = gpu_lib
    st = q.seeded_start(1000, 1, 298.0, seed=77)
    s = q.System.create(1000, 1, st.box_bohr, precision=q.FP64, dt_fs=0.5, propagator=q.TROTTER, seed=77)
    s.set_state(st.q, st.p)
    s.ctx.init_forces()
    s.ctx.run_steps(3, is_nvt=False)
    s.ctx.sync()
    out = s.get_state()
    o = Oracle(1000, 1, st.box_bohr, 298.0, 0.5)
    qq, pp = st.q.reshape(-1).copy(), st.p.reshape(-1).copy()
    point, lst, disp = o.build_lists(qq)
    f = np.zeros_like(qq)
    o.get_forces(qq, f, point, lst, 0)
    for _ in range(3):
        o.update_class(qq, pp, f, point, lst, disp)
    assert np.abs(out["q"] - qq).max() < 1e-10
