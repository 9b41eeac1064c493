"""Error paths that the kernels detect and report instead of failing silently
(the reference writes past the list on overflow, neighbour.cpp:56-58, and keeps
running on non-finite energies): the device sets a status bit, the host call
returns the matching status, and the context stays usable."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _packed_oxygens(st, n, width_bohr=6.0, seed=0):
    """Every molecule shifted so its oxygen lies in a small cube: all O-O pairs
    fall inside r_skin (the molecules overlap; only the list build reads them)."""
    rng = np.random.default_rng(seed)
    q = st.q.reshape(-1, n, 3, 3).copy()
    target = rng.uniform(0.0, width_bohr, size=(q.shape[0], n, 1, 3))
    q += target - q[:, :, :1, :]
    return q.reshape(-1)


def test_list_overflow_is_reported_and_the_context_recovers(gpu_lib):
    q = gpu_lib
    n = 512
    st = q.seeded_start(n, 1, 298.0, seed=7)
    s = q.System.create(n, 1, st.box_bohr, precision=q.MIXED, propagator=q.TROTTER)
    assert n * (n - 1) // 2 > s.info.list_size  # all pairs cannot fit
    point, lst, disp = s.new_lists()
    with pytest.raises(q.QtgError) as ei:
        s.neighbour_list(_packed_oxygens(st, n), point, lst, disp, 0)
    assert ei.value.status == 3
    # the lattice start still builds, and matches a fresh context's list
    s.neighbour_list(st.q, point, lst, disp, 0)
    ref = q.System.create(n, 1, st.box_bohr, precision=q.MIXED, propagator=q.TROTTER)
    p2, l2, d2 = ref.new_lists()
    ref.neighbour_list(st.q, p2, l2, d2, 0)
    assert np.array_equal(point, p2) and np.array_equal(lst, l2)


def test_non_finite_forces_stop_the_stepper(gpu_lib):
    q = gpu_lib
    st = q.seeded_start(27, 2, 298.0, seed=9)
    s = q.System.create(27, 2, st.box_bohr, precision=q.MIXED, propagator=q.TROTTER)
    bad = st.q.copy()
    bad.reshape(-1)[5] = np.nan
    s.set_state(bad, st.p)
    with pytest.raises(q.QtgError) as ei:
        s.ctx.init_forces()
    assert ei.value.status == 4
    # a finite state afterwards runs normally
    s.set_state(st.q, st.p)
    s.ctx.init_forces()
    s.ctx.run_steps(3, is_nvt=True)
    s.ctx.sync()
    assert np.all(np.isfinite(s.get_state()["q"]))
