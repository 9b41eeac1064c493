"""Per-call stepping (the update_sc_nospline drop-in): the Verlet list goes back
to the caller only when the skin test rebuilt it (and then whole, cleared past
the new list as the reference clears it), masses and charges are uploaded only
when they change, and the transfer counters see exactly that."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(q, N=64, P=4):
    st = q.seeded_start(N, P, 298.0, seed=41)
    s = q.System.create(N, P, st.box_bohr, precision=q.MIXED, propagator=q.TROTTER, thermostat=q.PILE_G, seed=41)
    qq, pp = st.q.reshape(-1).copy(), st.p.reshape(-1).copy()
    point, lst, disp = s.build_lists(qq)
    f = np.zeros_like(qq)
    s.force_eval_trotter(qq, f, s.charges(), point, lst)
    return s, qq, pp, point, lst, disp, f, f.copy()


def _used_mask(s, point):
    P, N, cap = s.P, s.N, s.info.list_size
    mask = np.zeros(P * cap, bool)
    for b in range(P):
        mask[b * cap: b * cap + point[b * N + N - 1]] = True
    return mask


def test_list_comes_back_only_after_a_rebuild(gpu_lib):
    q = gpu_lib
    s, qq, pp, point, lst, disp, f, fp = _setup(q)
    mass, chg = s.masses(), s.charges()
    used = _used_mask(s, point)
    lst[~used] = -7  # entries past each bead's list: never read, and untouched without a rebuild
    before = lst.copy()
    h0 = s.ctx.transfer_bytes()
    _, heat, _ = s.update_sc_nospline(qq, pp, mass, f, fp, chg, point, lst, disp, True, 0.0)
    h1 = s.ctx.transfer_bytes()
    assert np.array_equal(lst, before)  # no rebuild: untouched
    assert h1[1] - h0[1] < lst.nbytes  # and the list was not downloaded
    # a second call with the same masses and charges uploads neither
    _, heat, _ = s.update_sc_nospline(qq, pp, mass, f, fp, chg, point, lst, disp, True, heat)
    h2 = s.ctx.transfer_bytes()
    assert (h2[0] - h1[0]) <= (h1[0] - h0[0])
    # displacements beyond the skin force a rebuild on the next call
    disp[:] = 0.0
    disp[0::3] = 10.0  # |disp| = 10 bohr for every molecule: beyond any skin margin
    _, heat, _ = s.update_sc_nospline(qq, pp, mass, f, fp, chg, point, lst, disp, True, heat)
    h3 = s.ctx.transfer_bytes()
    assert h3[1] - h2[1] >= lst.nbytes
    ref_point, ref_list, _ = s.build_lists(qq)
    assert np.array_equal(point, ref_point)
    new_used = _used_mask(s, point)
    assert np.array_equal(lst[new_used], ref_list[new_used])
    # a rebuild clears the whole list first, as the reference's neighbour_list does
    # (neighbour.cpp:23-25): past the new list the caller's array now reads zero
    assert np.all(lst[~new_used] == 0)


def test_mixed_step_reads_neither_list_nor_fphys(gpu_lib):
    """Mixed precision takes the dense Lennard-Jones kernel, and fphys is output
    only: a step with the caller's point/list/fphys overwritten by junk gives the
    same state as one with the real arrays, and leaves the junk in place."""
    q = gpu_lib
    runs = []
    for junk in (False, True):
        s, qq, pp, point, lst, disp, f, fp = _setup(q)
        if junk:
            point[:] = -3
            lst[:] = -7
            fp[:] = np.nan
        _, heat, _ = s.update_sc_nospline(qq, pp, s.masses(), f, fp, s.charges(), point, lst, disp, True, 0.0)
        runs.append((qq.copy(), pp.copy(), f.copy(), fp.copy(), heat))
        if junk:
            assert np.all(point == -3) and np.all(lst == -7)  # no rebuild: neither written
    for a, b in zip(runs[0][:4], runs[1][:4]):
        assert np.array_equal(a, b)
    assert runs[0][4] == runs[1][4]


def test_only_rebuilt_beads_come_back(gpu_lib):
    q = gpu_lib
    s, qq, pp, point, lst, disp, f, fp = _setup(q)
    P, N, cap = s.P, s.N, s.info.list_size
    point0, lst0 = point.copy(), lst.copy()
    # a step without a rebuild: the downloads every step makes
    disp[:] = 0.0
    h0 = s.ctx.transfer_bytes()
    s.update_sc_nospline(qq, pp, s.masses(), f, fp, s.charges(), point, lst, disp, True, 0.0)
    h1 = s.ctx.transfer_bytes()
    assert np.array_equal(point, point0) and np.array_equal(lst, lst0)
    disp[:] = 0.0
    b = 2
    disp[b * 3 * N: (b + 1) * 3 * N: 3] = 10.0  # bead b only: beyond the skin margin
    s.update_sc_nospline(qq, pp, s.masses(), f, fp, s.charges(), point, lst, disp, True, 0.0)
    h2 = s.ctx.transfer_bytes()
    ref_point, ref_list, _ = s.build_lists(qq)
    for k in range(P):
        sl_p, sl_l = slice(k * N, (k + 1) * N), slice(k * cap, (k + 1) * cap)
        if k == b:
            assert np.array_equal(point[sl_p], ref_point[sl_p])
            assert np.array_equal(lst[sl_l], ref_list[sl_l])
        else:
            assert np.array_equal(point[sl_p], point0[sl_p])
            assert np.array_equal(lst[sl_l], lst0[sl_l])
    # exactly one bead's point and list came down on top of the every-step downloads
    assert (h2[1] - h1[1]) - (h1[1] - h0[1]) == 4 * (N + cap)
    assert np.all(disp[b * 3 * N: (b + 1) * 3 * N] == 0.0)


def test_staged_and_copied_steps_agree(gpu_lib):
    """Arrays in page-locked host memory move inside the step's graph by the stage
    kernels; pageable arrays by copy calls. Both give the same state and heat bits
    (the per-bead energies are sums of FP64 atomic adds, whose order may vary), and
    the staged call launches three stage kernels on top of the step's own (stage
    in; stage out of q and disp beside the forces, of f and fphys beside the
    closing kick; the closing kick itself writes p back and posts the small
    results)."""
    torch = pytest.importorskip("torch")
    q = gpu_lib
    out = []
    for pinned in (False, True):
        s, qq, pp, point, lst, disp, f, fp = _setup(q)
        if pinned:
            qq, pp, disp, f, fp = (torch.from_numpy(a.copy()).pin_memory().numpy() for a in (qq, pp, disp, f, fp))
        heat, launches, e = 0.0, [], 0.0
        for _ in range(3):
            k0 = s.ctx.kernel_launches()
            e, heat, _ = s.update_sc_nospline(qq, pp, s.masses(), f, fp, s.charges(), point, lst, disp, True, heat)
            launches.append(s.ctx.kernel_launches() - k0)
        out.append((qq.copy(), pp.copy(), f.copy(), fp.copy(), disp.copy(), heat, e, launches))
    for a, b in zip(out[0][:5], out[1][:5]):
        assert np.array_equal(a, b)
    assert out[0][5] == out[1][5] != 0.0
    assert abs(out[0][6] - out[1][6]) <= 1e-12 * abs(out[0][6])
    assert all(x == out[0][7][0] + 3 for x in out[1][7]), (out[0][7], out[1][7])
