"""qtg_kwald_noalloc, the reciprocal-space Ewald entry point that allocates no
device memory. It is for callers that are handed preallocated GPU buffers and
may not call cudaMalloc themselves: engine and framework plugins that own the
GPU memory budget, where an allocation of their own would escape that budget
or fail under its cap.

Checks, at the FP64 tolerance of the other parity tests (1e-9 relative):
* the reference's own kwald output (the kw_* golden fixtures: 64, 216 and 512
  waters, made from the reference's sources);
* qtg_kwald on the same inputs, on calls in a row on different systems, so
  that anything the shared static scratch kept from one call would show --
  including the largest k set the scratch holds (k_max = 12, 512 waters);
* the free device memory does not change across calls after the first;
* sizes beyond the limits are rejected with QTG_ERR_ARG.
Kept in its own file, collected last.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

TOL = 1e-9


def _sites(q, n_mols):
    """Charge sites (M, H1, H2) of bead 0, as forces.cpp:558-564 builds them."""
    g = 0.73612
    a = q[0].reshape(n_mols, 3, 3)
    s = a.copy()
    s[:, 0, :] = g * a[:, 0, :] + 0.5 * (1.0 - g) * (a[:, 1, :] + a[:, 2, :])
    return np.ascontiguousarray(s.reshape(-1))


def _ctx_kwald(q_mod, n_mols, box, sites, eps=1e-6):
    s = q_mod.System.create(n_mols, 1, box, precision=q_mod.FP64, eps_ewald=eps)
    f = np.zeros(9 * n_mols)
    e = s.kwald(sites, f, s.charges())
    return f, e, s.info.k_max


class _Buffers:
    """Device buffers the caller owns (allocated before the calls under test)."""

    def __init__(self, q_mod, torch, n_mols):
        dev = torch.device("cuda:0")
        self.torch = torch
        self.sites = torch.zeros(9 * n_mols, dtype=torch.float64, device=dev)
        self.charge = torch.from_numpy(q_mod.default_charges(n_mols)).to(dev)
        self.f = torch.zeros(9 * n_mols, dtype=torch.float64, device=dev)
        self.e = torch.zeros(1, dtype=torch.float64, device=dev)
        self.n_mols = n_mols

    def call(self, L, sites, box, eps=1e-6):
        torch = self.torch
        self.sites.copy_(torch.from_numpy(sites))
        self.f.zero_()
        stream = torch.cuda.current_stream()
        b = (C.c_double * 3)(*[float(x) for x in box])
        st = L.qtg_kwald_noalloc(C.c_void_p(self.sites.data_ptr()), C.c_void_p(self.charge.data_ptr()),
                                 3 * self.n_mols, b, eps, C.c_void_p(self.f.data_ptr()),
                                 C.c_void_p(self.e.data_ptr()), C.c_void_p(stream.cuda_stream))
        torch.cuda.synchronize()
        return st, self.f.cpu().numpy(), float(self.e.cpu().numpy()[0])


def _check(f, e, f_ref, e_ref):
    assert abs(e - e_ref) <= TOL * abs(e_ref)
    err = np.sqrt(np.mean((f - f_ref) ** 2) / np.mean(f_ref ** 2))
    assert err < TOL, err
    np.testing.assert_allclose(f, f_ref, rtol=0, atol=TOL * np.abs(f_ref).max())


def test_noalloc_kwald_matches_the_reference_fixtures():
    torch = pytest.importorskip("torch")
    import qtip4pf_water_gb300 as q

    L = q.load()
    for case in ("n512_p1", "n64_p1", "n216_p1"):
        g = load_golden(case)
        n = int(g["n_mols"])
        buf = _Buffers(q, torch, n)
        st, f, e = buf.call(L, np.ascontiguousarray(g["kw_sites"]), g["box"], float(g["eps_ewald"]))
        assert st == 0
        _check(f, e, g["kw_forces"], float(g["kw_energy"]))


def test_noalloc_kwald_matches_kwald_on_calls_in_a_row():
    torch = pytest.importorskip("torch")
    import qtip4pf_water_gb300 as q

    L = q.load()
    # different systems back to back; the third takes the largest k set (k_max 12)
    runs = ((512, 91, 1e-6), (64, 92, 1e-6), (512, 93, 1e-8), (216, 94, 1e-6))
    bufs = {n: _Buffers(q, torch, n) for n in (64, 216, 512)}
    refs = []
    for n_mols, seed, eps in runs:
        st = q.seeded_start(n_mols, 1, 298.0, seed=seed)
        sites = _sites(st.q, n_mols)
        f_ref, e_ref, kmax = _ctx_kwald(q, n_mols, st.box_bohr, sites, eps)
        refs.append((sites, st.box_bohr, f_ref, e_ref, kmax))
    assert refs[2][4] == 12
    torch.cuda.synchronize()
    # first call on this device (sets the device up), then every call again while
    # the free device memory is watched
    buf = bufs[runs[0][0]]
    assert buf.call(L, refs[0][0], refs[0][1], runs[0][2])[0] == 0
    free0 = torch.cuda.mem_get_info()[0]
    for (n_mols, _, eps), (sites, box, f_ref, e_ref, _) in zip(runs, refs):
        st, f, e = bufs[n_mols].call(L, sites, box, eps)
        assert st == 0
        _check(f, e, f_ref, e_ref)
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_sizes_beyond_its_limit():
    torch = pytest.importorskip("torch")
    import qtip4pf_water_gb300 as q

    L = q.load()
    b = (C.c_double * 3)(30.0, 30.0, 30.0)
    x = torch.zeros(16, dtype=torch.float64, device="cuda:0")
    p = C.c_void_p(x.data_ptr())
    assert L.qtg_kwald_noalloc(p, p, 1539, b, 1e-6, p, p, None) == 1  # beyond 1536 sites
    assert L.qtg_kwald_noalloc(p, p, 10, b, 1e-6, p, p, None) == 1    # not whole molecules
    # 512 waters at eps 1e-9 need k_max 13, one beyond the scratch's 12
    st = q.seeded_start(512, 1, 298.0, seed=95)
    bb = (C.c_double * 3)(*[float(v) for v in st.box_bohr])
    assert L.qtg_kwald_noalloc(p, p, 1536, bb, 1e-9, p, p, None) == 1
