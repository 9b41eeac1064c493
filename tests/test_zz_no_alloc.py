"""qtg_kwald_noalloc, the reciprocal-space Ewald entry point that allocates no
device memory (for callers that are handed preallocated GPU buffers and may
not call cudaMalloc, e.g. engine plugins and work issued during another
library's stream capture).

It must give what qtg_kwald gives on the same inputs, within the FP64
tolerance of the other parity tests (1e-9 relative), on two calls in a row --
the second on a different system, so that anything left in the shared static
scratch by the first call would show. Kept in its own file, collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-9


def _sites(q, n_mols):
    """Charge sites (M, H1, H2) of bead 0, as forces.cpp:558-564 builds them."""
    g = 0.73612
    a = q[0].reshape(n_mols, 3, 3)
    s = a.copy()
    s[:, 0, :] = g * a[:, 0, :] + 0.5 * (1.0 - g) * (a[:, 1, :] + a[:, 2, :])
    return np.ascontiguousarray(s.reshape(-1))


def _reference_kwald(q_mod, n_mols, box, sites):
    s = q_mod.System.create(n_mols, 1, box, precision=q_mod.FP64)
    f = np.zeros(9 * n_mols)
    e = s.kwald(sites, f, s.charges())
    return f, e


def _noalloc_kwald(q_mod, torch, n_mols, box, sites):
    L = q_mod.load()
    dev = torch.device("cuda:0")
    d_sites = torch.from_numpy(sites).to(dev)
    d_charge = torch.from_numpy(q_mod.default_charges(n_mols)).to(dev)
    d_f = torch.zeros(9 * n_mols, dtype=torch.float64, device=dev)
    d_e = torch.zeros(1, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    b = (C.c_double * 3)(*[float(x) for x in box])
    st = L.qtg_kwald_noalloc(C.c_void_p(d_sites.data_ptr()), C.c_void_p(d_charge.data_ptr()), 3 * n_mols, b,
                             1e-6, C.c_void_p(d_f.data_ptr()), C.c_void_p(d_e.data_ptr()),
                             C.c_void_p(stream.cuda_stream))
    assert st == 0
    torch.cuda.synchronize()
    return d_f.cpu().numpy(), float(d_e.cpu().numpy()[0])


def test_noalloc_kwald_matches_kwald_twice():
    torch = pytest.importorskip("torch")
    import qtip4pf_water_gb300 as q

    # two different systems in a row: 512 waters, then 64 waters
    for n_mols, seed in ((512, 91), (64, 92)):
        st = q.seeded_start(n_mols, 1, 298.0, seed=seed)
        sites = _sites(st.q, n_mols)
        f_ref, e_ref = _reference_kwald(q, n_mols, st.box_bohr, sites)
        f, e = _noalloc_kwald(q, torch, n_mols, st.box_bohr, sites)
        assert abs(e - e_ref) <= TOL * abs(e_ref)
        err = np.sqrt(np.mean((f - f_ref) ** 2) / np.mean(f_ref ** 2))
        assert err < TOL, err
        np.testing.assert_allclose(f, f_ref, rtol=0, atol=TOL * np.abs(f_ref).max())


def test_noalloc_rejects_sizes_beyond_its_limit():
    torch = pytest.importorskip("torch")
    import qtip4pf_water_gb300 as q

    L = q.load()
    b = (C.c_double * 3)(30.0, 30.0, 30.0)
    x = torch.zeros(16, dtype=torch.float64, device="cuda:0")
    p = C.c_void_p(x.data_ptr())
    assert L.qtg_kwald_noalloc(p, p, 1539, b, 1e-6, p, p, None) == 1  # beyond 1536 sites
    assert L.qtg_kwald_noalloc(p, p, 10, b, 1e-6, p, p, None) == 1    # not whole molecules
