"""CPU checks of the surrogate oracle: the hand-derived backward pass against
finite differences, and basic invariances of the symmetry functions."""
import numpy as np

from oracle import surrogate_oracle as so


def _exact_forward(p, x):
    z1 = x @ p["w1"].T + p["b1"]
    h1 = so.silu(z1)
    z2 = h1 @ p["w2"].T + p["b2"]
    h2 = so.silu(z2)
    y = h2 @ p["w3"].T + p["b3"]
    return y, dict(x=x, z1=z1, h1=h1, z2=z2, h2=h2, w1=p["w1"], w2=p["w2"], w3=p["w3"])


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = so.init_params(3)
    for k in ("b1", "b2", "b3"):
        p[k] = rng.standard_normal(p[k].shape) * 0.1
    x = rng.standard_normal((7, 96))
    t = rng.standard_normal((7, 16))
    y, cache = _exact_forward(p, x)
    _, dy = so.mse_loss(y, t)
    g = so.mlp_backward(cache, dy, bf16_grads=False)
    eps = 1e-6
    for name in ("w1", "w2", "w3", "b1", "b2", "b3"):
        flat = p[name].reshape(-1)
        for idx in rng.choice(flat.size, 5, replace=False):
            if name == "w3" and idx // 64 >= 9:
                continue
            old = flat[idx]
            flat[idx] = old + eps
            lp = so.mse_loss(_exact_forward(p, x)[0], t)[0]
            flat[idx] = old - eps
            lm = so.mse_loss(_exact_forward(p, x)[0], t)[0]
            flat[idx] = old
            fd = (lp - lm) / (2 * eps)
            an = g[name].reshape(-1)[idx]
            assert abs(fd - an) <= 1e-6 * max(1.0, abs(fd)), (name, idx, fd, an)


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 1e-3])
    r = so.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == 1.0078125
    assert abs(r[3] + 3.140625) < 1e-12
    assert np.all(np.abs(r - x) <= np.abs(x) * 2.0 ** -8)


def test_descriptors_are_translation_invariant_and_species_resolved():
    from qtip4pf_water_gb300.start import seeded_start

    st = seeded_start(64, 1, 298.0, seed=4)
    d0 = so.sym_descriptors(st.q, st.box_bohr)
    shifted = st.q.reshape(-1, 3) + np.array([1.7, -0.3, 2.2])
    d1 = so.sym_descriptors(shifted.reshape(-1), st.box_bohr)
    assert d0.shape == (192, 32)
    assert np.allclose(d0, d1, rtol=1e-10, atol=1e-12)
    assert np.all(d0 >= 0.0) and np.all(d0[:, :8] > 0.0)
    # the O of a water sees its own two H at ~0.94 A in the H block of G2
    assert np.all(d0[0::3, 15] > 2 * np.exp(-1.5 * 0.95 ** 2) * so.fcut(0.95) * 0.9)


def test_g5_pair_sums_equal_their_moment_form():
    """The device forms G5 from per-atom moments of each species set (W = sum w,
    V = sum w u, M = sum w u u^T, Q = sum w^2); the oracle sums the neighbour
    pairs explicitly. Both forms of the same sums agree to round-off."""
    from qtip4pf_water_gb300.start import seeded_start

    st = seeded_start(64, 1, 298.0, seed=6)
    d = so.sym_descriptors(st.q, st.box_bohr)
    x = st.q.reshape(-1, 3) * so.BOHR_A
    L = st.box_bohr * so.BOHR_A
    h_atom = np.arange(len(x)) % 3 != 0
    for i in (0, 1, 2, 50, 100, 191):
        dd = x - x[i]
        dd -= L * np.rint(dd / L)
        r = np.sqrt((dd * dd).sum(1))
        m = r < so.RC_A
        m[i] = False
        u, fc, h = dd[m] / r[m, None], so.fcut(r[m]), h_atom[m]
        for e, eta in enumerate((0.005, 0.02)):
            w = np.exp(-eta * r[m] ** 2) * fc
            mom = {}
            for name, sel in (("O", ~h), ("H", h)):
                ws, us = w[sel], u[sel]
                mom[name] = (ws.sum(), ws @ us, np.einsum("j,ja,jb->ab", ws, us, us), ws @ ws)
            same = [sum(0.5 * (f(mom[s]) - mom[s][3]) for s in "OH")
                    for f in (lambda t: t[0] ** 2, lambda t: t[1] @ t[1], lambda t: (t[2] * t[2]).sum())]
            mixed = [mom["O"][0] * mom["H"][0], mom["O"][1] @ mom["H"][1], (mom["O"][2] * mom["H"][2]).sum()]
            for k, (zeta, lam) in enumerate(((1, 1), (1, -1), (2, 1), (2, -1))):
                for base, (v0, v1, v2) in ((16, same), (24, mixed)):
                    g = v0 + lam * v1 if zeta == 1 else 0.5 * (v0 + 2 * lam * v1 + v2)
                    assert abs(g - d[i, base + 4 * e + k]) <= 1e-10 * max(1.0, abs(g)), (i, base, e, k)
