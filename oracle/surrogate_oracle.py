"""CPU oracle of the learned centroid correction (test infrastructure only).

FP64 numpy restatement of what qtip4pf_water_gb300/csrc/surrogate.cu computes:

* sym_descriptors  Behler-Parrinello radial G2 and angular G5 symmetry
  functions within 6 A, 32 per atom, with the same parameter sets and layout
  as the device kernel (Behler & Parrinello, Phys. Rev. Lett. 98, 146401
  (2007); Behler, J. Chem. Phys. 134, 074106 (2011), eq. 27: the angular form
  without the r_jk terms), here as the explicit sum over neighbour pairs (the
  device forms the same sums from per-atom moments);
* mlp_forward / mlp_backward  the per-molecule network 96 -> 64 -> 64 -> 16
  (SiLU), with the device's BF16 rounding of inputs, weights and hidden
  activations emulated and everything else in FP64; the backward pass is the
  hand-derived chain rule, checked here against finite differences.

The reference has no such component (its CMD correction is a tabulated spline,
forces.cpp:452-466), so nothing here is pinned to the reference: the pins are
the finite-difference checks in tests/test_surrogate_oracle.py.
"""
from __future__ import annotations

import numpy as np

BOHR_A = 0.529177210903
RC_A = 6.0
G2_ETA = np.array([0.001, 0.01, 0.03, 0.06, 0.15, 0.3, 0.7, 1.5])
G5_ZETA = np.array([1, 1, 2, 2, 1, 1, 2, 2], dtype=np.float64)
G5_LAMBDA = np.array([1, -1, 1, -1, 1, -1, 1, -1], dtype=np.float64)
G5_ETA = np.array([0.005] * 4 + [0.02] * 4)


def fcut(r, rc=RC_A):
    return np.where(r < rc, 0.5 * (np.cos(np.pi * r / rc) + 1.0), 0.0)


def sym_descriptors(pos_bohr: np.ndarray, box_bohr, rc=RC_A) -> np.ndarray:
    """pos_bohr: [3N*3] (O H1 H2 per molecule) -> float64[3N][32]."""
    x = np.asarray(pos_bohr, dtype=np.float64).reshape(-1, 3) * BOHR_A
    L = np.broadcast_to(np.asarray(box_bohr, dtype=np.float64), (3,)) * BOHR_A
    na = len(x)
    sp = (np.arange(na) % 3 != 0).astype(int)  # 0 = O, 1 = H
    out = np.zeros((na, 32))
    for i in range(na):
        d = x - x[i]
        d -= L * np.rint(d / L)
        r = np.sqrt((d * d).sum(1))
        m = (r < rc)
        m[i] = False
        idx = np.nonzero(m)[0]
        dj, rj, sj = d[idx], r[idx], sp[idx]
        fc = fcut(rj, rc)
        g2 = np.exp(-G2_ETA[None, :] * (rj * rj)[:, None]) * fc[:, None]
        out[i, 0:8] = g2[sj == 0].sum(0)
        out[i, 8:16] = g2[sj == 1].sum(0)
        n = len(idx)
        if n < 2:
            continue
        # G5_i = 2^(1 - zeta) sum_{j < k} (1 + lambda cos theta_jik)^zeta
        #        exp(-eta (r_ij^2 + r_ik^2)) f_c(r_ij) f_c(r_ik), per pair class
        a, b = np.triu_indices(n, 1)
        cs = (dj[a] * dj[b]).sum(1) / (rj[a] * rj[b])
        s2 = rj[a] ** 2 + rj[b] ** 2
        f2 = fc[a] * fc[b]
        same = sj[a] == sj[b]
        for k in range(8):
            base = 1.0 + G5_LAMBDA[k] * cs
            ang = 2.0 ** (1.0 - G5_ZETA[k]) * base ** G5_ZETA[k]
            v = ang * np.exp(-G5_ETA[k] * s2) * f2
            out[i, 16 + k] = v[same].sum()
            out[i, 24 + k] = v[~same].sum()
    return out


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def mlp_forward(p: dict, x: np.ndarray):
    """p: w1 [64][96], w2 [64][64], w3 [16][64], b1, b2, b3 (float). x [m][96].
    Returns (y [m][16], cache) with the device's BF16 roundings."""
    w1, w2, w3 = bf16(p["w1"]), bf16(p["w2"]), bf16(p["w3"])
    xb = bf16(x)
    z1 = xb @ w1.T + p["b1"]
    h1 = bf16(silu(z1))
    z2 = h1 @ w2.T + p["b2"]
    h2 = bf16(silu(z2))
    y = h2 @ w3.T + p["b3"]
    return y, dict(x=xb, z1=z1, h1=h1, z2=z2, h2=h2, w1=w1, w2=w2, w3=w3)


def mse_loss(y, t, n_valid=9):
    """Mean squared error over the n_valid outputs of every row, and dL/dy."""
    m = y.shape[0]
    d = np.zeros_like(y)
    d[:, :n_valid] = y[:, :n_valid] - t[:, :n_valid]
    loss = (d * d).sum() / (m * n_valid)
    return loss, 2.0 * d / (m * n_valid)


def mlp_backward(cache: dict, dy: np.ndarray, bf16_grads: bool = True) -> dict:
    """Gradients of the weights and biases for upstream gradient dy [m][16]. With
    bf16_grads, the backpropagated gradients are rounded to BF16 where the device
    stages them as tensor-core operands."""
    r = bf16 if bf16_grads else (lambda v: v)
    dz3 = r(dy)
    g = {"w3": dz3.T @ cache["h2"], "b3": dz3.sum(0)}
    dh2 = dz3 @ cache["w3"]
    dz2 = r(dh2 * dsilu(cache["z2"]))
    g["w2"] = dz2.T @ cache["h1"]
    g["b2"] = dz2.sum(0)
    dh1 = dz2 @ cache["w2"]
    dz1 = r(dh1 * dsilu(cache["z1"]))
    g["w1"] = dz1.T @ cache["x"]
    g["b1"] = dz1.sum(0)
    return g


def init_params(seed: int, n_in=96, n_h=64, n_out=16, n_valid=9) -> dict:
    """He-style initialisation (the same formula the device trainer uses)."""
    rng = np.random.default_rng(seed)
    p = {"w1": rng.standard_normal((n_h, n_in)) * np.sqrt(2.0 / n_in),
         "w2": rng.standard_normal((n_h, n_h)) * np.sqrt(2.0 / n_h),
         "w3": rng.standard_normal((n_out, n_h)) * np.sqrt(1.0 / n_h),
         "b1": np.zeros(n_h), "b2": np.zeros(n_h), "b3": np.zeros(n_out)}
    p["w3"][n_valid:] = 0.0
    return p
