"""Learned centroid-force correction for centroid molecular dynamics (CMD).

The correction is the constrained-PIMD mean centroid force minus the classical
qTIP4P/F force at the same centroid configuration. A per-molecule network
(csrc/surrogate.cu) maps the symmetry functions of the molecule's three atoms
to that correction in the molecule's frame. This module runs the pipeline on
the device:

  generate()   centroid configurations sampled by batched PIMD replicas from
               seeded lattice starts; for each, a centroid-constrained PIMD run
               accumulates the mean centroid force, and a P = 1 evaluation gives
               the classical force at the centroid
  features()   descriptors, per-molecule rows in both H labellings, targets in
               the molecular frames
  Correction   the network: training with the tensor-core kernels and Adam,
               prediction, evaluation, attachment to a P = 1 context (surrogate
               CMD)

Torch supplies device buffers only; every kernel is the library's own.
"""
from __future__ import annotations

import numpy as np

from . import (FP64, MIXED, MLP_NPARAMS, MLP_NW, PILE_G, PILE_L, TROTTER, Context, MlpWeights, adam_step,
               mlp_forward, mlp_train_batch, seeded_start, surrogate_status, sym_descriptors, system_desc)

N_IN, N_OUT = 96, 9


def _torch():
    import torch

    return torch


# ---- molecular frames (the device's k_frames, in FP64) -------------------------------
def frames(pos, box):
    """pos [9N] bohr -> E [N][3][3], rows e1, e2, e3 of labelling (H1, H2)."""
    r = np.asarray(pos, dtype=np.float64).reshape(-1, 3, 3)
    L = np.broadcast_to(np.asarray(box, dtype=np.float64), (3,))
    d1, d2 = r[:, 1] - r[:, 0], r[:, 2] - r[:, 0]
    d1 -= L * np.rint(d1 / L)
    d2 -= L * np.rint(d2 / L)
    e1 = d1 + d2
    e1 /= np.linalg.norm(e1, axis=1, keepdims=True)
    e2 = d1 - d2
    e2 -= (e2 * e1).sum(1, keepdims=True) * e1
    e2 /= np.linalg.norm(e2, axis=1, keepdims=True)
    return np.stack([e1, e2, np.cross(e1, e2)], axis=1)


SWAP = np.diag([1.0, -1.0, -1.0])  # frame of the swapped labelling: (e1, -e2, -e3)


def to_frame_targets(F, E):
    """Lab forces F [N][9] -> targets [2N][9]: rows (O, H1, H2) in frame E and
    rows (O, H2, H1) in the swapped frame."""
    f = F.reshape(-1, 3, 3)
    a = np.einsum("nij,naj->nai", E, f).reshape(-1, 9)
    Es = np.einsum("ij,njk->nik", SWAP, E)
    b = np.einsum("nij,naj->nai", Es, f[:, [0, 2, 1]]).reshape(-1, 9)
    return np.concatenate([a, b])


def from_frame_outputs(Y, E):
    """Network outputs [2N][>=9] (both labellings) -> symmetrised lab forces [N][9]."""
    n = E.shape[0]
    ya, yb = Y[:n, :9].reshape(n, 3, 3), Y[n:, :9].reshape(n, 3, 3)
    Es = np.einsum("ij,njk->nik", SWAP, E)
    fa = np.einsum("nij,nai->naj", E, ya)
    fb = np.einsum("nij,nai->naj", Es, yb)[:, [0, 2, 1]]
    return (0.5 * (fa + fb)).reshape(n, 9)


# ---- data generation -------------------------------------------------------------------
class Dataset:
    def __init__(self, n_mols, box, centroids, fmean, fclass, meta):
        self.n_mols, self.box = n_mols, np.asarray(box, dtype=np.float64)
        self.centroids, self.fmean, self.fclass = centroids, fmean, fclass
        self.meta = meta

    def __len__(self):
        return len(self.centroids)

    def split(self, n_first):
        a = Dataset(self.n_mols, self.box, self.centroids[:n_first], self.fmean[:n_first], self.fclass[:n_first],
                    self.meta)
        b = Dataset(self.n_mols, self.box, self.centroids[n_first:], self.fmean[n_first:], self.fclass[n_first:],
                    self.meta)
        return a, b


def classical_forces(centroids, n_mols, box, precision=MIXED, batch=32):
    """qTIP4P/F forces at each centroid configuration (P = 1 evaluations, batched)."""
    out = np.zeros_like(centroids)
    for i0 in range(0, len(centroids), batch):
        part = centroids[i0:i0 + batch]
        ctx = Context([system_desc(n_mols, 1, box, propagator=TROTTER, thermostat=PILE_L) for _ in part], precision)
        for s, c in zip(ctx.systems, part):
            s.set_state(c)
        ctx.init_forces()
        for k, s in enumerate(ctx.systems):
            out[i0 + k] = s.get_state()["fphys"]
        ctx.close()
    return out


def generate(n_mols=216, n_beads=32, n_configs=64, replicas=32, temp=298.0, equil_steps=2000, sample_every=200,
             constrained_steps=2000, seed=5, precision=MIXED, dt_fs=0.25):
    """Centroid configurations and their constrained-PIMD mean centroid forces.

    `replicas` PIMD systems (Trotter, PILE-G) start from seeded lattice starts and
    are equilibrated; then, repeatedly, each advances `sample_every` free steps,
    its centroid is frozen for `constrained_steps` (internal modes thermostatted
    by PILE-L) while the mean centroid force accumulates, and it is released."""
    starts = [seeded_start(n_mols, n_beads, temp, seed=seed * 1000 + r) for r in range(replicas)]
    box = starts[0].box_bohr
    descs = [system_desc(n_mols, n_beads, box, temp_K=temp, dt_fs=dt_fs, propagator=TROTTER, thermostat=PILE_L,
                         seed=seed * 1000 + r) for r in range(replicas)]
    ctx = Context(descs, precision)
    for s, st in zip(ctx.systems, starts):
        s.set_state(st.q, st.p)
    ctx.init_forces()
    ctx.run_steps(equil_steps, is_nvt=True)
    cents, fmean = [], []
    while len(cents) < n_configs:
        ctx.run_steps(sample_every, is_nvt=True)
        ctx.sync()
        snap = [s.get_state()["q"].reshape(n_beads, -1).mean(axis=0) for s in ctx.systems]
        for s in ctx.systems:
            s.set_centroid_fixed(True)
            s.reset_centroid_force()
        ctx.run_steps(constrained_steps, is_nvt=True)
        ctx.sync()
        for s, c in zip(ctx.systems, snap):
            f, n = s.centroid_force()
            assert n == constrained_steps
            cents.append(c)
            fmean.append(f)
            s.set_centroid_fixed(False)
    ctx.close()
    cents, fmean = np.array(cents[:n_configs]), np.array(fmean[:n_configs])
    fclass = classical_forces(cents, n_mols, box, precision)
    meta = dict(n_mols=n_mols, n_beads=n_beads, temp_K=temp, replicas=replicas, equil_steps=equil_steps,
                sample_every=sample_every, constrained_steps=constrained_steps, seed=seed, dt_fs=dt_fs)
    return Dataset(n_mols, box, cents, fmean, fclass, meta)


def descriptors(centroids, n_mols, box, chunk=256):
    """Symmetry functions of every atom of every configuration: float32[n][3N][32]."""
    torch = _torch()
    out = np.zeros((len(centroids), 3 * n_mols, 32), dtype=np.float32)
    for i0 in range(0, len(centroids), chunk):
        part = np.ascontiguousarray(centroids[i0:i0 + chunk], dtype=np.float64)
        pos = torch.tensor(part, device="cuda")
        d = torch.empty((len(part), 3 * n_mols, 32), dtype=torch.float32, device="cuda")
        sym_descriptors(pos.data_ptr(), len(part), n_mols, box, d.data_ptr())
        out[i0:i0 + len(part)] = d.cpu().numpy()
    if surrogate_status() != 0:
        raise RuntimeError("descriptor kernel reported an error")
    return out


def mol_rows(desc):
    """Per-configuration descriptors [3N][32] -> network rows [2N][96]: (O, H1, H2) then (O, H2, H1)."""
    d = desc.reshape(-1, 3, 32)
    return np.concatenate([d.reshape(-1, 96), d[:, [0, 2, 1]].reshape(-1, 96)])


def features(ds: Dataset):
    """Inputs X [rows][96] and frame targets T [rows][9] of the dataset (correction = fmean - fclass)."""
    D = descriptors(ds.centroids, ds.n_mols, ds.box)
    X, T = [], []
    for c in range(len(ds)):
        E = frames(ds.centroids[c], ds.box)
        X.append(mol_rows(D[c]))
        T.append(to_frame_targets((ds.fmean[c] - ds.fclass[c]).reshape(-1, 9), E))
    return np.concatenate(X), np.concatenate(T)


# ---- the network -------------------------------------------------------------------------
class Correction:
    """Per-molecule network with FP32 master parameters on the device."""

    def __init__(self, seed=0):
        torch = _torch()
        rng = np.random.default_rng(seed)
        w1 = rng.standard_normal((64, 96)) * np.sqrt(2.0 / 96)
        w2 = rng.standard_normal((64, 64)) * np.sqrt(2.0 / 64)
        w3 = np.zeros((16, 64))
        w3[:9] = rng.standard_normal((9, 64)) * np.sqrt(1.0 / 64) * 0.1
        flat = np.concatenate([w1.ravel(), w2.ravel(), w3.ravel(), np.zeros(64 + 64 + 16)])
        assert flat.size == MLP_NPARAMS
        self.params = torch.tensor(flat, dtype=torch.float32, device="cuda")
        self.m1 = torch.zeros_like(self.params)
        self.m2 = torch.zeros_like(self.params)
        self.wbf = self.params[:MLP_NW].to(torch.bfloat16).contiguous()
        self.mean = np.zeros(96, np.float32)
        self.inv_std = np.ones(96, np.float32)
        self.out_scale = 1.0
        self.step = 0
        self.history = []

    def weights(self):
        P, B = self.params.data_ptr(), self.wbf.data_ptr()
        return MlpWeights(B, B + 2 * 64 * 96, B + 2 * (64 * 96 + 64 * 64), P + 4 * MLP_NW, P + 4 * (MLP_NW + 64),
                          P + 4 * (MLP_NW + 128))

    def norm(self):
        return np.concatenate([self.mean, self.inv_std]).astype(np.float32)

    def _inputs(self, X):
        torch = _torch()
        Xn = (np.asarray(X, np.float32) - self.mean) * self.inv_std
        return torch.tensor(Xn, device="cuda").to(torch.bfloat16).contiguous()

    def fit(self, X, T, steps=2000, lr=3e-3, lr_final=3e-4, log_every=100):
        """Full-batch Adam on the tensor-core trainer; inputs normalised per column,
        targets by their RMS (out_scale)."""
        torch = _torch()
        self.mean = X.mean(0).astype(np.float32)
        self.inv_std = (1.0 / np.maximum(X.std(0), 1e-6)).astype(np.float32)
        self.out_scale = float(np.sqrt(np.mean(T ** 2)))
        m = len(X)
        xd = self._inputs(X)
        t = np.zeros((m, 16), np.float32)
        t[:, :9] = T / self.out_scale
        td = torch.tensor(t, device="cuda")
        max_ctas = 512
        part = torch.zeros((max_ctas, MLP_NPARAMS + 1), dtype=torch.float32, device="cuda")
        grad = torch.zeros(MLP_NPARAMS + 1, dtype=torch.float32, device="cuda")
        for k in range(steps):
            mlp_train_batch(self.weights(), xd.data_ptr(), td.data_ptr(), m, 2.0 / (m * 9), part.data_ptr(),
                            max_ctas, grad.data_ptr())
            self.step += 1
            rate = lr * (lr_final / lr) ** (k / max(1, steps - 1))
            adam_step(self.params.data_ptr(), self.m1.data_ptr(), self.m2.data_ptr(), grad.data_ptr(), MLP_NPARAMS,
                      self.step, rate, self.wbf.data_ptr(), MLP_NW)
            if k % log_every == 0 or k == steps - 1:
                self.history.append((k, float(grad[-1].item()) / (m * 9)))
        if surrogate_status() != 0:
            raise RuntimeError("training kernel reported an error")
        return self.history[-1][1]

    def predict(self, X):
        """Frame-space corrections [rows][9] (Hartree/bohr)."""
        torch = _torch()
        xd = self._inputs(X)
        y = torch.empty((len(X), 16), dtype=torch.float32, device="cuda")
        mlp_forward(self.weights(), xd.data_ptr(), len(X), y.data_ptr())
        return y.cpu().numpy()[:, :9].astype(np.float64) * self.out_scale

    def lab_corrections(self, ds: Dataset, desc=None):
        D = descriptors(ds.centroids, ds.n_mols, ds.box) if desc is None else desc
        out = np.zeros_like(ds.fmean)
        for c in range(len(ds)):
            E = frames(ds.centroids[c], ds.box)
            out[c] = from_frame_outputs(self.predict(mol_rows(D[c])), E).reshape(-1)
        return out

    def evaluate(self, ds: Dataset):
        """Centroid-force RMS error relative to the constrained-PIMD mean force,
        without the correction (classical force) and with it."""
        corr = self.lab_corrections(ds)
        ref = ds.fmean
        den = np.sqrt(np.mean(ref ** 2))
        e0 = np.sqrt(np.mean((ds.fclass - ref) ** 2)) / den
        e1 = np.sqrt(np.mean((ds.fclass + corr - ref) ** 2)) / den
        # the part of the error that is the correction itself (what the network must learn)
        target = ref - ds.fclass
        e_corr = np.sqrt(np.mean((corr - target) ** 2)) / np.sqrt(np.mean(target ** 2))
        return {"rms_rel_err_classical": float(e0), "rms_rel_err_corrected": float(e1),
                "rms_rel_err_of_correction": float(e_corr), "configs": len(ds)}

    def attach(self, system):
        system.attach_surrogate(self.weights(), self.norm(), self.out_scale)
